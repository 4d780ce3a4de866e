// Oracle: a CPU restatement of LehrFEM++'s assembly-and-solve path.
//
// TEST INFRASTRUCTURE ONLY.  This code is the checker for the GPU library in
// lehrfempp_gb300/: only tests/, __graft_entry__.smoke() and bench.py's
// cpu_baseline / --impl reference legs may load it.  The product never links,
// imports or calls anything under oracle/.
//
// Every function restates one piece of the reference (file:line relative to
// the LehrFEM++ source tree).  The structure follows the reference closely
// (std::map edge numbering, per-cell provider Eval with a per-quadrature-point
// loop, triplet push_back in cell order) because the oracle's job is to
// reproduce the reference's numbering and arithmetic, not to be fast.
//
// Pinning: the oracle is checked against every golden vector the reference's
// own tests hold for this path (tests/test_oracle_golden.py): the 10x10 and
// 36x36 assembled matrices of lib/lf/assemble/test/assembly_tests.cc, the
// fix-dof exact solution of lib/lf/assemble/test/coomatrix_tests.cc, the
// reaction-diffusion bilinear-form values of
// lib/lf/uscalfe/test/lagr_fe_tests.cc:807-883, volume row sums and quadrature
// exactness.
#pragma once

#include <array>
#include <cstdint>
#include <functional>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

namespace lfo {

using idx_t = int64_t;

struct Error : std::runtime_error {
  using std::runtime_error::runtime_error;
};

// ---------------------------------------------------------------- quadrature
// lib/lf/quad/quad_rule.h:58-195: points (2 x n, column k = point k), weights.
struct QuadRule {
  int degree = 0;
  std::vector<double> x, y, w;
  int n() const { return static_cast<int>(w.size()); }
};
// lib/lf/quad/gauss_quadrature.cc:16-69 (points on [0,1], weights sum to 1).
void GaussLegendre(int n, std::vector<double>& pts, std::vector<double>& wts);
// lib/lf/quad/make_quad_rule.cc:21-157 for kTria (the tables of
// quad/quad_rules_tria.cc for degrees 1..50, 3 -> 4; conical rule otherwise)
// and kQuad (tensor Gauss-Legendre, n = deg/2+1).
QuadRule MakeQuadRule(bool is_quad, int degree);

// ------------------------------------------------------ reference elements
// Lagrangian reference shape functions of lib/lf/uscalfe/lagr_fe.h:57-1484.
// phi[i], dphi[i][0..1] at one reference point.
int NumShapeFunctions(bool is_quad, int degree);
void EvalShape(bool is_quad, int degree, double xh, double yh, double* phi,
               double (*dphi)[2]);
// Evaluation nodes (x,y per local shape function) used by NodalProjection.
void EvaluationNodes(bool is_quad, int degree, std::vector<double>& xy);

// ---------------------------------------------------------------- geometry
// lib/lf/geometry/tria_o1.cc:50-74 and quad_o1.cc:67-156.
struct CellGeom {
  bool is_quad;
  double v[4][2];
  // JacobianInverseGramian (= (J^T)^{-1} for 2D), |det J| and Global().
  void JinvT(double xh, double yh, double out[2][2]) const;
  double IntegrationElement(double xh, double yh) const;
  void Global(double xh, double yh, double out[2]) const;
};
// tria_o1.cc:10-48 / quad_o1.cc:12-58 (tol 1e-8); returns false if degenerate.
bool NonDegenerate(const CellGeom& g, double tol = 1.0e-8);

// -------------------------------------------------------------------- mesh
// The numbering of lib/lf/mesh/hybrid2d/mesh.cc:178-810.
struct Mesh {
  idx_t num_nodes = 0;
  std::vector<double> xy;                       // 2 per node
  idx_t num_cells = 0;
  std::vector<std::array<idx_t, 4>> cell_nodes;  // -1 padded (tria)
  idx_t num_edges = 0;
  std::vector<std::array<idx_t, 2>> edge_nodes;  // by global edge index
  std::vector<std::array<idx_t, 4>> cell_edges;  // global edge indices
  std::vector<std::array<int8_t, 4>> cell_ori;   // +1 / -1
  std::vector<int32_t> edge_num_cells;           // CountNumSuperEntities
  bool IsQuad(idx_t c) const { return cell_nodes[c][3] >= 0; }
  int NumVerts(idx_t c) const { return IsQuad(c) ? 4 : 3; }
  CellGeom Geom(idx_t c) const;
};
// hybrid2d::Mesh ctor: preset edges keep their registration index, edges
// created by cells are numbered afterwards in std::map (min,max) order; an
// edge's direction is that of its first creator.
Mesh BuildMesh(idx_t num_nodes, const double* xy, idx_t num_cells,
               const int64_t* cell_nodes /*4 per cell, -1 pad*/,
               idx_t num_preset, const int64_t* preset_edges /*2 per edge*/);

// Structured builders: lib/lf/mesh/utils/tp_triag_mesh_builder.cc:18-178 and
// tp_quad_mesh_builder.cc:18-94.  Return the factory input arrays.
struct FactoryInput {
  std::vector<double> xy;
  std::vector<int64_t> cells;   // 4 per cell
  std::vector<int64_t> edges;   // 2 per preset edge
};
FactoryInput TPTriagInput(idx_t nx, idx_t ny, double x0, double y0, double x1,
                          double y1);
FactoryInput TPQuadInput(idx_t nx, idx_t ny, double x0, double y0, double x1,
                         double y1);
// lib/lf/mesh/test_utils/test_meshes.cc:14 selector 0 (scale 1).
FactoryInput TestMesh0Input(double scale = 1.0);

// lib/lf/mesh/utils/special_entity_sets.cc:64-90 (all codims).
void FlagEntitiesOnBoundary(const Mesh& m, std::vector<uint8_t>& node_flags,
                            std::vector<uint8_t>& edge_flags);

// ------------------------------------------------------------- dof handler
// lib/lf/assemble/dofhandler.cc:86-338 (UniformFEDofHandler).
struct DofHandler {
  const Mesh* mesh = nullptr;
  int np = 0, ns = 0, nt = 0, nq = 0;  // interior dofs per point/seg/tria/quad
  int n_node = 0, n_edge = 0, n_tria = 0, n_quad = 0, n_cell = 0;
  idx_t num_dofs = 0;
  std::vector<idx_t> node_dofs, edge_dofs, cell_dofs;
  std::vector<std::pair<int, idx_t>> dof_entity;  // (codim, entity index)
  // Variable-degree hierarchic layout (DynamicFEDofHandler): per-cell local
  // dof counts and the per-entity degrees; empty for the uniform layouts.
  std::vector<int> nloc, edge_deg, cell_deg;
  int NumLocalDofs(idx_t c) const { return !nloc.empty() ? nloc[c] : mesh->IsQuad(c) ? n_quad : n_tria; }
  const idx_t* GlobalDofIndices(idx_t c) const { return &cell_dofs[c * n_cell]; }
};
DofHandler MakeDofHandler(const Mesh& m, int np, int ns, int nt, int nq,
                          bool check_edge_orientation = true);
// uniform_scalar_fe_space.h:241-342 for FeSpaceLagrangeO{1,2,3}.
DofHandler MakeLagrangeDofHandler(const Mesh& m, int degree);
// HierarchicScalarFESpace(mesh, degree_functor) (fe/hierarchic_scalar_fe_space.h:
// 93-116, Init :178-220) numbered by DynamicFEDofHandler (assemble/dofhandler.h:
// 550-680): one dof per node, edge_deg[e] - 1 per edge, the interior count of
// the cell's degree per cell; node dofs, then edge dofs, then cell dofs, each
// by entity index; a cell's local dofs are its vertices, per local edge the
// edge's dofs (reversed on a negatively oriented edge), then its interior.
DofHandler MakeHierVarDofHandler(const Mesh& m, const std::vector<int>& edge_deg, const std::vector<int>& cell_deg);

// ---------------------------------------------------------- mesh functions
// A scalar MeshFunction (mesh_function_traits.h:149-155) evaluated on a cell
// at reference points.  Kinds: constant (mesh_function_constant.h:25-45),
// per-cell array, O1 nodal interpolant (fe/mesh_function_fe.h:44-115),
// analytic x->f(x) (mesh_function_global.h:54-94), and exp of a per-cell
// array (a log-coefficient; no reference counterpart).
struct MeshFunction {
  enum Kind { kZero = 0, kConstant = 1, kPerCell = 2, kNodalO1 = 3, kAnalytic = 4, kPerCellExp = 5 };
  int kind = kZero;
  double value = 0.0;
  std::vector<double> data;
  std::function<double(double, double)> fn;
  // 2x2 tensor-valued diffusion coefficient (the matrix-valued DIFF_COEFF of
  // loc_comp_ellbvp.h:85-127): (cell, x, y) -> row-major a00, a01, a10, a11.
  // Set for the tensor kinds 6 (constant), 7 (per cell) and 8 (bilinear
  // entries), and by the reference's tensor-coefficient known answer.
  std::function<void(idx_t, double, double, double*)> tensor_fn;
  bool IsTensor() const { return static_cast<bool>(tensor_fn); }
  void Eval(const Mesh& m, idx_t cell, const QuadRule& qr,
            std::vector<double>& out) const;
  void EvalTensor(const Mesh& m, idx_t cell, const QuadRule& qr,
                  std::vector<std::array<double, 4>>& out) const;
};

// Built-in analytic families (shared meaning with the library's lfg_coeff).
std::function<double(double, double)> AnalyticFunction(int func_id,
                                                       const double* p);

// ---------------------------------------------------------------- assembly
struct Triplet {
  int32_t row, col;
  double value;
};
// lib/lf/assemble/coomatrix.h:51-225.
struct COOMatrix {
  idx_t rows = 0, cols = 0;
  std::vector<Triplet> triplets;
  void AddToEntry(idx_t i, idx_t j, double v) {
    triplets.push_back({static_cast<int32_t>(i), static_cast<int32_t>(j), v});
  }
};

// ReactionDiffusionElementMatrixProvider (uscalfe/loc_comp_ellbvp.h:85-339).
struct RDProvider {
  const Mesh* mesh;
  int degree;
  MeshFunction alpha, gamma;
  QuadRule qr_tria, qr_quad;
  bool have_tria = false, have_quad = false;
  // per-rule precomputed shape function tables (precomputed_scalar_...h:72-78)
  std::vector<double> phi_t, dphi_t, phi_q, dphi_q;
  void Init();
  void Eval(idx_t cell, std::vector<double>& mat /* n*n row major */) const;
};
// ScalarLoadElementVectorProvider (loc_comp_ellbvp.h:562-746).
struct LoadProvider {
  const Mesh* mesh;
  int degree;
  MeshFunction f;
  QuadRule qr_tria, qr_quad;
  std::vector<double> phi_t, phi_q;
  void Init();
  void Eval(idx_t cell, std::vector<double>& vec) const;
};

// AssembleMatrixLocally / AssembleVectorLocally (assemble/assembler.h:114-365).
void AssembleMatrixLocally(const DofHandler& dh,
                           const std::function<void(idx_t, std::vector<double>&)>& eval,
                           COOMatrix& A);

// ------------------------------------------------- boundary-edge providers
// FeLagrangeO{1,2,3}Segment shape functions (lagr_fe.h:284, 563-700, 1155-1277).
void EvalSegmentShape(int degree, double t, double* phi);
// A MeshFunction on edge e at segment parameters t (SegmentO1: x = p0 + t (p1 - p0)
// with (p0, p1) the edge's endpoints in edge direction).  Per-cell data is
// indexed by edge here; the O1 nodal interpolant restricts to the edge.
void EvalOnEdge(const MeshFunction& f, const Mesh& m, idx_t e, const std::vector<double>& t,
                std::vector<double>& out);
// AssembleMatrixLocally(1, dh, dh, MassEdgeMatrixProvider(fes, gamma, selector), A)
// (assembler.h:114-186 with codim 1; loc_comp_ellbvp.h:367-529): edges in index
// order, active iff flags[e] (all when flags is null), A_e = sum_k w_k |e|
// gamma(x_k) phi_k phi_k^T on the Gauss rule of degree qdeg.
void AssembleEdgeMass(const DofHandler& dh, int degree, const MeshFunction& gamma, const uint8_t* flags, int qdeg,
                      COOMatrix& A);
// AssembleVectorLocally(1, dh, ScalarLoadEdgeVectorProvider(fes, g, selector), b)
// (assembler.h:298-327; loc_comp_ellbvp.h:784-921): b[dof_i] += sum_k w_k |e| g(x_k) phi_i(t_k).
void AssembleEdgeLoad(const DofHandler& dh, int degree, const MeshFunction& g, const uint8_t* flags, int qdeg,
                      std::vector<double>& b);
void AssembleVectorLocally(const DofHandler& dh,
                           const std::function<void(idx_t, std::vector<double>&)>& eval,
                           std::vector<double>& b);

// FixFlaggedSolutionComponents (assemble/fix_dof.h:86-138).
void FixFlaggedSolutionComponents(const uint8_t* flags, const double* values,
                                  COOMatrix& A, std::vector<double>& b);
// FixFlaggedSolutionCompAlt (fix_dof.h:183-219).
void FixFlaggedSolutionCompAlt(const uint8_t* flags, const double* values,
                               COOMatrix& A, std::vector<double>& b);
// FixSolutionComponentsLse (fix_dof.h:250-280): (dof, value) pairs; repeated
// dofs accumulate their values in list order; then FixFlaggedSolutionCompAlt.
void FixSolutionComponentsLse(const std::vector<std::pair<idx_t, double>>& fixed, COOMatrix& A,
                              std::vector<double>& b);

// COOMatrix::makeSparse (coomatrix.h:172-180) = Eigen setFromTriplets: per
// (row,col) the duplicates are summed in triplet order.  Output is CSR.
void MakeSparseCSR(const COOMatrix& A, std::vector<int64_t>& rowptr,
                   std::vector<int32_t>& colind, std::vector<double>& val);

// fe/fe_tools.h:198-259 NodalProjection for Lagrangian spaces.
void NodalProjection(const DofHandler& dh, int degree,
                     const std::function<double(double, double)>& u,
                     std::vector<double>& out);

// ------------------------------------------------------ post-processing ----
// Gauss-Jacobi points/weights for alpha = 1, beta = 0 on [-1, 1]
// (quad/gauss_quadrature.cc:71-196).
void GaussJacobi10(int n, std::vector<double>& pts, std::vector<double>& wts);
// Exact gradient of a built-in analytic function (out[0], out[1]).
std::function<void(double, double, double*)> AnalyticGradient(int func_id, const double* p);

// The integrands the GPU library offers in closed form, over a mesh function
// u (with its gradient) and an FE function u_h = MeshFunctionFE(dh, dofs)
// (dofs null: u_h = 0):
//   kind 0: u_h + u            kind 1: (u_h - u)^2 (squaredNorm(mf_fe - mf_u))
//   kind 2: |grad u_h - grad u|^2 (squaredNorm(mf_grad_fe - mf_grad_u))
struct Integrand {
  int kind = 0;
  MeshFunction u;
  std::function<void(double, double, double*)> grad_u;  // analytic u only
  const DofHandler* dh = nullptr;
  int degree = 0;
  const double* dofs = nullptr;
  // u_h on a hierarchic space: its uniform degree, or 0 for per-entity
  // degrees (-1: Lagrangian of `degree`)
  int hier = -1;
};
// IntegrateMeshFunction (fe/fe_tools.h:110-165) with make_QuadRule(., qdeg)
// per reference element; flags select entities of the given codim (null:
// all).  As in the reference, entity 0 is always counted.
double IntegrateMeshFunction(const Mesh& m, const Integrand& g, int qdeg, const uint8_t* flags, int codim);
// MeshFunctionFE / MeshFunctionGradFE (fe/mesh_function_fe.h:72-91,
// fe/mesh_function_grad_fe.h:93-118) on one cell at reference points xy.
void EvalFE(const DofHandler& dh, int degree, const double* dofs, idx_t cell, const std::vector<double>& xy,
            double* vals, double* grads);
// The same with u_h on a hierarchic space (uniform degree p, 0: per entity).
void EvalFEHier(const DofHandler& dh, int p, const double* dofs, idx_t cell, const std::vector<double>& xy,
                double* vals, double* grads);
// NodalProjection (fe/fe_tools.h:198-259) of a mesh function, cells selected
// by flags (null: all); a dof shared by cells gets the last cell's value.
void NodalProjectionMF(const DofHandler& dh, int degree, const MeshFunction& u, const uint8_t* cell_flags,
                       std::vector<double>& out);
// InitEssentialConditionFromFunction (fe/fe_tools.h:263-329) over the edges
// selected by edge_flags.
void InitEssentialCondition(const DofHandler& dh, int degree, const uint8_t* edge_flags, const MeshFunction& g,
                            std::vector<uint8_t>& flags, std::vector<double>& vals);

// ------------------------------------------------ hierarchic (hp) FE ----
// fe/hierarchic_fe.cc: scaled Legendre and (integrated) Jacobi polynomials.
double HierLegendre(unsigned n, double x, double t = 1.0);
double HierILegendre(unsigned n, double x, double t = 1.0);
double HierILegendreDx(unsigned n, double x, double t = 1.0);
double HierILegendreDt(unsigned n, double x, double t = 1.0);
double HierJacobi(unsigned n, double alpha, double beta, double x);
double HierIJacobi(unsigned n, double alpha, double x);
// FeHierarchicTria / FeHierarchicQuad (fe/hierarchic_fe.h:473-1680) of
// uniform degree p with the cell's relative edge orientations ori[j] = +1/-1.
void EvalHierShape(bool is_quad, int p, const int8_t* ori, double x, double y, double* phi, double (*dphi)[2]);
// The same with the interior degree pc and per-edge degrees pe[j]
// (FeHierarchicTria(interior_degree, edge_degrees, ...), hierarchic_fe.h:482-501,
// and FeHierarchicQuad, :1150-1170): 3 or 4 vertex functions, pe[j] - 1
// functions per local edge, then the interior functions of degree pc.
void EvalHierShapeVar(bool is_quad, int pc, const int* pe, const int8_t* ori, double x, double y, double* phi,
                      double (*dphi)[2]);
int HierNumShapeVar(bool is_quad, int pc, const int* pe);
// fe::DiffusionElementMatrixProvider + fe::MassElementMatrixProvider
// (fe/loc_comp_ellbvp.h:169-214, 349-378; rule degree 2p) summed, assembled
// over a HierarchicScalarFESpace of uniform degree p (dh from
// MakeDofHandler(m, 1, p-1, ...)); fe::ScalarLoadElementVectorProvider
// (:642-685).  qdeg 0 = 2p.  On a variable-degree space (dh.cell_deg not
// empty) p is ignored: each cell uses its own degrees and, for qdeg 0, the
// rule of degree 2 max(pc, pe[j], 1) (2 * Degree(), loc_comp_ellbvp.h:186).
void AssembleHierMatrix(const DofHandler& dh, int p, const MeshFunction& alpha, const MeshFunction& gamma,
                        int qdeg, COOMatrix& A);
// EvaluationNodes / NodalValuesToDofs of FeHierarchicTria / FeHierarchicQuad
// (hierarchic_fe.h:820-1083, 1445-1665) for interior degree pc, edge degrees
// pe and relative orientations ori; and fe::NodalProjection (fe_tools.h:
// 198-259) on a hierarchic space (p: the uniform degree, or 0 for a
// variable-degree dof handler): a shared dof takes the last selected cell's
// value.
void HierEvaluationNodes(bool is_quad, int pc, const int* pe, const int8_t* ori, std::vector<double>& xy);
void HierNodalValuesToDofs(bool is_quad, int pc, const int* pe, const int8_t* ori, const std::vector<double>& v,
                           std::vector<double>& dofs);
void NodalProjectionHier(const DofHandler& dh, int p, const MeshFunction& u, const uint8_t* cell_flags,
                         std::vector<double>& out);
void AssembleHierLoad(const DofHandler& dh, int p, const MeshFunction& f, int qdeg, std::vector<double>& b);

}  // namespace lfo
