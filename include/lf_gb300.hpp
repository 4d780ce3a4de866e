// C++ facade over the C-ABI in lfg.h, shaped like the lf::assemble API that a
// LehrFEM++ driver calls for the assembly-and-solve path.  Header only; link
// with liblfg.so.  All matrices and vectors live in device memory.
//
//   reference (LehrFEM++)                          facade (this header)
//   mesh::utils::TPTriagMeshBuilder / TPQuad...    mesh::TPTriagMeshBuilder / TPQuadMeshBuilder
//     (mesh/utils/tp_triag_mesh_builder.h:25,        (same setter names, Build() -> shared_ptr<Mesh>)
//      tp_quad_mesh_builder.h:18)
//   mesh::hybrid2d::MeshFactory + Build            mesh::Mesh::FromCells (nodes, cells, preset edges)
//   uscalfe::FeSpaceLagrangeO{1,2,3}               uscalfe::FeSpaceLagrangeO<P> (P = 1, 2, 3)
//     (uscalfe/fe_space_lagrange_o{1,2,3}.h)
//   MeshFunctionConstant / per-cell / FE / Global  uscalfe::MeshFunction::{Constant, PerCell,
//                                                    PerCellExp, NodalO1, Analytic}
//   ReactionDiffusionElementMatrixProvider         uscalfe::ReactionDiffusionElementMatrixProvider
//     (uscalfe/loc_comp_ellbvp.h:87-160)             (space, alpha, gamma[, rule degrees])
//   ScalarLoadElementVectorProvider                uscalfe::ScalarLoadElementVectorProvider
//     (uscalfe/loc_comp_ellbvp.h:558-600)
//   assemble::COOMatrix (assemble/coomatrix.h:52)  assemble::COOMatrix (rows, cols, AddToEntry,
//                                                    setZero, triplets, makeSparse)
//   assemble::AssembleMatrixLocally                assemble::AssembleMatrixLocally(0, dofh, dofh,
//     (assemble/assembler.h:115)                     provider, A)
//   assemble::AssembleVectorLocally (:299)         assemble::AssembleVectorLocally(0, dofh, provider, b)
//   assemble::FixFlaggedSolutionComponents         assemble::FixFlaggedSolutionComponents(flags,
//     (assemble/fix_dof.h:87)                        values, A, b): the selector is given as two
//                                                    device arrays (flag, value per dof)
//   assemble::FixFlaggedSolutionCompAlt (:184),    the same names; FixSolutionComponentsLse takes
//   assemble::FixSolutionComponentsLse (:251)        fixed_components_t (host (dof, value) pairs)
//   Eigen::SparseLU / CG on makeSparse()           solve::SolvePCG (Jacobi PCG, FP64 or mixed)
//   MassEdgeMatrixProvider, ScalarLoadEdgeVectorProvider (loc_comp_ellbvp.h:367-529,
//     784-921) with AssembleMatrixLocally / AssembleVectorLocally(1, ...)
//                                                  the same names; edge selector = device flags
//   fe::MeshFunctionFE / MeshFunctionGradFE        fe::MeshFunctionFE / fe::MeshFunctionGradFE
//     (fe/mesh_function_fe.h:44, mesh_function_grad_fe.h:44)  (space + device dof vector; evaluated on
//                                                    every cell at shared reference points)
//   fe::IntegrateMeshFunction(mesh, squaredNorm(   fe::IntegrateMeshFunction(mesh, fe::SquaredNormDiff(
//     mf_fe - mf_u), degree) (fe/fe_tools.h:158)     mf_fe, u), degree[, pred, codim]) and the other
//                                                    closed integrands (fe::Value, fe::SquaredNorm)
//   fe::NodalProjection (fe/fe_tools.h:198)        fe::NodalProjection(fes, u[, pred])
//   fe::InitEssentialConditionFromFunction         fe::InitEssentialConditionFromFunction(fes, edge
//     (fe/fe_tools.h:263)                            flags, g) -> (flags, values) device vectors
//   fe::HierarchicScalarFESpace(mesh, degree)      fe::HierarchicScalarFESpace(mesh, degree) (uniform degree)
//     (fe/hierarchic_scalar_fe_space.h:36)           and (mesh, degree_functor) with degree_functor(
//   fe::HierarchicScalarFESpace(mesh, functor)       mesh::EntityRef{codim, index}) per edge and cell
//     (fe/hierarchic_scalar_fe_space.h:93)
//   fe::DiffusionElementMatrixProvider,            fe::DiffusionElementMatrixProvider,
//   fe::MassElementMatrixProvider,                 fe::MassElementMatrixProvider,
//   fe::ScalarLoadElementVectorProvider            fe::ScalarLoadElementVectorProvider (on a hierarchic
//     (fe/loc_comp_ellbvp.h:76-700)                  space; the assemble:: functions take them)
//   io::GmshReader(factory, filename)              io::GmshReader(ctx, filename): mesh(),
//     (io/gmsh_reader.h)                             PhysicalEntityNr, IsPhysicalEntity,
//                                                    PhysicalEntityName2Nr / Nr2Name,
//                                                    PhysicalEntities (+ device flags per group)
//   (no counterpart)                               adjoint::InverseConductivityFunction
//
// Errors: every failing call throws lf::gb300::Error carrying the lfg_status
// code and the library's message (the reference throws or asserts likewise).
#pragma once

#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "lfg.h"

namespace lf::gb300 {

class Error : public std::runtime_error {
 public:
  Error(lfg_status code, const std::string& msg) : std::runtime_error(msg), code_(code) {}
  lfg_status code() const { return code_; }

 private:
  lfg_status code_;
};

class Context {
 public:
  explicit Context(int device = 0) {
    lfg_ctx* h = nullptr;
    const lfg_status st = lfg_ctx_create(device, &h);
    if (st != LFG_OK) throw Error(st, "lfg_ctx_create failed");
    h_ = h;
  }
  ~Context() {
    if (h_) lfg_ctx_destroy(h_);
  }
  Context(const Context&) = delete;
  Context& operator=(const Context&) = delete;
  lfg_ctx* get() const { return h_; }
  void Check(lfg_status st) const {
    if (st != LFG_OK) throw Error(st, lfg_ctx_last_error(h_));
  }
  void Synchronize() const { Check(lfg_ctx_synchronize(h_)); }

 private:
  lfg_ctx* h_ = nullptr;
};

// Device array of n elements of T.
template <class T>
class DeviceVector {
 public:
  DeviceVector(const Context& ctx, size_t n) : ctx_(&ctx), n_(n) {
    void* p = nullptr;
    ctx.Check(lfg_malloc(ctx.get(), (n ? n : 1) * sizeof(T), &p));
    p_ = static_cast<T*>(p);
  }
  DeviceVector(const Context& ctx, const std::vector<T>& host) : DeviceVector(ctx, host.size()) { Upload(host); }
  ~DeviceVector() {
    if (p_) lfg_free(ctx_->get(), p_);
  }
  DeviceVector(DeviceVector&& o) noexcept : ctx_(o.ctx_), p_(o.p_), n_(o.n_) { o.p_ = nullptr; }
  DeviceVector(const DeviceVector&) = delete;
  DeviceVector& operator=(const DeviceVector&) = delete;
  T* data() { return p_; }
  const T* data() const { return p_; }
  size_t size() const { return n_; }
  void Upload(const std::vector<T>& h) {
    if (h.size() != n_) throw Error(LFG_INVALID_ARG, "DeviceVector::Upload: size mismatch");
    ctx_->Check(lfg_memcpy_h2d(ctx_->get(), p_, h.data(), n_ * sizeof(T)));
    ctx_->Synchronize();
  }
  std::vector<T> Download() const {
    std::vector<T> h(n_);
    ctx_->Check(lfg_memcpy_d2h(ctx_->get(), h.data(), p_, n_ * sizeof(T)));
    return h;
  }
  void SetZero() { ctx_->Check(lfg_memset(ctx_->get(), p_, 0, n_ * sizeof(T))); }

 private:
  const Context* ctx_;
  T* p_ = nullptr;
  size_t n_ = 0;
};

namespace mesh {

class Mesh {
 public:
  // hybrid2d::MeshFactory input: nodes (x, y), cells (4 node indices, -1 in
  // the last slot for triangles), optional preset edges (2 node indices).
  static std::shared_ptr<Mesh> FromCells(const Context& ctx, const std::vector<double>& xy,
                                         const std::vector<int32_t>& cells,
                                         const std::vector<int32_t>& preset_edges = {}) {
    lfg_mesh* h = nullptr;
    ctx.Check(lfg_mesh_create(ctx.get(), static_cast<int64_t>(xy.size() / 2), xy.data(),
                              static_cast<int64_t>(cells.size() / 4), cells.data(),
                              static_cast<int64_t>(preset_edges.size() / 2),
                              preset_edges.empty() ? nullptr : preset_edges.data(), &h));
    return std::shared_ptr<Mesh>(new Mesh(ctx, h));
  }
  static std::shared_ptr<Mesh> Adopt(const Context& ctx, lfg_mesh* h) { return std::shared_ptr<Mesh>(new Mesh(ctx, h)); }
  ~Mesh() { lfg_mesh_destroy(h_); }
  Mesh(const Mesh&) = delete;
  Mesh& operator=(const Mesh&) = delete;
  // NumEntities(codim): 0 cells, 1 edges, 2 nodes.
  int64_t NumEntities(int codim) const {
    int64_t nv = 0, ne = 0, nc = 0, nt = 0, nq = 0;
    ctx_->Check(lfg_mesh_sizes(h_, &nv, &ne, &nc, &nt, &nq));
    return codim == 0 ? nc : codim == 1 ? ne : nv;
  }
  lfg_mesh* get() const { return h_; }
  const Context& ctx() const { return *ctx_; }

 private:
  Mesh(const Context& ctx, lfg_mesh* h) : ctx_(&ctx), h_(h) {}
  const Context* ctx_;
  lfg_mesh* h_;
};

// Structured builders with the reference's setters (corners, cell counts).
template <bool QUAD>
class TPMeshBuilder {
 public:
  explicit TPMeshBuilder(const Context& ctx) : ctx_(&ctx) {}
  TPMeshBuilder& setBottomLeftCorner(double x, double y) { x0_ = x; y0_ = y; return *this; }
  TPMeshBuilder& setTopRightCorner(double x, double y) { x1_ = x; y1_ = y; return *this; }
  TPMeshBuilder& setNumXCells(int64_t n) { nx_ = n; return *this; }
  TPMeshBuilder& setNumYCells(int64_t n) { ny_ = n; return *this; }
  std::shared_ptr<Mesh> Build() const {
    lfg_mesh* h = nullptr;
    ctx_->Check(QUAD ? lfg_mesh_create_tp_quad(ctx_->get(), nx_, ny_, x0_, y0_, x1_, y1_, &h)
                     : lfg_mesh_create_tp_triag(ctx_->get(), nx_, ny_, x0_, y0_, x1_, y1_, &h));
    return Mesh::Adopt(*ctx_, h);
  }

 private:
  const Context* ctx_;
  double x0_ = 0, y0_ = 0, x1_ = 1, y1_ = 1;
  int64_t nx_ = 1, ny_ = 1;
};
using TPTriagMeshBuilder = TPMeshBuilder<false>;
using TPQuadMeshBuilder = TPMeshBuilder<true>;

// An entity named by codimension (0 cell, 1 edge, 2 node) and index: what a
// degree functor receives (the reference passes const lf::mesh::Entity&).
struct EntityRef {
  int codim;
  int64_t index;
  int Codim() const { return codim; }
};

}  // namespace mesh

namespace uscalfe {

// Lagrangian FE space of degree P on a mesh; it is its own DofHandler.
class FeSpaceLagrange {
 public:
  FeSpaceLagrange(std::shared_ptr<const mesh::Mesh> m, int degree, bool hierarchic = false) : mesh_(std::move(m)) {
    lfg_space* h = nullptr;
    mesh_->ctx().Check(hierarchic ? lfg_space_create_hierarchic(mesh_->get(), degree, &h)
                                  : lfg_space_create_lagrange(mesh_->get(), degree, &h));
    h_ = h;
  }
  // Hierarchic space with a degree per edge (edge order) and per cell (cell order).
  FeSpaceLagrange(std::shared_ptr<const mesh::Mesh> m, const std::vector<int32_t>& edge_degree,
                  const std::vector<int32_t>& cell_degree)
      : mesh_(std::move(m)) {
    lfg_space* h = nullptr;
    mesh_->ctx().Check(lfg_space_create_hierarchic_var(mesh_->get(), edge_degree.data(), cell_degree.data(), &h));
    h_ = h;
  }
  ~FeSpaceLagrange() { lfg_space_destroy(h_); }
  FeSpaceLagrange(const FeSpaceLagrange&) = delete;
  FeSpaceLagrange& operator=(const FeSpaceLagrange&) = delete;
  int64_t NumDofs() const {
    int64_t nd = 0, nt = 0;
    int32_t a = 0, b = 0, c = 0;
    mesh_->ctx().Check(lfg_space_info(h_, &nd, &a, &b, &c, &nt));
    return nd;
  }
  int64_t NumTriplets() const {
    int64_t nd = 0, nt = 0;
    int32_t a = 0, b = 0, c = 0;
    mesh_->ctx().Check(lfg_space_info(h_, &nd, &a, &b, &c, &nt));
    return nt;
  }
  const FeSpaceLagrange& LocGlobMap() const { return *this; }
  std::shared_ptr<const mesh::Mesh> Mesh() const { return mesh_; }
  lfg_space* get() const { return h_; }
  const Context& ctx() const { return mesh_->ctx(); }
  // Boundary dof flags (flagEntitiesOnBoundary + dof entity lookup).
  DeviceVector<uint8_t> BoundaryDofFlags() const {
    DeviceVector<uint8_t> f(ctx(), static_cast<size_t>(NumDofs()));
    ctx().Check(lfg_space_boundary_dof_flags(h_, f.data()));
    return f;
  }

 private:
  std::shared_ptr<const mesh::Mesh> mesh_;
  lfg_space* h_ = nullptr;
};

template <int P>
std::shared_ptr<FeSpaceLagrange> FeSpaceLagrangeO(std::shared_ptr<const mesh::Mesh> m) {
  static_assert(P >= 1 && P <= 3, "Lagrangian degrees 1, 2, 3");
  return std::make_shared<FeSpaceLagrange>(std::move(m), P);
}

// Scalar coefficient descriptors (device data is referenced, not copied).
struct MeshFunction {
  lfg_coeff c{};
  static MeshFunction Zero() { return {}; }
  static MeshFunction Constant(double v) {
    MeshFunction f;
    f.c.kind = LFG_COEFF_CONSTANT;
    f.c.value = v;
    return f;
  }
  static MeshFunction PerCell(const double* dev) { return Data(LFG_COEFF_PER_CELL, dev); }
  static MeshFunction PerCellExp(const double* dev) { return Data(LFG_COEFF_PER_CELL_EXP, dev); }
  static MeshFunction NodalO1(const double* dev) { return Data(LFG_COEFF_NODAL_O1, dev); }
  static MeshFunction Analytic(int fn, const std::vector<double>& params) {  // LFG_FN_*
    MeshFunction f;
    f.c.kind = LFG_COEFF_ANALYTIC;
    f.c.func = fn;
    for (size_t i = 0; i < params.size() && i < 16; ++i) f.c.p[i] = params[i];
    return f;
  }

 private:
  static MeshFunction Data(int kind, const double* dev) {
    MeshFunction f;
    f.c.kind = kind;
    f.c.data_dev = dev;
    return f;
  }
};

class ReactionDiffusionElementMatrixProvider {
 public:
  // Rule degrees: 0 = the reference's default (2 * degree); per cell type.
  ReactionDiffusionElementMatrixProvider(std::shared_ptr<const FeSpaceLagrange> fes, MeshFunction alpha,
                                         MeshFunction gamma, int qr_degree_tria = 0, int qr_degree_quad = 0)
      : fes_(std::move(fes)) {
    p_.alpha = alpha.c;
    p_.gamma = gamma.c;
    p_.qr_degree_tria = qr_degree_tria;
    p_.qr_degree_quad = qr_degree_quad;
  }
  const lfg_rd_provider* get() const { return &p_; }

 private:
  std::shared_ptr<const FeSpaceLagrange> fes_;
  lfg_rd_provider p_{};
};

class ScalarLoadElementVectorProvider {
 public:
  ScalarLoadElementVectorProvider(std::shared_ptr<const FeSpaceLagrange> fes, MeshFunction f,
                                  int qr_degree_tria = 0, int qr_degree_quad = 0)
      : fes_(std::move(fes)) {
    p_.f = f.c;
    p_.qr_degree_tria = qr_degree_tria;
    p_.qr_degree_quad = qr_degree_quad;
  }
  const lfg_load_provider* get() const { return &p_; }

 private:
  std::shared_ptr<const FeSpaceLagrange> fes_;
  lfg_load_provider p_{};
};

// Boundary-edge providers (loc_comp_ellbvp.h:367-529, 784-921).  The edge
// selector is a device flag array (nullptr: every edge); per-cell coefficient
// data is indexed by edge.
class MassEdgeMatrixProvider {
 public:
  MassEdgeMatrixProvider(std::shared_ptr<const FeSpaceLagrange> fes, MeshFunction gamma,
                         const uint8_t* edge_flags_dev = nullptr, int qr_degree = 0)
      : fes_(std::move(fes)) {
    p_.gamma = gamma.c;
    p_.edge_flags_dev = edge_flags_dev;
    p_.qr_degree = qr_degree;
  }
  const lfg_edge_mass_provider* get() const { return &p_; }

 private:
  std::shared_ptr<const FeSpaceLagrange> fes_;
  lfg_edge_mass_provider p_{};
};

class ScalarLoadEdgeVectorProvider {
 public:
  ScalarLoadEdgeVectorProvider(std::shared_ptr<const FeSpaceLagrange> fes, MeshFunction g,
                               const uint8_t* edge_flags_dev = nullptr, int qr_degree = 0)
      : fes_(std::move(fes)) {
    p_.g = g.c;
    p_.edge_flags_dev = edge_flags_dev;
    p_.qr_degree = qr_degree;
  }
  const lfg_edge_load_provider* get() const { return &p_; }

 private:
  std::shared_ptr<const FeSpaceLagrange> fes_;
  lfg_edge_load_provider p_{};
};

}  // namespace uscalfe

namespace solve {

struct SolveOptions {
  int precision = LFG_SOLVE_FP64;  // or LFG_SOLVE_MIXED
  int max_iterations = 0;  // 0: library default
  double rtol = 1e-10;
  double inner_rtol = 1e-4;
  int check_every = 32;
};

class CSRMatrix {
 public:
  CSRMatrix(const Context& ctx, lfg_csr* h) : ctx_(&ctx), h_(h) {}
  ~CSRMatrix() {
    if (h_) lfg_csr_destroy(h_);
  }
  CSRMatrix(CSRMatrix&& o) noexcept : ctx_(o.ctx_), h_(o.h_) { o.h_ = nullptr; }
  CSRMatrix(const CSRMatrix&) = delete;
  CSRMatrix& operator=(const CSRMatrix&) = delete;
  lfg_csr* get() const { return h_; }
  int64_t nonZeros() const {
    int64_t r = 0, c = 0, nnz = 0;
    ctx_->Check(lfg_csr_info(h_, &r, &c, &nnz));
    return nnz;
  }

 private:
  const Context* ctx_;
  lfg_csr* h_;
};

// Jacobi PCG on a symmetric positive definite CSR matrix; x is the start
// vector and the result.  Throws on non-convergence (LFG_NOT_CONVERGED).
inline lfg_solve_stats SolvePCG(const Context& ctx, const CSRMatrix& A, const DeviceVector<double>& b,
                                DeviceVector<double>& x, const SolveOptions& o = {}) {
  lfg_solve_opts so{};
  so.precision = o.precision;
  so.max_iterations = o.max_iterations;
  so.rtol = o.rtol;
  so.inner_rtol = o.inner_rtol;
  so.check_every = o.check_every;
  lfg_solve_stats st{};
  ctx.Check(lfg_solve_pcg(A.get(), b.data(), x.data(), &so, &st));
  return st;
}

}  // namespace solve

namespace assemble {

using dim_t = unsigned int;

class COOMatrix {
 public:
  // capacity: triplets the device buffer holds (assembly appends n_K^2 per
  // cell; FixFlaggedSolutionComponents may append one per flagged dof).
  COOMatrix(const Context& ctx, int64_t rows, int64_t cols, int64_t capacity) : ctx_(&ctx), rows_(rows), cols_(cols) {
    ctx.Check(lfg_coo_create(ctx.get(), rows, cols, capacity, &h_));
  }
  ~COOMatrix() {
    if (h_) lfg_coo_destroy(h_);
  }
  COOMatrix(const COOMatrix&) = delete;
  COOMatrix& operator=(const COOMatrix&) = delete;
  int64_t rows() const { return rows_; }
  int64_t cols() const { return cols_; }
  void AddToEntry(int32_t i, int32_t j, double increment) {
    const lfg_triplet t{i, j, increment};
    ctx_->Check(lfg_coo_append_host(h_, &t, 1));
  }
  void setZero() { ctx_->Check(lfg_coo_set_zero(h_)); }
  int64_t size() const {
    int64_t n = 0;
    ctx_->Check(lfg_coo_size(h_, &n));
    return n;
  }
  // Device pointer to the triplets (row, col, value) in insertion order.
  const lfg_triplet* triplets() const {
    lfg_triplet* p = nullptr;
    ctx_->Check(lfg_coo_triplets(h_, &p));
    return p;
  }
  std::vector<lfg_triplet> Download() const {
    std::vector<lfg_triplet> t(static_cast<size_t>(size()));
    if (!t.empty()) ctx_->Check(lfg_coo_download(h_, t.data(), static_cast<int64_t>(t.size())));
    return t;
  }
  solve::CSRMatrix makeSparse() const {
    lfg_csr* c = nullptr;
    ctx_->Check(lfg_csr_from_coo(h_, &c));
    return solve::CSRMatrix(*ctx_, c);
  }
  lfg_coo* get() const { return h_; }
  const Context& ctx() const { return *ctx_; }

 private:
  const Context* ctx_;
  int64_t rows_, cols_;
  lfg_coo* h_ = nullptr;
};

// Cells only (codim 0): the element providers of this path have no edge or
// node contributions.  Trial and test spaces must be the same object.
inline void AssembleMatrixLocally(dim_t codim, const uscalfe::FeSpaceLagrange& trial,
                                  const uscalfe::FeSpaceLagrange& test,
                                  const uscalfe::ReactionDiffusionElementMatrixProvider& provider, COOMatrix& A) {
  if (codim != 0 || &trial != &test)
    throw Error(LFG_UNSUPPORTED, "AssembleMatrixLocally: cells of one space only");
  trial.ctx().Check(lfg_assemble_matrix_rd(trial.get(), provider.get(), A.get()));
}

inline void AssembleVectorLocally(dim_t codim, const uscalfe::FeSpaceLagrange& dofh,
                                  const uscalfe::ScalarLoadElementVectorProvider& provider,
                                  DeviceVector<double>& b) {
  if (codim != 0) throw Error(LFG_UNSUPPORTED, "AssembleVectorLocally: cells only");
  dofh.ctx().Check(lfg_assemble_vector_load(dofh.get(), provider.get(), b.data()));
}

// Codim 1: the boundary-edge providers.
inline void AssembleMatrixLocally(dim_t codim, const uscalfe::FeSpaceLagrange& trial,
                                  const uscalfe::FeSpaceLagrange& test,
                                  const uscalfe::MassEdgeMatrixProvider& provider, COOMatrix& A) {
  if (codim != 1 || &trial != &test)
    throw Error(LFG_UNSUPPORTED, "AssembleMatrixLocally: edge providers act on codim 1 of one space");
  trial.ctx().Check(lfg_assemble_matrix_edge_mass(trial.get(), provider.get(), A.get()));
}

inline void AssembleVectorLocally(dim_t codim, const uscalfe::FeSpaceLagrange& dofh,
                                  const uscalfe::ScalarLoadEdgeVectorProvider& provider,
                                  DeviceVector<double>& b) {
  if (codim != 1) throw Error(LFG_UNSUPPORTED, "AssembleVectorLocally: edge providers act on codim 1");
  dofh.ctx().Check(lfg_assemble_vector_edge_load(dofh.get(), provider.get(), b.data()));
}

inline void FixFlaggedSolutionComponents(const DeviceVector<uint8_t>& flags, const DeviceVector<double>& values,
                                         COOMatrix& A, DeviceVector<double>& b) {
  const lfg_status st = lfg_fix_flagged_solution_components(A.get(), flags.data(), values.data(), b.data());
  if (st != LFG_OK) throw Error(st, "FixFlaggedSolutionComponents failed");
}

// FixFlaggedSolutionCompAlt (assemble/fix_dof.h:183-219): only the fixed rows
// are removed.
inline void FixFlaggedSolutionCompAlt(const DeviceVector<uint8_t>& flags, const DeviceVector<double>& values,
                                      COOMatrix& A, DeviceVector<double>& b) {
  const lfg_status st = lfg_fix_flagged_solution_comp_alt(A.get(), flags.data(), values.data(), b.data());
  if (st != LFG_OK) throw Error(st, "FixFlaggedSolutionCompAlt failed");
}

// fixed_components_t / FixSolutionComponentsLse (assemble/fix_dof.h:228-280):
// (dof, value) pairs; a repeated dof is fixed to the sum of its values.
template <typename SCALAR>
using fixed_components_t = std::vector<std::pair<int64_t, SCALAR>>;

inline void FixSolutionComponentsLse(const fixed_components_t<double>& fixed_components, COOMatrix& A,
                                     DeviceVector<double>& b) {
  const Context& ctx = A.ctx();
  std::vector<int64_t> dofs;
  std::vector<double> vals;
  for (const auto& dv : fixed_components) {
    dofs.push_back(dv.first);
    vals.push_back(dv.second);
  }
  DeviceVector<int64_t> d(ctx, dofs);
  DeviceVector<double> v(ctx, vals);
  const lfg_status st = lfg_fix_solution_components_lse(A.get(), static_cast<int64_t>(dofs.size()), d.data(),
                                                        v.data(), b.data());
  if (st != LFG_OK) throw Error(st, "FixSolutionComponentsLse failed");
}

}  // namespace assemble

namespace fe {

// HierarchicScalarFESpace(mesh, degree): hierarchic (hp) shape functions of a
// uniform degree 1..20; the same space handle as the Lagrangian spaces.
inline std::shared_ptr<uscalfe::FeSpaceLagrange> HierarchicScalarFESpace(std::shared_ptr<const mesh::Mesh> m,
                                                                        int degree) {
  return std::make_shared<uscalfe::FeSpaceLagrange>(std::move(m), degree, true);
}
// HierarchicScalarFESpace(mesh, degree_functor) (fe/hierarchic_scalar_fe_space.h:
// 93-116): degree_functor(mesh::EntityRef) gives the degree (1..20) of every
// edge and every cell, each called once; dofs numbered like DynamicFEDofHandler.
template <class F, class = decltype(static_cast<int32_t>(std::declval<F&>()(std::declval<const mesh::EntityRef&>())))>
std::shared_ptr<uscalfe::FeSpaceLagrange> HierarchicScalarFESpace(std::shared_ptr<const mesh::Mesh> m,
                                                                 F&& degree_functor) {
  const int64_t ne = m->NumEntities(1), nc = m->NumEntities(0);
  std::vector<int32_t> ed(static_cast<size_t>(ne)), cd(static_cast<size_t>(nc));
  for (int64_t e = 0; e < ne; ++e) ed[e] = static_cast<int32_t>(degree_functor(mesh::EntityRef{1, e}));
  for (int64_t c = 0; c < nc; ++c) cd[c] = static_cast<int32_t>(degree_functor(mesh::EntityRef{0, c}));
  return std::make_shared<uscalfe::FeSpaceLagrange>(std::move(m), ed, cd);
}
// fe::DiffusionElementMatrixProvider(fe_space, alpha) and
// fe::MassElementMatrixProvider(fe_space, gamma) (fe/loc_comp_ellbvp.h:76,
// 256); rules make_QuadRule(ref_el, 2 * degree).
class DiffusionElementMatrixProvider : public uscalfe::ReactionDiffusionElementMatrixProvider {
 public:
  DiffusionElementMatrixProvider(std::shared_ptr<const uscalfe::FeSpaceLagrange> fes, uscalfe::MeshFunction alpha)
      : uscalfe::ReactionDiffusionElementMatrixProvider(std::move(fes), alpha, uscalfe::MeshFunction::Zero()) {}
};
class MassElementMatrixProvider : public uscalfe::ReactionDiffusionElementMatrixProvider {
 public:
  MassElementMatrixProvider(std::shared_ptr<const uscalfe::FeSpaceLagrange> fes, uscalfe::MeshFunction gamma)
      : uscalfe::ReactionDiffusionElementMatrixProvider(std::move(fes), uscalfe::MeshFunction::Zero(), gamma) {}
};
// fe::ScalarLoadElementVectorProvider (fe/loc_comp_ellbvp.h:569)
using ScalarLoadElementVectorProvider = uscalfe::ScalarLoadElementVectorProvider;

// An FE function u_h = sum_i dofs[i] b_i of a Lagrangian space; the dof
// vector is referenced and must outlive the mesh function.
class MeshFunctionFE {
 public:
  MeshFunctionFE(std::shared_ptr<const uscalfe::FeSpaceLagrange> fes, const DeviceVector<double>& dofs)
      : fes_(std::move(fes)), dofs_(&dofs) {}
  // Values on every cell at the reference points local_xy (x0, y0, x1, y1, ...):
  // result[cell * npts + k].
  DeviceVector<double> operator()(const std::vector<double>& local_xy) const {
    const int32_t np = static_cast<int32_t>(local_xy.size() / 2);
    DeviceVector<double> out(fes_->ctx(), static_cast<size_t>(fes_->Mesh()->NumEntities(0)) * np);
    fes_->ctx().Check(lfg_fe_eval(fes_->get(), dofs_->data(), np, local_xy.data(), out.data(), nullptr));
    return out;
  }
  const uscalfe::FeSpaceLagrange& space() const { return *fes_; }
  const DeviceVector<double>& dofs() const { return *dofs_; }

 private:
  std::shared_ptr<const uscalfe::FeSpaceLagrange> fes_;
  const DeviceVector<double>* dofs_;
};

class MeshFunctionGradFE {
 public:
  MeshFunctionGradFE(std::shared_ptr<const uscalfe::FeSpaceLagrange> fes, const DeviceVector<double>& dofs)
      : fe_(std::move(fes), dofs) {}
  // Gradients on every cell at the reference points: result[(cell * npts + k) * 2 + d].
  DeviceVector<double> operator()(const std::vector<double>& local_xy) const {
    const int32_t np = static_cast<int32_t>(local_xy.size() / 2);
    DeviceVector<double> out(fe_.space().ctx(), static_cast<size_t>(fe_.space().Mesh()->NumEntities(0)) * np * 2);
    fe_.space().ctx().Check(lfg_fe_eval(fe_.space().get(), fe_.dofs().data(), np, local_xy.data(), nullptr,
                                        out.data()));
    return out;
  }
  const MeshFunctionFE& function() const { return fe_; }

 private:
  MeshFunctionFE fe_;
};

// The integrands IntegrateMeshFunction evaluates on the device.
struct Integrand {
  lfg_integrand g{};
};
// u (a mesh function) and u_h + u
inline Integrand Value(uscalfe::MeshFunction u) {
  Integrand i;
  i.g.kind = LFG_INTEGRAND_VALUE;
  i.g.u = u.c;
  return i;
}
inline Integrand Value(const MeshFunctionFE& uh, uscalfe::MeshFunction u = uscalfe::MeshFunction::Zero()) {
  Integrand i = Value(u);
  i.g.space = uh.space().get();
  i.g.dofs_dev = uh.dofs().data();
  return i;
}
// squaredNorm(u), squaredNorm(mf_fe - mf_u), squaredNorm(mf_grad_fe - mf_grad_u)
inline Integrand SquaredNorm(uscalfe::MeshFunction u) {
  Integrand i;
  i.g.kind = LFG_INTEGRAND_SQ_DIFF;
  i.g.u = u.c;
  return i;
}
inline Integrand SquaredNormDiff(const MeshFunctionFE& uh, uscalfe::MeshFunction u) {
  Integrand i = SquaredNorm(u);
  i.g.space = uh.space().get();
  i.g.dofs_dev = uh.dofs().data();
  return i;
}
inline Integrand SquaredNormDiff(const MeshFunctionGradFE& gh, uscalfe::MeshFunction u) {
  Integrand i = SquaredNormDiff(gh.function(), u);
  i.g.kind = LFG_INTEGRAND_GRAD_SQ_DIFF;
  return i;
}
inline Integrand SquaredNorm(const MeshFunctionFE& uh) { return SquaredNormDiff(uh, uscalfe::MeshFunction::Zero()); }
inline Integrand SquaredNorm(const MeshFunctionGradFE& gh) {
  return SquaredNormDiff(gh, uscalfe::MeshFunction::Zero());
}

// IntegrateMeshFunction(mesh, mf, quad_degree, pred, codim) (fe/fe_tools.h:158).
inline double IntegrateMeshFunction(const mesh::Mesh& m, const Integrand& f, int quad_degree,
                                    const DeviceVector<uint8_t>* pred = nullptr, int codim = 0) {
  double r = 0.0;
  m.ctx().Check(lfg_integrate_mesh_function(m.get(), &f.g, quad_degree, pred ? pred->data() : nullptr, codim, &r));
  return r;
}

// NodalProjection(fe_space, u, pred) (fe/fe_tools.h:198-259), Lagrangian or
// hierarchic space.
inline DeviceVector<double> NodalProjection(const uscalfe::FeSpaceLagrange& fes, uscalfe::MeshFunction u,
                                            const DeviceVector<uint8_t>* pred = nullptr) {
  DeviceVector<double> out(fes.ctx(), static_cast<size_t>(fes.NumDofs()));
  fes.ctx().Check(lfg_nodal_projection(fes.get(), &u.c, pred ? pred->data() : nullptr, out.data()));
  return out;
}

// InitEssentialConditionFromFunction(fes, esscondflag, g) (fe/fe_tools.h:263-329):
// the (flag, value) pair per dof as two device vectors, ready for
// assemble::FixFlaggedSolutionComponents.
inline std::pair<DeviceVector<uint8_t>, DeviceVector<double>> InitEssentialConditionFromFunction(
    const uscalfe::FeSpaceLagrange& fes, const DeviceVector<uint8_t>& edge_flags, uscalfe::MeshFunction g) {
  const size_t nd = static_cast<size_t>(fes.NumDofs());
  std::pair<DeviceVector<uint8_t>, DeviceVector<double>> out{DeviceVector<uint8_t>(fes.ctx(), nd),
                                                             DeviceVector<double>(fes.ctx(), nd)};
  fes.ctx().Check(lfg_init_essential_condition(fes.get(), edge_flags.data(), &g.c, out.first.data(),
                                               out.second.data()));
  return out;
}

}  // namespace fe

namespace io {

// GmshReader for 2D first-order meshes (MSH 2.2 / 4.1, ASCII / binary).
class GmshReader {
 public:
  GmshReader(const Context& ctx, const std::string& filename) : ctx_(&ctx) {
    lfg_gmsh* g = nullptr;
    const lfg_status st = lfg_gmsh_open(filename.c_str(), &g);
    if (st != LFG_OK) throw Error(st, lfg_gmsh_last_error());
    g_.reset(g, [](lfg_gmsh* p) { lfg_gmsh_destroy(p); });
    lfg_mesh* m = nullptr;
    ctx.Check(lfg_gmsh_build_mesh(ctx.get(), g, &m));
    mesh_ = mesh::Mesh::Adopt(ctx, m);
  }
  std::shared_ptr<mesh::Mesh> mesh() const { return mesh_; }
  // PhysicalEntityNr(e) of entity `index` of `codim` (0 cells, 1 edges, 2 nodes).
  std::vector<int32_t> PhysicalEntityNr(int codim, int64_t index) const {
    const int64_t n = mesh_->NumEntities(codim);
    if (index < 0 || index >= n) throw Error(LFG_INVALID_ARG, "GmshReader::PhysicalEntityNr: index out of range");
    std::vector<int64_t> off(static_cast<size_t>(n) + 1);
    Check(lfg_gmsh_physical_entity_nrs(g_.get(), codim, n, off.data(), nullptr));
    std::vector<int32_t> all(static_cast<size_t>(off.back()) + 1);
    Check(lfg_gmsh_physical_entity_nrs(g_.get(), codim, n, off.data(), all.data()));
    return std::vector<int32_t>(all.begin() + off[index], all.begin() + off[index + 1]);
  }
  bool IsPhysicalEntity(int codim, int64_t index, int32_t nr) const {
    for (int32_t x : PhysicalEntityNr(codim, index))
      if (x == nr) return true;
    return false;
  }
  // IsPhysicalEntity(e, nr) for every entity of codim, as a device selector
  // (e.g. the edge flags of MassEdgeMatrixProvider).
  DeviceVector<uint8_t> PhysicalEntityFlags(int codim, int32_t nr) const {
    const int64_t n = mesh_->NumEntities(codim);
    std::vector<uint8_t> h(static_cast<size_t>(n));
    Check(lfg_gmsh_is_physical_entity(g_.get(), codim, nr, n, h.data()));
    return DeviceVector<uint8_t>(*ctx_, h);
  }
  int32_t PhysicalEntityName2Nr(const std::string& name, int codim = -1) const {
    int32_t nr = 0;
    Check(lfg_gmsh_name_to_nr(g_.get(), name.c_str(), codim, &nr));
    return nr;
  }
  std::string PhysicalEntityNr2Name(int32_t nr, int codim = -1) const {
    std::vector<char> buf(4096);
    Check(lfg_gmsh_nr_to_name(g_.get(), nr, codim, buf.data(), static_cast<int64_t>(buf.size())));
    return std::string(buf.data());
  }
  std::vector<std::pair<int32_t, std::string>> PhysicalEntities(int codim) const {
    int32_t cnt = 0;
    Check(lfg_gmsh_physical_entities(g_.get(), codim, &cnt, nullptr));
    std::vector<int32_t> nrs(static_cast<size_t>(cnt) + 1);
    Check(lfg_gmsh_physical_entities(g_.get(), codim, &cnt, nrs.data()));
    std::vector<std::pair<int32_t, std::string>> out;
    for (int32_t i = 0; i < cnt; ++i) out.emplace_back(nrs[i], PhysicalEntityNr2Name(nrs[i], codim));
    return out;
  }

 private:
  static void Check(lfg_status st) {
    if (st != LFG_OK) throw Error(st, lfg_gmsh_last_error());
  }
  const Context* ctx_;
  std::shared_ptr<lfg_gmsh> g_;
  std::shared_ptr<mesh::Mesh> mesh_;
};

}  // namespace io

namespace adjoint {

// theta -> J(theta) = 1/2 ||u(theta) - u_obs||^2 with alpha = exp(theta) per
// cell, gamma = 0: a forward/backward Function object in the shape of
// torch.autograd.Function (Forward saves what Backward needs; Backward maps
// dL/dJ to dL/dtheta).  recompute = true keeps only theta between the calls.
class InverseConductivityFunction {
 public:
  struct Options {
    double f = 1.0;  // constant load
    int qr_degree_tria = 0, qr_degree_quad = 0;
    const uint8_t* flags_dev = nullptr;     // Dirichlet dofs (nullptr: boundary)
    const double* dirichlet_dev = nullptr;  // values there (nullptr: 0)
    solve::SolveOptions solve{LFG_SOLVE_FP64, 0, 1e-12, 1e-4, 32};
    bool recompute = false;
  };
  InverseConductivityFunction(std::shared_ptr<const uscalfe::FeSpaceLagrange> fes, const DeviceVector<double>& u_obs,
                              const Options& o)
      : fes_(std::move(fes)) {
    lfg_rd_adjoint_opts ao{};
    ao.load.f.kind = LFG_COEFF_CONSTANT;
    ao.load.f.value = o.f;
    ao.qr_degree_tria = o.qr_degree_tria;
    ao.qr_degree_quad = o.qr_degree_quad;
    ao.flags_dev = o.flags_dev;
    ao.dirichlet_dev = o.dirichlet_dev;
    ao.solve.precision = o.solve.precision;
    ao.solve.max_iterations = o.solve.max_iterations;
    ao.solve.rtol = o.solve.rtol;
    ao.solve.inner_rtol = o.solve.inner_rtol;
    ao.solve.check_every = o.solve.check_every;
    ao.recompute = o.recompute ? 1 : 0;
    fes_->ctx().Check(lfg_rd_adjoint_create(fes_->get(), &ao, u_obs.data(), &h_));
  }
  ~InverseConductivityFunction() {
    if (h_) lfg_rd_adjoint_destroy(h_);
  }
  InverseConductivityFunction(const InverseConductivityFunction&) = delete;
  InverseConductivityFunction& operator=(const InverseConductivityFunction&) = delete;

  double Forward(const DeviceVector<double>& theta, DeviceVector<double>* u_out = nullptr) {
    double J = 0.0;
    fes_->ctx().Check(lfg_rd_adjoint_forward(h_, theta.data(), &J, u_out ? u_out->data() : nullptr));
    return J;
  }
  void Backward(double grad_output, DeviceVector<double>& grad_theta) {
    fes_->ctx().Check(lfg_rd_adjoint_backward(h_, grad_output, grad_theta.data()));
  }
  int64_t SavedBytes() const {
    int64_t n = 0;
    fes_->ctx().Check(lfg_rd_adjoint_stats(h_, nullptr, nullptr, &n));
    return n;
  }
  std::pair<lfg_solve_stats, lfg_solve_stats> Stats() const {
    lfg_solve_stats f{}, a{};
    fes_->ctx().Check(lfg_rd_adjoint_stats(h_, &f, &a, nullptr));
    return {f, a};
  }

 private:
  std::shared_ptr<const uscalfe::FeSpaceLagrange> fes_;
  lfg_rd_adjoint* h_ = nullptr;
};

}  // namespace adjoint
}  // namespace lf::gb300
