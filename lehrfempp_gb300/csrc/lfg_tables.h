// Reference-element data built on the host (no CUDA dependency): quadrature
// rules, Lagrangian shape functions and the df32 (binary32-pair) tables of
// the element kernels.
#pragma once

#include <vector>

namespace lfg {

struct Rule {
  int n = 0;
  std::vector<double> x, y, w;
};
// make_QuadRule (quad/make_quad_rule.cc:21-157): triangles from the
// reference's tables for degree 1..50 (3 -> 4; quad/quad_rules_tria.cc),
// otherwise (degree 0 and above 50) the conical Gauss-Legendre x
// Gauss-Jacobi(1,0) product rule with degree/2+1 points per direction (the
// reference's rule beyond its tables, make_quad_rule.cc:139-152); quads tensor
// Gauss-Legendre with degree/2+1 points per direction, x slow / y fast.
// False for a degree outside [0, kMaxRuleDegree].
constexpr int kMaxRuleDegree = 100;
bool MakeRule(bool is_quad, int degree, Rule& out);
int NumShape(bool is_quad, int degree);
void Shape(bool is_quad, int degree, double x, double y, double* phi, double (*dphi)[2]);
// Hierarchic (hp) reference elements of uniform degree p >= 1
// (fe/hierarchic_fe.h: FeHierarchicTria, FeHierarchicQuad): vertex functions,
// per local edge p-1 integrated Legendre functions in the edge's own
// direction, then the interior functions.  `pattern` bit j set = local edge j
// negatively oriented (the cell's relative orientation): such an edge's
// functions use the reversed edge coordinate and sit in reversed slots, and
// the triangle's interior functions follow edge 0's direction.  Counts equal
// the Lagrangian ones, (p+1)(p+2)/2 and (p+1)^2.
void HierShape(bool is_quad, int p, int pattern, double x, double y, double* phi, double (*dphi)[2]);
// Variable degrees (HierarchicScalarFESpace with a degree functor): a cell
// with interior degree pc and edge degrees pe[0..nvert) has
// HierNumShapeVar(...) shape functions, which are the slots sel[0..n) of the
// uniform degree-D basis (D >= pc and every pe), same pattern convention.
int HierNumShapeVar(bool is_quad, int pc, const int* pe);
void HierVarSlots(bool is_quad, int pc, const int* pe, int pattern, int D, int* sel);
// EvaluationNodes and NodalValuesToDofs of FeHierarchicTria / FeHierarchicQuad
// (fe/hierarchic_fe.h:820-1083, 1445-1680) with interior degree pc, edge
// degrees pe and orientation pattern `pattern`, in matrix form: xy[2 k],
// xy[2 k + 1] is evaluation node k, and the dofs of a function with values v
// at the nodes are M v (M row-major, HierNumShapeVar rows x node count).
constexpr int kMaxHierDualDegree = 20;
void HierDual(bool is_quad, int pc, const int* pe, int pattern, std::vector<double>& xy, std::vector<double>& M);
// Integrated Legendre function of the segment element: L_n(t) = int_0^t P_{n-1}(2s-1) ds
// for n >= 2 (FeHierarchicSegment's shape function n), and its derivative.
double HierSegment(int n, double t, double* dt);

// Reference coordinates of the evaluation nodes of the Lagrangian element
// (EvaluationNodes, uscalfe/lagr_fe.h): xy[2 i], xy[2 i + 1] is the node of
// local shape function i (phi_j(node_i) = delta_ij).
void NodeCoords(bool is_quad, int degree, std::vector<double>& xy);

// df32 tables (pairs of floats; offsets in pairs):
//   R[E][4]    folded sums sum_k w_k {g_i0 g_j0, g_i0 g_j1 + g_i1 g_j0, g_i1 g_j1, phi_i phi_j}
//   L[n]       folded load sums sum_k w_k phi_i
//   T[nq][E][4] the same terms per point (no weight)
//   W[nq]      point weights,  t[m] 1D abscissae            (t: quads)
//   X[nq][2]   reference point coordinates, O1[nq][4] O1 shape values there
//   SC[23]     Taylor coefficients of sin(pi r) (11) and cos(pi r) (12)
//   SF[3][n1][n1][m]  1D products {l'_a l'_b, l_a l_b, l'_a l_b} at the m
//              Gauss abscissae, for quads whose basis is the tensor product
//              phi_{loc[a n1 + b]}(x, y) = l_a(x) l_b(y) of a 1D basis of
//              degree n1 - 1 (n1 = 0: not a tensor basis, no SF block)
struct DfLayout {
  int n = 0, E = 0, nq = 0, m = 0;
  int off_R = 0, off_L = 0, off_T = 0, off_W = 0, off_t = 0, total = 0;
  int off_X = 0, off_O1 = 0, off_SC = 0;
  int n1 = 0, off_SF = 0;
  int loc[16] = {};
};
bool BuildDfTables(bool is_quad, int degree, int rule_degree, std::vector<float>& out, DfLayout& L);

// Segment rule of make_quad_rule.cc:22-27 (Gauss-Legendre, rule_degree/2+1
// points on [0, 1]) and the segment Lagrange basis of `degree` at its points,
// phi[k * n + i], n = degree + 1, local order: the two endpoints, then the
// interior nodes along the segment (FeLagrangeO{1,2,3}Segment numbering).
bool SegmentTables(int degree, int rule_degree, std::vector<double>& t, std::vector<double>& w,
                   std::vector<double>& phi);

}  // namespace lfg
