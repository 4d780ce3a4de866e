// Host-side reference-element data: quadrature rules and Lagrangian shape
// functions, tabulated once per (cell type, degree, rule) and shipped to the
// device.  Only these tables reach the GPU (lf::quad and the reference finite
// elements are set-up work in the reference too:
// uscalfe/precomputed_scalar_reference_finite_element.h:43-184).
#include <algorithm>
#include <cmath>
#include <cstring>

#include "../../include/lfg.h"
#include "lfg_tables.h"

namespace lfg {
namespace {
#include "tria_rules.inc"

// binary32 pair of a long double value: hi rounded to nearest, lo the rest.
void Split(long double v, float* dst) {
  const float h = static_cast<float>(v);
  dst[0] = h;
  dst[1] = static_cast<float>(v - static_cast<long double>(h));
}

// Gauss-Legendre on [0,1] by Newton iteration on the Legendre recurrence
// (the algorithm of quad/gauss_quadrature.cc:16-69), in long double.
void GaussLegendre01(int n, std::vector<double>& x, std::vector<double>& w) {
  x.assign(n, 0.0);
  w.assign(n, 0.0);
  const long double pi = 3.141592653589793238462643383279502884L;
  for (int i = 0; i < (n + 1) / 2; ++i) {
    long double z = std::cos(pi * (i + 0.75L) / (n + 0.5L)), zprev, dp;
    for (int it = 0; it < 100; ++it) {
      long double p0 = 1.0L, p1 = 0.0L;
      for (int j = 0; j < n; ++j) {
        const long double pm = p1;
        p1 = p0;
        p0 = ((2.0L * j + 1.0L) * z * p1 - j * pm) / (j + 1.0L);
      }
      dp = n * (z * p0 - p1) / (z * z - 1.0L);
      zprev = z;
      z = zprev - p0 / dp;
      if (std::fabs(z - zprev) <= 1e-17L) break;
    }
    x[i] = static_cast<double>(0.5L * (1.0L - z));
    x[n - 1 - i] = static_cast<double>(0.5L * (1.0L + z));
    w[i] = w[n - 1 - i] = static_cast<double>(1.0L / ((1.0L - z * z) * dp * dp));
  }
}

// 1D Lagrange basis of degree p on the nodes used by the reference's segment
// elements: O1 {0,1}; O2 {0,1,1/2}; O3 {0,1,1/3,2/3} (lagr_fe.h:284,563,1155).
void Seg(int p, double t, double* b, double* db) {
  if (p == 1) {
    b[0] = 1.0 - t; b[1] = t;
    db[0] = -1.0;   db[1] = 1.0;
  } else if (p == 2) {
    b[0] = 2.0 * (1.0 - t) * (0.5 - t);
    b[1] = 2.0 * t * (t - 0.5);
    b[2] = 4.0 * (1.0 - t) * t;
    db[0] = 4.0 * t - 3.0;
    db[1] = 4.0 * t - 1.0;
    db[2] = 4.0 - 8.0 * t;
  } else {
    const double a = 1.0 / 3.0, c = 2.0 / 3.0;
    b[0] = 4.5 * (1.0 - t) * (a - t) * (c - t);
    b[1] = 4.5 * t * (t - a) * (t - c);
    b[2] = 13.5 * t * (1.0 - t) * (c - t);
    b[3] = 13.5 * t * (1.0 - t) * (t - a);
    db[0] = -13.5 * t * t + 18.0 * t - 5.5;
    db[1] = 13.5 * t * t - 9.0 * t + 1.0;
    db[2] = 40.5 * t * t - 45.0 * t + 9.0;
    db[3] = -40.5 * t * t + 36.0 * t - 4.5;
  }
}

// Local numbering of the tensor-product quad elements: vertices, then per
// edge its interior nodes in edge direction, then interior nodes
// (lagr_fe.h:914-925, 1462-1480).  Entry = (1D index in x, 1D index in y).
const int kQuadO1[4][2] = {{0, 0}, {1, 0}, {1, 1}, {0, 1}};
const int kQuadO2[9][2] = {{0, 0}, {1, 0}, {1, 1}, {0, 1}, {2, 0}, {1, 2}, {2, 1}, {0, 2}, {2, 2}};
const int kQuadO3[16][2] = {{0, 0}, {1, 0}, {1, 1}, {0, 1}, {2, 0}, {3, 0}, {1, 2}, {1, 3},
                            {3, 1}, {2, 1}, {0, 3}, {0, 2}, {2, 2}, {3, 2}, {3, 3}, {2, 3}};

// Gauss-Jacobi rule for the weight (1 - t) on [-1, 1] (alpha = 1, beta = 0).
// Nodes: eigenvalues of the symmetric Jacobi matrix of the monic recurrence,
//   a_k = -1 / ((2k+1)(2k+3)),  b_k^2 = k (k+1) / (2k+1)^2,
// isolated one by one with Sturm-sequence bisection (long double).  Weights:
// the Christoffel numbers w = 4 / ((1 - t^2) P_n'(t)^2) of P_n^(1,0), with
//   (m+1)(2m-1) P_m = ((4m^2-1) t + 1) P_{m-1} - (m-1)(2m+1) P_{m-2},
//   P_n'(t) = 2 n (n+1) P_{n-1}(t) / ((2n+1)(1 - t^2))   at a root.
void GaussJacobi10(int n, std::vector<long double>& t, std::vector<long double>& w) {
  std::vector<long double> a(n), b2(n, 0.0L);
  for (int k = 0; k < n; ++k) {
    a[k] = -1.0L / ((2.0L * k + 1.0L) * (2.0L * k + 3.0L));
    if (k > 0) b2[k] = static_cast<long double>(k) * (k + 1) / ((2.0L * k + 1.0L) * (2.0L * k + 1.0L));
  }
  // number of eigenvalues below x
  auto below = [&](long double x) {
    int cnt = 0;
    long double q = 1.0L;
    for (int k = 0; k < n; ++k) {
      q = (a[k] - x) - (k > 0 ? b2[k] / q : 0.0L);
      if (q == 0.0L) q = -1e-300L;
      if (q < 0.0L) ++cnt;
    }
    return cnt;
  };
  t.assign(n, 0.0L);
  w.assign(n, 0.0L);
  for (int i = 0; i < n; ++i) {
    long double lo = -1.0L, hi = 1.0L;  // the spectrum lies in (-1, 1)
    for (int it = 0; it < 200 && hi - lo > 1e-19L; ++it) {
      const long double mid = 0.5L * (lo + hi);
      if (below(mid) > i) hi = mid; else lo = mid;
    }
    const long double x = 0.5L * (lo + hi);
    long double pm2 = 0.0L, pm1 = 1.0L;  // P_{-1}, P_0
    for (int m = 1; m < n; ++m) {
      const long double p = (((4.0L * m * m - 1.0L) * x + 1.0L) * pm1 - (m - 1.0L) * (2.0L * m + 1.0L) * pm2) /
                            ((m + 1.0L) * (2.0L * m - 1.0L));
      pm2 = pm1;
      pm1 = p;
    }
    const long double dp = 2.0L * n * (n + 1.0L) * pm1 / ((2.0L * n + 1.0L) * (1.0L - x * x));
    t[i] = x;
    w[i] = 4.0L / ((1.0L - x * x) * dp * dp);
  }
}

}  // namespace

// Conical (collapsed) product rule on the reference triangle with
// m = degree/2 + 1 points per direction, exact to degree 2m - 1: Gauss-Legendre
// u_a on [0,1] (slow index) times Gauss-Jacobi(1,0) s_b = (t_b + 1)/2 (fast),
// x = u_a (1 - s_b), y = s_b, weight W_a w_b / 4.  This is the rule
// make_quad_rule.cc:139-152 builds for degrees without a hard-coded table.
void ConicalTriaRule(int degree, Rule& r) {
  const int m = degree / 2 + 1;
  std::vector<double> u, W;
  GaussLegendre01(m, u, W);
  std::vector<long double> t, w;
  GaussJacobi10(m, t, w);
  r = Rule();
  for (int a = 0; a < m; ++a)
    for (int b = 0; b < m; ++b) {
      const long double s = 0.5L * (t[b] + 1.0L);
      r.x.push_back(static_cast<double>(static_cast<long double>(u[a]) * (1.0L - s)));
      r.y.push_back(static_cast<double>(s));
      r.w.push_back(static_cast<double>(static_cast<long double>(W[a]) * w[b] * 0.25L));
    }
  r.n = static_cast<int>(r.w.size());
}

bool MakeRule(bool is_quad, int degree, Rule& r) {
  r = Rule();
  if (degree < 0 || degree > kMaxRuleDegree) return false;
  if (is_quad) {
    const int m = degree / 2 + 1;  // make_quad_rule.cc:28
    std::vector<double> x, w;
    GaussLegendre01(m, x, w);
    for (int a = 0; a < m; ++a)
      for (int b = 0; b < m; ++b) {
        r.x.push_back(x[a]);
        r.y.push_back(x[b]);
        r.w.push_back(w[a] * w[b]);
      }
  } else {
    const int d = degree == 3 ? 4 : degree;
    if (d < 1 || d > kTriaRuleMaxDegree || kTriaRuleIndex[d][0] == 0) {
      ConicalTriaRule(degree, r);
      return true;
    }
    for (int k = 0; k < kTriaRuleIndex[d][0]; ++k) {
      const double* row = kTriaRuleRows[kTriaRuleIndex[d][1] + k];
      r.x.push_back(row[0]);
      r.y.push_back(row[1]);
      r.w.push_back(row[2]);
    }
  }
  r.n = static_cast<int>(r.w.size());
  return true;
}

// ------------------------------------------------ hierarchic (hp) elements
namespace {
using ld = long double;

// Legendre polynomials in homogeneous form, P_n(x; t) = t^n P_n((2x - t) / t):
// P_0 = 1, P_1 = 2x - t, (n+1) P_{n+1} = (2n+1)(2x - t) P_n - n t^2 P_{n-1}.
void ScaledLegendre(int nmax, ld x, ld t, ld* P) {
  P[0] = 1.0L;
  if (nmax >= 1) P[1] = 2.0L * x - t;
  for (int n = 1; n < nmax; ++n)
    P[n + 1] = ((2.0L * n + 1.0L) * (2.0L * x - t) * P[n] - n * t * t * P[n - 1]) / (n + 1.0L);
}

// Integrated Legendre function L_n(x; t) = (P_n - t^2 P_{n-2}) / (2 (2n - 1)),
// n >= 2 (for t = 1 the integral of P_{n-1}(2s - 1) over [0, x]), with
// dL/dx = P_{n-1}, dL/dt = -(P_{n-1} + t P_{n-2}) / 2.
void IntLegendre(int n, ld x, ld t, ld& L, ld& Lx, ld& Lt) {
  ld P[64];
  ScaledLegendre(n, x, t, P);
  L = (P[n] - t * t * P[n - 2]) / (2.0L * (2.0L * n - 1.0L));
  Lx = P[n - 1];
  Lt = -0.5L * (P[n - 1] + t * P[n - 2]);
}

// Jacobi polynomial P_k^{(a,0)}(2x - 1) by the standard three-term recurrence.
ld JacobiA0(int k, ld a, ld x) {
  const ld z = 2.0L * x - 1.0L;
  ld p0 = 1.0L;
  if (k == 0) return p0;
  ld p1 = 0.5L * (a + (a + 2.0L) * z);
  for (int m = 1; m < k; ++m) {
    const ld c = 2.0L * m + a;
    const ld a1 = 2.0L * (m + 1) * (m + 1 + a) * c;
    const ld a2 = (c + 1.0L) * a * a;
    const ld a3 = c * (c + 1.0L) * (c + 2.0L);
    const ld a4 = 2.0L * (m + a) * m * (c + 2.0L);
    const ld p2 = ((a2 + a3 * z) * p1 - a4 * p0) / a1;
    p0 = p1;
    p1 = p2;
  }
  return p1;
}

// Integrated Jacobi function IJ_n^a(x) = int_0^x P_{n-1}^{(a,0)}(2s - 1) ds
// (n >= 1), by Gauss-Legendre quadrature on [0, x] that is exact for its
// degree n - 1; derivative P_{n-1}^{(a,0)}(2x - 1).
ld IntJacobi(int n, ld a, ld x, ld& dx) {
  dx = JacobiA0(n - 1, a, x);
  std::vector<double> gx, gw;
  const int m = (n - 1) / 2 + 1;
  GaussLegendre01(m, gx, gw);
  ld s = 0.0L;
  for (int k = 0; k < m; ++k) s += static_cast<ld>(gw[k]) * JacobiA0(n - 1, a, x * static_cast<ld>(gx[k]));
  return s * x;
}
}  // namespace

double HierSegment(int n, double t, double* dt) {
  ld L, Lx, Lt;
  IntLegendre(n, t, 1.0L, L, Lx, Lt);
  if (dt) *dt = static_cast<double>(Lx);
  return static_cast<double>(L);
}

void HierShape(bool is_quad, int p, int pat, double xd, double yd, double* phi, double (*dphi)[2]) {
  const ld x = xd, y = yd;
  auto put = [&](int slot, ld v, ld gx, ld gy) {
    phi[slot] = static_cast<double>(v);
    dphi[slot][0] = static_cast<double>(gx);
    dphi[slot][1] = static_cast<double>(gy);
  };
  if (!is_quad) {
    // barycentric coordinates of the vertices and their gradients
    const ld l[3] = {1.0L - x - y, x, y};
    const ld gl[3][2] = {{-1.0L, -1.0L}, {1.0L, 0.0L}, {0.0L, 1.0L}};
    for (int v = 0; v < 3; ++v) put(v, l[v], gl[v][0], gl[v][1]);
    int slot = 3;
    for (int e = 0; e < 3; ++e) {
      const int a = e, b = (e + 1) % 3;  // local edge e runs from vertex a to vertex b
      const bool neg = (pat >> e) & 1;
      const int s = neg ? a : b;          // the edge coordinate grows towards its end vertex
      const ld t = l[a] + l[b];
      const ld gt[2] = {gl[a][0] + gl[b][0], gl[a][1] + gl[b][1]};
      for (int i = 0; i < p - 1; ++i) {
        ld L, Lx, Lt;
        IntLegendre(i + 2, l[s], t, L, Lx, Lt);
        const int k = neg ? slot + (p - 2 - i) : slot + i;
        put(k, L, Lx * gl[s][0] + Lt * gt[0], Lx * gl[s][1] + Lt * gt[1]);
      }
      slot += p - 1;
    }
    // interior: edge-0 function of order i times an integrated Jacobi function of l2
    const int s0 = (pat & 1) ? 0 : 1;
    const ld t0 = l[0] + l[1];
    for (int i = 0; i + 3 <= p; ++i) {
      ld E, Ex, Et;
      IntLegendre(i + 2, l[s0], t0, E, Ex, Et);
      const ld Egx = Ex * gl[s0][0] + Et * (gl[0][0] + gl[1][0]);
      const ld Egy = Ex * gl[s0][1] + Et * (gl[0][1] + gl[1][1]);
      for (int j = 0; j + i + 3 <= p; ++j) {
        ld dJ;
        const ld J = IntJacobi(j + 1, 2.0L * i + 4.0L, l[2], dJ);
        put(slot++, E * J, Egx * J + E * dJ * gl[2][0], Egy * J + E * dJ * gl[2][1]);
      }
    }
    return;
  }
  // quadrilateral: products of segment functions b_0 = 1 - t, b_1 = t,
  // b_k = L_k(t) (k >= 2), in x and y, and of their reversals b_k(1 - t)
  auto seg = [&](int k, ld t, ld& d) -> ld {
    if (k == 0) { d = -1.0L; return 1.0L - t; }
    if (k == 1) { d = 1.0L; return t; }
    ld L, Lx, Lt;
    IntLegendre(k, t, 1.0L, L, Lx, Lt);
    d = Lx;
    return L;
  };
  // term b_kx(sx) * b_ky(sy) with sx = x or 1 - x (rx), sy = y or 1 - y (ry)
  auto prod = [&](int slot, int kx, bool rx, int ky, bool ry) {
    ld dx, dy;
    const ld bx = seg(kx, rx ? 1.0L - x : x, dx);
    const ld by = seg(ky, ry ? 1.0L - y : y, dy);
    put(slot, bx * by, (rx ? -dx : dx) * by, bx * (ry ? -dy : dy));
  };
  prod(0, 0, false, 0, false);
  prod(1, 1, false, 0, false);
  prod(2, 1, false, 1, false);
  prod(3, 0, false, 1, false);
  int slot = 4;
  for (int e = 0; e < 4; ++e) {
    const bool neg = (pat >> e) & 1;
    for (int i = 0; i < p - 1; ++i) {
      const int k = neg ? slot + (p - 2 - i) : slot + i;
      switch (e) {
        case 0: prod(k, i + 2, neg, 0, false); break;   // bottom, x from v0 to v1
        case 1: prod(k, 1, false, i + 2, neg); break;   // right, y from v1 to v2
        case 2: prod(k, i + 2, !neg, 1, false); break;  // top, x from v2 back to v3
        default: prod(k, 0, false, i + 2, !neg); break; // left, y from v3 back to v0
      }
    }
    slot += p - 1;
  }
  for (int i = 0; i < p - 1; ++i)
    for (int j = 0; j < p - 1; ++j) prod(slot++, j + 2, false, i + 2, false);
}

void NodeCoords(bool is_quad, int degree, std::vector<double>& xy) {
  xy.clear();
  if (is_quad) {
    // 1D nodes of the segment elements: {0, 1}, {0, 1, 1/2}, {0, 1, 1/3, 2/3}
    const double s[3][4] = {{0.0, 1.0}, {0.0, 1.0, 0.5}, {0.0, 1.0, 1.0 / 3.0, 2.0 / 3.0}};
    const int(*map)[2] = degree == 1 ? kQuadO1 : degree == 2 ? kQuadO2 : kQuadO3;
    for (int i = 0; i < NumShape(true, degree); ++i) {
      xy.push_back(s[degree - 1][map[i][0]]);
      xy.push_back(s[degree - 1][map[i][1]]);
    }
    return;
  }
  // vertices, then per edge (0,1), (1,2), (2,0) its interior nodes from the
  // first endpoint on, then the barycentre (the nodes of Shape's basis)
  const double V[3][2] = {{0.0, 0.0}, {1.0, 0.0}, {0.0, 1.0}};
  for (auto& v : V) {
    xy.push_back(v[0]);
    xy.push_back(v[1]);
  }
  const int e[3][2] = {{0, 1}, {1, 2}, {2, 0}};
  for (int k = 0; k < 3 && degree >= 2; ++k)
    for (int j = 1; j < degree; ++j) {
      const double tb = static_cast<double>(j) / degree, ta = static_cast<double>(degree - j) / degree;
      xy.push_back(ta * V[e[k][0]][0] + tb * V[e[k][1]][0]);
      xy.push_back(ta * V[e[k][0]][1] + tb * V[e[k][1]][1]);
    }
  if (degree == 3) {
    xy.push_back(1.0 / 3.0);
    xy.push_back(1.0 / 3.0);
  }
}

int NumShape(bool is_quad, int degree) {
  return is_quad ? (degree + 1) * (degree + 1) : (degree + 1) * (degree + 2) / 2;
}

void Shape(bool is_quad, int degree, double x, double y, double* phi, double (*dphi)[2]) {
  if (is_quad) {
    double bx[4], dbx[4], by[4], dby[4];
    Seg(degree, x, bx, dbx);
    Seg(degree, y, by, dby);
    const int(*map)[2] = degree == 1 ? kQuadO1 : degree == 2 ? kQuadO2 : kQuadO3;
    for (int i = 0; i < NumShape(true, degree); ++i) {
      const int a = map[i][0], b = map[i][1];
      phi[i] = bx[a] * by[b];
      dphi[i][0] = dbx[a] * by[b];
      dphi[i][1] = bx[a] * dby[b];
    }
    return;
  }
  // Triangles in barycentric coordinates l0 = 1-x-y, l1 = x, l2 = y with
  // d l0 = (-1,-1), d l1 = (1,0), d l2 = (0,1).
  const double l[3] = {1.0 - x - y, x, y};
  const double dl[3][2] = {{-1.0, -1.0}, {1.0, 0.0}, {0.0, 1.0}};
  if (degree == 1) {
    for (int i = 0; i < 3; ++i) {
      phi[i] = l[i];
      dphi[i][0] = dl[i][0];
      dphi[i][1] = dl[i][1];
    }
    return;
  }
  if (degree == 2) {
    // vertices: l(2l-1); edge midpoints of (0,1), (1,2), (2,0): 4 la lb
    for (int i = 0; i < 3; ++i) {
      phi[i] = l[i] * (2.0 * l[i] - 1.0);
      for (int d = 0; d < 2; ++d) dphi[i][d] = (4.0 * l[i] - 1.0) * dl[i][d];
    }
    const int e[3][2] = {{0, 1}, {1, 2}, {2, 0}};
    for (int k = 0; k < 3; ++k) {
      const int a = e[k][0], b = e[k][1];
      phi[3 + k] = 4.0 * l[a] * l[b];
      for (int d = 0; d < 2; ++d) dphi[3 + k][d] = 4.0 * (dl[a][d] * l[b] + l[a] * dl[b][d]);
    }
    return;
  }
  // degree 3: vertices 9/2 l(l-1/3)(l-2/3); edge (a,b) nodes at 1/3 and 2/3
  // from a: 27/2 la lb (la-1/3) then 27/2 la lb (lb-1/3); bubble 27 l0 l1 l2.
  const double t = 1.0 / 3.0, tt = 2.0 / 3.0;
  for (int i = 0; i < 3; ++i) {
    phi[i] = 4.5 * l[i] * (l[i] - t) * (l[i] - tt);
    const double dv = 4.5 * ((l[i] - t) * (l[i] - tt) + l[i] * (l[i] - tt) + l[i] * (l[i] - t));
    for (int d = 0; d < 2; ++d) dphi[i][d] = dv * dl[i][d];
  }
  const int e[3][2] = {{0, 1}, {1, 2}, {2, 0}};
  for (int k = 0; k < 3; ++k) {
    const int a = e[k][0], b = e[k][1];
    phi[3 + 2 * k] = 13.5 * l[a] * l[b] * (l[a] - t);
    phi[4 + 2 * k] = 13.5 * l[a] * l[b] * (l[b] - t);
    for (int d = 0; d < 2; ++d) {
      dphi[3 + 2 * k][d] = 13.5 * (dl[a][d] * l[b] * (l[a] - t) + l[a] * dl[b][d] * (l[a] - t) +
                                   l[a] * l[b] * dl[a][d]);
      dphi[4 + 2 * k][d] = 13.5 * (dl[a][d] * l[b] * (l[b] - t) + l[a] * dl[b][d] * (l[b] - t) +
                                   l[a] * l[b] * dl[b][d]);
    }
  }
  phi[9] = 27.0 * l[0] * l[1] * l[2];
  for (int d = 0; d < 2; ++d)
    dphi[9][d] = 27.0 * (dl[0][d] * l[1] * l[2] + l[0] * dl[1][d] * l[2] + l[0] * l[1] * dl[2][d]);
}

// If the quadrilateral Lagrangian basis of `degree` is the tensor product of
// the 1D Lagrange basis on the equispaced nodes {0, 1/p, ..., 1}, i.e.
// phi_{loc[a n1 + b]}(x, y) = l_a(x) l_b(y) with gradients to match at every
// point of the rule, fill loc and the 1D product tables
// sf[kind][a][b][p] (kind 0: l'_a l'_b, 1: l_a l_b, 2: l'_a l_b at the m
// abscissae of the tensor Gauss rule) and return true.
static bool TensorBasis(int degree, const Rule& r, int m, int* loc, std::vector<long double>& sf) {
  const int n1 = degree + 1, n = n1 * n1;
  if (n > 16 || m * m != r.n) return false;
  std::vector<long double> node(n1);
  for (int a = 0; a < n1; ++a) node[a] = static_cast<long double>(a) / degree;
  auto l1 = [&](int a, long double x, long double* d) {
    long double v = 1.0L, dv = 0.0L;
    for (int k = 0; k < n1; ++k) {
      if (k == a) continue;
      const long double f = (x - node[k]) / (node[a] - node[k]);
      dv = dv * f + v / (node[a] - node[k]);
      v *= f;
    }
    *d = dv;
    return v;
  };
  double phi[16], dphi[16][2];
  for (int a = 0; a < n1; ++a)
    for (int b = 0; b < n1; ++b) {
      Shape(true, degree, static_cast<double>(node[a]), static_cast<double>(node[b]), phi, dphi);
      int hit = -1;
      for (int i = 0; i < n; ++i) {
        if (std::fabs(phi[i] - 1.0) < 1e-12) hit = i;
        else if (std::fabs(phi[i]) > 1e-12) return false;
      }
      if (hit < 0) return false;
      loc[a * n1 + b] = hit;
    }
  for (int k = 0; k < r.n; ++k) {
    Shape(true, degree, r.x[k], r.y[k], phi, dphi);
    for (int a = 0; a < n1; ++a)
      for (int b = 0; b < n1; ++b) {
        long double da, db;
        const long double la = l1(a, r.x[k], &da), lb = l1(b, r.y[k], &db);
        const int i = loc[a * n1 + b];
        if (std::fabs(static_cast<double>(la * lb) - phi[i]) > 1e-12 ||
            std::fabs(static_cast<double>(da * lb) - dphi[i][0]) > 1e-11 ||
            std::fabs(static_cast<double>(la * db) - dphi[i][1]) > 1e-11)
          return false;
      }
  }
  // abscissae: x of points (p, 0) (x slow, y fast)
  sf.assign(3 * n1 * n1 * m, 0.0L);
  for (int a = 0; a < n1; ++a)
    for (int b = 0; b < n1; ++b)
      for (int p = 0; p < m; ++p) {
        long double da, db;
        const long double x = r.x[p * m];
        const long double la = l1(a, x, &da), lb = l1(b, x, &db);
        sf[((0 * n1 + a) * n1 + b) * m + p] = da * db;
        sf[((1 * n1 + a) * n1 + b) * m + p] = la * lb;
        sf[((2 * n1 + a) * n1 + b) * m + p] = da * lb;
      }
  return true;
}

bool BuildDfTables(bool quad, int degree, int rule_degree, std::vector<float>& out, DfLayout& L) {
  Rule r;
  if (!MakeRule(quad, rule_degree, r)) return false;
  L = DfLayout();
  L.n = NumShape(quad, degree);
  L.E = L.n * (L.n + 1) / 2;
  L.nq = r.n;
  L.m = quad ? rule_degree / 2 + 1 : 0;  // Gauss-Legendre points per direction (make_quad_rule.cc:28)
  L.off_R = 0;
  L.off_L = L.off_R + L.E * 4;
  L.off_T = L.off_L + L.n;
  L.off_W = L.off_T + L.nq * L.E * 4;
  L.off_t = L.off_W + L.nq;
  L.off_X = L.off_t + L.m;
  L.off_O1 = L.off_X + 2 * L.nq;
  L.off_SC = L.off_O1 + 4 * L.nq;
  L.off_SF = L.off_SC + 23;
  L.total = L.off_SF;
  std::vector<long double> sf;
  if (quad && degree >= 2 && TensorBasis(degree, r, L.m, L.loc, sf)) {
    L.n1 = degree + 1;
    L.total += static_cast<int>(sf.size());
  }
  out.assign(2 * static_cast<size_t>(L.total), 0.0f);
  for (size_t q = 0; q < (L.n1 ? sf.size() : 0); ++q) Split(sf[q], &out[2 * (L.off_SF + q)]);
  std::vector<long double> R(L.E * 4, 0.0L), Ls(L.n, 0.0L);
  double phi[16], dphi[16][2], p1[16], d1[16][2];
  // sin(pi r) = sum_k (-1)^k pi^(2k+1) r^(2k+1) / (2k+1)!, cos likewise
  const long double pi = 3.141592653589793238462643383279502884L;
  long double term = pi;  // pi^(2k+1) / (2k+1)!
  for (int k = 0; k < 11; ++k) {
    Split((k & 1) ? -term : term, &out[2 * (L.off_SC + k)]);
    term *= pi * pi / ((2.0L * k + 2.0L) * (2.0L * k + 3.0L));
  }
  term = 1.0L;  // pi^(2k) / (2k)!
  for (int k = 0; k < 12; ++k) {
    Split((k & 1) ? -term : term, &out[2 * (L.off_SC + 11 + k)]);
    term *= pi * pi / ((2.0L * k + 1.0L) * (2.0L * k + 2.0L));
  }
  for (int k = 0; k < r.n; ++k) {
    Shape(quad, degree, r.x[k], r.y[k], phi, dphi);
    Shape(quad, 1, r.x[k], r.y[k], p1, d1);
    Split(r.x[k], &out[2 * (L.off_X + 2 * k)]);
    Split(r.y[k], &out[2 * (L.off_X + 2 * k + 1)]);
    for (int v = 0; v < (quad ? 4 : 3); ++v) Split(p1[v], &out[2 * (L.off_O1 + 4 * k + v)]);
    const long double w = r.w[k];
    int e = 0;
    for (int i = 0; i < L.n; ++i)
      for (int j = i; j < L.n; ++j, ++e) {
        const long double gi0 = dphi[i][0], gi1 = dphi[i][1], gj0 = dphi[j][0], gj1 = dphi[j][1];
        const long double t[4] = {gi0 * gj0, gi0 * gj1 + gi1 * gj0, gi1 * gj1,
                                  static_cast<long double>(phi[i]) * phi[j]};
        for (int q = 0; q < 4; ++q) {
          R[4 * e + q] += w * t[q];
          Split(t[q], &out[2 * (L.off_T + (k * L.E + e) * 4 + q)]);
        }
      }
    for (int i = 0; i < L.n; ++i) Ls[i] += w * phi[i];
    Split(w, &out[2 * (L.off_W + k)]);
  }
  for (int q = 0; q < L.E * 4; ++q) Split(R[q], &out[2 * (L.off_R + q)]);
  for (int i = 0; i < L.n; ++i) Split(Ls[i], &out[2 * (L.off_L + i)]);
  if (quad) {
    // 1D abscissae: the x coordinate of points (p, 0), p = 0..m-1
    for (int p = 0; p < L.m; ++p) Split(r.x[p * L.m], &out[2 * (L.off_t + p)]);
  }
  return true;
}

bool SegmentTables(int degree, int rule_degree, std::vector<double>& t, std::vector<double>& w,
                   std::vector<double>& phi) {
  if (degree < 1 || degree > 3 || rule_degree < 0) return false;
  const int m = rule_degree / 2 + 1;
  GaussLegendre01(m, t, w);
  const int n = degree + 1;
  // nodes 0, 1, then 1/p, ..., (p-1)/p
  std::vector<long double> node(n);
  node[0] = 0.0L;
  node[1] = 1.0L;
  for (int a = 2; a < n; ++a) node[a] = static_cast<long double>(a - 1) / degree;
  phi.assign(static_cast<size_t>(m) * n, 0.0);
  for (int k = 0; k < m; ++k)
    for (int a = 0; a < n; ++a) {
      long double v = 1.0L;
      for (int b = 0; b < n; ++b)
        if (b != a) v *= (static_cast<long double>(t[k]) - node[b]) / (node[a] - node[b]);
      phi[static_cast<size_t>(k) * n + a] = static_cast<double>(v);
    }
  return true;
}

namespace {
// P_n^{(a,b)}(2x - 1) by the three-term recurrence of the Jacobi polynomials
// (Abramowitz & Stegun 22.7.1).
ld JacobiAB(int n, ld a, ld b, ld x) {
  const ld z = 2.0L * x - 1.0L;
  ld p0 = 1.0L;
  if (n == 0) return p0;
  ld p1 = (a + 1.0L) + 0.5L * (a + b + 2.0L) * (z - 1.0L);
  for (int k = 2; k <= n; ++k) {
    const ld c = 2.0L * k + a + b;
    const ld p2 = ((c - 1.0L) * (c * (c - 2.0L) * z + a * a - b * b) * p1 -
                   2.0L * (k + a - 1.0L) * (k + b - 1.0L) * c * p0) /
                  (2.0L * k * (k + a + b) * (c - 2.0L));
    p0 = p1;
    p1 = p2;
  }
  return p1;
}

// d/dx P_n(2x - 1) of the shifted Legendre polynomial (n >= 0).
ld LegendreDx01(int n, ld x) {
  if (n == 0) return 0.0L;
  ld P[64];
  ScaledLegendre(n, x, 1.0L, P);
  // P_n'(z) = sum_{k = n-1, n-3, ...} (2k + 1) P_k(z), and dz/dx = 2
  ld s = 0.0L;
  for (int k = n - 1; k >= 0; k -= 2) s += (2.0L * k + 1.0L) * P[k];
  return 2.0L * s;
}

// Rows of the segment dual of degree d (FeHierarchicSegment::NodalValuesToDofs,
// hierarchic_fe.h:367-390) for i = 2..d: the coefficients on the value at 0,
// at 1 and at the Gauss points t of the segment rule of degree 2(d - 1).
struct SegDual {
  std::vector<double> t;        // d points
  std::vector<double> c0, c1;   // [i - 2]
  std::vector<double> cq;       // [(i - 2) * d + q]
};
SegDual MakeSegDual(int d) {
  SegDual S;
  std::vector<double> w;
  GaussLegendre01(d, S.t, w);  // 2(d - 1) / 2 + 1 = d points
  for (int i = 2; i <= d; ++i) {
    const ld f = 2.0L * i - 1.0L;
    ld P[64];
    ScaledLegendre(i - 1, 0.0L, 1.0L, P);
    const ld p0 = P[i - 1];
    ScaledLegendre(i - 1, 1.0L, 1.0L, P);
    const ld p1 = P[i - 1];
    S.c0.push_back(static_cast<double>(-p0 * f));
    S.c1.push_back(static_cast<double>(p1 * f));
    for (int q = 0; q < d; ++q)
      S.cq.push_back(static_cast<double>(-static_cast<ld>(w[q]) * LegendreDx01(i - 1, S.t[q]) * f));
  }
  return S;
}
}  // namespace

int HierNumShapeVar(bool is_quad, int pc, const int* pe) {
  const int nv = is_quad ? 4 : 3;
  int n = nv;
  for (int j = 0; j < nv; ++j) n += pe[j] - 1;
  return n + (is_quad ? (pc - 1) * (pc - 1) : (pc - 1) * (pc - 2) / 2);
}

void HierVarSlots(bool is_quad, int pc, const int* pe, int pat, int D, int* sel) {
  const int nv = is_quad ? 4 : 3;
  int k = 0;
  for (int j = 0; j < nv; ++j) sel[k++] = j;
  for (int j = 0; j < nv; ++j) {
    const int ns = pe[j] - 1, ub = nv + j * (D - 1);
    const bool neg = (pat >> j) & 1;
    for (int a = 0; a < ns; ++a) sel[k++] = ub + (neg ? D - 1 - ns + a : a);
  }
  const int ub = nv * D;
  if (is_quad) {
    for (int i = 0; i < pc - 1; ++i)
      for (int jj = 0; jj < pc - 1; ++jj) sel[k++] = ub + i * (D - 1) + jj;
  } else {
    for (int i = 0; i < pc - 2; ++i)
      for (int jj = 0; jj < pc - 2 - i; ++jj) sel[k++] = ub + i * (D - 2) - i * (i - 1) / 2 + jj;
  }
}

void HierDual(bool is_quad, int pc, const int* pe, int pat, std::vector<double>& xy, std::vector<double>& M) {
  const int nv = is_quad ? 4 : 3;
  const int n = HierNumShapeVar(is_quad, pc, pe);
  xy.clear();
  auto add = [&](double x, double y) {
    xy.push_back(x);
    xy.push_back(y);
  };
  // vertices, then the Gauss points of every edge of degree >= 2 in the edge's
  // own direction (hierarchic_fe.h:835-873, 1470-1515)
  const double vx[4] = {0, 1, is_quad ? 1.0 : 0.0, 0}, vy[4] = {0, 0, 1, 1};
  for (int j = 0; j < nv; ++j) add(vx[j], vy[j]);
  std::vector<SegDual> ed(nv);
  std::vector<int> ecol(nv, 0);
  for (int j = 0; j < nv; ++j) {
    if (pe[j] <= 1) continue;
    ed[j] = MakeSegDual(pe[j]);
    ecol[j] = static_cast<int>(xy.size() / 2);
    const int a = j, b = (j + 1) % nv;
    const bool neg = (pat >> j) & 1;
    for (double u : ed[j].t) {
      // the edge runs from local vertex a to b; a negative one is parametrised from b
      const double s = neg ? 1.0 - u : u;
      add(vx[a] + s * (vx[b] - vx[a]), vy[a] + s * (vy[b] - vy[a]));
    }
  }
  const int icol = static_cast<int>(xy.size() / 2);
  Rule tr;
  SegDual fd;
  int D = pc, nq1 = 0;
  if (!is_quad) {
    MakeRule(false, 2 * (pc - 1), tr);  // always part of the nodes (hierarchic_fe.h:874-876)
    for (int q = 0; q < tr.n; ++q) add(tr.x[q], tr.y[q]);
  } else if (pc > 1) {
    for (int j = 0; j < nv; ++j) D = std::max(D, pe[j]);
    fd = MakeSegDual(D);
    nq1 = D + 2;
    std::vector<double> pts = {0.0, 1.0};
    pts.insert(pts.end(), fd.t.begin(), fd.t.end());
    for (int r = 0; r < nq1; ++r)
      for (int k = 0; k < nq1; ++k) add(pts[k], pts[r]);
  }
  const int ne = static_cast<int>(xy.size() / 2);
  M.assign(static_cast<size_t>(n) * ne, 0.0);
  auto at = [&](int row, int col) -> double& { return M[static_cast<size_t>(row) * ne + col]; };
  for (int j = 0; j < nv; ++j) at(j, j) = 1.0;
  // edge dofs: the segment dual along the edge; a negative edge's slots are
  // reversed and its start is local vertex b
  int slot = nv;
  for (int j = 0; j < nv; ++j) {
    const int pj = pe[j];
    if (pj <= 1) continue;
    const bool neg = (pat >> j) & 1;
    const int va = neg ? (j + 1) % nv : j, vb = neg ? j : (j + 1) % nv;
    for (int i = 2; i <= pj; ++i) {
      const int row = slot + (neg ? pj - i : i - 2);
      at(row, va) += ed[j].c0[i - 2];
      at(row, vb) += ed[j].c1[i - 2];
      for (int q = 0; q < pj; ++q) at(row, ecol[j] + q) += ed[j].cq[static_cast<size_t>(i - 2) * pj + q];
    }
    slot += pj - 1;
  }
  const int nb = slot;
  if (is_quad) {
    // interior: the degree-D segment dual along x on every node row, then
    // along y (hierarchic_fe.h:1640-1665); dof (a, b) at slot a + b (pc - 1)
    if (pc <= 1) return;
    auto S = [&](int i, int node) -> double {  // row i >= 2 of the segment dual, node 0 / 1 / 2 + q
      return node == 0 ? fd.c0[i - 2] : node == 1 ? fd.c1[i - 2] : fd.cq[static_cast<size_t>(i - 2) * D + node - 2];
    };
    const int m = pc - 1;
    for (int b = 0; b < m; ++b)
      for (int a = 0; a < m; ++a) {
        const int row = nb + a + b * m;
        for (int r = 0; r < nq1; ++r) {
          const double sy = S(b + 2, r);
          for (int k = 0; k < nq1; ++k) at(row, icol + r * nq1 + k) = sy * S(a + 2, k);
        }
      }
    return;
  }
  if (pc <= 2) return;
  // triangle interior (hierarchic_fe.h:1024-1083): F v with the integrated
  // Legendre / Jacobi duals over the interior rule, then orthogonalised
  // against the vertex and edge duals: M_face = F - (F Phi_b^T) M_b, Phi_b
  // the boundary shape functions at the nodes (hierarchic_fe.h:891-915)
  const int nf = n - nb;
  std::vector<double> F(static_cast<size_t>(nf) * ne, 0.0);
  {
    int idx = 0;
    for (int i = 0; i < pc - 2; ++i)
      for (int j = 0; j < pc - i - 2; ++j, ++idx) {
        const ld a = 2.0L * i + 4.0L, f = (2.0L * i + 3.0L) * (2.0L * j + 2.0L * i + 5.0L);
        for (int q = 0; q < tr.n; ++q) {
          const ld x = tr.x[q], y = tr.y[q];
          ld xn = x / (1.0L - y);
          if (pat & 1) xn = 1.0L - xn;
          const ld psidd = LegendreDx01(i + 1, xn);
          const ld jdd = j == 0 ? 0.0L : JacobiAB(j - 1, a + 1.0L, 1.0L, y) * (a + j + 1.0L);
          const ld jd = JacobiAB(j, a, 0.0L, y);
          const ld term = std::pow(1.0L - y, i + 1) * jdd - a * std::pow(1.0L - y, i) * jd;
          F[static_cast<size_t>(idx) * ne + icol + q] = static_cast<double>(tr.w[q] * psidd * term * f);
        }
      }
  }
  D = pc;
  for (int j = 0; j < nv; ++j) D = std::max(D, pe[j]);
  const int nD = (D + 1) * (D + 2) / 2;
  std::vector<int> sel(n);
  HierVarSlots(false, pc, pe, pat, D, sel.data());
  std::vector<double> phi(nD), dphi(2 * nD);
  std::vector<long double> G(static_cast<size_t>(nf) * nb, 0.0L);  // F Phi_b^T
  for (int k = icol; k < ne; ++k) {  // F is zero outside the interior nodes
    HierShape(false, D, pat, xy[2 * k], xy[2 * k + 1], phi.data(), reinterpret_cast<double(*)[2]>(dphi.data()));
    for (int r = 0; r < nf; ++r) {
      const ld fr = F[static_cast<size_t>(r) * ne + k];
      for (int a = 0; a < nb; ++a) G[static_cast<size_t>(r) * nb + a] += fr * phi[sel[a]];
    }
  }
  for (int r = 0; r < nf; ++r)
    for (int k = 0; k < ne; ++k) {
      ld s = F[static_cast<size_t>(r) * ne + k];
      for (int a = 0; a < nb; ++a) s -= G[static_cast<size_t>(r) * nb + a] * at(a, k);
      at(nb + r, k) = static_cast<double>(s);
    }
}

}  // namespace lfg

extern "C" lfg_status lfg_quad_rule(int32_t is_quad, int32_t degree, double* x, double* y, double* w, int32_t* n) {
  if (!n) return LFG_INVALID_ARG;
  lfg::Rule r;
  if (!lfg::MakeRule(is_quad != 0, degree, r)) return LFG_INVALID_ARG;
  if (x || y || w) {
    if (!x || !y || !w || *n < r.n) return LFG_INVALID_ARG;
    std::memcpy(x, r.x.data(), r.n * sizeof(double));
    std::memcpy(y, r.y.data(), r.n * sizeof(double));
    std::memcpy(w, r.w.data(), r.n * sizeof(double));
  }
  *n = r.n;
  return LFG_OK;
}

extern "C" lfg_status lfg_hier_dual(int32_t is_quad, int32_t interior_degree, const int32_t* edge_degrees,
                                    int32_t pattern, double* xy, double* M, int32_t* n_nodes, int32_t* n_dofs) {
  if (!edge_degrees || !n_nodes || !n_dofs) return LFG_INVALID_ARG;
  const int nv = is_quad ? 4 : 3;
  int pe[4] = {1, 1, 1, 1};
  if (interior_degree < 1 || interior_degree > lfg::kMaxHierDualDegree) return LFG_INVALID_ARG;
  for (int j = 0; j < nv; ++j) {
    if (edge_degrees[j] < 1 || edge_degrees[j] > lfg::kMaxHierDualDegree) return LFG_INVALID_ARG;
    pe[j] = edge_degrees[j];
  }
  if (pattern < 0 || pattern >= (1 << nv)) return LFG_INVALID_ARG;
  std::vector<double> nodes, m;
  lfg::HierDual(is_quad != 0, interior_degree, pe, pattern, nodes, m);
  const int ne = static_cast<int>(nodes.size() / 2), n = lfg::HierNumShapeVar(is_quad != 0, interior_degree, pe);
  if (xy || M) {
    if (!xy || !M || *n_nodes < ne || *n_dofs < n) return LFG_INVALID_ARG;
    std::memcpy(xy, nodes.data(), nodes.size() * sizeof(double));
    std::memcpy(M, m.data(), m.size() * sizeof(double));
  }
  *n_nodes = ne;
  *n_dofs = n;
  return LFG_OK;
}
