// Oracle (test infrastructure only): CPU restatement of the LehrFEM++ path.
// See lfo.h for scope and the rule that only tests / smoke / bench baselines
// may use it.  File:line citations are relative to the LehrFEM++ source tree.
#include <algorithm>
#include <cmath>
#include <numeric>

#include "lfo.h"

namespace lfo {

#include "tria_rules.inc"

// =========================================================== quadrature ====

// lib/lf/quad/gauss_quadrature.cc:16-69.  The reference runs Newton's method in
// a 57-bit binary float; long double (64-bit mantissa on x86-64, 113-bit on
// aarch64) gives the same roots after rounding to double up to 1 ulp.
void GaussLegendre(int n, std::vector<double>& pts, std::vector<double>& wts) {
  if (n <= 0) throw Error("GaussLegendre: num_points must be positive");
  pts.assign(n, 0.0);
  wts.assign(n, 0.0);
  const long double pi = 3.141592653589793238462643383279502884L;
  const int m = (n + 1) / 2;
  for (int i = 0; i < m; ++i) {
    long double z = std::cos(pi * (i + 0.75L) / (n + 0.5L));
    long double z1, pp;
    int guard = 0;
    do {
      long double p1 = 1.0L, p2 = 0.0L, p3;
      for (int j = 0; j < n; ++j) {
        p3 = p2;
        p2 = p1;
        p1 = ((2.0L * j + 1.0L) * z * p2 - j * p3) / (j + 1.0L);
      }
      pp = n * (z * p1 - p2) / (z * z - 1.0L);
      z1 = z;
      z = z1 - p1 / pp;
    } while (std::fabs(z - z1) > 1e-17L && ++guard < 100);
    pts[i] = static_cast<double>(0.5L * (1.0L - z));
    pts[n - 1 - i] = static_cast<double>(0.5L * (1.0L + z));
    wts[i] = static_cast<double>(1.0L / ((1.0L - z * z) * pp * pp));
    wts[n - 1 - i] = wts[i];
  }
}

// lib/lf/quad/gauss_quadrature.cc:71-196 for alpha = 1, beta = 0: roots of
// P_n^(1,0) bracketed by a sign scan on a fine grid, then bisection and a
// Newton polish on the three-term recurrence (long double); weights are the
// Christoffel numbers 4 / ((1 - z^2) P_n'(z)^2).
namespace {
void Jacobi10(int n, long double z, long double& pn, long double& pn1) {
  // (m+1)(2m-1) P_m = ((4m^2-1) z + 1) P_{m-1} - (m-1)(2m+1) P_{m-2}
  long double a = 0.0L, b = 1.0L;  // P_{-1}, P_0
  for (int m = 1; m <= n; ++m) {
    const long double c = (((4.0L * m * m - 1.0L) * z + 1.0L) * b - (m - 1.0L) * (2.0L * m + 1.0L) * a) /
                          ((m + 1.0L) * (2.0L * m - 1.0L));
    a = b;
    b = c;
  }
  pn = b;
  pn1 = a;
}
}  // namespace

void GaussJacobi10(int n, std::vector<double>& pts, std::vector<double>& wts) {
  if (n <= 0) throw Error("GaussJacobi: num_points must be positive");
  pts.clear();
  wts.clear();
  const int K = 64 * n * n + 64;
  long double zl = -1.0L, pl, q;
  Jacobi10(n, zl, pl, q);
  for (int k = 1; k <= K; ++k) {
    const long double zr = -1.0L + 2.0L * k / K;
    long double pr;
    Jacobi10(n, zr, pr, q);
    if ((pl < 0) != (pr < 0) || pr == 0.0L) {
      long double lo = zl, hi = zr, plo = pl;
      for (int it = 0; it < 200 && hi - lo > 1e-20L; ++it) {
        const long double mid = 0.5L * (lo + hi);
        long double pm;
        Jacobi10(n, mid, pm, q);
        if ((pm < 0) == (plo < 0)) { lo = mid; plo = pm; } else hi = mid;
      }
      long double z = 0.5L * (lo + hi), pn, pn1;
      Jacobi10(n, z, pn, pn1);
      const long double dp = (n * (1.0L - (2.0L * n + 1.0L) * z) * pn + 2.0L * n * (n + 1.0L) * pn1) /
                             ((2.0L * n + 1.0L) * (1.0L - z * z));
      if (dp != 0.0L) z -= pn / dp;
      Jacobi10(n, z, pn, pn1);
      const long double d2 = (n * (1.0L - (2.0L * n + 1.0L) * z) * pn + 2.0L * n * (n + 1.0L) * pn1) /
                             ((2.0L * n + 1.0L) * (1.0L - z * z));
      pts.push_back(static_cast<double>(z));
      wts.push_back(static_cast<double>(4.0L / ((1.0L - z * z) * d2 * d2)));
      if (pr == 0.0L) {  // skip past an exact grid root
        ++k;
        Jacobi10(n, -1.0L + 2.0L * k / K, pr, q);
        zl = -1.0L + 2.0L * k / K;
        pl = pr;
        continue;
      }
    }
    zl = zr;
    pl = pr;
  }
  if (static_cast<int>(pts.size()) != n) throw Error("GaussJacobi: root isolation failed");
}

// lib/lf/quad/make_quad_rule.cc:21-157.
QuadRule MakeQuadRule(bool is_quad, int degree) {
  QuadRule qr;
  if (is_quad) {
    const int n = degree / 2 + 1;
    std::vector<double> p, w;
    GaussLegendre(n, p, w);
    // points row0 = kron(x, ones(n)) (x slow), row1 = repeat(x) (y fast);
    // weights = kron(w, w)  (make_quad_rule.cc:28-37)
    for (int a = 0; a < n; ++a)
      for (int b = 0; b < n; ++b) {
        qr.x.push_back(p[a]);
        qr.y.push_back(p[b]);
        qr.w.push_back(w[a] * w[b]);
      }
    qr.degree = 2 * n - 1;
    return qr;
  }
  int d = degree;
  if (d == 3) d = 4;  // make_quad_rule.cc:44-46
  if (d < 1 || d > kTriaRuleMaxDegree || kTriaRuleIndex[d][0] == 0) {
    // make_quad_rule.cc:139-152: the collapsed (conical) Gauss rule with
    // n = degree/2 + 1 Gauss-Legendre points u_a (slow) and Gauss-Jacobi(1,0)
    // points (fast) mapped to [0,1]: x = u_a (1 - s_b), y = s_b,
    // w = W_a w_b / 4, for degree 0 and degrees above the tables (50).
    if (degree < 0) throw Error("MakeQuadRule: negative degree");
    const int n = degree / 2 + 1;
    std::vector<double> u, W, t, w;
    GaussLegendre(n, u, W);
    GaussJacobi10(n, t, w);
    for (int a = 0; a < n; ++a)
      for (int b = 0; b < n; ++b) {
        const double s = (t[b] + 1.0) / 2.0;
        qr.x.push_back(u[a] * (1.0 - s));
        qr.y.push_back(s);
        qr.w.push_back(W[a] * (w[b] * 0.25));
      }
    qr.degree = 2 * n - 1;
    return qr;
  }
  const int np = kTriaRuleIndex[d][0], off = kTriaRuleIndex[d][1];
  for (int k = 0; k < np; ++k) {
    qr.x.push_back(kTriaRuleRows[off + k][0]);
    qr.y.push_back(kTriaRuleRows[off + k][1]);
    qr.w.push_back(kTriaRuleRows[off + k][2]);
  }
  qr.degree = d;
  return qr;
}

// ================================================== reference elements ====
namespace {
// FeLagrangeO2Segment (lagr_fe.h:563-700)
inline void SegO2(double x, double b[3], double db[3]) {
  b[0] = 2.0 * (1.0 - x) * (0.5 - x);
  b[1] = 2.0 * x * (x - 0.5);
  b[2] = 4.0 * (1.0 - x) * x;
  db[0] = 4.0 * x - 3.0;
  db[1] = 4.0 * x - 1.0;
  db[2] = 4.0 - 8.0 * x;
}
// FeLagrangeO3Segment (lagr_fe.h:1155-1277)
inline void SegO3(double x, double b[4], double db[4]) {
  b[0] = 4.5 * (1.0 - x) * (1.0 / 3.0 - x) * (2.0 / 3.0 - x);
  b[1] = 4.5 * x * (x - 1.0 / 3.0) * (x - 2.0 / 3.0);
  b[2] = 13.5 * x * (1 - x) * (2.0 / 3.0 - x);
  b[3] = 13.5 * x * (1 - x) * (x - 1.0 / 3.0);
  db[0] = -13.5 * x * x + 18.0 * x - 5.5;
  db[1] = 13.5 * x * x - 9.0 * x + 1.0;
  db[2] = 40.5 * x * x - 45 * x + 9;
  db[3] = -40.5 * x * x + 36 * x - 4.5;
}
// ksegment_to_quad_mapping_ of FeLagrangeO2Quad (lagr_fe.h:914-925) and
// FeLagrangeO3Quad (lagr_fe.h:1462-1480).
const int kO2QuadMap[9][2] = {{0, 0}, {1, 0}, {1, 1}, {0, 1}, {2, 0},
                              {1, 2}, {2, 1}, {0, 2}, {2, 2}};
const int kO3QuadMap[16][2] = {{0, 0}, {1, 0}, {1, 1}, {0, 1}, {2, 0}, {3, 0},
                               {1, 2}, {1, 3}, {3, 1}, {2, 1}, {0, 3}, {0, 2},
                               {2, 2}, {3, 2}, {3, 3}, {2, 3}};
}  // namespace

int NumShapeFunctions(bool is_quad, int degree) {
  static const int t[4] = {0, 3, 6, 10}, q[4] = {0, 4, 9, 16};
  if (degree < 1 || degree > 3) throw Error("degree must be 1..3");
  return is_quad ? q[degree] : t[degree];
}

void EvalShape(bool is_quad, int degree, double x0, double x1, double* phi,
               double (*dphi)[2]) {
  if (!is_quad && degree == 1) {  // FeLagrangeO1Tria lagr_fe.h:57-160
    phi[0] = 1.0 - x0 - x1;
    phi[1] = x0;
    phi[2] = x1;
    dphi[0][0] = -1; dphi[0][1] = -1;
    dphi[1][0] = 1;  dphi[1][1] = 0;
    dphi[2][0] = 0;  dphi[2][1] = 1;
  } else if (is_quad && degree == 1) {  // FeLagrangeO1Quad lagr_fe.h:165-280
    phi[0] = (1 - x0) * (1 - x1);
    phi[1] = x0 * (1 - x1);
    phi[2] = x0 * x1;
    phi[3] = (1 - x0) * x1;
    dphi[0][0] = x1 - 1.0;  dphi[0][1] = x0 - 1.0;
    dphi[1][0] = 1.0 - x1;  dphi[1][1] = -x0;
    dphi[2][0] = x1;        dphi[2][1] = x0;
    dphi[3][0] = -x1;       dphi[3][1] = 1.0 - x0;
  } else if (!is_quad && degree == 2) {  // FeLagrangeO2Tria lagr_fe.h:400-560
    phi[0] = 2.0 * (1 - x0 - x1) * (0.5 - x0 - x1);
    phi[1] = 2.0 * x0 * (x0 - 0.5);
    phi[2] = 2.0 * x1 * (x1 - 0.5);
    phi[3] = 4.0 * (1 - x0 - x1) * x0;
    phi[4] = 4.0 * x0 * x1;
    phi[5] = 4.0 * (1 - x0 - x1) * x1;
    dphi[0][0] = -3.0 + 4.0 * x0 + 4.0 * x1;  dphi[0][1] = -3.0 + 4.0 * x0 + 4.0 * x1;
    dphi[1][0] = 4.0 * x0 - 1.0;              dphi[1][1] = 0.0;
    dphi[2][0] = 0.0;                         dphi[2][1] = 4.0 * x1 - 1.0;
    dphi[3][0] = 4 - 0 - 8.0 * x0 - 4.0 * x1; dphi[3][1] = -4 * x0;
    dphi[4][0] = 4.0 * x1;                    dphi[4][1] = 4.0 * x0;
    dphi[5][0] = -4.0 * x1;                   dphi[5][1] = 4.0 - 8.0 * x1 - 4.0 * x0;
  } else if (is_quad && degree == 2) {  // FeLagrangeO2Quad lagr_fe.h:713-925
    double bx[3], dbx[3], by[3], dby[3];
    SegO2(x0, bx, dbx);
    SegO2(x1, by, dby);
    for (int i = 0; i < 9; ++i) {
      const int a = kO2QuadMap[i][0], b = kO2QuadMap[i][1];
      phi[i] = bx[a] * by[b];
      dphi[i][0] = dbx[a] * by[b];
      dphi[i][1] = dby[b] * bx[a];
    }
  } else if (!is_quad && degree == 3) {  // FeLagrangeO3Tria lagr_fe.h:945-1150
    const double l0 = 1 - x0 - x1, l1 = x0, l2 = x1;
    const double t = 1 / 3.0, tt = 2 / 3.0;
    phi[0] = 4.5 * l0 * (l0 - t) * (l0 - tt);
    phi[1] = 4.5 * l1 * (l1 - t) * (l1 - tt);
    phi[2] = 4.5 * l2 * (l2 - t) * (l2 - tt);
    phi[3] = 13.5 * l0 * l1 * (l0 - t);
    phi[4] = 13.5 * l0 * l1 * (l1 - t);
    phi[5] = 13.5 * l1 * l2 * (l1 - t);
    phi[6] = 13.5 * l1 * l2 * (l2 - t);
    phi[7] = 13.5 * l2 * l0 * (l2 - t);
    phi[8] = 13.5 * l2 * l0 * (l0 - t);
    phi[9] = 27.0 * l0 * l1 * l2;
    const double g0 = -4.5 * ((l0 - t) * (l0 - tt) + l0 * (l0 - tt) + l0 * (l0 - t));
    dphi[0][0] = g0;
    dphi[0][1] = g0;
    dphi[1][0] = 4.5 * ((l1 - t) * (l1 - tt) + l1 * (l1 - tt) + l1 * (l1 - t));
    dphi[1][1] = 0.0;
    dphi[2][0] = 0.0;
    dphi[2][1] = 4.5 * ((l2 - t) * (l2 - tt) + l2 * (l2 - tt) + l2 * (l2 - t));
    dphi[3][0] = 13.5 * (-l1 * (l0 - t) + l0 * (l0 - t) - l0 * l1);
    dphi[3][1] = -13.5 * (l1 * (l0 - t) + l0 * l1);
    dphi[4][0] = 13.5 * (-l1 * (l1 - t) + l0 * (l1 - t) + l0 * l1);
    dphi[4][1] = -13.5 * l1 * (l1 - t);
    dphi[5][0] = 13.5 * (l2 * (l1 - t) + l1 * l2);
    dphi[5][1] = 13.5 * (l1 * (l1 - t));
    dphi[6][0] = 13.5 * (l2 * (l2 - t));
    dphi[6][1] = 13.5 * (l1 * (l2 - t) + l1 * l2);
    dphi[7][0] = -13.5 * l2 * (l2 - t);
    dphi[7][1] = 13.5 * (l0 * (l2 - t) - l2 * (l2 - t) + l0 * l2);
    dphi[8][0] = -13.5 * (l2 * (l0 - t) + l2 * l0);
    dphi[8][1] = 13.5 * (l0 * (l0 - t) - l2 * (l0 - t) - l2 * l0);
    dphi[9][0] = 27.0 * (-l1 * l2 + l0 * l2);
    dphi[9][1] = 27.0 * (-l1 * l2 + l0 * l1);
  } else if (is_quad && degree == 3) {  // FeLagrangeO3Quad lagr_fe.h:1279-1480
    double bx[4], dbx[4], by[4], dby[4];
    SegO3(x0, bx, dbx);
    SegO3(x1, by, dby);
    for (int i = 0; i < 16; ++i) {
      const int a = kO3QuadMap[i][0], b = kO3QuadMap[i][1];
      phi[i] = bx[a] * by[b];
      dphi[i][0] = dbx[a] * by[b];
      dphi[i][1] = dby[b] * bx[a];
    }
  } else {
    throw Error("EvalShape: unsupported degree");
  }
}

void EvaluationNodes(bool is_quad, int degree, std::vector<double>& xy) {
  const double t = 1.0 / 3.0;
  xy.clear();
  auto add = [&](double a, double b) { xy.push_back(a); xy.push_back(b); };
  if (!is_quad) {
    add(0, 0); add(1, 0); add(0, 1);
    if (degree == 2) { add(0.5, 0); add(0.5, 0.5); add(0, 0.5); }
    if (degree == 3) {
      // edges << 1,2,2,1,0,0 / 0,0,1,2,2,1 scaled by 1/3 (lagr_fe.h:1124-1136)
      const double ex[6] = {1, 2, 2, 1, 0, 0}, ey[6] = {0, 0, 1, 2, 2, 1};
      for (int k = 0; k < 6; ++k) add(ex[k] * t, ey[k] * t);
      add(1.0 / 3.0, 1.0 / 3.0);
    }
  } else {
    add(0, 0); add(1, 0); add(1, 1); add(0, 1);
    if (degree == 2) {
      add(0.5, 0); add(1, 0.5); add(0.5, 1); add(0, 0.5); add(0.5, 0.5);
    }
    if (degree == 3) {
      const double mx[8] = {1, 2, 3, 3, 2, 1, 0, 0}, my[8] = {0, 0, 1, 2, 3, 3, 2, 1};
      for (int k = 0; k < 8; ++k) add(mx[k] * t, my[k] * t);
      const double ix[4] = {1, 2, 2, 1}, iy[4] = {1, 1, 2, 2};
      for (int k = 0; k < 4; ++k) add(ix[k] * t, iy[k] * t);
    }
  }
}

// ============================================================ geometry ====
namespace {
// Eigen 2x2 inverse of M = J^T (Eigen/src/LU/InverseImpl.h, size-2 path):
// invdet = 1/det; inv = [m11, -m01; -m10, m00] * invdet.
inline void InverseTranspose(const double J[2][2], double out[2][2]) {
  const double m00 = J[0][0], m01 = J[1][0], m10 = J[0][1], m11 = J[1][1];
  const double det = m00 * m11 - m10 * m01;
  const double invdet = 1.0 / det;
  out[0][0] = m11 * invdet;
  out[1][0] = -m10 * invdet;
  out[0][1] = -m01 * invdet;
  out[1][1] = m00 * invdet;
}
inline void Jacobian(const CellGeom& g, double xh, double yh, double J[2][2]) {
  if (!g.is_quad) {  // tria_o1.cc:56
    for (int d = 0; d < 2; ++d) {
      J[d][0] = g.v[1][d] - g.v[0][d];
      J[d][1] = g.v[2][d] - g.v[0][d];
    }
  } else {  // quad_o1.cc:93-99
    for (int d = 0; d < 2; ++d) {
      J[d][0] = (g.v[1][d] - g.v[0][d]) * (1 - yh) + (g.v[2][d] - g.v[3][d]) * yh;
      J[d][1] = (g.v[3][d] - g.v[0][d]) * (1 - xh) + (g.v[2][d] - g.v[1][d]) * xh;
    }
  }
}
}  // namespace

void CellGeom::JinvT(double xh, double yh, double out[2][2]) const {
  double J[2][2];
  Jacobian(*this, xh, yh, J);
  InverseTranspose(J, out);
}
double CellGeom::IntegrationElement(double xh, double yh) const {
  double J[2][2];
  Jacobian(*this, xh, yh, J);
  return std::abs(J[0][0] * J[1][1] - J[1][0] * J[0][1]);
}
void CellGeom::Global(double xh, double yh, double out[2]) const {
  for (int d = 0; d < 2; ++d) {
    if (!is_quad) {  // tria_o1.cc:68-72
      out[d] = v[0][d] * (1 - xh - yh) + v[1][d] * xh + v[2][d] * yh;
    } else {  // quad_o1.cc:73-87
      out[d] = v[0][d] * ((1 - xh) * (1 - yh)) + v[1][d] * (xh * (1 - yh)) +
               v[2][d] * (xh * yh) + v[3][d] * ((1 - xh) * yh);
    }
  }
}

bool NonDegenerate(const CellGeom& g, double tol) {
  const int nv = g.is_quad ? 4 : 3;
  double lensq[4], circum = 0;
  for (int k = 0; k < nv; ++k) {
    const double* a = g.v[k];
    const double* b = g.v[(k + 1) % nv];
    lensq[k] = (b[0] - a[0]) * (b[0] - a[0]) + (b[1] - a[1]) * (b[1] - a[1]);
    circum += lensq[k];
  }
  for (int k = 0; k < nv; ++k)
    if (!(lensq[k] > tol * circum)) return false;
  const double ar1 = (g.v[1][0] - g.v[0][0]) * (g.v[2][1] - g.v[0][1]) -
                     (g.v[1][1] - g.v[0][1]) * (g.v[2][0] - g.v[0][0]);
  double area = std::fabs(ar1);
  if (g.is_quad) {
    const double ar2 = (g.v[3][0] - g.v[0][0]) * (g.v[2][1] - g.v[0][1]) -
                       (g.v[3][1] - g.v[0][1]) * (g.v[2][0] - g.v[0][0]);
    area += std::fabs(ar2);
  }
  return area > tol * circum;
}

// ================================================================ mesh ====

CellGeom Mesh::Geom(idx_t c) const {
  CellGeom g;
  g.is_quad = IsQuad(c);
  for (int k = 0; k < 4; ++k) {
    const idx_t v = cell_nodes[c][k];
    g.v[k][0] = v >= 0 ? xy[2 * v] : 0.0;
    g.v[k][1] = v >= 0 ? xy[2 * v + 1] : 0.0;
  }
  return g;
}

namespace {
// EndpointIndexPair of hybrid2d/mesh.cc:130-165: compares by (min,max) and
// remembers the endpoint order of whoever created it.
struct EdgeKey {
  idx_t lo, hi;
  bool operator<(const EdgeKey& o) const { return lo == o.lo ? hi < o.hi : lo < o.lo; }
};
struct EdgeData {
  idx_t p0, p1;
  idx_t global_index;
  std::vector<std::pair<idx_t, int>> adj;  // (cell, local edge)
};
}  // namespace

Mesh BuildMesh(idx_t num_nodes, const double* xy, idx_t num_cells,
               const int64_t* cn, idx_t num_preset, const int64_t* pe) {
  Mesh m;
  m.num_nodes = num_nodes;
  m.xy.assign(xy, xy + 2 * num_nodes);
  m.num_cells = num_cells;
  m.cell_nodes.resize(num_cells);
  std::map<EdgeKey, EdgeData> edge_map;
  // predefined edges (mesh.cc:237-274)
  idx_t edge_index = 0;
  for (idx_t e = 0; e < num_preset; ++e) {
    const idx_t a = pe[2 * e], b = pe[2 * e + 1];
    if (a < 0 || b < 0 || a >= num_nodes || b >= num_nodes || a == b)
      throw Error("illegal preset edge " + std::to_string(e));
    EdgeKey k{std::min(a, b), std::max(a, b)};
    auto ins = edge_map.insert({k, EdgeData{a, b, edge_index, {}}});
    if (!ins.second) throw Error("duplicate preset edge " + std::to_string(e));
    ++edge_index;
  }
  // cells (mesh.cc:305-437)
  for (idx_t c = 0; c < num_cells; ++c) {
    for (int k = 0; k < 4; ++k) m.cell_nodes[c][k] = cn[4 * c + k];
    const int nv = m.cell_nodes[c][3] < 0 ? 3 : 4;
    for (int k = 0; k < nv; ++k)
      if (m.cell_nodes[c][k] < 0 || m.cell_nodes[c][k] >= num_nodes)
        throw Error("cell " + std::to_string(c) + ": invalid node index");
    for (int j = 0; j < nv; ++j) {
      // local edge j = (v_j, v_{j+1 mod nv}) (base/ref_el.h:126-129)
      const idx_t a = m.cell_nodes[c][j], b = m.cell_nodes[c][(j + 1) % nv];
      if (a == b) throw Error("cell " + std::to_string(c) + ": loop edge");
      EdgeKey k{std::min(a, b), std::max(a, b)};
      auto it = edge_map.find(k);
      if (it == edge_map.end()) {
        edge_map.insert({k, EdgeData{a, b, -1, {{c, j}}}});
      } else {
        it->second.adj.push_back({c, j});
      }
    }
  }
  // number the remaining edges in map order (mesh.cc:523-563)
  m.num_edges = static_cast<idx_t>(edge_map.size());
  m.edge_nodes.assign(m.num_edges, {-1, -1});
  m.edge_num_cells.assign(m.num_edges, 0);
  m.cell_edges.assign(num_cells, {-1, -1, -1, -1});
  m.cell_ori.assign(num_cells, {0, 0, 0, 0});
  for (auto& kv : edge_map) {
    EdgeData& ed = kv.second;
    if (ed.global_index == -1) ed.global_index = edge_index++;
    m.edge_nodes[ed.global_index] = {ed.p0, ed.p1};
    m.edge_num_cells[ed.global_index] = static_cast<int32_t>(ed.adj.size());
    for (auto& a : ed.adj) m.cell_edges[a.first][a.second] = ed.global_index;
  }
  // relative orientations (hybrid2d/triangle.cc:71-77, quad.cc:76)
  for (idx_t c = 0; c < num_cells; ++c) {
    const int nv = m.NumVerts(c);
    for (int j = 0; j < nv; ++j)
      m.cell_ori[c][j] = (m.edge_nodes[m.cell_edges[c][j]][0] == m.cell_nodes[c][j]) ? 1 : -1;
  }
  return m;
}

FactoryInput TPTriagInput(idx_t nx, idx_t ny, double x0, double y0, double x1,
                          double y1) {
  FactoryInput in;
  const double hx = (x1 - x0) / nx, hy = (y1 - y0) / ny;
  auto vid = [&](idx_t i, idx_t j) { return i + j * (nx + 1); };  // VertexIndex
  for (idx_t j = 0; j <= ny; ++j)
    for (idx_t i = 0; i <= nx; ++i) {
      in.xy.push_back(x0 + static_cast<double>(static_cast<uint64_t>(i)) * hx);
      in.xy.push_back(y0 + static_cast<double>(static_cast<uint64_t>(j)) * hy);
    }
  auto edge = [&](idx_t a, idx_t b) { in.edges.push_back(a); in.edges.push_back(b); };
  for (idx_t i = 0; i < nx; ++i)
    for (idx_t j = 0; j <= ny; ++j) edge(vid(i, j), vid(i + 1, j));
  for (idx_t i = 0; i <= nx; ++i)
    for (idx_t j = 0; j < ny; ++j) edge(vid(i, j), vid(i, j + 1));
  for (idx_t i = 0; i < nx; ++i)
    for (idx_t j = 0; j < ny; ++j) edge(vid(i, j), vid(i + 1, j + 1));
  for (idx_t i = 0; i < nx; ++i)
    for (idx_t j = 0; j < ny; ++j) {
      const int64_t up[4] = {vid(i, j), vid(i + 1, j + 1), vid(i, j + 1), -1};
      const int64_t lo[4] = {vid(i, j), vid(i + 1, j), vid(i + 1, j + 1), -1};
      in.cells.insert(in.cells.end(), up, up + 4);
      in.cells.insert(in.cells.end(), lo, lo + 4);
    }
  return in;
}

FactoryInput TPQuadInput(idx_t nx, idx_t ny, double x0, double y0, double x1,
                         double y1) {
  FactoryInput in;
  const double hx = (x1 - x0) / nx, hy = (y1 - y0) / ny;
  auto vid = [&](idx_t i, idx_t j) { return i + j * (nx + 1); };
  for (idx_t j = 0; j <= ny; ++j)
    for (idx_t i = 0; i <= nx; ++i) {
      in.xy.push_back(x0 + static_cast<double>(static_cast<uint64_t>(i)) * hx);
      in.xy.push_back(y0 + static_cast<double>(static_cast<uint64_t>(j)) * hy);
    }
  for (idx_t i = 0; i < nx; ++i)
    for (idx_t j = 0; j < ny; ++j) {
      const int64_t q[4] = {vid(i, j), vid(i + 1, j), vid(i + 1, j + 1), vid(i, j + 1)};
      in.cells.insert(in.cells.end(), q, q + 4);
    }
  return in;
}

FactoryInput TestMesh0Input(double s) {
  FactoryInput in;
  const double pts[10][2] = {{1.5, 2}, {1, 1}, {2, 1}, {0, 0}, {1.5, 0},
                             {3, 0},   {3, 2}, {3, 3}, {0, 3}, {0, 1}};
  for (auto& p : pts) { in.xy.push_back(p[0] * s); in.xy.push_back(p[1] * s); }
  const int64_t cells[9][4] = {{0, 8, 9, -1}, {3, 4, 1, -1}, {4, 2, 1, -1},
                               {4, 5, 2, -1}, {5, 6, 2, -1}, {3, 1, 0, 9},
                               {2, 6, 7, 0},  {0, 7, 8, -1}, {0, 1, 2, -1}};
  for (auto& c : cells) in.cells.insert(in.cells.end(), c, c + 4);
  return in;
}

void FlagEntitiesOnBoundary(const Mesh& m, std::vector<uint8_t>& nf,
                            std::vector<uint8_t>& ef) {
  nf.assign(m.num_nodes, 0);
  ef.assign(m.num_edges, 0);
  for (idx_t e = 0; e < m.num_edges; ++e)
    if (m.edge_num_cells[e] == 1) {
      ef[e] = 1;
      nf[m.edge_nodes[e][0]] = 1;
      nf[m.edge_nodes[e][1]] = 1;
    }
}

// ========================================================= dof handler ====

DofHandler MakeDofHandler(const Mesh& m, int np, int ns, int nt, int nq,
                          bool check_edge_orientation) {
  DofHandler d;
  d.mesh = &m;
  d.np = np; d.ns = ns; d.nt = nt; d.nq = nq;
  // InitTotalNumDofs (dofhandler.cc:131-139)
  d.n_node = np;
  d.n_edge = 2 * np + ns;
  d.n_tria = 3 * np + 3 * ns + nt;
  d.n_quad = 4 * np + 4 * ns + nq;
  d.n_cell = std::max(d.n_tria, d.n_quad);
  idx_t dof = 0;
  // Step I: nodes
  d.node_dofs.assign(m.num_nodes * np, -1);
  for (idx_t v = 0; v < m.num_nodes; ++v)
    for (int j = 0; j < np; ++j) {
      d.node_dofs[v * np + j] = dof++;
      d.dof_entity.push_back({2, v});
    }
  // Step II: edges (endpoint dofs copied in edge direction, then interior)
  d.edge_dofs.assign(m.num_edges * d.n_edge, -1);
  for (idx_t e = 0; e < m.num_edges; ++e) {
    idx_t off = e * d.n_edge;
    for (int k = 0; k < 2; ++k)
      for (int j = 0; j < np; ++j) d.edge_dofs[off++] = d.node_dofs[m.edge_nodes[e][k] * np + j];
    for (int j = 0; j < ns; ++j) {
      d.edge_dofs[off++] = dof++;
      d.dof_entity.push_back({1, e});
    }
  }
  // Step III: cells
  const int ext_edge = d.n_edge - ns;
  d.cell_dofs.assign(m.num_cells * d.n_cell, -1);
  for (idx_t c = 0; c < m.num_cells; ++c) {
    idx_t off = c * d.n_cell;
    const int nv = m.NumVerts(c);
    for (int k = 0; k < nv; ++k)
      for (int j = 0; j < np; ++j) d.cell_dofs[off++] = d.node_dofs[m.cell_nodes[c][k] * np + j];
    for (int k = 0; k < nv; ++k) {
      const idx_t e = m.cell_edges[c][k];
      const idx_t base = e * d.n_edge + ext_edge;
      if (!check_edge_orientation || m.cell_ori[c][k] > 0) {
        for (int j = 0; j < ns; ++j) d.cell_dofs[off++] = d.edge_dofs[base + j];
      } else {
        for (int j = ns - 1; j >= 0; --j) d.cell_dofs[off++] = d.edge_dofs[base + j];
      }
    }
    const int nint = nv == 3 ? nt : nq;
    for (int j = 0; j < nint; ++j) {
      d.cell_dofs[off++] = dof++;
      d.dof_entity.push_back({0, c});
    }
  }
  d.num_dofs = dof;
  return d;
}

DofHandler MakeHierVarDofHandler(const Mesh& m, const std::vector<int>& edge_deg, const std::vector<int>& cell_deg) {
  if (static_cast<idx_t>(edge_deg.size()) != m.num_edges || static_cast<idx_t>(cell_deg.size()) != m.num_cells)
    throw Error("one degree per edge and per cell expected");
  for (int d : edge_deg)
    if (d < 1) throw Error("edge degrees must be >= 1");
  for (int d : cell_deg)
    if (d < 1) throw Error("cell degrees must be >= 1");
  DofHandler d;
  d.mesh = &m;
  d.np = 1;
  d.edge_deg = edge_deg;
  d.cell_deg = cell_deg;
  idx_t dof = 0;
  // Step I: one dof per node, in node order
  d.node_dofs.assign(m.num_nodes, -1);
  for (idx_t v = 0; v < m.num_nodes; ++v) {
    d.node_dofs[v] = dof++;
    d.dof_entity.push_back({2, v});
  }
  // Step II: edge_deg[e] - 1 interior dofs per edge, in edge order
  std::vector<idx_t> edge_first(m.num_edges);
  for (idx_t e = 0; e < m.num_edges; ++e) {
    edge_first[e] = dof;
    for (int j = 0; j < edge_deg[e] - 1; ++j) {
      ++dof;
      d.dof_entity.push_back({1, e});
    }
  }
  // Step III: per cell its vertices, its edges' dofs, its interior dofs
  d.nloc.assign(m.num_cells, 0);
  int nmax = 0;
  for (idx_t c = 0; c < m.num_cells; ++c) {
    const int nv = m.NumVerts(c);
    int pe[4] = {1, 1, 1, 1};
    for (int k = 0; k < nv; ++k) pe[k] = edge_deg[m.cell_edges[c][k]];
    d.nloc[c] = HierNumShapeVar(nv == 4, cell_deg[c], pe);
    nmax = std::max(nmax, d.nloc[c]);
  }
  d.n_cell = nmax;
  d.cell_dofs.assign(m.num_cells * static_cast<idx_t>(nmax), -1);
  for (idx_t c = 0; c < m.num_cells; ++c) {
    idx_t off = c * nmax;
    const int nv = m.NumVerts(c);
    for (int k = 0; k < nv; ++k) d.cell_dofs[off++] = d.node_dofs[m.cell_nodes[c][k]];
    for (int k = 0; k < nv; ++k) {
      const idx_t e = m.cell_edges[c][k];
      const int ns = edge_deg[e] - 1;
      if (m.cell_ori[c][k] > 0) {
        for (int j = 0; j < ns; ++j) d.cell_dofs[off++] = edge_first[e] + j;
      } else {
        for (int j = ns - 1; j >= 0; --j) d.cell_dofs[off++] = edge_first[e] + j;
      }
    }
    const int pc = cell_deg[c];
    const int nint = nv == 4 ? (pc - 1) * (pc - 1) : (pc <= 2 ? 0 : (pc - 2) * (pc - 1) / 2);
    for (int j = 0; j < nint; ++j) {
      d.cell_dofs[off++] = dof++;
      d.dof_entity.push_back({0, c});
    }
  }
  d.num_dofs = dof;
  return d;
}

DofHandler MakeLagrangeDofHandler(const Mesh& m, int degree) {
  // {pt:1, seg:p-1, tria:(p-1)(p-2)/2, quad:(p-1)^2} (lagr_fe.h NumRefShapeFunctions)
  const int p = degree;
  return MakeDofHandler(m, 1, p - 1, (p - 1) * (p - 2) / 2, (p - 1) * (p - 1));
}

// ====================================================== mesh functions ====

std::function<double(double, double)> AnalyticFunction(int func_id, const double* p) {
  std::vector<double> q(p, p + 16);
  const double pi = 3.14159265358979323846;
  switch (func_id) {
    case 1:  // polynomial sum_{i,j<=3} p[4i+j] x^i y^j
      return [q](double x, double y) {
        double xi[4] = {1, x, x * x, x * x * x}, yj[4] = {1, y, y * y, y * y * y};
        double s = 0;
        for (int i = 0; i < 4; ++i)
          for (int j = 0; j < 4; ++j) s += q[4 * i + j] * (xi[i] * yj[j]);
        return s;
      };
    case 2:  // p0 + p1 sin(p2 pi x) sin(p3 pi y)
      return [q, pi](double x, double y) {
        return q[0] + q[1] * (std::sin(q[2] * pi * x) * std::sin(q[3] * pi * y));
      };
    case 3:  // p0 + p1 sin(p2 pi x) cos(p3 pi y)
      return [q, pi](double x, double y) {
        return q[0] + q[1] * (std::sin(q[2] * pi * x) * std::cos(q[3] * pi * y));
      };
    case 4:  // p0 + p1 exp(p2 + p3 x + p4 y + p5 x y)
      return [q](double x, double y) {
        return q[0] + q[1] * std::exp(q[2] + q[3] * x + q[4] * y + q[5] * (x * y));
      };
    case 5:  // p0 + (p1 + p2 x + p3 y + p4 x y) sin(pi (p5 x + p6)) sin(pi (p7 y + p8))
      return [q, pi](double x, double y) {
        const double l = q[1] + q[2] * x + q[3] * y + q[4] * (x * y);
        return q[0] + l * (std::sin(pi * (q[5] * x + q[6])) * std::sin(pi * (q[7] * y + q[8])));
      };
    default:
      throw Error("unknown analytic function id " + std::to_string(func_id));
  }
}

std::function<void(double, double, double*)> AnalyticGradient(int func_id, const double* p) {
  std::vector<double> q(p, p + 16);
  const double pi = 3.14159265358979323846;
  switch (func_id) {
    case 1:
      return [q](double x, double y, double* g) {
        double xi[4] = {1, x, x * x, x * x * x}, yj[4] = {1, y, y * y, y * y * y};
        g[0] = g[1] = 0.0;
        for (int i = 0; i < 4; ++i)
          for (int j = 0; j < 4; ++j) {
            if (i > 0) g[0] += q[4 * i + j] * (i * xi[i - 1] * yj[j]);
            if (j > 0) g[1] += q[4 * i + j] * (xi[i] * j * yj[j - 1]);
          }
      };
    case 2:
      return [q, pi](double x, double y, double* g) {
        const double ax = q[2] * pi * x, ay = q[3] * pi * y;
        g[0] = q[1] * q[2] * pi * std::cos(ax) * std::sin(ay);
        g[1] = q[1] * q[3] * pi * std::sin(ax) * std::cos(ay);
      };
    case 3:
      return [q, pi](double x, double y, double* g) {
        const double ax = q[2] * pi * x, ay = q[3] * pi * y;
        g[0] = q[1] * q[2] * pi * std::cos(ax) * std::cos(ay);
        g[1] = -q[1] * q[3] * pi * std::sin(ax) * std::sin(ay);
      };
    case 4:
      return [q](double x, double y, double* g) {
        const double e = q[1] * std::exp(q[2] + q[3] * x + q[4] * y + q[5] * (x * y));
        g[0] = e * (q[3] + q[5] * y);
        g[1] = e * (q[4] + q[5] * x);
      };
    case 5:
      return [q, pi](double x, double y, double* g) {
        const double l = q[1] + q[2] * x + q[3] * y + q[4] * (x * y);
        const double ax = pi * (q[5] * x + q[6]), ay = pi * (q[7] * y + q[8]);
        g[0] = (q[2] + q[4] * y) * std::sin(ax) * std::sin(ay) + l * pi * q[5] * std::cos(ax) * std::sin(ay);
        g[1] = (q[3] + q[4] * x) * std::sin(ax) * std::sin(ay) + l * std::sin(ax) * pi * q[7] * std::cos(ay);
      };
    default:
      throw Error("unknown analytic function id " + std::to_string(func_id));
  }
}

void MeshFunction::Eval(const Mesh& m, idx_t cell, const QuadRule& qr,
                        std::vector<double>& out) const {
  out.assign(qr.n(), 0.0);
  switch (kind) {
    case kZero: return;
    case kConstant:
      for (auto& o : out) o = value;
      return;
    case kPerCell:
      for (auto& o : out) o = data[cell];
      return;
    case kPerCellExp:
      for (auto& o : out) o = std::exp(data[cell]);
      return;
    case kNodalO1: {
      // MeshFunctionFE over an O1 space: value = local dofs . shape values
      const bool q = m.IsQuad(cell);
      const int nv = m.NumVerts(cell);
      double phi[16], dphi[16][2];
      for (int k = 0; k < qr.n(); ++k) {
        EvalShape(q, 1, qr.x[k], qr.y[k], phi, dphi);
        double s = 0;
        for (int j = 0; j < nv; ++j) s += data[m.cell_nodes[cell][j]] * phi[j];
        out[k] = s;
      }
      return;
    }
    case kAnalytic: {
      const CellGeom g = m.Geom(cell);
      for (int k = 0; k < qr.n(); ++k) {
        double X[2];
        g.Global(qr.x[k], qr.y[k], X);
        out[k] = fn(X[0], X[1]);
      }
      return;
    }
  }
  throw Error("bad mesh function kind");
}

void MeshFunction::EvalTensor(const Mesh& m, idx_t cell, const QuadRule& qr,
                              std::vector<std::array<double, 4>>& out) const {
  out.assign(qr.n(), {0, 0, 0, 0});
  const CellGeom g = m.Geom(cell);
  for (int k = 0; k < qr.n(); ++k) {
    double X[2];
    g.Global(qr.x[k], qr.y[k], X);
    tensor_fn(cell, X[0], X[1], out[k].data());
  }
}

// ============================================================ providers ====
namespace {
void Tabulate(bool is_quad, int degree, const QuadRule& qr, std::vector<double>& phi,
              std::vector<double>& dphi) {
  const int n = NumShapeFunctions(is_quad, degree);
  phi.assign(static_cast<size_t>(n) * qr.n(), 0.0);
  dphi.assign(static_cast<size_t>(n) * qr.n() * 2, 0.0);
  double p[16], dp[16][2];
  for (int k = 0; k < qr.n(); ++k) {
    EvalShape(is_quad, degree, qr.x[k], qr.y[k], p, dp);
    for (int i = 0; i < n; ++i) {
      phi[k * n + i] = p[i];
      dphi[(k * n + i) * 2 + 0] = dp[i][0];
      dphi[(k * n + i) * 2 + 1] = dp[i][1];
    }
  }
}
}  // namespace

void RDProvider::Init() {
  if (have_tria) Tabulate(false, degree, qr_tria, phi_t, dphi_t);
  if (have_quad) Tabulate(true, degree, qr_quad, phi_q, dphi_q);
}

// ReactionDiffusionElementMatrixProvider::Eval (loc_comp_ellbvp.h:266-339).
void RDProvider::Eval(idx_t cell, std::vector<double>& mat) const {
  const bool q = mesh->IsQuad(cell);
  if ((q && !have_quad) || (!q && !have_tria))
    throw Error("No local shape function information or no quadrature rule for "
                "reference element type");  // loc_comp_ellbvp.h:278-287
  const QuadRule& qr = q ? qr_quad : qr_tria;
  const std::vector<double>& phi = q ? phi_q : phi_t;
  const std::vector<double>& dphi = q ? dphi_q : dphi_t;
  const int n = NumShapeFunctions(q, degree);
  const CellGeom g = mesh->Geom(cell);
  if (!NonDegenerate(g)) throw Error("degenerate cell " + std::to_string(cell));
  std::vector<double> av, gv;
  std::vector<std::array<double, 4>> at;
  if (alpha.IsTensor()) alpha.EvalTensor(*mesh, cell, qr, at);
  else alpha.Eval(*mesh, cell, qr, av);
  gamma.Eval(*mesh, cell, qr, gv);
  mat.assign(static_cast<size_t>(n) * n, 0.0);
  std::vector<double> G(2 * n), AG(2 * n);
  for (int k = 0; k < qr.n(); ++k) {
    const double w = qr.w[k] * g.IntegrationElement(qr.x[k], qr.y[k]);
    double JT[2][2];
    g.JinvT(qr.x[k], qr.y[k], JT);
    // trf_grad = JinvT * grad^T (2 x n)
    for (int i = 0; i < n; ++i) {
      const double gx = dphi[(k * n + i) * 2], gy = dphi[(k * n + i) * 2 + 1];
      G[i] = JT[0][0] * gx + JT[0][1] * gy;
      G[n + i] = JT[1][0] * gx + JT[1][1] * gy;
    }
    if (alpha.IsTensor()) {
      const auto& A = at[k];
      for (int i = 0; i < n; ++i) {
        AG[i] = A[0] * G[i] + A[1] * G[n + i];
        AG[n + i] = A[2] * G[i] + A[3] * G[n + i];
      }
    } else {
      for (int i = 0; i < 2 * n; ++i) AG[i] = av[k] * G[i];
    }
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) {
        const double gg = G[i] * AG[j] + G[n + i] * AG[n + j];
        const double mm = (gv[k] * phi[k * n + i]) * phi[k * n + j];
        mat[i * n + j] += w * (gg + mm);
      }
  }
}

void LoadProvider::Init() {
  std::vector<double> d;
  Tabulate(false, degree, qr_tria, phi_t, d);
  Tabulate(true, degree, qr_quad, phi_q, d);
}

// ScalarLoadElementVectorProvider::Eval (loc_comp_ellbvp.h:691-746).
void LoadProvider::Eval(idx_t cell, std::vector<double>& vec) const {
  const bool q = mesh->IsQuad(cell);
  const QuadRule& qr = q ? qr_quad : qr_tria;
  const std::vector<double>& phi = q ? phi_q : phi_t;
  const int n = NumShapeFunctions(q, degree);
  const CellGeom g = mesh->Geom(cell);
  std::vector<double> fv;
  f.Eval(*mesh, cell, qr, fv);
  vec.assign(n, 0.0);
  for (int k = 0; k < qr.n(); ++k) {
    const double s = qr.w[k] * g.IntegrationElement(qr.x[k], qr.y[k]) * fv[k];
    for (int i = 0; i < n; ++i) vec[i] += s * phi[k * n + i];
  }
}

// ============================================================ assembly ====

void AssembleMatrixLocally(const DofHandler& dh,
                           const std::function<void(idx_t, std::vector<double>&)>& eval,
                           COOMatrix& A) {
  std::vector<double> em;
  for (idx_t c = 0; c < dh.mesh->num_cells; ++c) {
    const int n = dh.NumLocalDofs(c);
    const idx_t* dofs = dh.GlobalDofIndices(c);
    eval(c, em);
    const int ld = static_cast<int>(std::lround(std::sqrt(static_cast<double>(em.size()))));
    if (ld < n) throw Error("element matrix too small");
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) A.AddToEntry(dofs[i], dofs[j], em[i * ld + j]);
  }
}

void AssembleVectorLocally(const DofHandler& dh,
                           const std::function<void(idx_t, std::vector<double>&)>& eval,
                           std::vector<double>& b) {
  std::vector<double> ev;
  for (idx_t c = 0; c < dh.mesh->num_cells; ++c) {
    const int n = dh.NumLocalDofs(c);
    const idx_t* dofs = dh.GlobalDofIndices(c);
    eval(c, ev);
    for (int i = 0; i < n; ++i) b[dofs[i]] += ev[i];
  }
}

// ============================================== boundary-edge providers ====

void EvalSegmentShape(int degree, double t, double* phi) {
  double d[4];
  if (degree == 1) {  // FeLagrangeO1Segment (lagr_fe.h:284-398)
    phi[0] = 1.0 - t;
    phi[1] = t;
  } else if (degree == 2) {
    SegO2(t, phi, d);
  } else if (degree == 3) {
    SegO3(t, phi, d);
  } else {
    throw Error("segment degree must be 1..3");
  }
}

void EvalOnEdge(const MeshFunction& f, const Mesh& m, idx_t e, const std::vector<double>& t,
                std::vector<double>& out) {
  const idx_t a = m.edge_nodes[e][0], b = m.edge_nodes[e][1];
  out.assign(t.size(), 0.0);
  for (size_t k = 0; k < t.size(); ++k) {
    switch (f.kind) {
      case MeshFunction::kZero: break;
      case MeshFunction::kConstant: out[k] = f.value; break;
      case MeshFunction::kPerCell: out[k] = f.data[e]; break;
      case MeshFunction::kPerCellExp: out[k] = std::exp(f.data[e]); break;
      case MeshFunction::kNodalO1: out[k] = f.data[a] * (1.0 - t[k]) + f.data[b] * t[k]; break;
      case MeshFunction::kAnalytic: {
        const double x = m.xy[2 * a] + t[k] * (m.xy[2 * b] - m.xy[2 * a]);
        const double y = m.xy[2 * a + 1] + t[k] * (m.xy[2 * b + 1] - m.xy[2 * a + 1]);
        out[k] = f.fn(x, y);
        break;
      }
      default: throw Error("bad mesh function kind on an edge");
    }
  }
}

namespace {
// Edge length |p1 - p0| (SegmentO1::IntegrationElement) and the segment
// Gauss rule of make_quad_rule.cc:22-27 (degree / 2 + 1 points on [0, 1]).
double EdgeLength(const Mesh& m, idx_t e) {
  const idx_t a = m.edge_nodes[e][0], b = m.edge_nodes[e][1];
  return std::hypot(m.xy[2 * b] - m.xy[2 * a], m.xy[2 * b + 1] - m.xy[2 * a + 1]);
}
}  // namespace

void AssembleEdgeMass(const DofHandler& dh, int degree, const MeshFunction& gamma, const uint8_t* flags, int qdeg,
                      COOMatrix& A) {
  std::vector<double> t, w, gv;
  GaussLegendre(qdeg / 2 + 1, t, w);
  const int n = dh.n_edge;
  std::vector<double> phi(t.size() * n), mat(n * n);
  for (size_t k = 0; k < t.size(); ++k) EvalSegmentShape(degree, t[k], &phi[k * n]);
  const Mesh& m = *dh.mesh;
  for (idx_t e = 0; e < m.num_edges; ++e) {
    if (flags && !flags[e]) continue;
    const double len = EdgeLength(m, e);
    EvalOnEdge(gamma, m, e, t, gv);
    std::fill(mat.begin(), mat.end(), 0.0);
    for (size_t k = 0; k < t.size(); ++k) {
      const double s = (w[k] * len) * gv[k];
      for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) mat[i * n + j] += phi[k * n + i] * phi[k * n + j] * s;
    }
    const idx_t* dofs = &dh.edge_dofs[e * n];
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) A.AddToEntry(dofs[i], dofs[j], mat[i * n + j]);
  }
}

void AssembleEdgeLoad(const DofHandler& dh, int degree, const MeshFunction& g, const uint8_t* flags, int qdeg,
                      std::vector<double>& b) {
  std::vector<double> t, w, gv;
  GaussLegendre(qdeg / 2 + 1, t, w);
  const int n = dh.n_edge;
  std::vector<double> phi(t.size() * n), vec(n);
  for (size_t k = 0; k < t.size(); ++k) EvalSegmentShape(degree, t[k], &phi[k * n]);
  const Mesh& m = *dh.mesh;
  for (idx_t e = 0; e < m.num_edges; ++e) {
    if (flags && !flags[e]) continue;
    const double len = EdgeLength(m, e);
    EvalOnEdge(g, m, e, t, gv);
    std::fill(vec.begin(), vec.end(), 0.0);
    for (size_t k = 0; k < t.size(); ++k) {
      const double s = (w[k] * len) * gv[k];
      for (int i = 0; i < n; ++i) vec[i] += phi[k * n + i] * s;
    }
    const idx_t* dofs = &dh.edge_dofs[e * n];
    for (int i = 0; i < n; ++i) b[dofs[i]] += vec[i];
  }
}

void FixFlaggedSolutionComponents(const uint8_t* flags, const double* values,
                                  COOMatrix& A, std::vector<double>& b) {
  const idx_t N = A.cols;
  {
    std::vector<double> tmp(N);
    for (idx_t k = 0; k < N; ++k) tmp[k] = flags[k] ? values[k] : 0.0;
    // MatVecMult(-1.0, tmp, b) (coomatrix.h:248-260)
    for (const Triplet& t : A.triplets) b[t.row] += t.value * (-1.0 * tmp[t.col]);
  }
  for (idx_t k = 0; k < N; ++k)
    if (flags[k]) b[k] = values[k];
  // setZero(pred): order-preserving std::remove_if (coomatrix.h:108-115)
  auto last = std::remove_if(A.triplets.begin(), A.triplets.end(), [&](const Triplet& t) {
    return flags[t.row] || flags[t.col];
  });
  A.triplets.erase(last, A.triplets.end());
  for (idx_t k = 0; k < N; ++k)
    if (flags[k]) A.AddToEntry(k, k, 1.0);
}

void FixFlaggedSolutionCompAlt(const uint8_t* flags, const double* values,
                               COOMatrix& A, std::vector<double>& b) {
  const idx_t N = A.cols;
  for (idx_t k = 0; k < N; ++k)
    if (flags[k]) b[k] = values[k];
  auto last = std::remove_if(A.triplets.begin(), A.triplets.end(),
                             [&](const Triplet& t) { return flags[t.row] != 0; });
  A.triplets.erase(last, A.triplets.end());
  for (idx_t k = 0; k < N; ++k)
    if (flags[k]) A.AddToEntry(k, k, 1.0);
}

void FixSolutionComponentsLse(const std::vector<std::pair<idx_t, double>>& fixed, COOMatrix& A,
                              std::vector<double>& b) {
  const idx_t N = A.cols;
  if (A.rows != N) throw Error("Matrix must be square!");
  std::vector<double> fixed_vec(N, 0.0);
  std::vector<uint8_t> flags(N, 0);
  for (const auto& iv : fixed) {
    if (iv.first < 0 || iv.first >= N) throw Error("FixSolutionComponentsLse: index out of range");
    fixed_vec[iv.first] += iv.second;
    flags[iv.first] = 1;
  }
  FixFlaggedSolutionCompAlt(flags.data(), fixed_vec.data(), A, b);
}

void MakeSparseCSR(const COOMatrix& A, std::vector<int64_t>& rowptr,
                   std::vector<int32_t>& colind, std::vector<double>& val) {
  const size_t nt = A.triplets.size();
  std::vector<size_t> perm(nt);
  std::iota(perm.begin(), perm.end(), 0);
  std::stable_sort(perm.begin(), perm.end(), [&](size_t a, size_t b) {
    const Triplet &x = A.triplets[a], &y = A.triplets[b];
    return x.row != y.row ? x.row < y.row : x.col < y.col;
  });
  rowptr.assign(A.rows + 1, 0);
  colind.clear();
  val.clear();
  for (size_t k = 0; k < nt; ++k) {
    const Triplet& t = A.triplets[perm[k]];
    if (!colind.empty() && k > 0) {
      const Triplet& p = A.triplets[perm[k - 1]];
      if (p.row == t.row && p.col == t.col) {
        val.back() = val.back() + t.value;  // collapseDuplicates: acc + next
        continue;
      }
    }
    colind.push_back(t.col);
    val.push_back(t.value);
    rowptr[t.row + 1]++;
  }
  for (idx_t r = 0; r < A.rows; ++r) rowptr[r + 1] += rowptr[r];
}

void NodalProjection(const DofHandler& dh, int degree,
                     const std::function<double(double, double)>& u,
                     std::vector<double>& out) {
  out.assign(dh.num_dofs, 0.0);
  std::vector<double> nodes;
  for (idx_t c = 0; c < dh.mesh->num_cells; ++c) {
    const bool q = dh.mesh->IsQuad(c);
    EvaluationNodes(q, degree, nodes);
    const CellGeom g = dh.mesh->Geom(c);
    const int n = dh.NumLocalDofs(c);
    const idx_t* dofs = dh.GlobalDofIndices(c);
    for (int j = 0; j < n; ++j) {
      double X[2];
      g.Global(nodes[2 * j], nodes[2 * j + 1], X);
      out[dofs[j]] = u(X[0], X[1]);
    }
  }
}

// ====================================================== post-processing ====

namespace {
// u and grad u of a mesh function at reference point (xh, yh) of a cell
// (grad only where defined: analytic families, O1 interpolant; cell-wise
// constants have zero gradient).
void MFPoint(const MeshFunction& u, const std::function<void(double, double, double*)>& grad_u, const Mesh& m,
             idx_t c, const CellGeom& geo, double xh, double yh, double* val, double* grad) {
  double X[2];
  geo.Global(xh, yh, X);
  double g[2] = {0.0, 0.0};
  double v = 0.0;
  switch (u.kind) {
    case MeshFunction::kZero: break;
    case MeshFunction::kConstant: v = u.value; break;
    case MeshFunction::kPerCell: v = u.data[c]; break;
    case MeshFunction::kPerCellExp: v = std::exp(u.data[c]); break;
    case MeshFunction::kNodalO1: {
      double phi[16], dphi[16][2], JT[2][2];
      EvalShape(m.IsQuad(c), 1, xh, yh, phi, dphi);
      double gh[2] = {0.0, 0.0};
      for (int j = 0; j < m.NumVerts(c); ++j) {
        const double d = u.data[m.cell_nodes[c][j]];
        v += d * phi[j];
        gh[0] += d * dphi[j][0];
        gh[1] += d * dphi[j][1];
      }
      geo.JinvT(xh, yh, JT);
      g[0] = JT[0][0] * gh[0] + JT[0][1] * gh[1];
      g[1] = JT[1][0] * gh[0] + JT[1][1] * gh[1];
      break;
    }
    case MeshFunction::kAnalytic:
      v = u.fn(X[0], X[1]);
      if (grad && grad_u) grad_u(X[0], X[1], g);
      break;
    default: throw Error("bad mesh function kind");
  }
  *val = v;
  if (grad) { grad[0] = g[0]; grad[1] = g[1]; }
}

// u_h and grad u_h (mesh_function_fe.h:72-91, mesh_function_grad_fe.h:93-118)
int HierCellDegrees(const DofHandler& dh, idx_t c, int p, int& pc, int (&pe)[4]);

// MeshFunctionFE / MeshFunctionGradFE on a hierarchic space: the cell's
// FeHierarchicTria / Quad shape functions (its own degrees and orientations).
void FEPointHier(const DofHandler& dh, int p, const double* dofs, idx_t c, const CellGeom& geo, double xh, double yh,
                 double* val, double* grad) {
  const Mesh& m = *dh.mesh;
  const bool q = m.IsQuad(c);
  int pc, pe[4];
  HierCellDegrees(dh, c, p, pc, pe);
  int8_t ori[4];
  for (int j = 0; j < 4; ++j) ori[j] = m.cell_ori[c][j];
  const int n = HierNumShapeVar(q, pc, pe);
  std::vector<double> phi(n), dphi(2 * n);
  EvalHierShapeVar(q, pc, pe, ori, xh, yh, phi.data(), reinterpret_cast<double(*)[2]>(dphi.data()));
  const idx_t* d = dh.GlobalDofIndices(c);
  double v = 0.0, gh[2] = {0.0, 0.0};
  for (int i = 0; i < n; ++i) {
    v += dofs[d[i]] * phi[i];
    gh[0] += dofs[d[i]] * dphi[2 * i];
    gh[1] += dofs[d[i]] * dphi[2 * i + 1];
  }
  *val = v;
  if (grad) {
    double JT[2][2];
    geo.JinvT(xh, yh, JT);
    grad[0] = JT[0][0] * gh[0] + JT[0][1] * gh[1];
    grad[1] = JT[1][0] * gh[0] + JT[1][1] * gh[1];
  }
}

void FEPoint(const DofHandler& dh, int degree, const double* dofs, idx_t c, const CellGeom& geo, double xh,
             double yh, double* val, double* grad) {
  const bool q = dh.mesh->IsQuad(c);
  double phi[16], dphi[16][2], JT[2][2];
  EvalShape(q, degree, xh, yh, phi, dphi);
  const idx_t* d = dh.GlobalDofIndices(c);
  double v = 0.0, gh[2] = {0.0, 0.0};
  for (int i = 0; i < dh.NumLocalDofs(c); ++i) {
    v += dofs[d[i]] * phi[i];
    gh[0] += dofs[d[i]] * dphi[i][0];
    gh[1] += dofs[d[i]] * dphi[i][1];
  }
  *val = v;
  if (grad) {
    geo.JinvT(xh, yh, JT);
    grad[0] = JT[0][0] * gh[0] + JT[0][1] * gh[1];
    grad[1] = JT[1][0] * gh[0] + JT[1][1] * gh[1];
  }
}

double IntegrandAt(const Integrand& g, const Mesh& m, idx_t c, const CellGeom& geo, double xh, double yh) {
  const bool need_grad = g.kind == 2;
  double uv = 0.0, ug[2] = {0.0, 0.0}, hv = 0.0, hg[2] = {0.0, 0.0};
  MFPoint(g.u, g.grad_u, m, c, geo, xh, yh, &uv, need_grad ? ug : nullptr);
  if (g.dofs && g.hier >= 0) FEPointHier(*g.dh, g.hier, g.dofs, c, geo, xh, yh, &hv, need_grad ? hg : nullptr);
  else if (g.dofs) FEPoint(*g.dh, g.degree, g.dofs, c, geo, xh, yh, &hv, need_grad ? hg : nullptr);
  switch (g.kind) {
    case 0: return hv + uv;
    case 1: return (hv - uv) * (hv - uv);
    case 2: {
      const double a = hg[0] - ug[0], b = hg[1] - ug[1];
      return a * a + b * b;
    }
  }
  throw Error("bad integrand kind");
}

// LocalIntegral (fe_tools.h:35-68): values . (weights .* IntegrationElement)
double LocalCell(const Integrand& g, const Mesh& m, idx_t c, const QuadRule& qt, const QuadRule& qq) {
  const CellGeom geo = m.Geom(c);
  const QuadRule& qr = m.IsQuad(c) ? qq : qt;
  double s = 0.0;
  for (int k = 0; k < qr.n(); ++k)
    s += IntegrandAt(g, m, c, geo, qr.x[k], qr.y[k]) * (qr.w[k] * geo.IntegrationElement(qr.x[k], qr.y[k]));
  return s;
}

double LocalEdge(const Integrand& g, const Mesh& m, idx_t e, const std::vector<double>& t,
                 const std::vector<double>& w) {
  const idx_t a = m.edge_nodes[e][0], b = m.edge_nodes[e][1];
  const double len = std::hypot(m.xy[2 * b] - m.xy[2 * a], m.xy[2 * b + 1] - m.xy[2 * a + 1]);
  std::vector<double> uv;
  EvalOnEdge(g.u, m, e, t, uv);
  const int n = g.dofs ? g.dh->n_edge : 0;
  std::vector<double> phi(n);
  double s = 0.0;
  for (size_t k = 0; k < t.size(); ++k) {
    double hv = 0.0;
    if (g.dofs) {
      EvalSegmentShape(g.degree, t[k], phi.data());
      const idx_t* d = &g.dh->edge_dofs[e * n];
      for (int i = 0; i < n; ++i) hv += g.dofs[d[i]] * phi[i];
    }
    const double v = g.kind == 0 ? hv + uv[k] : (hv - uv[k]) * (hv - uv[k]);
    s += v * (w[k] * len);
  }
  return s;
}
}  // namespace

double IntegrateMeshFunction(const Mesh& m, const Integrand& g, int qdeg, const uint8_t* flags, int codim) {
  if (codim == 0) {
    const QuadRule qt = MakeQuadRule(false, qdeg), qq = MakeQuadRule(true, qdeg);
    if (m.num_cells == 0) return 0.0;
    // fe_tools.h:117-124: entity 0 starts the sum unconditionally
    double r = LocalCell(g, m, 0, qt, qq);
    for (idx_t c = 1; c < m.num_cells; ++c) {
      if (flags && !flags[c]) continue;
      r = r + LocalCell(g, m, c, qt, qq);
    }
    return r;
  }
  if (codim != 1) throw Error("IntegrateMeshFunction: codim must be 0 or 1");
  if (g.kind == 2) throw Error("IntegrateMeshFunction: gradients on edges are not supported");
  if (g.dofs && g.hier >= 0) throw Error("IntegrateMeshFunction: hierarchic u_h on edges is not supported");
  std::vector<double> t, w;
  GaussLegendre(qdeg / 2 + 1, t, w);
  if (m.num_edges == 0) return 0.0;
  double r = LocalEdge(g, m, 0, t, w);
  for (idx_t e = 1; e < m.num_edges; ++e) {
    if (flags && !flags[e]) continue;
    r = r + LocalEdge(g, m, e, t, w);
  }
  return r;
}

void EvalFE(const DofHandler& dh, int degree, const double* dofs, idx_t cell, const std::vector<double>& xy,
            double* vals, double* grads) {
  const CellGeom geo = dh.mesh->Geom(cell);
  const size_t np = xy.size() / 2;
  for (size_t k = 0; k < np; ++k) {
    double v, g[2];
    FEPoint(dh, degree, dofs, cell, geo, xy[2 * k], xy[2 * k + 1], &v, grads ? g : nullptr);
    if (vals) vals[k] = v;
    if (grads) { grads[2 * k] = g[0]; grads[2 * k + 1] = g[1]; }
  }
}

void EvalFEHier(const DofHandler& dh, int p, const double* dofs, idx_t cell, const std::vector<double>& xy,
                double* vals, double* grads) {
  const CellGeom geo = dh.mesh->Geom(cell);
  const size_t np = xy.size() / 2;
  for (size_t k = 0; k < np; ++k) {
    double v, g[2];
    FEPointHier(dh, p, dofs, cell, geo, xy[2 * k], xy[2 * k + 1], &v, grads ? g : nullptr);
    if (vals) vals[k] = v;
    if (grads) {
      grads[2 * k] = g[0];
      grads[2 * k + 1] = g[1];
    }
  }
}

void NodalProjectionMF(const DofHandler& dh, int degree, const MeshFunction& u, const uint8_t* cell_flags,
                       std::vector<double>& out) {
  out.assign(dh.num_dofs, 0.0);
  std::vector<double> nodes;
  const Mesh& m = *dh.mesh;
  for (idx_t c = 0; c < m.num_cells; ++c) {
    if (cell_flags && !cell_flags[c]) continue;
    EvaluationNodes(m.IsQuad(c), degree, nodes);
    QuadRule pts;  // the evaluation nodes as points of a (weightless) rule
    pts.x.resize(nodes.size() / 2);
    pts.y.resize(nodes.size() / 2);
    pts.w.assign(nodes.size() / 2, 0.0);
    for (size_t j = 0; j < nodes.size() / 2; ++j) {
      pts.x[j] = nodes[2 * j];
      pts.y[j] = nodes[2 * j + 1];
    }
    std::vector<double> v;
    u.Eval(m, c, pts, v);
    const idx_t* d = dh.GlobalDofIndices(c);
    // NodalValuesToDofs of a Lagrangian element is the identity; "setting,
    // not adding": a later cell overwrites a shared dof
    for (int j = 0; j < dh.NumLocalDofs(c); ++j) out[d[j]] = v[j];
  }
}

void InitEssentialCondition(const DofHandler& dh, int degree, const uint8_t* edge_flags, const MeshFunction& g,
                            std::vector<uint8_t>& flags, std::vector<double>& vals) {
  flags.assign(dh.num_dofs, 0);
  vals.assign(dh.num_dofs, 0.0);
  const Mesh& m = *dh.mesh;
  const int n = dh.n_edge;
  // segment evaluation nodes: 0, 1, then the interior nodes 1/p .. (p-1)/p
  std::vector<double> t = {0.0, 1.0};
  for (int a = 1; a < degree; ++a) t.push_back(static_cast<double>(a) / degree);
  std::vector<double> v;
  for (idx_t e = 0; e < m.num_edges; ++e) {
    if (edge_flags && !edge_flags[e]) continue;
    EvalOnEdge(g, m, e, t, v);
    const idx_t* d = &dh.edge_dofs[e * n];
    for (int i = 0; i < n; ++i) {
      flags[d[i]] = 1;
      vals[d[i]] = v[i];
    }
  }
}

}  // namespace lfo

// ====================================================== hierarchic (hp) FE ==
namespace lfo {

// fe/hierarchic_fe.cc:10-27 -- shifted, scaled Legendre polynomials by their
// three-term recurrence.
double HierLegendre(unsigned n, double x, double t) {
  if (n == 0) return 1.0;
  if (n == 1) return 2 * x - t;
  double pm = 1.0, pc = 2 * x - t;
  for (unsigned i = 2; i <= n; ++i) {
    const double pn = (2.0 * i - 1) * (2 * x - t) / i * pc - (i - 1.0) * t * t / i * pm;
    pm = pc;
    pc = pn;
  }
  return pc;
}

// fe/hierarchic_fe.cc:29-45
double HierILegendre(unsigned n, double x, double t) {
  if (n == 1) return x;
  return (HierLegendre(n, x, t) - t * t * HierLegendre(n - 2, x, t)) / (2.0 * (2.0 * n - 1));
}
double HierILegendreDx(unsigned n, double x, double t) { return HierLegendre(n - 1, x, t); }
double HierILegendreDt(unsigned n, double x, double t) {
  if (n == 1) return 0.0;
  return -0.5 * (HierLegendre(n - 1, x, t) + t * HierLegendre(n - 2, x, t));
}

// fe/hierarchic_fe.cc:55-81 -- Jacobi polynomials P_n^(alpha,beta)(2x - 1).
double HierJacobi(unsigned n, double alpha, double beta, double x) {
  x = 2 * x - 1;
  if (n == 0) return 1.0;
  const double ab = alpha + beta;
  double p0 = 1.0, p1 = 0.5 * (alpha - beta + x * (ab + 2));
  for (unsigned j = 1; j < n; ++j) {
    const double a1 = 2 * (j + 1) * (j + ab + 1) * (2 * j + ab);
    const double a2 = (2 * j + ab + 1) * (alpha * alpha - beta * beta);
    const double a3 = (2 * j + ab) * (2 * j + ab + 1) * (2 * j + ab + 2);
    const double a4 = 2 * (j + alpha) * (j + beta) * (2 * j + ab + 2);
    const double p2 = ((a2 + a3 * x) * p1 - a4 * p0) / a1;
    p0 = p1;
    p1 = p2;
  }
  return p1;
}

// fe/hierarchic_fe.cc:87-127 -- integrated Jacobi polynomials through the
// recurrence of P^(alpha-1, 0)-type terms and the final three-term
// combination of that file.
double HierIJacobi(unsigned n, double alpha, double x) {
  if (n == 0) return -1.0;
  if (n == 1) return x;
  auto coef = [alpha](unsigned j, double& a, double& b, double& c, double& d) {
    a = 2.0 * j * (j + alpha) * (2.0 * j + alpha - 2);
    b = 2.0 * j + alpha - 1;
    c = (2.0 * j + alpha) * (2.0 * j + alpha - 2);
    d = 2.0 * (j + alpha - 1) * (j - 1.0) * (2.0 * j + alpha);
  };
  double a, b, c, d;
  double q2 = 1.0, q1 = (2 + alpha) * x - 1;  // terms j-2, j-1
  coef(2, a, b, c, d);
  double q0 = (b * (c * (2 * x - 1) + alpha * alpha) * q1 - d * q2) / a;
  for (unsigned j = 2; j < n; ++j) {
    coef(j + 1, a, b, c, d);
    const double qn = (b * (c * (2 * x - 1) + alpha * alpha) * q0 - d * q1) / a;
    q2 = q1;
    q1 = q0;
    q0 = qn;
  }
  const double an = (n + alpha) / ((2.0 * n + alpha - 1) * (2.0 * n + alpha));
  const double bn = alpha / ((2.0 * n + alpha - 2) * (2.0 * n + alpha));
  const double cn = (n - 1.0) / ((2.0 * n + alpha - 2) * (2.0 * n + alpha - 1));
  return an * q0 + bn * q1 - cn * q2;
}

void EvalHierShape(bool is_quad, int p, const int8_t* ori, double x, double y, double* phi, double (*dphi)[2]) {
  const int pe[4] = {p, p, p, p};
  EvalHierShapeVar(is_quad, p, pe, ori, x, y, phi, dphi);
}

int HierNumShapeVar(bool is_quad, int pc, const int* pe) {
  const int nv = is_quad ? 4 : 3;
  int n = nv;
  for (int j = 0; j < nv; ++j) n += pe[j] - 1;
  // NumRefShapeFunctions(0) (hierarchic_fe.h:528-535, :1198-1205)
  n += is_quad ? (pc - 1) * (pc - 1) : (pc <= 2 ? 0 : (pc - 2) * (pc - 1) / 2);
  return n;
}

void EvalHierShapeVar(bool is_quad, int pc, const int* pe, const int8_t* ori, double x, double y, double* phi,
                      double (*dphi)[2]) {
  if (!is_quad) {
    // FeHierarchicTria::EvalReferenceShapeFunctions / Gradients... (hierarchic_fe.h:576-870)
    const double l[3] = {1 - x - y, x, y};
    const double g[3][2] = {{-1, -1}, {1, 0}, {0, 1}};
    for (int v = 0; v < 3; ++v) {
      phi[v] = l[v];
      dphi[v][0] = g[v][0];
      dphi[v][1] = g[v][1];
    }
    int cur = 3;
    for (int e = 0; e < 3; ++e) {
      const int a = e, b = (e + 1) % 3;
      const double t = l[a] + l[b];
      const double tx = g[a][0] + g[b][0], ty = g[a][1] + g[b][1];
      const int p = pe[e];
      for (int i = 0; i < p - 1; ++i) {
        const int src = ori[e] > 0 ? b : a;
        const int row = ori[e] > 0 ? cur + i : cur + p - 2 - i;
        phi[row] = HierILegendre(i + 2, l[src], t);
        const double lx = HierILegendreDx(i + 2, l[src], t), lt = HierILegendreDt(i + 2, l[src], t);
        dphi[row][0] = lx * g[src][0] + lt * tx;
        dphi[row][1] = lx * g[src][1] + lt * ty;
      }
      cur += p - 1;
    }
    const int p = pc;
    if (p > 2) {
      const int src = ori[0] > 0 ? 1 : 0;
      const double t = l[0] + l[1];
      for (int i = 0; i < p - 2; ++i) {
        const double ev = HierILegendre(i + 2, l[src], t);
        const double lx = HierILegendreDx(i + 2, l[src], t), lt = HierILegendreDt(i + 2, l[src], t);
        const double ex = lx * g[src][0] + lt * (g[0][0] + g[1][0]);
        const double ey = lx * g[src][1] + lt * (g[0][1] + g[1][1]);
        for (int j = 0; j < p - i - 2; ++j) {
          const double ji = HierIJacobi(j + 1, 2.0 * i + 4, l[2]);
          const double jd = HierJacobi(j, 2.0 * i + 4, 0.0, l[2]);  // IJacobiDx(j+1) = Jacobi(j)
          phi[cur] = ev * ji;
          dphi[cur][0] = ji * ex + ev * jd * g[2][0];
          dphi[cur][1] = ji * ey + ev * jd * g[2][1];
          ++cur;
        }
      }
    }
    return;
  }
  // FeHierarchicQuad (hierarchic_fe.h:1238-1430): products of the segment
  // functions s_0 = 1 - t, s_1 = t, s_k = ILegendre(k, t), in x, y, 1-x, 1-y.
  auto s = [](int k, double t) { return k == 0 ? 1 - t : k == 1 ? t : HierILegendre(k, t); };
  auto ds = [](int k, double t) { return k == 0 ? -1.0 : k == 1 ? 1.0 : HierILegendreDx(k, t); };
  auto term = [&](int row, int kx, double sx, double sgnx, int ky, double sy, double sgny) {
    phi[row] = s(kx, sx) * s(ky, sy);
    dphi[row][0] = sgnx * ds(kx, sx) * s(ky, sy);
    dphi[row][1] = s(kx, sx) * sgny * ds(ky, sy);
  };
  term(0, 0, x, 1, 0, y, 1);
  term(1, 1, x, 1, 0, y, 1);
  term(2, 1, x, 1, 1, y, 1);
  term(3, 0, x, 1, 1, y, 1);
  int cur = 4;
  for (int i = 0; i < pe[0] - 1; ++i) {
    if (ori[0] > 0) term(cur + i, 2 + i, x, 1, 0, y, 1);
    else term(cur + pe[0] - 2 - i, 2 + i, 1 - x, -1, 0, y, 1);
  }
  cur += pe[0] - 1;
  for (int i = 0; i < pe[1] - 1; ++i) {
    if (ori[1] > 0) term(cur + i, 1, x, 1, 2 + i, y, 1);
    else term(cur + pe[1] - 2 - i, 1, x, 1, 2 + i, 1 - y, -1);
  }
  cur += pe[1] - 1;
  for (int i = 0; i < pe[2] - 1; ++i) {
    if (ori[2] > 0) term(cur + i, 2 + i, 1 - x, -1, 1, y, 1);
    else term(cur + pe[2] - 2 - i, 2 + i, x, 1, 1, y, 1);
  }
  cur += pe[2] - 1;
  for (int i = 0; i < pe[3] - 1; ++i) {
    if (ori[3] > 0) term(cur + i, 0, x, 1, 2 + i, 1 - y, -1);
    else term(cur + pe[3] - 2 - i, 0, x, 1, 2 + i, y, 1);
  }
  cur += pe[3] - 1;
  for (int i = 0; i < pc - 1; ++i)
    for (int j = 0; j < pc - 1; ++j) term(cur++, j + 2, x, 1, i + 2, y, 1);
}

namespace {

// Degrees of cell c: uniform p, or the cell's and its edges' own degrees on a
// variable-degree space; returns the cell's Degree() (hierarchic_fe.h:506-509).
int HierCellDegrees(const DofHandler& dh, idx_t c, int p, int& pc, int (&pe)[4]) {
  const Mesh& m = *dh.mesh;
  pc = p;
  for (int j = 0; j < 4; ++j) pe[j] = p;
  if (dh.cell_deg.empty()) return std::max(p, 1);
  pc = dh.cell_deg[c];
  int deg = std::max(pc, 1);
  for (int j = 0; j < m.NumVerts(c); ++j) {
    pe[j] = dh.edge_deg[m.cell_edges[c][j]];
    deg = std::max(deg, pe[j]);
  }
  return deg;
}

void HierCellData(const DofHandler& dh, idx_t c, int p, int qdeg, std::vector<double>& phi, std::vector<double>& dphi,
                  QuadRule& qr) {
  const Mesh& m = *dh.mesh;
  const bool q = m.IsQuad(c);
  int pc, pe[4];
  const int deg = HierCellDegrees(dh, c, p, pc, pe);
  qr = MakeQuadRule(q, qdeg > 0 ? qdeg : 2 * deg);
  int8_t ori[4];
  for (int j = 0; j < 4; ++j) ori[j] = m.cell_ori[c][j];
  const int n = HierNumShapeVar(q, pc, pe);
  phi.assign(static_cast<size_t>(qr.n()) * n, 0.0);
  dphi.assign(static_cast<size_t>(qr.n()) * n * 2, 0.0);
  for (int k = 0; k < qr.n(); ++k)
    EvalHierShapeVar(q, pc, pe, ori, qr.x[k], qr.y[k], &phi[k * n],
                     reinterpret_cast<double(*)[2]>(&dphi[static_cast<size_t>(k) * n * 2]));
}
}  // namespace

// ---- NodalProjection on hierarchic spaces (fe/fe_tools.h:198-259 with the
// EvaluationNodes / NodalValuesToDofs of FeHierarchicSegment, FeHierarchicTria
// and FeHierarchicQuad, hierarchic_fe.h:330-390, 820-1060, 1445-1680).
namespace {
// LegendreDx / JacobiDx / IJacobiDx of hierarchic_fe.cc:53-60, 170-185 (t = 1).
double HLegendreDx(unsigned n, double x) {
  if (n == 0) return 0.0;
  return 2.0 * n * HierLegendre(n - 1, x) + (2.0 * x - 1.0) * HLegendreDx(n - 1, x);
}
double HJacobiDx(unsigned n, double alpha, double x) {
  if (n == 0) return 0.0;
  return HierJacobi(n - 1, alpha + 1, 1, x) * (alpha + n + 1);
}
double HIJacobiDx(unsigned n, double alpha, double x) { return HierJacobi(n - 1, alpha, 0, x); }

// The segment rule of degree d (make_quad_rule.cc:22-27): Gauss-Legendre
// with d/2 + 1 points on [0, 1].
void SegmentRule(int d, std::vector<double>& t, std::vector<double>& w) { GaussLegendre(d / 2 + 1, t, w); }

// FeHierarchicSegment(p)::NodalValuesToDofs (hierarchic_fe.h:367-390):
// values at 0, 1 and the points of the segment rule of degree 2(p-1).
void SegmentValuesToDofs(int p, const double* v, double* dofs) {
  std::vector<double> t, w;
  SegmentRule(2 * (p - 1), t, w);
  dofs[0] = v[0];
  dofs[1] = v[1];
  for (int i = 2; i <= p; ++i) {
    const double P0 = HierILegendreDx(i, 0.0), P1 = HierILegendreDx(i, 1.0);
    double integ = 0.0;
    for (size_t q = 0; q < t.size(); ++q) integ += w[q] * HLegendreDx(i - 1, t[q]) * v[2 + q];
    dofs[i] = (P1 * v[1] - P0 * v[0] - integ) * (2 * i - 1);
  }
}

// Edge dofs of one local edge (degree pe >= 2) from the values at its two
// end vertices (va: start of the local edge, vb: its end) and at its rule
// points, written in the cell's slots: positive orientation in order,
// negative reversed (hierarchic_fe.h:938-1017, 1560-1637).
void EdgeValuesToDofs(int pe, bool positive, double va, double vb, const double* vals, double* out) {
  std::vector<double> t, w;
  SegmentRule(2 * (pe - 1), t, w);
  for (int i = 2; i <= pe; ++i) {
    const double P0 = HierILegendreDx(i, 0.0), P1 = HierILegendreDx(i, 1.0);
    double integ = 0.0;
    for (size_t q = 0; q < t.size(); ++q) integ += w[q] * HLegendreDx(i - 1, t[q]) * vals[q];
    if (positive) out[i - 2] = (P1 * vb - P0 * va - integ) * (2 * i - 1);
    else out[pe - i] = (P1 * va - P0 * vb - integ) * (2 * i - 1);
  }
}

// FeHierarchicTria::NodalValuesToFaceDofs (hierarchic_fe.h:1024-1083): the
// interior values are v[off ..].
void TriaFaceDofs(int pc, bool ori0_positive, const double* v, int off, double* out) {
  if (pc <= 2) return;
  const QuadRule qt = MakeQuadRule(false, 2 * (pc - 1));
  int idx = 0;
  for (int i = 0; i < pc - 2; ++i)
    for (int j = 0; j < pc - i - 2; ++j) {
      double s = 0.0;
      for (int q = 0; q < qt.n(); ++q) {
        const double x = qt.x[q], y = qt.y[q];
        const double xn = x / (1.0 - y);
        const double xa = ori0_positive ? xn : 1.0 - xn;
        const double ypow = std::pow(1.0 - y, i), ypowp1 = std::pow(1.0 - y, i + 1);
        const double psidd = HLegendreDx(i + 1, xa);
        const double jacdd = HJacobiDx(j, 2 * i + 4, y), jacd = HIJacobiDx(j + 1, 2 * i + 4, y);
        s += qt.w[q] * v[off + q] * psidd * (ypowp1 * jacdd - (2 * i + 4) * ypow * jacd);
      }
      out[idx++] = s * (2 * i + 3) * (2 * j + 2 * i + 5);
    }
}
}  // namespace

void HierEvaluationNodes(bool is_quad, int pc, const int* pe, const int8_t* ori, std::vector<double>& xy) {
  xy.clear();
  auto add = [&](double x, double y) {
    xy.push_back(x);
    xy.push_back(y);
  };
  std::vector<double> t, w;
  if (!is_quad) {  // hierarchic_fe.h:828-878
    add(0, 0);
    add(1, 0);
    add(0, 1);
    for (int j = 0; j < 3; ++j) {
      if (pe[j] <= 1) continue;
      SegmentRule(2 * (pe[j] - 1), t, w);
      for (double u : t) {
        if (j == 0) add(ori[0] > 0 ? u : 1 - u, 0);
        else if (j == 1) ori[1] > 0 ? add(1 - u, u) : add(u, 1 - u);
        else add(0, ori[2] > 0 ? 1 - u : u);
      }
    }
    const QuadRule qt = MakeQuadRule(false, 2 * (pc - 1));
    for (int q = 0; q < qt.n(); ++q) add(qt.x[q], qt.y[q]);
    return;
  }
  add(0, 0);  // hierarchic_fe.h:1452-1525
  add(1, 0);
  add(1, 1);
  add(0, 1);
  for (int j = 0; j < 4; ++j) {
    if (pe[j] <= 1) continue;
    SegmentRule(2 * (pe[j] - 1), t, w);
    for (double u : t) {
      if (j == 0) add(ori[0] > 0 ? u : 1 - u, 0);
      else if (j == 1) add(1, ori[1] > 0 ? u : 1 - u);
      else if (j == 2) add(ori[2] > 0 ? 1 - u : u, 1);
      else add(0, ori[3] > 0 ? 1 - u : u);
    }
  }
  if (pc > 1) {
    const int D = std::max({pc, pe[0], pe[1], pe[2], pe[3]});
    SegmentRule(2 * (D - 1), t, w);
    std::vector<double> pts = {0.0, 1.0};
    pts.insert(pts.end(), t.begin(), t.end());
    for (double yv : pts)
      for (double xv : pts) add(xv, yv);
  }
}

void HierNodalValuesToDofs(bool is_quad, int pc, const int* pe, const int8_t* ori, const std::vector<double>& v,
                           std::vector<double>& dofs) {
  const int nv = is_quad ? 4 : 3;
  const int n = HierNumShapeVar(is_quad, pc, pe);
  dofs.assign(n, 0.0);
  for (int k = 0; k < nv; ++k) dofs[k] = v[k];
  // edge dofs
  std::vector<double> t, w;
  int node = nv, slot = nv;
  for (int j = 0; j < nv; ++j) {
    if (pe[j] <= 1) continue;
    SegmentRule(2 * (pe[j] - 1), t, w);
    EdgeValuesToDofs(pe[j], ori[j] > 0, v[j], v[(j + 1) % nv], &v[node], &dofs[slot]);
    node += static_cast<int>(t.size());
    slot += pe[j] - 1;
  }
  if (!is_quad) {
    if (pc <= 2) return;
    // face dofs, then the boundary part of the function taken out of them
    // (hierarchic_fe.h:891-915)
    TriaFaceDofs(pc, ori[0] > 0, v.data(), node, &dofs[slot]);
    std::vector<double> xy;
    HierEvaluationNodes(false, pc, pe, ori, xy);
    const int ne = static_cast<int>(xy.size() / 2);
    std::vector<double> bf(ne, 0.0), phi(n), dphi(2 * n);
    for (int k = 0; k < ne; ++k) {
      EvalHierShapeVar(false, pc, pe, ori, xy[2 * k], xy[2 * k + 1], phi.data(),
                       reinterpret_cast<double(*)[2]>(dphi.data()));
      for (int a = 0; a < slot; ++a) bf[k] += dofs[a] * phi[a];
    }
    std::vector<double> bfd(n - slot, 0.0);
    TriaFaceDofs(pc, ori[0] > 0, bf.data(), node, bfd.data());
    for (int a = slot; a < n; ++a) dofs[a] -= bfd[a - slot];
    return;
  }
  if (pc <= 1) return;
  // face dofs of the quadrilateral (hierarchic_fe.h:1640-1665): the 1D dual of
  // degree D along x on every node row, then along y on every x-coefficient
  const int D = std::max({pc, pe[0], pe[1], pe[2], pe[3]});
  const int nq = D + 2, m = pc - 1;
  std::vector<double> row(D + 1), tmp(static_cast<size_t>(nq) * m), col(nq), res(D + 1);
  for (int i = 0; i < nq; ++i) {
    SegmentValuesToDofs(D, &v[node + nq * i], row.data());
    for (int a = 0; a < m; ++a) tmp[static_cast<size_t>(i) * m + a] = row[2 + a];
  }
  for (int a = 0; a < m; ++a) {  // dof_temp2 row a: the y-dual of the x-coefficient a
    for (int i = 0; i < nq; ++i) col[i] = tmp[static_cast<size_t>(i) * m + a];
    SegmentValuesToDofs(D, col.data(), res.data());
    for (int b = 0; b < m; ++b) dofs[slot + b * m + a] = res[2 + b];  // column-major flattening
  }
}

void NodalProjectionHier(const DofHandler& dh, int p, const MeshFunction& u, const uint8_t* cell_flags,
                         std::vector<double>& out) {
  const Mesh& m = *dh.mesh;
  out.assign(dh.num_dofs, 0.0);
  std::vector<double> xy, v, dofs;
  for (idx_t c = 0; c < m.num_cells; ++c) {
    if (cell_flags && !cell_flags[c]) continue;
    const bool q = m.IsQuad(c);
    int pc, pe[4];
    HierCellDegrees(dh, c, p, pc, pe);
    int8_t ori[4];
    for (int j = 0; j < 4; ++j) ori[j] = m.cell_ori[c][j];
    HierEvaluationNodes(q, pc, pe, ori, xy);
    QuadRule pts;
    pts.x.resize(xy.size() / 2);
    pts.y.resize(xy.size() / 2);
    pts.w.assign(xy.size() / 2, 0.0);
    for (size_t k = 0; k < xy.size() / 2; ++k) {
      pts.x[k] = xy[2 * k];
      pts.y[k] = xy[2 * k + 1];
    }
    u.Eval(m, c, pts, v);
    HierNodalValuesToDofs(q, pc, pe, ori, v, dofs);
    const idx_t* d = dh.GlobalDofIndices(c);
    for (int j = 0; j < dh.NumLocalDofs(c); ++j) out[d[j]] = dofs[j];  // set, not add
  }
}

void AssembleHierMatrix(const DofHandler& dh, int p, const MeshFunction& alpha, const MeshFunction& gamma,
                        int qdeg, COOMatrix& A) {
  const Mesh& m = *dh.mesh;
  std::vector<double> phi, dphi, av, gv, mat;
  QuadRule qr;
  AssembleMatrixLocally(dh, [&](idx_t c, std::vector<double>& out) {
    HierCellData(dh, c, p, qdeg, phi, dphi, qr);
    const int n = dh.NumLocalDofs(c);
    const CellGeom geo = m.Geom(c);
    alpha.Eval(m, c, qr, av);
    gamma.Eval(m, c, qr, gv);
    out.assign(static_cast<size_t>(n) * n, 0.0);
    std::vector<double> gx(n), gy(n);
    for (int k = 0; k < qr.n(); ++k) {
      const double w = qr.w[k] * geo.IntegrationElement(qr.x[k], qr.y[k]);
      double JT[2][2];
      geo.JinvT(qr.x[k], qr.y[k], JT);
      for (int i = 0; i < n; ++i) {
        const double* d = &dphi[(static_cast<size_t>(k) * n + i) * 2];
        gx[i] = JT[0][0] * d[0] + JT[0][1] * d[1];
        gy[i] = JT[1][0] * d[0] + JT[1][1] * d[1];
      }
      for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j)
          out[i * n + j] += w * (gx[i] * (av[k] * gx[j]) + gy[i] * (av[k] * gy[j])) +
                            w * (gv[k] * phi[k * n + i]) * phi[k * n + j];
    }
  }, A);
}

void AssembleHierLoad(const DofHandler& dh, int p, const MeshFunction& f, int qdeg, std::vector<double>& b) {
  const Mesh& m = *dh.mesh;
  std::vector<double> phi, dphi, fv;
  QuadRule qr;
  AssembleVectorLocally(dh, [&](idx_t c, std::vector<double>& out) {
    HierCellData(dh, c, p, qdeg, phi, dphi, qr);
    const int n = dh.NumLocalDofs(c);
    const CellGeom geo = m.Geom(c);
    f.Eval(m, c, qr, fv);
    out.assign(n, 0.0);
    for (int k = 0; k < qr.n(); ++k) {
      const double s = qr.w[k] * geo.IntegrationElement(qr.x[k], qr.y[k]) * fv[k];
      for (int i = 0; i < n; ++i) out[i] += s * phi[k * n + i];
    }
  }, b);
}

}  // namespace lfo
