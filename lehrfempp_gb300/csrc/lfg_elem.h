// Element matrices of ReactionDiffusionElementMatrixProvider for cells with
// cell-constant alpha / gamma (uscalfe/loc_comp_ellbvp.h:266-339), in df32
// arithmetic (lfg_df32.h).  Host + device code: the kernels in
// lfg_assemble.cu and the CPU precision test use these functions.
//
// Upper-triangle entry e = (i, j), i <= j, in the order
//   for i in 0..n-1: for j in i..n-1.
// Tables (built by lfg_tables.cc, split into binary32 pairs):
//   triangle  R[e][4]     = sum_k w_k {g_i0 g_j0, g_i0 g_j1 + g_i1 g_j0, g_i1 g_j1, phi_i phi_j}
//   quad      T[k][e][4]  = the same terms at point k (no weight), and per point
//             W[k] = w_k, 1D abscissae t[m] (points are x slow, y fast).
// With c = w |det J| alpha J^-1 J^-T = w alpha adj(J) adj(J)^T / |det J| the
// entries are  A(i,j) = sum_k c00 T0 + c01 T1 + c11 T2 + w |det J| gamma T3.
#pragma once

#include "lfg_df32.h"

#if defined(__CUDACC__)
#define DF_UNROLL _Pragma("unroll")
#define DF_NOUNROLL _Pragma("unroll 1")
#else
#define DF_UNROLL
#define DF_NOUNROLL
#endif

namespace lfg {
namespace elem {

using df::f2;

// df32 is used when the cell's inputs keep every intermediate in binary32
// range; other cells take the FP64 route.
DF_HD bool DfSafe(double x) {
  const double a = x < 0 ? -x : x;
  return a == 0.0 || (a >= 9.094947017729282e-13 && a <= 1.099511627776e12);  // [2^-40, 2^40]
}

// ------------------------------------------------------------------ triangles

// |det J| J^-1 J^-T (3 entries) and |det J| of the affine map with columns
// (j00, j10) = v1 - v0 and (j01, j11) = v2 - v0 (geometry/tria_o1.cc:56-61).
DF_HD void TriaMetricDF(f2 j00, f2 j01, f2 j10, f2 j11, f2& m00, f2& m01, f2& m11, f2& adet) {
  using namespace df;
  const f2 det = Sub(Mul(j00, j11), Mul(j10, j01));
  adet = Abs(det);
  const f2 r = Rcp(adet);
  m00 = Mul(Add(Mul(j11, j11), Mul(j01, j01)), r);
  m01 = Neg(Mul(Add(Mul(j11, j10), Mul(j01, j00)), r));
  m11 = Mul(Add(Mul(j10, j10), Mul(j00, j00)), r);
}

// Upper triangle of the triangle element matrix, E = n(n+1)/2 values.
template <int E, bool MASS>
DF_HD void TriaUniformDF(const double (&jac)[4] /* j00, j01, j10, j11 */, double alpha, double gamma,
                         const f2* R /* [E][4] */, double* out) {
  using namespace df;
  f2 m00, m01, m11, adet;
  TriaMetricDF(FromDouble(jac[0]), FromDouble(jac[1]), FromDouble(jac[2]), FromDouble(jac[3]), m00, m01, m11, adet);
  const f2 al = FromDouble(alpha);
  const f2 a00 = Mul(al, m00), a01 = Mul(al, m01), a11 = Mul(al, m11);
  f2 mm = {0.0f, 0.0f};
  if (MASS) mm = Mul(FromDouble(gamma), adet);
  DF_UNROLL
  for (int e = 0; e < E; ++e) {
    Acc acc;
    acc.AddProd(a00, R[4 * e + 0]);
    acc.AddProd(a01, R[4 * e + 1]);
    acc.AddProd(a11, R[4 * e + 2]);
    if (MASS) acc.AddProd(mm, R[4 * e + 3]);
    out[e] = ToDouble(acc.Value());
  }
}

// FP64 version of the same formula (cells outside the df32 range).
template <int E, bool MASS>
DF_HD void TriaUniformF64(const double (&jac)[4], double alpha, double gamma, const double* R, double* out) {
  const double j00 = jac[0], j01 = jac[1], j10 = jac[2], j11 = jac[3];
  const double det = j00 * j11 - j10 * j01;
  const double adet = det < 0 ? -det : det;
  const double inv = 1.0 / adet;
  const double a00 = alpha * ((j11 * j11 + j01 * j01) * inv);
  const double a01 = alpha * (-(j11 * j10 + j01 * j00) * inv);
  const double a11 = alpha * ((j10 * j10 + j00 * j00) * inv);
  const double mm = MASS ? gamma * adet : 0.0;
  for (int e = 0; e < E; ++e) {
    double r = a00 * R[4 * e];
    r = fma(a01, R[4 * e + 1], r);
    r = fma(a11, R[4 * e + 2], r);
    if (MASS) r = fma(mm, R[4 * e + 3], r);
    out[e] = r;
  }
}

// ------------------------------------------- point-varying coefficients (df32)

// Entries contracted together (a divisor of E), as for the quadrilaterals.
template <int E>
constexpr int ContractGroupT() {
  return E % 5 == 0 ? 5 : (E % 4 == 0 ? 4 : (E % 3 == 0 ? 3 : 1));
}

// sin(pi u) and cos(pi u) of a df32 argument, |u| < 2^22.  Periodicity:
// u = n + r with n the nearest integer to u.h (exact: r = (u.h - n) + u.l),
// sin(pi u) = (-1)^n sin(pi r), cos(pi u) = (-1)^n cos(pi r), |r| <= 1/2 + eps.
// Then the Taylor series sin(pi r) = r sum_k S_k r^2k (k < 11) and
// cos(pi r) = sum_k C_k r^2k (k < 12), S_k = (-1)^k pi^(2k+1) / (2k+1)!,
// C_k = (-1)^k pi^(2k) / (2k)!, in Horner form in r^2 (truncation below
// 3e-16 for |pi r| <= pi/2).  Coefficient pairs come from the host.
DF_HD void SinCosPiDF(f2 u, const f2* S /* [11] */, const f2* C /* [12] */, f2& sn, f2& cs) {
  using namespace df;
  const float n = rintf(u.h);  // round to nearest (even): exact integer
  const f2 t = TwoSum(u.h, -n);
  const f2 r = Add(t, Make(u.l));
  const f2 r2 = Mul(r, r);
  f2 ps = S[10];
  DF_UNROLL
  for (int k = 9; k >= 0; --k) ps = MulAdd(ps, r2, S[k]);
  f2 pc = C[11];
  DF_UNROLL
  for (int k = 10; k >= 0; --k) pc = MulAdd(pc, r2, C[k]);
  sn = Mul(ps, r);
  cs = pc;
  const long ni = static_cast<long>(n);
  if (ni & 1) {
    sn = Neg(sn);
    cs = Neg(cs);
  }
}

// Analytic coefficient families at a df32 point (see lfg.h LFG_FN_*):
// POLY sum p[4i+j] x^i y^j (Horner), SINSIN / SINCOS p0 + p1 sin(p2 pi x)
// {sin, cos}(p3 pi y).
struct AnalyticDF {
  int func = 0;
  f2 p[16];
};

DF_HD f2 EvalAnalyticDF(const AnalyticDF& f, f2 x, f2 y, const f2* S, const f2* C) {
  using namespace df;
  if (f.func == 1) {  // LFG_FN_POLY
    f2 acc = Make(0.0f);
    DF_UNROLL
    for (int i = 3; i >= 0; --i) {
      f2 py = f.p[4 * i + 3];
      DF_UNROLL
      for (int j = 2; j >= 0; --j) py = MulAdd(py, y, f.p[4 * i + j]);
      acc = MulAdd(acc, x, py);
    }
    return acc;
  }
  f2 sx, cx, sy, cy;
  SinCosPiDF(Mul(f.p[2], x), S, C, sx, cx);
  SinCosPiDF(Mul(f.p[3], y), S, C, sy, cy);
  return MulAdd(f.p[1], Mul(sx, f.func == 2 ? sy : cy), f.p[0]);
}

// sin and cos of a small df32 angle, |t| <= 0.1: Taylor series in t^2
// (next terms below 3e-19), coefficients S[0..4] = (-1)^k / (2k+1)!,
// C[0..5] = (-1)^k / (2k)! as df32 pairs.
DF_HD void SinCosSmallDF(f2 t, const f2* S, const f2* C, f2& sn, f2& cs) {
  using namespace df;
  const f2 t2 = Mul(t, t);
  f2 ps = S[4];
  DF_UNROLL
  for (int k = 3; k >= 0; --k) ps = MulAdd(ps, t2, S[k]);
  f2 pc = C[5];
  DF_UNROLL
  for (int k = 4; k >= 0; --k) pc = MulAdd(pc, t2, C[k]);
  sn = Mul(ps, t);
  cs = pc;
}

// Contraction of an affine triangle with point coefficients c[k] = {c00, c01,
// c11} (c = w_k alpha_k |det J| J^-1 J^-T) over the per-point tables
// T[k][e][0..2], plus an optional cell-constant mass term mm * R[e][3].
template <int E, int NQ>
DF_HD void TriaVaryContractDF(const f2 (*c)[3], const f2* T /* [NQ][E][4] */, f2 mm, bool mass,
                              const f2* R /* [E][4] */, double* out) {
  using namespace df;
  constexpr int G = ContractGroupT<E>();
  DF_NOUNROLL
  for (int e0 = 0; e0 < E; e0 += G) {
    Acc acc[G];
    DF_UNROLL
    for (int k = 0; k < NQ; ++k) {
      const f2* te = T + (static_cast<long>(k) * E + e0) * 4;
      DF_UNROLL
      for (int ab = 0; ab < 3; ++ab) {
        DF_UNROLL
        for (int g = 0; g < G; ++g) acc[g].AddProd(c[k][ab], te[g * 4 + ab]);
      }
    }
    if (mass) {
      DF_UNROLL
      for (int g = 0; g < G; ++g) acc[g].AddProd(mm, R[(e0 + g) * 4 + 3]);
    }
    DF_UNROLL
    for (int g = 0; g < G; ++g) out[e0 + g] = ToDouble(acc[g].Value());
  }
}

// -------------------------------------------------------------- quadrilaterals

// Per-point coefficients c[k] = {c00, c01, c11, m} of a bilinear quadrilateral
// on an M x M tensor rule.  a = v1 - v0, c = v3 - v0, d = v0 - v1 + v2 - v3
// (FP64 differences, geometry/quad_o1.cc:93-99 rewritten: J col0 = a + d yh,
// col1 = c + d xh), everything after the differences in df32.
template <int M, bool MASS>
DF_HD void QuadPointCoeffsDF(const double (&acd)[6] /* ax, ay, cx, cy, dx, dy */, double alpha, double gamma,
                             const f2* t /* [M] abscissae */, const f2* W /* [M*M] weights */, f2 (*c)[4]) {
  using namespace df;
  const f2 ax = FromDouble(acd[0]), ay = FromDouble(acd[1]), cx = FromDouble(acd[2]), cy = FromDouble(acd[3]);
  const f2 dx = FromDouble(acd[4]), dy = FromDouble(acd[5]);
  const f2 al = FromDouble(alpha);
  const f2 ga = MASS ? FromDouble(gamma) : f2{0.0f, 0.0f};
  f2 j00[M], j10[M], j01[M], j11[M], m00[M], m11[M];
  DF_UNROLL
  for (int q = 0; q < M; ++q) {  // column 0 at yh = t[q], column 1 at xh = t[q]
    j00[q] = MulAdd(dx, t[q], ax);
    j10[q] = MulAdd(dy, t[q], ay);
    j01[q] = MulAdd(dx, t[q], cx);
    j11[q] = MulAdd(dy, t[q], cy);
  }
  DF_UNROLL
  for (int q = 0; q < M; ++q) {
    m00[q] = Add(Mul(j11[q], j11[q]), Mul(j01[q], j01[q]));  // depends on xh only
    m11[q] = Add(Mul(j10[q], j10[q]), Mul(j00[q], j00[q]));  // depends on yh only
  }
  DF_UNROLL
  for (int p = 0; p < M; ++p) {    // xh index
    DF_UNROLL
    for (int q = 0; q < M; ++q) {  // yh index
      const int k = p * M + q;
      const f2 det = Sub(Mul(j00[q], j11[p]), Mul(j10[q], j01[p]));
      const f2 adet = Abs(det);
      const f2 s = Mul(Mul(W[k], al), Rcp(adet));
      const f2 m01 = Neg(Add(Mul(j11[p], j10[q]), Mul(j01[p], j00[q])));
      c[k][0] = Mul(s, m00[p]);
      c[k][1] = Mul(s, m01);
      c[k][2] = Mul(s, m11[q]);
      if (MASS) c[k][3] = Mul(Mul(W[k], adet), ga);
    }
  }
}

// The same coefficients for the points k in [K0, K1) only (c[k - K0]), with
// gamma = 0: the tensor-core quad kernel splits the points of a cell between
// two threads.
template <int M, int K0, int K1>
DF_HD void QuadPointCoeffsRangeDF(const double (&acd)[6], double alpha, const f2* t, const f2* W, f2 (*c)[3]) {
  using namespace df;
  const f2 ax = FromDouble(acd[0]), ay = FromDouble(acd[1]), cx = FromDouble(acd[2]), cy = FromDouble(acd[3]);
  const f2 dx = FromDouble(acd[4]), dy = FromDouble(acd[5]);
  const f2 al = FromDouble(alpha);
  f2 j00[M], j10[M], j01[M], j11[M], m00[M], m11[M];
  DF_UNROLL
  for (int q = 0; q < M; ++q) {
    j00[q] = MulAdd(dx, t[q], ax);
    j10[q] = MulAdd(dy, t[q], ay);
    j01[q] = MulAdd(dx, t[q], cx);
    j11[q] = MulAdd(dy, t[q], cy);
  }
  DF_UNROLL
  for (int q = 0; q < M; ++q) {
    m00[q] = Add(Mul(j11[q], j11[q]), Mul(j01[q], j01[q]));
    m11[q] = Add(Mul(j10[q], j10[q]), Mul(j00[q], j00[q]));
  }
  DF_UNROLL
  for (int k = K0; k < K1; ++k) {
    const int p = k / M, q = k % M;
    const f2 det = Sub(Mul(j00[q], j11[p]), Mul(j10[q], j01[p]));
    const f2 s = Mul(Mul(W[k], al), Rcp(Abs(det)));
    const f2 m01 = Neg(Add(Mul(j11[p], j10[q]), Mul(j01[p], j00[q])));
    c[k - K0][0] = Mul(s, m00[p]);
    c[k - K0][1] = Mul(s, m01);
    c[k - K0][2] = Mul(s, m11[q]);
  }
}

// Upper-triangle index of the unordered pair {i, j} in "for i: for j >= i" order.
template <int N>
DF_HD int UpperIdx(int i, int j) {
  const int a = i < j ? i : j, b = i < j ? j : i;
  return a * N - (a * (a - 1)) / 2 + (b - a);
}

// Sum-factorised contraction for tensor-product bases (Q2, Q3 on the tensor
// Gauss rule).  With phi_{(a,b)}(x,y) = l_a(x) l_b(y), points k = p M + q at
// (x_p, y_q) and c[k] = {c00, c01, c11, m}:
//   H0(a,a',q) = sum_p c00 l'_a l'_a'(x_p),  H2 = sum_p c11 l_a l_a',
//   H1(a,a',q) = sum_p c01 l'_a l_a',        H3 = sum_p m l_a l_a',
//   A((a,b),(a',b')) = sum_q H0(a,a') l_b l_b' + H1(a,a') l_b l'_b'
//                           + H1(a',a) l'_b l_b' + H2(a,a') l'_b l'_b' [+ H3 l_b l_b'](y_q).
// Unordered x pairs a <= a' run as a runtime loop (H stays in registers);
// each pair owns the 9 (a < a') or 6 (a = a') unordered entries of its
// y pairs.  Q2: 729 products per cell instead of 1215.  sf = [3][N1][N1][M]
// ({l'l', ll, l'l}), loc[a N1 + b] = local dof of (a, b).
template <int N1, int M, bool MASS>
DF_HD void QuadSumFactDF(const f2 (*c)[4], const f2* sf, const int* loc, double* out) {
  using namespace df;
  constexpr int N = N1 * N1;
  const f2* DD = sf;
  const f2* VV = sf + N1 * N1 * M;
  const f2* DV = sf + 2 * N1 * N1 * M;
  DF_NOUNROLL
  for (int pr = 0; pr < N1 * N1; ++pr) {
    const int a = pr / N1, a2 = pr - a * N1;
    if (a2 < a) continue;
    f2 h0[M], h1[M], h1t[M], h2[M], h3[M];
    DF_UNROLL
    for (int q = 0; q < M; ++q) {
      Acc s0, s1, s1t, s2, s3;
      DF_UNROLL
      for (int p = 0; p < M; ++p) {
        const int k = p * M + q;
        s0.AddProd(c[k][0], DD[pr * M + p]);
        s1.AddProd(c[k][1], DV[pr * M + p]);
        s1t.AddProd(c[k][1], DV[(a2 * N1 + a) * M + p]);
        s2.AddProd(c[k][2], VV[pr * M + p]);
        if (MASS) s3.AddProd(c[k][3], VV[pr * M + p]);
      }
      h0[q] = s0.Value();
      h1[q] = s1.Value();
      h1t[q] = s1t.Value();
      h2[q] = s2.Value();
      h3[q] = MASS ? s3.Value() : f2{0.0f, 0.0f};
    }
    DF_UNROLL
    for (int yb = 0; yb < N1 * N1; ++yb) {
      const int b = yb / N1, b2 = yb % N1, yt = b2 * N1 + b;
      if (a != a2 || b2 >= b) {
        Acc acc;
        DF_UNROLL
        for (int q = 0; q < M; ++q) {
          acc.AddProd(h0[q], VV[yb * M + q]);
          acc.AddProd(h1[q], DV[yt * M + q]);
          acc.AddProd(h1t[q], DV[yb * M + q]);
          acc.AddProd(h2[q], DD[yb * M + q]);
          if (MASS) acc.AddProd(h3[q], VV[yb * M + q]);
        }
        out[UpperIdx<N>(loc[a * N1 + b], loc[a2 * N1 + b2])] = ToDouble(acc.Value());
      }
    }
  }
}

// Number of upper-triangle entries contracted together (a divisor of E): the
// G accumulators give instruction-level parallelism while the loop over the
// E/G groups stays a runtime loop, so the code fits the instruction cache.
template <int E>
constexpr int ContractGroup() {
  return E % 5 == 0 ? 5 : (E % 4 == 0 ? 4 : (E % 3 == 0 ? 3 : 1));
}

// All upper-triangle entries: sum over points of c . T.
template <int E, int NQ, bool MASS>
DF_HD void QuadContractDF(const f2 (*c)[4], const f2* T /* [NQ][E][4] */, double* out) {
  using namespace df;
  constexpr int G = ContractGroup<E>();
  DF_NOUNROLL
  for (int e0 = 0; e0 < E; e0 += G) {
    Acc acc[G];
    DF_UNROLL
    for (int k = 0; k < NQ; ++k) {
      const f2* te = T + (static_cast<long>(k) * E + e0) * 4;
      DF_UNROLL
      for (int ab = 0; ab < (MASS ? 4 : 3); ++ab) {
        DF_UNROLL
        for (int g = 0; g < G; ++g) acc[g].AddProd(c[k][ab], te[g * 4 + ab]);
      }
    }
    DF_UNROLL
    for (int g = 0; g < G; ++g) out[e0 + g] = ToDouble(acc[g].Value());
  }
}

}  // namespace elem
}  // namespace lfg
