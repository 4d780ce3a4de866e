// CPU check of the df32 element arithmetic used by the GPU kernels
// (lehrfempp_gb300/csrc/lfg_elem.h, lfg_df32.h): element matrices of random
// triangles and bilinear quadrilaterals are compared with a long-double
// evaluation of the reference's quadrature sum (loc_comp_ellbvp.h:324-337).
// Quadrilaterals of degree 2 and 3 also run through the sum-factorised
// contraction ("quadsf"), which the kernels use for tensor-product bases.
// Prints one line per case: "<type> <degree> <rule> <cells> <h> <mass> <max |err|/max|A_K|>".
#include <cmath>
#include <cstdio>
#include <random>
#include <vector>

#include "lfg_elem.h"
#include "lfg_tables.h"

using lfg::df::f2;

namespace {

// alpha of the point-varying cases: 0 constant (alpha_c), 1 sincos
// 1 + 0.5 sin(4 pi x) cos(4 pi y), 2 polynomial 1 + x^2 + y^2 - 0.5 x y^3.
long double AlphaRef(int kind, long double alpha_c, long double x, long double y) {
  const long double pi = 3.141592653589793238462643383279502884L;
  if (kind == 1) return 1.0L + 0.5L * std::sin(4.0L * pi * x) * std::cos(4.0L * pi * y);
  if (kind == 2) return 1.0L + x * x + y * y - 0.5L * x * y * y * y;
  return alpha_c;
}

// long double reference: sum_k w_k |det J_k| [alpha G_i.G_j + gamma phi_i phi_j]
void Reference(bool quad, int degree, const lfg::Rule& r, const double (*v)[2], double alpha, double gamma,
               std::vector<long double>& A, int akind = 0) {
  const int n = lfg::NumShape(quad, degree);
  A.assign(n * n, 0.0L);
  double phi[16], dphi[16][2];
  for (int k = 0; k < r.n; ++k) {
    const long double x = r.x[k], y = r.y[k];
    long double J[2][2];
    for (int d = 0; d < 2; ++d) {
      if (!quad) {
        J[d][0] = (long double)v[1][d] - v[0][d];
        J[d][1] = (long double)v[2][d] - v[0][d];
      } else {
        J[d][0] = ((long double)v[1][d] - v[0][d]) * (1 - y) + ((long double)v[2][d] - v[3][d]) * y;
        J[d][1] = ((long double)v[3][d] - v[0][d]) * (1 - x) + ((long double)v[2][d] - v[1][d]) * x;
      }
    }
    const long double det = J[0][0] * J[1][1] - J[1][0] * J[0][1];
    const long double JT[2][2] = {{J[1][1] / det, -J[1][0] / det}, {-J[0][1] / det, J[0][0] / det}};
    lfg::Shape(quad, degree, r.x[k], r.y[k], phi, dphi);
    const long double w = r.w[k] * std::fabs(det);
    long double al = alpha;
    if (akind && !quad) {
      const long double l0 = 1.0L - x - y;
      al = AlphaRef(akind, alpha, v[0][0] * l0 + v[1][0] * x + v[2][0] * y, v[0][1] * l0 + v[1][1] * x + v[2][1] * y);
    }
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) {
        long double gi[2], gj[2];
        for (int d = 0; d < 2; ++d) {
          gi[d] = JT[d][0] * dphi[i][0] + JT[d][1] * dphi[i][1];
          gj[d] = JT[d][0] * dphi[j][0] + JT[d][1] * dphi[j][1];
        }
        A[i * n + j] += w * (al * (gi[0] * gj[0] + gi[1] * gj[1]) + (long double)gamma * phi[i] * phi[j]);
      }
  }
}

template <int N>
double RunCase(bool quad, int degree, int rule, int cells, double h, bool mass, std::mt19937_64& rng,
               bool sf = false) {
  constexpr int E = N * (N + 1) / 2;
  std::vector<float> tab;
  lfg::DfLayout L;
  if (!lfg::BuildDfTables(quad, degree, rule, tab, L)) return -1;
  if (sf && L.n1 != degree + 1) return -1;  // no tensor-product tables
  const f2* T = reinterpret_cast<const f2*>(tab.data());
  lfg::Rule r;
  lfg::MakeRule(quad, rule, r);
  std::uniform_real_distribution<double> U(-0.2, 0.2);
  std::normal_distribution<double> Nrm(0.0, 1.0);
  std::uniform_real_distribution<double> Pos(0.0, 1.0);
  double worst = 0.0;
  std::vector<long double> A;
  for (int c = 0; c < cells; ++c) {
    // a jittered square / triangle at a random place of the unit square
    const double x0 = std::floor(Pos(rng) / h) * h, y0 = std::floor(Pos(rng) / h) * h;
    double v[4][2] = {{x0, y0}, {x0 + h, y0}, {x0 + h, y0 + h}, {x0, y0 + h}};
    for (auto& p : v) {
      p[0] += U(rng) * h;
      p[1] += U(rng) * h;
    }
    if (!quad && (c & 1)) {  // the "up" triangle of the TPTriag split
      v[1][0] = v[2][0]; v[1][1] = v[2][1];
      v[2][0] = v[3][0]; v[2][1] = v[3][1];
    }
    const double alpha = std::exp(Nrm(rng)), gamma = mass ? std::exp(Nrm(rng)) : 0.0;
    Reference(quad, degree, r, v, alpha, gamma, A);
    double got[E];
    if (!quad) {
      const double jac[4] = {v[1][0] - v[0][0], v[2][0] - v[0][0], v[1][1] - v[0][1], v[2][1] - v[0][1]};
      if (mass) lfg::elem::TriaUniformDF<E, true>(jac, alpha, gamma, T + L.off_R, got);
      else lfg::elem::TriaUniformDF<E, false>(jac, alpha, gamma, T + L.off_R, got);
    } else {
      const double acd[6] = {v[1][0] - v[0][0], v[1][1] - v[0][1], v[3][0] - v[0][0], v[3][1] - v[0][1],
                             (v[0][0] - v[1][0]) + (v[2][0] - v[3][0]), (v[0][1] - v[1][1]) + (v[2][1] - v[3][1])};
      f2 cpt[25][4];
      const int m = L.m;
      auto contract = [&](auto mass_tag) {
        constexpr bool MS = decltype(mass_tag)::value;
        if (m == 2) lfg::elem::QuadPointCoeffsDF<2, MS>(acd, alpha, gamma, T + L.off_t, T + L.off_W, cpt);
        if (m == 3) lfg::elem::QuadPointCoeffsDF<3, MS>(acd, alpha, gamma, T + L.off_t, T + L.off_W, cpt);
        if (m == 4) lfg::elem::QuadPointCoeffsDF<4, MS>(acd, alpha, gamma, T + L.off_t, T + L.off_W, cpt);
        constexpr int N1 = N == 9 ? 3 : (N == 16 ? 4 : 2);
        if (sf && m == 3) lfg::elem::QuadSumFactDF<N1, 3, MS>(cpt, T + L.off_SF, L.loc, got);
        else if (sf && m == 4) lfg::elem::QuadSumFactDF<N1, 4, MS>(cpt, T + L.off_SF, L.loc, got);
        else if (m == 2) lfg::elem::QuadContractDF<E, 4, MS>(cpt, T + L.off_T, got);
        else if (m == 3) lfg::elem::QuadContractDF<E, 9, MS>(cpt, T + L.off_T, got);
        else if (m == 4) lfg::elem::QuadContractDF<E, 16, MS>(cpt, T + L.off_T, got);
      };
      if (mass) contract(std::true_type{});
      else contract(std::false_type{});
    }
    long double scale = 0.0L;
    for (auto a : A) scale = std::max(scale, std::fabs(a));
    int e = 0;
    for (int i = 0; i < N; ++i)
      for (int j = i; j < N; ++j, ++e) {
        const double err = static_cast<double>(std::fabs(static_cast<long double>(got[e]) - A[i * N + j]) / scale);
        worst = std::max(worst, err);
      }
  }
  return worst;
}

// Point-varying alpha on affine triangles (the RDTriaVaryDfKernel math).
template <int N, int NQ>
double RunVary(int degree, int rule, int akind, int cells, double h, std::mt19937_64& rng) {
  constexpr int E = N * (N + 1) / 2;
  std::vector<float> tab;
  lfg::DfLayout L;
  if (!lfg::BuildDfTables(false, degree, rule, tab, L) || L.nq != NQ) return -1;
  const f2* T = reinterpret_cast<const f2*>(tab.data());
  lfg::Rule r;
  lfg::MakeRule(false, rule, r);
  lfg::elem::AnalyticDF af;
  const double p_sincos[4] = {1.0, 0.5, 4.0, 4.0};
  double pp[16] = {0};
  pp[0] = 1.0; pp[8] = 1.0; pp[2] = 1.0; pp[4 * 1 + 3] = -0.5;  // 1 + x^2 + y^2 - 0.5 x y^3
  af.func = akind == 1 ? 3 : 1;
  for (int i = 0; i < 16; ++i) af.p[i] = lfg::df::FromDouble(akind == 1 ? (i < 4 ? p_sincos[i] : 0.0) : pp[i]);
  std::uniform_real_distribution<double> U(-0.2, 0.2), Pos(0.0, 1.0);
  double worst = 0.0;
  std::vector<long double> A;
  for (int c = 0; c < cells; ++c) {
    const double x0 = std::floor(Pos(rng) / h) * h, y0 = std::floor(Pos(rng) / h) * h;
    double v[4][2] = {{x0, y0}, {x0 + h, y0}, {x0 + h, y0 + h}, {x0, y0 + h}};
    for (auto& p : v) {
      p[0] += U(rng) * h;
      p[1] += U(rng) * h;
    }
    if (c & 1) {
      v[1][0] = v[2][0]; v[1][1] = v[2][1];
      v[2][0] = v[3][0]; v[2][1] = v[3][1];
    }
    const double gamma = 1.0;
    Reference(false, degree, r, v, 0.0, gamma, A, akind);
    using namespace lfg::df;
    const f2 j00 = FromDouble(v[1][0] - v[0][0]), j01 = FromDouble(v[2][0] - v[0][0]);
    const f2 j10 = FromDouble(v[1][1] - v[0][1]), j11 = FromDouble(v[2][1] - v[0][1]);
    f2 m00, m01, m11, adet;
    lfg::elem::TriaMetricDF(j00, j01, j10, j11, m00, m01, m11, adet);
    const f2 xx0 = FromDouble(v[0][0]), yy0 = FromDouble(v[0][1]);
    f2 cpt[NQ][3];
    for (int k = 0; k < NQ; ++k) {
      const f2 xh = T[L.off_X + 2 * k], yh = T[L.off_X + 2 * k + 1];
      const f2 X = MulAdd(j01, yh, MulAdd(j00, xh, xx0));
      const f2 Y = MulAdd(j11, yh, MulAdd(j10, xh, yy0));
      const f2 al = lfg::elem::EvalAnalyticDF(af, X, Y, T + L.off_SC, T + L.off_SC + 11);
      const f2 sw = Mul(T[L.off_W + k], al);
      cpt[k][0] = Mul(sw, m00);
      cpt[k][1] = Mul(sw, m01);
      cpt[k][2] = Mul(sw, m11);
    }
    const f2 mm = Mul(FromDouble(gamma), adet);
    double got[E];
    lfg::elem::TriaVaryContractDF<E, NQ>(cpt, T + L.off_T, mm, true, T + L.off_R, got);
    long double scale = 0.0L;
    for (auto a : A) scale = std::max(scale, std::fabs(a));
    int e = 0;
    for (int i = 0; i < N; ++i)
      for (int j = i; j < N; ++j, ++e)
        worst = std::max(worst, static_cast<double>(std::fabs(static_cast<long double>(got[e]) - A[i * N + j]) / scale));
  }
  return worst;
}

// sin(pi u), cos(pi u) in df32 against long double on [-8, 8].
double RunSinCos(int samples, std::mt19937_64& rng) {
  std::vector<float> tab;
  lfg::DfLayout L;
  lfg::BuildDfTables(false, 1, 2, tab, L);
  const f2* T = reinterpret_cast<const f2*>(tab.data());
  std::uniform_real_distribution<double> U(-8.0, 8.0);
  const long double pi = 3.141592653589793238462643383279502884L;
  double worst = 0.0;
  for (int i = 0; i < samples; ++i) {
    const double u = i < 64 ? (i - 32) * 0.25 : U(rng);  // include the multiples of 1/4
    f2 sn, cs;
    lfg::elem::SinCosPiDF(lfg::df::FromDouble(u), T + L.off_SC, T + L.off_SC + 11, sn, cs);
    const long double es = std::sin(pi * (long double)u), ec = std::cos(pi * (long double)u);
    worst = std::max(worst, (double)std::fabs((long double)lfg::df::ToDouble(sn) - es));
    worst = std::max(worst, (double)std::fabs((long double)lfg::df::ToDouble(cs) - ec));
  }
  return worst;
}

}  // namespace

int main(int argc, char** argv) {
  const int cells = argc > 1 ? std::atoi(argv[1]) : 20000;
  std::mt19937_64 rng(12345);
  const double hs[3] = {1.0 / 2048, 1.0 / 64, 1.0};
  for (int mass = 0; mass < 2; ++mass)
    for (double h : hs) {
      std::printf("tria 1 2 %d %.3g %d %.3e\n", cells, h, mass, RunCase<3>(false, 1, 2, cells, h, mass, rng));
      std::printf("tria 2 4 %d %.3g %d %.3e\n", cells, h, mass, RunCase<6>(false, 2, 4, cells, h, mass, rng));
      std::printf("tria 3 6 %d %.3g %d %.3e\n", cells, h, mass, RunCase<10>(false, 3, 6, cells, h, mass, rng));
      std::printf("quad 1 2 %d %.3g %d %.3e\n", cells, h, mass, RunCase<4>(true, 1, 2, cells, h, mass, rng));
      std::printf("quad 2 4 %d %.3g %d %.3e\n", cells, h, mass, RunCase<9>(true, 2, 4, cells, h, mass, rng));
      std::printf("quad 3 6 %d %.3g %d %.3e\n", cells, h, mass, RunCase<16>(true, 3, 6, cells, h, mass, rng));
      std::printf("quadsf 2 4 %d %.3g %d %.3e\n", cells, h, mass, RunCase<9>(true, 2, 4, cells, h, mass, rng, true));
      std::printf("quadsf 3 6 %d %.3g %d %.3e\n", cells, h, mass, RunCase<16>(true, 3, 6, cells, h, mass, rng, true));
    }
  for (double h : hs) {
    std::printf("triavary_sincos 3 6 %d %.3g 1 %.3e\n", cells, h, RunVary<10, 12>(3, 6, 1, cells, h, rng));
    std::printf("triavary_poly 1 4 %d %.3g 1 %.3e\n", cells, h, RunVary<3, 6>(1, 4, 2, cells, h, rng));
    std::printf("triavary_sincos 2 4 %d %.3g 1 %.3e\n", cells, h, RunVary<6, 6>(2, 4, 1, cells, h, rng));
  }
  std::printf("sincospi 0 0 %d 0 0 %.3e\n", cells * 10, RunSinCos(cells * 10, rng));
  return 0;
}
