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

// long double reference: sum_k w_k |det J_k| [alpha G_i.G_j + gamma phi_i phi_j]
void Reference(bool quad, int degree, const lfg::Rule& r, const double (*v)[2], double alpha, double gamma,
               std::vector<long double>& A) {
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
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) {
        long double gi[2], gj[2];
        for (int d = 0; d < 2; ++d) {
          gi[d] = JT[d][0] * dphi[i][0] + JT[d][1] * dphi[i][1];
          gj[d] = JT[d][0] * dphi[j][0] + JT[d][1] * dphi[j][1];
        }
        A[i * n + j] += w * (alpha * (gi[0] * gj[0] + gi[1] * gj[1]) + (long double)gamma * phi[i] * phi[j]);
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
  return 0;
}
