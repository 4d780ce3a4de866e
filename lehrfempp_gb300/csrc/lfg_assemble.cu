// Element kernels: AssembleMatrixLocally with ReactionDiffusionElementMatrixProvider
// and AssembleVectorLocally with ScalarLoadElementVectorProvider
// (assemble/assembler.h:114-365, uscalfe/loc_comp_ellbvp.h:266-339, 691-746).
//
// Output contract (bit-exact indices and order): the triplets of cell K start
// at coo_base + sum_{K' < K} n_{K'}^2 and run over (i, j) row-major with
// row = dofs_K[i], col = dofs_K[j].  Values are the element matrix entries in
// FP64.  The reference's per-quadrature-point sum
//     A_K = sum_k w_k |det J_k| [ G_k^T alpha_k G_k + gamma_k phi_k phi_k^T ],
//     G_k = J_k^{-T} grad(phi_hat)(q_k)
// is evaluated as
//     A_K(i,j) = sum_k [ c00_k T0 + c01_k T1 + c11_k T2 + m_k T3 ](k; i, j)
// with c = w |det J| alpha J^{-1} J^{-T} (3 numbers per point), m = w |det J| gamma
// and the cell-independent tables T(k; i,j) = {g_i0 g_j0, g_i0 g_j1 + g_i1 g_j0,
// g_i1 g_j1, phi_i phi_j} of reference gradients g.  Only the upper triangle
// i <= j is computed (the element matrix is symmetric) and mirrored.
// For affine triangles with cell-constant alpha/gamma the point sum is folded
// into R(i,j) = sum_k w_k T(k; i,j) once per rule, so a cell costs 3-4 FMAs
// per entry.  Both are exact reformulations; they differ from the reference
// only by rounding (checked to 1e-12 of max|A_K| in the parity tests).
//
// The device does FP64 arithmetic; cells are processed one per thread from
// per-type cell lists (triangles and quadrilaterals run as separate launches
// so a warp never diverges on the cell type).
#include <algorithm>
#include <cmath>
#include <map>

#include <cuda_fp16.h>

#include "lfg_api.h"
#include "lfg_coeff.h"
#include "lfg_elem.h"
#include "lfg_internal.h"
#include "lfg_tc.h"

namespace lfg {
void EnsureIncidence(lfg_space* sp);

namespace {

constexpr int kMaxQ = 25;

Tab TabLayout(int n, int nq) {
  Tab t;
  t.n = n; t.nq = nq; t.E = n * (n + 1) / 2;
  t.off_w = 0;
  t.off_qx = nq;
  t.off_qy = 2 * nq;
  t.off_phi = 3 * nq;
  t.off_T = t.off_phi + nq * n;
  t.off_R = t.off_T + nq * t.E * 4;
  t.off_L = t.off_R + t.E * 4;
  t.off_o1 = t.off_L + n;
  t.off_G = t.off_o1 + nq * 4;  // reference gradients [nq][n][2]
  t.total = t.off_G + nq * n * 2;
  return t;
}

struct AsmArgs {
  const int32_t* bucket;
  int64_t count;
  const int4* cells;
  const double2* xy;
  const int32_t* cell_dofs;
  int n_cell;
  const int64_t* tri_offset;  // per cell (triplet matrices) or loc_offset (vectors)
  lfg_triplet* out;
  double* vout;
  const double* tab;
  Tab L;
  CoeffDev alpha, gamma;
  unsigned long long* fallback;  // cells that took the FP64 route (diagnostics)
};

// ------------------------------------------------------------- device helpers

__device__ __forceinline__ void StoreTriplet(lfg_triplet* p, int r, int c, double v) {
  const long long bits = __double_as_longlong(v);
  int4 w = make_int4(r, c, static_cast<int>(bits & 0xffffffffll), static_cast<int>(bits >> 32));
  *reinterpret_cast<int4*>(p) = w;
}

// Value of a coefficient at reference point k of cell c.
template <bool QUAD>
__device__ double EvalCoeff(const CoeffDev& f, int c, const int4& cn, const double2 (&v)[4], int k,
                            const double* sw, const double* sqx, const double* sqy,
                            const double* so1) {
  switch (f.kind) {
    case LFG_COEFF_ZERO: return 0.0;
    case LFG_COEFF_CONSTANT: return f.value;
    case LFG_COEFF_PER_CELL: return f.data[c];
    case LFG_COEFF_PER_CELL_EXP: return exp(f.data[c]);
    case LFG_COEFF_NODAL_O1: {
      double s = f.data[cn.x] * so1[k * 4 + 0];
      s += f.data[cn.y] * so1[k * 4 + 1];
      s += f.data[cn.z] * so1[k * 4 + 2];
      if (QUAD) s += f.data[cn.w] * so1[k * 4 + 3];
      return s;
    }
    case LFG_COEFF_ANALYTIC: {
      const double xh = sqx[k], yh = sqy[k];
      double X, Y;
      if (!QUAD) {
        const double l0 = 1.0 - xh - yh;
        X = v[0].x * l0 + v[1].x * xh + v[2].x * yh;
        Y = v[0].y * l0 + v[1].y * xh + v[2].y * yh;
      } else {
        const double b0 = (1 - xh) * (1 - yh), b1 = xh * (1 - yh), b2 = xh * yh, b3 = (1 - xh) * yh;
        X = v[0].x * b0 + v[1].x * b1 + v[2].x * b2 + v[3].x * b3;
        Y = v[0].y * b0 + v[1].y * b1 + v[2].y * b2 + v[3].y * b3;
      }
      return EvalAnalytic(f, X, Y);
    }
  }
  return 0.0;
}

__device__ __forceinline__ double CellConst(const CoeffDev& f, int c) {
  switch (f.kind) {
    case LFG_COEFF_CONSTANT: return f.value;
    case LFG_COEFF_PER_CELL: return f.data[c];
    case LFG_COEFF_PER_CELL_EXP: return exp(f.data[c]);
  }
  return 0.0;
}

template <bool QUAD>
__device__ __forceinline__ void LoadVerts(const AsmArgs& a, int c, int4& cn, double2 (&v)[4]) {
  cn = a.cells[c];
  v[0] = a.xy[cn.x];
  v[1] = a.xy[cn.y];
  v[2] = a.xy[cn.z];
  v[3] = QUAD ? a.xy[cn.w] : make_double2(0.0, 0.0);
}

// |det J| * J^{-1} J^{-T} of an affine triangle: adj(J) adj(J)^T / |det J|.
__device__ __forceinline__ void TriaMetric(const double2 (&v)[4], double& m00, double& m01,
                                           double& m11, double& adet) {
  const double j00 = v[1].x - v[0].x, j01 = v[2].x - v[0].x;
  const double j10 = v[1].y - v[0].y, j11 = v[2].y - v[0].y;
  const double det = j00 * j11 - j10 * j01;
  adet = fabs(det);
  const double inv = 1.0 / adet;
  m00 = (j11 * j11 + j01 * j01) * inv;
  m01 = -(j11 * j10 + j01 * j00) * inv;
  m11 = (j10 * j10 + j00 * j00) * inv;
}

// Same at reference point (xh, yh) of a bilinear quadrilateral (quad_o1.cc:93-99).
__device__ __forceinline__ void QuadMetric(const double2 (&v)[4], double xh, double yh, double& m00,
                                           double& m01, double& m11, double& adet) {
  const double j00 = (v[1].x - v[0].x) * (1 - yh) + (v[2].x - v[3].x) * yh;
  const double j10 = (v[1].y - v[0].y) * (1 - yh) + (v[2].y - v[3].y) * yh;
  const double j01 = (v[3].x - v[0].x) * (1 - xh) + (v[2].x - v[1].x) * xh;
  const double j11 = (v[3].y - v[0].y) * (1 - xh) + (v[2].y - v[1].y) * xh;
  const double det = j00 * j11 - j10 * j01;
  adet = fabs(det);
  const double inv = 1.0 / adet;
  m00 = (j11 * j11 + j01 * j01) * inv;
  m01 = -(j11 * j10 + j01 * j00) * inv;
  m11 = (j10 * j10 + j00 * j00) * inv;
}

__device__ __forceinline__ void LoadTable(const double* __restrict__ g, double* s, int n) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) s[i] = g[i];
  __syncthreads();
}

// -------------------------------------------------- general (per point) path
// One thread per cell.  Accumulators are kept in registers in chunks of at
// most 64 upper-triangle entries; every chunk re-runs the point loop.
template <int DEG, bool QUAD, bool VARY, bool MASS>
__global__ void __launch_bounds__(128) RDGeneralKernel(AsmArgs a) {
  constexpr int N = QUAD ? (DEG + 1) * (DEG + 1) : (DEG + 1) * (DEG + 2) / 2;
  constexpr int E = N * (N + 1) / 2;
  constexpr int CH = E < 64 ? E : 64;
  extern __shared__ double sm[];
  LoadTable(a.tab, sm, a.L.total);
  const double* sw = sm + a.L.off_w;
  const double* sqx = sm + a.L.off_qx;
  const double* sqy = sm + a.L.off_qy;
  const double* sT = sm + a.L.off_T;
  const double* so1 = sm + a.L.off_o1;
  const int nq = a.L.nq;
  for (int64_t t = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; t < a.count;
       t += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int c = a.bucket[t];
    int4 cn;
    double2 v[4];
    LoadVerts<QUAD>(a, c, cn, v);
    double tm00 = 0, tm01 = 0, tm11 = 0, tdet = 0;
    if (!QUAD) TriaMetric(v, tm00, tm01, tm11, tdet);
    double al = 0, ga = 0;
    if (!VARY) {
      al = CellConst(a.alpha, c);
      ga = CellConst(a.gamma, c);
    }
    int dofs[N];
#pragma unroll
    for (int i = 0; i < N; ++i) dofs[i] = a.cell_dofs[static_cast<int64_t>(c) * a.n_cell + i];
    lfg_triplet* base = a.out + a.tri_offset[c];
#pragma unroll
    for (int e0 = 0; e0 < E; e0 += CH) {
      double acc[CH];
#pragma unroll
      for (int e = 0; e < CH; ++e) acc[e] = 0.0;
      for (int k = 0; k < nq; ++k) {
        double m00, m01, m11, adet;
        if (QUAD) QuadMetric(v, sqx[k], sqy[k], m00, m01, m11, adet);
        else { m00 = tm00; m01 = tm01; m11 = tm11; adet = tdet; }
        double alk = al, gak = ga;
        if (VARY) {
          alk = EvalCoeff<QUAD>(a.alpha, c, cn, v, k, sw, sqx, sqy, so1);
          if (MASS) gak = EvalCoeff<QUAD>(a.gamma, c, cn, v, k, sw, sqx, sqy, so1);
        }
        const double s = sw[k] * alk;
        const double c00 = s * m00, c01 = s * m01, c11 = s * m11;
        const double mk = sw[k] * adet * gak;
        const double* Tk = sT + k * E * 4;
#pragma unroll
        for (int e = 0; e < CH; ++e) {
          if (e0 + e < E) {
            const double* T = Tk + (e0 + e) * 4;
            double r = acc[e];
            r = fma(c00, T[0], r);
            r = fma(c01, T[1], r);
            r = fma(c11, T[2], r);
            if (MASS) r = fma(mk, T[3], r);
            acc[e] = r;
          }
        }
      }
      // scatter the chunk's entries to (i, j) and (j, i)
      int e = 0;
#pragma unroll
      for (int i = 0; i < N; ++i) {
#pragma unroll
        for (int j = i; j < N; ++j, ++e) {
          if (e >= e0 && e < e0 + CH) {
            const double val = acc[e - e0];
            StoreTriplet(base + i * N + j, dofs[i], dofs[j], val);
            if (j != i) StoreTriplet(base + j * N + i, dofs[j], dofs[i], val);
          }
        }
      }
    }
  }
}

// ------------------------------------------- matrix-valued diffusion coefficient
// ReactionDiffusionElementMatrixProvider::Eval (loc_comp_ellbvp.h:266-339)
// with a 2x2 DIFF_COEFF alpha_k, not necessarily symmetric:
//   A_K(i, j) = sum_k w_k |det J_k| [(J_k^-T gh_i)^T alpha_k (J_k^-T gh_j)
//                                     + gamma_k phi_i phi_j].
// With P = adj(J) (J^-1 = P / det J) the gradient term is gh_i^T B_k gh_j,
// B_k = w_k P alpha_k P^T / |det J_k|.  FP64, one thread per cell; the full
// n x n block (no symmetry), one row at a time.

// alpha_k at reference point (xh, yh) of cell c, row-major.
template <bool QUAD>
__device__ void EvalTensorCoeff(const CoeffDev& f, int c, const double2 (&v)[4], double xh, double yh,
                                double (&A)[4]) {
  if (f.kind == LFG_COEFF_TENSOR_CONSTANT) {
    for (int e = 0; e < 4; ++e) A[e] = f.p[e];
  } else if (f.kind == LFG_COEFF_TENSOR_PER_CELL) {
    for (int e = 0; e < 4; ++e) A[e] = f.data[4 * static_cast<int64_t>(c) + e];
  } else {
    double X, Y;
    if (!QUAD) {
      const double l0 = 1.0 - xh - yh;
      X = v[0].x * l0 + v[1].x * xh + v[2].x * yh;
      Y = v[0].y * l0 + v[1].y * xh + v[2].y * yh;
    } else {
      const double b0 = (1 - xh) * (1 - yh), b1 = xh * (1 - yh), b2 = xh * yh, b3 = (1 - xh) * yh;
      X = v[0].x * b0 + v[1].x * b1 + v[2].x * b2 + v[3].x * b3;
      Y = v[0].y * b0 + v[1].y * b1 + v[2].y * b2 + v[3].y * b3;
    }
    for (int e = 0; e < 4; ++e) A[e] = f.p[4 * e] + f.p[4 * e + 1] * X + f.p[4 * e + 2] * Y + f.p[4 * e + 3] * (X * Y);
  }
}

// Jacobian (columns d/dxh, d/dyh) at a reference point: tria_o1.cc:50-74 /
// quad_o1.cc:93-99.
template <bool QUAD>
__device__ __forceinline__ void Jacobian(const double2 (&v)[4], double xh, double yh, double& j00, double& j01,
                                         double& j10, double& j11) {
  if (!QUAD) {
    j00 = v[1].x - v[0].x; j01 = v[2].x - v[0].x;
    j10 = v[1].y - v[0].y; j11 = v[2].y - v[0].y;
  } else {
    j00 = (v[1].x - v[0].x) * (1 - yh) + (v[2].x - v[3].x) * yh;
    j10 = (v[1].y - v[0].y) * (1 - yh) + (v[2].y - v[3].y) * yh;
    j01 = (v[3].x - v[0].x) * (1 - xh) + (v[2].x - v[1].x) * xh;
    j11 = (v[3].y - v[0].y) * (1 - xh) + (v[2].y - v[1].y) * xh;
  }
}

// Shared memory: the rule (w, xh, yh), phi [nq][n], then the O1 values
// [nq][4] and the reference gradients [nq][n][2] (the T / R / L blocks of the
// table are not needed).
template <int DEG, bool QUAD, bool MASS>
__global__ void __launch_bounds__(128) RDTensorKernel(AsmArgs a) {
  constexpr int N = QUAD ? (DEG + 1) * (DEG + 1) : (DEG + 1) * (DEG + 2) / 2;
  extern __shared__ double sm[];
  const int nq = a.L.nq;
  const int head = a.L.off_T, tail = a.L.total - a.L.off_o1;
  for (int i = threadIdx.x; i < head; i += blockDim.x) sm[i] = a.tab[i];
  for (int i = threadIdx.x; i < tail; i += blockDim.x) sm[head + i] = a.tab[a.L.off_o1 + i];
  __syncthreads();
  const double* sw = sm + a.L.off_w;
  const double* sqx = sm + a.L.off_qx;
  const double* sqy = sm + a.L.off_qy;
  const double* sphi = sm + a.L.off_phi;
  const double* so1 = sm + head;
  const double* sG = so1 + nq * 4;
  for (int64_t t = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; t < a.count;
       t += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int c = a.bucket[t];
    int4 cn;
    double2 v[4];
    LoadVerts<QUAD>(a, c, cn, v);
    int dofs[N];
#pragma unroll
    for (int i = 0; i < N; ++i) dofs[i] = a.cell_dofs[static_cast<int64_t>(c) * a.n_cell + i];
    lfg_triplet* base = a.out + a.tri_offset[c];
    for (int i = 0; i < N; ++i) {
      double acc[N];
#pragma unroll
      for (int j = 0; j < N; ++j) acc[j] = 0.0;
      for (int k = 0; k < nq; ++k) {
        double j00, j01, j10, j11;
        Jacobian<QUAD>(v, sqx[k], sqy[k], j00, j01, j10, j11);
        const double adet = fabs(j00 * j11 - j10 * j01);
        double A[4];
        EvalTensorCoeff<QUAD>(a.alpha, c, v, sqx[k], sqy[k], A);
        // P = adj(J) = [[j11, -j01], [-j10, j00]]; Q = P alpha; B = w Q P^T / |det J|
        const double q00 = j11 * A[0] - j01 * A[2], q01 = j11 * A[1] - j01 * A[3];
        const double q10 = -j10 * A[0] + j00 * A[2], q11 = -j10 * A[1] + j00 * A[3];
        const double s = sw[k] / adet;
        const double b00 = s * (q00 * j11 - q01 * j01), b01 = s * (-q00 * j10 + q01 * j00);
        const double b10 = s * (q10 * j11 - q11 * j01), b11 = s * (-q10 * j10 + q11 * j00);
        const double gi0 = sG[(k * N + i) * 2], gi1 = sG[(k * N + i) * 2 + 1];
        const double r0 = gi0 * b00 + gi1 * b10, r1 = gi0 * b01 + gi1 * b11;
        double mi = 0.0;
        if (MASS) mi = sw[k] * adet * EvalCoeff<QUAD>(a.gamma, c, cn, v, k, sw, sqx, sqy, so1) * sphi[k * N + i];
#pragma unroll
        for (int j = 0; j < N; ++j) {
          double r = fma(r0, sG[(k * N + j) * 2], acc[j]);
          r = fma(r1, sG[(k * N + j) * 2 + 1], r);
          if (MASS) r = fma(mi, sphi[k * N + j], r);
          acc[j] = r;
        }
      }
#pragma unroll
      for (int j = 0; j < N; ++j) StoreTriplet(base + i * N + j, dofs[i], dofs[j], acc[j]);
    }
  }
}

// ------------------------------------ cell-constant coefficients, df32 path
// Triangles and quadrilaterals with constant / per-cell alpha and gamma.  One
// thread per cell computes the upper triangle of A_K in df32 (lfg_elem.h):
// FP64 only for the coordinate differences, everything else on the FP32
// pipes (GB300 issues ~60 FP32 FMAs per FP64 operation).  Cells whose inputs
// leave the df32-safe range take the FP64 formula instead.  The values and
// dof indices of a 128-cell tile are staged in shared memory and written out
// as fully coalesced 16-byte triplets (every 32-byte sector is written whole).

// Upper-triangle index of (i, j), i <= j, in "for i: for j >= i" order.
template <int N>
__device__ __forceinline__ int UpperIndex(int i, int j) {
  const int a = i < j ? i : j, b = i < j ? j : i;
  return a * N - (a * (a - 1)) / 2 + (b - a);
}

// (i, j, upper index) of triplet w = i N + j of an element block, packed as
// i | j << 8 | u << 16; filled once per CTA (no per-triplet index arithmetic).
template <int N>
__device__ __forceinline__ void FillTripletMap(int* smap) {
  for (int w = threadIdx.x; w < N * N; w += blockDim.x) {
    const int i = w / N, j = w - i * N;
    smap[w] = i | (j << 8) | (UpperIndex<N>(i, j) << 16);
  }
}

// Writes the staged tile: triplet w of cell cl goes to out + off[cl] + w;
// consecutive threads take consecutive triplets of the tile (blocks of
// consecutive cells are mostly adjacent), so stores are 16-byte coalesced.
template <int N>
__device__ __forceinline__ void WriteTile(lfg_triplet* out, int ncell, const double* svals,
                                          const int* sdofs, const int64_t* soff, const int* smap) {
  constexpr int NN = N * N, E = N * (N + 1) / 2;
  for (int q = threadIdx.x; q < ncell * NN; q += blockDim.x) {
    const int cl = q / NN, w = q - cl * NN;
    const int m = smap[w];
    const int* dofs = sdofs + cl * N;
    StoreTriplet(out + soff[cl] + w, dofs[m & 0xff], dofs[(m >> 8) & 0xff], svals[cl * E + (m >> 16)]);
  }
}

struct DfArgs {
  const float* tab;  // df32 table block (pairs)
  DfLayout L;
};

template <int DEG, bool MASS>
__global__ void __launch_bounds__(128) RDTriaDfKernel(AsmArgs a, DfArgs d) {
  using elem::f2;
  constexpr int N = (DEG + 1) * (DEG + 2) / 2;
  constexpr int E = N * (N + 1) / 2;
  constexpr int TILE = 128;
  extern __shared__ __align__(16) unsigned char smraw[];
  f2* sR = reinterpret_cast<f2*>(smraw);
  double* svals = reinterpret_cast<double*>(smraw + ((E * 4 * sizeof(f2) + 15) & ~15));
  int64_t* soff = reinterpret_cast<int64_t*>(svals + TILE * E);
  int* sdofs = reinterpret_cast<int*>(soff + TILE);
  __shared__ int smap[N * N];
  const f2* gR = reinterpret_cast<const f2*>(d.tab) + d.L.off_R;
  for (int i = threadIdx.x; i < E * 4; i += blockDim.x) sR[i] = gR[i];
  FillTripletMap<N>(smap);
  __syncthreads();
  for (int64_t t0 = static_cast<int64_t>(blockIdx.x) * TILE; t0 < a.count;
       t0 += static_cast<int64_t>(gridDim.x) * TILE) {
    const int ncell = static_cast<int>(a.count - t0 < TILE ? a.count - t0 : TILE);
    if (threadIdx.x < ncell) {
      const int c = a.bucket[t0 + threadIdx.x];
      int4 cn;
      double2 v[4];
      LoadVerts<false>(a, c, cn, v);
      const double jac[4] = {v[1].x - v[0].x, v[2].x - v[0].x, v[1].y - v[0].y, v[2].y - v[0].y};
      const double al = CellConst(a.alpha, c);
      const double ga = MASS ? CellConst(a.gamma, c) : 0.0;
      double* vals = svals + threadIdx.x * E;
      if (elem::DfSafe(jac[0]) && elem::DfSafe(jac[1]) && elem::DfSafe(jac[2]) && elem::DfSafe(jac[3]) &&
          elem::DfSafe(al) && elem::DfSafe(ga)) {
        elem::TriaUniformDF<E, MASS>(jac, al, ga, sR, vals);
      } else {
        elem::TriaUniformF64<E, MASS>(jac, al, ga, a.tab + a.L.off_R, vals);
        atomicAdd(a.fallback, 1ull);
      }
#pragma unroll
      for (int i = 0; i < N; ++i) sdofs[threadIdx.x * N + i] = a.cell_dofs[static_cast<int64_t>(c) * a.n_cell + i];
      soff[threadIdx.x] = a.tri_offset[c];
    }
    __syncthreads();
    WriteTile<N>(a.out, ncell, svals, sdofs, soff, smap);
    __syncthreads();
  }
}

// ------------------------------ point-varying alpha on triangles, df32 path
// Affine triangles whose alpha varies over the cell (analytic families, O1
// nodal interpolant) and whose gamma is cell-constant: per point
// c_k = w_k alpha(x_k) |det J| J^-1 J^-T in df32 (the analytic families through
// SinCosPiDF / Horner, the global point from the FP64 vertex differences),
// A(e) = sum_k c_k . T_k(e) + gamma |det J| R_mass(e).  Cells with an input or
// a point value outside the df32 range take the FP64 per-point formula.

// FP64 per-point formula for one affine triangle with point-varying alpha
// (rarely taken; runtime loops keep it small).
template <int N>
__device__ void TriaVaryF64(const AsmArgs& a, int c, const int4& cn, const double2 (&v)[4], double* vals) {
  constexpr int E = N * (N + 1) / 2;
  const double* tab = a.tab;
  const Tab& L = a.L;
  double m00, m01, m11, adet;
  TriaMetric(v, m00, m01, m11, adet);
  const double ga = CellConst(a.gamma, c);
  for (int e = 0; e < E; ++e) vals[e] = 0.0;
#pragma unroll 1
  for (int k = 0; k < L.nq; ++k) {
    const double al = EvalCoeff<false>(a.alpha, c, cn, v, k, tab + L.off_w, tab + L.off_qx, tab + L.off_qy,
                                       tab + L.off_o1);
    const double s = tab[L.off_w + k] * al;
    const double mk = tab[L.off_w + k] * adet * ga;
    const double* Tk = tab + L.off_T + k * E * 4;
#pragma unroll 1
    for (int e = 0; e < E; ++e) {
      double r = vals[e];
      r = fma(s * m00, Tk[e * 4 + 0], r);
      r = fma(s * m01, Tk[e * 4 + 1], r);
      r = fma(s * m11, Tk[e * 4 + 2], r);
      r = fma(mk, Tk[e * 4 + 3], r);
      vals[e] = r;
    }
  }
}

template <int DEG, int NQ>
__global__ void __launch_bounds__(128) RDTriaVaryDfKernel(AsmArgs a, DfArgs d) {
  using elem::f2;
  namespace df = lfg::df;
  constexpr int N = (DEG + 1) * (DEG + 2) / 2;
  constexpr int E = N * (N + 1) / 2;
  constexpr int TILE = 128;
  constexpr int TP = NQ * E * 4 + E * 4 + NQ + 2 * NQ + 4 * NQ + 23;  // T, R, W, X, O1, SC
  extern __shared__ __align__(16) unsigned char smraw[];
  f2* sT = reinterpret_cast<f2*>(smraw);
  f2* sR = sT + NQ * E * 4;
  f2* sW = sR + E * 4;
  f2* sX = sW + NQ;
  f2* sO1 = sX + 2 * NQ;
  f2* sSC = sO1 + 4 * NQ;
  double* svals = reinterpret_cast<double*>(smraw + ((TP * sizeof(f2) + 15) & ~15));
  int64_t* soff = reinterpret_cast<int64_t*>(svals + TILE * E);
  int* sdofs = reinterpret_cast<int*>(soff + TILE);
  __shared__ int smap[N * N];
  const f2* g = reinterpret_cast<const f2*>(d.tab);
  for (int i = threadIdx.x; i < NQ * E * 4; i += blockDim.x) sT[i] = g[d.L.off_T + i];
  for (int i = threadIdx.x; i < E * 4; i += blockDim.x) sR[i] = g[d.L.off_R + i];
  for (int i = threadIdx.x; i < NQ; i += blockDim.x) sW[i] = g[d.L.off_W + i];
  for (int i = threadIdx.x; i < 2 * NQ; i += blockDim.x) sX[i] = g[d.L.off_X + i];
  for (int i = threadIdx.x; i < 4 * NQ; i += blockDim.x) sO1[i] = g[d.L.off_O1 + i];
  for (int i = threadIdx.x; i < 23; i += blockDim.x) sSC[i] = g[d.L.off_SC + i];
  FillTripletMap<N>(smap);
  __syncthreads();
  elem::AnalyticDF af;
  af.func = a.alpha.func;
#pragma unroll
  for (int i = 0; i < 16; ++i) af.p[i] = df::FromDouble(a.alpha.p[i]);
  const bool mass = a.gamma.kind != LFG_COEFF_ZERO;
  for (int64_t t0 = static_cast<int64_t>(blockIdx.x) * TILE; t0 < a.count;
       t0 += static_cast<int64_t>(gridDim.x) * TILE) {
    const int ncell = static_cast<int>(a.count - t0 < TILE ? a.count - t0 : TILE);
    if (threadIdx.x < ncell) {
      const int c = a.bucket[t0 + threadIdx.x];
      int4 cn;
      double2 v[4];
      LoadVerts<false>(a, c, cn, v);
      const double jac[4] = {v[1].x - v[0].x, v[2].x - v[0].x, v[1].y - v[0].y, v[2].y - v[0].y};
      const double ga = mass ? CellConst(a.gamma, c) : 0.0;
      double* vals = svals + threadIdx.x * E;
      bool safe = elem::DfSafe(ga) && elem::DfSafe(v[0].x) && elem::DfSafe(v[0].y);
#pragma unroll
      for (int k = 0; k < 4; ++k) safe = safe && elem::DfSafe(jac[k]);
      f2 cpt[NQ][3];
      f2 mm = df::Make(0.0f);
      if (safe) {
        const f2 j00 = df::FromDouble(jac[0]), j01 = df::FromDouble(jac[1]);
        const f2 j10 = df::FromDouble(jac[2]), j11 = df::FromDouble(jac[3]);
        f2 m00, m01, m11, adet;
        elem::TriaMetricDF(j00, j01, j10, j11, m00, m01, m11, adet);
        const f2 x0 = df::FromDouble(v[0].x), y0 = df::FromDouble(v[0].y);
        f2 nod[3];
        if (a.alpha.kind == LFG_COEFF_NODAL_O1) {
          const double n0 = a.alpha.data[cn.x], n1 = a.alpha.data[cn.y], n2 = a.alpha.data[cn.z];
          safe = elem::DfSafe(n0) && elem::DfSafe(n1) && elem::DfSafe(n2);
          nod[0] = df::FromDouble(n0);
          nod[1] = df::FromDouble(n1);
          nod[2] = df::FromDouble(n2);
        }
#pragma unroll
        for (int k = 0; k < NQ; ++k) {
          f2 al;
          if (a.alpha.kind == LFG_COEFF_NODAL_O1) {
            al = df::Mul(nod[0], sO1[4 * k]);
            al = df::MulAdd(nod[1], sO1[4 * k + 1], al);
            al = df::MulAdd(nod[2], sO1[4 * k + 2], al);
          } else {
            const f2 xh = sX[2 * k], yh = sX[2 * k + 1];
            const f2 X = df::MulAdd(j01, yh, df::MulAdd(j00, xh, x0));
            const f2 Y = df::MulAdd(j11, yh, df::MulAdd(j10, xh, y0));
            al = elem::EvalAnalyticDF(af, X, Y, sSC, sSC + 11);
          }
          // 2^-30 margin below the df32 range of the products
          const float aa = fabsf(al.h);
          safe = safe && (aa == 0.0f || (aa > 8.0e-10f && aa < 1.0e9f));
          const f2 s = df::Mul(sW[k], al);
          cpt[k][0] = df::Mul(s, m00);
          cpt[k][1] = df::Mul(s, m01);
          cpt[k][2] = df::Mul(s, m11);
        }
        if (mass) mm = df::Mul(df::FromDouble(ga), adet);
      }
      if (safe) {
        elem::TriaVaryContractDF<E, NQ>(cpt, sT, mm, mass, sR, vals);
      } else {
        TriaVaryF64<N>(a, c, cn, v, vals);
        atomicAdd(a.fallback, 1ull);
      }
#pragma unroll
      for (int i = 0; i < N; ++i) sdofs[threadIdx.x * N + i] = a.cell_dofs[static_cast<int64_t>(c) * a.n_cell + i];
      soff[threadIdx.x] = a.tri_offset[c];
    }
    __syncthreads();
    WriteTile<N>(a.out, ncell, svals, sdofs, soff, smap);
    __syncthreads();
  }
}

// FP64 per-point formula of a quadrilateral with cell-constant coefficients
// (cells outside the df32 range), accumulating into vals[E].
template <int N, bool MASS>
__device__ void QuadUniformF64(const double2 (&v)[4], double al, double ga, const double* tab, const Tab& L,
                               double* vals) {
  constexpr int E = N * (N + 1) / 2;
  for (int e = 0; e < E; ++e) vals[e] = 0.0;
  for (int k = 0; k < L.nq; ++k) {
    double m00, m01, m11, adet;
    QuadMetric(v, tab[L.off_qx + k], tab[L.off_qy + k], m00, m01, m11, adet);
    const double s = tab[L.off_w + k] * al;
    const double mk = tab[L.off_w + k] * adet * ga;
    const double* Tk = tab + L.off_T + k * E * 4;
    for (int e = 0; e < E; ++e) {
      double r = vals[e];
      r = fma(s * m00, Tk[e * 4 + 0], r);
      r = fma(s * m01, Tk[e * 4 + 1], r);
      r = fma(s * m11, Tk[e * 4 + 2], r);
      if (MASS) r = fma(mk, Tk[e * 4 + 3], r);
      vals[e] = r;
    }
  }
}

// Per-point term tables of the direct quad contraction live in shared
// memory: [NQ][E][4], then W[NQ], t[M].
template <int DEG, int M>
constexpr int QuadTabPairs() {
  return M * M * ((DEG + 1) * (DEG + 1) * ((DEG + 1) * (DEG + 1) + 1) / 2) * 4;
}

// The sum-factorised path's tables ([3][N1][N1][M] 1D products, W[M*M],
// t[M]) live in constant memory, one slot per (degree 2-3, points 2-4): with
// the slot offset and the loop indices known at compile time, the stage-2
// operands are read by the arithmetic instructions straight from the
// constant bank (no load instruction, no index arithmetic).
template <int DEG, int M>
constexpr int SfSlotPairs() {
  return 3 * (DEG + 1) * (DEG + 1) * M + M * M + M;
}
constexpr int SfSlotIndex(int deg, int m) { return (deg - 2) * 3 + (m - 2); }
template <int DEG, int M>
constexpr int SfSlotOffset() {
  int off = 0;
  for (int d = 2; d <= 3; ++d)
    for (int m = 2; m <= 4; ++m) {
      if (d == DEG && m == M) return off;
      off += 3 * (d + 1) * (d + 1) * m + m * m + m;
    }
  return off;
}
constexpr int kSfConstPairs = SfSlotOffset<4, 2>();  // past the last slot
__constant__ float2 c_sf_tables[kSfConstPairs];

template <int DEG, int M, bool MASS, bool SF>
__global__ void __launch_bounds__(128) RDQuadDfKernel(AsmArgs a, DfArgs d) {
  using elem::f2;
  constexpr int N = (DEG + 1) * (DEG + 1);
  constexpr int E = N * (N + 1) / 2;
  constexpr int NQ = M * M;
  constexpr int TILE = E > 64 ? 64 : 128;
  constexpr int TP = SF ? 0 : QuadTabPairs<DEG, M>();
  constexpr int SMT = SF ? 0 : TP + NQ + M;  // table pairs in shared memory
  extern __shared__ __align__(16) unsigned char smraw[];
  f2* sT = reinterpret_cast<f2*>(smraw);
  const f2* tW;
  const f2* tt;
  const f2* tsf = nullptr;
  if (SF) {
    const f2* slot = reinterpret_cast<const f2*>(c_sf_tables) + SfSlotOffset<(SF ? DEG : 2), M>();
    tsf = slot;
    tW = slot + 3 * (DEG + 1) * (DEG + 1) * M;
    tt = tW + NQ;
  } else {
    tW = sT + TP;
    tt = tW + NQ;
  }
  double* svals = reinterpret_cast<double*>(smraw + ((SMT * sizeof(f2) + 15) & ~15));
  int64_t* soff = reinterpret_cast<int64_t*>(svals + TILE * E);
  int* sdofs = reinterpret_cast<int*>(soff + TILE);
  __shared__ int sloc[16];
  __shared__ int smap[N * N];
  FillTripletMap<N>(smap);
  const f2* g = reinterpret_cast<const f2*>(d.tab);
  if (!SF) {
    for (int i = threadIdx.x; i < TP; i += blockDim.x) sT[i] = g[d.L.off_T + i];
    for (int i = threadIdx.x; i < NQ; i += blockDim.x) sT[TP + i] = g[d.L.off_W + i];
    for (int i = threadIdx.x; i < M; i += blockDim.x) sT[TP + NQ + i] = g[d.L.off_t + i];
  }
  if (threadIdx.x == 0) {
#pragma unroll
    for (int i = 0; i < 16; ++i) sloc[i] = d.L.loc[i];  // static indices: no local copy of the parameter
  }
  __syncthreads();
  for (int64_t t0 = static_cast<int64_t>(blockIdx.x) * TILE; t0 < a.count;
       t0 += static_cast<int64_t>(gridDim.x) * TILE) {
    const int ncell = static_cast<int>(a.count - t0 < TILE ? a.count - t0 : TILE);
    if (threadIdx.x < ncell) {
      const int c = a.bucket[t0 + threadIdx.x];
      int4 cn;
      double2 v[4];
      LoadVerts<true>(a, c, cn, v);
      // J col0 = a + d yh, col1 = c + d xh (quad_o1.cc:93-99)
      const double acd[6] = {v[1].x - v[0].x, v[1].y - v[0].y, v[3].x - v[0].x, v[3].y - v[0].y,
                             (v[0].x - v[1].x) + (v[2].x - v[3].x), (v[0].y - v[1].y) + (v[2].y - v[3].y)};
      const double al = CellConst(a.alpha, c);
      const double ga = MASS ? CellConst(a.gamma, c) : 0.0;
      double* vals = svals + threadIdx.x * E;
      bool safe = elem::DfSafe(al) && elem::DfSafe(ga);
#pragma unroll
      for (int k = 0; k < 6; ++k) safe = safe && elem::DfSafe(acd[k]);
      if (safe) {
        f2 cpt[NQ][4];
        elem::QuadPointCoeffsDF<M, MASS>(acd, al, ga, tt, tW, cpt);
        if (SF) elem::QuadSumFactDF<DEG + 1, M, MASS>(cpt, tsf, sloc, vals);
        else elem::QuadContractDF<E, NQ, MASS>(cpt, sT, vals);
      } else {
        QuadUniformF64<N, MASS>(v, al, ga, a.tab, a.L, vals);
        atomicAdd(a.fallback, 1ull);
      }
#pragma unroll
      for (int i = 0; i < N; ++i) sdofs[threadIdx.x * N + i] = a.cell_dofs[static_cast<int64_t>(c) * a.n_cell + i];
      soff[threadIdx.x] = a.tri_offset[c];
    }
    __syncthreads();
    WriteTile<N>(a.out, ncell, svals, sdofs, soff, smap);
    __syncthreads();
  }
}

// ------------------------------------------ quadrilaterals on the tensor cores
// Q2 on bilinear quadrilaterals, cell-constant alpha, gamma = 0, tensor Gauss
// rule of M x M points (M = 2, 3).  The direct contraction
//     A_K(e) = sum_kap c_kap(K) T(kap; e),  kap = 3 k + ab (point k, metric entry ab)
// is a (128 cells x K) by (K x 45 entries) product per tile.  It runs on the
// FP16 tensor cores (tcgen05, FP32 accumulation in tensor memory) without
// losing FP64 accuracy, by splitting both operands into integer digits of 9
// bits (an Ozaki-type splitting):
//   row (cell):     c = 2^Er  sum_{i=1..6} a_i 2^-9i,  Er from the row's largest |c|,
//   column (entry): T = 2^Ec  sum_{j=1..6} b_j 2^-9j,  Ec from the column's largest |T| (host),
// |a_i|, |b_j| <= 257.  A digit product is an integer below 2^17, and the sum
// over the 27 kap of all pairs of one level L = i + j stays below 2^24 for
// L <= 5 (at most 4 pairs), so the FP32 accumulators of levels 2, 3, 4, 5 are
// exact.  Levels 6 and 7 share a fifth accumulator in which the level-7 terms
// enter with 2^-9-scaled table digits; it rounds only below 2^-54 of
// 2^(Er + Ec).  Levels >= 8 are left out (below 2^-48 of 2^(Er + Ec)).  The
// epilogue recombines the five accumulators of an entry into one int64
// (G2 2^36 + G3 2^27 + G4 2^18 + G5 2^9 + G67) and one binary64.
//
// Tensor memory: 5 accumulators x 48 columns (45 entries padded) = 240 of the
// 256 columns this CTA allocates; two CTAs share an SM.  Per tile and K step
// of 16: five MMAs (A digit i against table digits 1..6-i in one N = (6-i) x 48
// product whose columns land on levels i+1..6) and six N = 48 MMAs for level 7.
// Shared memory: A digits [6][128 x KP] (reused for the FP64 tile after the
// MMAs), table digits [2][6 x 48 x KP] (plain, 2^-9 scaled), column exponents,
// tile dof indices and offsets.  Cells outside the df32-safe range take the
// FP64 formula in the epilogue.
// Threads: 256 per CTA, two per cell (row r = TMEM lane r): half 0 computes
// the points [0, P0) and fills K columns [0, KP/2), half 1 the other points
// and columns; in the epilogue each half converts 24 of the 48 entry columns.
// The tile is then written one warp per cell, 32 consecutive triplets per store.
constexpr uint32_t kTcMaxPolls = 1u << 22;
constexpr int kTcNP = 48;       // accumulator columns per level (45 entries + 3)
constexpr int kTcCols = 256;    // tensor memory columns per CTA

__host__ __device__ constexpr int TcKP(int m) { return (3 * m * m + 15) / 16 * 16; }
__host__ __device__ constexpr int TcABytes(int m) {
  return 6 * 256 * TcKP(m) > 128 * 45 * 8 ? 6 * 256 * TcKP(m) : 128 * 45 * 8;
}
__host__ __device__ constexpr int TcBHalfBytes(int m) { return 6 * kTcNP * TcKP(m) * 2; }
// one 16-row block whose row 0 picks K column KP-1 of A digit 1 (the row info)
__host__ __device__ constexpr int TcInfoBytes(int m) { return 16 * TcKP(m) * 2; }
__host__ __device__ constexpr int TcEcOffset(int m) { return 2 * TcBHalfBytes(m) + TcInfoBytes(m); }
__host__ __device__ constexpr int TcImageBytes(int m) { return TcEcOffset(m) + kTcNP * 4; }
__host__ __device__ constexpr int TcSmemBytes(int m) {
  return TcABytes(m) + TcImageBytes(m) + 128 * 9 * 4 + 128 * 8;
}

__device__ __forceinline__ uint32_t HSub2(uint32_t a, uint32_t b) {
  uint32_t d;
  asm("sub.rn.f16x2 %0, %1, %2;" : "=r"(d) : "r"(a), "r"(b));
  return d;
}

// G2 2^36 + G3 2^27 + G4 2^18 + G5 2^9 + G67 scaled by 2^shift, as binary64.
__device__ __forceinline__ double TcCombine(float g2, float g3, float g4, float g5, float g67, int shift) {
  // |G2|, |G3| < 2^22: integer bits by the 1.5 2^23 shift on the FP32 pipe
  const int i2 = __float_as_int(__fadd_rn(g2, 12582912.0f)) - 0x4B400000;
  const int i3 = __float_as_int(__fadd_rn(g3, 12582912.0f)) - 0x4B400000;
  const int hi = i2 * 512 + i3;
  const long long mid = static_cast<long long>(__float2int_rn(g4)) * 512 + __float2int_rn(g5);
  const long long t = static_cast<long long>(hi) * (1ll << 27) + mid * 512 + __float2int_rn(g67);
  if (t == 0) return 0.0;
  return __longlong_as_double(__double_as_longlong(__ll2double_rn(t)) + (static_cast<long long>(shift) << 52));
}

// elem::DfSafe on the exponent bits (integer pipe; |x| = 2^40 exactly counts
// as outside, which only sends such a cell to the FP64 formula).
__device__ __forceinline__ bool DfSafeBits(double x) {
  const unsigned long long u = static_cast<unsigned long long>(__double_as_longlong(x)) << 1;
  const uint32_t ex = static_cast<uint32_t>(u >> 53);
  return u == 0 || (ex >= 1023u - 40u && ex < 1023u + 40u);
}

// FP64 formula for a cell outside the df32 range (rare; kept out of line so
// that it stays out of the instruction cache of the main path).
__device__ __noinline__ void TcFallback(const double2 (&v)[4], double al, const AsmArgs& a, double* vals) {
  QuadUniformF64<9, false>(v, al, 0.0, a.tab, a.L, vals);
}

// Inputs of cell bucket[t0 + r] (vertices, alpha), loaded one tile ahead.
__device__ __forceinline__ void TcFetch(const AsmArgs& a, int64_t t0, int r, int& c, double2 (&v)[4], double& al) {
  if (t0 + r < a.count) {
    int4 cn;
    c = a.bucket[t0 + r];
    LoadVerts<true>(a, c, cn, v);
    al = CellConst(a.alpha, c);
  }
}

// Kappa column of (point k, entry ab): the points [0, P0) of thread half 0
// fill columns [0, KP/2), the points [P0, NQ) of half 1 columns [KP/2, KP).
__host__ __device__ constexpr int TcKappa(int m, int k, int ab) {
  return k < (m * m + 1) / 2 ? 3 * k + ab : TcKP(m) / 2 + 3 * (k - (m * m + 1) / 2) + ab;
}

template <int M>
__global__ void __launch_bounds__(256) RDQuadTcKernel(AsmArgs a, DfArgs d, const uint4* __restrict__ image,
                                                      int* __restrict__ tc_timeouts) {
  using elem::f2;
  constexpr int N = 9, E = 45, NQ = M * M, KP = TcKP(M), KS = KP / 16, NP = kTcNP;
  constexpr int P0 = (NQ + 1) / 2;   // points of thread half 0
  constexpr int PH = P0;             // point slots per half (half 1 has NQ - P0 <= P0)
  constexpr int HC = KP / 16;        // K cores (8 columns) per half
  constexpr uint32_t SA = 256 * KP;  // one digit slice of the A tile, bytes
  constexpr uint32_t SBO = KP * 16;  // 8-row group stride of both operands
  static_assert(3 * P0 <= KP / 2, "a half's points must fit its columns");
  extern __shared__ __align__(1024) unsigned char smraw[];
  unsigned char* sA = smraw;
  unsigned char* sB = smraw + TcABytes(M);
  const int* sEc = reinterpret_cast<const int*>(sB + TcEcOffset(M));
  int* sdofs = reinterpret_cast<int*>(sB + TcImageBytes(M));
  int64_t* soff = reinterpret_cast<int64_t*>(sdofs + 128 * N);
  double* svals = reinterpret_cast<double*>(sA);
  __shared__ f2 sWt[NQ + M];
  __shared__ uint32_t smax[2][128];
  __shared__ __align__(8) uint64_t mbar;
  __shared__ uint32_t s_taddr;

  {
    const f2* g = reinterpret_cast<const f2*>(d.tab);
    for (int i = threadIdx.x; i < NQ; i += blockDim.x) sWt[i] = g[d.L.off_W + i];
    for (int i = threadIdx.x; i < M; i += blockDim.x) sWt[NQ + i] = g[d.L.off_t + i];
    uint4* dst = reinterpret_cast<uint4*>(sB);
    for (int i = threadIdx.x; i < TcImageBytes(M) / 16; i += blockDim.x) dst[i] = image[i];
  }
  if (threadIdx.x == 0) tc::MbarInit(&mbar, 1);
  if (threadIdx.x < 32) tc::TmemAlloc(&s_taddr, kTcCols);
  tc::FenceProxyAsync();
  tc::FenceBeforeSync();
  __syncthreads();
  tc::FenceAfterSync();
  const uint32_t taddr = s_taddr;
  const int half = threadIdx.x >> 7, r = threadIdx.x & 127, warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t tlane = taddr + (static_cast<uint32_t>((r >> 5) * 32) << 16);
  // triplets lane, lane + 32, lane + 64 of a cell: i | j << 8 | upper index << 16
  int tmap[3];
#pragma unroll
  for (int t = 0; t < 3; ++t) {
    const int w = lane + 32 * t, i = w / N, j = w - i * N;
    tmap[t] = w < N * N ? (i | (j << 8) | (UpperIndex<N>(i, j) << 16)) : -1;
  }
  uint32_t phase = 0;
  bool abort = false;
  int c = 0;
  double2 v[4] = {};
  double al = 0.0;
  TcFetch(a, static_cast<int64_t>(blockIdx.x) * 128, r, c, v, al);

  for (int64_t t0 = static_cast<int64_t>(blockIdx.x) * 128; t0 < a.count && !abort;
       t0 += static_cast<int64_t>(gridDim.x) * 128) {
    const int ncell = static_cast<int>(a.count - t0 < 128 ? a.count - t0 : 128);
    // ---- cell r, points of this half: df32 coefficients
    bool safe = false;
    f2 cpt[PH][3];
#pragma unroll
    for (int k = 0; k < PH; ++k)
#pragma unroll
      for (int q = 0; q < 3; ++q) cpt[k][q] = f2{0.0f, 0.0f};
    float mx = 0.0f;
    if (half == 1 && r < ncell) {  // dof indices and triplet offset of the cell, for the write phase
      const int32_t* g = a.cell_dofs + static_cast<int64_t>(c) * a.n_cell;
#pragma unroll
      for (int i = 0; i < N; ++i) tc::CpAsync4(sdofs + r * N + i, g + i);
      tc::CpAsync8(soff + r, a.tri_offset + c);
    }
    tc::CpAsyncCommit();
    if (r < ncell) {
      const double acd[6] = {v[1].x - v[0].x, v[1].y - v[0].y, v[3].x - v[0].x, v[3].y - v[0].y,
                             (v[0].x - v[1].x) + (v[2].x - v[3].x), (v[0].y - v[1].y) + (v[2].y - v[3].y)};
      safe = DfSafeBits(al);
#pragma unroll
      for (int k = 0; k < 6; ++k) safe = safe && DfSafeBits(acd[k]);
      if (safe) {
        if (half == 0) elem::QuadPointCoeffsRangeDF<M, 0, P0>(acd, al, sWt + NQ, sWt, cpt);
        else elem::QuadPointCoeffsRangeDF<M, P0, NQ>(acd, al, sWt + NQ, sWt, cpt);
      }
#pragma unroll
      for (int k = 0; k < PH; ++k)
#pragma unroll
        for (int q = 0; q < 3; ++q) mx = fmaxf(mx, fabsf(cpt[k][q].h));
    }
    smax[half][r] = __float_as_uint(mx);
    __syncthreads();
    // ---- row exponent (both halves), digits of this half's columns -> A tile
    const uint32_t mb = max(smax[0][r], smax[1][r]);
    int e = mb ? static_cast<int>((mb >> 23) & 0xffu) - 127 : 0;
    if (e < -70 || e > 70) safe = false;
    if (!safe) {
#pragma unroll
      for (int k = 0; k < PH; ++k)
#pragma unroll
        for (int q = 0; q < 3; ++q) cpt[k][q] = f2{0.0f, 0.0f};
      e = 0;
    }
    const float scale = __uint_as_float(static_cast<uint32_t>(127 + 52 - e) << 23);  // 2^(52 - e)
    unsigned char* arow = sA + (r >> 3) * SBO + (r & 7) * 16 + half * HC * 128;
#pragma unroll
    for (int gk = 0; gk < HC; ++gk) {
      uint32_t w[6][4];
#pragma unroll
      for (int pr = 0; pr < 4; ++pr) {
        uint32_t p[2][6];
#pragma unroll
        for (int s = 0; s < 2; ++s) {
          const int kl = gk * 8 + 2 * pr + s;  // column within the half
          const f2 x = kl < 3 * PH ? cpt[kl / 3][kl % 3] : f2{0.0f, 0.0f};
          // V = round(c 2^(54-Er)) = vhi 2^27 + vlo; W = V + bias = whi 2^27 + wlo, wlo in [0, 2^27)
          const float hs = x.h * scale;
          const int vhi = __float2int_rn(hs * 7.450580596923828125e-9f);  // 2^-27
          const float rem = __fmaf_rn(static_cast<float>(vhi), -134217728.0f, hs);  // exact
          const int wlo0 = __float2int_rn(rem) + __float2int_rn(x.l * scale) + 256 * ((1 << 18) + (1 << 9) + 1);
          const int whi = vhi + 256 * ((1 << 9) + 1) + (wlo0 >> 27);
          const uint32_t wlo = static_cast<uint32_t>(wlo0) & ((1u << 27) - 1u);
          p[s][0] = 0x6600u + static_cast<uint32_t>(whi >> 18);
          p[s][1] = 0x6400u | ((static_cast<uint32_t>(whi) >> 9) & 511u);
          p[s][2] = 0x6400u | (static_cast<uint32_t>(whi) & 511u);
          p[s][3] = 0x6400u | ((wlo >> 18) & 511u);
          p[s][4] = 0x6400u | ((wlo >> 9) & 511u);
          p[s][5] = 0x6400u | (wlo & 511u);
        }
#pragma unroll
        for (int i = 0; i < 6; ++i)
          w[i][pr] = HSub2(__byte_perm(p[0][i], p[1][i], 0x5410), i == 0 ? 0x66006600u : 0x65006500u);
      }
#pragma unroll
      for (int i = 0; i < 6; ++i)
        *reinterpret_cast<uint4*>(arow + i * SA + gk * 128) = make_uint4(w[i][0], w[i][1], w[i][2], w[i][3]);
    }
    tc::FenceProxyAsync();
    __syncthreads();
    // ---- one thread issues the tile's MMAs
    if (threadIdx.x == 0) {
      tc::FenceAfterSync();
      const uint32_t a0 = tc::SmemAddr(sA), bu = tc::SmemAddr(sB), bs = bu + TcBHalfBytes(M);
#pragma unroll
      for (int s = 0; s < KS; ++s)
#pragma unroll
        for (int i = 1; i <= 5; ++i)
          tc::MmaF16(taddr + (i - 1) * NP, tc::SmemDesc(a0 + (i - 1) * SA + s * 256, 128, SBO),
                     tc::SmemDesc(bu + s * 256, 128, SBO), tc::IdescF16(128, (6 - i) * NP), s > 0 || i > 1);
#pragma unroll
      for (int s = 0; s < KS; ++s)
#pragma unroll
        for (int i = 1; i <= 6; ++i)
          tc::MmaF16(taddr + 4 * NP, tc::SmemDesc(a0 + (i - 1) * SA + s * 256, 128, SBO),
                     tc::SmemDesc(bs + (6 - i) * (NP / 8) * SBO + s * 256, 128, SBO), tc::IdescF16(128, NP), true);
      tc::Commit(&mbar);
    }
    // next tile's cell inputs load while the tensor cores work
    int c_n = 0;
    double2 v_n[4] = {};
    double al_n = 0.0;
    TcFetch(a, t0 + static_cast<int64_t>(gridDim.x) * 128, r, c_n, v_n, al_n);
    const bool ok = tc::MbarWait(&mbar, phase, kTcMaxPolls);
    phase ^= 1u;
    if (__syncthreads_or(!ok)) {
      if (threadIdx.x == 0) atomicAdd(tc_timeouts, 1);
      abort = true;
      break;
    }
    tc::FenceAfterSync();
    // ---- epilogue: entries [24 half, 24 half + 24) of row r
    double* vals = svals + r * E;
    const int shift = e + 2 - 54;
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      const int col = 24 * half + 8 * q;
      float G[5][8];
#pragma unroll
      for (int l = 0; l < 5; ++l) tc::Ld8(tlane + l * NP + col, G[l]);
      tc::WaitLd();
      if (safe) {
#pragma unroll
        for (int t = 0; t < 8; ++t) {
          const int en = col + t;
          if (en < E) vals[en] = TcCombine(G[0][t], G[1][t], G[2][t], G[3][t], G[4][t], shift + sEc[en]);
        }
      }
    }
    if (half == 0 && r < ncell && !safe) {
      TcFallback(v, al, a, vals);
      atomicAdd(a.fallback, 1ull);
    }
    tc::CpAsyncWaitAll();
    tc::FenceBeforeSync();
    __syncthreads();
    // ---- write: one warp per cell, 32 consecutive triplets per store
    for (int cl = warp; cl < ncell; cl += 8) {
      lfg_triplet* base = a.out + soff[cl];
      const int* dd = sdofs + cl * N;
      const double* vv = svals + cl * E;
#pragma unroll
      for (int t = 0; t < 3; ++t)
        if (tmap[t] >= 0)
          StoreTriplet(base + lane + 32 * t, dd[tmap[t] & 0xff], dd[(tmap[t] >> 8) & 0xff], vv[tmap[t] >> 16]);
    }
    c = c_n;
    al = al_n;
#pragma unroll
    for (int i = 0; i < 4; ++i) v[i] = v_n[i];
    __syncthreads();
  }
  if (abort) tc::MbarWait(&mbar, phase ^ 1u, kTcMaxPolls);  // let an MMA still in flight finish
  tc::FenceBeforeSync();
  __syncthreads();
  if (threadIdx.x < 32) {
    tc::FenceAfterSync();
    tc::TmemFree(taddr, kTcCols);
  }
}

// Warp-specialised variant, one CTA (16 warps) per SM, persistent.  Two
// producer groups of four warps (one thread per cell, all nine points)
// alternate tiles: tile j of the CTA goes to group j & 1, A-digit buffer
// j & 1 and tensor-memory accumulator block j & 1 (columns 256 (j & 1) ..
// + 255).  An eight-warp consumer group (two threads per cell) drains the
// accumulators of every tile in order into FP64 values and writes the
// triplets.  Hand-offs: mma_done[b] (tcgen05.commit: A buffer b is free and
// accumulator block b is ready), tmem_free[b] (the consumers have read
// accumulator block b).  The row exponent and df32-range flag of each cell
// travel through the accumulator block too (column 240: A digit 1 at K column
// KP-1 times a unit table column).  Every wait gives up after 2^22 polls; a
// group leaves its loop on the same iteration in all its threads.
constexpr int kWsThreads = 512;
__host__ __device__ constexpr int WsSmemBytes(int m) {
  return 2 * 6 * 256 * TcKP(m) + TcImageBytes(m) + 128 * 45 * 8 + 2 * (128 * 9 * 4 + 128 * 8);
}

template <int M>
__global__ void __launch_bounds__(kWsThreads, 1)
    RDQuadTcWsKernel(AsmArgs a, DfArgs d, const uint4* __restrict__ image, int* __restrict__ tc_timeouts) {
  using elem::f2;
  constexpr int N = 9, E = 45, NQ = M * M, KP = TcKP(M), KS = KP / 16, NP = kTcNP;
  constexpr int P0 = (NQ + 1) / 2;   // points in K columns [0, KP/2); the rest from KP/2
  constexpr uint32_t SA = 256 * KP;  // one digit slice of an A tile, bytes
  constexpr uint32_t SBO = KP * 16;  // 8-row group stride of both operands
  constexpr int ABUF = 6 * SA;
  extern __shared__ __align__(1024) unsigned char smraw[];
  unsigned char* sA = smraw;                          // [2][6][128 x KP]
  unsigned char* sB = smraw + 2 * ABUF;               // table digits, info block, Ec
  const int* sEc = reinterpret_cast<const int*>(sB + TcEcOffset(M));
  double* svals = reinterpret_cast<double*>(sB + TcImageBytes(M));      // [128][45]
  int* sdofs = reinterpret_cast<int*>(svals + 128 * E);                 // [2][128][9]
  int64_t* soff = reinterpret_cast<int64_t*>(sdofs + 2 * 128 * N);      // [2][128]
  __shared__ f2 sWt[NQ + M];
  __shared__ __align__(8) uint64_t mma_done[2];
  __shared__ __align__(8) uint64_t tmem_free[2];
  __shared__ uint32_t s_taddr;
  __shared__ int s_abort;

  {
    const f2* g = reinterpret_cast<const f2*>(d.tab);
    for (int i = threadIdx.x; i < NQ; i += blockDim.x) sWt[i] = g[d.L.off_W + i];
    for (int i = threadIdx.x; i < M; i += blockDim.x) sWt[NQ + i] = g[d.L.off_t + i];
    uint4* dst = reinterpret_cast<uint4*>(sB);
    for (int i = threadIdx.x; i < TcImageBytes(M) / 16; i += blockDim.x) dst[i] = image[i];
  }
  if (threadIdx.x == 0) {
    tc::MbarInit(&mma_done[0], 1);
    tc::MbarInit(&mma_done[1], 1);
    tc::MbarInit(&tmem_free[0], 256);
    tc::MbarInit(&tmem_free[1], 256);
    s_abort = 0;
  }
  if (threadIdx.x < 32) tc::TmemAlloc(&s_taddr, 512);
  tc::FenceProxyAsync();
  tc::FenceBeforeSync();
  __syncthreads();
  tc::FenceAfterSync();
  const uint32_t taddr = s_taddr;
  const int64_t tiles = (a.count + 127) / 128;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  if (threadIdx.x < 256) {
    // ================= producers: group b, one thread per cell =================
    const int b = threadIdx.x >> 7, r = threadIdx.x & 127;
    const int bar = 1 + b;
    unsigned char* Ab = sA + b * ABUF;
    const uint32_t dcol = taddr + 256 * b;
    int c = 0;
    double2 v[4] = {};
    double al = 0.0;
    const int64_t first = blockIdx.x + static_cast<int64_t>(b) * gridDim.x;
    if (first < tiles) TcFetch(a, first * 128, r, c, v, al);
    int m = 0;
    for (;; ++m) {
      const int64_t tile = blockIdx.x + static_cast<int64_t>(b + 2 * m) * gridDim.x;
      if (tile >= tiles) break;
      const int64_t t0 = tile * 128;
      const int ncell = static_cast<int>(a.count - t0 < 128 ? a.count - t0 : 128);
      const bool ok = m == 0 || tc::MbarWait(&mma_done[b], (m - 1) & 1, kTcMaxPolls);  // A buffer b free
      if (tc::NamedSyncOr(bar, 128, !ok || *reinterpret_cast<volatile int*>(&s_abort) != 0)) {
        if (r == 0 && !ok) atomicAdd(tc_timeouts, 1);
        s_abort = 1;
        break;
      }
      bool safe = false;
      f2 cpt[NQ][4];
#pragma unroll
      for (int k = 0; k < NQ; ++k)
#pragma unroll
        for (int q = 0; q < 3; ++q) cpt[k][q] = f2{0.0f, 0.0f};
      if (r < ncell) {
        const double acd[6] = {v[1].x - v[0].x, v[1].y - v[0].y, v[3].x - v[0].x, v[3].y - v[0].y,
                               (v[0].x - v[1].x) + (v[2].x - v[3].x), (v[0].y - v[1].y) + (v[2].y - v[3].y)};
        safe = DfSafeBits(al);
#pragma unroll
        for (int k = 0; k < 6; ++k) safe = safe && DfSafeBits(acd[k]);
        if (safe) elem::QuadPointCoeffsDF<M, false>(acd, al, 0.0, sWt + NQ, sWt, cpt);
      }
      float mx = 0.0f;
#pragma unroll
      for (int k = 0; k < NQ; ++k)
#pragma unroll
        for (int q = 0; q < 3; ++q) mx = fmaxf(mx, fabsf(cpt[k][q].h));
      int e = mx > 0.0f ? static_cast<int>((__float_as_uint(mx) >> 23) & 0xffu) - 127 : 0;
      if (e < -70 || e > 70) safe = false;
      if (!safe) {
#pragma unroll
        for (int k = 0; k < NQ; ++k)
#pragma unroll
          for (int q = 0; q < 3; ++q) cpt[k][q] = f2{0.0f, 0.0f};
        e = 0;
      }
      const float scale = __uint_as_float(static_cast<uint32_t>(127 + 52 - e) << 23);  // 2^(52 - e)
      unsigned char* arow = Ab + (r >> 3) * SBO + (r & 7) * 16;
#pragma unroll
      for (int gk = 0; gk < KP / 8; ++gk) {
        uint32_t w[6][4];
#pragma unroll
        for (int pr = 0; pr < 4; ++pr) {
          uint32_t p[2][6];
#pragma unroll
          for (int s = 0; s < 2; ++s) {
            // K column -> (point, entry) in the TcKappa order of the table image
            const int kap = gk * 8 + 2 * pr + s, kl = kap < KP / 2 ? kap : kap - KP / 2;
            const int k = (kap < KP / 2 ? 0 : P0) + kl / 3;
            const bool used = kap < KP / 2 ? kl < 3 * P0 : kl < 3 * (NQ - P0);
            const f2 x = used ? cpt[k][kl % 3] : f2{0.0f, 0.0f};
            const float hs = x.h * scale;
            const int vhi = __float2int_rn(hs * 7.450580596923828125e-9f);  // 2^-27
            const float rem = __fmaf_rn(static_cast<float>(vhi), -134217728.0f, hs);  // exact
            const int wlo0 = __float2int_rn(rem) + __float2int_rn(x.l * scale) + 256 * ((1 << 18) + (1 << 9) + 1);
            const int whi = vhi + 256 * ((1 << 9) + 1) + (wlo0 >> 27);
            const uint32_t wlo = static_cast<uint32_t>(wlo0) & ((1u << 27) - 1u);
            p[s][0] = 0x6600u + static_cast<uint32_t>(whi >> 18);
            p[s][1] = 0x6400u | ((static_cast<uint32_t>(whi) >> 9) & 511u);
            p[s][2] = 0x6400u | (static_cast<uint32_t>(whi) & 511u);
            p[s][3] = 0x6400u | ((wlo >> 18) & 511u);
            p[s][4] = 0x6400u | ((wlo >> 9) & 511u);
            p[s][5] = 0x6400u | (wlo & 511u);
          }
#pragma unroll
          for (int i = 0; i < 6; ++i)
            w[i][pr] = HSub2(__byte_perm(p[0][i], p[1][i], 0x5410), i == 0 ? 0x66006600u : 0x65006500u);
        }
        if (gk == KP / 8 - 1) {  // row info in digit 1, K column KP - 1: e + 128, or 0 off the df32 range
          const uint32_t info = __half_as_ushort(__float2half_rn(safe ? static_cast<float>(e + 128) : 0.0f));
          w[0][3] = (w[0][3] & 0xffffu) | (info << 16);
        }
#pragma unroll
        for (int i = 0; i < 6; ++i)
          *reinterpret_cast<uint4*>(arow + i * SA + gk * 128) = make_uint4(w[i][0], w[i][1], w[i][2], w[i][3]);
      }
      tc::FenceProxyAsync();
      tc::NamedSync(bar, 128);
      if (r == 0) {
        bool free_ok = m == 0 || tc::MbarWait(&tmem_free[b], (m - 1) & 1, kTcMaxPolls);
        if (!free_ok) {
          atomicAdd(tc_timeouts, 1);
          s_abort = 1;
        } else {
          tc::FenceAfterSync();
          const uint32_t a0 = tc::SmemAddr(Ab), bu = tc::SmemAddr(sB), bs = bu + TcBHalfBytes(M);
          const uint32_t bi = bu + 2 * TcBHalfBytes(M);
#pragma unroll
          for (int s = 0; s < KS; ++s)
#pragma unroll
            for (int i = 1; i <= 5; ++i)
              tc::MmaF16(dcol + (i - 1) * NP, tc::SmemDesc(a0 + (i - 1) * SA + s * 256, 128, SBO),
                         tc::SmemDesc(bu + s * 256, 128, SBO), tc::IdescF16(128, (6 - i) * NP), s > 0 || i > 1);
#pragma unroll
          for (int s = 0; s < KS; ++s)
#pragma unroll
            for (int i = 1; i <= 6; ++i)
              tc::MmaF16(dcol + 4 * NP, tc::SmemDesc(a0 + (i - 1) * SA + s * 256, 128, SBO),
                         tc::SmemDesc(bs + (6 - i) * (NP / 8) * SBO + s * 256, 128, SBO), tc::IdescF16(128, NP),
                         true);
          tc::MmaF16(dcol + 5 * NP, tc::SmemDesc(a0 + (KS - 1) * 256, 128, SBO),
                     tc::SmemDesc(bi + (KS - 1) * 256, 128, SBO), tc::IdescF16(128, 16), false);
          tc::Commit(&mma_done[b]);
        }
      }
      // inputs of this group's next tile load while the tensor cores work
      const int64_t nxt = tile + 2 * static_cast<int64_t>(gridDim.x);
      if (nxt < tiles) TcFetch(a, nxt * 128, r, c, v, al);
    }
    // the group's last MMAs finish before the tensor memory is released
    if (r == 0 && m > 0) tc::MbarWait(&mma_done[b], (m - 1) & 1, kTcMaxPolls);
  } else {
    // ================= consumers: two threads per cell =================
    // The cells of TMEM lane quarter q (32 cells) belong to consumer warps q
    // (half 0) and q + 4 (half 1); each quarter reads, recombines, stages and
    // writes its own cells and synchronises on its own named barrier, so the
    // quarters drift apart and one quarter's triplet writes overlap another's
    // recombination.
    const int et = threadIdx.x - 256, half = et >> 7, r = et & 127, q4 = r >> 5, qbar = 4 + q4;
    const uint32_t tl = static_cast<uint32_t>(q4 * 32) << 16;
    int tmap[3];
#pragma unroll
    for (int t = 0; t < 3; ++t) {
      const int w = lane + 32 * t, i = w / N, j = w - i * N;
      tmap[t] = w < N * N ? (i | (j << 8) | (UpperIndex<N>(i, j) << 16)) : -1;
    }
    // dof indices of tile 0 (half 1 stages them; tile j uses buffer j & 1)
    if (half == 1 && blockIdx.x < tiles && static_cast<int64_t>(blockIdx.x) * 128 + r < a.count) {
      const int c0 = a.bucket[static_cast<int64_t>(blockIdx.x) * 128 + r];
      const int32_t* g = a.cell_dofs + static_cast<int64_t>(c0) * a.n_cell;
#pragma unroll
      for (int i = 0; i < N; ++i) tc::CpAsync4(sdofs + r * N + i, g + i);
      tc::CpAsync8(soff + r, a.tri_offset + c0);
    }
    tc::CpAsyncCommit();
    for (int j = 0;; ++j) {
      const int64_t tile = blockIdx.x + static_cast<int64_t>(j) * gridDim.x;
      if (tile >= tiles) break;
      const int64_t t0 = tile * 128;
      const int ncell = static_cast<int>(a.count - t0 < 128 ? a.count - t0 : 128);
      const int b = j & 1;
      const int64_t t1 = t0 + static_cast<int64_t>(gridDim.x) * 128;  // next tile
      int c_next = -1;
      if (half == 1 && t1 + r < a.count) c_next = a.bucket[t1 + r];
      const bool ok = tc::MbarWait(&mma_done[b], (j >> 1) & 1, kTcMaxPolls);
      if (tc::NamedSyncOr(qbar, 64, !ok || *reinterpret_cast<volatile int*>(&s_abort) != 0)) {
        if ((et & 127) == 32 * q4 && half == 0 && !ok) atomicAdd(tc_timeouts, 1);
        s_abort = 1;
        break;
      }
      tc::FenceAfterSync();
      const uint32_t acc = taddr + 256 * b + tl;
      float inf[8];
      tc::Ld8(acc + 5 * NP, inf);
      tc::WaitLd();
      const int info = static_cast<int>(inf[0]);
      const bool safe = info != 0;
      const int shift = info - 128 + 2 - 54;
      double* vals = svals + r * E;
#pragma unroll
      for (int q = 0; q < 3; ++q) {
        const int col = 24 * half + 8 * q;
        float G[5][8];
#pragma unroll
        for (int l = 0; l < 5; ++l) tc::Ld8(acc + l * NP + col, G[l]);
        tc::WaitLd();
        if (safe) {
#pragma unroll
          for (int t = 0; t < 8; ++t) {
            const int en = col + t;
            if (en < E) vals[en] = TcCombine(G[0][t], G[1][t], G[2][t], G[3][t], G[4][t], shift + sEc[en]);
          }
        }
      }
      tc::FenceBeforeSync();
      tc::MbarArrive(&tmem_free[b]);
      if (half == 0 && r < ncell && !safe) {
        int cf = 0;
        double2 vf[4] = {};
        double alf = 0.0;
        TcFetch(a, t0, r, cf, vf, alf);
        TcFallback(vf, alf, a, vals);
        atomicAdd(a.fallback, 1ull);
      }
      // stage the next tile's dof indices (its buffer was read by tile j - 1)
      if (c_next >= 0) {
        const int32_t* g = a.cell_dofs + static_cast<int64_t>(c_next) * a.n_cell;
        int* dn = sdofs + ((j + 1) & 1) * 128 * N + r * N;
#pragma unroll
        for (int i = 0; i < N; ++i) tc::CpAsync4(dn + i, g + i);
        tc::CpAsync8(soff + ((j + 1) & 1) * 128 + r, a.tri_offset + c_next);
      }
      tc::CpAsyncCommit();
      asm volatile("cp.async.wait_group 1;" ::: "memory");  // this tile's group has landed
      tc::NamedSync(qbar, 64);
      const int* sd = sdofs + b * 128 * N;
      const int64_t* so = soff + b * 128;
      for (int cl = 32 * q4 + half; cl < ncell && cl < 32 * q4 + 32; cl += 2) {
        lfg_triplet* base = a.out + so[cl];
        const int* dd = sd + cl * N;
        const double* vv = svals + cl * E;
#pragma unroll
        for (int t = 0; t < 3; ++t)
          if (tmap[t] >= 0)
            StoreTriplet(base + lane + 32 * t, dd[tmap[t] & 0xff], dd[(tmap[t] >> 8) & 0xff], vv[tmap[t] >> 16]);
      }
      tc::NamedSync(qbar, 64);
    }
    tc::CpAsyncWaitAll();
  }
  tc::FenceBeforeSync();
  __syncthreads();
  if (warp == 0) {
    tc::FenceAfterSync();
    tc::TmemFree(taddr, 512);
  }
}

// Warp-specialised variant with the triplet writes moved to the producers.
// The consumers (eight warps, two threads per cell) only recombine: they
// write the FP64 entries of tile j into the A-digit buffer of tile j's
// producer group -- free once tile j's MMAs have completed, and as large as
// the 128 x 45 values for M = 3 -- and arrive on vals_ready[b].  The
// producer group then writes tile j's triplets from there (it has slack:
// it waits for a free accumulator block otherwise) before it splits the
// digits of its next tile into the same buffer.  So the staged values are
// double-buffered (one buffer per group) without extra shared memory, and a
// tile's recombination overlaps the previous tile's writes.  Hand-offs per
// group b: mma_done[b] (tile's MMAs complete), tmem_free[b] and vals_ready[b]
// (the consumers have read accumulator block b and written the values).
// Every wait gives up after 2^22 polls.
__host__ __device__ constexpr int Ws2BufBytes(int m) {
  return 6 * 256 * TcKP(m) > 128 * 45 * 8 ? 6 * 256 * TcKP(m) : 128 * 45 * 8;
}
__host__ __device__ constexpr int Ws2SmemBytes(int m) {
  return 2 * Ws2BufBytes(m) + TcImageBytes(m) + 2 * (128 * 9 * 4 + 128 * 8);
}

template <int M>
__global__ void __launch_bounds__(kWsThreads, 1)
    RDQuadTcWs2Kernel(AsmArgs a, DfArgs d, const uint4* __restrict__ image, int* __restrict__ tc_timeouts) {
  using elem::f2;
  constexpr int N = 9, E = 45, NQ = M * M, KP = TcKP(M), KS = KP / 16, NP = kTcNP;
  constexpr int P0 = (NQ + 1) / 2;   // points in K columns [0, KP/2); the rest from KP/2
  constexpr uint32_t SA = 256 * KP;  // one digit slice of an A tile, bytes
  constexpr uint32_t SBO = KP * 16;  // 8-row group stride of both operands
  constexpr int ABUF = Ws2BufBytes(M);
  extern __shared__ __align__(1024) unsigned char smraw[];
  unsigned char* sA = smraw;                                          // [2][ABUF]: digits, then values
  unsigned char* sB = smraw + 2 * ABUF;                               // table digits, info block, Ec
  const int* sEc = reinterpret_cast<const int*>(sB + TcEcOffset(M));
  int* sdofs = reinterpret_cast<int*>(sB + TcImageBytes(M));          // [2][128][9]
  int64_t* soff = reinterpret_cast<int64_t*>(sdofs + 2 * 128 * N);    // [2][128]
  __shared__ f2 sWt[NQ + M];
  __shared__ __align__(8) uint64_t mma_done[2];
  __shared__ __align__(8) uint64_t tmem_free[2];
  __shared__ __align__(8) uint64_t vals_ready[2];
  __shared__ uint32_t s_taddr;
  __shared__ int s_abort;

  {
    const f2* g = reinterpret_cast<const f2*>(d.tab);
    for (int i = threadIdx.x; i < NQ; i += blockDim.x) sWt[i] = g[d.L.off_W + i];
    for (int i = threadIdx.x; i < M; i += blockDim.x) sWt[NQ + i] = g[d.L.off_t + i];
    uint4* dst = reinterpret_cast<uint4*>(sB);
    for (int i = threadIdx.x; i < TcImageBytes(M) / 16; i += blockDim.x) dst[i] = image[i];
  }
  if (threadIdx.x == 0) {
    for (int b = 0; b < 2; ++b) {
      tc::MbarInit(&mma_done[b], 1);
      tc::MbarInit(&tmem_free[b], 256);
      tc::MbarInit(&vals_ready[b], 256);
    }
    s_abort = 0;
  }
  if (threadIdx.x < 32) tc::TmemAlloc(&s_taddr, 512);
  tc::FenceProxyAsync();
  tc::FenceBeforeSync();
  __syncthreads();
  tc::FenceAfterSync();
  const uint32_t taddr = s_taddr;
  const int64_t tiles = (a.count + 127) / 128;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int tmap[3];
#pragma unroll
  for (int t = 0; t < 3; ++t) {
    const int w = lane + 32 * t, i = w / N, j = w - i * N;
    tmap[t] = w < N * N ? (i | (j << 8) | (UpperIndex<N>(i, j) << 16)) : -1;
  }

  if (threadIdx.x < 256) {
    // ================= producers: group b, one thread per cell =================
    const int b = threadIdx.x >> 7, r = threadIdx.x & 127, wg = (threadIdx.x >> 5) & 3;
    const int bar = 1 + b;
    unsigned char* Ab = sA + b * ABUF;
    const double* vals_b = reinterpret_cast<const double*>(Ab);
    int* sd_b = sdofs + b * 128 * N;
    int64_t* so_b = soff + b * 128;
    const uint32_t dcol = taddr + 256 * b;
    int c = 0;
    double2 v[4] = {};
    double al = 0.0;
    const int64_t first = blockIdx.x + static_cast<int64_t>(b) * gridDim.x;
    if (first < tiles) TcFetch(a, first * 128, r, c, v, al);
    int m = 0, issued = 0;
    int prev_ncell = 0;
    // writes the previous tile of this group (its values are in Ab once the
    // consumers arrive on vals_ready[b]); false when a wait gave up
    auto write_prev = [&](int mp) -> bool {
      const bool ok = tc::MbarWait(&vals_ready[b], mp & 1, kTcMaxPolls);
      asm volatile("cp.async.wait_all;" ::: "memory");  // this group's staged dofs / offsets
      if (tc::NamedSyncOr(bar, 128, !ok || *reinterpret_cast<volatile int*>(&s_abort) != 0)) {
        if (r == 0 && !ok) atomicAdd(tc_timeouts, 1);
        s_abort = 1;
        return false;
      }
      for (int cl = 32 * wg; cl < prev_ncell && cl < 32 * wg + 32; ++cl) {
        lfg_triplet* base = a.out + so_b[cl];
        const int* dd = sd_b + cl * N;
        const double* vv = vals_b + cl * E;
#pragma unroll
        for (int t = 0; t < 3; ++t)
          if (tmap[t] >= 0)
            StoreTriplet(base + lane + 32 * t, dd[tmap[t] & 0xff], dd[(tmap[t] >> 8) & 0xff], vv[tmap[t] >> 16]);
      }
      tc::NamedSync(bar, 128);  // Ab and the staged dofs are free again
      return true;
    };
    bool alive = true;
    for (;; ++m) {
      const int64_t tile = blockIdx.x + static_cast<int64_t>(b + 2 * m) * gridDim.x;
      if (tile >= tiles) break;
      const int64_t t0 = tile * 128;
      const int ncell = static_cast<int>(a.count - t0 < 128 ? a.count - t0 : 128);
      if (m > 0 && !write_prev(m - 1)) {
        alive = false;
        break;
      }
      // this tile's dof rows and triplet offsets, staged for its writes
      if (r < ncell) {
        const int32_t* g = a.cell_dofs + static_cast<int64_t>(c) * a.n_cell;
#pragma unroll
        for (int i = 0; i < N; ++i) tc::CpAsync4(sd_b + r * N + i, g + i);
        tc::CpAsync8(so_b + r, a.tri_offset + c);
      }
      tc::CpAsyncCommit();
      bool safe = false;
      f2 cpt[NQ][4];
#pragma unroll
      for (int k = 0; k < NQ; ++k)
#pragma unroll
        for (int q = 0; q < 3; ++q) cpt[k][q] = f2{0.0f, 0.0f};
      if (r < ncell) {
        const double acd[6] = {v[1].x - v[0].x, v[1].y - v[0].y, v[3].x - v[0].x, v[3].y - v[0].y,
                               (v[0].x - v[1].x) + (v[2].x - v[3].x), (v[0].y - v[1].y) + (v[2].y - v[3].y)};
        safe = DfSafeBits(al);
#pragma unroll
        for (int k = 0; k < 6; ++k) safe = safe && DfSafeBits(acd[k]);
        if (safe) elem::QuadPointCoeffsDF<M, false>(acd, al, 0.0, sWt + NQ, sWt, cpt);
      }
      float mx = 0.0f;
#pragma unroll
      for (int k = 0; k < NQ; ++k)
#pragma unroll
        for (int q = 0; q < 3; ++q) mx = fmaxf(mx, fabsf(cpt[k][q].h));
      int e = mx > 0.0f ? static_cast<int>((__float_as_uint(mx) >> 23) & 0xffu) - 127 : 0;
      if (e < -70 || e > 70) safe = false;
      if (!safe) {
#pragma unroll
        for (int k = 0; k < NQ; ++k)
#pragma unroll
          for (int q = 0; q < 3; ++q) cpt[k][q] = f2{0.0f, 0.0f};
        e = 0;
      }
      const float scale = __uint_as_float(static_cast<uint32_t>(127 + 52 - e) << 23);  // 2^(52 - e)
      unsigned char* arow = Ab + (r >> 3) * SBO + (r & 7) * 16;
#pragma unroll
      for (int gk = 0; gk < KP / 8; ++gk) {
        uint32_t w[6][4];
#pragma unroll
        for (int pr = 0; pr < 4; ++pr) {
          uint32_t p[2][6];
#pragma unroll
          for (int s = 0; s < 2; ++s) {
            const int kap = gk * 8 + 2 * pr + s, kl = kap < KP / 2 ? kap : kap - KP / 2;
            const int k = (kap < KP / 2 ? 0 : P0) + kl / 3;
            const bool used = kap < KP / 2 ? kl < 3 * P0 : kl < 3 * (NQ - P0);
            const f2 x = used ? cpt[k][kl % 3] : f2{0.0f, 0.0f};
            const float hs = x.h * scale;
            const int vhi = __float2int_rn(hs * 7.450580596923828125e-9f);  // 2^-27
            const float rem = __fmaf_rn(static_cast<float>(vhi), -134217728.0f, hs);  // exact
            const int wlo0 = __float2int_rn(rem) + __float2int_rn(x.l * scale) + 256 * ((1 << 18) + (1 << 9) + 1);
            const int whi = vhi + 256 * ((1 << 9) + 1) + (wlo0 >> 27);
            const uint32_t wlo = static_cast<uint32_t>(wlo0) & ((1u << 27) - 1u);
            p[s][0] = 0x6600u + static_cast<uint32_t>(whi >> 18);
            p[s][1] = 0x6400u | ((static_cast<uint32_t>(whi) >> 9) & 511u);
            p[s][2] = 0x6400u | (static_cast<uint32_t>(whi) & 511u);
            p[s][3] = 0x6400u | ((wlo >> 18) & 511u);
            p[s][4] = 0x6400u | ((wlo >> 9) & 511u);
            p[s][5] = 0x6400u | (wlo & 511u);
          }
#pragma unroll
          for (int i = 0; i < 6; ++i)
            w[i][pr] = HSub2(__byte_perm(p[0][i], p[1][i], 0x5410), i == 0 ? 0x66006600u : 0x65006500u);
        }
        if (gk == KP / 8 - 1) {  // row info in digit 1, K column KP - 1: e + 128, or 0 off the df32 range
          const uint32_t info = __half_as_ushort(__float2half_rn(safe ? static_cast<float>(e + 128) : 0.0f));
          w[0][3] = (w[0][3] & 0xffffu) | (info << 16);
        }
#pragma unroll
        for (int i = 0; i < 6; ++i)
          *reinterpret_cast<uint4*>(arow + i * SA + gk * 128) = make_uint4(w[i][0], w[i][1], w[i][2], w[i][3]);
      }
      tc::FenceProxyAsync();
      tc::NamedSync(bar, 128);
      if (r == 0) {
        bool free_ok = m == 0 || tc::MbarWait(&tmem_free[b], (m - 1) & 1, kTcMaxPolls);
        if (!free_ok) {
          atomicAdd(tc_timeouts, 1);
          s_abort = 1;
        } else {
          tc::FenceAfterSync();
          const uint32_t a0 = tc::SmemAddr(Ab), bu = tc::SmemAddr(sB), bs = bu + TcBHalfBytes(M);
          const uint32_t bi = bu + 2 * TcBHalfBytes(M);
#pragma unroll
          for (int s = 0; s < KS; ++s)
#pragma unroll
            for (int i = 1; i <= 5; ++i)
              tc::MmaF16(dcol + (i - 1) * NP, tc::SmemDesc(a0 + (i - 1) * SA + s * 256, 128, SBO),
                         tc::SmemDesc(bu + s * 256, 128, SBO), tc::IdescF16(128, (6 - i) * NP), s > 0 || i > 1);
#pragma unroll
          for (int s = 0; s < KS; ++s)
#pragma unroll
            for (int i = 1; i <= 6; ++i)
              tc::MmaF16(dcol + 4 * NP, tc::SmemDesc(a0 + (i - 1) * SA + s * 256, 128, SBO),
                         tc::SmemDesc(bs + (6 - i) * (NP / 8) * SBO + s * 256, 128, SBO), tc::IdescF16(128, NP),
                         true);
          tc::MmaF16(dcol + 5 * NP, tc::SmemDesc(a0 + (KS - 1) * 256, 128, SBO),
                     tc::SmemDesc(bi + (KS - 1) * 256, 128, SBO), tc::IdescF16(128, 16), false);
          tc::Commit(&mma_done[b]);
        }
      }
      ++issued;
      prev_ncell = ncell;
      // inputs of this group's next tile load while the tensor cores work
      const int64_t nxt = tile + 2 * static_cast<int64_t>(gridDim.x);
      if (nxt < tiles) TcFetch(a, nxt * 128, r, c, v, al);
    }
    // the group's last tile
    if (alive && m > 0) write_prev(m - 1);
    // after an abort an MMA may still be in flight: it finishes before the
    // tensor memory is released (a completed phase returns at once)
    if (r == 0 && issued > 0) tc::MbarWait(&mma_done[b], (issued - 1) & 1, kTcMaxPolls);
  } else {
    // ================= consumers: two threads per cell, recombination only =================
    const int et = threadIdx.x - 256, half = et >> 7, r = et & 127, q4 = r >> 5;
    const uint32_t tl = static_cast<uint32_t>(q4 * 32) << 16;
    for (int j = 0;; ++j) {
      const int64_t tile = blockIdx.x + static_cast<int64_t>(j) * gridDim.x;
      if (tile >= tiles) break;
      const int64_t t0 = tile * 128;
      const int ncell = static_cast<int>(a.count - t0 < 128 ? a.count - t0 : 128);
      const int b = j & 1;
      const bool ok = tc::MbarWait(&mma_done[b], (j >> 1) & 1, kTcMaxPolls);
      if (!ok || *reinterpret_cast<volatile int*>(&s_abort) != 0) {
        if (!ok && et == 0) atomicAdd(tc_timeouts, 1);
        s_abort = 1;
        break;
      }
      tc::FenceAfterSync();
      const uint32_t acc = taddr + 256 * b + tl;
      float inf[8];
      tc::Ld8(acc + 5 * NP, inf);
      tc::WaitLd();
      const int info = static_cast<int>(inf[0]);
      const bool safe = info != 0;
      const int shift = info - 128 + 2 - 54;
      double* vals = reinterpret_cast<double*>(sA + b * ABUF) + r * E;
#pragma unroll
      for (int q = 0; q < 3; ++q) {
        const int col = 24 * half + 8 * q;
        float G[5][8];
#pragma unroll
        for (int l = 0; l < 5; ++l) tc::Ld8(acc + l * NP + col, G[l]);
        tc::WaitLd();
        if (safe) {
#pragma unroll
          for (int t = 0; t < 8; ++t) {
            const int en = col + t;
            if (en < E) vals[en] = TcCombine(G[0][t], G[1][t], G[2][t], G[3][t], G[4][t], shift + sEc[en]);
          }
        }
      }
      tc::FenceBeforeSync();
      tc::MbarArrive(&tmem_free[b]);
      if (half == 0 && r < ncell && !safe) {
        int cf = 0;
        double2 vf[4] = {};
        double alf = 0.0;
        TcFetch(a, t0, r, cf, vf, alf);
        TcFallback(vf, alf, a, vals);
        atomicAdd(a.fallback, 1ull);
      }
      tc::MbarArrive(&vals_ready[b]);
    }
  }
  tc::FenceBeforeSync();
  __syncthreads();
  if (warp == 0) {
    tc::FenceAfterSync();
    tc::TmemFree(taddr, 512);
  }
}

// ------------------------- O3 triangles, point-varying alpha, tensor cores
// Affine triangles, FeSpaceLagrangeO3, the 12-point degree-6 rule, alpha
// varying over the cell (analytic families / O1 nodal), gamma cell-constant:
//     A_K(e) = sum_k w_k alpha(x_k) [M00 T0 + M01 T1 + M11 T2](k; e) + gamma |det J| R_mass(e)
// with M = |det J| J^-1 J^-T.  The 36 point coefficients c(k, ab) = w_k
// alpha_k M_ab and m = gamma |det J| form a row of K = 37 columns (48 with
// padding); the table rows are T(k; e, ab) and the folded mass table.  The
// exact digit splitting, levels and recombination are those of
// RDQuadTcKernel; here 55 entries (64 accumulator columns per level, 320 in
// all, plus the row-info column 320) fill one CTA's 512 tensor-memory
// columns, so one tile is in flight per SM: 16 warps, 8 producer warps (two
// threads per cell: points 0-5 -> K columns 0-17; points 6-11 and the mass
// -> columns 24-42) and 8 consumer warps, hand-offs as in RDQuadTcWsKernel
// with single A and accumulator buffers.
constexpr int kTtN = 10, kTtE = 55, kTtNQ = 12, kTtNP = 64, kTtKP = 48;
constexpr int kTtSA = 128 * kTtKP * 2;                    // one digit slice of A
constexpr int kTtBHalf = 6 * kTtNP * kTtKP * 2;           // plain (or scaled) table digits
constexpr int kTtInfo = 16 * kTtKP * 2;
constexpr int kTtEcOff = 2 * kTtBHalf + kTtInfo;
constexpr int kTtImage = kTtEcOff + kTtNP * 4;
constexpr int kTtSmem = 6 * kTtSA + kTtImage + 128 * kTtE * 8 + 2 * (128 * kTtN * 4 + 128 * 8);

__host__ __device__ constexpr int TtKappa(int k, int ab) { return k < 6 ? 3 * k + ab : 24 + 3 * (k - 6) + ab; }

// FAM: 0 alpha O1-nodal, 1 polynomial, 2 sin sin / sin cos (evaluated as
// sin/cos at the first vertex, once per cell, turned to the points by the
// angle-addition formulas with short series of the small offsets when
// pi |p| (|J_0| + |J_1|) <= 0.1, else the full reduction per point).
template <int FAM>
__global__ void __launch_bounds__(512, 1) RDTriaTcKernel(AsmArgs a, DfArgs d, const uint4* __restrict__ image,
                                                         int* __restrict__ tc_timeouts) {
  using elem::f2;
  namespace df = lfg::df;
  constexpr int N = kTtN, E = kTtE, NQ = kTtNQ, NP = kTtNP, KP = kTtKP, KS = KP / 16;
  constexpr uint32_t SA = kTtSA, SBO = KP * 16;
  extern __shared__ __align__(1024) unsigned char smraw[];
  unsigned char* sA = smraw;
  unsigned char* sB = smraw + 6 * SA;
  const int* sEc = reinterpret_cast<const int*>(sB + kTtEcOff);
  double* svals = reinterpret_cast<double*>(sB + kTtImage);
  int* sdofs = reinterpret_cast<int*>(svals + 128 * E);            // [2][128][10]
  int64_t* soff = reinterpret_cast<int64_t*>(sdofs + 2 * 128 * N);  // [2][128]
  __shared__ f2 sW[NQ], sX[2 * NQ], sO1[4 * NQ], sSC[23], sSm[11];
  __shared__ elem::AnalyticDF sAf;
  __shared__ uint32_t smax[2][128];
  __shared__ __align__(8) uint64_t mma_done, tmem_free;
  __shared__ uint32_t s_taddr;
  __shared__ int s_abort;
  {
    const f2* g = reinterpret_cast<const f2*>(d.tab);
    for (int i = threadIdx.x; i < NQ; i += blockDim.x) sW[i] = g[d.L.off_W + i];
    for (int i = threadIdx.x; i < 2 * NQ; i += blockDim.x) sX[i] = g[d.L.off_X + i];
    for (int i = threadIdx.x; i < 4 * NQ; i += blockDim.x) sO1[i] = g[d.L.off_O1 + i];
    for (int i = threadIdx.x; i < 23; i += blockDim.x) sSC[i] = g[d.L.off_SC + i];
    for (int i = threadIdx.x; i < 16; i += blockDim.x) sAf.p[i] = df::FromDouble(a.alpha.p[i]);
    if (threadIdx.x < 11) {  // small-angle series: 1/1!, -1/3!, .., 1/9!; 1/0!, -1/2!, .., -1/10!
      const int k = threadIdx.x < 5 ? 2 * threadIdx.x + 1 : 2 * (threadIdx.x - 5);
      double f = 1.0;
      for (int i = 2; i <= k; ++i) f *= i;
      const int sgn = (threadIdx.x < 5 ? threadIdx.x : threadIdx.x - 5) & 1;
      sSm[threadIdx.x] = df::FromDouble(sgn ? -1.0 / f : 1.0 / f);
    }
    if (threadIdx.x == 0) sAf.func = a.alpha.func;
    uint4* dst = reinterpret_cast<uint4*>(sB);
    for (int i = threadIdx.x; i < kTtImage / 16; i += blockDim.x) dst[i] = image[i];
  }
  if (threadIdx.x == 0) {
    tc::MbarInit(&mma_done, 1);
    tc::MbarInit(&tmem_free, 256);
    s_abort = 0;
  }
  if (threadIdx.x < 32) tc::TmemAlloc(&s_taddr, 512);
  tc::FenceProxyAsync();
  tc::FenceBeforeSync();
  __syncthreads();
  tc::FenceAfterSync();
  const uint32_t taddr = s_taddr;
  const int64_t tiles = (a.count + 127) / 128;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const bool mass = a.gamma.kind != LFG_COEFF_ZERO;
  const bool sinsin = a.alpha.func == LFG_FN_SINSIN;

  if (threadIdx.x < 256) {
    // ================= producers: two threads per cell =================
    const int half = threadIdx.x >> 7, r = threadIdx.x & 127;
    int c = 0;
    double2 v[4] = {};
    double ga = 0.0;
    int4 cn = make_int4(0, 0, 0, 0);
    auto fetch = [&](int64_t t0) {
      if (t0 + r < a.count) {
        c = a.bucket[t0 + r];
        LoadVerts<false>(a, c, cn, v);
        ga = mass ? CellConst(a.gamma, c) : 0.0;
      }
    };
    if (blockIdx.x < tiles) fetch(static_cast<int64_t>(blockIdx.x) * 128);
    int j = 0;
    for (;; ++j) {
      const int64_t tile = blockIdx.x + static_cast<int64_t>(j) * gridDim.x;
      if (tile >= tiles) break;
      const int64_t t0 = tile * 128;
      const int ncell = static_cast<int>(a.count - t0 < 128 ? a.count - t0 : 128);
      // ---- coefficients of this thread's six points (+ the mass column in half 1)
      bool safe = false;
      f2 cpt[6][3];
      f2 mm = df::Make(0.0f);
#pragma unroll
      for (int k = 0; k < 6; ++k)
#pragma unroll
        for (int q = 0; q < 3; ++q) cpt[k][q] = f2{0.0f, 0.0f};
      if (r < ncell) {
        const double jac[4] = {v[1].x - v[0].x, v[2].x - v[0].x, v[1].y - v[0].y, v[2].y - v[0].y};
        safe = DfSafeBits(ga) && DfSafeBits(v[0].x) && DfSafeBits(v[0].y);
#pragma unroll
        for (int k = 0; k < 4; ++k) safe = safe && DfSafeBits(jac[k]);
        f2 nod[3] = {};
        if (safe && FAM == 0) {
          const double n0 = a.alpha.data[cn.x], n1 = a.alpha.data[cn.y], n2 = a.alpha.data[cn.z];
          safe = DfSafeBits(n0) && DfSafeBits(n1) && DfSafeBits(n2);
          nod[0] = df::FromDouble(n0);
          nod[1] = df::FromDouble(n1);
          nod[2] = df::FromDouble(n2);
        }
        if (safe) {
          const f2 j00 = df::FromDouble(jac[0]), j01 = df::FromDouble(jac[1]);
          const f2 j10 = df::FromDouble(jac[2]), j11 = df::FromDouble(jac[3]);
          f2 m00, m01, m11, adet;
          elem::TriaMetricDF(j00, j01, j10, j11, m00, m01, m11, adet);
          const f2 x0 = df::FromDouble(v[0].x), y0 = df::FromDouble(v[0].y);
          // trig families: sin/cos at the first vertex, once per cell
          f2 sA = {}, cA = {}, sB = {}, cB = {}, pi = {};
          bool small = false;
          if (FAM == 2) {
            const float bound = 3.1416f * fmaxf(fabsf(sAf.p[2].h) * (fabsf(j00.h) + fabsf(j01.h)),
                                                fabsf(sAf.p[3].h) * (fabsf(j10.h) + fabsf(j11.h)));
            small = bound <= 0.0999f;
            if (small) {
              elem::SinCosPiDF(df::Mul(sAf.p[2], x0), sSC, sSC + 11, sA, cA);
              elem::SinCosPiDF(df::Mul(sAf.p[3], y0), sSC, sSC + 11, sB, cB);
              pi = df::FromDouble(3.14159265358979323846);
            }
          }
#pragma unroll
          for (int kk = 0; kk < 6; ++kk) {
            const int k = 6 * half + kk;
            f2 al;
            if (FAM == 0) {
              al = df::Mul(nod[0], sO1[4 * k]);
              al = df::MulAdd(nod[1], sO1[4 * k + 1], al);
              al = df::MulAdd(nod[2], sO1[4 * k + 2], al);
            } else if (FAM == 2 && small) {
              const f2 xh = sX[2 * k], yh = sX[2 * k + 1];
              const f2 dx = df::MulAdd(j01, yh, df::Mul(j00, xh));  // X - x0
              const f2 dy = df::MulAdd(j11, yh, df::Mul(j10, xh));
              f2 s1, c1, s2, c2;
              elem::SinCosSmallDF(df::Mul(pi, df::Mul(sAf.p[2], dx)), sSm, sSm + 5, s1, c1);
              elem::SinCosSmallDF(df::Mul(pi, df::Mul(sAf.p[3], dy)), sSm, sSm + 5, s2, c2);
              const f2 sx = df::Add(df::Mul(sA, c1), df::Mul(cA, s1));  // sin(a + t)
              const f2 fy = sinsin ? df::Add(df::Mul(sB, c2), df::Mul(cB, s2))   // sin(b + u)
                                   : df::Sub(df::Mul(cB, c2), df::Mul(sB, s2));  // cos(b + u)
              al = df::MulAdd(sAf.p[1], df::Mul(sx, fy), sAf.p[0]);
            } else {
              const f2 xh = sX[2 * k], yh = sX[2 * k + 1];
              const f2 X = df::MulAdd(j01, yh, df::MulAdd(j00, xh, x0));
              const f2 Y = df::MulAdd(j11, yh, df::MulAdd(j10, xh, y0));
              al = elem::EvalAnalyticDF(sAf, X, Y, sSC, sSC + 11);
            }
            const float aa = fabsf(al.h);  // 2^-30 margin below the df32 range of the products
            safe = safe && (aa == 0.0f || (aa > 8.0e-10f && aa < 1.0e9f));
            const f2 s = df::Mul(sW[k], al);
            cpt[kk][0] = df::Mul(s, m00);
            cpt[kk][1] = df::Mul(s, m01);
            cpt[kk][2] = df::Mul(s, m11);
          }
          if (mass && half == 1) mm = df::Mul(df::FromDouble(ga), adet);
        }
      }
      float mx = fabsf(mm.h);
#pragma unroll
      for (int k = 0; k < 6; ++k)
#pragma unroll
        for (int q = 0; q < 3; ++q) mx = fmaxf(mx, fabsf(cpt[k][q].h));
      // both threads of the cell agree on the row maximum and on the range flag
      smax[half][r] = safe ? __float_as_uint(mx) : 0xffffffffu;
      tc::NamedSync(1, 256);
      const uint32_t m0 = smax[0][r], m1 = smax[1][r];
      safe = r < ncell && m0 != 0xffffffffu && m1 != 0xffffffffu;
      const uint32_t mb = safe ? max(m0, m1) : 0u;
      int e = mb ? static_cast<int>((mb >> 23) & 0xffu) - 127 : 0;
      if (e < -70 || e > 70) safe = false;
      if (!safe) {
#pragma unroll
        for (int k = 0; k < 6; ++k)
#pragma unroll
          for (int q = 0; q < 3; ++q) cpt[k][q] = f2{0.0f, 0.0f};
        mm = f2{0.0f, 0.0f};
        e = 0;
      }
      // ---- the A buffer is free once the previous tile's MMAs are done
      const bool ok = j == 0 || tc::MbarWait(&mma_done, (j - 1) & 1, kTcMaxPolls);
      if (tc::NamedSyncOr(1, 256, !ok || *reinterpret_cast<volatile int*>(&s_abort) != 0)) {
        if (threadIdx.x == 0 && !ok) atomicAdd(tc_timeouts, 1);
        s_abort = 1;
        break;
      }
      const float scale = __uint_as_float(static_cast<uint32_t>(127 + 52 - e) << 23);  // 2^(52 - e)
      unsigned char* arow = sA + (r >> 3) * SBO + (r & 7) * 16;
#pragma unroll
      for (int gk = 0; gk < 3; ++gk) {
        const int G = 3 * half + gk;
        uint32_t w[6][4];
#pragma unroll
        for (int pr = 0; pr < 4; ++pr) {
          uint32_t p[2][6];
#pragma unroll
          for (int s = 0; s < 2; ++s) {
            const int kl = gk * 8 + 2 * pr + s;  // column within this half: point kl / 3, mass at 18 (half 1)
            f2 x = f2{0.0f, 0.0f};
            if (kl < 18) x = cpt[kl / 3][kl % 3];
            else if (kl == 18 && half == 1) x = mm;
            const float hs = x.h * scale;
            const int vhi = __float2int_rn(hs * 7.450580596923828125e-9f);  // 2^-27
            const float rem = __fmaf_rn(static_cast<float>(vhi), -134217728.0f, hs);  // exact
            const int wlo0 = __float2int_rn(rem) + __float2int_rn(x.l * scale) + 256 * ((1 << 18) + (1 << 9) + 1);
            const int whi = vhi + 256 * ((1 << 9) + 1) + (wlo0 >> 27);
            const uint32_t wlo = static_cast<uint32_t>(wlo0) & ((1u << 27) - 1u);
            p[s][0] = 0x6600u + static_cast<uint32_t>(whi >> 18);
            p[s][1] = 0x6400u | ((static_cast<uint32_t>(whi) >> 9) & 511u);
            p[s][2] = 0x6400u | (static_cast<uint32_t>(whi) & 511u);
            p[s][3] = 0x6400u | ((wlo >> 18) & 511u);
            p[s][4] = 0x6400u | ((wlo >> 9) & 511u);
            p[s][5] = 0x6400u | (wlo & 511u);
          }
#pragma unroll
          for (int i = 0; i < 6; ++i)
            w[i][pr] = HSub2(__byte_perm(p[0][i], p[1][i], 0x5410), i == 0 ? 0x66006600u : 0x65006500u);
        }
        if (G == KP / 8 - 1) {  // row info in digit 1, K column KP - 1
          const uint32_t info = __half_as_ushort(__float2half_rn(safe ? static_cast<float>(e + 128) : 0.0f));
          w[0][3] = (w[0][3] & 0xffffu) | (info << 16);
        }
#pragma unroll
        for (int i = 0; i < 6; ++i)
          *reinterpret_cast<uint4*>(arow + i * SA + G * 128) = make_uint4(w[i][0], w[i][1], w[i][2], w[i][3]);
      }
      tc::FenceProxyAsync();
      tc::NamedSync(1, 256);
      if (threadIdx.x == 0) {
        const bool free_ok = j == 0 || tc::MbarWait(&tmem_free, (j - 1) & 1, kTcMaxPolls);
        if (!free_ok) {
          atomicAdd(tc_timeouts, 1);
          s_abort = 1;
        } else {
          tc::FenceAfterSync();
          const uint32_t a0 = tc::SmemAddr(sA), bu = tc::SmemAddr(sB), bs = bu + kTtBHalf, bi = bu + 2 * kTtBHalf;
#pragma unroll
          for (int s = 0; s < KS; ++s) {
            const uint64_t b0 = tc::SmemDesc(bu + s * 256, 128, SBO);
            // digit 1 against table digits 1..4 (levels 2..5) and digit 5 (level 6)
            tc::MmaF16(taddr, tc::SmemDesc(a0 + s * 256, 128, SBO), b0, tc::IdescF16(128, 256), s > 0);
            tc::MmaF16(taddr + 4 * NP, tc::SmemDesc(a0 + s * 256, 128, SBO),
                       tc::SmemDesc(bu + 4 * (NP / 8) * SBO + s * 256, 128, SBO), tc::IdescF16(128, NP), s > 0);
#pragma unroll
            for (int i = 2; i <= 5; ++i)  // digit i against table digits 1..6-i (levels i+1..6)
              tc::MmaF16(taddr + (i - 1) * NP, tc::SmemDesc(a0 + (i - 1) * SA + s * 256, 128, SBO), b0,
                         tc::IdescF16(128, (6 - i) * NP), true);
#pragma unroll
            for (int i = 1; i <= 6; ++i)  // level 7, 2^-9-scaled table digits
              tc::MmaF16(taddr + 4 * NP, tc::SmemDesc(a0 + (i - 1) * SA + s * 256, 128, SBO),
                         tc::SmemDesc(bs + (6 - i) * (NP / 8) * SBO + s * 256, 128, SBO), tc::IdescF16(128, NP),
                         true);
          }
          tc::MmaF16(taddr + 5 * NP, tc::SmemDesc(a0 + (KS - 1) * 256, 128, SBO),
                     tc::SmemDesc(bi + (KS - 1) * 256, 128, SBO), tc::IdescF16(128, 16), false);
          tc::Commit(&mma_done);
        }
      }
      const int64_t nxt = tile + gridDim.x;
      if (nxt < tiles) fetch(nxt * 128);
    }
    if (threadIdx.x == 0 && j > 0) tc::MbarWait(&mma_done, (j - 1) & 1, kTcMaxPolls);
  } else {
    // ================= consumers: two threads per cell =================
    const int et = threadIdx.x - 256, half = et >> 7, r = et & 127, ew = et >> 5;
    const uint32_t tl = static_cast<uint32_t>((r >> 5) * 32) << 16;
    int tmap[4];
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      const int w = lane + 32 * t, i = w / N, jj = w - i * N;
      tmap[t] = w < N * N ? (i | (jj << 8) | (UpperIndex<N>(i, jj) << 16)) : -1;
    }
    if (half == 1 && blockIdx.x < tiles && static_cast<int64_t>(blockIdx.x) * 128 + r < a.count) {
      const int c0 = a.bucket[static_cast<int64_t>(blockIdx.x) * 128 + r];
      const int32_t* g = a.cell_dofs + static_cast<int64_t>(c0) * a.n_cell;
#pragma unroll
      for (int i = 0; i < N; ++i) tc::CpAsync4(sdofs + r * N + i, g + i);
      tc::CpAsync8(soff + r, a.tri_offset + c0);
    }
    tc::CpAsyncCommit();
    for (int j = 0;; ++j) {
      const int64_t tile = blockIdx.x + static_cast<int64_t>(j) * gridDim.x;
      if (tile >= tiles) break;
      const int64_t t0 = tile * 128;
      const int ncell = static_cast<int>(a.count - t0 < 128 ? a.count - t0 : 128);
      const int bb = j & 1;
      const int64_t t1 = t0 + static_cast<int64_t>(gridDim.x) * 128;
      int c_next = -1;
      if (half == 1 && t1 + r < a.count) c_next = a.bucket[t1 + r];
      const bool ok = tc::MbarWait(&mma_done, j & 1, kTcMaxPolls);
      if (tc::NamedSyncOr(3, 256, !ok || *reinterpret_cast<volatile int*>(&s_abort) != 0)) {
        if (et == 0 && !ok) atomicAdd(tc_timeouts, 1);
        s_abort = 1;
        break;
      }
      tc::FenceAfterSync();
      const uint32_t acc = taddr + tl;
      float inf[8];
      tc::Ld8(acc + 5 * NP, inf);
      tc::WaitLd();
      const int info = static_cast<int>(inf[0]);
      const bool safe = info != 0;
      const int shift = info - 128 + 2 - 54;
      double* vals = svals + r * E;
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int col = 32 * half + 8 * q;
        float G[5][8];
#pragma unroll
        for (int l = 0; l < 5; ++l) tc::Ld8(acc + l * NP + col, G[l]);
        tc::WaitLd();
        if (safe) {
#pragma unroll
          for (int t = 0; t < 8; ++t) {
            const int en = col + t;
            if (en < E) vals[en] = TcCombine(G[0][t], G[1][t], G[2][t], G[3][t], G[4][t], shift + sEc[en]);
          }
        }
      }
      tc::FenceBeforeSync();
      tc::MbarArrive(&tmem_free);
      if (half == 0 && r < ncell && !safe) {
        const int cf = a.bucket[t0 + r];
        int4 cnf;
        double2 vf[4];
        LoadVerts<false>(a, cf, cnf, vf);
        TriaVaryF64<N>(a, cf, cnf, vf, vals);
        atomicAdd(a.fallback, 1ull);
      }
      if (c_next >= 0) {
        const int32_t* g = a.cell_dofs + static_cast<int64_t>(c_next) * a.n_cell;
        int* dn = sdofs + ((j + 1) & 1) * 128 * N + r * N;
#pragma unroll
        for (int i = 0; i < N; ++i) tc::CpAsync4(dn + i, g + i);
        tc::CpAsync8(soff + ((j + 1) & 1) * 128 + r, a.tri_offset + c_next);
      }
      tc::CpAsyncCommit();
      asm volatile("cp.async.wait_group 1;" ::: "memory");
      tc::NamedSync(3, 256);
      const int* sd = sdofs + bb * 128 * N;
      const int64_t* so = soff + bb * 128;
      for (int cl = ew; cl < ncell; cl += 8) {
        lfg_triplet* base = a.out + so[cl];
        const int* dd = sd + cl * N;
        const double* vv = svals + cl * E;
#pragma unroll
        for (int t = 0; t < 4; ++t)
          if (tmap[t] >= 0)
            StoreTriplet(base + lane + 32 * t, dd[tmap[t] & 0xff], dd[(tmap[t] >> 8) & 0xff], vv[tmap[t] >> 16]);
      }
      tc::NamedSync(3, 256);
    }
    tc::CpAsyncWaitAll();
  }
  tc::FenceBeforeSync();
  __syncthreads();
  if (warp == 0) {
    tc::FenceAfterSync();
    tc::TmemFree(taddr, 512);
  }
}

// --------------------------------------------------------------- load vector
template <int DEG, bool QUAD, bool VARY>
__global__ void __launch_bounds__(128) LoadVectorKernel(AsmArgs a) {
  constexpr int N = QUAD ? (DEG + 1) * (DEG + 1) : (DEG + 1) * (DEG + 2) / 2;
  extern __shared__ double sm[];
  LoadTable(a.tab, sm, a.L.total);
  const double* sw = sm + a.L.off_w;
  const double* sqx = sm + a.L.off_qx;
  const double* sqy = sm + a.L.off_qy;
  const double* sphi = sm + a.L.off_phi;
  const double* sL = sm + a.L.off_L;
  const double* so1 = sm + a.L.off_o1;
  const int nq = a.L.nq;
  // Folded rules (exact reformulations of the point sum, computed per block):
  // bilinear quads with cell-constant f: |det J| is affine in (xh, yh), so
  //   sum_k w_k |det J_k| phi_i(k) = s (D0 L_i + D1 Lx_i + D2 Ly_i),
  //   Lx_i = sum_k w_k xh_k phi_i(k), Ly_i = sum_k w_k yh_k phi_i(k);
  // triangles with an O1-nodal f: sum_k w_k f(x_k) phi_i(k) = sum_v f_v M(v, i),
  //   M(v, i) = sum_k w_k lambda_v(k) phi_i(k).
  double* sF = sm + a.L.total;  // [3][N]
  const bool nodal = VARY && !QUAD && a.alpha.kind == LFG_COEFF_NODAL_O1;
  if ((QUAD && !VARY) || nodal) {
    for (int q = threadIdx.x; q < 3 * N; q += blockDim.x) {
      const int g = q / N, i = q - g * N;
      double acc = 0.0;
      for (int k = 0; k < nq; ++k) {
        const double wk = sw[k] * (QUAD ? (g == 0 ? 1.0 : (g == 1 ? sqx[k] : sqy[k])) : so1[k * 4 + g]);
        acc = fma(wk, sphi[k * N + i], acc);
      }
      sF[q] = acc;
    }
    __syncthreads();
  }
  for (int64_t t = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; t < a.count;
       t += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int c = a.bucket[t];
    int4 cn;
    double2 v[4];
    LoadVerts<QUAD>(a, c, cn, v);
    double vec[N];
    bool folded = false;
    if (QUAD && !VARY) {
      // det J = D0 + D1 xh + D2 yh (quad_o1.cc:93-99 rewritten); one sign on the cell
      const double ax = v[1].x - v[0].x, ay = v[1].y - v[0].y, cx = v[3].x - v[0].x, cy = v[3].y - v[0].y;
      const double dx = (v[0].x - v[1].x) + (v[2].x - v[3].x), dy = (v[0].y - v[1].y) + (v[2].y - v[3].y);
      const double D0 = ax * cy - ay * cx, D1 = ax * dy - ay * dx, D2 = dx * cy - dy * cx;
      const double c1 = D0 + D1, c2 = D0 + D2, c3 = c1 + D2;
      if ((D0 > 0 && c1 > 0 && c2 > 0 && c3 > 0) || (D0 < 0 && c1 < 0 && c2 < 0 && c3 < 0)) {
        const double f = (D0 > 0 ? 1.0 : -1.0) * CellConst(a.alpha, c);
#pragma unroll
        for (int i = 0; i < N; ++i) vec[i] = f * fma(D0, sF[i], fma(D1, sF[N + i], D2 * sF[2 * N + i]));
        folded = true;
      }
    }
    if (!QUAD && !VARY) {
      double m00, m01, m11, adet;
      TriaMetric(v, m00, m01, m11, adet);
      const double s = CellConst(a.alpha, c) * adet;
#pragma unroll
      for (int i = 0; i < N; ++i) vec[i] = s * sL[i];
    } else if (nodal) {
      double m00, m01, m11, adet;
      TriaMetric(v, m00, m01, m11, adet);
      const double f0 = a.alpha.data[cn.x] * adet, f1 = a.alpha.data[cn.y] * adet, f2 = a.alpha.data[cn.z] * adet;
#pragma unroll
      for (int i = 0; i < N; ++i) vec[i] = fma(f0, sF[i], fma(f1, sF[N + i], f2 * sF[2 * N + i]));
    } else if (!folded) {
#pragma unroll
      for (int i = 0; i < N; ++i) vec[i] = 0.0;
      double tdet = 0;
      if (!QUAD) {
        double m00, m01, m11;
        TriaMetric(v, m00, m01, m11, tdet);
      }
      for (int k = 0; k < nq; ++k) {
        double adet = tdet;
        if (QUAD) {
          double m00, m01, m11;
          QuadMetric(v, sqx[k], sqy[k], m00, m01, m11, adet);
        }
        const double f = VARY ? EvalCoeff<QUAD>(a.alpha, c, cn, v, k, sw, sqx, sqy, so1)
                              : CellConst(a.alpha, c);
        const double s = sw[k] * adet * f;
#pragma unroll
        for (int i = 0; i < N; ++i) vec[i] = fma(s, sphi[k * N + i], vec[i]);
      }
    }
    double* dst = a.vout + a.tri_offset[c];
#pragma unroll
    for (int i = 0; i < N; ++i) dst[i] = vec[i];
  }
}

// b[d] += contributions in ascending cell order (AssembleVectorLocally order).
__global__ void GatherVectorKernel(int64_t ndofs, const int64_t* __restrict__ ptr,
                                   const uint64_t* __restrict__ slot, const double* __restrict__ ev,
                                   double* __restrict__ b) {
  for (int64_t d = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; d < ndofs;
       d += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    double s = b[d];
    for (int64_t q = ptr[d]; q < ptr[d + 1]; ++q) s += ev[slot[q]];
    b[d] = s;
  }
}

// Tabulated providers.
__global__ void TabulatedMatrixKernel(int64_t nc, const int4* __restrict__ cells,
                                      const int32_t* __restrict__ cell_dofs, int n_cell, int n_tria,
                                      int n_quad, const double* __restrict__ elem, int ld,
                                      const int64_t* __restrict__ tri_offset, lfg_triplet* out) {
  for (int64_t c = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; c < nc;
       c += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int n = cells[c].w < 0 ? n_tria : n_quad;
    const int32_t* d = cell_dofs + c * n_cell;
    const double* em = elem + c * ld * ld;
    lfg_triplet* o = out + tri_offset[c];
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) StoreTriplet(o + i * n + j, d[i], d[j], em[i * ld + j]);
  }
}

__global__ void TabulatedVectorKernel(int64_t nc, const int64_t* __restrict__ loc_offset,
                                      const double* __restrict__ vec, int ld, double* ev) {
  for (int64_t c = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; c < nc;
       c += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int64_t b = loc_offset[c], n = loc_offset[c + 1] - b;
    for (int i = 0; i < n; ++i) ev[b + i] = vec[c * ld + i];
  }
}

// ---------------------------------------------------------- differentiation
// grad[c] = -scale_c * sum_k w_k (G_k lambda)^T (|det J_k| J_k^{-1} J_k^{-T}) (G_k u)
// with G_k lambda = sum_i lambda_i grad(phi_hat_i)(q_k) (reference gradients)
// and scale_c = exp(theta_c) or 1.  This is -lambda_K^T (dA_K/dtheta_c) u_K
// without forming A_K: 4n + 6 FP64 operations per point instead of the
// n^2-entry element matrix.  Flagged dofs contribute lambda_i = 0.
template <int DEG, bool QUAD>
__global__ void __launch_bounds__(128) GradRDKernel(AsmArgs a, const double* __restrict__ u,
                                                    const double* __restrict__ lam,
                                                    const uint8_t* __restrict__ flags, double gscale,
                                                    double* __restrict__ grad) {
  constexpr int N = QUAD ? (DEG + 1) * (DEG + 1) : (DEG + 1) * (DEG + 2) / 2;
  extern __shared__ double sm[];
  const int nq = a.L.nq;
  double* sw = sm;
  double* sqx = sw + nq;
  double* sqy = sqx + nq;
  double* sG = sqy + nq;
  for (int i = threadIdx.x; i < nq; i += blockDim.x) {
    sw[i] = a.tab[a.L.off_w + i];
    sqx[i] = a.tab[a.L.off_qx + i];
    sqy[i] = a.tab[a.L.off_qy + i];
  }
  for (int i = threadIdx.x; i < nq * N * 2; i += blockDim.x) sG[i] = a.tab[a.L.off_G + i];
  __syncthreads();
  for (int64_t t = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; t < a.count;
       t += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int c = a.bucket[t];
    int4 cn;
    double2 v[4];
    LoadVerts<QUAD>(a, c, cn, v);
    double uk[N], lk[N];
#pragma unroll
    for (int i = 0; i < N; ++i) {
      const int d = a.cell_dofs[static_cast<int64_t>(c) * a.n_cell + i];
      uk[i] = u[d];
      lk[i] = (flags && flags[d]) ? 0.0 : lam[d];
    }
    double m00 = 0, m01 = 0, m11 = 0, adet = 0;
    if (!QUAD) TriaMetric(v, m00, m01, m11, adet);
    double s = 0.0;
    for (int k = 0; k < nq; ++k) {
      if (QUAD) QuadMetric(v, sqx[k], sqy[k], m00, m01, m11, adet);
      const double* g = sG + k * N * 2;
      double gu0 = 0, gu1 = 0, gl0 = 0, gl1 = 0;
#pragma unroll
      for (int i = 0; i < N; ++i) {
        gu0 = fma(uk[i], g[2 * i], gu0);
        gu1 = fma(uk[i], g[2 * i + 1], gu1);
        gl0 = fma(lk[i], g[2 * i], gl0);
        gl1 = fma(lk[i], g[2 * i + 1], gl1);
      }
      double q = m00 * gl0 * gu0;
      q = fma(m01, fma(gl0, gu1, gl1 * gu0), q);
      q = fma(m11 * gl1, gu1, q);
      s = fma(sw[k], q, s);
    }
    const double scale = a.alpha.kind == LFG_COEFF_PER_CELL_EXP ? exp(a.alpha.data[c]) : 1.0;
    grad[c] = -gscale * scale * s;
  }
}

// Deterministic 1/2 sum (u - u_obs)^2: fixed chunks of kMisfitChunk entries,
// each summed by one block in a fixed order, then one block over the chunks.
constexpr int kMisfitChunk = 8192;

__global__ void __launch_bounds__(256) MisfitKernel(int64_t n, const double* __restrict__ u,
                                                    const double* __restrict__ uo, double* __restrict__ r,
                                                    double* __restrict__ part) {
  __shared__ double red[256];
  const int64_t b0 = static_cast<int64_t>(blockIdx.x) * kMisfitChunk;
  const int64_t b1 = b0 + kMisfitChunk < n ? b0 + kMisfitChunk : n;
  double s = 0.0;
  for (int64_t i = b0 + threadIdx.x; i < b1; i += 256) {
    const double d = u[i] - uo[i];
    if (r) r[i] = d;
    s = fma(d, d, s);
  }
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

__global__ void __launch_bounds__(256) SumPartsKernel(int64_t m, const double* __restrict__ part,
                                                      double scale, double* __restrict__ out) {
  __shared__ double red[256];
  double s = 0.0;
  for (int64_t i = threadIdx.x; i < m; i += 256) s += part[i];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = scale * red[0];
}

// ------------------------------------------------- boundary-edge providers
// One thread per edge.  Segment rule and basis come in by value (<= 16
// points, <= 4 shape functions).
struct EdgeRule {
  int nq, n;
  double t[16], w[16], phi[16 * 4];
};

struct EdgeArgs {
  int64_t ne;
  const int2* edges;       // endpoints in edge direction
  const double2* xy;
  const uint8_t* flags;    // null: every edge
  const int64_t* offset;   // per edge (null: e * stride)
  int64_t stride;          // n * n (matrix) or n (vector)
  int np, ns;              // dofs per node / edge interior
  int64_t node_dofs;       // num_nodes * np
  CoeffDev f;
};

__device__ __forceinline__ double EdgeCoeff(const CoeffDev& f, int64_t e, const int2& en, const double2& p0,
                                            const double2& p1, double t) {
  switch (f.kind) {
    case LFG_COEFF_CONSTANT: return f.value;
    case LFG_COEFF_PER_CELL: return f.data[e];
    case LFG_COEFF_PER_CELL_EXP: return exp(f.data[e]);
    case LFG_COEFF_NODAL_O1: return f.data[en.x] * (1.0 - t) + f.data[en.y] * t;
    case LFG_COEFF_ANALYTIC: return EvalAnalytic(f, p0.x + t * (p1.x - p0.x), p0.y + t * (p1.y - p0.y));
  }
  return 0.0;
}

// Global dofs of edge e: endpoint dofs in edge direction, then the interior
// dofs (dofhandler.cc:167-195 for codim 1).
__device__ __forceinline__ int EdgeDofs(const EdgeArgs& a, int64_t e, const int2& en, int* d) {
  int k = 0;
  for (int j = 0; j < a.np; ++j) d[k++] = static_cast<int>(static_cast<int64_t>(en.x) * a.np + j);
  for (int j = 0; j < a.np; ++j) d[k++] = static_cast<int>(static_cast<int64_t>(en.y) * a.np + j);
  for (int j = 0; j < a.ns; ++j) d[k++] = static_cast<int>(a.node_dofs + e * a.ns + j);
  return k;
}

__global__ void EdgeCountKernel(int64_t ne, const uint8_t* __restrict__ flags, int64_t per, int64_t* __restrict__ cnt) {
  for (int64_t e = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; e < ne;
       e += static_cast<int64_t>(gridDim.x) * blockDim.x)
    cnt[e] = flags[e] ? per : 0;
}

__global__ void EdgeMassKernel(EdgeArgs a, EdgeRule r, lfg_triplet* __restrict__ out) {
  for (int64_t e = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; e < a.ne;
       e += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    if (a.flags && !a.flags[e]) continue;
    const int2 en = a.edges[e];
    const double2 p0 = a.xy[en.x], p1 = a.xy[en.y];
    const double len = hypot(p1.x - p0.x, p1.y - p0.y);  // SegmentO1 integration element
    int d[8];
    const int n = EdgeDofs(a, e, en, d);
    double m[16];
    for (int q = 0; q < n * n; ++q) m[q] = 0.0;
    for (int k = 0; k < r.nq; ++k) {
      const double s = (r.w[k] * len) * EdgeCoeff(a.f, e, en, p0, p1, r.t[k]);
      for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) m[i * n + j] += r.phi[k * r.n + i] * r.phi[k * r.n + j] * s;
    }
    lfg_triplet* o = out + (a.offset ? a.offset[e] : e * a.stride);
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) StoreTriplet(o + i * n + j, d[i], d[j], m[i * n + j]);
  }
}

// Element vectors of the active edges into ev (at the edge's offset) and the
// (dof, slot) items of the ordered gather.
__global__ void EdgeLoadKernel(EdgeArgs a, EdgeRule r, double* __restrict__ ev, uint64_t* __restrict__ key,
                               uint32_t* __restrict__ slot) {
  for (int64_t e = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; e < a.ne;
       e += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    if (a.flags && !a.flags[e]) continue;
    const int2 en = a.edges[e];
    const double2 p0 = a.xy[en.x], p1 = a.xy[en.y];
    const double len = hypot(p1.x - p0.x, p1.y - p0.y);
    int d[8];
    const int n = EdgeDofs(a, e, en, d);
    double v[4] = {0.0, 0.0, 0.0, 0.0};
    for (int k = 0; k < r.nq; ++k) {
      const double s = (r.w[k] * len) * EdgeCoeff(a.f, e, en, p0, p1, r.t[k]);
      for (int i = 0; i < n; ++i) v[i] += r.phi[k * r.n + i] * s;
    }
    const int64_t off = a.offset ? a.offset[e] : e * a.stride;
    for (int i = 0; i < n; ++i) {
      ev[off + i] = v[i];
      key[off + i] = static_cast<uint64_t>(d[i]);
      slot[off + i] = static_cast<uint32_t>(off + i);
    }
  }
}

// b[dof] += contributions in edge order: after a stable sort of the items by
// dof, the head of each run adds the run's values left to right.
__global__ void EdgeGatherKernel(int64_t n, const uint64_t* __restrict__ key, const uint32_t* __restrict__ slot,
                                 const double* __restrict__ ev, double* __restrict__ b) {
  for (int64_t q = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; q < n;
       q += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    if (q > 0 && key[q - 1] == key[q]) continue;
    const uint64_t d = key[q];
    double s = b[d];
    for (int64_t p = q; p < n && key[p] == d; ++p) s += ev[slot[p]];
    b[d] = s;
  }
}

// ------------------------------------------------------------------ host side

void BuildTable(bool quad, int degree, int rule_degree, std::vector<double>& h, Tab& L) {
  Rule r;
  if (!MakeRule(quad, rule_degree, r))
    Fail(LFG_UNSUPPORTED, "no quadrature rule of degree " + std::to_string(rule_degree) +
                              (quad ? " for quadrilaterals" : " for triangles"));
  if (r.n > kMaxQ) Fail(LFG_UNSUPPORTED, "quadrature rule has too many points");
  const int n = NumShape(quad, degree);
  L = TabLayout(n, r.n);
  h.assign(L.total, 0.0);
  double phi[16], dphi[16][2], p1[16], d1[16][2];
  for (int k = 0; k < r.n; ++k) {
    h[L.off_w + k] = r.w[k];
    h[L.off_qx + k] = r.x[k];
    h[L.off_qy + k] = r.y[k];
    Shape(quad, degree, r.x[k], r.y[k], phi, dphi);
    Shape(quad, 1, r.x[k], r.y[k], p1, d1);
    for (int i = 0; i < n; ++i) h[L.off_phi + k * n + i] = phi[i];
    for (int i = 0; i < n; ++i) {
      h[L.off_G + (k * n + i) * 2 + 0] = dphi[i][0];
      h[L.off_G + (k * n + i) * 2 + 1] = dphi[i][1];
    }
    for (int i = 0; i < (quad ? 4 : 3); ++i) h[L.off_o1 + k * 4 + i] = p1[i];
    int e = 0;
    for (int i = 0; i < n; ++i)
      for (int j = i; j < n; ++j, ++e) {
        double* T = &h[L.off_T + (k * L.E + e) * 4];
        T[0] = dphi[i][0] * dphi[j][0];
        T[1] = dphi[i][0] * dphi[j][1] + dphi[i][1] * dphi[j][0];
        T[2] = dphi[i][1] * dphi[j][1];
        T[3] = phi[i] * phi[j];
      }
  }
  // folded tables in long double: R = sum_k w_k T_k, L = sum_k w_k phi_k
  for (int e = 0; e < L.E; ++e)
    for (int q = 0; q < 4; ++q) {
      long double s = 0.0L;
      for (int k = 0; k < r.n; ++k)
        s += static_cast<long double>(r.w[k]) * h[L.off_T + (k * L.E + e) * 4 + q];
      h[L.off_R + e * 4 + q] = static_cast<double>(s);
    }
  for (int i = 0; i < n; ++i) {
    long double s = 0.0L;
    for (int k = 0; k < r.n; ++k) s += static_cast<long double>(r.w[k]) * h[L.off_phi + k * n + i];
    h[L.off_L + i] = static_cast<double>(s);
  }
}

const double* GetTable(lfg_space* sp, bool quad, int degree, int rule_degree, Tab& L) {
  lfg_ctx* ctx = sp->mesh->ctx;
  const int key = (quad ? 1 << 20 : 0) | (degree << 10) | rule_degree;
  auto it = ctx->tables.find(key);
  if (it != ctx->tables.end()) {
    L = it->second.layout;
    return it->second.buf.as<double>();
  }
  std::vector<double> h;
  BuildTable(quad, degree, rule_degree, h, L);
  TableEntry& ent = ctx->tables[key];
  ent.layout = L;
  ent.buf.alloc(h.size() * sizeof(double), ctx->stream);
  LFG_CUDA(cudaMemcpyAsync(ent.buf.p, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice,
                           ctx->stream));
  LFG_CUDA(cudaStreamSynchronize(ctx->stream));
  return ent.buf.as<double>();
}

// df32 tables (binary32 pairs) of the cell-constant-coefficient kernels.
DfArgs GetDfTable(lfg_space* sp, bool quad, int degree, int rule_degree) {
  lfg_ctx* ctx = sp->mesh->ctx;
  const int key = (quad ? 1 << 20 : 0) | (degree << 10) | rule_degree;
  auto it = ctx->dftables.find(key);
  if (it == ctx->dftables.end()) {
    std::vector<float> h;
    DfLayout L;
    if (!BuildDfTables(quad, degree, rule_degree, h, L)) Fail(LFG_UNSUPPORTED, "no quadrature rule");
    DfTableEntry& ent = ctx->dftables[key];
    ent.layout = L;
    ent.buf.alloc(h.size() * sizeof(float), ctx->stream);
    LFG_CUDA(cudaMemcpyAsync(ent.buf.p, h.data(), h.size() * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
    LFG_CUDA(cudaStreamSynchronize(ctx->stream));
    it = ctx->dftables.find(key);
  }
  DfArgs d;
  d.tab = it->second.buf.as<float>();
  d.L = it->second.layout;
  return d;
}

bool Uniform(const lfg_coeff& c) {
  return c.kind == LFG_COEFF_ZERO || c.kind == LFG_COEFF_CONSTANT || c.kind == LFG_COEFF_PER_CELL ||
         c.kind == LFG_COEFF_PER_CELL_EXP;
}

template <class K, class... Args>
void Launch(K kernel, lfg_ctx* ctx, int64_t count, size_t smem, int block, const Args&... args) {
  if (count <= 0) return;
  LFG_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
  int per_sm = 0;
  LFG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, block, smem));
  if (per_sm < 1) per_sm = 1;
  int64_t blocks = (count + block - 1) / block;
  blocks = std::min<int64_t>(blocks, static_cast<int64_t>(ctx->num_sms) * per_sm);
  kernel<<<static_cast<unsigned>(blocks), block, smem, ctx->stream>>>(args...);
  LFG_LAUNCHED(ctx);
}

template <int DEG, int M, bool MASS>
void LaunchQuadDf(lfg_ctx* ctx, const AsmArgs& a, const DfArgs& d) {
  constexpr int N = (DEG + 1) * (DEG + 1), E = N * (N + 1) / 2, NQ = M * M, TILE = E > 64 ? 64 : 128;
  if (DEG >= 2 && d.L.n1 == DEG + 1 && d.L.m == M) {
    constexpr int SD = DEG >= 2 ? DEG : 2;  // (the branch is dead for DEG 1)
    const uint32_t bit = 1u << SfSlotIndex(SD, M);
    if (!(ctx->sf_const_ready & bit)) {
      // slot <- [1D products | W | t] from the df32 table block on the device
      constexpr int sfp = 3 * (SD + 1) * (SD + 1) * M;
      const size_t off = SfSlotOffset<SD, M>() * sizeof(float2);
      const float2* src = reinterpret_cast<const float2*>(d.tab);
      LFG_CUDA(cudaMemcpyToSymbolAsync(c_sf_tables, src + d.L.off_SF, sfp * sizeof(float2), off,
                                       cudaMemcpyDeviceToDevice, ctx->stream));
      LFG_CUDA(cudaMemcpyToSymbolAsync(c_sf_tables, src + d.L.off_W, NQ * sizeof(float2), off + sfp * sizeof(float2),
                                       cudaMemcpyDeviceToDevice, ctx->stream));
      LFG_CUDA(cudaMemcpyToSymbolAsync(c_sf_tables, src + d.L.off_t, M * sizeof(float2),
                                       off + (sfp + NQ) * sizeof(float2), cudaMemcpyDeviceToDevice, ctx->stream));
      ctx->sf_const_ready |= bit;
    }
    const size_t smem = TILE * (E * 8 + 8 + N * 4);
    Launch(RDQuadDfKernel<SD, M, MASS, true>, ctx, a.count, smem, 128, a, d);
    return;
  }
  constexpr int TP = QuadTabPairs<DEG, M>();
  const size_t smem = (((TP + NQ + M) * 8 + 15) & ~size_t(15)) + TILE * (E * 8 + 8 + N * 4);
  Launch(RDQuadDfKernel<DEG, M, MASS, false>, ctx, a.count, smem, 128, a, d);
}

// FP16 bit pattern of a value that FP16 represents exactly (|v| in [2^-14, 2^15] or 0).
uint16_t HalfBits(double v) {
  if (v == 0.0) return 0;
  const uint16_t s = v < 0.0 ? 0x8000 : 0;
  int ex;
  const double f = std::frexp(std::fabs(v), &ex);  // |v| = f 2^ex, f in [0.5, 1)
  const double m = (2.0 * f - 1.0) * 1024.0;
  if (ex + 14 < 1 || ex + 14 > 30 || m != std::floor(m)) Fail(LFG_UNSUPPORTED, "tensor-core table digit not exact");
  return static_cast<uint16_t>(s | ((ex + 14) << 10) | static_cast<int>(m));
}

// Table digits of RDQuadTcKernel for the quad table block `tab` (FP64 T read
// back from the device once): [plain | 2^-9 scaled] x [digit j = 1..6] x
// [48 entries] x [KP] in the core-matrix layout, then the 48 column exponents.
const uint4* GetQuadTcImage(lfg_ctx* ctx, const double* tab, const Tab& L, int m) {
  auto it = ctx->tc_images.find(tab);
  if (it != ctx->tc_images.end()) return it->second.as<uint4>();
  const int K = 3 * L.nq, KP = TcKP(m), E = L.E;
  std::vector<double> T(static_cast<size_t>(L.nq) * E * 4);
  LFG_CUDA(cudaMemcpyAsync(T.data(), tab + L.off_T, T.size() * sizeof(double), cudaMemcpyDeviceToHost,
                           ctx->stream));
  LFG_CUDA(cudaStreamSynchronize(ctx->stream));
  std::vector<uint16_t> img(static_cast<size_t>(TcImageBytes(m)) / 2, 0);
  uint16_t* plain = img.data();
  uint16_t* scaled = plain + TcBHalfBytes(m) / 2;
  uint16_t* info = plain + TcBHalfBytes(m);
  int32_t* ec = reinterpret_cast<int32_t*>(plain + TcEcOffset(m) / 2);
  info[((KP - 1) / 8) * 64 + 7] = HalfBits(1.0);  // row 0, K column KP - 1
  auto at = [&](int k, int ab, int e) { return T[(static_cast<size_t>(k) * E + e) * 4 + ab]; };
  for (int e = 0; e < E; ++e) {
    double mt = 0.0;
    for (int k = 0; k < L.nq; ++k)
      for (int ab = 0; ab < 3; ++ab) mt = std::max(mt, std::fabs(at(k, ab, e)));
    int ex = 0;
    if (mt > 0.0) std::frexp(mt, &ex);
    ec[e] = mt > 0.0 ? ex + 1 : 0;  // |T| 2^-Ec < 1/2
    for (int kab = 0; kab < K; ++kab) {
      const int kap = TcKappa(m, kab / 3, kab % 3);
      long long Y = std::llround(std::ldexp(at(kab / 3, kab % 3, e), 54 - ec[e]));
      int b[7];
      for (int j = 6; j >= 2; --j) {  // balanced 9-bit digits from the bottom
        long long rr = ((Y % 512) + 512) % 512;
        if (rr >= 256) rr -= 512;
        b[j] = static_cast<int>(rr);
        Y = (Y - rr) / 512;
      }
      b[1] = static_cast<int>(Y);
      for (int j = 1; j <= 6; ++j) {
        const int n = (j - 1) * kTcNP + e;
        const size_t off = static_cast<size_t>(n / 8) * (KP / 8) * 64 + (kap / 8) * 64 + (n % 8) * 8 + kap % 8;
        plain[off] = HalfBits(b[j]);
        scaled[off] = HalfBits(std::ldexp(static_cast<double>(b[j]), -9));
      }
    }
  }
  DevBuf& buf = ctx->tc_images[tab];
  buf.alloc(img.size() * 2, ctx->stream);
  LFG_CUDA(cudaMemcpyAsync(buf.p, img.data(), img.size() * 2, cudaMemcpyHostToDevice, ctx->stream));
  LFG_CUDA(cudaStreamSynchronize(ctx->stream));
  return buf.as<uint4>();
}

template <int M>
void LaunchQuadTcWs(lfg_ctx* ctx, const AsmArgs& a, const DfArgs& d) {
  const uint4* img = GetQuadTcImage(ctx, a.tab, a.L, M);
  int* timeouts = StatusWord(ctx) + 14;
  const size_t smem = WsSmemBytes(M);
  auto kernel = RDQuadTcWsKernel<M>;
  LFG_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
  const int64_t tiles = (a.count + 127) / 128;
  const int64_t grid = std::min<int64_t>(tiles, ctx->num_sms);  // one CTA per SM (512 TMEM columns each)
  if (grid <= 0) return;
  kernel<<<static_cast<unsigned>(grid), kWsThreads, smem, ctx->stream>>>(a, d, img, timeouts);
  LFG_LAUNCHED(ctx);
}

template <int M>
void LaunchQuadTcWs2(lfg_ctx* ctx, const AsmArgs& a, const DfArgs& d) {
  const uint4* img = GetQuadTcImage(ctx, a.tab, a.L, M);
  int* timeouts = StatusWord(ctx) + 14;
  const size_t smem = Ws2SmemBytes(M);
  auto kernel = RDQuadTcWs2Kernel<M>;
  LFG_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
  const int64_t tiles = (a.count + 127) / 128;
  const int64_t grid = std::min<int64_t>(tiles, ctx->num_sms);  // one CTA per SM (512 TMEM columns each)
  if (grid <= 0) return;
  kernel<<<static_cast<unsigned>(grid), kWsThreads, smem, ctx->stream>>>(a, d, img, timeouts);
  LFG_LAUNCHED(ctx);
}

template <int M>
void LaunchQuadTc(lfg_ctx* ctx, const AsmArgs& a, const DfArgs& d) {
  const uint4* img = GetQuadTcImage(ctx, a.tab, a.L, M);
  int* timeouts = StatusWord(ctx) + 14;
  // At least 80 KB of shared memory per CTA: never more than two CTAs on an
  // SM, so their 2 x 256 tensor-memory columns always fit and no allocation waits.
  const size_t smem = std::max<size_t>(TcSmemBytes(M), 80 * 1024);
  auto kernel = RDQuadTcKernel<M>;
  LFG_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
  LFG_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                                static_cast<int>(cudaSharedmemCarveoutMaxShared)));
  // Two CTAs per SM (shared memory admits two; the occupancy query assumes a
  // smaller carveout and answers one).  CTAs never wait on each other, so
  // the grid is correct whatever the residency.
  const int64_t tiles = (a.count + 127) / 128;
  const int64_t grid = std::min<int64_t>(tiles, static_cast<int64_t>(ctx->num_sms) * 2);
  if (grid <= 0) return;
  kernel<<<static_cast<unsigned>(grid), 256, smem, ctx->stream>>>(a, d, img, timeouts);
  LFG_LAUNCHED(ctx);
}

// Table digits of RDTriaTcKernel (O3 triangles, 12-point rule): columns
// TtKappa(k, ab) = T(k; e, ab), column 42 = the folded mass table R(e); same
// digit layout as GetQuadTcImage with 64 entries per digit block.
const uint4* GetTriaTcImage(lfg_ctx* ctx, const double* tab, const Tab& L) {
  auto it = ctx->tc_images.find(tab);
  if (it != ctx->tc_images.end()) return it->second.as<uint4>();
  const int E = L.E, KP = kTtKP;
  std::vector<double> h(static_cast<size_t>(L.total));
  LFG_CUDA(cudaMemcpyAsync(h.data(), tab, h.size() * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  LFG_CUDA(cudaStreamSynchronize(ctx->stream));
  std::vector<uint16_t> img(static_cast<size_t>(kTtImage) / 2, 0);
  uint16_t* plain = img.data();
  uint16_t* scaled = plain + kTtBHalf / 2;
  uint16_t* info = plain + kTtBHalf;
  int32_t* ec = reinterpret_cast<int32_t*>(plain + kTtEcOff / 2);
  info[((KP - 1) / 8) * 64 + 7] = HalfBits(1.0);
  std::vector<std::pair<int, double>> col;  // (kappa, value) of one entry
  for (int e = 0; e < E; ++e) {
    col.clear();
    for (int k = 0; k < L.nq; ++k)
      for (int ab = 0; ab < 3; ++ab) col.push_back({TtKappa(k, ab), h[L.off_T + (static_cast<size_t>(k) * E + e) * 4 + ab]});
    col.push_back({42, h[L.off_R + e * 4 + 3]});
    double mt = 0.0;
    for (auto& kv : col) mt = std::max(mt, std::fabs(kv.second));
    int ex = 0;
    if (mt > 0.0) std::frexp(mt, &ex);
    ec[e] = mt > 0.0 ? ex + 1 : 0;
    for (auto& kv : col) {
      long long Y = std::llround(std::ldexp(kv.second, 54 - ec[e]));
      int b[7];
      for (int j = 6; j >= 2; --j) {
        long long rr = ((Y % 512) + 512) % 512;
        if (rr >= 256) rr -= 512;
        b[j] = static_cast<int>(rr);
        Y = (Y - rr) / 512;
      }
      b[1] = static_cast<int>(Y);
      for (int j = 1; j <= 6; ++j) {
        const int n = (j - 1) * kTtNP + e, kap = kv.first;
        const size_t off = static_cast<size_t>(n / 8) * (KP / 8) * 64 + (kap / 8) * 64 + (n % 8) * 8 + kap % 8;
        plain[off] = HalfBits(b[j]);
        scaled[off] = HalfBits(std::ldexp(static_cast<double>(b[j]), -9));
      }
    }
  }
  DevBuf& buf = ctx->tc_images[tab];
  buf.alloc(img.size() * 2, ctx->stream);
  LFG_CUDA(cudaMemcpyAsync(buf.p, img.data(), img.size() * 2, cudaMemcpyHostToDevice, ctx->stream));
  LFG_CUDA(cudaStreamSynchronize(ctx->stream));
  return buf.as<uint4>();
}

void LaunchTriaTc(lfg_ctx* ctx, const AsmArgs& a, const DfArgs& d) {
  const uint4* img = GetTriaTcImage(ctx, a.tab, a.L);
  int* timeouts = StatusWord(ctx) + 14;
  const int fam = a.alpha.kind == LFG_COEFF_NODAL_O1 ? 0 : (a.alpha.func == LFG_FN_POLY ? 1 : 2);
  auto kernel = fam == 0 ? RDTriaTcKernel<0> : (fam == 1 ? RDTriaTcKernel<1> : RDTriaTcKernel<2>);
  LFG_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kTtSmem));
  const int64_t tiles = (a.count + 127) / 128;
  const int64_t grid = std::min<int64_t>(tiles, ctx->num_sms);  // one CTA per SM (512 TMEM columns)
  if (grid <= 0) return;
  kernel<<<static_cast<unsigned>(grid), 512, kTtSmem, ctx->stream>>>(a, d, img, timeouts);
  LFG_LAUNCHED(ctx);
}

template <int DEG, int NQ>
void LaunchTriaVaryDf(lfg_ctx* ctx, const AsmArgs& a, const DfArgs& d) {
  constexpr int N = (DEG + 1) * (DEG + 2) / 2, E = N * (N + 1) / 2;
  constexpr int TP = NQ * E * 4 + E * 4 + NQ + 2 * NQ + 4 * NQ + 23;
  const size_t smem = ((TP * 8 + 15) & ~size_t(15)) + 128 * (E * 8 + 8 + N * 4);
  Launch(RDTriaVaryDfKernel<DEG, NQ>, ctx, a.count, smem, 128, a, d);
}

// df32 kernel for point-varying alpha on triangles: alpha analytic or O1
// nodal, gamma cell-constant, a rule with a supported point count.
template <int DEG>
bool TryTriaVaryDf(lfg_ctx* ctx, const AsmArgs& a, const DfArgs& d) {
  if (!d.tab) return false;
  if (a.alpha.kind != LFG_COEFF_ANALYTIC && a.alpha.kind != LFG_COEFF_NODAL_O1) return false;
  // the df32 evaluator knows the polynomial and sin/cos families only
  if (a.alpha.kind == LFG_COEFF_ANALYTIC && a.alpha.func > LFG_FN_SINCOS) return false;
  const int gk = a.gamma.kind;
  if (gk != LFG_COEFF_ZERO && gk != LFG_COEFF_CONSTANT && gk != LFG_COEFF_PER_CELL && gk != LFG_COEFF_PER_CELL_EXP)
    return false;
  if (DEG == 3 && d.L.nq == kTtNQ && a.L.E == kTtE && a.L.nq == kTtNQ && ctx->tensor_cores) {
    ProfScope prof(ctx, "rd_tria_vary_tc");
    LaunchTriaTc(ctx, a, d);
    return true;
  }
  ProfScope prof(ctx, "rd_tria_vary_df");
  switch (d.L.nq) {
    case 1: LaunchTriaVaryDf<DEG, 1>(ctx, a, d); return true;
    case 3: LaunchTriaVaryDf<DEG, 3>(ctx, a, d); return true;
    case 6: LaunchTriaVaryDf<DEG, 6>(ctx, a, d); return true;
    case 7: LaunchTriaVaryDf<DEG, 7>(ctx, a, d); return true;
    case 12: LaunchTriaVaryDf<DEG, 12>(ctx, a, d); return true;
  }
  return false;
}

template <int DEG, bool QUAD>
void LaunchRD(lfg_ctx* ctx, const AsmArgs& a, const DfArgs& d, bool uniform, bool mass) {
  const size_t smem_gen = a.L.total * sizeof(double);
  if (!uniform && !QUAD && TryTriaVaryDf<DEG>(ctx, a, d)) return;
  if (uniform && d.tab && !QUAD) {
    constexpr int N = (DEG + 1) * (DEG + 2) / 2, E = N * (N + 1) / 2;
    const size_t smem = ((E * 4 * 8 + 15) & ~size_t(15)) + 128 * (E * 8 + 8 + N * 4);
    ProfScope prof(ctx, "rd_tria_df");
    if (mass) Launch(RDTriaDfKernel<DEG, true>, ctx, a.count, smem, 128, a, d);
    else Launch(RDTriaDfKernel<DEG, false>, ctx, a.count, smem, 128, a, d);
    return;
  }
  if (DEG == 2 && QUAD && uniform && !mass && d.tab && ctx->tensor_cores && a.L.E == 45 && d.L.n1 == 3 &&
      (d.L.m == 2 || d.L.m == 3) && a.L.nq == d.L.m * d.L.m) {
    ProfScope prof(ctx, "rd_quad_tc");
    if (ctx->tensor_cores == 2) {
      if (d.L.m == 2) LaunchQuadTc<2>(ctx, a, d);
      else LaunchQuadTc<3>(ctx, a, d);
    } else if (ctx->tensor_cores == 3) {
      if (d.L.m == 2) LaunchQuadTcWs2<2>(ctx, a, d);
      else LaunchQuadTcWs2<3>(ctx, a, d);
    } else {
      if (d.L.m == 2) LaunchQuadTcWs<2>(ctx, a, d);
      else LaunchQuadTcWs<3>(ctx, a, d);
    }
    return;
  }
  if (uniform && d.tab && QUAD && d.L.m >= 2 && d.L.m <= 4) {
    ProfScope prof(ctx, "rd_quad_df");
    switch (d.L.m * 2 + (mass ? 1 : 0)) {
      case 4: LaunchQuadDf<DEG, 2, false>(ctx, a, d); break;
      case 5: LaunchQuadDf<DEG, 2, true>(ctx, a, d); break;
      case 6: LaunchQuadDf<DEG, 3, false>(ctx, a, d); break;
      case 7: LaunchQuadDf<DEG, 3, true>(ctx, a, d); break;
      case 8: LaunchQuadDf<DEG, 4, false>(ctx, a, d); break;
      case 9: LaunchQuadDf<DEG, 4, true>(ctx, a, d); break;
    }
    return;
  }
  ProfScope prof(ctx, QUAD ? "rd_general_quad" : "rd_general_tria");
  if (uniform) {
    if (mass) Launch(RDGeneralKernel<DEG, QUAD, false, true>, ctx, a.count, smem_gen, 128, a);
    else Launch(RDGeneralKernel<DEG, QUAD, false, false>, ctx, a.count, smem_gen, 128, a);
  } else {
    if (mass) Launch(RDGeneralKernel<DEG, QUAD, true, true>, ctx, a.count, smem_gen, 128, a);
    else Launch(RDGeneralKernel<DEG, QUAD, true, false>, ctx, a.count, smem_gen, 128, a);
  }
}

template <int DEG, bool QUAD>
void LaunchTensor(lfg_ctx* ctx, const AsmArgs& a, bool mass) {
  const size_t smem = static_cast<size_t>(a.L.off_T + a.L.total - a.L.off_o1) * sizeof(double);
  ProfScope prof(ctx, QUAD ? "rd_tensor_quad" : "rd_tensor_tria");
  if (mass) Launch(RDTensorKernel<DEG, QUAD, true>, ctx, a.count, smem, 128, a);
  else Launch(RDTensorKernel<DEG, QUAD, false>, ctx, a.count, smem, 128, a);
}

template <bool QUAD>
void DispatchTensor(lfg_ctx* ctx, int degree, const AsmArgs& a, bool mass) {
  switch (degree) {
    case 1: LaunchTensor<1, QUAD>(ctx, a, mass); break;
    case 2: LaunchTensor<2, QUAD>(ctx, a, mass); break;
    case 3: LaunchTensor<3, QUAD>(ctx, a, mass); break;
  }
}

template <bool QUAD>
void DispatchRD(lfg_ctx* ctx, int degree, const AsmArgs& a, const DfArgs& d, bool uniform, bool mass) {
  switch (degree) {
    case 1: LaunchRD<1, QUAD>(ctx, a, d, uniform, mass); break;
    case 2: LaunchRD<2, QUAD>(ctx, a, d, uniform, mass); break;
    case 3: LaunchRD<3, QUAD>(ctx, a, d, uniform, mass); break;
  }
}

template <bool QUAD>
void DispatchLoad(lfg_ctx* ctx, int degree, const AsmArgs& a, bool vary) {
  const size_t smem = (a.L.total + 3 * 16) * sizeof(double);  // tables + the folded rules
  ProfScope prof(ctx, QUAD ? "load_quad" : "load_tria");
  switch (degree) {
    case 1: vary ? Launch(LoadVectorKernel<1, QUAD, true>, ctx, a.count, smem, 128, a)
                 : Launch(LoadVectorKernel<1, QUAD, false>, ctx, a.count, smem, 128, a); break;
    case 2: vary ? Launch(LoadVectorKernel<2, QUAD, true>, ctx, a.count, smem, 128, a)
                 : Launch(LoadVectorKernel<2, QUAD, false>, ctx, a.count, smem, 128, a); break;
    case 3: vary ? Launch(LoadVectorKernel<3, QUAD, true>, ctx, a.count, smem, 128, a)
                 : Launch(LoadVectorKernel<3, QUAD, false>, ctx, a.count, smem, 128, a); break;
  }
}

int RuleDegree(int requested, int degree) { return requested == 0 ? 2 * degree : requested; }

AsmArgs BaseArgs(lfg_space* sp) {
  AsmArgs a{};
  a.fallback = reinterpret_cast<unsigned long long*>(StatusWord(sp->mesh->ctx) + 12);
  a.cells = sp->mesh->cell_nodes.as<int4>();
  a.xy = sp->mesh->xy.as<double2>();
  a.cell_dofs = sp->cell_dofs.as<int32_t>();
  a.n_cell = sp->n_cell;
  return a;
}

}  // namespace

// Element vectors of the load provider into sp->scratch_vec (exposed for the
// vector assembly and the gradient path).
void LoadElementVectors(lfg_space* sp, const lfg_load_provider* pr, double* ev) {
  lfg_ctx* ctx = sp->mesh->ctx;
  lfg_mesh* m = sp->mesh;
  const int deg = sp->degree;
  AsmArgs a = BaseArgs(sp);
  a.tri_offset = sp->loc_offset.as<int64_t>();
  a.vout = ev;
  a.alpha = ToDev(pr->f, m, "load f");
  const bool vary = !Uniform(pr->f);
  if (m->ntria) {
    if (pr->qr_degree_tria < 0) Fail(LFG_MISSING_RULE, "no quadrature rule for triangles");
    a.tab = GetTable(sp, false, deg, RuleDegree(pr->qr_degree_tria, deg), a.L);
    a.bucket = m->tria_list.as<int32_t>();
    a.count = m->ntria;
    DispatchLoad<false>(ctx, deg, a, vary);
  }
  if (m->nquad) {
    if (pr->qr_degree_quad < 0) Fail(LFG_MISSING_RULE, "no quadrature rule for quadrilaterals");
    a.tab = GetTable(sp, true, deg, RuleDegree(pr->qr_degree_quad, deg), a.L);
    a.bucket = m->quad_list.as<int32_t>();
    a.count = m->nquad;
    DispatchLoad<true>(ctx, deg, a, vary);
  }
}

// Argument checks of the Lagrangian reaction-diffusion assembly.
void CheckRD(lfg_space* sp, const lfg_rd_provider* pr) {
  if (sp->degree < 1) Fail(LFG_UNSUPPORTED, "reaction-diffusion provider needs a Lagrangian space");
  lfg_mesh* m = sp->mesh;
  if (m->ntria && pr->qr_degree_tria < 0)
    Fail(LFG_MISSING_RULE, "No local shape function information or no quadrature rule for reference element type TRIA");
  if (m->nquad && pr->qr_degree_quad < 0)
    Fail(LFG_MISSING_RULE, "No local shape function information or no quadrature rule for reference element type QUAD");
}

// Element matrices of the triangles tria_list[t0, t1) and quadrilaterals
// quad_list[q0, q1) (each list ascending by cell index): cell c's n_c^2
// triplets go to out + tri_offset[c], row-major.
void AssembleRDCells(lfg_space* sp, const lfg_rd_provider* pr, lfg_triplet* out, int64_t t0, int64_t t1,
                     int64_t q0, int64_t q1) {
  lfg_mesh* m = sp->mesh;
  AsmArgs a = BaseArgs(sp);
  a.tri_offset = sp->tri_offset.as<int64_t>();
  a.out = out;
  a.alpha = ToDev(pr->alpha, m, "alpha", true);
  a.gamma = ToDev(pr->gamma, m, "gamma");
  const bool uniform = Uniform(pr->alpha) && Uniform(pr->gamma);
  const bool mass = pr->gamma.kind != LFG_COEFF_ZERO;
  const int deg = sp->degree;
  DfArgs none{nullptr, DfLayout()};
  if (IsTensor(pr->alpha.kind)) {
    for (int pass = 0; pass < 2; ++pass) {
      const bool quad = pass == 1;
      a.count = quad ? q1 - q0 : t1 - t0;
      if (a.count <= 0) continue;
      a.tab = GetTable(sp, quad, deg, RuleDegree(quad ? pr->qr_degree_quad : pr->qr_degree_tria, deg), a.L);
      a.bucket = quad ? m->quad_list.as<int32_t>() + q0 : m->tria_list.as<int32_t>() + t0;
      if (quad) DispatchTensor<true>(m->ctx, deg, a, mass);
      else DispatchTensor<false>(m->ctx, deg, a, mass);
    }
    return;
  }
  if (t1 > t0) {
    const int rd = RuleDegree(pr->qr_degree_tria, deg);
    a.tab = GetTable(sp, false, deg, rd, a.L);
    a.bucket = m->tria_list.as<int32_t>() + t0;
    a.count = t1 - t0;
    DispatchRD<false>(m->ctx, deg, a, GetDfTable(sp, false, deg, rd), uniform, mass);
  }
  if (q1 > q0) {
    const int rd = RuleDegree(pr->qr_degree_quad, deg);
    a.tab = GetTable(sp, true, deg, rd, a.L);
    a.bucket = m->quad_list.as<int32_t>() + q0;
    a.count = q1 - q0;
    DispatchRD<true>(m->ctx, deg, a, uniform ? GetDfTable(sp, true, deg, rd) : none, uniform, mass);
  }
}

__global__ void GatherI64Kernel(int64_t n, const int64_t* __restrict__ idx, const int64_t* __restrict__ src,
                                int64_t* __restrict__ out) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x)
    out[i] = src[idx[i]];
}

// grad[c] = -gscale * lambda_K^T (dA_K/dtheta_c) u_K for every cell (the
// differentiation entry point and the adjoint Function object share it).
void GradRDCellwise(lfg_space* sp, const lfg_rd_provider* pr, const double* u, const double* lam,
                    const uint8_t* flags, double gscale, double* grad) {
  if (!pr || !u || !lam || !grad) Fail(LFG_INVALID_ARG, "lfg_grad_rd_cellwise: null argument");
  if (sp->degree < 1) Fail(LFG_UNSUPPORTED, "gradient needs a Lagrangian space");
  if (pr->alpha.kind != LFG_COEFF_PER_CELL && pr->alpha.kind != LFG_COEFF_PER_CELL_EXP)
    Fail(LFG_UNSUPPORTED, "gradient: alpha must be a per-cell (or per-cell exp) coefficient");
  lfg_mesh* m = sp->mesh;
  lfg_ctx* ctx = m->ctx;
  if (m->ntria && pr->qr_degree_tria < 0) Fail(LFG_MISSING_RULE, "no quadrature rule for triangles");
  if (m->nquad && pr->qr_degree_quad < 0) Fail(LFG_MISSING_RULE, "no quadrature rule for quadrilaterals");
  AsmArgs a = BaseArgs(sp);
  a.alpha = ToDev(pr->alpha, m, "alpha");
  const int deg = sp->degree;
  ProfScope prof(ctx, "grad_rd");
  for (int pass = 0; pass < 2; ++pass) {
    const bool quad = pass == 1;
    a.count = quad ? m->nquad : m->ntria;
    if (!a.count) continue;
    a.tab = GetTable(sp, quad, deg, RuleDegree(quad ? pr->qr_degree_quad : pr->qr_degree_tria, deg), a.L);
    a.bucket = quad ? m->quad_list.as<int32_t>() : m->tria_list.as<int32_t>();
    const size_t smem = static_cast<size_t>(a.L.nq) * (3 + 2 * a.L.n) * sizeof(double);
    switch (deg * 2 + (quad ? 1 : 0)) {
      case 2: Launch(GradRDKernel<1, false>, ctx, a.count, smem, 128, a, u, lam, flags, gscale, grad); break;
      case 3: Launch(GradRDKernel<1, true>, ctx, a.count, smem, 128, a, u, lam, flags, gscale, grad); break;
      case 4: Launch(GradRDKernel<2, false>, ctx, a.count, smem, 128, a, u, lam, flags, gscale, grad); break;
      case 5: Launch(GradRDKernel<2, true>, ctx, a.count, smem, 128, a, u, lam, flags, gscale, grad); break;
      case 6: Launch(GradRDKernel<3, false>, ctx, a.count, smem, 128, a, u, lam, flags, gscale, grad); break;
      case 7: Launch(GradRDKernel<3, true>, ctx, a.count, smem, 128, a, u, lam, flags, gscale, grad); break;
    }
  }
}

}  // namespace lfg

using namespace lfg;

extern "C" {

lfg_status lfg_assemble_matrix_rd(lfg_space* sp, const lfg_rd_provider* pr, lfg_coo* coo) {
  if (!sp) return LFG_INVALID_ARG;
  LFG_API_BEGIN(sp->mesh->ctx)
  if (!pr || !coo) Fail(LFG_INVALID_ARG, "lfg_assemble_matrix_rd: null argument");
  if (sp->hier_degree > 0) {
    HierAssembleMatrix(sp, pr, coo);
    return LFG_OK;
  }
  CheckRD(sp, pr);
  if (coo->rows < sp->num_dofs || coo->cols < sp->num_dofs)
    Fail(LFG_INVALID_ARG, "COO matrix smaller than the number of dofs");
  if (coo->size + sp->num_triplets > coo->capacity)
    Fail(LFG_CAPACITY, "COO capacity " + std::to_string(coo->capacity) + " < " +
                           std::to_string(coo->size + sp->num_triplets));
  AssembleRDCells(sp, pr, coo->d + coo->size, 0, sp->mesh->ntria, 0, sp->mesh->nquad);
  coo->size += sp->num_triplets;
  LFG_API_END
}

lfg_status lfg_assemble_matrix_rd_to_host(lfg_space* sp, const lfg_rd_provider* pr, lfg_triplet* host,
                                          int64_t capacity, int64_t chunk_triplets, int64_t* count) {
  if (!sp) return LFG_INVALID_ARG;
  LFG_API_BEGIN(sp->mesh->ctx)
  if (!pr || !host) Fail(LFG_INVALID_ARG, "lfg_assemble_matrix_rd_to_host: null argument");
  if (sp->hier_degree > 0) Fail(LFG_UNSUPPORTED, "host output: Lagrangian spaces only");
  CheckRD(sp, pr);
  if (capacity < sp->num_triplets)
    Fail(LFG_CAPACITY, "host capacity " + std::to_string(capacity) + " < " + std::to_string(sp->num_triplets));
  lfg_mesh* m = sp->mesh;
  lfg_ctx* ctx = m->ctx;
  cudaStream_t s = ctx->stream;
  // page-locked output from lfg_host_alloc: the kernels store the triplets
  // straight into it over the host link (one pass, no staging ring)
  if (void* mapped = MappedHost(ctx, host, static_cast<size_t>(sp->num_triplets) * sizeof(lfg_triplet))) {
    // over the host link the quadrilateral kernel whose eight consumer warps
    // write the triplets keeps more stores in flight than the default, whose
    // four producer warps of a group write them (29.07 vs 29.60 ms for the
    // 5.13 GB of the hybrid 2048 x 2048 O2 matrix); same bits either way
    const int tc = ctx->tensor_cores;
    if (tc == 3) ctx->tensor_cores = 1;
    try {
      AssembleRDCells(sp, pr, static_cast<lfg_triplet*>(mapped), 0, m->ntria, 0, m->nquad);
    } catch (...) {
      ctx->tensor_cores = tc;
      throw;
    }
    ctx->tensor_cores = tc;
    LFG_CUDA(cudaStreamSynchronize(s));
    if (count) *count = sp->num_triplets;
    return LFG_OK;
  }
  const int64_t nc = m->nc;
  const int64_t nmax = std::max(sp->n_tria, sp->n_quad);
  const int64_t per_cell = nmax * nmax;
  if (chunk_triplets <= 0) chunk_triplets = int64_t(1) << 24;
  chunk_triplets = std::max(chunk_triplets, per_cell);
  const int64_t cells_per_chunk = std::max<int64_t>(1, chunk_triplets / per_cell);
  const int64_t nchunk = (nc + cells_per_chunk - 1) / cells_per_chunk;
  // host copies of the ascending type lists (the chunk boundaries are found
  // in them by binary search) and the triplet offsets of the boundary cells
  if (m->h_tria_list.size() != static_cast<size_t>(m->ntria) ||
      m->h_quad_list.size() != static_cast<size_t>(m->nquad)) {
    m->h_tria_list.resize(m->ntria);
    m->h_quad_list.resize(m->nquad);
    if (m->ntria)
      LFG_CUDA(cudaMemcpyAsync(m->h_tria_list.data(), m->tria_list.p, m->ntria * sizeof(int32_t),
                               cudaMemcpyDeviceToHost, s));
    if (m->nquad)
      LFG_CUDA(cudaMemcpyAsync(m->h_quad_list.data(), m->quad_list.p, m->nquad * sizeof(int32_t),
                               cudaMemcpyDeviceToHost, s));
  }
  std::vector<int64_t> bound(nchunk + 1), toff(nchunk + 1);
  for (int64_t k = 0; k <= nchunk; ++k) bound[k] = std::min(nc, k * cells_per_chunk);
  {
    DevBuf db, dout;
    db.alloc((nchunk + 1) * sizeof(int64_t), s);
    dout.alloc((nchunk + 1) * sizeof(int64_t), s);
    LFG_CUDA(cudaMemcpyAsync(db.p, bound.data(), (nchunk + 1) * sizeof(int64_t), cudaMemcpyHostToDevice, s));
    GatherI64Kernel<<<static_cast<unsigned>((nchunk + 256) / 256), 256, 0, s>>>(
        nchunk + 1, db.as<int64_t>(), sp->tri_offset.as<int64_t>(), dout.as<int64_t>());
    LFG_LAUNCHED(ctx);
    LFG_CUDA(cudaMemcpyAsync(toff.data(), dout.p, (nchunk + 1) * sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    LFG_CUDA(cudaStreamSynchronize(s));
  }
  // staging ring: the assembly of range k on the context stream overlaps the
  // download of range k - 1 on a second stream; events order the reuse
  constexpr int kRing = 3;
  int64_t slot_trip = 1;
  for (int64_t k = 0; k < nchunk; ++k) slot_trip = std::max(slot_trip, toff[k + 1] - toff[k]);
  DevBuf ring;
  ring.alloc(slot_trip * kRing * sizeof(lfg_triplet), s);
  cudaStream_t cs = nullptr;
  cudaEvent_t assembled[kRing] = {}, copied[kRing] = {};
  auto release = [&]() {
    if (cs) cudaStreamSynchronize(cs);
    for (int i = 0; i < kRing; ++i) {
      if (assembled[i]) cudaEventDestroy(assembled[i]);
      if (copied[i]) cudaEventDestroy(copied[i]);
    }
    if (cs) cudaStreamDestroy(cs);
  };
  try {
    LFG_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    for (int i = 0; i < kRing; ++i) {
      LFG_CUDA(cudaEventCreateWithFlags(&assembled[i], cudaEventDisableTiming));
      LFG_CUDA(cudaEventCreateWithFlags(&copied[i], cudaEventDisableTiming));
    }
    for (int64_t k = 0; k < nchunk; ++k) {
      const int slot = static_cast<int>(k % kRing);
      lfg_triplet* buf = ring.as<lfg_triplet>() + slot * slot_trip;
      if (k >= kRing) LFG_CUDA(cudaStreamWaitEvent(s, copied[slot], 0));  // the slot's last download is done
      const int64_t lo = bound[k], hi = bound[k + 1];
      const auto& tl = m->h_tria_list;
      const auto& ql = m->h_quad_list;
      const int64_t t0 = std::lower_bound(tl.begin(), tl.end(), lo) - tl.begin();
      const int64_t t1 = std::lower_bound(tl.begin(), tl.end(), hi) - tl.begin();
      const int64_t q0 = std::lower_bound(ql.begin(), ql.end(), lo) - ql.begin();
      const int64_t q1 = std::lower_bound(ql.begin(), ql.end(), hi) - ql.begin();
      // cell c of the range writes at out + tri_offset[c]; out sits toff[k]
      // triplets before the slot, so every store lands inside the slot
      AssembleRDCells(sp, pr, buf - toff[k], t0, t1, q0, q1);
      LFG_CUDA(cudaEventRecord(assembled[slot], s));
      LFG_CUDA(cudaStreamWaitEvent(cs, assembled[slot], 0));
      LFG_CUDA(cudaMemcpyAsync(host + toff[k], buf, (toff[k + 1] - toff[k]) * sizeof(lfg_triplet),
                               cudaMemcpyDeviceToHost, cs));
      LFG_CUDA(cudaEventRecord(copied[slot], cs));
    }
    LFG_CUDA(cudaStreamSynchronize(cs));
    LFG_CUDA(cudaStreamSynchronize(s));
  } catch (...) {
    release();
    throw;
  }
  release();
  if (count) *count = sp->num_triplets;
  LFG_API_END
}

lfg_status lfg_assemble_vector_load(lfg_space* sp, const lfg_load_provider* pr, double* b) {
  if (!sp) return LFG_INVALID_ARG;
  LFG_API_BEGIN(sp->mesh->ctx)
  if (!pr || !b) Fail(LFG_INVALID_ARG, "lfg_assemble_vector_load: null argument");
  if (sp->hier_degree > 0) {
    HierAssembleVector(sp, pr, b);
    return LFG_OK;
  }
  if (sp->degree < 1) Fail(LFG_UNSUPPORTED, "load provider needs a Lagrangian space");
  lfg_ctx* ctx = sp->mesh->ctx;
  EnsureIncidence(sp);
  LoadElementVectors(sp, pr, sp->scratch_vec.as<double>());
  GatherVectorKernel<<<GridFor(ctx, sp->num_dofs, 256), 256, 0, ctx->stream>>>(
      sp->num_dofs, sp->inc_ptr.as<int64_t>(), sp->inc_slot.as<uint64_t>(), sp->scratch_vec.as<double>(), b);
  LFG_LAUNCHED(ctx);
  LFG_API_END
}

}  // extern "C"

namespace lfg {
void GatherElementVectors(lfg_space* sp, double* b) {
  lfg_ctx* ctx = sp->mesh->ctx;
  GatherVectorKernel<<<GridFor(ctx, sp->num_dofs, 256), 256, 0, ctx->stream>>>(
      sp->num_dofs, sp->inc_ptr.as<int64_t>(), sp->inc_slot.as<uint64_t>(), sp->scratch_vec.as<double>(), b);
  LFG_LAUNCHED(ctx);
}
}  // namespace lfg

extern "C" {

lfg_status lfg_assemble_matrix_tabulated(lfg_space* sp, const double* elem, int32_t ld, lfg_coo* coo) {
  if (!sp) return LFG_INVALID_ARG;
  LFG_API_BEGIN(sp->mesh->ctx)
  if (!elem || !coo || ld < sp->n_cell) Fail(LFG_INVALID_ARG, "lfg_assemble_matrix_tabulated: bad argument");
  if (coo->rows < sp->num_dofs || coo->cols < sp->num_dofs)
    Fail(LFG_INVALID_ARG, "COO matrix smaller than the number of dofs");
  if (coo->size + sp->num_triplets > coo->capacity) Fail(LFG_CAPACITY, "COO capacity too small");
  lfg_ctx* ctx = sp->mesh->ctx;
  TabulatedMatrixKernel<<<GridFor(ctx, sp->mesh->nc, 128), 128, 0, ctx->stream>>>(
      sp->mesh->nc, sp->mesh->cell_nodes.as<int4>(), sp->cell_dofs.as<int32_t>(), sp->n_cell, sp->n_tria,
      sp->n_quad, elem, ld, sp->tri_offset.as<int64_t>(), coo->d + coo->size);
  LFG_LAUNCHED(ctx);
  coo->size += sp->num_triplets;
  LFG_API_END
}

lfg_status lfg_assemble_vector_tabulated(lfg_space* sp, const double* vec, int32_t ld, double* b) {
  if (!sp) return LFG_INVALID_ARG;
  LFG_API_BEGIN(sp->mesh->ctx)
  if (!vec || !b || ld < sp->n_cell) Fail(LFG_INVALID_ARG, "lfg_assemble_vector_tabulated: bad argument");
  lfg_ctx* ctx = sp->mesh->ctx;
  EnsureIncidence(sp);
  TabulatedVectorKernel<<<GridFor(ctx, sp->mesh->nc, 128), 128, 0, ctx->stream>>>(
      sp->mesh->nc, sp->loc_offset.as<int64_t>(), vec, ld, sp->scratch_vec.as<double>());
  LFG_LAUNCHED(ctx);
  GatherVectorKernel<<<GridFor(ctx, sp->num_dofs, 256), 256, 0, ctx->stream>>>(
      sp->num_dofs, sp->inc_ptr.as<int64_t>(), sp->inc_slot.as<uint64_t>(), sp->scratch_vec.as<double>(), b);
  LFG_LAUNCHED(ctx);
  LFG_API_END
}

lfg_status lfg_loss_l2_misfit(lfg_ctx* ctx, int64_t n, const double* u, const double* u_obs, double* loss,
                              double* misfit) {
  if (!ctx) return LFG_INVALID_ARG;
  LFG_API_BEGIN(ctx)
  if (n < 0 || (n > 0 && (!u || !u_obs)) || !loss) Fail(LFG_INVALID_ARG, "lfg_loss_l2_misfit: bad argument");
  const int64_t parts = n == 0 ? 1 : (n + kMisfitChunk - 1) / kMisfitChunk;
  DevBuf part;
  part.alloc((parts + 1) * sizeof(double), ctx->stream);
  double* p = part.as<double>();
  if (n == 0) {
    LFG_CUDA(cudaMemsetAsync(p, 0, sizeof(double), ctx->stream));
  } else {
    ProfScope prof(ctx, "misfit");
    MisfitKernel<<<static_cast<unsigned>(parts), 256, 0, ctx->stream>>>(n, u, u_obs, misfit, p);
    LFG_LAUNCHED(ctx);
  }
  SumPartsKernel<<<1, 256, 0, ctx->stream>>>(parts, p, 0.5, p + parts);
  LFG_LAUNCHED(ctx);
  D2HSync(ctx, loss, p + parts, sizeof(double));
  LFG_API_END
}

lfg_status lfg_grad_rd_cellwise(lfg_space* sp, const lfg_rd_provider* pr, const double* u, const double* lam,
                                const uint8_t* flags, double* grad) {
  if (!sp) return LFG_INVALID_ARG;
  LFG_API_BEGIN(sp->mesh->ctx)
  GradRDCellwise(sp, pr, u, lam, flags, 1.0, grad);
  LFG_API_END
}

}  // extern "C"

namespace lfg {
namespace {

EdgeRule MakeEdgeRule(int degree, int qr_degree) {
  std::vector<double> t, w, phi;
  if (qr_degree > 30 || !SegmentTables(degree, qr_degree, t, w, phi))
    Fail(LFG_UNSUPPORTED, "edge provider: segment rule of degree " + std::to_string(qr_degree) + " not available");
  EdgeRule r{};
  r.nq = static_cast<int>(t.size());
  r.n = degree + 1;
  for (int k = 0; k < r.nq; ++k) {
    r.t[k] = t[k];
    r.w[k] = w[k];
    for (int i = 0; i < r.n; ++i) r.phi[k * r.n + i] = phi[k * r.n + i];
  }
  return r;
}

// Per-edge output offsets (prefix of `per` over the active edges); returns
// the total.  Without flags the offsets are e * per and off stays empty.
int64_t EdgeOffsets(lfg_ctx* ctx, lfg_mesh* m, const uint8_t* flags, int64_t per, DevBuf& off) {
  if (!flags) return m->ne * per;
  off.alloc((m->ne + 1) * sizeof(int64_t), ctx->stream);
  EdgeCountKernel<<<GridFor(ctx, m->ne, 256), 256, 0, ctx->stream>>>(m->ne, flags, per, off.as<int64_t>());
  LFG_LAUNCHED(ctx);
  return ExclusiveScanI64(ctx, off.as<int64_t>(), off.as<int64_t>(), m->ne);
}

EdgeArgs BaseEdgeArgs(lfg_space* sp, const lfg_coeff& f, const uint8_t* flags, const char* what) {
  lfg_mesh* m = sp->mesh;
  if (sp->degree < 1) Fail(LFG_UNSUPPORTED, std::string(what) + ": needs a Lagrangian space");
  if (f.kind == LFG_COEFF_ZERO || f.kind == LFG_COEFF_CONSTANT || f.kind == LFG_COEFF_PER_CELL ||
      f.kind == LFG_COEFF_PER_CELL_EXP || f.kind == LFG_COEFF_NODAL_O1 || f.kind == LFG_COEFF_ANALYTIC) {
  } else {
    Fail(LFG_UNSUPPORTED, std::string(what) + ": unsupported coefficient kind");
  }
  EdgeArgs a{};
  a.ne = m->ne;
  a.edges = m->edge_nodes.as<int2>();
  a.xy = m->xy.as<double2>();
  a.flags = flags;
  a.np = sp->np;
  a.ns = sp->ns;
  a.node_dofs = m->nv * sp->np;
  a.f = ToDev(f, m, what);
  return a;
}

}  // namespace
}  // namespace lfg

extern "C" {

lfg_status lfg_assemble_matrix_edge_mass(lfg_space* sp, const lfg_edge_mass_provider* pr, lfg_coo* coo) {
  if (!sp) return LFG_INVALID_ARG;
  LFG_API_BEGIN(sp->mesh->ctx)
  if (!pr || !coo) Fail(LFG_INVALID_ARG, "lfg_assemble_matrix_edge_mass: null argument");
  if (coo->rows < sp->num_dofs || coo->cols < sp->num_dofs)
    Fail(LFG_INVALID_ARG, "COO matrix smaller than the number of dofs");
  lfg_ctx* ctx = sp->mesh->ctx;
  EdgeArgs a = BaseEdgeArgs(sp, pr->gamma, pr->edge_flags_dev, "edge mass");
  const EdgeRule r = MakeEdgeRule(sp->degree, pr->qr_degree > 0 ? pr->qr_degree : 2 * sp->degree);
  const int64_t n = 2 * sp->np + sp->ns;
  a.stride = n * n;
  DevBuf off;
  const int64_t total = EdgeOffsets(ctx, sp->mesh, pr->edge_flags_dev, n * n, off);
  if (coo->size + total > coo->capacity)
    Fail(LFG_CAPACITY, "COO capacity " + std::to_string(coo->capacity) + " < " + std::to_string(coo->size + total));
  a.offset = pr->edge_flags_dev ? off.as<int64_t>() : nullptr;
  if (a.ne > 0) {
    ProfScope prof(ctx, "edge_mass");
    EdgeMassKernel<<<GridFor(ctx, a.ne, 128), 128, 0, ctx->stream>>>(a, r, coo->d + coo->size);
    LFG_LAUNCHED(ctx);
  }
  coo->size += total;
  LFG_CUDA(cudaStreamSynchronize(ctx->stream));  // `off` is freed on return
  LFG_API_END
}

lfg_status lfg_assemble_vector_edge_load(lfg_space* sp, const lfg_edge_load_provider* pr, double* b) {
  if (!sp) return LFG_INVALID_ARG;
  LFG_API_BEGIN(sp->mesh->ctx)
  if (!pr || !b) Fail(LFG_INVALID_ARG, "lfg_assemble_vector_edge_load: null argument");
  lfg_ctx* ctx = sp->mesh->ctx;
  cudaStream_t s = ctx->stream;
  EdgeArgs a = BaseEdgeArgs(sp, pr->g, pr->edge_flags_dev, "edge load");
  const EdgeRule r = MakeEdgeRule(sp->degree, pr->qr_degree > 0 ? pr->qr_degree : 2 * sp->degree);
  const int64_t n = 2 * sp->np + sp->ns;
  a.stride = n;
  DevBuf off;
  const int64_t total = EdgeOffsets(ctx, sp->mesh, pr->edge_flags_dev, n, off);
  if (total >= (int64_t(1) << 32)) Fail(LFG_UNSUPPORTED, "more than 2^32 edge contributions");
  a.offset = pr->edge_flags_dev ? off.as<int64_t>() : nullptr;
  if (total > 0) {
    ProfScope prof(ctx, "edge_load");
    DevBuf ev, key, slot;
    ev.alloc(total * sizeof(double), s);
    key.alloc(total * sizeof(uint64_t), s);
    slot.alloc(total * sizeof(uint32_t), s);
    EdgeLoadKernel<<<GridFor(ctx, a.ne, 128), 128, 0, s>>>(a, r, ev.as<double>(), key.as<uint64_t>(),
                                                          slot.as<uint32_t>());
    LFG_LAUNCHED(ctx);
    int bits = 1;
    while ((int64_t(1) << bits) < sp->num_dofs + 1) ++bits;
    RadixSortPairs(ctx, key.as<uint64_t>(), slot.as<uint32_t>(), total, bits);
    EdgeGatherKernel<<<GridFor(ctx, total, 256), 256, 0, s>>>(total, key.as<uint64_t>(), slot.as<uint32_t>(),
                                                             ev.as<double>(), b);
    LFG_LAUNCHED(ctx);
    LFG_CUDA(cudaStreamSynchronize(s));
  }
  LFG_API_END
}

}  // extern "C"
