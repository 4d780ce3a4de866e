// Hierarchic (hp) FE of uniform degree p on the device: element matrices of
// fe::DiffusionElementMatrixProvider + fe::MassElementMatrixProvider
// (fe/loc_comp_ellbvp.h:169-214, 349-378) and element vectors of
// fe::ScalarLoadElementVectorProvider (:642-685) over a HierarchicScalarFESpace
// (fe/hierarchic_scalar_fe_space.h), assembled in AssembleMatrixLocally /
// AssembleVectorLocally order (bit-exact indices, FP64 values).
//
// The shape functions of a hierarchic cell depend on the relative
// orientation of its edges (fe/hierarchic_fe.h: reversed edge coordinate and
// reversed slots for a negatively oriented edge; the triangle's interior
// functions follow edge 0).  All 2^3 (triangle) or 2^4 (quadrilateral)
// orientation patterns are tabulated once on the host; a cell selects its
// table block by the orientation bits the mesh stores per cell.
//
// Kernels:
//  - affine triangles with cell-constant coefficients: the point sum is
//    folded into R_pat(i,j) = sum_k w_k {g_i0 g_j0, g_i0 g_j1 + g_i1 g_j0,
//    g_i1 g_j1, phi_i phi_j}, so an entry costs 4 FMAs; each CTA takes a tile
//    of cells, computes the upper triangle of every element matrix into
//    shared memory, then writes the n^2 triplets of each cell row-major with
//    coalesced 16-byte stores;
//  - everything else (quadrilaterals, point-varying coefficients): per cell
//    the per-point metric and coefficients go to shared memory, then every
//    (i, j) entry sums over the rule points.
#include <algorithm>
#include <string>
#include <vector>

#include "lfg_api.h"
#include "lfg_coeff.h"
#include "lfg_df32.h"
#include "lfg_elem.h"
#include "lfg_internal.h"

namespace lfg {
namespace {

constexpr int kHierBlock = 128;

// Table block (doubles): w[nq] | x[nq] | y[nq] | then per pattern:
//   phi[nq][n] | g[nq][n][2] | R[E][4] | R32[E][4] (binary32 pairs, one
//   double slot each)
struct HierTab {
  int n = 0, nq = 0, E = 0, npat = 0;
  int64_t off_pat = 0, stride = 0, o_g = 0, o_R = 0, o_R32 = 0, total = 0;
};

// Every block starts on a multiple of 4 doubles (32 bytes), so the vector
// loads of the kernels (16 bytes) stay aligned.
int64_t Pad4(int64_t x) { return (x + 3) & ~int64_t(3); }

HierTab HierLayout(bool quad, int n, int nq, bool folded) {
  HierTab t;
  t.n = n;
  t.nq = nq;
  t.E = n * (n + 1) / 2;
  t.npat = quad ? 16 : 8;
  t.off_pat = Pad4(3 * static_cast<int64_t>(nq));
  t.o_g = Pad4(static_cast<int64_t>(nq) * n);
  t.o_R = Pad4(t.o_g + 2 * static_cast<int64_t>(nq) * n);
  const int64_t eb = folded ? 4 * static_cast<int64_t>(t.E) : 0;  // folded sums only when requested
  t.o_R32 = Pad4(t.o_R + eb);
  t.stride = Pad4(t.o_R32 + eb);
  t.total = t.off_pat + t.npat * t.stride;
  return t;
}

void FillHierTable(bool quad, int p, const Rule& r, bool folded, std::vector<double>& h, HierTab& L);

void BuildHierTable(bool quad, int p, int rule_degree, bool folded, std::vector<double>& h, HierTab& L) {
  Rule r;
  if (!MakeRule(quad, rule_degree, r))
    Fail(LFG_UNSUPPORTED, "no quadrature rule of degree " + std::to_string(rule_degree));
  FillHierTable(quad, p, r, folded, h, L);
}

void FillHierTable(bool quad, int p, const Rule& r, bool folded, std::vector<double>& h, HierTab& L) {
  const int n = quad ? (p + 1) * (p + 1) : (p + 1) * (p + 2) / 2;
  L = HierLayout(quad, n, r.n, folded);
  h.assign(static_cast<size_t>(L.total), 0.0);
  for (int k = 0; k < r.n; ++k) {
    h[k] = r.w[k];
    h[r.n + k] = r.x[k];
    h[2 * r.n + k] = r.y[k];
  }
  std::vector<double> phi(n), dphi(2 * n);
  for (int pat = 0; pat < L.npat; ++pat) {
    double* B = h.data() + L.off_pat + pat * L.stride;
    for (int k = 0; k < r.n; ++k) {
      HierShape(quad, p, pat, r.x[k], r.y[k], phi.data(), reinterpret_cast<double(*)[2]>(dphi.data()));
      for (int i = 0; i < n; ++i) {
        B[static_cast<int64_t>(k) * n + i] = phi[i];
        B[L.o_g + (static_cast<int64_t>(k) * n + i) * 2] = dphi[2 * i];
        B[L.o_g + (static_cast<int64_t>(k) * n + i) * 2 + 1] = dphi[2 * i + 1];
      }
    }
    if (!folded) continue;
    // folded sums in long double, upper triangle row by row (used for affine
    // cells: triangles and parallelograms)
    int64_t e = 0;
    for (int i = 0; i < n; ++i)
      for (int j = i; j < n; ++j, ++e) {
        long double s0 = 0, s1 = 0, s2 = 0, s3 = 0;
        for (int k = 0; k < r.n; ++k) {
          const long double w = r.w[k];
          const double* g = B + L.o_g + static_cast<int64_t>(k) * n * 2;
          const double* f = B + static_cast<int64_t>(k) * n;
          s0 += w * g[2 * i] * g[2 * j];
          s1 += w * (static_cast<long double>(g[2 * i]) * g[2 * j + 1] + static_cast<long double>(g[2 * i + 1]) * g[2 * j]);
          s2 += w * g[2 * i + 1] * g[2 * j + 1];
          s3 += w * f[i] * f[j];
        }
        double* R = B + L.o_R + 4 * e;
        R[0] = static_cast<double>(s0);
        R[1] = static_cast<double>(s1);
        R[2] = static_cast<double>(s2);
        R[3] = static_cast<double>(s3);
        float* R32 = reinterpret_cast<float*>(B + L.o_R32 + 4 * e);
        const long double sv[4] = {s0, s1, s2, s3};
        for (int q = 0; q < 4; ++q) {
          const float hi = static_cast<float>(sv[q]);
          R32[2 * q] = hi;
          R32[2 * q + 1] = static_cast<float>(sv[q] - static_cast<long double>(hi));
        }
      }
  }
}

// Cached on the context per (cell type, degree, rule degree, with or without
// the folded sums of the affine kernel).
const double* GetHierTable(lfg_ctx* ctx, bool quad, int p, int rule_degree, bool folded, HierTab& L) {
  const int key = (1 << 23) | (folded ? 1 << 24 : 0) | (quad ? 1 << 20 : 0) | (p << 10) | rule_degree;
  auto it = ctx->tables.find(key);
  if (it == ctx->tables.end()) {
    std::vector<double> h;
    BuildHierTable(quad, p, rule_degree, folded, h, L);
    TableEntry& ent = ctx->tables[key];
    ent.layout = Tab{};
    ent.layout.n = L.n;
    ent.layout.nq = L.nq;
    ent.buf.alloc(h.size() * sizeof(double), ctx->stream);
    LFG_CUDA(cudaMemcpyAsync(ent.buf.p, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    LFG_CUDA(cudaStreamSynchronize(ctx->stream));
    return ent.buf.as<double>();
  }
  L = HierLayout(quad, it->second.layout.n, it->second.layout.nq, folded);
  return it->second.buf.as<double>();
}

// Division by a run-time constant d without a hardware divide:
// q / d = (q * m) >> 40 with m = 2^40 / d + 1, exact whenever q * d < 2^40
// (the error q (m - 2^40/d) / 2^40 < q / 2^40 < 1/d stays below the gap
// between q/d and the next integer).
struct FastDiv {
  uint64_t m = 1;
  int d = 1;
};
FastDiv MakeFastDiv(int d) {
  FastDiv f;
  f.d = d;
  f.m = (uint64_t(1) << 40) / static_cast<uint64_t>(d) + 1;
  return f;
}
__device__ __forceinline__ int Div(int q, const FastDiv& f) {
  return static_cast<int>((static_cast<uint64_t>(q) * f.m) >> 40);
}

struct HierArgs {
  const int32_t* list;  // cells of one type, ascending
  int64_t count;
  const int4* cells;
  const double2* xy;
  const uint8_t* ori;   // bit j: local edge j negatively oriented
  const int32_t* cell_dofs;
  int n_cell;
  const int64_t* tri_offset;
  lfg_triplet* out;
  const double* tab;
  HierTab L;
  CoeffDev alpha, gamma;
  unsigned long long* fallback;  // cells whose coefficients left the df32 range (FP64 route)
  FastDiv div_n, div_E, div_nn;  // by n, E = n(n+1)/2 and n^2
  // per-entity degrees: the cell's local shape function s is slot
  // sel[c * n_cell + s] of the degree-D table; its count is
  // loc_offset[c + 1] - loc_offset[c]
  const uint16_t* sel;
  const int64_t* loc_offset;
};

__device__ __forceinline__ void StoreTriplet(lfg_triplet* p, int r, int c, double v) {
  const long long bits = __double_as_longlong(v);
  *reinterpret_cast<int4*>(p) = make_int4(r, c, static_cast<int>(bits & 0xffffffffll), static_cast<int>(bits >> 32));
}

// |det J| J^{-1} J^{-T} (= adj(J) adj(J)^T / |det J|), |det J| and Global()
// at a reference point of a TriaO1 / QuadO1 cell.
template <bool QUAD>
__device__ __forceinline__ void Metric(const double2 (&v)[4], double xh, double yh, double& m00, double& m01,
                                       double& m11, double& adet, double& X, double& Y) {
  double j00, j01, j10, j11;
  if (!QUAD) {
    j00 = v[1].x - v[0].x; j01 = v[2].x - v[0].x;
    j10 = v[1].y - v[0].y; j11 = v[2].y - v[0].y;
    const double l0 = 1.0 - xh - yh;
    X = v[0].x * l0 + v[1].x * xh + v[2].x * yh;
    Y = v[0].y * l0 + v[1].y * xh + v[2].y * yh;
  } else {
    j00 = (v[1].x - v[0].x) * (1 - yh) + (v[2].x - v[3].x) * yh;
    j10 = (v[1].y - v[0].y) * (1 - yh) + (v[2].y - v[3].y) * yh;
    j01 = (v[3].x - v[0].x) * (1 - xh) + (v[2].x - v[1].x) * xh;
    j11 = (v[3].y - v[0].y) * (1 - xh) + (v[2].y - v[1].y) * xh;
    const double b0 = (1 - xh) * (1 - yh), b1 = xh * (1 - yh), b2 = xh * yh, b3 = (1 - xh) * yh;
    X = v[0].x * b0 + v[1].x * b1 + v[2].x * b2 + v[3].x * b3;
    Y = v[0].y * b0 + v[1].y * b1 + v[2].y * b2 + v[3].y * b3;
  }
  const double det = j00 * j11 - j10 * j01;
  adet = fabs(det);
  const double inv = 1.0 / adet;
  m00 = (j11 * j11 + j01 * j01) * inv;
  m01 = -(j11 * j10 + j01 * j00) * inv;
  m11 = (j10 * j10 + j00 * j00) * inv;
}

__device__ __forceinline__ double CellConstant(const CoeffDev& f, int c) {
  switch (f.kind) {
    case LFG_COEFF_CONSTANT: return f.value;
    case LFG_COEFF_PER_CELL: return f.data[c];
    case LFG_COEFF_PER_CELL_EXP: return exp(f.data[c]);
  }
  return 0.0;
}

template <bool QUAD>
__device__ __forceinline__ void LoadVerts(const HierArgs& a, int c, int4& cn, double2 (&v)[4]) {
  cn = a.cells[c];
  v[0] = a.xy[cn.x];
  v[1] = a.xy[cn.y];
  v[2] = a.xy[cn.z];
  v[3] = QUAD ? a.xy[cn.w] : make_double2(0.0, 0.0);
}

// Affine cells (triangles; parallelogram quadrilaterals), cell-constant
// alpha / gamma: tiles of T cells per CTA.  The four per-cell coefficients
// c = {alpha m00, alpha m01, alpha m11, gamma |det J|} are formed in FP64 and
// each upper-triangle entry c . R_pat(e) is contracted in df32 on the FP32
// pipes (4 error-free products, one FP64 add to convert), so the FP64 pipe
// does about half an operation per triplet; a cell whose coefficients leave
// the df32 range [2^-40, 2^40] is contracted in FP64 instead.
// Shared memory: vals[T][E] | coef[T][4] | coef32[T][4] | base[T] | pat[T] |
// cid[T] | safe[T] | dofs[T][n] | (VAR) nloc[T] | sel[T][n] | ent[T + 1] |
// trip[T + 1].  With VAR the cells have their own shape-function subsets of
// the degree-D table: cell t contracts only the m(m+1)/2 table entries its
// m = nloc[t] functions pair up (ent: their prefix over the tile) and writes
// its m^2 triplets consecutively (trip: their prefix), both as flat work
// lists over the tile.
template <bool QUAD, bool MASS, bool VAR>
__global__ void __launch_bounds__(kHierBlock) HierAffineKernel(HierArgs a, int T) {
  using namespace df;
  extern __shared__ __align__(16) double smem[];
  const int n = a.L.n, E = a.L.E, nn = n * n;
  double* vals = smem;
  double* coef = vals + static_cast<int64_t>(T) * E;
  f2* coef32 = reinterpret_cast<f2*>(coef + 4 * T);
  int64_t* base = reinterpret_cast<int64_t*>(coef32 + 4 * T);
  int* pat = reinterpret_cast<int*>(base + T);
  int* cid = pat + T;
  int* safe = cid + T;
  int* dofs = safe + T;
  int* nl = dofs + T * n;
  uint16_t* ss = reinterpret_cast<uint16_t*>(nl + T);
  int* ent = reinterpret_cast<int*>(ss + ((T * n + 1) & ~1));  // 4-byte aligned after the uint16 block
  int* trip = ent + T + 1;
  for (int64_t t0 = static_cast<int64_t>(blockIdx.x) * T; t0 < a.count; t0 += static_cast<int64_t>(gridDim.x) * T) {
    const int tn = static_cast<int>(min(static_cast<int64_t>(T), a.count - t0));
    for (int t = threadIdx.x; t < tn; t += blockDim.x) {
      const int c = a.list[t0 + t];
      const int4 cn = a.cells[c];
      const double2 v0 = a.xy[cn.x], v1 = a.xy[cn.y], v2 = a.xy[QUAD ? cn.w : cn.z];
      // affine map with columns v1 - v0 and (v2 or v3) - v0
      const double j00 = v1.x - v0.x, j01 = v2.x - v0.x, j10 = v1.y - v0.y, j11 = v2.y - v0.y;
      const double det = j00 * j11 - j10 * j01;
      const double adet = fabs(det), inv = 1.0 / adet;
      const double al = CellConstant(a.alpha, c), ga = MASS ? CellConstant(a.gamma, c) : 0.0;
      double cf[4];
      cf[0] = (j11 * j11 + j01 * j01) * inv * al;
      cf[1] = -(j11 * j10 + j01 * j00) * inv * al;
      cf[2] = (j10 * j10 + j00 * j00) * inv * al;
      cf[3] = adet * ga;
      bool ok = true;
      for (int q = 0; q < 4; ++q) {
        coef[4 * t + q] = cf[q];
        coef32[4 * t + q] = FromDouble(cf[q]);
        ok = ok && elem::DfSafe(cf[q]);
      }
      safe[t] = ok;
      if (!ok) atomicAdd(a.fallback, 1ull);
      base[t] = a.tri_offset[c];
      pat[t] = a.ori[c] & (QUAD ? 15 : 7);
      cid[t] = c;
      if (VAR) nl[t] = static_cast<int>(a.loc_offset[c + 1] - a.loc_offset[c]);
    }
    __syncthreads();
    if (VAR && threadIdx.x == 0) {
      ent[0] = trip[0] = 0;
      for (int t = 0; t < tn; ++t) {
        ent[t + 1] = ent[t] + nl[t] * (nl[t] + 1) / 2;
        trip[t + 1] = trip[t] + nl[t] * nl[t];
      }
    }
    for (int idx = threadIdx.x; idx < tn * n; idx += blockDim.x) {
      const int t = Div(idx, a.div_n), i = idx - t * n;
      dofs[idx] = a.cell_dofs[static_cast<int64_t>(cid[t]) * a.n_cell + i];
      if (VAR) ss[idx] = a.sel[static_cast<int64_t>(cid[t]) * a.n_cell + i];
    }
    if (VAR) __syncthreads();
    const int nwork = VAR ? ent[tn] : tn * E;
    for (int idx = threadIdx.x; idx < nwork; idx += blockDim.x) {
      int t, e;
      if (VAR) {
        // cell of work item idx, then its pair (i <= j) in row-major upper order
        int lo = 0, hi = tn - 1;
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if (ent[mid] <= idx) lo = mid;
          else hi = mid - 1;
        }
        t = lo;
        const int m = nl[t], k = idx - ent[t];
        const float b2 = 2.0f * m + 1.0f;
        int i = static_cast<int>((b2 - sqrtf(b2 * b2 - 8.0f * static_cast<float>(k))) * 0.5f);
        i = max(0, min(i, m - 1));
        while (i > 0 && i * m - ((i * (i - 1)) >> 1) > k) --i;
        while (i + 1 < m && (i + 1) * m - (((i + 1) * i) >> 1) <= k) ++i;
        const int j = i + (k - (i * m - ((i * (i - 1)) >> 1)));
        const int ui = ss[t * n + i], uj = ss[t * n + j];
        const int u0 = min(ui, uj), u1 = max(ui, uj);
        e = u0 * n - ((u0 * (u0 - 1)) >> 1) + (u1 - u0);
      } else {
        t = Div(idx, a.div_E);
        e = idx - t * E;
      }
      const int vidx = t * E + e;
      const double* blk = a.tab + a.L.off_pat + pat[t] * a.L.stride;
      if (safe[t]) {
        const float4 r01 = *reinterpret_cast<const float4*>(blk + a.L.o_R32 + 4 * static_cast<int64_t>(e));
        const float4 r23 = *reinterpret_cast<const float4*>(blk + a.L.o_R32 + 4 * static_cast<int64_t>(e) + 2);
        const f2* cf = coef32 + 4 * t;
        Acc acc;
        acc.AddProd(cf[0], f2{r01.x, r01.y});
        acc.AddProd(cf[1], f2{r01.z, r01.w});
        acc.AddProd(cf[2], f2{r23.x, r23.y});
        if (MASS) acc.AddProd(cf[3], f2{r23.z, r23.w});
        vals[vidx] = ToDouble(acc.Value());
      } else {
        const double* R = blk + a.L.o_R + 4 * static_cast<int64_t>(e);
        const double* cf = coef + 4 * t;
        vals[vidx] = cf[0] * R[0] + cf[1] * R[1] + cf[2] * R[2] + cf[3] * R[3];
      }
    }
    __syncthreads();
    const int nwrite = VAR ? trip[tn] : tn * nn;
    for (int q = threadIdx.x; q < nwrite; q += blockDim.x) {
      if (VAR) {
        int lo = 0, hi = tn - 1;
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if (trip[mid] <= q) lo = mid;
          else hi = mid - 1;
        }
        const int t = lo, m = nl[t], rr = q - trip[t];
        const int i = rr / m, j = rr - i * m;
        const int ui = ss[t * n + i], uj = ss[t * n + j];
        const int u0 = min(ui, uj), u1 = max(ui, uj);
        const int e = u0 * n - ((u0 * (u0 - 1)) >> 1) + (u1 - u0);
        StoreTriplet(a.out + base[t] + rr, dofs[t * n + i], dofs[t * n + j], vals[t * E + e]);
      } else {
        const int t = Div(q, a.div_nn), rr = q - t * nn;
        const int i = Div(rr, a.div_n), j = rr - i * n;
        const int lo = min(i, j), hi = max(i, j);
        const int e = lo * n - ((lo * (lo - 1)) >> 1) + (hi - lo);
        StoreTriplet(a.out + base[t] + rr, dofs[t * n + i], dofs[t * n + j], vals[t * E + e]);
      }
    }
    __syncthreads();
  }
}

// Quadrilaterals that are not parallelograms (their element map is bilinear):
// count[0] += 1 per such cell.
__global__ void NonAffineQuadsKernel(int64_t nq, const int32_t* __restrict__ list, const int4* __restrict__ cells,
                                     const double2* __restrict__ xy, unsigned long long* __restrict__ count) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < nq;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int4 cn = cells[list[i]];
    const double2 v0 = xy[cn.x], v1 = xy[cn.y], v2 = xy[cn.z], v3 = xy[cn.w];
    const bool par = (v2.x - v3.x == v1.x - v0.x) && (v2.y - v3.y == v1.y - v0.y) &&
                     (v2.x - v1.x == v3.x - v0.x) && (v2.y - v1.y == v3.y - v0.y);
    if (!par) atomicAdd(count, 1ull);
  }
}

// General path: one cell per CTA iteration.  Shared memory: coef[nq][4] |
// (SYM) vals[E] | dofs[n] | (VAR) sel[n].  SYM computes each upper-triangle
// entry once into shared memory and writes both halves from there (half the
// FP64 work); without SYM (elements too large for shared memory) every (i, j)
// sums its own point loop.  With VAR a cell has m <= n shape functions, the
// degree-D table slots sel[0..m).
template <bool QUAD, bool SYM, bool VAR>
__global__ void __launch_bounds__(kHierBlock) HierGeneralKernel(HierArgs a) {
  extern __shared__ __align__(16) double smem[];
  const int n = a.L.n, nq = a.L.nq;
  double* coef = smem;
  double* vals = coef + 4 * nq;
  int* dofs = reinterpret_cast<int*>(vals + (SYM ? a.L.E : 0));
  uint16_t* ss = reinterpret_cast<uint16_t*>(dofs + n);
  const double* __restrict__ tab = a.tab;
  for (int64_t ci = blockIdx.x; ci < a.count; ci += gridDim.x) {
    const int c = a.list[ci];
    const int m = VAR ? static_cast<int>(a.loc_offset[c + 1] - a.loc_offset[c]) : n, mm = m * m;
    int4 cn;
    double2 v[4];
    LoadVerts<QUAD>(a, c, cn, v);
    const int pat = a.ori[c] & (QUAD ? 15 : 7);
    for (int k = threadIdx.x; k < nq; k += blockDim.x) {
      const double xh = tab[nq + k], yh = tab[2 * nq + k], w = tab[k];
      double m00, m01, m11, adet, X, Y;
      Metric<QUAD>(v, xh, yh, m00, m01, m11, adet, X, Y);
      const double al = EvalCoeffPoint(a.alpha, c, cn, QUAD, xh, yh, X, Y);
      const double ga = EvalCoeffPoint(a.gamma, c, cn, QUAD, xh, yh, X, Y);
      coef[4 * k + 0] = w * al * m00;
      coef[4 * k + 1] = w * al * m01;
      coef[4 * k + 2] = w * al * m11;
      coef[4 * k + 3] = w * adet * ga;
    }
    for (int i = threadIdx.x; i < m; i += blockDim.x) {
      dofs[i] = a.cell_dofs[static_cast<int64_t>(c) * a.n_cell + i];
      if (VAR) ss[i] = a.sel[static_cast<int64_t>(c) * a.n_cell + i];
    }
    __syncthreads();
    const double* P = tab + a.L.off_pat + pat * a.L.stride;
    const double* G = P + a.L.o_g;
    const int64_t base = a.tri_offset[c];
    for (int q = threadIdx.x; q < mm; q += blockDim.x) {
      const int si = q / m, sj = q - si * m;
      if (SYM && sj < si) continue;
      const int i = VAR ? ss[si] : si, j = VAR ? ss[sj] : sj;
      double acc = 0.0;
      for (int k = 0; k < nq; ++k) {
        const double2 gi = *reinterpret_cast<const double2*>(G + (static_cast<int64_t>(k) * n + i) * 2);
        const double2 gj = *reinterpret_cast<const double2*>(G + (static_cast<int64_t>(k) * n + j) * 2);
        const double* cf = coef + 4 * k;
        acc += cf[0] * (gi.x * gj.x) + cf[1] * (gi.x * gj.y + gi.y * gj.x) + cf[2] * (gi.y * gj.y) +
               cf[3] * (P[static_cast<int64_t>(k) * n + i] * P[static_cast<int64_t>(k) * n + j]);
      }
      if (SYM) vals[si * m - si * (si - 1) / 2 + (sj - si)] = acc;
      else StoreTriplet(a.out + base + q, dofs[si], dofs[sj], acc);
    }
    if (SYM) {
      __syncthreads();
      for (int q = threadIdx.x; q < mm; q += blockDim.x) {
        const int i = q / m, j = q - i * m;
        const int lo = min(i, j), hi = max(i, j);
        StoreTriplet(a.out + base + q, dofs[i], dofs[j], vals[lo * m - lo * (lo - 1) / 2 + (hi - lo)]);
      }
    }
    __syncthreads();
  }
}

// Element vectors: s_k = (w_k |det J_k|) f(x_k), v_i = sum_k s_k phi_i(x_k),
// into ev at the cell's local offset.  Shared memory: s[nq].
template <bool QUAD, bool VAR>
__global__ void __launch_bounds__(kHierBlock) HierLoadKernel(HierArgs a, CoeffDev f, const int64_t* loc_offset,
                                                            double* ev) {
  extern __shared__ __align__(16) double smem[];
  const int n = a.L.n, nq = a.L.nq;
  const double* __restrict__ tab = a.tab;
  for (int64_t ci = blockIdx.x; ci < a.count; ci += gridDim.x) {
    const int c = a.list[ci];
    int4 cn;
    double2 v[4];
    LoadVerts<QUAD>(a, c, cn, v);
    const int pat = a.ori[c] & (QUAD ? 15 : 7);
    for (int k = threadIdx.x; k < nq; k += blockDim.x) {
      const double xh = tab[nq + k], yh = tab[2 * nq + k];
      double m00, m01, m11, adet, X, Y;
      Metric<QUAD>(v, xh, yh, m00, m01, m11, adet, X, Y);
      smem[k] = (tab[k] * adet) * EvalCoeffPoint(f, c, cn, QUAD, xh, yh, X, Y);
    }
    __syncthreads();
    const double* P = tab + a.L.off_pat + pat * a.L.stride;
    const int64_t b = loc_offset[c];
    const int m = VAR ? static_cast<int>(loc_offset[c + 1] - b) : n;
    for (int si = threadIdx.x; si < m; si += blockDim.x) {
      const int i = VAR ? a.sel[static_cast<int64_t>(c) * a.n_cell + si] : si;
      double s = 0.0;
      for (int k = 0; k < nq; ++k) s += smem[k] * P[static_cast<int64_t>(k) * n + i];
      ev[b + si] = s;
    }
    __syncthreads();
  }
}

}  // namespace

const double* HierShapeTable(lfg_ctx* ctx, bool quad, int p, int rule_degree, HierTabView& v) {
  HierTab L;
  const double* t = GetHierTable(ctx, quad, p, rule_degree, false, L);
  v.n = L.n;
  v.nq = L.nq;
  v.off_pat = L.off_pat;
  v.stride = L.stride;
  v.o_g = L.o_g;
  return t;
}

void HierShapeTableAt(bool quad, int p, const std::vector<double>& x, const std::vector<double>& y,
                      std::vector<double>& h, HierTabView& v) {
  Rule r;
  r.n = static_cast<int>(x.size());
  r.x = x;
  r.y = y;
  r.w.assign(x.size(), 0.0);
  HierTab L;
  FillHierTable(quad, p, r, false, h, L);
  v.n = L.n;
  v.nq = L.nq;
  v.off_pat = L.off_pat;
  v.stride = L.stride;
  v.o_g = L.o_g;
}

int HierRuleDegree(int requested, int p) { return requested == 0 ? 2 * p : requested; }

bool CellConstantKind(const lfg_coeff& c) {
  return c.kind == LFG_COEFF_ZERO || c.kind == LFG_COEFF_CONSTANT || c.kind == LFG_COEFF_PER_CELL ||
         c.kind == LFG_COEFF_PER_CELL_EXP;
}

HierArgs BaseHierArgs(lfg_space* sp) {
  lfg_mesh* m = sp->mesh;
  HierArgs a{};
  a.cells = m->cell_nodes.as<int4>();
  a.xy = m->xy.as<double2>();
  a.ori = m->cell_ori.as<uint8_t>();
  a.cell_dofs = sp->cell_dofs.as<int32_t>();
  a.n_cell = sp->n_cell;
  a.tri_offset = sp->tri_offset.as<int64_t>();
  a.sel = sp->hier_var ? sp->hv_sel.as<uint16_t>() : nullptr;
  a.loc_offset = sp->loc_offset.as<int64_t>();
  return a;
}

template <class K>
int HierGrid(lfg_ctx* ctx, K kernel, size_t smem, int64_t work_items) {
  LFG_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
  int per_sm = 0;
  LFG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kHierBlock, smem));
  if (per_sm < 1) Fail(LFG_UNSUPPORTED, "hierarchic element too large for one CTA's shared memory");
  const int64_t g = std::min<int64_t>(work_items, static_cast<int64_t>(ctx->num_sms) * per_sm);
  return static_cast<int>(std::max<int64_t>(g, 1));
}

constexpr size_t kHierSmemLimit = 200 * 1024;

// Quadrilaterals of the mesh that are not parallelograms (counted once).
int64_t NonAffineQuads(lfg_mesh* m) {
  if (m->nonaffine_quads >= 0) return m->nonaffine_quads;
  lfg_ctx* ctx = m->ctx;
  DevBuf cnt;
  cnt.alloc(sizeof(unsigned long long), ctx->stream);
  LFG_CUDA(cudaMemsetAsync(cnt.p, 0, sizeof(unsigned long long), ctx->stream));
  if (m->nquad) {
    NonAffineQuadsKernel<<<GridFor(ctx, m->nquad, 256), 256, 0, ctx->stream>>>(
        m->nquad, m->quad_list.as<int32_t>(), m->cell_nodes.as<int4>(), m->xy.as<double2>(),
        cnt.as<unsigned long long>());
    LFG_LAUNCHED(ctx);
  }
  unsigned long long h = 0;
  D2HSync(ctx, &h, cnt.p, sizeof(h));
  m->nonaffine_quads = static_cast<int64_t>(h);
  return m->nonaffine_quads;
}

template <bool QUAD, bool VAR>
void LaunchAffine(lfg_ctx* ctx, const HierArgs& a, bool mass) {
  const int n = a.L.n, E = a.L.E;
  auto smem_for = [&](int t) {
    return static_cast<size_t>(t) * E * 8 + static_cast<size_t>(t) * (4 * 8 + 4 * 8 + 8 + 4 * 4) +
           static_cast<size_t>(t) * n * 4 +
           (VAR ? static_cast<size_t>(t) * 4 + ((static_cast<size_t>(t) * n + 1) & ~size_t(1)) * 2 +
                      2 * (static_cast<size_t>(t) + 1) * 4
                : 0);
  };
  int T = std::max(1, std::min(32, 4096 / (n * n)));
  while (T > 1 && smem_for(T) > 96 * 1024) --T;
  const size_t smem = smem_for(T);
  const int64_t tiles = (a.count + T - 1) / T;
  ProfScope prof(ctx, QUAD ? "hier_quad_affine" : "hier_tria_affine");
  if (mass) {
    const int grid = HierGrid(ctx, HierAffineKernel<QUAD, true, VAR>, smem, tiles);
    HierAffineKernel<QUAD, true, VAR><<<grid, kHierBlock, smem, ctx->stream>>>(a, T);
  } else {
    const int grid = HierGrid(ctx, HierAffineKernel<QUAD, false, VAR>, smem, tiles);
    HierAffineKernel<QUAD, false, VAR><<<grid, kHierBlock, smem, ctx->stream>>>(a, T);
  }
  LFG_LAUNCHED(ctx);
}

bool AffineFits(bool quad, int p, bool var) {
  const size_t n = quad ? (p + 1) * (p + 1) : (p + 1) * (p + 2) / 2;
  return n * (n + 1) / 2 * 8 + 96 + n * 4 + (var ? 4 + 2 * n + 16 : 0) <= kHierSmemLimit;
}

template <bool QUAD, bool VAR>
void LaunchGeneral(lfg_ctx* ctx, const HierArgs& a) {
  const size_t base = static_cast<size_t>(a.L.nq) * 32 + static_cast<size_t>(a.L.n) * (VAR ? 6 : 4);
  const size_t sym = base + static_cast<size_t>(a.L.E) * 8;
  ProfScope prof(ctx, QUAD ? "hier_general_quad" : "hier_general_tria");
  if (sym <= kHierSmemLimit) {
    const int grid = HierGrid(ctx, HierGeneralKernel<QUAD, true, VAR>, sym, a.count);
    HierGeneralKernel<QUAD, true, VAR><<<grid, kHierBlock, sym, ctx->stream>>>(a);
  } else {
    const int grid = HierGrid(ctx, HierGeneralKernel<QUAD, false, VAR>, base, a.count);
    HierGeneralKernel<QUAD, false, VAR><<<grid, kHierBlock, base, ctx->stream>>>(a);
  }
  LFG_LAUNCHED(ctx);
}

// The cells of one type (all of them, or one degree group of a
// variable-degree space) against the degree-p table.
template <bool QUAD, bool VAR>
void LaunchHierCells(lfg_ctx* ctx, HierArgs a, int p, int rule_degree, bool uniform, bool mass) {
  const bool affine = uniform && AffineFits(QUAD, p, VAR);
  a.tab = GetHierTable(ctx, QUAD, p, rule_degree, affine, a.L);
  a.div_n = MakeFastDiv(a.L.n);
  a.div_E = MakeFastDiv(a.L.n * (a.L.n + 1) / 2);
  a.div_nn = MakeFastDiv(a.L.n * a.L.n);
  if (affine) LaunchAffine<QUAD, VAR>(ctx, a, mass);
  else LaunchGeneral<QUAD, VAR>(ctx, a);
}

void HierAssembleMatrix(lfg_space* sp, const lfg_rd_provider* pr, lfg_coo* coo) {
  lfg_mesh* m = sp->mesh;
  lfg_ctx* ctx = m->ctx;
  const int p = sp->hier_degree;
  if (coo->rows < sp->num_dofs || coo->cols < sp->num_dofs)
    Fail(LFG_INVALID_ARG, "COO matrix smaller than the number of dofs");
  if (m->ntria && pr->qr_degree_tria < 0)
    Fail(LFG_MISSING_RULE, "No local shape function information or no quadrature rule for reference element type TRIA");
  if (m->nquad && pr->qr_degree_quad < 0)
    Fail(LFG_MISSING_RULE, "No local shape function information or no quadrature rule for reference element type QUAD");
  if (coo->size + sp->num_triplets > coo->capacity)
    Fail(LFG_CAPACITY, "COO capacity " + std::to_string(coo->capacity) + " < " +
                           std::to_string(coo->size + sp->num_triplets));
  HierArgs a = BaseHierArgs(sp);
  a.out = coo->d + coo->size;
  a.alpha = ToDev(pr->alpha, m, "alpha");
  a.gamma = ToDev(pr->gamma, m, "gamma");
  a.fallback = reinterpret_cast<unsigned long long*>(StatusWord(ctx) + 12);
  const bool uniform = CellConstantKind(pr->alpha) && CellConstantKind(pr->gamma);
  const bool mass = pr->gamma.kind != LFG_COEFF_ZERO;
  // the folded kernel serves quadrilaterals only when all are parallelograms
  const bool quad_uniform = uniform && m->nquad > 0 && NonAffineQuads(m) == 0;
  if (sp->hier_var) {
    // one launch per (cell type, degree D) group, D's table and rule 2 D
    // (2 * Degree(), fe/loc_comp_ellbvp.h:186) unless a rule degree is given
    for (const HierGroup& g : sp->hv_groups) {
      a.list = sp->hv_sorted.as<int32_t>() + g.start;
      a.count = g.count;
      if (g.quad)
        LaunchHierCells<true, true>(ctx, a, g.degree, HierRuleDegree(pr->qr_degree_quad, g.degree),
                                    quad_uniform, mass);
      else
        LaunchHierCells<false, true>(ctx, a, g.degree, HierRuleDegree(pr->qr_degree_tria, g.degree), uniform, mass);
    }
    coo->size += sp->num_triplets;
    return;
  }
  if (m->ntria) {
    a.list = m->tria_list.as<int32_t>();
    a.count = m->ntria;
    LaunchHierCells<false, false>(ctx, a, p, HierRuleDegree(pr->qr_degree_tria, p), uniform, mass);
  }
  if (m->nquad) {
    a.list = m->quad_list.as<int32_t>();
    a.count = m->nquad;
    LaunchHierCells<true, false>(ctx, a, p, HierRuleDegree(pr->qr_degree_quad, p), quad_uniform, mass);
  }
  coo->size += sp->num_triplets;
}

void HierAssembleVector(lfg_space* sp, const lfg_load_provider* pr, double* b) {
  lfg_mesh* m = sp->mesh;
  lfg_ctx* ctx = m->ctx;
  const int p = sp->hier_degree;
  if (m->ntria && pr->qr_degree_tria < 0)
    Fail(LFG_MISSING_RULE, "No local shape function information or no quadrature rule for reference element type TRIA");
  if (m->nquad && pr->qr_degree_quad < 0)
    Fail(LFG_MISSING_RULE, "No local shape function information or no quadrature rule for reference element type QUAD");
  const CoeffDev f = ToDev(pr->f, m, "load f");
  EnsureIncidence(sp);
  HierArgs a = BaseHierArgs(sp);
  double* ev = sp->scratch_vec.as<double>();
  ProfScope prof(ctx, "hier_load");
  // (cell type, degree, first entry, count) of every launch
  std::vector<HierGroup> groups;
  if (sp->hier_var) {
    groups = sp->hv_groups;
  } else {
    for (int q = 0; q < 2; ++q) {
      HierGroup g;
      g.quad = q == 1;
      g.degree = p;
      g.count = g.quad ? m->nquad : m->ntria;
      if (g.count) groups.push_back(g);
    }
  }
  for (const HierGroup& g : groups) {
    a.tab = GetHierTable(ctx, g.quad, g.degree,
                         HierRuleDegree(g.quad ? pr->qr_degree_quad : pr->qr_degree_tria, g.degree), false, a.L);
    if (sp->hier_var) a.list = sp->hv_sorted.as<int32_t>() + g.start;
    else a.list = g.quad ? m->quad_list.as<int32_t>() : m->tria_list.as<int32_t>();
    a.count = g.count;
    const size_t smem = static_cast<size_t>(a.L.nq) * 8;
    const int64_t* lo = sp->loc_offset.as<int64_t>();
    if (g.quad && sp->hier_var) {
      const int grid = HierGrid(ctx, HierLoadKernel<true, true>, smem, g.count);
      HierLoadKernel<true, true><<<grid, kHierBlock, smem, ctx->stream>>>(a, f, lo, ev);
    } else if (g.quad) {
      const int grid = HierGrid(ctx, HierLoadKernel<true, false>, smem, g.count);
      HierLoadKernel<true, false><<<grid, kHierBlock, smem, ctx->stream>>>(a, f, lo, ev);
    } else if (sp->hier_var) {
      const int grid = HierGrid(ctx, HierLoadKernel<false, true>, smem, g.count);
      HierLoadKernel<false, true><<<grid, kHierBlock, smem, ctx->stream>>>(a, f, lo, ev);
    } else {
      const int grid = HierGrid(ctx, HierLoadKernel<false, false>, smem, g.count);
      HierLoadKernel<false, false><<<grid, kHierBlock, smem, ctx->stream>>>(a, f, lo, ev);
    }
    LFG_LAUNCHED(ctx);
  }
  GatherElementVectors(sp, b);
}

}  // namespace lfg
