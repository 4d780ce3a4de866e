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
#include "lfg_internal.h"

namespace lfg {
namespace {

constexpr int kHierBlock = 128;

// Table block (doubles): w[nq] | x[nq] | y[nq] | then per pattern:
//   phi[nq][n] | g[nq][n][2] | R[E][4] (triangles only)
struct HierTab {
  int n = 0, nq = 0, E = 0, npat = 0;
  int64_t off_pat = 0, stride = 0, o_g = 0, o_R = 0, total = 0;
};

// Every block starts on a multiple of 4 doubles (32 bytes), so the vector
// loads of the kernels (16 bytes) stay aligned.
int64_t Pad4(int64_t x) { return (x + 3) & ~int64_t(3); }

HierTab HierLayout(bool quad, int n, int nq) {
  HierTab t;
  t.n = n;
  t.nq = nq;
  t.E = n * (n + 1) / 2;
  t.npat = quad ? 16 : 8;
  t.off_pat = Pad4(3 * static_cast<int64_t>(nq));
  t.o_g = Pad4(static_cast<int64_t>(nq) * n);
  t.o_R = Pad4(t.o_g + 2 * static_cast<int64_t>(nq) * n);
  t.stride = Pad4(t.o_R + (quad ? 0 : 4 * static_cast<int64_t>(t.E)));
  t.total = t.off_pat + t.npat * t.stride;
  return t;
}

void BuildHierTable(bool quad, int p, int rule_degree, std::vector<double>& h, HierTab& L) {
  Rule r;
  if (!MakeRule(quad, rule_degree, r))
    Fail(LFG_UNSUPPORTED, "no quadrature rule of degree " + std::to_string(rule_degree));
  const int n = quad ? (p + 1) * (p + 1) : (p + 1) * (p + 2) / 2;
  L = HierLayout(quad, n, r.n);
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
    if (quad) continue;
    // folded sums in long double, upper triangle row by row
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
      }
  }
}

// Cached on the context per (cell type, degree, rule degree).
const double* GetHierTable(lfg_ctx* ctx, bool quad, int p, int rule_degree, HierTab& L) {
  const int key = (1 << 23) | (quad ? 1 << 20 : 0) | (p << 10) | rule_degree;
  auto it = ctx->tables.find(key);
  if (it == ctx->tables.end()) {
    std::vector<double> h;
    BuildHierTable(quad, p, rule_degree, h, L);
    TableEntry& ent = ctx->tables[key];
    ent.layout = Tab{};
    ent.layout.n = L.n;
    ent.layout.nq = L.nq;
    ent.buf.alloc(h.size() * sizeof(double), ctx->stream);
    LFG_CUDA(cudaMemcpyAsync(ent.buf.p, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    LFG_CUDA(cudaStreamSynchronize(ctx->stream));
    return ent.buf.as<double>();
  }
  L = HierLayout(quad, it->second.layout.n, it->second.layout.nq);
  return it->second.buf.as<double>();
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

// Affine triangles, cell-constant alpha / gamma: tiles of T cells per CTA.
// Shared memory: vals[T][E] | coef[T][4] | base[T] (int64) | pat[T] | dofs[T][n].
__global__ void __launch_bounds__(kHierBlock) HierTriaAffineKernel(HierArgs a, int T) {
  extern __shared__ __align__(16) double smem[];
  const int n = a.L.n, E = a.L.E, nn = n * n;
  double* vals = smem;
  double* coef = vals + static_cast<int64_t>(T) * E;
  int64_t* base = reinterpret_cast<int64_t*>(coef + 4 * T);
  int* pat = reinterpret_cast<int*>(base + T);
  int* cid = pat + T;
  int* dofs = cid + T;
  for (int64_t t0 = static_cast<int64_t>(blockIdx.x) * T; t0 < a.count; t0 += static_cast<int64_t>(gridDim.x) * T) {
    const int tn = static_cast<int>(min(static_cast<int64_t>(T), a.count - t0));
    for (int t = threadIdx.x; t < tn; t += blockDim.x) {
      const int c = a.list[t0 + t];
      int4 cn;
      double2 v[4];
      LoadVerts<false>(a, c, cn, v);
      double m00, m01, m11, adet, X, Y;
      Metric<false>(v, 0.0, 0.0, m00, m01, m11, adet, X, Y);
      const double al = CellConstant(a.alpha, c), ga = CellConstant(a.gamma, c);
      coef[4 * t + 0] = m00 * al;
      coef[4 * t + 1] = m01 * al;
      coef[4 * t + 2] = m11 * al;
      coef[4 * t + 3] = adet * ga;
      base[t] = a.tri_offset[c];
      pat[t] = a.ori[c] & 7;
      cid[t] = c;
    }
    __syncthreads();
    for (int idx = threadIdx.x; idx < tn * n; idx += blockDim.x) {
      const int t = idx / n, i = idx - t * n;
      dofs[idx] = a.cell_dofs[static_cast<int64_t>(cid[t]) * a.n_cell + i];
    }
    for (int idx = threadIdx.x; idx < tn * E; idx += blockDim.x) {
      const int t = idx / E, e = idx - t * E;
      const double* R = a.tab + a.L.off_pat + pat[t] * a.L.stride + a.L.o_R + 4 * static_cast<int64_t>(e);
      const double2 r01 = *reinterpret_cast<const double2*>(R);
      const double2 r23 = *reinterpret_cast<const double2*>(R + 2);
      const double* cf = coef + 4 * t;
      vals[idx] = cf[0] * r01.x + cf[1] * r01.y + cf[2] * r23.x + cf[3] * r23.y;
    }
    __syncthreads();
    for (int q = threadIdx.x; q < tn * nn; q += blockDim.x) {
      const int t = q / nn, rr = q - t * nn;
      const int i = rr / n, j = rr - i * n;
      const int lo = min(i, j), hi = max(i, j);
      const int e = lo * n - lo * (lo - 1) / 2 + (hi - lo);
      StoreTriplet(a.out + base[t] + rr, dofs[t * n + i], dofs[t * n + j], vals[t * E + e]);
    }
    __syncthreads();
  }
}

// General path: one cell per CTA iteration.  Shared memory: coef[nq][4] | dofs[n].
template <bool QUAD>
__global__ void __launch_bounds__(kHierBlock) HierGeneralKernel(HierArgs a) {
  extern __shared__ __align__(16) double smem[];
  const int n = a.L.n, nq = a.L.nq, nn = n * n;
  double* coef = smem;
  int* dofs = reinterpret_cast<int*>(coef + 4 * nq);
  const double* __restrict__ tab = a.tab;
  for (int64_t ci = blockIdx.x; ci < a.count; ci += gridDim.x) {
    const int c = a.list[ci];
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
    for (int i = threadIdx.x; i < n; i += blockDim.x) dofs[i] = a.cell_dofs[static_cast<int64_t>(c) * a.n_cell + i];
    __syncthreads();
    const double* P = tab + a.L.off_pat + pat * a.L.stride;
    const double* G = P + a.L.o_g;
    const int64_t base = a.tri_offset[c];
    for (int q = threadIdx.x; q < nn; q += blockDim.x) {
      const int i = q / n, j = q - i * n;
      double acc = 0.0;
      for (int k = 0; k < nq; ++k) {
        const double2 gi = *reinterpret_cast<const double2*>(G + (static_cast<int64_t>(k) * n + i) * 2);
        const double2 gj = *reinterpret_cast<const double2*>(G + (static_cast<int64_t>(k) * n + j) * 2);
        const double* cf = coef + 4 * k;
        acc += cf[0] * (gi.x * gj.x) + cf[1] * (gi.x * gj.y + gi.y * gj.x) + cf[2] * (gi.y * gj.y) +
               cf[3] * (P[static_cast<int64_t>(k) * n + i] * P[static_cast<int64_t>(k) * n + j]);
      }
      StoreTriplet(a.out + base + q, dofs[i], dofs[j], acc);
    }
    __syncthreads();
  }
}

// Element vectors: s_k = (w_k |det J_k|) f(x_k), v_i = sum_k s_k phi_i(x_k),
// into ev at the cell's local offset.  Shared memory: s[nq].
template <bool QUAD>
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
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      double s = 0.0;
      for (int k = 0; k < nq; ++k) s += smem[k] * P[static_cast<int64_t>(k) * n + i];
      ev[b + i] = s;
    }
    __syncthreads();
  }
}

}  // namespace

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
  const bool uniform = CellConstantKind(pr->alpha) && CellConstantKind(pr->gamma);
  if (m->ntria) {
    a.tab = GetHierTable(ctx, false, p, HierRuleDegree(pr->qr_degree_tria, p), a.L);
    a.list = m->tria_list.as<int32_t>();
    a.count = m->ntria;
    const int n = a.L.n, E = a.L.E;
    int T = std::max(1, std::min(32, 4096 / (n * n)));
    auto smem_for = [&](int t) {
      return static_cast<size_t>(t) * E * 8 + static_cast<size_t>(t) * (4 * 8 + 8 + 4 + 4) +
             static_cast<size_t>(t) * n * 4;
    };
    while (T > 1 && smem_for(T) > 96 * 1024) --T;
    if (uniform && smem_for(T) <= kHierSmemLimit) {
      ProfScope prof(ctx, "hier_tria_affine");
      const size_t smem = smem_for(T);
      const int grid = HierGrid(ctx, HierTriaAffineKernel, smem, (a.count + T - 1) / T);
      HierTriaAffineKernel<<<grid, kHierBlock, smem, ctx->stream>>>(a, T);
      LFG_LAUNCHED(ctx);
    } else {
      ProfScope prof(ctx, "hier_general_tria");
      const size_t smem = static_cast<size_t>(a.L.nq) * 32 + static_cast<size_t>(n) * 4;
      const int grid = HierGrid(ctx, HierGeneralKernel<false>, smem, a.count);
      HierGeneralKernel<false><<<grid, kHierBlock, smem, ctx->stream>>>(a);
      LFG_LAUNCHED(ctx);
    }
  }
  if (m->nquad) {
    a.tab = GetHierTable(ctx, true, p, HierRuleDegree(pr->qr_degree_quad, p), a.L);
    a.list = m->quad_list.as<int32_t>();
    a.count = m->nquad;
    ProfScope prof(ctx, "hier_general_quad");
    const size_t smem = static_cast<size_t>(a.L.nq) * 32 + static_cast<size_t>(a.L.n) * 4;
    const int grid = HierGrid(ctx, HierGeneralKernel<true>, smem, a.count);
    HierGeneralKernel<true><<<grid, kHierBlock, smem, ctx->stream>>>(a);
    LFG_LAUNCHED(ctx);
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
  for (int q = 0; q < 2; ++q) {
    const bool quad = q == 1;
    const int64_t count = quad ? m->nquad : m->ntria;
    if (!count) continue;
    a.tab = GetHierTable(ctx, quad, p, HierRuleDegree(quad ? pr->qr_degree_quad : pr->qr_degree_tria, p), a.L);
    a.list = quad ? m->quad_list.as<int32_t>() : m->tria_list.as<int32_t>();
    a.count = count;
    const size_t smem = static_cast<size_t>(a.L.nq) * 8;
    if (quad) {
      const int grid = HierGrid(ctx, HierLoadKernel<true>, smem, count);
      HierLoadKernel<true><<<grid, kHierBlock, smem, ctx->stream>>>(a, f, sp->loc_offset.as<int64_t>(), ev);
    } else {
      const int grid = HierGrid(ctx, HierLoadKernel<false>, smem, count);
      HierLoadKernel<false><<<grid, kHierBlock, smem, ctx->stream>>>(a, f, sp->loc_offset.as<int64_t>(), ev);
    }
    LFG_LAUNCHED(ctx);
  }
  GatherElementVectors(sp, b);
}

}  // namespace lfg
