// Post-processing on the device: IntegrateMeshFunction over the closed set of
// integrands, MeshFunctionFE / MeshFunctionGradFE evaluation, NodalProjection
// and InitEssentialConditionFromFunction (fe/fe_tools.h:110-329,
// fe/mesh_function_fe.h:44-115, fe/mesh_function_grad_fe.h:44-126).
//
// All FP64.  One thread per cell (or edge) with the reference-element tables
// (rule points, weights, shape values and gradients at the points) read
// through the read-only cache.  Integrals reduce per block in a fixed order
// and then over the block partials in a fixed order, so a result does not
// depend on scheduling.  "Last entity wins" writes (NodalProjection,
// InitEssentialConditionFromFunction) are resolved with an owner pass:
// owner[dof] = max selected entity index holding the dof (atomicMax, order
// independent), then only the owner writes.
#include <algorithm>
#include <string>
#include <vector>

#include "lfg_api.h"
#include "lfg_coeff.h"
#include "lfg_internal.h"
#include "lfg_tables.h"

namespace lfg {
namespace {

constexpr int kPostBlock = 256;

// Reference-element data at a point set (rule points or user points), doubles:
//   w[nq] | x[nq] | y[nq] | phi[nq][n] | grad[nq][n][2]   (n = 0: no FE part)
struct PostTab {
  int nq = 0, n = 0;
  int off_w = 0, off_x = 0, off_y = 0, off_phi = 0, off_g = 0, total = 0;
};

PostTab PostLayout(int nq, int n) {
  PostTab t;
  t.nq = nq;
  t.n = n;
  t.off_w = 0;
  t.off_x = nq;
  t.off_y = 2 * nq;
  t.off_phi = 3 * nq;
  t.off_g = t.off_phi + nq * n;
  t.total = t.off_g + nq * n * 2;
  return t;
}

void FillPostTab(bool quad, int fe_degree, const Rule& r, std::vector<double>& h, PostTab& L) {
  const int n = fe_degree > 0 ? NumShape(quad, fe_degree) : 0;
  L = PostLayout(r.n, n);
  h.assign(std::max(L.total, 1), 0.0);
  double phi[16], dphi[16][2];
  for (int k = 0; k < r.n; ++k) {
    h[L.off_w + k] = r.w[k];
    h[L.off_x + k] = r.x[k];
    h[L.off_y + k] = r.y[k];
    if (n == 0) continue;
    Shape(quad, fe_degree, r.x[k], r.y[k], phi, dphi);
    for (int i = 0; i < n; ++i) {
      h[L.off_phi + k * n + i] = phi[i];
      h[L.off_g + (k * n + i) * 2] = dphi[i][0];
      h[L.off_g + (k * n + i) * 2 + 1] = dphi[i][1];
    }
  }
}

// Cached per (cell type, FE degree, rule degree) on the context.
const double* GetPostTable(lfg_ctx* ctx, bool quad, int fe_degree, int rule_degree, PostTab& L) {
  const int key = (1 << 22) | (quad ? 1 << 20 : 0) | (fe_degree << 10) | rule_degree;
  auto it = ctx->tables.find(key);
  if (it != ctx->tables.end()) {
    L.nq = it->second.layout.nq;
    L = PostLayout(it->second.layout.nq, it->second.layout.n);
    return it->second.buf.as<double>();
  }
  Rule r;
  if (!MakeRule(quad, rule_degree, r))
    Fail(LFG_UNSUPPORTED, "no quadrature rule of degree " + std::to_string(rule_degree) +
                              (quad ? " for quadrilaterals" : " for triangles"));
  std::vector<double> h;
  FillPostTab(quad, fe_degree, r, h, L);
  TableEntry& ent = ctx->tables[key];
  ent.layout = Tab{};
  ent.layout.n = L.n;
  ent.layout.nq = L.nq;
  ent.buf.alloc(h.size() * sizeof(double), ctx->stream);
  LFG_CUDA(cudaMemcpyAsync(ent.buf.p, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  LFG_CUDA(cudaStreamSynchronize(ctx->stream));
  return ent.buf.as<double>();
}

// ------------------------------------------------------------ device helpers

struct CellSide {
  const int32_t* list;  // cell indices of this type
  int64_t count;
  const double* tab;    // PostTab block of this type
  PostTab L;
  int n_loc;            // local dofs of this type (FE part)
};

struct PostArgs {
  const int4* cells;
  const double2* xy;
  const uint8_t* flags;   // null: every entity
  CoeffDev u;
  const int32_t* cell_dofs;
  int n_cell;
  const double* dofs;     // null: u_h = 0
  int kind;
};

template <bool QUAD>
__device__ __forceinline__ void LoadCell(const PostArgs& a, int c, int4& cn, double2 (&v)[4]) {
  cn = a.cells[c];
  v[0] = a.xy[cn.x];
  v[1] = a.xy[cn.y];
  v[2] = a.xy[cn.z];
  v[3] = QUAD ? a.xy[cn.w] : make_double2(0.0, 0.0);
}

// Global(), |det J| and J^{-T} at a reference point (tria_o1.cc:50-74,
// quad_o1.cc:67-156).
template <bool QUAD>
__device__ __forceinline__ void Geometry(const double2 (&v)[4], double xh, double yh, double& X, double& Y,
                                         double& ie, double (&JT)[2][2]) {
  double j00, j01, j10, j11;
  if (!QUAD) {
    const double l0 = 1.0 - xh - yh;
    X = v[0].x * l0 + v[1].x * xh + v[2].x * yh;
    Y = v[0].y * l0 + v[1].y * xh + v[2].y * yh;
    j00 = v[1].x - v[0].x; j01 = v[2].x - v[0].x;
    j10 = v[1].y - v[0].y; j11 = v[2].y - v[0].y;
  } else {
    const double b0 = (1 - xh) * (1 - yh), b1 = xh * (1 - yh), b2 = xh * yh, b3 = (1 - xh) * yh;
    X = v[0].x * b0 + v[1].x * b1 + v[2].x * b2 + v[3].x * b3;
    Y = v[0].y * b0 + v[1].y * b1 + v[2].y * b2 + v[3].y * b3;
    j00 = (v[1].x - v[0].x) * (1 - yh) + (v[2].x - v[3].x) * yh;
    j10 = (v[1].y - v[0].y) * (1 - yh) + (v[2].y - v[3].y) * yh;
    j01 = (v[3].x - v[0].x) * (1 - xh) + (v[2].x - v[1].x) * xh;
    j11 = (v[3].y - v[0].y) * (1 - xh) + (v[2].y - v[1].y) * xh;
  }
  const double det = j00 * j11 - j10 * j01;
  ie = fabs(det);
  const double inv = 1.0 / det;
  JT[0][0] = j11 * inv;  JT[0][1] = -j10 * inv;
  JT[1][0] = -j01 * inv; JT[1][1] = j00 * inv;
}

// u (and grad u) of a mesh function at a reference point of cell c.
template <bool QUAD>
__device__ __forceinline__ double MFPoint(const CoeffDev& u, int c, const int4& cn, double xh, double yh, double X,
                                          double Y, const double (&JT)[2][2], bool grad, double& gx, double& gy) {
  gx = gy = 0.0;
  switch (u.kind) {
    case LFG_COEFF_CONSTANT: return u.value;
    case LFG_COEFF_PER_CELL: return u.data[c];
    case LFG_COEFF_PER_CELL_EXP: return exp(u.data[c]);
    case LFG_COEFF_NODAL_O1: {
      const double d0 = u.data[cn.x], d1 = u.data[cn.y], d2 = u.data[cn.z];
      double val, hx, hy;
      if (!QUAD) {
        val = d0 * (1.0 - xh - yh) + d1 * xh + d2 * yh;
        hx = d1 - d0;
        hy = d2 - d0;
      } else {
        const double d3 = u.data[cn.w];
        val = d0 * ((1 - xh) * (1 - yh)) + d1 * (xh * (1 - yh)) + d2 * (xh * yh) + d3 * ((1 - xh) * yh);
        hx = (d1 - d0) * (1 - yh) + (d2 - d3) * yh;
        hy = (d3 - d0) * (1 - xh) + (d2 - d1) * xh;
      }
      if (grad) {
        gx = JT[0][0] * hx + JT[0][1] * hy;
        gy = JT[1][0] * hx + JT[1][1] * hy;
      }
      return val;
    }
    case LFG_COEFF_ANALYTIC:
      if (grad) EvalAnalyticGrad(u, X, Y, gx, gy);
      return EvalAnalytic(u, X, Y);
  }
  return 0.0;
}

// grad u alone (cell-wise constants: 0).
template <bool QUAD>
__device__ __forceinline__ void MFGrad(const CoeffDev& u, const int4& cn, double xh, double yh, double X, double Y,
                                       const double (&JT)[2][2], double& gx, double& gy) {
  gx = gy = 0.0;
  if (u.kind == LFG_COEFF_ANALYTIC) {
    EvalAnalyticGrad(u, X, Y, gx, gy);
  } else if (u.kind == LFG_COEFF_NODAL_O1) {
    double hx, hy;
    if (!QUAD) {
      hx = u.data[cn.y] - u.data[cn.x];
      hy = u.data[cn.z] - u.data[cn.x];
    } else {
      const double d0 = u.data[cn.x], d1 = u.data[cn.y], d2 = u.data[cn.z], d3 = u.data[cn.w];
      hx = (d1 - d0) * (1 - yh) + (d2 - d3) * yh;
      hy = (d3 - d0) * (1 - xh) + (d2 - d1) * xh;
    }
    gx = JT[0][0] * hx + JT[0][1] * hy;
    gy = JT[1][0] * hx + JT[1][1] * hy;
  }
}

// Deterministic block sum of one double per thread into part[blockIdx.x].
__device__ __forceinline__ void BlockSumTo(double s, double* part) {
  __shared__ double red[kPostBlock];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = kPostBlock / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

// LocalIntegral (fe_tools.h:35-68) of every selected cell of one type:
// sum_k value_k (w_k |det J(q_k)|), summed per thread in list order.
template <bool QUAD, int DEG>
__host__ __device__ constexpr int LocalDofs() {
  return DEG == 0 ? 0 : QUAD ? (DEG + 1) * (DEG + 1) : (DEG + 1) * (DEG + 2) / 2;
}

// DEG: degree of the FE part (0: no u_h), fixing the local dof count; KIND:
// the integrand (compile time, so the value or the gradient of u that the
// integrand does not use is never computed).
template <bool QUAD, int DEG, int KIND>
__global__ void __launch_bounds__(kPostBlock) IntegrateCellsKernel(PostArgs a, CellSide s, double* part) {
  constexpr int N = LocalDofs<QUAD, DEG>();
  constexpr bool need_grad = KIND == LFG_INTEGRAND_GRAD_SQ_DIFF;
  const double* __restrict__ tab = s.tab;
  const PostTab L = s.L;
  double acc = 0.0;
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < s.count;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int c = s.list[i];
    if (a.flags && !a.flags[c] && c != 0) continue;
    int4 cn;
    double2 v[4];
    LoadCell<QUAD>(a, c, cn, v);
    double d[N > 0 ? N : 1];
#pragma unroll
    for (int j = 0; j < N; ++j) d[j] = a.dofs[a.cell_dofs[static_cast<int64_t>(c) * a.n_cell + j]];
    double local = 0.0;
    for (int k = 0; k < L.nq; ++k) {
      const double xh = tab[L.off_x + k], yh = tab[L.off_y + k];
      double X, Y, ie, JT[2][2];
      Geometry<QUAD>(v, xh, yh, X, Y, ie, JT);
      double gx, gy, uv = 0.0;
      if (need_grad) MFGrad<QUAD>(a.u, cn, xh, yh, X, Y, JT, gx, gy);
      else uv = MFPoint<QUAD>(a.u, c, cn, xh, yh, X, Y, JT, false, gx, gy);
      double hv = 0.0, hx = 0.0, hy = 0.0;
#pragma unroll
      for (int j = 0; j < N; ++j) {
        if (need_grad) {
          hx += d[j] * tab[L.off_g + (k * N + j) * 2];
          hy += d[j] * tab[L.off_g + (k * N + j) * 2 + 1];
        } else {
          hv += d[j] * tab[L.off_phi + k * N + j];
        }
      }
      double val;
      if (KIND == LFG_INTEGRAND_VALUE) {
        val = hv + uv;
      } else if (KIND == LFG_INTEGRAND_SQ_DIFF) {
        val = (hv - uv) * (hv - uv);
      } else {
        const double ex = (JT[0][0] * hx + JT[0][1] * hy) - gx;
        const double ey = (JT[1][0] * hx + JT[1][1] * hy) - gy;
        val = ex * ex + ey * ey;
      }
      local += val * (tab[L.off_w + k] * ie);
    }
    acc += local;
  }
  BlockSumTo(acc, part);
}

// IntegrateMeshFunction with u_h on a hierarchic space (uniform degree, or
// one degree group of a per-entity-degree space): one warp per cell.  The
// cell's dof values (and, with VAR, its slots in the degree-D table) go to
// shared memory; the lanes take the rule points, each forming u_h (or its
// gradient) from the table block of the cell's orientation pattern, the
// mesh function and the integrand, then the cell's integral is a fixed
// shuffle tree.  Per warp the cells are summed in list order, then the warps
// of a block in order, so the result does not depend on scheduling.
constexpr int kHierPostWarps = 4;
struct HierPostSide {
  const int32_t* list;
  int64_t count;
  const double* tab;
  HierTabView T;
  const uint8_t* ori;
  const uint16_t* sel;        // VAR: slot of each local shape function
  const int64_t* loc_offset;  // VAR: local counts
};

template <bool QUAD, int KIND, bool VAR>
__global__ void __launch_bounds__(32 * kHierPostWarps) IntegrateHierKernel(PostArgs a, HierPostSide h, double* part) {
  extern __shared__ __align__(16) double shd[];
  constexpr bool need_grad = KIND == LFG_INTEGRAND_GRAD_SQ_DIFF;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int n = h.T.n, nq = h.T.nq;
  double* sd = shd + warp * n;
  int* ss = reinterpret_cast<int*>(shd + kHierPostWarps * n) + warp * n;
  const double* __restrict__ tab = h.tab;
  double acc = 0.0;
  for (int64_t i = blockIdx.x * static_cast<int64_t>(kHierPostWarps) + warp; i < h.count;
       i += static_cast<int64_t>(gridDim.x) * kHierPostWarps) {
    const int c = h.list[i];
    if (a.flags && !a.flags[c] && c != 0) continue;  // warp-uniform
    const int m = VAR ? static_cast<int>(h.loc_offset[c + 1] - h.loc_offset[c]) : n;
    for (int j = lane; j < m; j += 32) {
      sd[j] = a.dofs[a.cell_dofs[static_cast<int64_t>(c) * a.n_cell + j]];
      ss[j] = VAR ? h.sel[static_cast<int64_t>(c) * a.n_cell + j] : j;
    }
    __syncwarp();
    int4 cn;
    double2 v[4];
    LoadCell<QUAD>(a, c, cn, v);
    const double* P = tab + h.T.off_pat + (h.ori[c] & (QUAD ? 15 : 7)) * h.T.stride;
    double local = 0.0;
    for (int k = lane; k < nq; k += 32) {
      const double xh = tab[nq + k], yh = tab[2 * nq + k];
      double X, Y, ie, JT[2][2];
      Geometry<QUAD>(v, xh, yh, X, Y, ie, JT);
      double gx, gy, uv = 0.0;
      if (need_grad) MFGrad<QUAD>(a.u, cn, xh, yh, X, Y, JT, gx, gy);
      else uv = MFPoint<QUAD>(a.u, c, cn, xh, yh, X, Y, JT, false, gx, gy);
      double hv = 0.0, hx = 0.0, hy = 0.0;
      const double* pk = P + static_cast<int64_t>(k) * n;
      const double* gk = P + h.T.o_g + static_cast<int64_t>(k) * n * 2;
      for (int j = 0; j < m; ++j) {
        const int sj = ss[j];
        if (need_grad) {
          hx = fma(sd[j], gk[2 * sj], hx);
          hy = fma(sd[j], gk[2 * sj + 1], hy);
        } else {
          hv = fma(sd[j], pk[sj], hv);
        }
      }
      double val;
      if (KIND == LFG_INTEGRAND_VALUE) {
        val = hv + uv;
      } else if (KIND == LFG_INTEGRAND_SQ_DIFF) {
        val = (hv - uv) * (hv - uv);
      } else {
        const double ex = (JT[0][0] * hx + JT[0][1] * hy) - gx;
        const double ey = (JT[1][0] * hx + JT[1][1] * hy) - gy;
        val = ex * ex + ey * ey;
      }
      local += val * (tab[k] * ie);
    }
    for (int o = 16; o > 0; o >>= 1) local += __shfl_xor_sync(0xffffffffu, local, o);
    acc += local;  // the same value in every lane
    __syncwarp();
  }
  __shared__ double wsum[kHierPostWarps];
  if (lane == 0) wsum[warp] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < kHierPostWarps; ++w) s += wsum[w];
    part[blockIdx.x] = s;
  }
}

// MeshFunctionFE / MeshFunctionGradFE of u_h on a hierarchic space at the
// table's points of every cell of one group: one warp per cell, lanes over
// the points.
template <bool QUAD, bool VAR>
__global__ void __launch_bounds__(32 * kHierPostWarps) FeEvalHierKernel(PostArgs a, HierPostSide h, double* vals,
                                                                        double* grads) {
  extern __shared__ __align__(16) double shd[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int n = h.T.n, nq = h.T.nq;
  double* sd = shd + warp * n;
  int* ss = reinterpret_cast<int*>(shd + kHierPostWarps * n) + warp * n;
  const double* __restrict__ tab = h.tab;
  for (int64_t i = blockIdx.x * static_cast<int64_t>(kHierPostWarps) + warp; i < h.count;
       i += static_cast<int64_t>(gridDim.x) * kHierPostWarps) {
    const int c = h.list[i];
    const int m = VAR ? static_cast<int>(h.loc_offset[c + 1] - h.loc_offset[c]) : n;
    for (int j = lane; j < m; j += 32) {
      sd[j] = a.dofs[a.cell_dofs[static_cast<int64_t>(c) * a.n_cell + j]];
      ss[j] = VAR ? h.sel[static_cast<int64_t>(c) * a.n_cell + j] : j;
    }
    __syncwarp();
    int4 cn;
    double2 v[4];
    LoadCell<QUAD>(a, c, cn, v);
    const double* P = tab + h.T.off_pat + (h.ori[c] & (QUAD ? 15 : 7)) * h.T.stride;
    for (int k = lane; k < nq; k += 32) {
      const double* pk = P + static_cast<int64_t>(k) * n;
      const double* gk = P + h.T.o_g + static_cast<int64_t>(k) * n * 2;
      double hv = 0.0, hx = 0.0, hy = 0.0;
      for (int j = 0; j < m; ++j) {
        const int sj = ss[j];
        if (vals) hv = fma(sd[j], pk[sj], hv);
        if (grads) {
          hx = fma(sd[j], gk[2 * sj], hx);
          hy = fma(sd[j], gk[2 * sj + 1], hy);
        }
      }
      const int64_t o = static_cast<int64_t>(c) * nq + k;
      if (vals) vals[o] = hv;
      if (grads) {
        double X, Y, ie, JT[2][2];
        Geometry<QUAD>(v, tab[nq + k], tab[2 * nq + k], X, Y, ie, JT);
        grads[2 * o] = JT[0][0] * hx + JT[0][1] * hy;
        grads[2 * o + 1] = JT[1][0] * hx + JT[1][1] * hy;
      }
    }
    __syncwarp();
  }
}

template <bool QUAD, bool VAR>
void LaunchIntegrateHier(int kind, int blocks, size_t smem, cudaStream_t st, const PostArgs& a,
                         const HierPostSide& h, double* part) {
  const int thr = 32 * kHierPostWarps;
  switch (kind) {
    case LFG_INTEGRAND_VALUE:
      LFG_CUDA(cudaFuncSetAttribute(IntegrateHierKernel<QUAD, LFG_INTEGRAND_VALUE, VAR>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
      IntegrateHierKernel<QUAD, LFG_INTEGRAND_VALUE, VAR><<<blocks, thr, smem, st>>>(a, h, part);
      break;
    case LFG_INTEGRAND_SQ_DIFF:
      LFG_CUDA(cudaFuncSetAttribute(IntegrateHierKernel<QUAD, LFG_INTEGRAND_SQ_DIFF, VAR>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
      IntegrateHierKernel<QUAD, LFG_INTEGRAND_SQ_DIFF, VAR><<<blocks, thr, smem, st>>>(a, h, part);
      break;
    default:
      LFG_CUDA(cudaFuncSetAttribute(IntegrateHierKernel<QUAD, LFG_INTEGRAND_GRAD_SQ_DIFF, VAR>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
      IntegrateHierKernel<QUAD, LFG_INTEGRAND_GRAD_SQ_DIFF, VAR><<<blocks, thr, smem, st>>>(a, h, part);
      break;
  }
}

// Segment rule and basis for edges (points t on [0,1] along the edge).
struct EdgeSide {
  int64_t ne;
  const int2* edges;
  const double* t;    // [nq]
  const double* w;    // [nq]
  const double* phi;  // [nq][n] segment basis of the FE degree
  int nq, n;
  int np, ns;         // dofs per node / per edge interior
  int64_t node_dofs;  // num_nodes * np
};

__device__ __forceinline__ double EdgeMF(const CoeffDev& f, int64_t e, const int2& en, const double2& p0,
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

// Global dofs of edge e: both endpoints' node dofs in edge direction, then
// the interior dofs (dofhandler.cc:167-195 for codim 1).
__device__ __forceinline__ int EdgeDofList(const EdgeSide& s, int64_t e, const int2& en, int64_t* d) {
  int k = 0;
  for (int j = 0; j < s.np; ++j) d[k++] = static_cast<int64_t>(en.x) * s.np + j;
  for (int j = 0; j < s.np; ++j) d[k++] = static_cast<int64_t>(en.y) * s.np + j;
  for (int j = 0; j < s.ns; ++j) d[k++] = s.node_dofs + e * s.ns + j;
  return k;
}

template <int DEG>
__global__ void __launch_bounds__(kPostBlock) IntegrateEdgesKernel(PostArgs a, EdgeSide s, double* part) {
  constexpr int N = DEG == 0 ? 0 : DEG + 1;
  double acc = 0.0;
  for (int64_t e = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; e < s.ne;
       e += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    if (a.flags && !a.flags[e] && e != 0) continue;
    const int2 en = s.edges[e];
    const double2 p0 = a.xy[en.x], p1 = a.xy[en.y];
    const double len = hypot(p1.x - p0.x, p1.y - p0.y);
    double d[N > 0 ? N : 1];
    if (N > 0) {
      int64_t g[N > 0 ? N : 1];
      EdgeDofList(s, e, en, g);
#pragma unroll
      for (int j = 0; j < N; ++j) d[j] = a.dofs[g[j]];
    }
    double local = 0.0;
    for (int k = 0; k < s.nq; ++k) {
      const double uv = EdgeMF(a.u, e, en, p0, p1, s.t[k]);
      double hv = 0.0;
#pragma unroll
      for (int j = 0; j < N; ++j) hv += d[j] * s.phi[k * s.n + j];
      const double val = a.kind == LFG_INTEGRAND_VALUE ? hv + uv : (hv - uv) * (hv - uv);
      local += val * (s.w[k] * len);
    }
    acc += local;
  }
  BlockSumTo(acc, part);
}

__global__ void __launch_bounds__(kPostBlock) SumPartialsKernel(int64_t m, const double* __restrict__ part,
                                                                double* __restrict__ out) {
  double s = 0.0;
  for (int64_t i = threadIdx.x; i < m; i += kPostBlock) s += part[i];
  BlockSumTo(s, out);
}

// MeshFunctionFE / MeshFunctionGradFE at the table's points on every cell of
// one type.
template <bool QUAD, int DEG>
__global__ void __launch_bounds__(kPostBlock) FEEvalKernel(PostArgs a, CellSide s, double* vals, double* grads) {
  constexpr int N = LocalDofs<QUAD, DEG>();
  const double* __restrict__ tab = s.tab;
  const PostTab L = s.L;
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < s.count;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int c = s.list[i];
    int4 cn;
    double2 v[4];
    LoadCell<QUAD>(a, c, cn, v);
    double d[N];
#pragma unroll
    for (int j = 0; j < N; ++j) d[j] = a.dofs[a.cell_dofs[static_cast<int64_t>(c) * a.n_cell + j]];
    for (int k = 0; k < L.nq; ++k) {
      const int64_t o = static_cast<int64_t>(c) * L.nq + k;
      double hv = 0.0, hx = 0.0, hy = 0.0;
#pragma unroll
      for (int j = 0; j < N; ++j) {
        hv += d[j] * tab[L.off_phi + k * N + j];
        hx += d[j] * tab[L.off_g + (k * N + j) * 2];
        hy += d[j] * tab[L.off_g + (k * N + j) * 2 + 1];
      }
      if (vals) vals[o] = hv;
      if (grads) {
        double X, Y, ie, JT[2][2];
        Geometry<QUAD>(v, tab[L.off_x + k], tab[L.off_y + k], X, Y, ie, JT);
        grads[2 * o] = JT[0][0] * hx + JT[0][1] * hy;
        grads[2 * o + 1] = JT[1][0] * hx + JT[1][1] * hy;
      }
    }
  }
}

// owner[dof] = max selected cell holding it.
__global__ void ProjectOwnerKernel(int64_t nc, const int4* __restrict__ cells, const uint8_t* __restrict__ flags,
                                   const int32_t* __restrict__ cell_dofs, int n_cell, int n_tria, int n_quad,
                                   int32_t* __restrict__ owner) {
  for (int64_t c = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; c < nc;
       c += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    if (flags && !flags[c]) continue;
    const int n = cells[c].w >= 0 ? n_quad : n_tria;
    for (int j = 0; j < n; ++j) atomicMax(&owner[cell_dofs[c * n_cell + j]], static_cast<int32_t>(c));
  }
}

struct NodeSet {
  double tx[10], ty[10];  // triangle evaluation nodes
  double qx[16], qy[16];  // quadrilateral evaluation nodes
  int n_tria, n_quad;
};

__global__ void ProjectKernel(PostArgs a, int64_t nc, NodeSet ns, const int32_t* __restrict__ owner,
                              double* __restrict__ out) {
  for (int64_t c = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; c < nc;
       c += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    if (a.flags && !a.flags[c]) continue;
    const bool quad = a.cells[c].w >= 0;
    int4 cn;
    double2 v[4];
    double JT[2][2];
    double gx, gy, X, Y, ie;
    if (quad) LoadCell<true>(a, static_cast<int>(c), cn, v);
    else LoadCell<false>(a, static_cast<int>(c), cn, v);
    const int n = quad ? ns.n_quad : ns.n_tria;
    for (int j = 0; j < n; ++j) {
      const int32_t d = a.cell_dofs[c * a.n_cell + j];
      if (owner[d] != c) continue;
      const double xh = quad ? ns.qx[j] : ns.tx[j], yh = quad ? ns.qy[j] : ns.ty[j];
      double val;
      if (quad) {
        Geometry<true>(v, xh, yh, X, Y, ie, JT);
        val = MFPoint<true>(a.u, static_cast<int>(c), cn, xh, yh, X, Y, JT, false, gx, gy);
      } else {
        Geometry<false>(v, xh, yh, X, Y, ie, JT);
        val = MFPoint<false>(a.u, static_cast<int>(c), cn, xh, yh, X, Y, JT, false, gx, gy);
      }
      out[d] = val;
    }
  }
}

// owner[dof] = max selected cell holding it, local counts from loc_offset
// (hierarchic spaces, whose counts may vary by cell).
__global__ void ProjectOwnerLocKernel(int64_t nc, const uint8_t* __restrict__ flags,
                                      const int32_t* __restrict__ cell_dofs, int n_cell,
                                      const int64_t* __restrict__ loc_offset, int32_t* __restrict__ owner) {
  for (int64_t c = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; c < nc;
       c += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    if (flags && !flags[c]) continue;
    const int n = static_cast<int>(loc_offset[c + 1] - loc_offset[c]);
    for (int j = 0; j < n; ++j) atomicMax(&owner[cell_dofs[c * n_cell + j]], static_cast<int32_t>(c));
  }
}

// One dual table of a hierarchic cell kind: evaluation nodes xy[2 ne] at
// off_xy, the NodalValuesToDofs matrix M[n][ne] at off_M (doubles into one
// table buffer).
struct HierDualDir {
  int64_t off_xy, off_M;
  int32_t ne, n;
};
constexpr int kHierProjWarps = 4;

// NodalProjection on a hierarchic space: one warp per cell.  The lanes
// evaluate u at the cell's evaluation nodes into shared memory, then each
// lane forms the dofs it owns as a row of M times those values (k ascending).
// The cell's table is tid[c], or (tid null: uniform degree) its orientation
// pattern, quadrilaterals after the 8 triangle patterns.
__global__ void __launch_bounds__(32 * kHierProjWarps)
    HierProjectKernel(PostArgs a, int64_t nc, const HierDualDir* __restrict__ dir, const double* __restrict__ tab,
                      const int32_t* __restrict__ tid, const uint8_t* __restrict__ ori, int ne_max,
                      const int32_t* __restrict__ owner, double* __restrict__ out) {
  extern __shared__ __align__(16) double sv[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  double* v = sv + warp * ne_max;
  for (int64_t c = blockIdx.x * static_cast<int64_t>(kHierProjWarps) + warp; c < nc;
       c += static_cast<int64_t>(gridDim.x) * kHierProjWarps) {
    if (a.flags && !a.flags[c]) continue;
    const bool quad = a.cells[c].w >= 0;
    const int t = tid ? tid[c] : (quad ? 8 + (ori[c] & 15) : (ori[c] & 7));
    const HierDualDir T = dir[t];
    int4 cn;
    double2 vx[4];
    double JT[2][2];
    double gx, gy, X, Y, ie;
    if (quad) LoadCell<true>(a, static_cast<int>(c), cn, vx);
    else LoadCell<false>(a, static_cast<int>(c), cn, vx);
    const double* xy = tab + T.off_xy;
    for (int k = lane; k < T.ne; k += 32) {
      const double xh = xy[2 * k], yh = xy[2 * k + 1];
      if (quad) {
        Geometry<true>(vx, xh, yh, X, Y, ie, JT);
        v[k] = MFPoint<true>(a.u, static_cast<int>(c), cn, xh, yh, X, Y, JT, false, gx, gy);
      } else {
        Geometry<false>(vx, xh, yh, X, Y, ie, JT);
        v[k] = MFPoint<false>(a.u, static_cast<int>(c), cn, xh, yh, X, Y, JT, false, gx, gy);
      }
    }
    __syncwarp();
    for (int j = lane; j < T.n; j += 32) {
      const int32_t d = a.cell_dofs[c * a.n_cell + j];
      if (owner[d] != c) continue;
      const double* Mr = tab + T.off_M + static_cast<int64_t>(j) * T.ne;
      double sum = 0.0;
      for (int k = 0; k < T.ne; ++k) sum = fma(Mr[k], v[k], sum);
      out[d] = sum;
    }
    __syncwarp();
  }
}

__global__ void EssentialOwnerKernel(EdgeSide s, const uint8_t* __restrict__ flags, int32_t* __restrict__ owner) {
  for (int64_t e = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; e < s.ne;
       e += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    if (!flags[e]) continue;
    int64_t d[8];
    const int n = EdgeDofList(s, e, s.edges[e], d);
    for (int j = 0; j < n; ++j) atomicMax(&owner[d[j]], static_cast<int32_t>(e));
  }
}

// Segment evaluation nodes 0, 1, 1/p, ..., (p-1)/p in edge direction.
__global__ void EssentialKernel(EdgeSide s, const double2* __restrict__ xy, const uint8_t* __restrict__ flags,
                                CoeffDev g, int degree, const int32_t* __restrict__ owner,
                                uint8_t* __restrict__ dflag, double* __restrict__ dval) {
  for (int64_t e = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; e < s.ne;
       e += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    if (!flags[e]) continue;
    const int2 en = s.edges[e];
    const double2 p0 = xy[en.x], p1 = xy[en.y];
    int64_t d[8];
    const int n = EdgeDofList(s, e, en, d);
    for (int j = 0; j < n; ++j) {
      if (owner[d[j]] != e) continue;
      // local dof j sits at node 0 (j < np), 1 (j < 2 np) or interior j - 2 np
      const double t = j < s.np ? 0.0 : j < 2 * s.np ? 1.0 : static_cast<double>(j - 2 * s.np + 1) / degree;
      dflag[d[j]] = 1;
      dval[d[j]] = EdgeMF(g, e, en, p0, p1, t);
    }
  }
}

__global__ void FillI32Kernel(int64_t n, int32_t v, int32_t* __restrict__ p) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x)
    p[i] = v;
}

template <bool QUAD, int KIND>
void LaunchCellsK(int deg, int grid, cudaStream_t st, const PostArgs& a, const CellSide& s, double* part) {
  switch (deg) {
    case 0: IntegrateCellsKernel<QUAD, 0, KIND><<<grid, kPostBlock, 0, st>>>(a, s, part); break;
    case 1: IntegrateCellsKernel<QUAD, 1, KIND><<<grid, kPostBlock, 0, st>>>(a, s, part); break;
    case 2: IntegrateCellsKernel<QUAD, 2, KIND><<<grid, kPostBlock, 0, st>>>(a, s, part); break;
    default: IntegrateCellsKernel<QUAD, 3, KIND><<<grid, kPostBlock, 0, st>>>(a, s, part); break;
  }
}

template <bool QUAD>
void LaunchCells(int deg, int grid, cudaStream_t st, const PostArgs& a, const CellSide& s, double* part) {
  switch (a.kind) {
    case LFG_INTEGRAND_VALUE: LaunchCellsK<QUAD, LFG_INTEGRAND_VALUE>(deg, grid, st, a, s, part); break;
    case LFG_INTEGRAND_SQ_DIFF: LaunchCellsK<QUAD, LFG_INTEGRAND_SQ_DIFF>(deg, grid, st, a, s, part); break;
    default: LaunchCellsK<QUAD, LFG_INTEGRAND_GRAD_SQ_DIFF>(deg, grid, st, a, s, part); break;
  }
}

template <bool QUAD>
void LaunchEval(int deg, int grid, cudaStream_t st, const PostArgs& a, const CellSide& s, double* v, double* g) {
  switch (deg) {
    case 1: FEEvalKernel<QUAD, 1><<<grid, kPostBlock, 0, st>>>(a, s, v, g); break;
    case 2: FEEvalKernel<QUAD, 2><<<grid, kPostBlock, 0, st>>>(a, s, v, g); break;
    default: FEEvalKernel<QUAD, 3><<<grid, kPostBlock, 0, st>>>(a, s, v, g); break;
  }
}

// Grid of a reduction launch: the block count is part of the summation
// order, so it depends only on the entity count and the SM count.
int ReduceBlocks(lfg_ctx* ctx, int64_t n) {
  const int64_t need = (n + kPostBlock - 1) / kPostBlock;
  return static_cast<int>(std::max<int64_t>(1, std::min<int64_t>(need, static_cast<int64_t>(ctx->num_sms) * 8)));
}

PostArgs BasePostArgs(lfg_mesh* m, const lfg_coeff& u, const char* what) {
  PostArgs a{};
  a.cells = m->cell_nodes.as<int4>();
  a.xy = m->xy.as<double2>();
  a.u = ToDev(u, m, what);
  return a;
}

EdgeSide BaseEdgeSide(lfg_mesh* m, const lfg_space* sp) {
  EdgeSide s{};
  s.ne = m->ne;
  s.edges = m->edge_nodes.as<int2>();
  if (sp) {
    s.np = sp->np;
    s.ns = sp->ns;
    s.node_dofs = m->nv * sp->np;
  }
  return s;
}

// Dual tables of a hierarchic space and the table of every cell.  Uniform
// degree: the 8 triangle and 16 quadrilateral orientation patterns (tid
// stays empty).  Per-entity degrees: one table per distinct (type, interior
// degree, edge degrees, pattern) among the cells, found on the host.
struct HierDualSet {
  std::vector<HierDualDir> dir;
  std::vector<double> tab;
  std::vector<int32_t> tid;
  int ne_max = 0;
};

void AddHierDual(HierDualSet& H, bool quad, int pc, const int* pe, int pat) {
  std::vector<double> xy, M;
  HierDual(quad, pc, pe, pat, xy, M);
  HierDualDir d{};
  d.ne = static_cast<int32_t>(xy.size() / 2);
  d.n = static_cast<int32_t>(d.ne ? M.size() / d.ne : 0);
  d.off_xy = static_cast<int64_t>(H.tab.size());
  H.tab.insert(H.tab.end(), xy.begin(), xy.end());
  d.off_M = static_cast<int64_t>(H.tab.size());
  H.tab.insert(H.tab.end(), M.begin(), M.end());
  H.dir.push_back(d);
  H.ne_max = std::max(H.ne_max, static_cast<int>(d.ne));
}

constexpr size_t kMaxHierDualTableBytes = size_t(1) << 30;

void BuildHierDuals(lfg_space* sp, HierDualSet& H) {
  lfg_mesh* m = sp->mesh;
  if (!sp->hier_var) {
    const int p = sp->hier_degree;
    const int pe[4] = {p, p, p, p};
    for (int q = 0; q < 2; ++q)
      for (int pat = 0; pat < (q ? 16 : 8); ++pat) {
        if ((q ? m->nquad : m->ntria) == 0) {
          H.dir.push_back(HierDualDir{0, 0, 0, 0});
          continue;
        }
        AddHierDual(H, q == 1, p, pe, pat);
      }
    return;
  }
  const int64_t nc = m->nc;
  std::vector<int4> cn(nc), ce(nc);
  std::vector<uint8_t> ori(nc);
  D2HSync(m->ctx, cn.data(), m->cell_nodes.p, nc * sizeof(int4));
  D2HSync(m->ctx, ce.data(), m->cell_edges.p, nc * sizeof(int4));
  D2HSync(m->ctx, ori.data(), m->cell_ori.p, nc);
  const auto& ed = sp->hv_edge_deg_host;
  H.tid.resize(nc);
  std::vector<std::pair<uint64_t, int32_t>> seen;  // sorted (key, table)
  for (int64_t c = 0; c < nc; ++c) {
    const bool quad = cn[c].w >= 0;
    const int nv = quad ? 4 : 3;
    const int e[4] = {ce[c].x, ce[c].y, ce[c].z, ce[c].w};
    int pe[4] = {1, 1, 1, 1};
    const int pc = sp->hv_cell_deg_host[c];
    const int pat = ori[c] & (quad ? 15 : 7);
    uint64_t key = (quad ? 1ull : 0ull) << 40 | static_cast<uint64_t>(pc) << 32 | static_cast<uint64_t>(pat) << 24;
    for (int j = 0; j < nv; ++j) {
      pe[j] = ed[e[j]];
      key |= static_cast<uint64_t>(pe[j]) << (6 * j);
    }
    auto it = std::lower_bound(seen.begin(), seen.end(), std::make_pair(key, int32_t(-1)));
    if (it != seen.end() && it->first == key) {
      H.tid[c] = it->second;
      continue;
    }
    const int32_t id = static_cast<int32_t>(H.dir.size());
    AddHierDual(H, quad, pc, pe, pat);
    if (H.tab.size() * sizeof(double) > kMaxHierDualTableBytes)
      Fail(LFG_UNSUPPORTED, "NodalProjection: the dual tables of this space's degree combinations exceed 1 GiB");
    seen.insert(it, std::make_pair(key, id));
    H.tid[c] = id;
  }
}

// MeshFunctionFE / MeshFunctionGradFE on a hierarchic space at npts reference
// points of every cell.
void FeEvalHier(lfg_space* sp, const double* dofs, int npts, const double* ref_points, double* vals, double* grads);

// IntegrateMeshFunction (codim 0) with u_h on a hierarchic space: one launch
// per (cell type, degree) group, block partials summed in one fixed order.
void IntegrateHier(lfg_mesh* m, lfg_space* sp, const lfg_integrand* g, int quad_degree, const uint8_t* flags,
                   double* result);

void RequireLagrange(const lfg_space* sp, const char* what) {
  if (sp->degree < 1 || sp->degree > 3)
    Fail(LFG_UNSUPPORTED, std::string(what) + ": needs a Lagrangian space of degree 1..3");
}

// The (cell type, degree) groups of a hierarchic space.
std::vector<HierGroup> HierGroups(const lfg_space* sp) {
  if (sp->hier_var) return sp->hv_groups;
  std::vector<HierGroup> groups;
  for (int q = 0; q < 2; ++q) {
    HierGroup gr;
    gr.quad = q == 1;
    gr.degree = sp->hier_degree;
    gr.count = gr.quad ? sp->mesh->nquad : sp->mesh->ntria;
    if (gr.count) groups.push_back(gr);
  }
  return groups;
}

void FeEvalHier(lfg_space* sp, const double* dofs, int npts, const double* ref_points, double* vals, double* grads) {
  lfg_mesh* m = sp->mesh;
  lfg_ctx* ctx = m->ctx;
  PostArgs a{};
  a.cells = m->cell_nodes.as<int4>();
  a.xy = m->xy.as<double2>();
  a.cell_dofs = sp->cell_dofs.as<int32_t>();
  a.n_cell = sp->n_cell;
  a.dofs = dofs;
  std::vector<double> x(npts), y(npts);
  for (int k = 0; k < npts; ++k) {
    x[k] = ref_points[2 * k];
    y[k] = ref_points[2 * k + 1];
  }
  ProfScope prof(ctx, "fe_eval_hier");
  for (const HierGroup& gr : HierGroups(sp)) {
    HierPostSide h{};
    std::vector<double> tab_h;
    HierShapeTableAt(gr.quad, gr.degree, x, y, tab_h, h.T);
    DevBuf tab;
    tab.alloc(tab_h.size() * sizeof(double), ctx->stream);
    LFG_CUDA(cudaMemcpyAsync(tab.p, tab_h.data(), tab_h.size() * sizeof(double), cudaMemcpyHostToDevice,
                             ctx->stream));
    h.tab = tab.as<double>();
    h.list = sp->hier_var ? sp->hv_sorted.as<int32_t>() + gr.start
                          : (gr.quad ? m->quad_list.as<int32_t>() : m->tria_list.as<int32_t>());
    h.count = gr.count;
    h.ori = m->cell_ori.as<uint8_t>();
    h.sel = sp->hier_var ? sp->hv_sel.as<uint16_t>() : nullptr;
    h.loc_offset = sp->loc_offset.as<int64_t>();
    const size_t smem = static_cast<size_t>(kHierPostWarps) * h.T.n * (sizeof(double) + sizeof(int));
    const int blocks = static_cast<int>(
        std::max<int64_t>(1, std::min<int64_t>((gr.count + kHierPostWarps - 1) / kHierPostWarps,
                                               static_cast<int64_t>(ctx->num_sms) * 8)));
    if (gr.quad && sp->hier_var) {
      LFG_CUDA(cudaFuncSetAttribute(FeEvalHierKernel<true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    static_cast<int>(smem)));
      FeEvalHierKernel<true, true><<<blocks, 32 * kHierPostWarps, smem, ctx->stream>>>(a, h, vals, grads);
    } else if (gr.quad) {
      LFG_CUDA(cudaFuncSetAttribute(FeEvalHierKernel<true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    static_cast<int>(smem)));
      FeEvalHierKernel<true, false><<<blocks, 32 * kHierPostWarps, smem, ctx->stream>>>(a, h, vals, grads);
    } else if (sp->hier_var) {
      LFG_CUDA(cudaFuncSetAttribute(FeEvalHierKernel<false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    static_cast<int>(smem)));
      FeEvalHierKernel<false, true><<<blocks, 32 * kHierPostWarps, smem, ctx->stream>>>(a, h, vals, grads);
    } else {
      LFG_CUDA(cudaFuncSetAttribute(FeEvalHierKernel<false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    static_cast<int>(smem)));
      FeEvalHierKernel<false, false><<<blocks, 32 * kHierPostWarps, smem, ctx->stream>>>(a, h, vals, grads);
    }
    LFG_LAUNCHED(ctx);
    // the table buffer is released stream-ordered after the launch
  }
}

void IntegrateHier(lfg_mesh* m, lfg_space* sp, const lfg_integrand* g, int quad_degree, const uint8_t* flags,
                   double* result) {
  lfg_ctx* ctx = m->ctx;
  PostArgs a = BasePostArgs(m, g->u, "IntegrateMeshFunction");
  a.flags = flags;
  a.kind = g->kind;
  a.dofs = g->dofs_dev;
  a.cell_dofs = sp->cell_dofs.as<int32_t>();
  a.n_cell = sp->n_cell;
  const std::vector<HierGroup> groups = HierGroups(sp);
  std::vector<int> blocks;
  int total = 0;
  for (const HierGroup& gr : groups) {
    const int64_t need = (gr.count + kHierPostWarps - 1) / kHierPostWarps;
    const int b = static_cast<int>(std::max<int64_t>(1, std::min<int64_t>(need, static_cast<int64_t>(ctx->num_sms) * 8)));
    blocks.push_back(b);
    total += b;
  }
  DevBuf part;
  part.alloc((total + 1) * sizeof(double), ctx->stream);
  double* p = part.as<double>();
  ProfScope prof(ctx, "integrate_cells_hier");
  int off = 0;
  for (size_t k = 0; k < groups.size(); ++k) {
    const HierGroup& gr = groups[k];
    HierPostSide h{};
    h.tab = HierShapeTable(ctx, gr.quad, gr.degree, quad_degree, h.T);
    h.list = sp->hier_var ? sp->hv_sorted.as<int32_t>() + gr.start
                          : (gr.quad ? m->quad_list.as<int32_t>() : m->tria_list.as<int32_t>());
    h.count = gr.count;
    h.ori = m->cell_ori.as<uint8_t>();
    h.sel = sp->hier_var ? sp->hv_sel.as<uint16_t>() : nullptr;
    h.loc_offset = sp->loc_offset.as<int64_t>();
    const size_t smem = static_cast<size_t>(kHierPostWarps) * h.T.n * (sizeof(double) + sizeof(int));
    if (gr.quad && sp->hier_var) LaunchIntegrateHier<true, true>(g->kind, blocks[k], smem, ctx->stream, a, h, p + off);
    else if (gr.quad) LaunchIntegrateHier<true, false>(g->kind, blocks[k], smem, ctx->stream, a, h, p + off);
    else if (sp->hier_var) LaunchIntegrateHier<false, true>(g->kind, blocks[k], smem, ctx->stream, a, h, p + off);
    else LaunchIntegrateHier<false, false>(g->kind, blocks[k], smem, ctx->stream, a, h, p + off);
    LFG_LAUNCHED(ctx);
    off += blocks[k];
  }
  if (total == 0) {
    LFG_CUDA(cudaMemsetAsync(p, 0, sizeof(double), ctx->stream));
  } else {
    SumPartialsKernel<<<1, kPostBlock, 0, ctx->stream>>>(total, p, p + total);
    LFG_LAUNCHED(ctx);
  }
  D2HSync(ctx, result, p + (total == 0 ? 0 : total), sizeof(double));
}

}  // namespace
}  // namespace lfg

using namespace lfg;

extern "C" {

lfg_status lfg_integrate_mesh_function(lfg_mesh* m, const lfg_integrand* g, int32_t quad_degree,
                                       const uint8_t* flags, int32_t codim, double* result) {
  if (!m || !g || !result) return LFG_INVALID_ARG;
  LFG_API_BEGIN(m->ctx)
  lfg_ctx* ctx = m->ctx;
  if (g->kind < LFG_INTEGRAND_VALUE || g->kind > LFG_INTEGRAND_GRAD_SQ_DIFF)
    Fail(LFG_INVALID_ARG, "IntegrateMeshFunction: unknown integrand kind");
  if (codim != 0 && codim != 1) Fail(LFG_UNSUPPORTED, "IntegrateMeshFunction: codim must be 0 or 1");
  if (quad_degree < 0 || quad_degree > kMaxRuleDegree)
    Fail(LFG_UNSUPPORTED, "IntegrateMeshFunction: quadrature degree out of range");
  lfg_space* sp = g->space;
  if (g->dofs_dev) {
    if (!sp) Fail(LFG_INVALID_ARG, "IntegrateMeshFunction: dofs without a space");
    if (sp->mesh != m) Fail(LFG_INVALID_ARG, "IntegrateMeshFunction: the space lives on another mesh");
    if (sp->hier_degree > 0) {
      if (codim != 0) Fail(LFG_UNSUPPORTED, "IntegrateMeshFunction: hierarchic u_h on edges is not supported");
      IntegrateHier(m, sp, g, quad_degree, flags, result);
      return LFG_OK;
    }
    RequireLagrange(sp, "IntegrateMeshFunction");
  }
  PostArgs a = BasePostArgs(m, g->u, "IntegrateMeshFunction");
  a.flags = flags;
  a.kind = g->kind;
  a.dofs = g->dofs_dev;
  if (sp) {
    a.cell_dofs = sp->cell_dofs.as<int32_t>();
    a.n_cell = sp->n_cell;
  }
  const int fe_deg = g->dofs_dev ? sp->degree : 0;
  DevBuf part;
  if (codim == 0) {
    const int bt = m->ntria ? ReduceBlocks(ctx, m->ntria) : 0, bq = m->nquad ? ReduceBlocks(ctx, m->nquad) : 0;
    part.alloc((bt + bq + 1) * sizeof(double), ctx->stream);
    double* p = part.as<double>();
    ProfScope prof(ctx, "integrate_cells");
    if (bt) {
      CellSide s{};
      s.list = m->tria_list.as<int32_t>();
      s.count = m->ntria;
      s.tab = GetPostTable(ctx, false, fe_deg, quad_degree, s.L);
      s.n_loc = sp ? sp->n_tria : 0;
      LaunchCells<false>(fe_deg, bt, ctx->stream, a, s, p);
      LFG_LAUNCHED(ctx);
    }
    if (bq) {
      CellSide s{};
      s.list = m->quad_list.as<int32_t>();
      s.count = m->nquad;
      s.tab = GetPostTable(ctx, true, fe_deg, quad_degree, s.L);
      s.n_loc = sp ? sp->n_quad : 0;
      LaunchCells<true>(fe_deg, bq, ctx->stream, a, s, p + bt);
      LFG_LAUNCHED(ctx);
    }
    if (bt + bq == 0) LFG_CUDA(cudaMemsetAsync(p, 0, sizeof(double), ctx->stream));
    else {
      SumPartialsKernel<<<1, kPostBlock, 0, ctx->stream>>>(bt + bq, p, p + bt + bq);
      LFG_LAUNCHED(ctx);
    }
    D2HSync(ctx, result, p + (bt + bq == 0 ? 0 : bt + bq), sizeof(double));
  } else {
    if (g->kind == LFG_INTEGRAND_GRAD_SQ_DIFF)
      Fail(LFG_UNSUPPORTED, "IntegrateMeshFunction: gradients on edges are not supported");
    std::vector<double> t, w, phi;
    if (!SegmentTables(fe_deg > 0 ? fe_deg : 1, quad_degree, t, w, phi))
      Fail(LFG_UNSUPPORTED, "IntegrateMeshFunction: no segment rule");
    EdgeSide s = BaseEdgeSide(m, g->dofs_dev ? sp : nullptr);
    s.nq = static_cast<int>(t.size());
    s.n = (fe_deg > 0 ? fe_deg : 1) + 1;
    std::vector<double> h;
    h.insert(h.end(), t.begin(), t.end());
    h.insert(h.end(), w.begin(), w.end());
    h.insert(h.end(), phi.begin(), phi.end());
    DevBuf tab;
    tab.alloc(h.size() * sizeof(double), ctx->stream);
    LFG_CUDA(cudaMemcpyAsync(tab.p, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    s.t = tab.as<double>();
    s.w = s.t + s.nq;
    s.phi = s.w + s.nq;
    const int be = m->ne ? ReduceBlocks(ctx, m->ne) : 0;
    part.alloc((be + 1) * sizeof(double), ctx->stream);
    double* p = part.as<double>();
    ProfScope prof(ctx, "integrate_edges");
    if (be) {
      switch (fe_deg) {
        case 0: IntegrateEdgesKernel<0><<<be, kPostBlock, 0, ctx->stream>>>(a, s, p); break;
        case 1: IntegrateEdgesKernel<1><<<be, kPostBlock, 0, ctx->stream>>>(a, s, p); break;
        case 2: IntegrateEdgesKernel<2><<<be, kPostBlock, 0, ctx->stream>>>(a, s, p); break;
        default: IntegrateEdgesKernel<3><<<be, kPostBlock, 0, ctx->stream>>>(a, s, p); break;
      }
      LFG_LAUNCHED(ctx);
      SumPartialsKernel<<<1, kPostBlock, 0, ctx->stream>>>(be, p, p + be);
      LFG_LAUNCHED(ctx);
    } else {
      LFG_CUDA(cudaMemsetAsync(p, 0, sizeof(double), ctx->stream));
    }
    D2HSync(ctx, result, p + be, sizeof(double));
  }
  LFG_API_END
}

lfg_status lfg_fe_eval(lfg_space* sp, const double* dofs, int32_t npts, const double* ref_points, double* vals,
                       double* grads) {
  if (!sp || !dofs || npts < 0 || (npts > 0 && !ref_points)) return LFG_INVALID_ARG;
  LFG_API_BEGIN(sp->mesh->ctx)
  lfg_ctx* ctx = sp->mesh->ctx;
  lfg_mesh* m = sp->mesh;
  if (sp->hier_degree > 0) {
    if (npts == 0 || (!vals && !grads)) return LFG_OK;
    FeEvalHier(sp, dofs, npts, ref_points, vals, grads);
    return LFG_OK;
  }
  RequireLagrange(sp, "MeshFunctionFE");
  if (npts == 0 || (!vals && !grads)) return LFG_OK;
  PostArgs a{};
  a.cells = m->cell_nodes.as<int4>();
  a.xy = m->xy.as<double2>();
  a.cell_dofs = sp->cell_dofs.as<int32_t>();
  a.n_cell = sp->n_cell;
  a.dofs = dofs;
  Rule r;
  r.n = npts;
  for (int k = 0; k < npts; ++k) {
    r.x.push_back(ref_points[2 * k]);
    r.y.push_back(ref_points[2 * k + 1]);
    r.w.push_back(0.0);
  }
  ProfScope prof(ctx, "fe_eval");
  for (int q = 0; q < 2; ++q) {
    const bool quad = q == 1;
    const int64_t count = quad ? m->nquad : m->ntria;
    if (!count) continue;
    std::vector<double> h;
    CellSide s{};
    FillPostTab(quad, sp->degree, r, h, s.L);
    DevBuf tab;
    tab.alloc(h.size() * sizeof(double), ctx->stream);
    LFG_CUDA(cudaMemcpyAsync(tab.p, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    s.list = quad ? m->quad_list.as<int32_t>() : m->tria_list.as<int32_t>();
    s.count = count;
    s.tab = tab.as<double>();
    s.n_loc = quad ? sp->n_quad : sp->n_tria;
    const int grid = GridFor(ctx, count, kPostBlock);
    if (quad) LaunchEval<true>(sp->degree, grid, ctx->stream, a, s, vals, grads);
    else LaunchEval<false>(sp->degree, grid, ctx->stream, a, s, vals, grads);
    LFG_LAUNCHED(ctx);
    // the table buffer is released stream-ordered after the launch
  }
  LFG_API_END
}

lfg_status lfg_nodal_projection(lfg_space* sp, const lfg_coeff* u, const uint8_t* cell_flags, double* out) {
  if (!sp || !u || !out) return LFG_INVALID_ARG;
  LFG_API_BEGIN(sp->mesh->ctx)
  lfg_ctx* ctx = sp->mesh->ctx;
  lfg_mesh* m = sp->mesh;
  if (sp->hier_degree > 0) {
    PostArgs a = BasePostArgs(m, *u, "NodalProjection");
    a.flags = cell_flags;
    a.cell_dofs = sp->cell_dofs.as<int32_t>();
    a.n_cell = sp->n_cell;
    ProfScope prof(ctx, "nodal_projection_hier");
    LFG_CUDA(cudaMemsetAsync(out, 0, sp->num_dofs * sizeof(double), ctx->stream));
    if (m->nc == 0 || sp->num_dofs == 0) return LFG_OK;
    HierDualSet H;
    BuildHierDuals(sp, H);
    DevBuf dir, tab, tid, owner;
    dir.alloc(H.dir.size() * sizeof(HierDualDir), ctx->stream);
    tab.alloc(std::max<size_t>(H.tab.size(), 1) * sizeof(double), ctx->stream);
    LFG_CUDA(cudaMemcpyAsync(dir.p, H.dir.data(), H.dir.size() * sizeof(HierDualDir), cudaMemcpyHostToDevice,
                             ctx->stream));
    LFG_CUDA(cudaMemcpyAsync(tab.p, H.tab.data(), H.tab.size() * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    if (!H.tid.empty()) {
      tid.alloc(H.tid.size() * sizeof(int32_t), ctx->stream);
      LFG_CUDA(cudaMemcpyAsync(tid.p, H.tid.data(), H.tid.size() * sizeof(int32_t), cudaMemcpyHostToDevice,
                               ctx->stream));
    }
    owner.alloc(sp->num_dofs * sizeof(int32_t), ctx->stream);
    FillI32Kernel<<<GridFor(ctx, sp->num_dofs, 256), 256, 0, ctx->stream>>>(sp->num_dofs, -1, owner.as<int32_t>());
    LFG_LAUNCHED(ctx);
    ProjectOwnerLocKernel<<<GridFor(ctx, m->nc, 256), 256, 0, ctx->stream>>>(
        m->nc, cell_flags, a.cell_dofs, sp->n_cell, sp->loc_offset.as<int64_t>(), owner.as<int32_t>());
    LFG_LAUNCHED(ctx);
    const size_t smem = static_cast<size_t>(kHierProjWarps) * std::max(H.ne_max, 1) * sizeof(double);
    if (smem > 48 * 1024)
      LFG_CUDA(cudaFuncSetAttribute(HierProjectKernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    static_cast<int>(smem)));
    const int64_t blocks = std::min<int64_t>((m->nc + kHierProjWarps - 1) / kHierProjWarps,
                                             static_cast<int64_t>(ctx->num_sms) * 16);
    HierProjectKernel<<<static_cast<int>(blocks), 32 * kHierProjWarps, smem, ctx->stream>>>(
        a, m->nc, dir.as<HierDualDir>(), tab.as<double>(), H.tid.empty() ? nullptr : tid.as<int32_t>(),
        m->cell_ori.as<uint8_t>(), std::max(H.ne_max, 1), owner.as<int32_t>(), out);
    LFG_LAUNCHED(ctx);
    // the host tables must outlive their (pageable, possibly deferred) copies
    LFG_CUDA(cudaStreamSynchronize(ctx->stream));
    return LFG_OK;
  }
  RequireLagrange(sp, "NodalProjection");
  PostArgs a = BasePostArgs(m, *u, "NodalProjection");
  a.flags = cell_flags;
  a.cell_dofs = sp->cell_dofs.as<int32_t>();
  a.n_cell = sp->n_cell;
  NodeSet ns{};
  std::vector<double> xy;
  NodeCoords(false, sp->degree, xy);
  ns.n_tria = static_cast<int>(xy.size() / 2);
  for (int j = 0; j < ns.n_tria; ++j) { ns.tx[j] = xy[2 * j]; ns.ty[j] = xy[2 * j + 1]; }
  NodeCoords(true, sp->degree, xy);
  ns.n_quad = static_cast<int>(xy.size() / 2);
  for (int j = 0; j < ns.n_quad; ++j) { ns.qx[j] = xy[2 * j]; ns.qy[j] = xy[2 * j + 1]; }
  if (ns.n_tria != sp->n_tria || ns.n_quad != sp->n_quad) Fail(LFG_UNSUPPORTED, "NodalProjection: evaluation nodes do not match the space");
  ProfScope prof(ctx, "nodal_projection");
  LFG_CUDA(cudaMemsetAsync(out, 0, sp->num_dofs * sizeof(double), ctx->stream));
  if (m->nc == 0 || sp->num_dofs == 0) return LFG_OK;
  DevBuf owner;
  owner.alloc(sp->num_dofs * sizeof(int32_t), ctx->stream);
  FillI32Kernel<<<GridFor(ctx, sp->num_dofs, 256), 256, 0, ctx->stream>>>(sp->num_dofs, -1, owner.as<int32_t>());
  LFG_LAUNCHED(ctx);
  ProjectOwnerKernel<<<GridFor(ctx, m->nc, 256), 256, 0, ctx->stream>>>(
      m->nc, a.cells, cell_flags, a.cell_dofs, sp->n_cell, sp->n_tria, sp->n_quad, owner.as<int32_t>());
  LFG_LAUNCHED(ctx);
  ProjectKernel<<<GridFor(ctx, m->nc, 128), 128, 0, ctx->stream>>>(a, m->nc, ns, owner.as<int32_t>(), out);
  LFG_LAUNCHED(ctx);
  LFG_API_END
}

lfg_status lfg_init_essential_condition(lfg_space* sp, const uint8_t* edge_flags, const lfg_coeff* g,
                                        uint8_t* dof_flags, double* dof_values) {
  if (!sp || !edge_flags || !g || !dof_flags || !dof_values) return LFG_INVALID_ARG;
  LFG_API_BEGIN(sp->mesh->ctx)
  lfg_ctx* ctx = sp->mesh->ctx;
  lfg_mesh* m = sp->mesh;
  RequireLagrange(sp, "InitEssentialConditionFromFunction");
  const CoeffDev gd = ToDev(*g, m, "InitEssentialConditionFromFunction");
  EdgeSide s = BaseEdgeSide(m, sp);
  ProfScope prof(ctx, "essential_condition");
  LFG_CUDA(cudaMemsetAsync(dof_flags, 0, sp->num_dofs, ctx->stream));
  LFG_CUDA(cudaMemsetAsync(dof_values, 0, sp->num_dofs * sizeof(double), ctx->stream));
  if (m->ne == 0 || sp->num_dofs == 0) return LFG_OK;
  DevBuf owner;
  owner.alloc(sp->num_dofs * sizeof(int32_t), ctx->stream);
  FillI32Kernel<<<GridFor(ctx, sp->num_dofs, 256), 256, 0, ctx->stream>>>(sp->num_dofs, -1, owner.as<int32_t>());
  LFG_LAUNCHED(ctx);
  EssentialOwnerKernel<<<GridFor(ctx, m->ne, 256), 256, 0, ctx->stream>>>(s, edge_flags, owner.as<int32_t>());
  LFG_LAUNCHED(ctx);
  EssentialKernel<<<GridFor(ctx, m->ne, 256), 256, 0, ctx->stream>>>(
      s, m->xy.as<double2>(), edge_flags, gd, sp->degree, owner.as<int32_t>(), dof_flags, dof_values);
  LFG_LAUNCHED(ctx);
  LFG_API_END
}

}  // extern "C"
