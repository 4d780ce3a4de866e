// COO -> CSR (COOMatrix::makeSparse, assemble/coomatrix.h:172-180) and the
// solve: CSR SpMV and Jacobi-preconditioned CG in FP64 and in mixed precision
// (FP32 inner iterations inside FP64 iterative refinement).
//
// makeSparse goes through Eigen::SparseMatrix::setFromTriplets, which sums the
// duplicates of each (row, col) in triplet order.  Here the triplets are
// sorted by (row, col) with a stable radix sort (so duplicates stay in triplet
// order) and each run is summed left to right, which reproduces those sums
// bit for bit.
//
// The solver keeps every scalar on the device: a PCG iteration is three
// kernels (SpMV fused with <p, Ap>; x/r/z update fused with <r, z> and <r, r>;
// p update), block partial sums are reduced by every consumer block in the
// same fixed order (deterministic), and the iteration body is captured in a
// CUDA graph replayed `check_every` iterations at a time.
#include <algorithm>
#include <cmath>
#include <vector>

#include "lfg_api.h"
#include "lfg_internal.h"

namespace lfg {
namespace {

int BitsFor(int64_t n) {
  int b = 1;
  while ((int64_t(1) << b) < n + 1) ++b;
  return b;
}

__global__ void CooKeysKernel(int64_t n, const lfg_triplet* __restrict__ t, int cbits,
                              uint64_t* __restrict__ keys, uint32_t* __restrict__ vals, int32_t* st,
                              int64_t rows, int64_t cols) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const lfg_triplet tr = t[i];
    if (tr.row < 0 || tr.row >= rows || tr.col < 0 || tr.col >= cols) {
      atomicCAS(st, 0, 1);
      keys[i] = 0;
    } else {
      keys[i] = (static_cast<uint64_t>(tr.row) << cbits) | static_cast<uint64_t>(tr.col);
    }
    vals[i] = static_cast<uint32_t>(i);
  }
}

__global__ void HeadsKernel(int64_t n, const uint64_t* __restrict__ keys, int64_t* __restrict__ head) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x)
    head[i] = (i == 0 || keys[i] != keys[i - 1]);
}

__global__ void ReduceRunsKernel(int64_t n, const uint64_t* __restrict__ keys,
                                 const uint32_t* __restrict__ order, const int64_t* __restrict__ slot,
                                 const lfg_triplet* __restrict__ t, int cbits,
                                 int32_t* __restrict__ col, double* __restrict__ val,
                                 int32_t* __restrict__ row_of_slot) {
  const uint64_t cmask = (1ull << cbits) - 1ull;
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const uint64_t k = keys[i];
    if (i > 0 && keys[i - 1] == k) continue;
    double s = t[order[i]].value;
    for (int64_t m = i + 1; m < n && keys[m] == k; ++m) s = s + t[order[m]].value;
    const int64_t q = slot[i];
    col[q] = static_cast<int32_t>(k & cmask);
    val[q] = s;
    row_of_slot[q] = static_cast<int32_t>(k >> cbits);
  }
}

__global__ void RowPtrKernel(int64_t nnz, const int32_t* __restrict__ row_of_slot, int64_t rows,
                             int64_t* __restrict__ rowptr) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < nnz;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int64_t r = row_of_slot[i];
    const int64_t prev = i == 0 ? -1 : row_of_slot[i - 1];
    for (int64_t q = prev + 1; q <= r; ++q) rowptr[q] = i;
    if (i == nnz - 1)
      for (int64_t q = r + 1; q <= rows; ++q) rowptr[q] = nnz;
  }
}

__global__ void RowPtrEmptyKernel(int64_t rows, int64_t* rowptr) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i <= rows;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x)
    rowptr[i] = 0;
}

// ------------------------------------------------------------------- SpMV
// Eight lanes per row (rows of a Lagrangian FE matrix hold 7..~40 entries);
// the lane partial sums are combined in a fixed shuffle order.
constexpr int kLanes = 8;

// Row r's dot product by the 8 lanes of its group.  All 32 lanes of the warp
// call this together (rows past the end contribute zero), so the full-mask
// shuffles never see an exited lane.
template <class T, class V>
__device__ __forceinline__ T RowDot(const int32_t* __restrict__ rp, const int32_t* __restrict__ col,
                                    const V* __restrict__ val, const T* __restrict__ x, int64_t r,
                                    int64_t rows, int sub) {
  T s = T(0);
  if (r < rows)
    for (int q = rp[r] + sub; q < rp[r + 1]; q += kLanes) s = fma(static_cast<T>(val[q]), x[col[q]], s);
#pragma unroll
  for (int o = kLanes / 2; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o, kLanes);
  return s;
}

// Warp-uniform row loop: each warp owns 32 / kLanes consecutive rows per trip.
#define LFG_ROW_LOOP(r)                                                                     \
  const int sub = threadIdx.x % kLanes;                                                     \
  const int64_t warp_id = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) >> 5; \
  const int64_t nwarps = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;              \
  const int grp = (threadIdx.x & 31) / kLanes;                                              \
  for (int64_t wb = warp_id * (32 / kLanes); wb < rows; wb += nwarps * (32 / kLanes))       \
    for (int64_t r = wb + grp, once = 0; once < 1; ++once)

__global__ void SpmvKernel(int64_t rows, const int32_t* __restrict__ rp, const int32_t* __restrict__ col,
                           const double* __restrict__ val, const double* __restrict__ x,
                           double* __restrict__ y) {
  LFG_ROW_LOOP(r) {
    const double s = RowDot<double, double>(rp, col, val, x, r, rows, sub);
    if (sub == 0 && r < rows) y[r] = s;
  }
}

// r = b - A x (FP64) with <r, r> block partials.
__global__ void ResidualKernel(int64_t rows, const int32_t* __restrict__ rp, const int32_t* __restrict__ col,
                               const double* __restrict__ val, const double* __restrict__ x,
                               const double* __restrict__ b, double* __restrict__ r,
                               double* __restrict__ part) {
  __shared__ double red[32];
  double acc = 0.0;
  LFG_ROW_LOOP(i) {
    const double s = RowDot<double, double>(rp, col, val, x, i, rows, sub);
    if (sub == 0 && i < rows) {
      const double ri = b[i] - s;
      r[i] = ri;
      acc = fma(ri, ri, acc);
    }
  }
  // block reduction in fixed order
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < (blockDim.x >> 5); ++w) s += red[w];
    part[blockIdx.x] = s;
  }
}

// ------------------------------------------------------------------- PCG
constexpr int kPcgBlock = 256;

template <class T>
__device__ double BlockSum(double v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int w = 0; w < (blockDim.x >> 5); ++w) s += red[w];
  return s;
}

// Every block sums the same partial array in the same order.
__device__ double SumPartials(const double* __restrict__ part, int n, double* red) {
  double v = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) v += part[i];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double s = 0.0;
  for (int w = 0; w < (blockDim.x >> 5); ++w) s += red[w];
  __syncthreads();
  return s;
}

// q = A p and partials of <p, q>.
template <class T>
__global__ void __launch_bounds__(kPcgBlock) PcgSpmvKernel(int64_t rows, const int32_t* __restrict__ rp,
                                                           const int32_t* __restrict__ col,
                                                           const T* __restrict__ val, const T* __restrict__ p,
                                                           T* __restrict__ q, double* __restrict__ part) {
  __shared__ double red[32];
  T acc = T(0);
  LFG_ROW_LOOP(i) {
    const T s = RowDot<T, T>(rp, col, val, p, i, rows, sub);
    if (sub == 0 && i < rows) {
      q[i] = s;
      acc = fma(p[i], s, acc);
    }
  }
  const double tot = BlockSum<T>(static_cast<double>(acc), red);
  if (threadIdx.x == 0) part[blockIdx.x] = tot;
}

// alpha = rz / <p,q>; x += alpha p; r -= alpha q; z = D^-1 r; partials <r,z>, <r,r>.
template <class T>
__global__ void __launch_bounds__(kPcgBlock) PcgUpdateKernel(int64_t rows, const double* __restrict__ pq_part,
                                                             const double* __restrict__ rz_old_part, int nparts,
                                                             const T* __restrict__ dinv, const T* __restrict__ p,
                                                             const T* __restrict__ q, T* __restrict__ x,
                                                             T* __restrict__ r, T* __restrict__ z,
                                                             double* __restrict__ rz_part,
                                                             double* __restrict__ rr_part) {
  __shared__ double red[32];
  const double pq = SumPartials(pq_part, nparts, red);
  const double rz = SumPartials(rz_old_part, nparts, red);
  const T alpha = static_cast<T>(pq != 0.0 ? rz / pq : 0.0);
  T arz = T(0), arr = T(0);
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < rows;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    x[i] = fma(alpha, p[i], x[i]);
    const T ri = fma(-alpha, q[i], r[i]);
    r[i] = ri;
    const T zi = dinv[i] * ri;
    z[i] = zi;
    arz = fma(ri, zi, arz);
    arr = fma(ri, ri, arr);
  }
  const double s1 = BlockSum<T>(static_cast<double>(arz), red);
  const double s2 = BlockSum<T>(static_cast<double>(arr), red);
  if (threadIdx.x == 0) {
    rz_part[blockIdx.x] = s1;
    rr_part[blockIdx.x] = s2;
  }
}

// beta = rz_new / rz_old; p = z + beta p.
template <class T>
__global__ void __launch_bounds__(kPcgBlock) PcgDirectionKernel(int64_t rows, const double* __restrict__ rz_new_part,
                                                                const double* __restrict__ rz_old_part, int nparts,
                                                                const T* __restrict__ z, T* __restrict__ p) {
  __shared__ double red[32];
  const double rn = SumPartials(rz_new_part, nparts, red);
  const double ro = SumPartials(rz_old_part, nparts, red);
  const T beta = static_cast<T>(ro != 0.0 ? rn / ro : 0.0);
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < rows;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x)
    p[i] = fma(beta, p[i], z[i]);
}

// z = D^-1 r, p = z, partials <r,z>, <r,r> (PCG start).
template <class T>
__global__ void __launch_bounds__(kPcgBlock) PcgStartKernel(int64_t rows, const T* __restrict__ dinv,
                                                            const T* __restrict__ r, T* __restrict__ z,
                                                            T* __restrict__ p, double* __restrict__ rz_part,
                                                            double* __restrict__ rr_part) {
  __shared__ double red[32];
  T arz = T(0), arr = T(0);
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < rows;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const T ri = r[i];
    const T zi = dinv[i] * ri;
    z[i] = zi;
    p[i] = zi;
    arz = fma(ri, zi, arz);
    arr = fma(ri, ri, arr);
  }
  const double s1 = BlockSum<T>(static_cast<double>(arz), red);
  const double s2 = BlockSum<T>(static_cast<double>(arr), red);
  if (threadIdx.x == 0) {
    rz_part[blockIdx.x] = s1;
    rr_part[blockIdx.x] = s2;
  }
}

__global__ void DiagKernel(int64_t rows, const int64_t* __restrict__ rp, const int32_t* __restrict__ col,
                           const double* __restrict__ val, double* __restrict__ dinv,
                           float* __restrict__ dinv32, int32_t* st) {
  for (int64_t r = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; r < rows;
       r += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    double d = 0.0;
    for (int64_t q = rp[r]; q < rp[r + 1]; ++q)
      if (col[q] == r) d = val[q];
    if (!(d > 0.0)) atomicCAS(st, 0, static_cast<int>(r) + 1);
    dinv[r] = d > 0.0 ? 1.0 / d : 0.0;
    dinv32[r] = static_cast<float>(dinv[r]);
  }
}

__global__ void ToFloatKernel(int64_t n, const double* __restrict__ a, float* __restrict__ b) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x)
    b[i] = static_cast<float>(a[i]);
}

__global__ void RowPtr32Kernel(int64_t n, const int64_t* __restrict__ a, int32_t* __restrict__ b) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x)
    b[i] = static_cast<int32_t>(a[i]);
}

// mixed precision helpers: r32 = r64 * s; x64 += d32 / s
__global__ void ScaleToFloatKernel(int64_t n, const double* __restrict__ r, double s, float* __restrict__ r32,
                                   float* __restrict__ d32) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    r32[i] = static_cast<float>(r[i] * s);
    d32[i] = 0.0f;
  }
}

__global__ void AddCorrectionKernel(int64_t n, const float* __restrict__ d, double inv_s, double* __restrict__ x) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x)
    x[i] += static_cast<double>(d[i]) * inv_s;
}

double HostSum(lfg_ctx* ctx, const double* part, int n, std::vector<double>& tmp) {
  tmp.resize(n);
  LFG_CUDA(cudaMemcpyAsync(tmp.data(), part, n * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  LFG_CUDA(cudaStreamSynchronize(ctx->stream));
  double s = 0.0;
  for (double v : tmp) s += v;
  return s;
}

void PrepareSolve(lfg_csr* A) {
  lfg_ctx* ctx = A->ctx;
  cudaStream_t s = ctx->stream;
  if (A->dinv.p) return;
  if (A->nnz >= (int64_t(1) << 31)) Fail(LFG_UNSUPPORTED, "solver needs nnz < 2^31");
  A->rowptr32.alloc((A->rows + 1) * sizeof(int32_t), s);
  RowPtr32Kernel<<<GridFor(ctx, A->rows + 1, 256), 256, 0, s>>>(A->rows + 1, A->rowptr.as<int64_t>(),
                                                               A->rowptr32.as<int32_t>());
  LFG_LAUNCHED(ctx);
  A->dinv.alloc(A->rows * sizeof(double), s);
  A->dinv32.alloc(A->rows * sizeof(float), s);
  ReadAndClearStatus(ctx);
  DiagKernel<<<GridFor(ctx, A->rows, 256), 256, 0, s>>>(A->rows, A->rowptr.as<int64_t>(), A->col.as<int32_t>(),
                                                        A->val.as<double>(), A->dinv.as<double>(),
                                                        A->dinv32.as<float>(), StatusWord(ctx));
  LFG_LAUNCHED(ctx);
  int32_t code = ReadAndClearStatus(ctx);
  if (code) {
    A->dinv.reset();
    Fail(LFG_INVALID_ARG, "Jacobi preconditioner: non-positive diagonal in row " + std::to_string(code - 1));
  }
}

void EnsureFloatValues(lfg_csr* A) {
  if (A->val32.p) return;
  lfg_ctx* ctx = A->ctx;
  A->val32.alloc(std::max<int64_t>(A->nnz, 1) * sizeof(float), ctx->stream);
  ToFloatKernel<<<GridFor(ctx, A->nnz, 256), 256, 0, ctx->stream>>>(A->nnz, A->val.as<double>(), A->val32.as<float>());
  LFG_LAUNCHED(ctx);
}

// PCG on A x = b in precision T (x holds the initial guess; the FP64 path
// starts from r = b - A x, the FP32 inner path from r = b with x = 0).
template <class T>
struct PcgState {
  DevBuf r, z, p, q;
  DevBuf pq, rz[2], rr;
  int nb = 0;
};

template <class T>
int RunPcg(lfg_csr* A, const T* val, const T* dinv, T* x, T* r_init_owner, int64_t n, double target_rr,
           int max_it, int check_every, PcgState<T>& S, double& rr_out) {
  // r is S.r (already filled); returns iterations done
  lfg_ctx* ctx = A->ctx;
  cudaStream_t s = ctx->stream;
  const int nb = S.nb;
  const int32_t* rp = A->rowptr32.as<int32_t>();
  const int32_t* col = A->col.as<int32_t>();
  const int spmv_blocks = nb;
  std::vector<double> tmp;
  PcgStartKernel<T><<<nb, kPcgBlock, 0, s>>>(n, dinv, S.r.template as<T>(), S.z.template as<T>(),
                                             S.p.template as<T>(), S.rz[0].template as<double>(),
                                             S.rr.template as<double>());
  LFG_LAUNCHED(ctx);
  double rr = HostSum(ctx, S.rr.template as<double>(), nb, tmp);
  int it = 0;
  if (rr <= target_rr) {
    rr_out = rr;
    return 0;
  }
  // capture `check_every` iterations (an even count: the two <r,z> buffers alternate)
  const int body = std::max(2, check_every + (check_every & 1));
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  LFG_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
  for (int k = 0; k < body; ++k) {
    double* rz_old = S.rz[k & 1].template as<double>();
    double* rz_new = S.rz[(k + 1) & 1].template as<double>();
    PcgSpmvKernel<T><<<spmv_blocks, kPcgBlock, 0, s>>>(n, rp, col, val, S.p.template as<T>(), S.q.template as<T>(),
                                                       S.pq.template as<double>());
    PcgUpdateKernel<T><<<nb, kPcgBlock, 0, s>>>(n, S.pq.template as<double>(), rz_old, nb, dinv, S.p.template as<T>(),
                                                S.q.template as<T>(), x, S.r.template as<T>(), S.z.template as<T>(),
                                                rz_new, S.rr.template as<double>());
    PcgDirectionKernel<T><<<nb, kPcgBlock, 0, s>>>(n, rz_new, rz_old, nb, S.z.template as<T>(), S.p.template as<T>());
  }
  cudaError_t ce = cudaStreamEndCapture(s, &graph);
  LFG_CUDA(ce);
  LFG_CUDA(cudaGraphInstantiate(&exec, graph, 0));
  try {
    while (it < max_it) {
      LFG_CUDA(cudaGraphLaunch(exec, s));
      CountLaunch(ctx, 3 * body);
      it += body;
      rr = HostSum(ctx, S.rr.template as<double>(), nb, tmp);
      if (!(rr > target_rr)) break;  // also stops on NaN
    }
  } catch (...) {
    cudaGraphExecDestroy(exec);
    cudaGraphDestroy(graph);
    throw;
  }
  cudaGraphExecDestroy(exec);
  cudaGraphDestroy(graph);
  rr_out = rr;
  return it;
}

template <class T>
void AllocState(lfg_ctx* ctx, int64_t n, PcgState<T>& S) {
  cudaStream_t s = ctx->stream;
  S.nb = std::max(1, std::min<int>(ctx->num_sms * 8, static_cast<int>((n + kPcgBlock - 1) / kPcgBlock)));
  S.r.alloc(n * sizeof(T), s);
  S.z.alloc(n * sizeof(T), s);
  S.p.alloc(n * sizeof(T), s);
  S.q.alloc(n * sizeof(T), s);
  S.pq.alloc(S.nb * sizeof(double), s);
  S.rz[0].alloc(S.nb * sizeof(double), s);
  S.rz[1].alloc(S.nb * sizeof(double), s);
  S.rr.alloc(S.nb * sizeof(double), s);
}

}  // namespace
}  // namespace lfg

using namespace lfg;

extern "C" {

lfg_status lfg_csr_from_coo(lfg_coo* coo, lfg_csr** out) {
  if (!coo) return LFG_INVALID_ARG;
  LFG_API_BEGIN(coo->ctx)
  if (!out) Fail(LFG_INVALID_ARG, "lfg_csr_from_coo: null output");
  if (coo->rows <= 0 || coo->cols <= 0)
    Fail(LFG_INVALID_ARG, "matrix has zero rows or columns, this is probably an error.");
  lfg_ctx* ctx = coo->ctx;
  cudaStream_t s = ctx->stream;
  const int64_t n = coo->size;
  if (n >= (int64_t(1) << 32)) Fail(LFG_UNSUPPORTED, "more than 2^32 triplets");
  auto* A = new lfg_csr;
  A->ref.Set(ctx);
  A->ctx = ctx;
  A->rows = coo->rows;
  A->cols = coo->cols;
  try {
    A->rowptr.alloc((A->rows + 1) * sizeof(int64_t), s);
    if (n == 0) {
      A->nnz = 0;
      RowPtrEmptyKernel<<<GridFor(ctx, A->rows + 1, 256), 256, 0, s>>>(A->rows, A->rowptr.as<int64_t>());
      LFG_LAUNCHED(ctx);
    } else {
      const int cbits = BitsFor(coo->cols), rbits = BitsFor(coo->rows);
      DevBuf keys, order, head;
      keys.alloc(n * sizeof(uint64_t), s);
      order.alloc(n * sizeof(uint32_t), s);
      ReadAndClearStatus(ctx);
      CooKeysKernel<<<GridFor(ctx, n, 256), 256, 0, s>>>(n, coo->d, cbits, keys.as<uint64_t>(), order.as<uint32_t>(),
                                                         StatusWord(ctx), coo->rows, coo->cols);
      LFG_LAUNCHED(ctx);
      if (ReadAndClearStatus(ctx)) Fail(LFG_INVALID_ARG, "triplet index out of range");
      RadixSortPairs(ctx, keys.as<uint64_t>(), order.as<uint32_t>(), n, rbits + cbits);
      head.alloc(n * sizeof(int64_t), s);
      HeadsKernel<<<GridFor(ctx, n, 256), 256, 0, s>>>(n, keys.as<uint64_t>(), head.as<int64_t>());
      LFG_LAUNCHED(ctx);
      A->nnz = ExclusiveScanI64(ctx, head.as<int64_t>(), head.as<int64_t>(), n);
      A->col.alloc(A->nnz * sizeof(int32_t), s);
      A->val.alloc(A->nnz * sizeof(double), s);
      DevBuf rows_of;
      rows_of.alloc(A->nnz * sizeof(int32_t), s);
      ReduceRunsKernel<<<GridFor(ctx, n, 256), 256, 0, s>>>(n, keys.as<uint64_t>(), order.as<uint32_t>(),
                                                            head.as<int64_t>(), coo->d, cbits, A->col.as<int32_t>(),
                                                            A->val.as<double>(), rows_of.as<int32_t>());
      LFG_LAUNCHED(ctx);
      RowPtrKernel<<<GridFor(ctx, A->nnz, 256), 256, 0, s>>>(A->nnz, rows_of.as<int32_t>(), A->rows,
                                                             A->rowptr.as<int64_t>());
      LFG_LAUNCHED(ctx);
    }
    LFG_CUDA(cudaStreamSynchronize(s));
  } catch (...) {
    delete A;
    throw;
  }
  *out = A;
  LFG_API_END
}

lfg_status lfg_csr_destroy(lfg_csr* A) {
  if (!A) return LFG_INVALID_ARG;
  cudaSetDevice(A->ctx->device);
  delete A;
  return LFG_OK;
}

lfg_status lfg_csr_info(const lfg_csr* A, int64_t* rows, int64_t* cols, int64_t* nnz) {
  if (!A) return LFG_INVALID_ARG;
  if (rows) *rows = A->rows;
  if (cols) *cols = A->cols;
  if (nnz) *nnz = A->nnz;
  return LFG_OK;
}

lfg_status lfg_csr_download(lfg_csr* A, int64_t* rowptr, int32_t* col, double* val) {
  if (!A) return LFG_INVALID_ARG;
  LFG_API_BEGIN(A->ctx)
  cudaStream_t s = A->ctx->stream;
  if (rowptr) LFG_CUDA(cudaMemcpyAsync(rowptr, A->rowptr.p, (A->rows + 1) * sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  if (col && A->nnz) LFG_CUDA(cudaMemcpyAsync(col, A->col.p, A->nnz * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
  if (val && A->nnz) LFG_CUDA(cudaMemcpyAsync(val, A->val.p, A->nnz * sizeof(double), cudaMemcpyDeviceToHost, s));
  LFG_CUDA(cudaStreamSynchronize(s));
  LFG_API_END
}

lfg_status lfg_csr_spmv(lfg_csr* A, const double* x, double* y) {
  if (!A) return LFG_INVALID_ARG;
  LFG_API_BEGIN(A->ctx)
  if (!x || !y) Fail(LFG_INVALID_ARG, "lfg_csr_spmv: null vector");
  if (A->nnz >= (int64_t(1) << 31)) Fail(LFG_UNSUPPORTED, "SpMV needs nnz < 2^31");
  lfg_ctx* ctx = A->ctx;
  if (!A->rowptr32.p) {
    A->rowptr32.alloc((A->rows + 1) * sizeof(int32_t), ctx->stream);
    RowPtr32Kernel<<<GridFor(ctx, A->rows + 1, 256), 256, 0, ctx->stream>>>(A->rows + 1, A->rowptr.as<int64_t>(),
                                                                            A->rowptr32.as<int32_t>());
    LFG_LAUNCHED(ctx);
  }
  SpmvKernel<<<GridFor(ctx, A->rows * kLanes, 256), 256, 0, ctx->stream>>>(
      A->rows, A->rowptr32.as<int32_t>(), A->col.as<int32_t>(), A->val.as<double>(), x, y);
  LFG_LAUNCHED(ctx);
  LFG_API_END
}

lfg_status lfg_solve_pcg(lfg_csr* A, const double* b, double* x, const lfg_solve_opts* opts,
                         lfg_solve_stats* stats) {
  if (!A) return LFG_INVALID_ARG;
  LFG_API_BEGIN(A->ctx)
  if (!b || !x || !opts) Fail(LFG_INVALID_ARG, "lfg_solve_pcg: null argument");
  if (A->rows != A->cols) Fail(LFG_INVALID_ARG, "matrix must be square");
  lfg_ctx* ctx = A->ctx;
  cudaStream_t s = ctx->stream;
  const int64_t n = A->rows;
  PrepareSolve(A);
  const int check = opts->check_every > 0 ? opts->check_every : 32;
  const int max_it = opts->max_iterations > 0 ? opts->max_iterations : 100000;
  const double rtol = opts->rtol > 0 ? opts->rtol : 1e-10;
  std::vector<double> tmp;
  lfg_solve_stats st{};
  // ||b||
  DevBuf rb;
  PcgState<double> S64;
  AllocState(ctx, n, S64);
  const int nb = S64.nb;
  const int rblocks = nb;
  // r = b - A*0 to get ||b||
  {
    DevBuf zero;
    zero.alloc(n * sizeof(double), s);
    LFG_CUDA(cudaMemsetAsync(zero.p, 0, n * sizeof(double), s));
    ResidualKernel<<<rblocks, kPcgBlock, 0, s>>>(n, A->rowptr32.as<int32_t>(), A->col.as<int32_t>(), A->val.as<double>(),
                                                 zero.as<double>(), b, S64.r.as<double>(), S64.rr.as<double>());
    LFG_LAUNCHED(ctx);
  }
  const double bb = HostSum(ctx, S64.rr.as<double>(), nb, tmp);
  const double bnorm = std::sqrt(bb);
  ResidualKernel<<<rblocks, kPcgBlock, 0, s>>>(n, A->rowptr32.as<int32_t>(), A->col.as<int32_t>(), A->val.as<double>(),
                                               x, b, S64.r.as<double>(), S64.rr.as<double>());
  LFG_LAUNCHED(ctx);
  double rr = HostSum(ctx, S64.rr.as<double>(), nb, tmp);
  const double target = (rtol * bnorm) * (rtol * bnorm);
  if (bnorm == 0.0) {
    LFG_CUDA(cudaMemsetAsync(x, 0, n * sizeof(double), s));
    st.converged = 1;
    st.rel_residual = 0.0;
  } else if (opts->precision == LFG_SOLVE_FP64) {
    // The recursively updated residual drifts from b - A x near rounding
    // level; when it reports convergence but the true residual does not,
    // restart from the true residual (kept only while each restart gains at
    // least a factor 2 in the residual norm).
    int total = 0, restarts = 0;
    double rr_prev = rr;
    while (true) {
      double rr_end = rr;
      total += RunPcg<double>(A, A->val.as<double>(), A->dinv.as<double>(), x, nullptr, n, target, max_it - total,
                              check, S64, rr_end);
      ++restarts;
      ResidualKernel<<<rblocks, kPcgBlock, 0, s>>>(n, A->rowptr32.as<int32_t>(), A->col.as<int32_t>(),
                                                   A->val.as<double>(), x, b, S64.r.as<double>(), S64.rr.as<double>());
      LFG_LAUNCHED(ctx);
      rr = HostSum(ctx, S64.rr.as<double>(), nb, tmp);
      if (rr <= target || total >= max_it || restarts >= 16 || !(rr < 0.25 * rr_prev)) break;
      rr_prev = rr;
    }
    st.iterations = total;
    st.rel_residual = std::sqrt(rr) / bnorm;
    st.converged = st.rel_residual <= rtol * 1.0000001 || rr <= target;
    st.refinements = restarts;
  } else if (opts->precision == LFG_SOLVE_MIXED) {
    EnsureFloatValues(A);
    PcgState<float> S32;
    AllocState(ctx, n, S32);
    DevBuf d32;
    d32.alloc(n * sizeof(float), s);
    const double inner = opts->inner_rtol > 0 ? opts->inner_rtol : 1e-4;
    int total = 0, outer = 0;
    while (total < max_it && outer < 200) {
      const double rnorm = std::sqrt(rr);
      if (rr <= target) break;
      // inner FP32 PCG on A d = r / ||r||
      const double scale = 1.0 / rnorm;
      ScaleToFloatKernel<<<GridFor(ctx, n, 256), 256, 0, s>>>(n, S64.r.as<double>(), scale, S32.r.as<float>(),
                                                              d32.as<float>());
      LFG_LAUNCHED(ctx);
      // inner target relative to ||r/||r|| || = 1, but never below what the outer loop needs
      const double need = std::max(inner, 0.5 * std::sqrt(target) / rnorm);
      double rr_in = 0.0;
      const int it = RunPcg<float>(A, A->val32.as<float>(), A->dinv32.as<float>(), d32.as<float>(), nullptr, n,
                                   need * need, max_it - total, check, S32, rr_in);
      total += std::max(it, 1);
      AddCorrectionKernel<<<GridFor(ctx, n, 256), 256, 0, s>>>(n, d32.as<float>(), rnorm, x);
      LFG_LAUNCHED(ctx);
      ResidualKernel<<<rblocks, kPcgBlock, 0, s>>>(n, A->rowptr32.as<int32_t>(), A->col.as<int32_t>(),
                                                   A->val.as<double>(), x, b, S64.r.as<double>(), S64.rr.as<double>());
      LFG_LAUNCHED(ctx);
      const double rr_new = HostSum(ctx, S64.rr.as<double>(), nb, tmp);
      ++outer;
      if (!(rr_new < rr)) {  // stagnation: no progress in FP32
        rr = rr_new;
        break;
      }
      rr = rr_new;
    }
    st.iterations = total;
    st.refinements = outer;
    st.rel_residual = std::sqrt(rr) / bnorm;
    st.converged = rr <= target;
  } else {
    Fail(LFG_INVALID_ARG, "unknown solve precision");
  }
  if (stats) *stats = st;
  if (!st.converged) {
    char buf[128];
    std::snprintf(buf, sizeof(buf), "PCG not converged: rel. residual %.3e after %d iterations", st.rel_residual,
                  st.iterations);
    Fail(LFG_NOT_CONVERGED, buf);
  }
  LFG_API_END
}

}  // extern "C"
