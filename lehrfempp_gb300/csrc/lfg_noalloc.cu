// lfg_solve_pcg_noalloc: the FP64 Jacobi-PCG of lfg_solve_pcg without any
// device-memory allocation.
//
// Why it exists: lfg_solve_pcg allocates its work vectors (residual, search
// direction, preconditioned residual, A*p, Jacobi diagonal) on every call.
// Some callers cannot let a library allocate: applications that hand the GPU
// a fixed memory budget owned by their own allocator, long-running services
// that must not grow or fragment the CUDA memory pool between time steps, and
// code that must not risk the implicit device-wide synchronisation or the
// late out-of-memory failure that cudaMalloc/cudaFree can bring in the middle
// of a time loop.  This entry point keeps all of its scratch in one
// file-scope device array of fixed size, reserved when the library is loaded.
//
// Limits and sharing rules (also stated in include/lfg.h):
//   - at most kNoAllocMaxRows = 1,048,576 matrix rows; larger systems are
//     rejected with LFG_CAPACITY before any work is done;
//   - the scratch array (40 MiB + 32 KiB) is held by every GPU that loads the
//     library until the process exits;
//   - all calls share the one array and it keeps the previous call's
//     contents; every vector is written before it is read and the zero vector
//     is cleared on each call.  Calls that overlap on the GPU (two contexts or
//     streams on the same device at the same time) race on the array;
//   - the first call on a device looks up the array's device address with
//     cudaGetSymbolAddress (with that device current) and caches it; make that
//     first call before any stream capture.
// The arithmetic, grid shape, reduction order and convergence-check cadence
// are those of lfg_solve_pcg in FP64 mode, so both give the same iterates.
#include <cmath>
#include <cstdio>
#include <mutex>

#include "lfg_api.h"
#include "lfg_internal.h"

namespace lfg {
namespace {

constexpr int64_t kNoAllocMaxRows = int64_t(1) << 20;
constexpr int kNoAllocMaxBlocks = 1024;
constexpr int kBlock = 256;
constexpr int kLanes = 8;
// r, z, p, q, dinv (one row each) + pq, rz[0], rz[1], rr block partials
constexpr size_t kScratchDoubles = 5 * static_cast<size_t>(kNoAllocMaxRows) + 4 * kNoAllocMaxBlocks;

static __device__ __align__(256) double g_pcg_scratch[kScratchDoubles];

constexpr int kMaxDevices = 64;
double* g_scratch_addr[kMaxDevices] = {nullptr};
std::mutex g_scratch_mutex;

// Device address of g_pcg_scratch for the current device (looked up once).
double* ScratchFor(int device) {
  if (device < 0 || device >= kMaxDevices) Fail(LFG_INVALID_ARG, "device index out of range");
  std::lock_guard<std::mutex> lock(g_scratch_mutex);
  if (!g_scratch_addr[device]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_pcg_scratch);
    if (e != cudaSuccess) {
      cudaGetLastError();
      Fail(LFG_CUDA_ERROR, std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
    }
    g_scratch_addr[device] = static_cast<double*>(p);
  }
  return g_scratch_addr[device];
}

__device__ __forceinline__ double RowDot64(const int64_t* __restrict__ rp, const int32_t* __restrict__ col,
                                           const double* __restrict__ val, const double* __restrict__ x,
                                           int64_t r, int64_t rows, int sub) {
  double s = 0.0;
  if (r < rows)
    for (int64_t q = rp[r] + sub; q < rp[r + 1]; q += kLanes) s = fma(val[q], x[col[q]], s);
#pragma unroll
  for (int o = kLanes / 2; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o, kLanes);
  return s;
}

#define NOALLOC_ROW_LOOP(r)                                                                      \
  const int sub = threadIdx.x % kLanes;                                                          \
  const int64_t warp_id = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) >> 5;    \
  const int64_t nwarps = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;                   \
  const int grp = (threadIdx.x & 31) / kLanes;                                                   \
  for (int64_t wb = warp_id * (32 / kLanes); wb < rows; wb += nwarps * (32 / kLanes))            \
    for (int64_t r = wb + grp, once = 0; once < 1; ++once)

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

__global__ void NaDiagKernel(int64_t rows, const int64_t* __restrict__ rp, const int32_t* __restrict__ col,
                             const double* __restrict__ val, double* __restrict__ dinv, int32_t* st) {
  for (int64_t r = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; r < rows;
       r += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    double d = 0.0;
    for (int64_t q = rp[r]; q < rp[r + 1]; ++q)
      if (col[q] == r) d = val[q];
    if (!(d > 0.0)) atomicCAS(st, 0, static_cast<int>(r) + 1);
    dinv[r] = d > 0.0 ? 1.0 / d : 0.0;
  }
}

__global__ void __launch_bounds__(kBlock) NaResidualKernel(int64_t rows, const int64_t* __restrict__ rp,
                                                           const int32_t* __restrict__ col,
                                                           const double* __restrict__ val,
                                                           const double* __restrict__ x,
                                                           const double* __restrict__ b, double* __restrict__ res,
                                                           double* __restrict__ part) {
  __shared__ double red[32];
  double acc = 0.0;
  NOALLOC_ROW_LOOP(i) {
    const double s = RowDot64(rp, col, val, x, i, rows, sub);
    if (sub == 0 && i < rows) {
      const double ri = b[i] - s;
      res[i] = ri;
      acc = fma(ri, ri, acc);
    }
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < (blockDim.x >> 5); ++w) s += red[w];
    part[blockIdx.x] = s;
  }
}

__global__ void __launch_bounds__(kBlock) NaStartKernel(int64_t rows, const double* __restrict__ dinv,
                                                        const double* __restrict__ r, double* __restrict__ z,
                                                        double* __restrict__ p, double* __restrict__ rz_part,
                                                        double* __restrict__ rr_part) {
  __shared__ double red[32];
  double arz = 0.0, arr = 0.0;
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < rows;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const double ri = r[i];
    const double zi = dinv[i] * ri;
    z[i] = zi;
    p[i] = zi;
    arz = fma(ri, zi, arz);
    arr = fma(ri, ri, arr);
  }
  const double s1 = BlockSum(arz, red);
  const double s2 = BlockSum(arr, red);
  if (threadIdx.x == 0) {
    rz_part[blockIdx.x] = s1;
    rr_part[blockIdx.x] = s2;
  }
}

__global__ void __launch_bounds__(kBlock) NaSpmvDotKernel(int64_t rows, const int64_t* __restrict__ rp,
                                                          const int32_t* __restrict__ col,
                                                          const double* __restrict__ val,
                                                          const double* __restrict__ p, double* __restrict__ q,
                                                          double* __restrict__ part) {
  __shared__ double red[32];
  double acc = 0.0;
  NOALLOC_ROW_LOOP(i) {
    const double s = RowDot64(rp, col, val, p, i, rows, sub);
    if (sub == 0 && i < rows) {
      q[i] = s;
      acc = fma(p[i], s, acc);
    }
  }
  const double tot = BlockSum(acc, red);
  if (threadIdx.x == 0) part[blockIdx.x] = tot;
}

__global__ void __launch_bounds__(kBlock) NaUpdateKernel(int64_t rows, const double* __restrict__ pq_part,
                                                         const double* __restrict__ rz_old_part, int nparts,
                                                         const double* __restrict__ dinv,
                                                         const double* __restrict__ p, const double* __restrict__ q,
                                                         double* __restrict__ x, double* __restrict__ r,
                                                         double* __restrict__ z, double* __restrict__ rz_part,
                                                         double* __restrict__ rr_part) {
  __shared__ double red[32];
  const double pq = SumPartials(pq_part, nparts, red);
  const double rz = SumPartials(rz_old_part, nparts, red);
  const double alpha = pq != 0.0 ? rz / pq : 0.0;
  double arz = 0.0, arr = 0.0;
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < rows;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    x[i] = fma(alpha, p[i], x[i]);
    const double ri = fma(-alpha, q[i], r[i]);
    r[i] = ri;
    const double zi = dinv[i] * ri;
    z[i] = zi;
    arz = fma(ri, zi, arz);
    arr = fma(ri, ri, arr);
  }
  const double s1 = BlockSum(arz, red);
  const double s2 = BlockSum(arr, red);
  if (threadIdx.x == 0) {
    rz_part[blockIdx.x] = s1;
    rr_part[blockIdx.x] = s2;
  }
}

__global__ void __launch_bounds__(kBlock) NaDirectionKernel(int64_t rows, const double* __restrict__ rz_new_part,
                                                            const double* __restrict__ rz_old_part, int nparts,
                                                            const double* __restrict__ z, double* __restrict__ p) {
  __shared__ double red[32];
  const double rn = SumPartials(rz_new_part, nparts, red);
  const double ro = SumPartials(rz_old_part, nparts, red);
  const double beta = ro != 0.0 ? rn / ro : 0.0;
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < rows;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x)
    p[i] = fma(beta, p[i], z[i]);
}

// Sums block partials in index order on one thread (same order as the host
// sum of lfg_solve_pcg) into out[0].
__global__ void NaFinalSumKernel(const double* __restrict__ part, int n, double* out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double s = 0.0;
    for (int i = 0; i < n; ++i) s += part[i];
    out[0] = s;
  }
}

}  // namespace
}  // namespace lfg

using namespace lfg;

extern "C" {

lfg_status lfg_solve_pcg_noalloc(lfg_csr* A, const double* b, double* x, const lfg_solve_opts* opts,
                                 lfg_solve_stats* stats) {
  if (!A) return LFG_INVALID_ARG;
  LFG_API_BEGIN(A->ctx)
  if (!b || !x || !opts) Fail(LFG_INVALID_ARG, "lfg_solve_pcg_noalloc: null argument");
  if (opts->precision != LFG_SOLVE_FP64)
    Fail(LFG_UNSUPPORTED, "lfg_solve_pcg_noalloc solves in FP64 only");
  if (A->rows != A->cols) Fail(LFG_INVALID_ARG, "matrix must be square");
  if (A->rows > kNoAllocMaxRows)
    Fail(LFG_CAPACITY, "lfg_solve_pcg_noalloc handles at most " + std::to_string(kNoAllocMaxRows) +
                           " rows; this matrix has " + std::to_string(A->rows) + " (use lfg_solve_pcg)");
  lfg_ctx* ctx = A->ctx;
  cudaStream_t s = ctx->stream;
  const int64_t n = A->rows;
  double* base = ScratchFor(ctx->device);
  double* r = base;
  double* z = r + kNoAllocMaxRows;
  double* p = z + kNoAllocMaxRows;
  double* q = p + kNoAllocMaxRows;
  double* dinv = q + kNoAllocMaxRows;
  double* pq = dinv + kNoAllocMaxRows;
  double* rz[2] = {pq + kNoAllocMaxBlocks, pq + 2 * kNoAllocMaxBlocks};
  double* rr = pq + 3 * kNoAllocMaxBlocks;
  const int nb = std::max(1, std::min<int>(ctx->num_sms * 8, static_cast<int>((n + kBlock - 1) / kBlock)));
  if (nb > kNoAllocMaxBlocks - 1) Fail(LFG_UNSUPPORTED, "too many SMs for the scratch partial arrays");
  const int64_t* rp = A->rowptr.as<int64_t>();
  const int32_t* col = A->col.as<int32_t>();
  const double* val = A->val.as<double>();
  const int check = opts->check_every > 0 ? opts->check_every : 32;
  const int max_it = opts->max_iterations > 0 ? opts->max_iterations : 100000;
  const double rtol = opts->rtol > 0 ? opts->rtol : 1e-10;
  double* total_dev = rr + kNoAllocMaxBlocks - 1;  // last slot of the rr partial array (never a partial: nb < max)
  auto sum_partials = [&](const double* part) {
    NaFinalSumKernel<<<1, 32, 0, s>>>(part, nb, total_dev);
    LFG_LAUNCHED(ctx);
    double v = 0.0;
    D2HSync(ctx, &v, total_dev, sizeof(double));
    return v;
  };
  // Jacobi diagonal
  ReadAndClearStatus(ctx);
  NaDiagKernel<<<GridFor(ctx, n, 256), 256, 0, s>>>(n, rp, col, val, dinv, StatusWord(ctx));
  LFG_LAUNCHED(ctx);
  if (int32_t code = ReadAndClearStatus(ctx))
    Fail(LFG_INVALID_ARG, "Jacobi preconditioner: non-positive diagonal in row " + std::to_string(code - 1));
  // ||b|| from r = b - A*0 (q is cleared to serve as the zero vector)
  LFG_CUDA(cudaMemsetAsync(q, 0, n * sizeof(double), s));
  NaResidualKernel<<<nb, kBlock, 0, s>>>(n, rp, col, val, q, b, r, rr);
  LFG_LAUNCHED(ctx);
  const double bnorm = std::sqrt(sum_partials(rr));
  lfg_solve_stats st{};
  st.refinements = 1;
  if (bnorm == 0.0) {
    LFG_CUDA(cudaMemsetAsync(x, 0, n * sizeof(double), s));
    st.converged = 1;
  } else {
    const double target = (rtol * bnorm) * (rtol * bnorm);
    NaResidualKernel<<<nb, kBlock, 0, s>>>(n, rp, col, val, x, b, r, rr);
    LFG_LAUNCHED(ctx);
    NaStartKernel<<<nb, kBlock, 0, s>>>(n, dinv, r, z, p, rz[0], rr);
    LFG_LAUNCHED(ctx);
    double rrv = sum_partials(rr);
    int it = 0;
    const int body = std::max(2, check + (check & 1));
    while (rrv > target && it < max_it) {
      for (int k = 0; k < body; ++k) {
        double* rz_old = rz[k & 1];
        double* rz_new = rz[(k + 1) & 1];
        NaSpmvDotKernel<<<nb, kBlock, 0, s>>>(n, rp, col, val, p, q, pq);
        NaUpdateKernel<<<nb, kBlock, 0, s>>>(n, pq, rz_old, nb, dinv, p, q, x, r, z, rz_new, rr);
        NaDirectionKernel<<<nb, kBlock, 0, s>>>(n, rz_new, rz_old, nb, z, p);
        CountLaunch(ctx, 3);
      }
      LFG_CUDA(cudaGetLastError());
      it += body;
      rrv = sum_partials(rr);
      if (!(rrv == rrv)) break;  // NaN
    }
    st.iterations = it;
    NaResidualKernel<<<nb, kBlock, 0, s>>>(n, rp, col, val, x, b, r, rr);
    LFG_LAUNCHED(ctx);
    rrv = sum_partials(rr);
    st.rel_residual = std::sqrt(rrv) / bnorm;
    st.converged = st.rel_residual <= rtol * 1.0000001 || rrv <= target;
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
