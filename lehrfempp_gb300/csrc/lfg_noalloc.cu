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
//   - the scratch array (40 MiB + 48 KiB) is held by every GPU that loads the
//     library until the process exits;
//   - all calls share the one array and it keeps the previous call's
//     contents; every vector is written before it is read, and the zero
//     vector and the scalar block (reduction counter included) are cleared on
//     each call.  Calls that overlap on the GPU (two contexts or streams on
//     the same device at the same time) race on the array;
//   - the first call on a device looks up the array's device address with
//     cudaGetSymbolAddress (with that device current) and caches it; make that
//     first call before any stream capture.
// The algorithm and the convergence test are those of lfg_solve_pcg in FP64
// mode (same three-kernel iteration, same check cadence, same restart from
// the true residual when the recursive one drifts).  The SpMV differs: this
// path reads the CSR arrays directly (eight lanes per row) because the SELL-32
// copy that lfg_solve_pcg builds would need an allocation, so the rounding of
// the two solvers differs and their iteration counts can differ slightly.
#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstdio>
#include <mutex>

#include "lfg_api.h"
#include "lfg_internal.h"

namespace lfg {
namespace {

constexpr int64_t kNoAllocMaxRows = int64_t(1) << 20;
constexpr int kNoAllocMaxBlocks = 2048;  // grids are clamped to this; every row loop is grid-stride
constexpr int kBlock = 256;
constexpr int kLanes = 8;

// Scalars of one run, on the device (same roles as lfg_solve_pcg's): rz[cur]
// is <r, z> of the current residual, the update kernel writes rz[cur ^ 1].
struct NaScalars {
  double rz[2];
  double alpha, beta, rr, pq, total;
  unsigned int counter;
  unsigned int pad;
};
constexpr size_t kScalarDoubles = (sizeof(NaScalars) + sizeof(double) - 1) / sizeof(double);

// Layout (in doubles): r, z, p, q, dinv (one row each), then the block
// partials of the iteration kernels (two per block), of the residual kernel
// (one per block), then the scalar block.
constexpr size_t kOffPart = 5 * static_cast<size_t>(kNoAllocMaxRows);
constexpr size_t kOffRes = kOffPart + 2 * kNoAllocMaxBlocks;
constexpr size_t kOffScal = kOffRes + kNoAllocMaxBlocks;
constexpr size_t kScratchDoubles = kOffScal + kScalarDoubles;

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

// Warp-uniform row loop: each warp owns 32 / kLanes consecutive rows per trip.
#define NOALLOC_ROW_LOOP(r)                                                                      \
  const int sub = threadIdx.x % kLanes;                                                          \
  const int64_t warp_id = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) >> 5;    \
  const int64_t nwarps = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;                   \
  const int grp = (threadIdx.x & 31) / kLanes;                                                   \
  for (int64_t wb = warp_id * (32 / kLanes); wb < rows; wb += nwarps * (32 / kLanes))            \
    for (int64_t r = wb + grp, once = 0; once < 1; ++once)

// Block sum (warp shuffles, then warps in order); result in thread 0.
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

// Publishes this block's partials (already written by thread 0) and tells
// whether this block finished last.  No block waits for another.
__device__ __forceinline__ bool FinishedLast(unsigned int* counter) {
  __shared__ bool last;
  if (threadIdx.x == 0) {
    __threadfence();
    last = atomicAdd(counter, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  return last;
}

// Sum of part[j * stride + off], j < n, in a fixed order; last block only.
__device__ double SumParts(const double* part, int n, int stride, int off, double* red) {
  double v = 0.0;
  for (int j = threadIdx.x; j < n; j += blockDim.x) v += __ldcg(part + static_cast<int64_t>(j) * stride + off);
  return BlockSum(v, red);
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

// r = b - A x with <r, r>: block partials, then the last block writes the
// sum to sc->total.
__global__ void __launch_bounds__(kBlock) NaResidualKernel(int64_t rows, const int64_t* __restrict__ rp,
                                                           const int32_t* __restrict__ col,
                                                           const double* __restrict__ val,
                                                           const double* __restrict__ x,
                                                           const double* __restrict__ b, double* __restrict__ res,
                                                           double* __restrict__ part, NaScalars* __restrict__ sc) {
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
  const double tot = BlockSum(acc, red);
  if (threadIdx.x == 0) part[blockIdx.x] = tot;
  if (FinishedLast(&sc->counter)) {
    const double s = SumParts(part, gridDim.x, 1, 0, red);
    if (threadIdx.x == 0) {
      sc->total = s;
      sc->counter = 0;
    }
  }
}

// z = D^-1 r, p = z, rz[0] = <r, z>, rr = <r, r>, beta = 0.
__global__ void __launch_bounds__(kBlock) NaStartKernel(int64_t rows, const double* __restrict__ dinv,
                                                        const double* __restrict__ r, double* __restrict__ z,
                                                        double* __restrict__ p, double* __restrict__ part,
                                                        NaScalars* __restrict__ sc) {
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
    part[2 * blockIdx.x] = s1;
    part[2 * blockIdx.x + 1] = s2;
  }
  if (FinishedLast(&sc->counter)) {
    const double rz = SumParts(part, gridDim.x, 2, 0, red);
    const double rr = SumParts(part, gridDim.x, 2, 1, red);
    if (threadIdx.x == 0) {
      sc->rz[0] = rz;
      sc->rz[1] = 0.0;
      sc->alpha = 0.0;
      sc->beta = 0.0;
      sc->rr = rr;
      sc->counter = 0;
    }
  }
}

// p = z + beta p.
__global__ void __launch_bounds__(kBlock) NaDirectionKernel(int64_t rows, const double* __restrict__ z,
                                                            double* __restrict__ p,
                                                            const NaScalars* __restrict__ sc) {
  const double beta = sc->beta;
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < rows;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x)
    p[i] = fma(beta, p[i], z[i]);
}

// q = A p and alpha = rz[cur] / <p, q>.
__global__ void __launch_bounds__(kBlock) NaSpmvDotKernel(int64_t rows, const int64_t* __restrict__ rp,
                                                          const int32_t* __restrict__ col,
                                                          const double* __restrict__ val,
                                                          const double* __restrict__ p, double* __restrict__ q,
                                                          int cur, double* __restrict__ part,
                                                          NaScalars* __restrict__ sc) {
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
  if (FinishedLast(&sc->counter)) {
    const double pq = SumParts(part, gridDim.x, 1, 0, red);
    if (threadIdx.x == 0) {
      sc->pq = pq;
      sc->alpha = pq != 0.0 ? sc->rz[cur] / pq : 0.0;
      sc->counter = 0;
    }
  }
}

// x += alpha p; r -= alpha q; z = D^-1 r; rz[cur ^ 1] = <r, z>, beta, and
// rr = <r, r> on the last iteration of a check period (with_rr).
__global__ void __launch_bounds__(kBlock) NaUpdateKernel(int64_t rows, const double* __restrict__ dinv,
                                                         const double* __restrict__ p, const double* __restrict__ q,
                                                         double* __restrict__ x, double* __restrict__ r,
                                                         double* __restrict__ z, int cur, bool with_rr,
                                                         double* __restrict__ part, NaScalars* __restrict__ sc) {
  __shared__ double red[32];
  const double alpha = sc->alpha;
  double arz = 0.0, arr = 0.0;
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < rows;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    x[i] = fma(alpha, p[i], x[i]);
    const double ri = fma(-alpha, q[i], r[i]);
    r[i] = ri;
    const double zi = dinv[i] * ri;
    z[i] = zi;
    arz = fma(ri, zi, arz);
    if (with_rr) arr = fma(ri, ri, arr);
  }
  const double s1 = BlockSum(arz, red);
  const double s2 = with_rr ? BlockSum(arr, red) : 0.0;
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = s1;
    part[2 * blockIdx.x + 1] = s2;
  }
  if (FinishedLast(&sc->counter)) {
    const double rz = SumParts(part, gridDim.x, 2, 0, red);
    const double rr = with_rr ? SumParts(part, gridDim.x, 2, 1, red) : 0.0;
    if (threadIdx.x == 0) {
      const double rz_old = sc->rz[cur];
      sc->rz[cur ^ 1] = rz;
      sc->beta = rz_old != 0.0 ? rz / rz_old : 0.0;
      if (with_rr) sc->rr = rr;
      sc->counter = 0;
    }
  }
}

double ReadScalar(lfg_ctx* ctx, const NaScalars* sc, size_t offset) {
  double v = 0.0;
  D2HSync(ctx, &v, reinterpret_cast<const char*>(sc) + offset, sizeof(double));
  return v;
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
  double* part = base + kOffPart;
  double* res = base + kOffRes;
  NaScalars* sc = reinterpret_cast<NaScalars*>(base + kOffScal);
  const int nb = static_cast<int>(std::clamp<int64_t>(
      std::min<int64_t>(static_cast<int64_t>(ctx->num_sms) * 8, (n + kBlock - 1) / kBlock), 1, kNoAllocMaxBlocks));
  const int64_t* rp = A->rowptr.as<int64_t>();
  const int32_t* col = A->col.as<int32_t>();
  const double* val = A->val.as<double>();
  const int check = opts->check_every > 0 ? opts->check_every : 32;
  const int max_it = opts->max_iterations > 0 ? opts->max_iterations : 100000;
  const double rtol = opts->rtol > 0 ? opts->rtol : 1e-10;
  // The array keeps the last call's contents: start from a cleared scalar
  // block (its reduction counter must be zero).
  LFG_CUDA(cudaMemsetAsync(sc, 0, sizeof(NaScalars), s));
  auto residual = [&]() {  // r = b - A x, returns <r, r>
    NaResidualKernel<<<nb, kBlock, 0, s>>>(n, rp, col, val, x, b, r, res, sc);
    LFG_LAUNCHED(ctx);
    return ReadScalar(ctx, sc, offsetof(NaScalars, total));
  };
  // Jacobi diagonal
  ReadAndClearStatus(ctx);
  NaDiagKernel<<<GridFor(ctx, n, 256), 256, 0, s>>>(n, rp, col, val, dinv, StatusWord(ctx));
  LFG_LAUNCHED(ctx);
  if (int32_t code = ReadAndClearStatus(ctx))
    Fail(LFG_INVALID_ARG, "Jacobi preconditioner: non-positive diagonal in row " + std::to_string(code - 1));
  // ||b|| from r = b - A*0 (q is cleared to serve as the zero vector)
  LFG_CUDA(cudaMemsetAsync(q, 0, n * sizeof(double), s));
  NaResidualKernel<<<nb, kBlock, 0, s>>>(n, rp, col, val, q, b, r, res, sc);
  LFG_LAUNCHED(ctx);
  const double bnorm = std::sqrt(ReadScalar(ctx, sc, offsetof(NaScalars, total)));
  lfg_solve_stats st{};
  if (bnorm == 0.0) {
    LFG_CUDA(cudaMemsetAsync(x, 0, n * sizeof(double), s));
    st.converged = 1;
  } else {
    const double target = (rtol * bnorm) * (rtol * bnorm);
    const int body = std::max(2, check + (check & 1));
    double rr = residual();
    // Same restart rule as lfg_solve_pcg: when the recursive residual reports
    // convergence but the true one does not, restart from the true residual,
    // kept while each restart gains at least a factor 2 in the residual norm.
    int total = 0, restarts = 0;
    double rr_prev = rr;
    while (true) {
      NaStartKernel<<<nb, kBlock, 0, s>>>(n, dinv, r, z, p, part, sc);
      LFG_LAUNCHED(ctx);
      double rr_rec = ReadScalar(ctx, sc, offsetof(NaScalars, rr));
      while (rr_rec > target && total < max_it) {
        for (int k = 0; k < body; ++k) {
          const int cur = k & 1;
          NaDirectionKernel<<<nb, kBlock, 0, s>>>(n, z, p, sc);
          NaSpmvDotKernel<<<nb, kBlock, 0, s>>>(n, rp, col, val, p, q, cur, part, sc);
          NaUpdateKernel<<<nb, kBlock, 0, s>>>(n, dinv, p, q, x, r, z, cur, k == body - 1, part, sc);
          CountLaunch(ctx, 3);
        }
        LFG_CUDA(cudaGetLastError());
        total += body;
        rr_rec = ReadScalar(ctx, sc, offsetof(NaScalars, rr));
        if (!(rr_rec == rr_rec)) break;  // NaN
      }
      ++restarts;
      rr = residual();
      if (rr <= target || total >= max_it || restarts >= 16 || !(rr < 0.25 * rr_prev)) break;
      rr_prev = rr;
    }
    st.iterations = total;
    st.refinements = restarts;
    st.rel_residual = std::sqrt(rr) / bnorm;
    st.converged = st.rel_residual <= rtol * 1.0000001 || rr <= target;
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
