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
// The solver keeps every scalar on the device.  A PCG iteration is three
// kernels: (1) the search direction p = z + beta p; (2) q = A p over a SELL-32
// copy of the matrix (one thread per row, the row's entries stored
// column-major across the warp, so every load of a slice is coalesced and a
// thread's loads are independent) with <p, q> -> alpha; (3) x += alpha p,
// r -= alpha q, z = D^-1 r with <r, z> -> beta (and <r, r> on the last
// iteration of a graph replay).  Each kernel's block partials are summed by
// the last block to finish (counter + fence), in block order, so alpha and
// beta are deterministic and computed once; the next kernel reads them from
// device memory.  The iteration body is captured in a CUDA graph replayed
// `check_every` iterations at a time; the host reads one residual norm per
// replay.  (Forming p inside the SpMV instead -- recomputing neighbour values
// -- doubles the gathers and measured slower in FP32 and FP64.)
#include <algorithm>
#include <cstddef>
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
constexpr double kDefaultInnerRtol = 1e-4;  // mixed: relative reduction per inner FP32 solve
constexpr int kSlice = 32;

// Scalars of one PCG run, on the device.  rz[cur] is <r, z> of the current
// residual; the update kernel writes rz[cur ^ 1].
struct PcgScalars {
  double rz[2];
  double alpha, beta, rr, pq;
  double trr;  // <t, t> of the true residual t = rhs - A x (inner FP32 solves, gap monitor)
  unsigned int counter;
  unsigned int pad;
};

// Block sum of v (warp shuffles, then warps in order); result in thread 0.
__device__ __forceinline__ double BlockSum(double v, double* red) {
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

// Sum of part[j * stride + off], j < n, in a fixed order (per-thread strided
// sums, then BlockSum); called by the last block only.
__device__ double SumParts(const double* part, int n, int stride, int off, double* red) {
  double v = 0.0;
  for (int j = threadIdx.x; j < n; j += blockDim.x) v += __ldcg(part + static_cast<int64_t>(j) * stride + off);
  return BlockSum(v, red);
}

// Per-thread dot-product accumulator: FP64 for FP64 vectors; for FP32
// vectors a float sum of the thread's few terms, widened once (every FP32 ->
// FP64 conversion and FP64 FMA runs on GB300's narrow FP64 pipe).
template <class T>
struct DotAcc {
  double v = 0.0;
  __device__ void add(T a, T b) { v = fma(a, b, v); }
  __device__ double get() const { return v; }
};
template <>
struct DotAcc<float> {
  float v = 0.0f;
  __device__ void add(float a, float b) { v = fmaf(a, b, v); }
  __device__ double get() const { return static_cast<double>(v); }
};

// One row of q = A p over the SELL copy.  With `rowsum` (the FP32 copy of
// the mixed solver) the row is applied in difference form,
//     (A p)_r = sum_k a_rk (p_k - p_r) + s_r p_r,   s_r = sum_k a_rk (FP64),
// so that rounding the entries to FP32 perturbs each term relative to the
// differences p_k - p_r: the FP32 operator then stays close to A on the
// smooth, small-eigenvalue modes even when cond(A) times the FP32 unit
// roundoff exceeds 1 (rounding the entries alone shifts each row's sum by
// about that much).  The diagonal entry drops out (p_r - p_r = 0).
template <class T>
__device__ __forceinline__ T SellRow(const int32_t* __restrict__ cp, const T* __restrict__ vp, int w,
                                     const T* __restrict__ p, int64_t r, const T* __restrict__ rowsum) {
  T sum = T(0);
  if (rowsum) {
    const T pr = p[r];
#pragma unroll 4
    for (int k = 0; k < w; ++k) sum = fma(vp[k * kSlice], p[cp[k * kSlice]] - pr, sum);
    return fma(rowsum[r], pr, sum);
  }
#pragma unroll 4
  for (int k = 0; k < w; ++k) sum = fma(vp[k * kSlice], p[cp[k * kSlice]], sum);
  return sum;
}

// q = A p (SELL-32) and alpha = rz[cur] / <p, q>.
template <class T>
__global__ void __launch_bounds__(kPcgBlock) PcgSpmvKernel(int64_t rows, int64_t nslices,
                                                           const int64_t* __restrict__ sptr,
                                                           const int32_t* __restrict__ scol, const T* __restrict__ sval,
                                                           const T* __restrict__ rowsum,
                                                           const T* __restrict__ p, T* __restrict__ q, int cur,
                                                           double* __restrict__ part, PcgScalars* __restrict__ sc) {
  __shared__ double red[32];
  const int lane = threadIdx.x & 31;
  const int64_t warp = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) >> 5;
  const int64_t nwarps = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
  DotAcc<T> acc;
  for (int64_t sl = warp; sl < nslices; sl += nwarps) {
    const int64_t r = sl * kSlice + lane;
    const int64_t b0 = sptr[sl];
    const int w = static_cast<int>((sptr[sl + 1] - b0) / kSlice);
    if (r < rows) {
      const T sum = SellRow<T>(scol + b0 + lane, sval + b0 + lane, w, p, r, rowsum);
      q[r] = sum;
      acc.add(p[r], sum);
    }
  }
  const double tot = BlockSum(acc.get(), red);
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

// x += alpha p; r -= alpha q; z = D^-1 r; rz[cur ^ 1] = <r, z>, rr = <r, r>
// (only when with_rr: the host reads it once per graph replay), beta =
// rz[cur ^ 1] / rz[cur].  Several elements per thread and trip, loads
// first, so each thread keeps several independent loads in flight.
template <class T>
__global__ void __launch_bounds__(kPcgBlock, 4) PcgUpdateKernel(int64_t rows, const T* __restrict__ dinv,
                                                             const T* __restrict__ p, const T* __restrict__ q,
                                                             T* __restrict__ x, T* __restrict__ r,
                                                             T* __restrict__ z, int cur, bool with_rr,
                                                             double* __restrict__ part, PcgScalars* __restrict__ sc) {
  __shared__ double red[32];
  __shared__ T salpha;
  if (threadIdx.x == 0) salpha = static_cast<T>(sc->alpha);
  __syncthreads();
  const T alpha = salpha;
  DotAcc<T> arz, arr;
  constexpr int U = sizeof(T) == 8 ? 2 : 4;  // elements per thread and trip
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t i0 = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i0 < rows; i0 += U * stride) {
    T pv[U], qv[U], xv[U], rv[U], dv[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int64_t i = i0 + u * stride;
      if (i < rows) {
        pv[u] = p[i]; qv[u] = q[i]; xv[u] = x[i]; rv[u] = r[i]; dv[u] = dinv[i];
      }
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int64_t i = i0 + u * stride;
      if (i < rows) {
        x[i] = fma(alpha, pv[u], xv[u]);
        const T ri = fma(-alpha, qv[u], rv[u]);
        r[i] = ri;
        const T zi = dv[u] * ri;
        z[i] = zi;
        arz.add(ri, zi);
        if (with_rr) arr.add(ri, ri);
      }
    }
  }
  const double s1 = BlockSum(arz.get(), red);
  const double s2 = with_rr ? BlockSum(arr.get(), red) : 0.0;
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

// p = z + beta p.
template <class T>
__global__ void __launch_bounds__(kPcgBlock) PcgDirectionKernel(int64_t rows, const T* __restrict__ z,
                                                                T* __restrict__ p, const PcgScalars* __restrict__ sc) {
  __shared__ T sbeta;
  if (threadIdx.x == 0) sbeta = static_cast<T>(sc->beta);
  __syncthreads();
  const T beta = sbeta;
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < rows;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x)
    p[i] = fma(beta, p[i], z[i]);
}

// z = D^-1 r, p = z (so the first direction update, with beta = 0, keeps
// p = z), rz[0] = <r, z>, rr = <r, r>.
template <class T>
__global__ void __launch_bounds__(kPcgBlock) PcgStartKernel(int64_t rows, const T* __restrict__ dinv,
                                                            const T* __restrict__ r, T* __restrict__ z,
                                                            T* __restrict__ p, double* __restrict__ part,
                                                            PcgScalars* __restrict__ sc) {
  __shared__ double red[32];
  double arz = 0.0, arr = 0.0;
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < rows;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const T ri = r[i];
    const T zi = dinv[i] * ri;
    z[i] = zi;
    p[i] = zi;
    arz = fma(static_cast<double>(ri), static_cast<double>(zi), arz);
    arr = fma(static_cast<double>(ri), static_cast<double>(ri), arr);
  }  // (once per run: FP64 accumulation regardless of T)
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
      sc->beta = 0.0;
      sc->alpha = 0.0;
      sc->rr = rr;
      sc->counter = 0;
    }
  }
}

// t = rhs - A x over the SELL copy in precision T; sc->trr = <t, t> (block
// partials, then the last block).  The inner FP32 solve runs it once per
// graph replay to see whether its recursively updated residual still tracks
// the true one.
template <class T>
__global__ void __launch_bounds__(kPcgBlock) PcgTrueResidualKernel(int64_t rows, int64_t nslices,
                                                                   const int64_t* __restrict__ sptr,
                                                                   const int32_t* __restrict__ scol,
                                                                   const T* __restrict__ sval,
                                                                   const T* __restrict__ rowsum,
                                                                   const T* __restrict__ x, const T* __restrict__ rhs,
                                                                   double* __restrict__ part,
                                                                   PcgScalars* __restrict__ sc) {
  __shared__ double red[32];
  const int lane = threadIdx.x & 31;
  const int64_t warp = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) >> 5;
  const int64_t nwarps = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
  DotAcc<T> acc;
  for (int64_t sl = warp; sl < nslices; sl += nwarps) {
    const int64_t r = sl * kSlice + lane;
    const int64_t b0 = sptr[sl];
    const int w = static_cast<int>((sptr[sl + 1] - b0) / kSlice);
    if (r < rows) {
      const T t = rhs[r] - SellRow<T>(scol + b0 + lane, sval + b0 + lane, w, x, r, rowsum);
      acc.add(t, t);
    }
  }
  const double tot = BlockSum(acc.get(), red);
  if (threadIdx.x == 0) part[blockIdx.x] = tot;
  if (FinishedLast(&sc->counter)) {
    const double v = SumParts(part, gridDim.x, 1, 0, red);
    if (threadIdx.x == 0) {
      sc->trr = v;
      sc->counter = 0;
    }
  }
}

// SELL-32 construction: width of each slice (longest row, times 32)...
__global__ void SellWidthKernel(int64_t rows, int64_t nslices, const int64_t* __restrict__ rp,
                                int64_t* __restrict__ width) {
  for (int64_t sl = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; sl < nslices;
       sl += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    int64_t w = 0;
    for (int l = 0; l < kSlice; ++l) {
      const int64_t r = sl * kSlice + l;
      if (r < rows) w = max(w, rp[r + 1] - rp[r]);
    }
    width[sl] = w * kSlice;
  }
}

// ... and the entries, column-major per slice; padding entries point at the
// row itself with value 0.
__global__ void SellFillKernel(int64_t rows, const int64_t* __restrict__ rp, const int32_t* __restrict__ col,
                               const double* __restrict__ val, const int64_t* __restrict__ sptr,
                               int32_t* __restrict__ scol, double* __restrict__ sval) {
  for (int64_t r = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; r < rows;
       r += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int64_t sl = r / kSlice, lane = r % kSlice;
    const int64_t b0 = sptr[sl] + lane;
    const int w = static_cast<int>((sptr[sl + 1] - sptr[sl]) / kSlice);
    const int64_t a = rp[r], len = rp[r + 1] - a;
    for (int k = 0; k < w; ++k) {
      const bool in = k < len;
      scol[b0 + static_cast<int64_t>(k) * kSlice] = in ? col[a + k] : static_cast<int32_t>(r);
      sval[b0 + static_cast<int64_t>(k) * kSlice] = in ? val[a + k] : 0.0;
    }
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

// s_r = sum_k a_rk in FP64 (left to right), rounded once to FP32.
__global__ void RowSumKernel(int64_t rows, const int64_t* __restrict__ rp, const double* __restrict__ val,
                             float* __restrict__ out) {
  for (int64_t r = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; r < rows;
       r += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    double s = 0.0;
    for (int64_t q = rp[r]; q < rp[r + 1]; ++q) s += val[q];
    out[r] = static_cast<float>(s);
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

__global__ void AddCorrectionKernel(int64_t n, float* __restrict__ d, double s, double* __restrict__ x) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    x[i] += static_cast<double>(d[i]) * s;
    d[i] = 0.0f;
  }
}

double HostSum(lfg_ctx* ctx, const double* part, int n, std::vector<double>& tmp) {
  tmp.resize(n);
  LFG_CUDA(cudaMemcpyAsync(tmp.data(), part, n * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  LFG_CUDA(cudaStreamSynchronize(ctx->stream));
  double s = 0.0;
  for (double v : tmp) s += v;
  return s;
}

}  // namespace

// Jacobi diagonal + SELL-32 copy (once per matrix); shared with the batched solver.
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
  // SELL-32 copy
  A->nslices = (A->rows + kSlice - 1) / kSlice;
  A->sell_ptr.alloc((A->nslices + 1) * sizeof(int64_t), s);
  SellWidthKernel<<<GridFor(ctx, A->nslices, 256), 256, 0, s>>>(A->rows, A->nslices, A->rowptr.as<int64_t>(),
                                                               A->sell_ptr.as<int64_t>());
  LFG_LAUNCHED(ctx);
  A->sell_nnz = ExclusiveScanI64(ctx, A->sell_ptr.as<int64_t>(), A->sell_ptr.as<int64_t>(), A->nslices);
  LFG_CUDA(cudaMemcpyAsync(A->sell_ptr.as<int64_t>() + A->nslices, &A->sell_nnz, sizeof(int64_t),
                           cudaMemcpyHostToDevice, s));
  if (A->sell_nnz >= (int64_t(1) << 31)) Fail(LFG_UNSUPPORTED, "solver needs padded nnz < 2^31");
  A->sell_col.alloc(std::max<int64_t>(A->sell_nnz, 1) * sizeof(int32_t), s);
  A->sell_val.alloc(std::max<int64_t>(A->sell_nnz, 1) * sizeof(double), s);
  SellFillKernel<<<GridFor(ctx, A->rows, 256), 256, 0, s>>>(A->rows, A->rowptr.as<int64_t>(), A->col.as<int32_t>(),
                                                            A->val.as<double>(), A->sell_ptr.as<int64_t>(),
                                                            A->sell_col.as<int32_t>(), A->sell_val.as<double>());
  LFG_LAUNCHED(ctx);
  LFG_CUDA(cudaStreamSynchronize(s));  // the host copy of sell_nnz above is a stack value
}

void EnsureFloatValues(lfg_csr* A) {
  lfg_ctx* ctx = A->ctx;
  if (!A->rowsum32.p) {
    A->rowsum32.alloc(std::max<int64_t>(A->rows, 1) * sizeof(float), ctx->stream);
    RowSumKernel<<<GridFor(ctx, A->rows, 256), 256, 0, ctx->stream>>>(A->rows, A->rowptr.as<int64_t>(),
                                                                      A->val.as<double>(), A->rowsum32.as<float>());
    LFG_LAUNCHED(ctx);
  }
  if (!A->val32.p) {
    A->val32.alloc(std::max<int64_t>(A->nnz, 1) * sizeof(float), ctx->stream);
    ToFloatKernel<<<GridFor(ctx, A->nnz, 256), 256, 0, ctx->stream>>>(A->nnz, A->val.as<double>(),
                                                                       A->val32.as<float>());
    LFG_LAUNCHED(ctx);
  }
  if (!A->sell_val32.p) {
    A->sell_val32.alloc(std::max<int64_t>(A->sell_nnz, 1) * sizeof(float), ctx->stream);
    ToFloatKernel<<<GridFor(ctx, A->sell_nnz, 256), 256, 0, ctx->stream>>>(A->sell_nnz, A->sell_val.as<double>(),
                                                                            A->sell_val32.as<float>());
    LFG_LAUNCHED(ctx);
  }
}

namespace {

// Work vectors of one PCG run in precision T.  r is filled by the caller;
// res holds the block partials of the FP64 residual kernel.
template <class T>
struct PcgState {
  DevBuf r, z, p, q;
  DevBuf part, res, scal;
  int nb = 0;
};

template <class T>
void AllocState(lfg_ctx* ctx, int64_t n, PcgState<T>& S) {
  cudaStream_t s = ctx->stream;
  S.nb = std::max(1, std::min<int>(ctx->num_sms * 8, static_cast<int>((n + kPcgBlock - 1) / kPcgBlock)));
  S.r.alloc(n * sizeof(T), s);
  S.z.alloc(n * sizeof(T), s);
  S.p.alloc(n * sizeof(T), s);
  S.q.alloc(n * sizeof(T), s);
  S.part.alloc(2 * static_cast<size_t>(ctx->num_sms) * 8 * sizeof(double), s);  // >= 2 * any grid used
  S.res.alloc(S.nb * sizeof(double), s);
  S.scal.alloc(sizeof(PcgScalars), s);
  LFG_CUDA(cudaMemsetAsync(S.scal.p, 0, sizeof(PcgScalars), s));
}

double ReadRR(lfg_ctx* ctx, const DevBuf& scal) {
  double rr = 0.0;
  D2HSync(ctx, &rr, reinterpret_cast<const char*>(scal.p) + offsetof(PcgScalars, rr), sizeof(double));
  return rr;
}

// An instantiated CUDA graph of PCG iterations.
struct PcgGraph {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int launches = 0;
  void Release() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    exec = nullptr;
    graph = nullptr;
  }
};

// The captured iteration body: `body` PCG iterations (even: the p buffers
// and rz slots alternate).
template <class T>
PcgGraph CapturePcg(lfg_csr* A, const T* sval, const T* rowsum, const T* dinv, T* x, int64_t n, int body,
                    PcgState<T>& S) {
  lfg_ctx* ctx = A->ctx;
  cudaStream_t s = ctx->stream;
  const int spmv_blocks = static_cast<int>(std::max<int64_t>(
      1, std::min<int64_t>(static_cast<int64_t>(ctx->num_sms) * 8, (A->nslices + 7) / 8)));
  constexpr int U = sizeof(T) == 8 ? 2 : 4;
  const int update_blocks = static_cast<int>(std::max<int64_t>(
      1, std::min<int64_t>(static_cast<int64_t>(ctx->num_sms) * 4, (n + U * kPcgBlock - 1) / (U * kPcgBlock))));
  PcgScalars* sc = S.scal.template as<PcgScalars>();
  double* part = S.part.template as<double>();
  PcgGraph g;
  g.launches = 3 * body;
  cudaGraph_t graph = nullptr;
  LFG_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
  for (int k = 0; k < body; ++k) {
    const int cur = k & 1;
    T* p = S.p.template as<T>();
    PcgDirectionKernel<T><<<GridFor(ctx, n, kPcgBlock), kPcgBlock, 0, s>>>(n, S.z.template as<T>(), p, sc);
    PcgSpmvKernel<T><<<spmv_blocks, kPcgBlock, 0, s>>>(n, A->nslices, A->sell_ptr.as<int64_t>(),
                                                       A->sell_col.as<int32_t>(), sval, rowsum, p, S.q.template as<T>(),
                                                       cur, part, sc);
    PcgUpdateKernel<T><<<update_blocks, kPcgBlock, 0, s>>>(n, dinv, p, S.q.template as<T>(), x, S.r.template as<T>(),
                                                           S.z.template as<T>(), cur, k == body - 1, part, sc);
  }
  cudaError_t ce = cudaStreamEndCapture(s, &graph);
  LFG_CUDA(ce);
  g.graph = graph;
  LFG_CUDA(cudaGraphInstantiate(&g.exec, graph, 0));
  return g;
}

// PCG on A x = b in precision T from the residual already in S.r (x holds
// the matching iterate).  Returns the iterations done; rr_out = <r, r> of the
// recursively updated residual.  With `rhs` (the inner FP32 solves of the
// mixed solver, x = 0 at the start) the true residual rhs - A x is measured
// after every graph replay, and the solve stops as soon as its norm exceeds
// twice the recursive residual's: from there on the FP32 iterates no longer
// improve the solution, and the FP64 refinement takes over.
template <class T>
int RunPcg(lfg_csr* A, const T* sval, const T* rowsum, const T* dinv, T* x, int64_t n, double target_rr,
           int max_it, int check_every, PcgState<T>& S, double& rr_out, const T* rhs = nullptr) {
  lfg_ctx* ctx = A->ctx;
  cudaStream_t s = ctx->stream;
  PcgStartKernel<T><<<S.nb, kPcgBlock, 0, s>>>(n, dinv, S.r.template as<T>(), S.z.template as<T>(),
                                               S.p.template as<T>(), S.part.template as<double>(),
                                               S.scal.template as<PcgScalars>());
  LFG_LAUNCHED(ctx);
  double rr = ReadRR(ctx, S.scal);
  int it = 0;
  if (!(rr > target_rr)) {
    rr_out = rr;
    return 0;
  }
  const int body = std::max(2, check_every + (check_every & 1));
  PcgGraph g = CapturePcg<T>(A, sval, rowsum, dinv, x, n, body, S);
  const int spmv_blocks = static_cast<int>(std::max<int64_t>(
      1, std::min<int64_t>(static_cast<int64_t>(ctx->num_sms) * 8, (A->nslices + 7) / 8)));
  try {
    while (it < max_it) {
      LFG_CUDA(cudaGraphLaunch(g.exec, s));
      CountLaunch(ctx, g.launches);
      it += body;
      if (rhs) {
        PcgTrueResidualKernel<T><<<spmv_blocks, kPcgBlock, 0, s>>>(
            n, A->nslices, A->sell_ptr.as<int64_t>(), A->sell_col.as<int32_t>(), sval, rowsum, x, rhs,
            S.part.template as<double>(), S.scal.template as<PcgScalars>());
        LFG_LAUNCHED(ctx);
        PcgScalars h{};
        D2HSync(ctx, &h, S.scal.p, sizeof(PcgScalars));
        rr = h.rr;
        if (!(rr > target_rr)) break;
        if (!(h.trr <= 4.0 * rr)) break;  // the recursion lost the true residual (or NaN)
        continue;
      }
      rr = ReadRR(ctx, S.scal);
      if (!(rr > target_rr)) break;  // also stops on NaN
    }
  } catch (...) {
    g.Release();
    throw;
  }
  g.Release();
  rr_out = rr;
  return it;
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
                                                 zero.as<double>(), b, S64.r.as<double>(), S64.res.as<double>());
    LFG_LAUNCHED(ctx);
  }
  const double bb = HostSum(ctx, S64.res.as<double>(), nb, tmp);
  const double bnorm = std::sqrt(bb);
  ResidualKernel<<<rblocks, kPcgBlock, 0, s>>>(n, A->rowptr32.as<int32_t>(), A->col.as<int32_t>(), A->val.as<double>(),
                                               x, b, S64.r.as<double>(), S64.res.as<double>());
  LFG_LAUNCHED(ctx);
  double rr = HostSum(ctx, S64.res.as<double>(), nb, tmp);
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
      total += RunPcg<double>(A, A->sell_val.as<double>(), nullptr, A->dinv.as<double>(), x, n, target, max_it - total,
                              check, S64, rr_end);
      ++restarts;
      ResidualKernel<<<rblocks, kPcgBlock, 0, s>>>(n, A->rowptr32.as<int32_t>(), A->col.as<int32_t>(),
                                                   A->val.as<double>(), x, b, S64.r.as<double>(), S64.res.as<double>());
      LFG_LAUNCHED(ctx);
      rr = HostSum(ctx, S64.res.as<double>(), nb, tmp);
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
    DevBuf d32, rhs32, x_old;
    d32.alloc(n * sizeof(float), s);
    rhs32.alloc(n * sizeof(float), s);
    x_old.alloc(n * sizeof(double), s);
    const double inner = opts->inner_rtol > 0 ? opts->inner_rtol : kDefaultInnerRtol;
    int total = 0, outer = 0;
    bool fp32_failed = false;
    while (total < max_it && outer < 200) {
      const double rnorm = std::sqrt(rr);
      if (rr <= target) break;
      // inner FP32 PCG on A d = r / ||r|| (d starts at 0)
      ScaleToFloatKernel<<<GridFor(ctx, n, 256), 256, 0, s>>>(n, S64.r.as<double>(), 1.0 / rnorm, S32.r.as<float>(),
                                                              d32.as<float>());
      LFG_LAUNCHED(ctx);
      LFG_CUDA(cudaMemcpyAsync(rhs32.p, S32.r.p, n * sizeof(float), cudaMemcpyDeviceToDevice, s));
      LFG_CUDA(cudaMemcpyAsync(x_old.p, x, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
      // inner target relative to ||r / ||r|| || = 1, never below what the outer loop needs
      const double need = std::max(inner, 0.5 * std::sqrt(target) / rnorm);
      double rr_in = 0.0;
      const int it = RunPcg<float>(A, A->sell_val32.as<float>(), A->rowsum32.as<float>(), A->dinv32.as<float>(), d32.as<float>(), n,
                                   need * need, max_it - total, check, S32, rr_in, rhs32.as<float>());
      total += std::max(it, 1);
      AddCorrectionKernel<<<GridFor(ctx, n, 256), 256, 0, s>>>(n, d32.as<float>(), rnorm, x);
      LFG_LAUNCHED(ctx);
      ResidualKernel<<<rblocks, kPcgBlock, 0, s>>>(n, A->rowptr32.as<int32_t>(), A->col.as<int32_t>(),
                                                   A->val.as<double>(), x, b, S64.r.as<double>(), S64.res.as<double>());
      LFG_LAUNCHED(ctx);
      const double rr_new = HostSum(ctx, S64.res.as<double>(), nb, tmp);
      ++outer;
      if (!(rr_new < 0.25 * rr)) {
        // the FP32 correction did not halve the FP64 residual: FP32 cannot
        // make progress on this system.  Keep the better iterate and finish
        // in FP64 (same restart rule as the FP64 solver).
        if (!(rr_new < rr)) {
          LFG_CUDA(cudaMemcpyAsync(x, x_old.p, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
          ResidualKernel<<<rblocks, kPcgBlock, 0, s>>>(n, A->rowptr32.as<int32_t>(), A->col.as<int32_t>(),
                                                       A->val.as<double>(), x, b, S64.r.as<double>(),
                                                       S64.res.as<double>());
          LFG_LAUNCHED(ctx);
        } else {
          rr = rr_new;
        }
        fp32_failed = true;
        break;
      }
      rr = rr_new;
    }
    if (fp32_failed) {
      rr = HostSum(ctx, S64.res.as<double>(), nb, tmp);
      double rr_prev = rr;
      int restarts = 0;
      while (rr > target && total < max_it) {
        double rr_end = rr;
        total += RunPcg<double>(A, A->sell_val.as<double>(), nullptr, A->dinv.as<double>(), x, n, target, max_it - total,
                                check, S64, rr_end);
        ++restarts;
        ResidualKernel<<<rblocks, kPcgBlock, 0, s>>>(n, A->rowptr32.as<int32_t>(), A->col.as<int32_t>(),
                                                     A->val.as<double>(), x, b, S64.r.as<double>(),
                                                     S64.res.as<double>());
        LFG_LAUNCHED(ctx);
        rr = HostSum(ctx, S64.res.as<double>(), nb, tmp);
        if (restarts >= 16 || !(rr < 0.25 * rr_prev)) break;
        rr_prev = rr;
      }
      outer += restarts;
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
