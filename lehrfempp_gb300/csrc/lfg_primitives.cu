// Device primitives used by the setup and conversion kernels: an exclusive
// scan and a stable LSD radix sort of (key, value) pairs.  Both are plain
// hand-written CUDA (no CUB/Thrust): the scan is a reduce-then-scan over
// 2048-element tiles, the sort moves 4 key bits per pass and keeps equal keys
// in input order (stability is what makes the edge numbering and the
// COO->CSR duplicate order reproduce the reference).
#include <algorithm>

#include "lfg_api.h"
#include "lfg_internal.h"

namespace lfg {
namespace {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;

template <class T>
__device__ T WarpInclusiveScan(T v) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    T u = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += u;
  }
  return v;
}

// Exclusive block scan of one value per thread; returns the block total.
template <class T>
__device__ T BlockExclusiveScan(T v, T& total) {
  __shared__ T warp_tot[32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nwarps = blockDim.x >> 5;
  T inc = WarpInclusiveScan(v);
  if (lane == 31) warp_tot[warp] = inc;
  __syncthreads();
  if (warp == 0) {
    T w = lane < nwarps ? warp_tot[lane] : T(0);
    T wi = WarpInclusiveScan(w);
    if (lane < nwarps) warp_tot[lane] = wi - w;
    if (lane == nwarps - 1) warp_tot[31] = wi;
  }
  __syncthreads();
  T res = warp_tot[warp] + inc - v;
  total = warp_tot[31];
  __syncthreads();
  return res;
}

__global__ void TileSumKernel(const int64_t* __restrict__ in, int64_t n, int64_t* __restrict__ sums) {
  const int64_t base = static_cast<int64_t>(blockIdx.x) * kScanTile;
  int64_t s = 0;
  for (int k = 0; k < kScanItems; ++k) {
    const int64_t i = base + k * kScanThreads + threadIdx.x;
    if (i < n) s += in[i];
  }
  int64_t tot;
  BlockExclusiveScan(s, tot);
  if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

__global__ void TileScanKernel(const int64_t* in, int64_t n, const int64_t* __restrict__ offsets,
                               int64_t* out) {
  __shared__ int64_t tile[kScanTile];
  const int64_t base = static_cast<int64_t>(blockIdx.x) * kScanTile;
  for (int k = 0; k < kScanItems; ++k) {
    const int idx = k * kScanThreads + threadIdx.x;
    tile[idx] = (base + idx < n) ? in[base + idx] : 0;
  }
  __syncthreads();
  int64_t local[kScanItems];
  int64_t s = 0;
  for (int k = 0; k < kScanItems; ++k) {
    local[k] = s;
    s += tile[threadIdx.x * kScanItems + k];
  }
  int64_t tot;
  const int64_t pre = BlockExclusiveScan(s, tot) + (offsets ? offsets[blockIdx.x] : 0);
  for (int k = 0; k < kScanItems; ++k) tile[threadIdx.x * kScanItems + k] = local[k] + pre;
  __syncthreads();
  for (int k = 0; k < kScanItems; ++k) {
    const int idx = k * kScanThreads + threadIdx.x;
    if (base + idx < n) out[base + idx] = tile[idx];
  }
}

void ScanRec(lfg_ctx* ctx, const int64_t* in, int64_t* out, int64_t n, int64_t* total_dev) {
  const int64_t tiles = (n + kScanTile - 1) / kScanTile;
  DevBuf sums;
  sums.alloc((tiles + 1) * sizeof(int64_t), ctx->stream);
  TileSumKernel<<<static_cast<unsigned>(tiles), kScanThreads, 0, ctx->stream>>>(in, n, sums.as<int64_t>());
  LFG_LAUNCHED(ctx);
  if (tiles == 1) {
    LFG_CUDA(cudaMemcpyAsync(total_dev, sums.p, sizeof(int64_t), cudaMemcpyDeviceToDevice, ctx->stream));
    TileScanKernel<<<1, kScanThreads, 0, ctx->stream>>>(in, n, nullptr, out);
    LFG_LAUNCHED(ctx);
    return;
  }
  DevBuf offs;
  offs.alloc(tiles * sizeof(int64_t), ctx->stream);
  ScanRec(ctx, sums.as<int64_t>(), offs.as<int64_t>(), tiles, total_dev);
  TileScanKernel<<<static_cast<unsigned>(tiles), kScanThreads, 0, ctx->stream>>>(in, n, offs.as<int64_t>(), out);
  LFG_LAUNCHED(ctx);
}

// ------------------------------------------------------------- radix sort
constexpr int kSortThreads = 256;
constexpr int kSortItems = 16;
constexpr int kSortTile = kSortThreads * kSortItems;
constexpr int kDigits = 16;  // 4 bits per pass
constexpr int kSortTilePadded = kSortTile + kSortTile / 16;
__device__ __forceinline__ int Pad(int i) { return i + (i >> 4); }

__global__ void DigitHistKernel(const uint64_t* __restrict__ keys, int64_t n, int shift,
                                int64_t ntiles, int64_t* __restrict__ counts) {
  __shared__ int cnt[kDigits];
  if (threadIdx.x < kDigits) cnt[threadIdx.x] = 0;
  __syncthreads();
  const int64_t base = static_cast<int64_t>(blockIdx.x) * kSortTile;
  for (int k = 0; k < kSortItems; ++k) {
    const int64_t i = base + k * kSortThreads + threadIdx.x;
    if (i < n) atomicAdd(&cnt[(keys[i] >> shift) & (kDigits - 1)], 1);
  }
  __syncthreads();
  if (threadIdx.x < kDigits) counts[threadIdx.x * ntiles + blockIdx.x] = cnt[threadIdx.x];
}

template <class V>
__global__ void __launch_bounds__(kSortThreads)
ScatterKernel(const uint64_t* __restrict__ keys_in, const V* __restrict__ vals_in, int64_t n,
              int shift, int64_t ntiles, const int64_t* __restrict__ offsets,
              uint64_t* __restrict__ keys_out, V* __restrict__ vals_out) {
  extern __shared__ unsigned char smem_raw[];
  // one pad slot per 16 elements keeps the per-thread sequential reads
  // (stride 16) off a single shared-memory bank
  uint64_t* skey = reinterpret_cast<uint64_t*>(smem_raw);
  V* sval = reinterpret_cast<V*>(skey + kSortTilePadded);
  const int64_t base = static_cast<int64_t>(blockIdx.x) * kSortTile;
  const int valid = static_cast<int>(n - base < kSortTile ? n - base : kSortTile);
  for (int k = 0; k < kSortItems; ++k) {
    const int idx = k * kSortThreads + threadIdx.x;
    if (idx < valid) {
      skey[Pad(idx)] = keys_in[base + idx];
      sval[Pad(idx)] = vals_in[base + idx];
    }
  }
  __syncthreads();
  // per-thread digit counts over its contiguous chunk
  int cnt[kDigits];
#pragma unroll
  for (int d = 0; d < kDigits; ++d) cnt[d] = 0;
  const int first = threadIdx.x * kSortItems;
#pragma unroll
  for (int k = 0; k < kSortItems; ++k) {
    const int idx = first + k;
    if (idx < valid) {
      const int d = static_cast<int>((skey[Pad(idx)] >> shift) & (kDigits - 1));
#pragma unroll
      for (int e = 0; e < kDigits; ++e) cnt[e] += (e == d);
    }
  }
  // exclusive prefix over threads, per digit
  int pre[kDigits];
#pragma unroll
  for (int d = 0; d < kDigits; ++d) {
    int tot;
    pre[d] = BlockExclusiveScan(cnt[d], tot);
  }
  int64_t gbase[kDigits];
#pragma unroll
  for (int d = 0; d < kDigits; ++d) gbase[d] = offsets[d * ntiles + blockIdx.x] + pre[d];
#pragma unroll
  for (int k = 0; k < kSortItems; ++k) {
    const int idx = first + k;
    if (idx < valid) {
      const uint64_t key = skey[Pad(idx)];
      const int d = static_cast<int>((key >> shift) & (kDigits - 1));
      int64_t pos = 0;
#pragma unroll
      for (int e = 0; e < kDigits; ++e)
        if (e == d) pos = gbase[e]++;
      keys_out[pos] = key;
      vals_out[pos] = sval[Pad(idx)];
    }
  }
}

template <class V>
void RadixSortImpl(lfg_ctx* ctx, uint64_t* keys, V* vals, int64_t n, int bits) {
  if (n <= 1 || bits <= 0) return;
  const int64_t ntiles = (n + kSortTile - 1) / kSortTile;
  DevBuf k2, v2, counts, offsets;
  k2.alloc(n * sizeof(uint64_t), ctx->stream);
  v2.alloc(n * sizeof(V), ctx->stream);
  counts.alloc(kDigits * ntiles * sizeof(int64_t), ctx->stream);
  offsets.alloc(kDigits * ntiles * sizeof(int64_t), ctx->stream);
  const size_t smem = kSortTilePadded * (sizeof(uint64_t) + sizeof(V));
  LFG_CUDA(cudaFuncSetAttribute(ScatterKernel<V>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                static_cast<int>(smem)));
  uint64_t* kin = keys;
  V* vin = vals;
  uint64_t* kout = k2.as<uint64_t>();
  V* vout = v2.as<V>();
  const int passes = (bits + 3) / 4;
  for (int p = 0; p < passes; ++p) {
    const int shift = 4 * p;
    DigitHistKernel<<<static_cast<unsigned>(ntiles), kSortThreads, 0, ctx->stream>>>(
        kin, n, shift, ntiles, counts.as<int64_t>());
    LFG_LAUNCHED(ctx);
    ScanRec(ctx, counts.as<int64_t>(), offsets.as<int64_t>(), kDigits * ntiles,
            reinterpret_cast<int64_t*>(StatusWord(ctx) + 8));  // total unused; parked in the status block
    ScatterKernel<V><<<static_cast<unsigned>(ntiles), kSortThreads, smem, ctx->stream>>>(
        kin, vin, n, shift, ntiles, offsets.as<int64_t>(), kout, vout);
    LFG_LAUNCHED(ctx);
    std::swap(kin, kout);
    std::swap(vin, vout);
  }
  if (kin != keys) {
    LFG_CUDA(cudaMemcpyAsync(keys, kin, n * sizeof(uint64_t), cudaMemcpyDeviceToDevice, ctx->stream));
    LFG_CUDA(cudaMemcpyAsync(vals, vin, n * sizeof(V), cudaMemcpyDeviceToDevice, ctx->stream));
  }
}

}  // namespace

int64_t ExclusiveScanI64(lfg_ctx* ctx, const int64_t* in, int64_t* out, int64_t n) {
  if (n <= 0) return 0;
  int64_t* total_dev = reinterpret_cast<int64_t*>(StatusWord(ctx) + 4);
  ScanRec(ctx, in, out, n, total_dev);
  int64_t total = 0;
  D2HSync(ctx, &total, total_dev, sizeof(total));
  return total;
}

void RadixSortPairs(lfg_ctx* ctx, uint64_t* keys, uint32_t* vals, int64_t n, int bits) {
  RadixSortImpl<uint32_t>(ctx, keys, vals, n, bits);
}

void RadixSortPairs64(lfg_ctx* ctx, uint64_t* keys, uint64_t* vals, int64_t n, int bits) {
  RadixSortImpl<uint64_t>(ctx, keys, vals, n, bits);
}

}  // namespace lfg
