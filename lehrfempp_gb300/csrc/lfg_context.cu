// Context, memory helpers, timing and error plumbing of the C-ABI.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <new>

#include "lfg_api.h"
#include "lfg_internal.h"

namespace lfg {

void Fail(lfg_status code, const std::string& msg) { throw Failure{code, msg}; }

void CudaCheck(cudaError_t e, const char* what) {
  if (e != cudaSuccess) {
    cudaGetLastError();  // clear a sticky-free error so the context stays usable
    Fail(e == cudaErrorMemoryAllocation ? LFG_OUT_OF_MEMORY : LFG_CUDA_ERROR,
         std::string(what) + ": " + cudaGetErrorString(e));
  }
}

void DevBuf::alloc(size_t n, cudaStream_t s) {
  reset();
  stream = s;
  if (n == 0) return;
  LFG_CUDA(cudaMallocAsync(&p, n, s));
  bytes = n;
}

void DevBuf::reset() {
  if (p) cudaFreeAsync(p, stream);
  p = nullptr;
  bytes = 0;
}

int GridFor(lfg_ctx* ctx, int64_t n, int block, int per_thread) {
  int64_t need = (n + static_cast<int64_t>(block) * per_thread - 1) / (static_cast<int64_t>(block) * per_thread);
  const int64_t cap = static_cast<int64_t>(ctx->num_sms) * 32;
  if (need > cap) need = cap;
  return need < 1 ? 1 : static_cast<int>(need);
}

void CountLaunch(lfg_ctx* ctx, int n) { ctx->launches += n; }

int32_t* StatusWord(lfg_ctx* ctx) { return ctx->status.as<int32_t>(); }

void D2HSync(lfg_ctx* ctx, void* host, const void* dev, size_t bytes) {
  if (bytes > kPinnedSmallBytes) {  // larger reads go straight to the (pageable) destination
    LFG_CUDA(cudaMemcpyAsync(host, dev, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    LFG_CUDA(cudaStreamSynchronize(ctx->stream));
    return;
  }
  LFG_CUDA(cudaMemcpyAsync(ctx->pinned_small, dev, bytes, cudaMemcpyDeviceToHost, ctx->stream));
  LFG_CUDA(cudaStreamSynchronize(ctx->stream));
  std::memcpy(host, ctx->pinned_small, bytes);
}

void* MappedHost(lfg_ctx* ctx, const void* host, size_t bytes) {
  const uintptr_t h = reinterpret_cast<uintptr_t>(host);
  auto it = ctx->host_allocs.upper_bound(h);
  if (it == ctx->host_allocs.begin()) return nullptr;
  --it;
  const uintptr_t off = h - it->first;
  if (off > it->second || bytes > it->second - off) return nullptr;
  void* base = nullptr;
  LFG_CUDA(cudaHostGetDevicePointer(&base, reinterpret_cast<void*>(it->first), 0));
  return static_cast<char*>(base) + off;
}

__global__ void MappedCopyKernel(const int4* __restrict__ src, int4* __restrict__ dst, size_t n) {
  for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<size_t>(gridDim.x) * blockDim.x)
    dst[i] = src[i];
}

void CopyToHost(lfg_ctx* ctx, void* host, const void* dev, size_t bytes) {
  if (!bytes) return;
  void* mapped = bytes >= kMappedCopyBytes ? MappedHost(ctx, host, bytes) : nullptr;
  if (mapped && ((reinterpret_cast<uintptr_t>(mapped) | reinterpret_cast<uintptr_t>(dev) | bytes) & 15) == 0) {
    const size_t n = bytes / 16;
    const unsigned grid = static_cast<unsigned>(std::min<size_t>((n + 255) / 256, static_cast<size_t>(ctx->num_sms) * 8));
    MappedCopyKernel<<<grid, 256, 0, ctx->stream>>>(static_cast<const int4*>(dev), static_cast<int4*>(mapped), n);
    LFG_LAUNCHED(ctx);
    return;
  }
  LFG_CUDA(cudaMemcpyAsync(host, dev, bytes, cudaMemcpyDeviceToHost, ctx->stream));
}

int32_t ReadAndClearStatus(lfg_ctx* ctx, int32_t* detail) {
  int32_t w[2] = {0, 0};
  D2HSync(ctx, w, ctx->status.p, sizeof(w));
  if (w[0] != 0) LFG_CUDA(cudaMemsetAsync(ctx->status.p, 0, 2 * sizeof(int32_t), ctx->stream));
  if (detail) *detail = w[1];
  return w[0];
}

namespace {
cudaEvent_t TakeEvent(lfg_ctx* ctx) {
  if (!ctx->event_pool.empty()) {
    cudaEvent_t e = ctx->event_pool.back();
    ctx->event_pool.pop_back();
    return e;
  }
  cudaEvent_t e;
  LFG_CUDA(cudaEventCreate(&e));
  return e;
}

void ResolveProfile(lfg_ctx* ctx) {
  if (ctx->prof_pending.empty()) return;
  LFG_CUDA(cudaStreamSynchronize(ctx->stream));
  for (auto& r : ctx->prof_pending) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, r.a, r.b);
    auto& t = ctx->prof_totals[r.family];
    t.first += ms;
    t.second += 1;
    ctx->event_pool.push_back(r.a);
    ctx->event_pool.push_back(r.b);
  }
  ctx->prof_pending.clear();
}

// Independent FMA chains; the result is consumed so the loop is kept.
__global__ void Fp64FmaKernel(double* out, int iters, double a, double b) {
  double x[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) x[k] = threadIdx.x + k;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 8; ++k) x[k] = fma(x[k], a, b);
  }
  double s = 0;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += x[k];
  if (s == 12345.678) out[0] = s;
}
}  // namespace

ProfScope::ProfScope(lfg_ctx* c, const char* family) : ctx(c) {
  if (!ctx->profiling) return;
  lfg_ctx::ProfRec r{family, TakeEvent(ctx), TakeEvent(ctx)};
  LFG_CUDA(cudaEventRecord(r.a, ctx->stream));
  ctx->prof_pending.push_back(r);
  idx = ctx->prof_pending.size() - 1;
}

ProfScope::~ProfScope() {
  if (idx != static_cast<size_t>(-1)) cudaEventRecord(ctx->prof_pending[idx].b, ctx->stream);
}

}  // namespace lfg

using namespace lfg;

extern "C" {

lfg_status lfg_profile_enable(lfg_ctx* ctx, int enable) {
  LFG_API_BEGIN(ctx)
  ctx->profiling = enable != 0;
  LFG_API_END
}

lfg_status lfg_profile_read(lfg_ctx* ctx, const char* family, double* total_ms, int64_t* launches) {
  LFG_API_BEGIN(ctx)
  if (!family) Fail(LFG_INVALID_ARG, "null family");
  if (std::string(family) == "tc_timeouts") {
    int32_t n = 0;
    D2HSync(ctx, &n, StatusWord(ctx) + 14, sizeof(n));
    if (total_ms) *total_ms = static_cast<double>(n);
    if (launches) *launches = n;
    return LFG_OK;
  }
  if (std::string(family) == "fp64_fallback_cells") {  // element-kernel cells computed in FP64
    unsigned long long n = 0;
    D2HSync(ctx, &n, StatusWord(ctx) + 12, sizeof(n));
    if (total_ms) *total_ms = static_cast<double>(n);
    if (launches) *launches = static_cast<int64_t>(n);
    return LFG_OK;
  }
  ResolveProfile(ctx);
  auto it = ctx->prof_totals.find(family);
  if (total_ms) *total_ms = it == ctx->prof_totals.end() ? 0.0 : it->second.first;
  if (launches) *launches = it == ctx->prof_totals.end() ? 0 : it->second.second;
  LFG_API_END
}

lfg_status lfg_profile_reset(lfg_ctx* ctx) {
  LFG_API_BEGIN(ctx)
  ResolveProfile(ctx);
  ctx->prof_totals.clear();
  LFG_API_END
}

lfg_status lfg_measure_fp64_peak(lfg_ctx* ctx, double* tflops) {
  LFG_API_BEGIN(ctx)
  if (!tflops) Fail(LFG_INVALID_ARG, "null output");
  DevBuf out;
  out.alloc(64, ctx->stream);
  const int iters = 4096, threads = 256, blocks = ctx->num_sms * 8;
  Fp64FmaKernel<<<blocks, threads, 0, ctx->stream>>>(out.as<double>(), iters, 0.999999, 1e-7);  // warm-up
  LFG_LAUNCHED(ctx);
  float best = 1e30f;
  for (int rep = 0; rep < 3; ++rep) {
    LFG_CUDA(cudaEventRecord(ctx->t0, ctx->stream));
    Fp64FmaKernel<<<blocks, threads, 0, ctx->stream>>>(out.as<double>(), iters, 0.999999, 1e-7);
    LFG_LAUNCHED(ctx);
    LFG_CUDA(cudaEventRecord(ctx->t1, ctx->stream));
    LFG_CUDA(cudaEventSynchronize(ctx->t1));
    float ms;
    LFG_CUDA(cudaEventElapsedTime(&ms, ctx->t0, ctx->t1));
    best = ms < best ? ms : best;
  }
  *tflops = 2.0 * 8 * iters * static_cast<double>(blocks) * threads / (best * 1e-3) / 1e12;
  LFG_API_END
}

lfg_status lfg_ctx_create(int device, lfg_ctx** out) {
  if (!out) return LFG_INVALID_ARG;
  *out = nullptr;
  lfg_ctx* ctx = nullptr;
  try {
    ctx = new lfg_ctx;
    ctx->device = device;
    LFG_CUDA(cudaSetDevice(device));
    LFG_CUDA(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
    LFG_CUDA(cudaEventCreate(&ctx->t0));
    LFG_CUDA(cudaEventCreate(&ctx->t1));
    LFG_CUDA(cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device));
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
      uint64_t thr = UINT64_MAX;
      cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
    }
    ctx->status.alloc(64, ctx->stream);
    LFG_CUDA(cudaMemsetAsync(ctx->status.p, 0, 64, ctx->stream));
    LFG_CUDA(cudaMallocHost(&ctx->pinned_small, kPinnedSmallBytes));
    LFG_CUDA(cudaStreamSynchronize(ctx->stream));
    *out = ctx;
    return LFG_OK;
  } catch (const Failure& f) {
    std::fprintf(stderr, "lfg_ctx_create: %s\n", f.msg.c_str());
    delete ctx;
    return f.code;
  } catch (const std::bad_alloc&) {
    delete ctx;
    return LFG_OUT_OF_MEMORY;
  }
}

}  // extern "C"

namespace lfg {
namespace {
void FreeCtx(lfg_ctx* ctx) {
  cudaSetDevice(ctx->device);
  ctx->flush.reset();
  ctx->status.reset();
  ctx->tables.clear();
  ctx->dftables.clear();
  ctx->tc_images.clear();
  cudaStreamSynchronize(ctx->stream);
  for (auto& r : ctx->prof_pending) {
    cudaEventDestroy(r.a);
    cudaEventDestroy(r.b);
  }
  for (cudaEvent_t e : ctx->event_pool) cudaEventDestroy(e);
  if (ctx->pinned_small) cudaFreeHost(ctx->pinned_small);
  cudaEventDestroy(ctx->t0);
  cudaEventDestroy(ctx->t1);
  cudaStreamDestroy(ctx->stream);
  delete ctx;
}
}  // namespace

void RetainCtx(lfg_ctx* ctx) { ++ctx->refs; }

void ReleaseCtx(lfg_ctx* ctx) {
  if (--ctx->refs == 0 && ctx->destroyed) FreeCtx(ctx);
}
}  // namespace lfg

extern "C" {

lfg_status lfg_ctx_destroy(lfg_ctx* ctx) {
  if (!ctx || ctx->destroyed) return LFG_INVALID_ARG;
  ctx->destroyed = true;
  if (ctx->refs == 0) lfg::FreeCtx(ctx);
  return LFG_OK;
}

const char* lfg_ctx_last_error(const lfg_ctx* ctx) {
  return ctx ? ctx->last_error.c_str() : "null context";
}

void* lfg_ctx_stream(lfg_ctx* ctx) { return ctx ? static_cast<void*>(ctx->stream) : nullptr; }

lfg_status lfg_ctx_synchronize(lfg_ctx* ctx) {
  LFG_API_BEGIN(ctx)
  LFG_CUDA(cudaStreamSynchronize(ctx->stream));
  int32_t timeouts = 0;
  D2HSync(ctx, &timeouts, StatusWord(ctx) + 14, sizeof(timeouts));
  if (timeouts) {
    LFG_CUDA(cudaMemsetAsync(StatusWord(ctx) + 14, 0, sizeof(int32_t), ctx->stream));
    Fail(LFG_CUDA_ERROR, "tensor-core pipeline wait timed out; element matrices of the affected launch are invalid");
  }
  LFG_API_END
}

lfg_status lfg_ctx_set_tensor_cores(lfg_ctx* ctx, int enable) {
  LFG_API_BEGIN(ctx)
  if (enable < 0 || enable > 3) Fail(LFG_INVALID_ARG, "lfg_ctx_set_tensor_cores: enable must be 0, 1, 2 or 3");
  ctx->tensor_cores = enable;
  LFG_API_END
}

lfg_status lfg_ctx_launch_count(const lfg_ctx* ctx, int64_t* launches) {
  if (!ctx || !launches) return LFG_INVALID_ARG;
  *launches = ctx->launches;
  return LFG_OK;
}

lfg_status lfg_malloc(lfg_ctx* ctx, size_t bytes, void** dev) {
  LFG_API_BEGIN(ctx)
  if (!dev) Fail(LFG_INVALID_ARG, "lfg_malloc: null output");
  *dev = nullptr;
  if (bytes) {
    LFG_CUDA(cudaMallocAsync(dev, bytes, ctx->stream));
  }
  LFG_API_END
}

lfg_status lfg_free(lfg_ctx* ctx, void* dev) {
  LFG_API_BEGIN(ctx)
  if (dev) LFG_CUDA(cudaFreeAsync(dev, ctx->stream));
  LFG_API_END
}

lfg_status lfg_host_alloc(lfg_ctx* ctx, size_t bytes, void** host) {
  LFG_API_BEGIN(ctx)
  if (!host) Fail(LFG_INVALID_ARG, "lfg_host_alloc: null output");
  LFG_CUDA(cudaMallocHost(host, bytes ? bytes : 1));
  ctx->host_allocs[reinterpret_cast<uintptr_t>(*host)] = bytes ? bytes : 1;
  LFG_API_END
}

lfg_status lfg_host_free(lfg_ctx* ctx, void* host) {
  LFG_API_BEGIN(ctx)
  if (host) {
    ctx->host_allocs.erase(reinterpret_cast<uintptr_t>(host));
    LFG_CUDA(cudaFreeHost(host));
  }
  LFG_API_END
}

lfg_status lfg_memcpy_h2d(lfg_ctx* ctx, void* dst, const void* src, size_t bytes) {
  LFG_API_BEGIN(ctx)
  if (bytes) LFG_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, ctx->stream));
  LFG_API_END
}

lfg_status lfg_memcpy_d2h(lfg_ctx* ctx, void* dst, const void* src, size_t bytes) {
  LFG_API_BEGIN(ctx)
  if (bytes) {
    CopyToHost(ctx, dst, src, bytes);
    LFG_CUDA(cudaStreamSynchronize(ctx->stream));
  }
  LFG_API_END
}

lfg_status lfg_memcpy_d2d(lfg_ctx* ctx, void* dst, const void* src, size_t bytes) {
  LFG_API_BEGIN(ctx)
  if (bytes) LFG_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, ctx->stream));
  LFG_API_END
}

lfg_status lfg_memset(lfg_ctx* ctx, void* dev, int value, size_t bytes) {
  LFG_API_BEGIN(ctx)
  if (bytes) LFG_CUDA(cudaMemsetAsync(dev, value, bytes, ctx->stream));
  LFG_API_END
}

lfg_status lfg_timer_begin(lfg_ctx* ctx) {
  LFG_API_BEGIN(ctx)
  LFG_CUDA(cudaEventRecord(ctx->t0, ctx->stream));
  LFG_API_END
}

lfg_status lfg_timer_end(lfg_ctx* ctx, float* ms) {
  LFG_API_BEGIN(ctx)
  LFG_CUDA(cudaEventRecord(ctx->t1, ctx->stream));
  LFG_CUDA(cudaEventSynchronize(ctx->t1));
  LFG_CUDA(cudaEventElapsedTime(ms, ctx->t0, ctx->t1));
  LFG_API_END
}

lfg_status lfg_l2_flush(lfg_ctx* ctx) {
  LFG_API_BEGIN(ctx)
  const size_t bytes = size_t(512) << 20;  // 512 MB > 129 MB L2
  if (ctx->flush.bytes < bytes) ctx->flush.alloc(bytes, ctx->stream);
  LFG_CUDA(cudaMemsetAsync(ctx->flush.p, ctx->launches & 0xff, bytes, ctx->stream));
  LFG_API_END
}

}  // extern "C"
