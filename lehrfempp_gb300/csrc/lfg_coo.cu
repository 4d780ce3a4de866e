// COOMatrix on the device and FixFlaggedSolutionComponents
// (assemble/coomatrix.h:51-225, assemble/fix_dof.h:86-280).
#include <algorithm>

#include "lfg_api.h"
#include "lfg_internal.h"

namespace lfg {
namespace {

// b[row] += value * (-xhat[col]) for triplets in fixed columns (the only ones
// whose contribution is non-zero in A.MatVecMult(-1.0, xhat, b)).
__global__ void FixRhsKernel(int64_t n, const lfg_triplet* __restrict__ t,
                             const uint8_t* __restrict__ flags, const double* __restrict__ vals,
                             double* b) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const lfg_triplet tr = t[i];
    if (flags[tr.col]) atomicAdd(&b[tr.row], tr.value * (-1.0 * vals[tr.col]));
  }
}

__global__ void FixSetRhsKernel(int64_t ndofs, const uint8_t* __restrict__ flags,
                                const double* __restrict__ vals, double* b) {
  for (int64_t k = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; k < ndofs;
       k += static_cast<int64_t>(gridDim.x) * blockDim.x)
    if (flags[k]) b[k] = vals[k];
}

__global__ void KeepFlagsKernel(int64_t n, const lfg_triplet* __restrict__ t,
                                const uint8_t* __restrict__ flags, bool cols_too, int64_t N,
                                int64_t* __restrict__ keep, int32_t* st) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const lfg_triplet tr = t[i];
    if (tr.row < 0 || tr.row >= N || tr.col < 0 || tr.col >= N) {  // checked, never dereferenced
      atomicCAS(st, 0, 1);
      keep[i] = 1;
      continue;
    }
    keep[i] = !(flags[tr.row] || (cols_too && flags[tr.col]));
  }
}

__global__ void FlagCountKernel(int64_t ndofs, const uint8_t* __restrict__ flags, int64_t* f) {
  for (int64_t k = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; k < ndofs;
       k += static_cast<int64_t>(gridDim.x) * blockDim.x)
    f[k] = flags[k] != 0;
}

__global__ void CompactKernel(int64_t n, const lfg_triplet* __restrict__ in,
                              const uint8_t* __restrict__ flags, bool cols_too,
                              const int64_t* __restrict__ pos, lfg_triplet* __restrict__ out) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const lfg_triplet tr = in[i];
    if (!(flags[tr.row] || (cols_too && flags[tr.col]))) out[pos[i]] = tr;
  }
}

__global__ void AppendDiagKernel(int64_t ndofs, const uint8_t* __restrict__ flags,
                                 const int64_t* __restrict__ rank, lfg_triplet* out) {
  for (int64_t k = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; k < ndofs;
       k += static_cast<int64_t>(gridDim.x) * blockDim.x)
    if (flags[k]) {
      lfg_triplet d;
      d.row = static_cast<int32_t>(k);
      d.col = static_cast<int32_t>(k);
      d.value = 1.0;
      out[rank[k]] = d;
    }
}

// FixSolutionComponentsLse's (dof, value) list: keys = dof, payload = list
// position; out-of-range dofs are reported through the status word.
__global__ void LseKeysKernel(int64_t count, const int64_t* __restrict__ dofs, int64_t N,
                              uint64_t* __restrict__ keys, uint32_t* __restrict__ pos, int32_t* st) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < count;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int64_t d = dofs[i];
    if (d < 0 || d >= N) {
      atomicCAS(st, 0, 1);
      keys[i] = 0;
    } else {
      keys[i] = static_cast<uint64_t>(d);
    }
    pos[i] = static_cast<uint32_t>(i);
  }
}

// After a stable sort by dof: the first item of every run writes
// flags[dof] = 1 and fixed[dof] = 0 + v_1 + v_2 + ... in list order (the
// `fixed_vec[idx] += value` loop of fix_dof.h:266-272).
__global__ void LseRunsKernel(int64_t count, const uint64_t* __restrict__ keys, const uint32_t* __restrict__ pos,
                              const double* __restrict__ vals, uint8_t* __restrict__ flags,
                              double* __restrict__ fixed) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < count;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const uint64_t k = keys[i];
    if (i > 0 && keys[i - 1] == k) continue;
    double s = 0.0;
    for (int64_t m = i; m < count && keys[m] == k; ++m) s += vals[pos[m]];
    fixed[k] = s;
    flags[k] = 1;
  }
}

void Fix(lfg_coo* coo, const uint8_t* flags, const double* vals, double* b, bool cols_too) {
  lfg_ctx* ctx = coo->ctx;
  cudaStream_t s = ctx->stream;
  if (coo->rows != coo->cols) Fail(LFG_INVALID_ARG, "Matrix must be square!");
  const int64_t n = coo->size, N = coo->rows;
  DevBuf keep, fl;
  keep.alloc((n + 1) * sizeof(int64_t), s);
  fl.alloc((N + 1) * sizeof(int64_t), s);
  ReadAndClearStatus(ctx);
  KeepFlagsKernel<<<GridFor(ctx, n, 256), 256, 0, s>>>(n, coo->d, flags, cols_too, N, keep.as<int64_t>(),
                                                       StatusWord(ctx));
  LFG_LAUNCHED(ctx);
  if (ReadAndClearStatus(ctx)) Fail(LFG_INVALID_ARG, "triplet index out of range");
  FlagCountKernel<<<GridFor(ctx, N, 256), 256, 0, s>>>(N, flags, fl.as<int64_t>());
  LFG_LAUNCHED(ctx);
  const int64_t kept = n ? ExclusiveScanI64(ctx, keep.as<int64_t>(), keep.as<int64_t>(), n) : 0;
  const int64_t nfix = ExclusiveScanI64(ctx, fl.as<int64_t>(), fl.as<int64_t>(), N);
  if (kept + nfix > coo->capacity)
    Fail(LFG_CAPACITY, "COO capacity too small for the appended diagonal entries");
  // all checks passed: modify b, then the triplets
  if (cols_too && n) {
    FixRhsKernel<<<GridFor(ctx, n, 256), 256, 0, s>>>(n, coo->d, flags, vals, b);
    LFG_LAUNCHED(ctx);
  }
  FixSetRhsKernel<<<GridFor(ctx, N, 256), 256, 0, s>>>(N, flags, vals, b);
  LFG_LAUNCHED(ctx);
  if (n) {
    DevBuf tmp;
    tmp.alloc(std::max<int64_t>(kept, 1) * sizeof(lfg_triplet), s);
    CompactKernel<<<GridFor(ctx, n, 256), 256, 0, s>>>(n, coo->d, flags, cols_too, keep.as<int64_t>(),
                                                       tmp.as<lfg_triplet>());
    LFG_LAUNCHED(ctx);
    if (kept)
      LFG_CUDA(cudaMemcpyAsync(coo->d, tmp.p, kept * sizeof(lfg_triplet), cudaMemcpyDeviceToDevice, s));
  }
  AppendDiagKernel<<<GridFor(ctx, N, 256), 256, 0, s>>>(N, flags, fl.as<int64_t>(), coo->d + kept);
  LFG_LAUNCHED(ctx);
  coo->size = kept + nfix;
}

}  // namespace
}  // namespace lfg

using namespace lfg;

extern "C" {

lfg_status lfg_coo_create(lfg_ctx* ctx, int64_t rows, int64_t cols, int64_t capacity, lfg_coo** out) {
  LFG_API_BEGIN(ctx)
  if (!out || rows < 0 || cols < 0 || capacity < 0) Fail(LFG_INVALID_ARG, "lfg_coo_create: bad argument");
  if (rows >= (int64_t(1) << 31) || cols >= (int64_t(1) << 31))
    Fail(LFG_INVALID_ARG, "COO dimensions exceed the int32 triplet index range");
  auto* c = new lfg_coo;
  c->ref.Set(ctx);
  c->ctx = ctx;
  c->rows = rows;
  c->cols = cols;
  c->capacity = capacity;
  try {
    c->owned.alloc(std::max<int64_t>(capacity, 1) * sizeof(lfg_triplet), ctx->stream);
  } catch (...) {
    delete c;
    throw;
  }
  c->d = c->owned.as<lfg_triplet>();
  *out = c;
  LFG_API_END
}

lfg_status lfg_coo_wrap(lfg_ctx* ctx, int64_t rows, int64_t cols, lfg_triplet* d, int64_t capacity,
                        int64_t size, lfg_coo** out) {
  LFG_API_BEGIN(ctx)
  if (!out || !d || size < 0 || size > capacity) Fail(LFG_INVALID_ARG, "lfg_coo_wrap: bad argument");
  if (reinterpret_cast<uintptr_t>(d) % 16) Fail(LFG_INVALID_ARG, "triplet buffer must be 16-byte aligned");
  auto* c = new lfg_coo;
  c->ref.Set(ctx);
  c->ctx = ctx;
  c->rows = rows;
  c->cols = cols;
  c->capacity = capacity;
  c->size = size;
  c->d = d;
  *out = c;
  LFG_API_END
}

lfg_status lfg_coo_destroy(lfg_coo* coo) {
  if (!coo) return LFG_INVALID_ARG;
  cudaSetDevice(coo->ctx->device);
  delete coo;
  return LFG_OK;
}

lfg_status lfg_coo_size(const lfg_coo* coo, int64_t* size) {
  if (!coo || !size) return LFG_INVALID_ARG;
  *size = coo->size;
  return LFG_OK;
}

lfg_status lfg_coo_triplets(lfg_coo* coo, lfg_triplet** d) {
  if (!coo || !d) return LFG_INVALID_ARG;
  *d = coo->d;
  return LFG_OK;
}

lfg_status lfg_coo_set_zero(lfg_coo* coo) {
  if (!coo) return LFG_INVALID_ARG;
  coo->size = 0;
  return LFG_OK;
}

lfg_status lfg_coo_download(lfg_coo* coo, lfg_triplet* host, int64_t count) {
  if (!coo) return LFG_INVALID_ARG;
  LFG_API_BEGIN(coo->ctx)
  if (!host || count < 0 || count > coo->size) Fail(LFG_INVALID_ARG, "lfg_coo_download: bad count");
  if (count) {
    CopyToHost(coo->ctx, host, coo->d, count * sizeof(lfg_triplet));
    LFG_CUDA(cudaStreamSynchronize(coo->ctx->stream));
  }
  LFG_API_END
}

lfg_status lfg_coo_append_host(lfg_coo* coo, const lfg_triplet* host, int64_t count) {
  if (!coo) return LFG_INVALID_ARG;
  LFG_API_BEGIN(coo->ctx)
  if ((count && !host) || count < 0) Fail(LFG_INVALID_ARG, "lfg_coo_append_host: bad argument");
  if (coo->size + count > coo->capacity) Fail(LFG_CAPACITY, "COO capacity too small");
  for (int64_t k = 0; k < count; ++k)  // AddToEntry's range assertion (coomatrix.h:87-91)
    if (host[k].row < 0 || host[k].row >= coo->rows || host[k].col < 0 || host[k].col >= coo->cols)
      Fail(LFG_INVALID_ARG, "triplet " + std::to_string(k) + " out of range");
  if (count)
    LFG_CUDA(cudaMemcpyAsync(coo->d + coo->size, host, count * sizeof(lfg_triplet), cudaMemcpyHostToDevice,
                             coo->ctx->stream));
  coo->size += count;
  LFG_API_END
}

lfg_status lfg_fix_flagged_solution_components(lfg_coo* coo, const uint8_t* flags, const double* vals,
                                               double* b) {
  if (!coo) return LFG_INVALID_ARG;
  LFG_API_BEGIN(coo->ctx)
  if (!flags || !vals || !b) Fail(LFG_INVALID_ARG, "fix: null argument");
  Fix(coo, flags, vals, b, true);
  LFG_API_END
}

lfg_status lfg_fix_flagged_solution_comp_alt(lfg_coo* coo, const uint8_t* flags, const double* vals,
                                             double* b) {
  if (!coo) return LFG_INVALID_ARG;
  LFG_API_BEGIN(coo->ctx)
  if (!flags || !vals || !b) Fail(LFG_INVALID_ARG, "fix: null argument");
  Fix(coo, flags, vals, b, false);
  LFG_API_END
}

lfg_status lfg_fix_solution_components_lse(lfg_coo* coo, int64_t count, const int64_t* dofs, const double* vals,
                                           double* b) {
  if (!coo) return LFG_INVALID_ARG;
  LFG_API_BEGIN(coo->ctx)
  if (count < 0 || (count > 0 && (!dofs || !vals)) || !b)
    Fail(LFG_INVALID_ARG, "lfg_fix_solution_components_lse: bad argument");
  if (count >= (int64_t(1) << 32)) Fail(LFG_UNSUPPORTED, "more than 2^32 fixed components");
  if (coo->rows != coo->cols) Fail(LFG_INVALID_ARG, "Matrix must be square!");
  lfg_ctx* ctx = coo->ctx;
  cudaStream_t s = ctx->stream;
  const int64_t N = coo->rows;
  DevBuf flags, fixed;
  flags.alloc(std::max<int64_t>(N, 1), s);
  fixed.alloc(std::max<int64_t>(N, 1) * sizeof(double), s);
  LFG_CUDA(cudaMemsetAsync(flags.p, 0, std::max<int64_t>(N, 1), s));
  LFG_CUDA(cudaMemsetAsync(fixed.p, 0, std::max<int64_t>(N, 1) * sizeof(double), s));
  if (count) {
    DevBuf keys, pos;
    keys.alloc(count * sizeof(uint64_t), s);
    pos.alloc(count * sizeof(uint32_t), s);
    ReadAndClearStatus(ctx);
    LseKeysKernel<<<GridFor(ctx, count, 256), 256, 0, s>>>(count, dofs, N, keys.as<uint64_t>(), pos.as<uint32_t>(),
                                                          StatusWord(ctx));
    LFG_LAUNCHED(ctx);
    if (ReadAndClearStatus(ctx)) Fail(LFG_INVALID_ARG, "fixed component index out of range [0, N)");
    int bits = 1;
    while ((int64_t(1) << bits) < N + 1) ++bits;
    RadixSortPairs(ctx, keys.as<uint64_t>(), pos.as<uint32_t>(), count, bits);
    LseRunsKernel<<<GridFor(ctx, count, 256), 256, 0, s>>>(count, keys.as<uint64_t>(), pos.as<uint32_t>(), vals,
                                                          flags.as<uint8_t>(), fixed.as<double>());
    LFG_LAUNCHED(ctx);
  }
  Fix(coo, flags.as<uint8_t>(), fixed.as<double>(), b, false);
  LFG_API_END
}

}  // extern "C"
