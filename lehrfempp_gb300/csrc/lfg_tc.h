// Fifth-generation tensor cores (tcgen05) on sm_103a: inline-PTX wrappers for
// the pieces one CTA-local MMA pipeline needs -- tensor-memory allocation,
// shared-memory matrix descriptors, the instruction descriptor of
// kind::f16 with FP32 accumulation, tcgen05.mma / commit, TMEM loads, and
// mbarrier waits with an iteration limit.
//
// Operand layout used throughout (no swizzle, both operands K-major): a
// matrix of R rows and KP columns (KP a multiple of 16) of 16-bit elements is
// stored as 8x8 "core matrices" of 128 contiguous bytes (8 rows of 16 bytes);
// the core matrix of row group g and column group c sits at
//     g * (KP / 8) * 128 + c * 128
// bytes from the matrix start, i.e. the leading (K) byte offset is 128 and
// the stride (8-row group) byte offset is KP * 16.  One MMA consumes K = 16,
// so the k-th K step starts 256 bytes further.
#pragma once

#include <cstdint>

namespace lfg {
namespace tc {

__device__ __forceinline__ uint32_t SmemAddr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Shared-memory matrix descriptor: start >> 4 in bits 0-13, leading byte
// offset >> 4 in 16-29, stride byte offset >> 4 in 32-45, the fixed 0b001 in
// 46-48, base offset 0, relative leading offsets, no swizzle (bits 61-63 = 0).
__device__ __forceinline__ uint64_t SmemDesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return static_cast<uint64_t>((saddr & 0x3FFFFu) >> 4) | (static_cast<uint64_t>((lbo >> 4) & 0x3FFFu) << 16) |
         (static_cast<uint64_t>((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::f16: D in FP32 (bits 4-5 = 1), A and B
// FP16 (bits 7-9, 10-12 = 0), both K-major (bits 15, 16 = 0), N >> 3 in bits
// 17-22, M >> 4 in bits 24-28.
__host__ __device__ constexpr uint32_t IdescF16(int m, int n) {
  return (1u << 4) | (static_cast<uint32_t>(n >> 3) << 17) | (static_cast<uint32_t>(m >> 4) << 24);
}

// --- tensor memory (one warp allocates and frees)
__device__ __forceinline__ void TmemAlloc(uint32_t* smem_dst, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(SmemAddr(smem_dst)),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void TmemFree(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void FenceBeforeSync() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void FenceAfterSync() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// Generic-proxy shared-memory writes become visible to the tensor cores.
__device__ __forceinline__ void FenceProxyAsync() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// D[tmem] (+)= A[smem] * B[smem]^T, issued by one thread.
__device__ __forceinline__ void MmaF16(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                      bool accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate ? 1u : 0u)
      : "memory");
}

// The mbarrier completes one phase when every MMA issued so far by this
// thread has finished (its shared-memory reads included).
__device__ __forceinline__ void Commit(uint64_t* mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   SmemAddr(mbar))
               : "memory");
}

// 16 consecutive 32-bit columns of this thread's TMEM lane (warp w of the
// CTA reads lanes 32 (w % 4) .. 32 (w % 4) + 31; taddr carries the lane in
// bits 16-31 and the column in bits 0-15).
__device__ __forceinline__ void Ld16(uint32_t taddr, float (&r)[16]) {
  uint32_t u[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(u[0]), "=r"(u[1]), "=r"(u[2]), "=r"(u[3]), "=r"(u[4]), "=r"(u[5]), "=r"(u[6]), "=r"(u[7]),
        "=r"(u[8]), "=r"(u[9]), "=r"(u[10]), "=r"(u[11]), "=r"(u[12]), "=r"(u[13]), "=r"(u[14]), "=r"(u[15])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) r[i] = __uint_as_float(u[i]);
}
__device__ __forceinline__ void Ld8(uint32_t taddr, float (&r)[8]) {
  uint32_t u[8];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=r"(u[0]), "=r"(u[1]), "=r"(u[2]), "=r"(u[3]), "=r"(u[4]), "=r"(u[5]), "=r"(u[6]), "=r"(u[7])
               : "r"(taddr)
               : "memory");
#pragma unroll
  for (int i = 0; i < 8; ++i) r[i] = __uint_as_float(u[i]);
}
__device__ __forceinline__ void WaitLd() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// --- asynchronous global -> shared copies (no registers, no stall at issue)
__device__ __forceinline__ void CpAsync4(void* smem, const void* gmem) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(SmemAddr(smem)), "l"(gmem) : "memory");
}
__device__ __forceinline__ void CpAsync8(void* smem, const void* gmem) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(SmemAddr(smem)), "l"(gmem) : "memory");
}
__device__ __forceinline__ void CpAsyncCommit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void CpAsyncWaitAll() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

// --- named barriers (ids 1..15; count = threads taking part, a multiple of 32)
__device__ __forceinline__ void NamedSync(int id, int count) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(count) : "memory");
}
// bar.sync with an OR over the participants' predicates (the same answer in all of them).
__device__ __forceinline__ bool NamedSyncOr(int id, int count, bool pred) {
  uint32_t out;
  asm volatile(
      "{\n\t.reg .pred pi, po;\n\t"
      "setp.ne.u32 pi, %1, 0;\n\t"
      "bar.red.or.pred po, %2, %3, pi;\n\t"
      "selp.u32 %0, 1, 0, po;\n\t}"
      : "=r"(out)
      : "r"(pred ? 1u : 0u), "r"(id), "r"(count)
      : "memory");
  return out != 0;
}

// --- mbarrier
__device__ __forceinline__ void MbarInit(uint64_t* mbar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(SmemAddr(mbar)), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ bool MbarTryWait(uint64_t* mbar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(SmemAddr(mbar)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ void MbarArrive(uint64_t* mbar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(SmemAddr(mbar)) : "memory");
}
// Waits for the phase with the given parity to complete; gives up after
// max_iter polls (each poll may suspend the thread for a short,
// hardware-chosen time) and returns false.
__device__ __forceinline__ bool MbarWait(uint64_t* mbar, uint32_t parity, uint32_t max_iter) {
  for (uint32_t it = 0; it < max_iter; ++it)
    if (MbarTryWait(mbar, parity)) return true;
  return false;
}

}  // namespace tc
}  // namespace lfg
