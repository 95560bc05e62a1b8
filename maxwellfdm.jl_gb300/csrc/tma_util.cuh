// Inline-PTX helpers of the TMA operator kernels (stencil.cu, stencil2.cu):
// shared-memory addresses, mbarrier set-up and bounded waits, and the tiled
// bulk tensor copies (cp.async.bulk.tensor) that complete on an mbarrier.
#pragma once

#include <cuda.h>
#include <stdint.h>

namespace fdfd {

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
// Transaction bytes expected in the current phase, without an arrival (the
// arrival comes later, so the phase cannot complete before it).
__device__ __forceinline__ void mbar_expect_only(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.expect_tx.relaxed.cta.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
// Plain arrival (count 1) on the current phase.
__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void tma_copy3d(uint32_t dst, const CUtensorMap *map, int c0, int c1, int c2,
                                           uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
      "[%5];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(bar)
      : "memory");
}
__device__ __forceinline__ void tma_copy4d(uint32_t dst, const CUtensorMap *map, int c0, int c1, int c2, int c3,
                                           uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
      "[%6];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(bar)
      : "memory");
}
// Bounded wait on an mbarrier phase: gives up after `limit` SM clocks
// (WAIT_LIMIT ≈ 2^31, about one second) and reports false instead of
// spinning forever.  limit = 0 tests the phase once without waiting.
constexpr long long WAIT_LIMIT = 1ll << 31;
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, long long limit = WAIT_LIMIT) {
  if (limit <= 0) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    return done != 0;
  }
  const long long t0 = clock64();
  while (true) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
    if (clock64() - t0 > limit) return false;
  }
}

// The same wait for threads that have nothing else to do meanwhile: each
// try_wait may suspend the thread for up to `hint_ns` until the phase
// completes, so a late copy costs a few polls rather than a spinning loop.
__device__ __forceinline__ bool mbar_wait_sleep(uint32_t bar, uint32_t parity, long long limit, uint32_t hint_ns) {
  if (limit <= 0) return mbar_wait(bar, parity, 0);
  const long long t0 = clock64();
  while (true) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(bar), "r"(parity), "r"(hint_ns)
        : "memory");
    if (done) return true;
    if (clock64() - t0 > limit) return false;
  }
}

}  // namespace fdfd
