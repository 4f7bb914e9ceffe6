// mbarrier helpers shared by the kernels that stage operands with bulk /
// tensor copies.  Every wait is bounded by a wall-clock limit: on expiry the
// caller's error word records a code and the wait reports failure instead of
// spinning forever.
#pragma once
#include <cstdint>

namespace mnpbem {

constexpr unsigned long long MBAR_WAIT_NS = 2000000000ull;  // 2 s per wait

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ unsigned long long gtimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}
// bounded wait with a limit of limit_ns; false (and err |= code) when it expires
__device__ __forceinline__ bool mbar_wait_ns(uint32_t bar, uint32_t parity, int* err, int code,
                                             unsigned long long limit_ns) {
  if (mbar_try_wait(bar, parity)) return true;
  const unsigned long long t0 = gtimer();
  while (true) {
    if (mbar_try_wait(bar, parity)) return true;
    if (gtimer() - t0 > limit_ns) {
      atomicOr(err, code);
      return false;
    }
  }
}
// bounded wait with the library's limit (MBAR_WAIT_NS)
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, int* err, int code) {
  return mbar_wait_ns(bar, parity, err, code, MBAR_WAIT_NS);
}

}  // namespace mnpbem
