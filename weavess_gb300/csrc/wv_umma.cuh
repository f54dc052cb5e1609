// Helpers for kernels that drive Blackwell's 5th-generation tensor cores
// (tcgen05) directly: shared-memory matrix and instruction descriptors for
// BF16 operands in the canonical no-swizzle K-major layout, and bounded
// mbarrier waits.  Used by the MLP GEMM (wv_umma.cu) and the local join's
// Gram tiles (wv_nnd.cu).
#pragma once
#include <cstdint>

namespace wv {
namespace umma {

constexpr long long WAIT_LIMIT = 1ll << 26;  // polls before a wait gives up

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// shared-memory matrix descriptor (no swizzle): start address, leading byte
// offset (between core matrices adjacent in K) and stride byte offset
// (between 8-row groups), in 16-byte units; bit 46 is the descriptor version
__device__ __forceinline__ uint64_t desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFF);
  d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// instruction descriptor, kind::f16: D FP32, A and B BF16, both K-major,
// N >> 3 and M >> 4
__host__ __device__ constexpr uint32_t idesc(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred P;\n mbarrier.try_wait.parity.shared::cta.b64 P, [%1], %2;\n selp.u32 %0, 1, 0, P;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// bounded wait: false on time-out
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) {
  for (long long i = 0; i < WAIT_LIMIT; i++)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

}  // namespace umma
}  // namespace wv
