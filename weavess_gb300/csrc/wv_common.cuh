// Shared device helpers for the WEAVESS GB300 kernels.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "stl_order.cuh"

namespace wv {

constexpr unsigned FULL = 0xffffffffu;
constexpr uint32_t FLAG = 0x80000000u;    // "not yet expanded" bit packed with an id
constexpr uint32_t ID_MASK = 0x7fffffffu;
constexpr uint32_t INVALID = 0xffffffffu;

// device-side error codes written to a status word (first error wins)
enum DevErr : int {
  DEV_OK = 0,
  DEV_BAD_ID = 1,       // an adjacency id >= n (corrupt graph)
  DEV_OVERFLOW = 2,     // a bounded buffer would have overflowed
  DEV_TIMEOUT = 3,      // a bounded wait gave up
};

__device__ __forceinline__ void set_err(int *status, int code) {
  if (status) atomicCAS(status, 0, code);
}

// (dist, id) ordered by distance only -- the comparison every WEAVESS sort uses
struct DI {
  float d;
  uint32_t i;
};
struct DILess {
  __host__ __device__ bool operator()(const DI &a, const DI &b) const { return a.d < b.d; }
};

// ---- cp.async (LDGSTS) 16-byte global -> shared copies ----
__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
  unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem));
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::); }

// One group of four in WEAVESS's distance order (distance.h:20-25):
// ((d0*d0 + d1*d1) + d2*d2) + d3*d3, every operation rounded separately
// (no FMA), so the FP32 result equals the reference's for any input.
// packed FP32 (two independent round-to-nearest FMAs per instruction):
// acc.{lo,hi} += a.{0,1} * b.{0,1}
__device__ __forceinline__ void fma2(unsigned long long &acc, float a0, float a1, float b0, float b1) {
  asm("{\n .reg .b64 pa, pb;\n mov.b64 pa, {%1, %2};\n mov.b64 pb, {%3, %4};\n fma.rn.f32x2 %0, pa, pb, %0;\n}"
      : "+l"(acc)
      : "f"(a0), "f"(a1), "f"(b0), "f"(b1));
}
__device__ __forceinline__ float sum2(unsigned long long acc) {
  float lo, hi;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(acc));
  return lo + hi;
}

__device__ __forceinline__ float group4(float4 a, float4 b) {
  float d0 = __fsub_rn(a.x, b.x), d1 = __fsub_rn(a.y, b.y), d2 = __fsub_rn(a.z, b.z), d3 = __fsub_rn(a.w, b.w);
  float s = __fadd_rn(__fmul_rn(d0, d0), __fmul_rn(d1, d1));
  s = __fadd_rn(s, __fmul_rn(d2, d2));
  return __fadd_rn(s, __fmul_rn(d3, d3));
}

// Exact-order squared L2 of up to 32 rows against one vector held in shared
// memory, one row per lane.  Rows are staged through shared memory in chunks
// of 128 floats with coalesced 16-byte cp.async copies (one row chunk per warp
// instruction), then each lane folds its row sequentially in the reference's
// order.  `stage` holds 32 * (128 + 4) floats per warp (padding keeps the
// per-lane float4 reads bank-conflict free).  Requires d % 4 == 0.
// Returns the distance for this lane's row (undefined when lane >= cnt).
constexpr int CHUNK = 128;
constexpr int STAGE_STRIDE = CHUNK + 4;
constexpr int STAGE_FLOATS = 32 * STAGE_STRIDE;

__device__ __forceinline__ float warp_l2_rows(const float *__restrict__ base, uint32_t d, uint32_t my_id, int cnt,
                                              const float *qv, float *stage, int lane) {
  float acc = 0.f;
  for (uint32_t c0 = 0; c0 < d; c0 += CHUNK) {
    const uint32_t w = min((uint32_t)CHUNK, d - c0);  // floats in this chunk (multiple of 4)
    const uint32_t nv = w >> 2;                       // float4s per row chunk
    for (int r = 0; r < cnt; r++) {
      uint32_t id = __shfl_sync(FULL, my_id, r);
      if ((uint32_t)lane < nv) cp_async16(stage + r * STAGE_STRIDE + 4 * lane, base + (size_t)id * d + c0 + 4 * lane);
    }
    cp_async_wait_all();
    __syncwarp();
    if (lane < cnt) {
      const float4 *row = reinterpret_cast<const float4 *>(stage + lane * STAGE_STRIDE);
      const float4 *q4 = reinterpret_cast<const float4 *>(qv + c0);
#pragma unroll 8
      for (uint32_t g = 0; g < nv; g++) acc = __fadd_rn(acc, group4(row[g], q4[g]));
    }
    __syncwarp();
  }
  return acc;
}

}  // namespace wv
