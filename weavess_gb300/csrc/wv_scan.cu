// Exclusive prefix sums over u32 arrays (three-phase: block scan, scan of the
// block totals (recursively), add-back).  Used to lay out per-node event and
// per-target offer segments.
#include "wv_common.cuh"
#include "wv_scan.h"

namespace wv {
namespace {

constexpr int SCAN_T = 512;   // threads per block
constexpr int SCAN_I = 4;     // items per thread
constexpr int SCAN_B = SCAN_T * SCAN_I;

__device__ inline uint32_t block_exclusive(uint32_t v, uint32_t *warp_tot, uint32_t &total) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  uint32_t x = v;
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(FULL, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_tot[w] = x;
  __syncthreads();
  if (w == 0) {
    uint32_t t = lane < SCAN_T / 32 ? warp_tot[lane] : 0;
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t y = __shfl_up_sync(FULL, t, o);
      if (lane >= o) t += y;
    }
    if (lane < SCAN_T / 32) warp_tot[lane] = t;
  }
  __syncthreads();
  uint32_t before = w > 0 ? warp_tot[w - 1] : 0;
  total = warp_tot[SCAN_T / 32 - 1];
  return before + x - v;
}

__global__ void k_scan_blocks(const uint32_t *in, uint32_t *out, size_t n, uint32_t *sums) {
  __shared__ uint32_t wt[SCAN_T / 32];
  size_t base = (size_t)blockIdx.x * SCAN_B + threadIdx.x * SCAN_I;
  uint32_t v[SCAN_I], s = 0;
#pragma unroll
  for (int i = 0; i < SCAN_I; i++) {
    v[i] = base + i < n ? in[base + i] : 0u;
    s += v[i];
  }
  uint32_t tot;
  uint32_t ex = block_exclusive(s, wt, tot);
#pragma unroll
  for (int i = 0; i < SCAN_I; i++) {
    if (base + i < n) out[base + i] = ex;
    ex += v[i];
  }
  if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

__global__ void k_scan_add(uint32_t *out, size_t n, const uint32_t *offs) {
  size_t base = (size_t)blockIdx.x * SCAN_B + threadIdx.x * SCAN_I;
  uint32_t o = offs[blockIdx.x];
#pragma unroll
  for (int i = 0; i < SCAN_I; i++)
    if (base + i < n) out[base + i] += o;
}

}  // namespace

size_t scan_scratch_words(size_t n) {
  size_t w = 0;
  while (n > 1) {
    size_t b = (n + SCAN_B - 1) / SCAN_B;
    w += 2 * b + 2;
    n = b;
  }
  return w + 4;
}

cudaError_t exclusive_scan_u32(const uint32_t *in, uint32_t *out, size_t n, uint32_t *scratch, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  size_t blocks = (n + SCAN_B - 1) / SCAN_B;
  uint32_t *sums = scratch, *sums_ex = scratch + blocks + 1;
  k_scan_blocks<<<(unsigned)blocks, SCAN_T, 0, s>>>(in, out, n, sums);
  if (blocks > 1) {
    cudaError_t e = exclusive_scan_u32(sums, sums_ex, blocks, scratch + 2 * blocks + 2, s);
    if (e != cudaSuccess) return e;
    k_scan_add<<<(unsigned)blocks, SCAN_T, 0, s>>>(out, n, sums_ex);
  }
  return cudaGetLastError();
}

}  // namespace wv
