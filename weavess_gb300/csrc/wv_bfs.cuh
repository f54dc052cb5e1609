// Frontier kernels of a level-synchronous breadth-first walk over rows
// (ids / deg, width w), shared by the index statistics and the SSG
// connectivity pass.  `bits` marks reached nodes.
#pragma once
#include <cstdint>

#include "wv_common.cuh"

namespace wv {

// expands the frontier one level: every unmarked neighbour is marked and
// appended to `next` (a warp per frontier node)
static __global__ void k_bfs_level(const uint32_t *ids, const uint32_t *deg, uint32_t w, uint32_t n, const uint32_t *front,
                            uint32_t nfront, uint32_t *bits, uint32_t *next, uint32_t *nnext, int *status) {
  const int lane = threadIdx.x & 31;
  const uint32_t wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t f = wid; f < nfront; f += nw) {
    const uint32_t u = front[f];
    uint32_t dg = deg[u];
    if (dg > w) {
      if (lane == 0) set_err(status, DEV_BAD_ID);
      dg = w;
    }
    for (uint32_t j = lane; j < dg; j += 32) {
      const uint32_t v = ids[(size_t)u * w + j];
      if (v >= n) {
        set_err(status, DEV_BAD_ID);
        continue;
      }
      const uint32_t bit = 1u << (v & 31);
      if (!(atomicOr(bits + (v >> 5), bit) & bit)) next[atomicAdd(nnext, 1u)] = v;
    }
  }
}

// first node id whose bit is clear (n if none): one block
static __global__ void k_first_unreached(const uint32_t *bits, uint32_t n, uint32_t *out) {
  __shared__ uint32_t best;
  if (threadIdx.x == 0) best = n;
  __syncthreads();
  const uint32_t words = (n + 31) / 32;
  for (uint32_t i = threadIdx.x; i < words; i += blockDim.x) {
    uint32_t free = ~bits[i];
    if (i == words - 1 && (n & 31)) free &= (1u << (n & 31)) - 1u;
    if (free) atomicMin(&best, i * 32 + (uint32_t)(__ffs(free) - 1));
  }
  __syncthreads();
  if (threadIdx.x == 0) *out = best;
}

}  // namespace wv
