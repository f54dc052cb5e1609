// Segmented ascending sort of u64 keys: segment i is keys[off[i], off[i] +
// cnt[i]).  Segments up to SEG_WARP_CAP keys are sorted by one warp in shared
// memory (bitonic); longer ones by one block in a global scratch region.
#include "wv_common.cuh"
#include "wv_ctx.h"
#include "wv_segsort.h"

namespace wv {
namespace {

constexpr int SEG_WARPS = 4;
constexpr uint32_t SEG_WARP_CAP = 1024;

__global__ void __launch_bounds__(SEG_WARPS * 32)
    k_seg_small(unsigned long long *keys, const uint32_t *off, const uint32_t *cnt, uint32_t nseg, uint32_t *big,
                uint32_t *nbig, uint32_t *maxbig) {
  __shared__ unsigned long long sk[SEG_WARPS][SEG_WARP_CAP];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t sg = blockIdx.x * SEG_WARPS + warp;
  if (sg >= nseg) return;
  const uint32_t c = cnt[sg], o = off[sg];
  if (c <= 1) return;
  if (c > SEG_WARP_CAP) {
    if (lane == 0) {
      big[atomicAdd(nbig, 1u)] = sg;
      atomicMax(maxbig, c);
    }
    return;
  }
  uint32_t P = 1;
  while (P < c) P <<= 1;
  unsigned long long *k = sk[warp];
  for (uint32_t i = lane; i < P; i += 32) k[i] = i < c ? keys[o + i] : ~0ull;
  __syncwarp();
  for (uint32_t sz = 2; sz <= P; sz <<= 1)
    for (uint32_t j = sz >> 1; j > 0; j >>= 1) {
      for (uint32_t i = lane; i < P; i += 32) {
        uint32_t l = i ^ j;
        if (l > i) {
          bool up = (i & sz) == 0;
          unsigned long long a = k[i], b = k[l];
          if ((a > b) == up) {
            k[i] = b;
            k[l] = a;
          }
        }
      }
      __syncwarp();
    }
  for (uint32_t i = lane; i < c; i += 32) keys[o + i] = k[i];
}

__global__ void __launch_bounds__(1024)
    k_seg_big(unsigned long long *keys, const uint32_t *off, const uint32_t *cnt, const uint32_t *big,
              unsigned long long *scratch, uint32_t P) {
  const uint32_t sg = big[blockIdx.x], c = cnt[sg], o = off[sg];
  unsigned long long *k = scratch + (size_t)blockIdx.x * P;
  for (uint32_t i = threadIdx.x; i < P; i += blockDim.x) k[i] = i < c ? keys[o + i] : ~0ull;
  __syncthreads();
  for (uint32_t sz = 2; sz <= P; sz <<= 1)
    for (uint32_t j = sz >> 1; j > 0; j >>= 1) {
      for (uint32_t i = threadIdx.x; i < P; i += blockDim.x) {
        uint32_t l = i ^ j;
        if (l > i) {
          bool up = (i & sz) == 0;
          unsigned long long a = k[i], b = k[l];
          if ((a > b) == up) {
            k[i] = b;
            k[l] = a;
          }
        }
      }
      __syncthreads();
    }
  for (uint32_t i = threadIdx.x; i < c; i += blockDim.x) keys[o + i] = k[i];
}

}  // namespace

int segsort_u64(wv_ctx *c, unsigned long long *keys, const uint32_t *off, const uint32_t *cnt, uint32_t nseg) {
  if (nseg == 0) return WV_OK;
  cudaError_t e = cudaSuccess;
  uint32_t *big = c->buf<uint32_t>("seg_big", nseg, &e);
  uint32_t *small = c->buf<uint32_t>("seg_small", 4, &e);
  WV_CUDA(c, e);
  WV_CUDA(c, cudaMemsetAsync(small, 0, 16, c->stream));
  k_seg_small<<<(nseg + SEG_WARPS - 1) / SEG_WARPS, SEG_WARPS * 32, 0, c->stream>>>(keys, off, cnt, nseg, big, small,
                                                                                  small + 1);
  WV_CUDA(c, cudaGetLastError());
  uint32_t h[2];
  WV_CUDA(c, cudaMemcpyAsync(h, small, 8, cudaMemcpyDeviceToHost, c->stream));
  WV_CUDA(c, cudaStreamSynchronize(c->stream));
  if (h[0]) {
    uint32_t P = 1;
    while (P < h[1]) P <<= 1;
    unsigned long long *scr = c->buf<unsigned long long>("seg_scr", (size_t)h[0] * P, &e);
    WV_CUDA(c, e);
    k_seg_big<<<h[0], 1024, 0, c->stream>>>(keys, off, cnt, big, scr, P);
    WV_CUDA(c, cudaGetLastError());
  }
  return WV_OK;
}

}  // namespace wv
