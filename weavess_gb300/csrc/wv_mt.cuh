// std::mt19937 (Matsumoto & Nishimura) pieces shared by the kernels that must
// reproduce the reference's mt19937 draws: the seeding recurrence, the twist
// of one word and the tempering.
#pragma once
#include <cstdint>

namespace wv {

__device__ __forceinline__ uint32_t mt_temper(uint32_t y) {
  y ^= y >> 11;
  y ^= (y << 7) & 0x9d2c5680u;
  y ^= (y << 15) & 0xefc60000u;
  y ^= y >> 18;
  return y;
}
// the new value of word i from words i, i + 1 and i + 397 (mod 624)
__device__ __forceinline__ uint32_t mt_mix(uint32_t cur, uint32_t next, uint32_t far) {
  uint32_t y = (cur & 0x80000000u) | (next & 0x7fffffffu);
  return far ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
}
// state word i from word i - 1 (seeding)
__device__ __forceinline__ uint32_t mt_seed_next(uint32_t prev, uint32_t i) {
  return 1812433253u * (prev ^ (prev >> 30)) + i;
}

// one in-place twist of the 624-word state by a warp, in the four
// dependency-ordered phases of the sequential loop: words [0, 227) read only
// old words, [227, 454) read the new words i - 227, [454, 623) the new words
// i - 227, and word 623 wraps to the new word 0
__device__ __forceinline__ void mt_twist_warp(uint32_t *mt, int lane) {
  uint32_t v[8];
#pragma unroll
  for (int r = 0; r < 8; r++) {
    const int t = lane + 32 * r;
    if (t < 227) v[r] = mt_mix(mt[t], mt[t + 1], mt[t + 397]);
  }
  __syncwarp();
#pragma unroll
  for (int r = 0; r < 8; r++) {
    const int t = lane + 32 * r;
    if (t < 227) mt[t] = v[r];
  }
  __syncwarp();
#pragma unroll
  for (int r = 0; r < 8; r++) {
    const int t = lane + 32 * r;
    if (t < 227) v[r] = mt_mix(mt[t + 227], mt[t + 228], mt[t]);
  }
  __syncwarp();
#pragma unroll
  for (int r = 0; r < 8; r++) {
    const int t = lane + 32 * r;
    if (t < 227) mt[t + 227] = v[r];
  }
  __syncwarp();
#pragma unroll
  for (int r = 0; r < 6; r++) {
    const int t = lane + 32 * r;
    if (t < 169) v[r] = mt_mix(mt[t + 454], mt[t + 455], mt[t + 227]);
  }
  __syncwarp();
#pragma unroll
  for (int r = 0; r < 6; r++) {
    const int t = lane + 32 * r;
    if (t < 169) mt[t + 454] = v[r];
  }
  __syncwarp();
  if (lane == 0) mt[623] = mt_mix(mt[623], mt[0], mt[396]);
  __syncwarp();
}

}  // namespace wv
