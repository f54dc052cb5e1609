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

__host__ __device__ inline uint32_t pow2_ge(uint32_t x) {
  uint32_t p = 1;
  while (p < x) p <<= 1;
  return p;
}

// The tail of GenRandom (include/weavess/util.h:13-27) for one warp: key[0..L)
// holds the residues rng() % (N - L) in draw order (key has room for
// pow2_ge(L) words); they are sorted ascending, each one that does not exceed
// its predecessor becomes predecessor + 1 -- a_i = max(v_i, a_{i-1} + 1) =
// i + max_{j <= i}(v_j - j), a prefix maximum -- and (a_i + off) % N is
// written to out[i].  Integer keys: any correct sort gives std::sort's order.
__device__ inline void warp_gen_random_tail(uint32_t *key, uint32_t L, uint32_t off, uint32_t N, uint32_t *out,
                                            int lane) {
  const uint32_t P = pow2_ge(L);
  for (uint32_t i = L + lane; i < P; i += 32) key[i] = 0xffffffffu;
  __syncwarp();
  // ascending bitonic sort of key[0..P)
  for (uint32_t k = 2; k <= P; k <<= 1)
    for (uint32_t j = k >> 1; j > 0; j >>= 1) {
      for (uint32_t i = lane; i < P; i += 32) {
        const uint32_t l = i ^ j;
        if (l > i) {
          const uint32_t a = key[i], b = key[l];
          const bool up = (i & k) == 0;
          if ((a > b) == up) {
            key[i] = b;
            key[l] = a;
          }
        }
      }
      __syncwarp();
    }
  long long carry = -(1ll << 40);
  for (uint32_t b = 0; b < L; b += 32) {
    const uint32_t i = b + lane;
    long long m = i < L ? (long long)key[i] - (long long)i : -(1ll << 40);
    for (int o = 1; o < 32; o <<= 1) {
      const long long y = __shfl_up_sync(0xffffffffu, m, o);
      if (lane >= o) m = max(m, y);
    }
    m = max(m, carry);
    carry = __shfl_sync(0xffffffffu, m, 31);
    if (i < L) {
      const unsigned long long a = (unsigned long long)(m + (long long)i);
      out[i] = (uint32_t)((a + off) % N);
    }
  }
  __syncwarp();
}

}  // namespace wv
