// Pieces shared by the beam-search kernels (wv_search.cu: the exact
// traversal; wv_beam.cu: the throughput form): the per-warp shared-memory
// sizes, pool scans, the visited set and the FP32 row distances.
#pragma once
#include <cstdint>

#include "wv_common.cuh"

namespace wv {
namespace {

constexpr int WARPS = 4;  // warps per block of the default shape
constexpr uint32_t EMPTY = 0xffffffffu;
// a visited-hash entry of an unexpanded seed: route mode does not mark seeds
// visited, so the first time a seed comes back as a neighbour it is still
// counted (and rejected as already pooled); ids are below 2^31
constexpr uint32_t SEEDBIT = 0x80000000u;

__host__ __device__ inline size_t align16(size_t x) { return (x + 15) & ~size_t(15); }
__host__ __device__ inline uint32_t pow2_at_least(uint32_t x) {
  uint32_t p = 1;
  while (p < x) p <<= 1;
  return p;
}
// pool: L entries, merged in place
__host__ __device__ inline uint32_t pool_cap(uint32_t Lmax) { return (Lmax + 3) & ~3u; }
// hash area (32-bit words, a power of two), also the scratch of the seed
// sort and the rerank.  Default: >= 2048 and room for the bitonic keys
// (2 * pow2(L) <= pow2(2L + 256)), the introsort's 2L + 256 words and the
// rerank's 2L words.  The least area a launch may ask for holds the bitonic
// keys and the rerank (2 * pow2(L)); the introsort then works in the warp's
// global scratch (the host allows that area only when the scratch is big
// enough).
__host__ __device__ inline uint32_t hash_cap(uint32_t Lmax) { return pow2_at_least(max(2048u, 2 * Lmax + 256)); }
__host__ __device__ inline uint32_t hash_min(uint32_t Lmax) { return max(512u, 2 * pow2_at_least(Lmax)); }
// the area a launch uses: the default, or the power of two asked for (not
// below the least)
__host__ __device__ inline uint32_t hash_slots(uint32_t Lmax, uint32_t want) {
  if (want == 0) return hash_cap(Lmax);
  return max(pow2_at_least(want), hash_min(Lmax));
}

// first index >= from with the FLAG bit set, or L
__device__ inline int first_flag(const uint32_t *pi, int from, int L, int lane) {
  for (int b = from; b < L; b += 32) {
    int i = b + lane;
    unsigned m = __ballot_sync(FULL, i < L && (pi[i] & FLAG));
    if (m) return b + __ffs(m) - 1;
  }
  return L;
}

// number of entries of the sorted array a[0..n) with a[i] < x (lower bound)
template <class T>
__device__ inline int lower_bound_of(const T *a, int n, T x) {
  int lo = 0, hi = n;
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (a[mid] < x) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// number of entries of the sorted array a[0..n) with a[i] <= x (upper bound)
template <class T>
__device__ inline int upper_bound_of(const T *a, int n, T x) {
  int lo = 0, hi = n;
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (a[mid] <= x) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

__device__ __forceinline__ uint32_t hslot(uint32_t id, uint32_t mask) { return (id * 2654435761u) & mask; }

// Visited set: an open-addressing hash in shared memory while it is at most
// half full, then the warp's own n-bit bitset in global memory for ids the
// hash does not hold.  Exact either way.
//
// Narrow form (whenever n is small enough): 16-bit entries, twice the slots
// of the wide form in the same bytes.  An id is mapped by a bijection y of
// its B-bit value (B = bits of n - 1, at least log2(slots) + 1); the low
// log2(slots) bits of y are its home slot and the rest its quotient q.  An
// entry stores q and the probe distance t of its slot from home (linear
// probing, no deletions), so (slot - t, q) gives y back: an entry matches an
// id exactly.  A probe longer than the distance field holds sends that id
// to the bitset (and the hash to its spill mode).  Bit 15 marks a seed.
// Wide form: the ids themselves (32-bit), bit 31 marking a seed.
struct Visited {
  uint32_t *hash, mask, inserted, limit;
  bool spill;      // the hash is full (or an id overflowed): new ids go to the bitset
  bool seed_over;  // a seed did not fit (narrow form): candidates are checked against the pool
  bool narrow;
  uint32_t nbits, shift, cbits, qbits, dmax;  // narrow form: B, B - log2(slots), log2(slots), quotient bits, longest probe
  uint32_t *bits, *touched, ntouch;

  // slots: a power of two (the number of 32-bit words of the area)
  __device__ void init(uint32_t *area, uint32_t words, uint32_t n, bool force_wide) {
    hash = area;
    uint32_t lg = 0;
    while ((2u << lg) <= words) lg++;  // words = 2^lg
    uint32_t B = 1;
    while (B < 32 && (n - 1) >> B) B++;
    const uint32_t c = lg + 1;  // narrow slots = 2 * words
    if (B < c + 1) B = c + 1;
    const uint32_t qb = B - c;
    narrow = !force_wide && qb + 1 + 4 <= 16;  // room for a probe distance of at least 4 bits
    if (narrow) {
      mask = 2 * words - 1;
      nbits = B;
      cbits = c;
      shift = B - c;
      qbits = qb;
      dmax = (1u << (15 - qb)) - 2;  // the all-ones entry stays EMPTY
    } else {
      mask = words - 1;
    }
    limit = (mask + 1) / 2;
    inserted = 0;
    spill = seed_over = false;
    ntouch = 0;
  }
  __device__ void clear(int lane) {
    const uint32_t words = narrow ? (mask + 1) / 2 : mask + 1;
    for (uint32_t i = lane; i < words; i += 32) hash[i] = EMPTY;
    __syncwarp();
    for (uint32_t i = lane; i < ntouch; i += 32) bits[touched[i]] = 0u;
    __syncwarp();
    inserted = 0;
    spill = seed_over = false;
    ntouch = 0;
  }
  __device__ __forceinline__ uint32_t mixed(uint32_t id) const {
    const uint32_t m = nbits >= 32 ? 0xffffffffu : ((1u << nbits) - 1u);
    uint32_t y = (id * 0x9E3779B1u) & m;
    return y ^ (y >> shift);
  }
  __device__ __forceinline__ uint16_t *h16() const { return reinterpret_cast<uint16_t *>(hash); }

  // insert `id` (seed: marked); returns 1 inserted, 0 present, -1 no room
  // within the probe limit (narrow form)
  __device__ int insert(uint32_t id, bool seed, bool &was_seed) {
    was_seed = false;
    if (narrow) {
      const uint32_t y = mixed(id), home = y & mask, q = y >> cbits;
      for (uint32_t t = 0; t <= dmax; t++) {
        const uint32_t h = (home + t) & mask;
        const uint16_t e = (uint16_t)(q | (t << qbits));
        const uint16_t old = atomicCAS(h16() + h, (uint16_t)0xffff, (uint16_t)(seed ? (e | 0x8000) : e));
        if (old == 0xffff) return 1;
        if (old == e) return 0;
        if (old == (e | 0x8000)) {
          if (!seed) {
            h16()[h] = e;
            was_seed = true;
            return 1;  // fresh: the first time a seed is met as a neighbour
          }
          return 0;
        }
      }
      return -1;
    }
    uint32_t h = hslot(id, mask);
    while (true) {
      const uint32_t old = atomicCAS(&hash[h], EMPTY, seed ? (id | SEEDBIT) : id);
      if (old == EMPTY) return 1;
      if (old == id) return 0;
      if (old == (id | SEEDBIT)) {
        if (!seed) {
          hash[h] = id;
          was_seed = true;
          return 1;
        }
        return 0;
      }
      h = (h + 1) & mask;
    }
  }
  // spill mode: 1 found (was_seed: a seed, now converted), 0 absent
  __device__ int find(uint32_t id, bool &was_seed) {
    was_seed = false;
    if (narrow) {
      const uint32_t y = mixed(id), home = y & mask, q = y >> cbits;
      for (uint32_t t = 0; t <= dmax; t++) {
        const uint32_t h = (home + t) & mask;
        const uint16_t e = (uint16_t)(q | (t << qbits));
        const uint16_t v = h16()[h];
        if (v == 0xffff) return 0;
        if (v == e) return 1;
        if (v == (e | 0x8000)) {
          h16()[h] = e;
          was_seed = true;
          return 1;
        }
      }
      return 0;
    }
    uint32_t h = hslot(id, mask);
    while (true) {
      const uint32_t v = hash[h];
      if (v == id) return 1;
      if (v == (id | SEEDBIT)) {
        hash[h] = id;
        was_seed = true;
        return 1;
      }
      if (v == EMPTY) return 0;
      h = (h + 1) & mask;
    }
  }

  // route mode: records the seeds (not visited) so that a seed met again is
  // known; warp-uniform call, ids distinct among the `want` lanes; the hash
  // has room for every seed (limit >= SEARCH_MAX_L + 128)
  __device__ void add_seed(bool want, uint32_t id) {
    int r = 0;
    if (want) {
      bool ws;
      r = insert(id, true, ws);
    }
    inserted += __popc(__ballot_sync(FULL, r == 1));
    if (__any_sync(FULL, r < 0)) seed_over = true;
  }
  // warp-uniform call; `want` lanes test `id` (ids distinct among lanes);
  // returns true for lanes whose id was not visited before; `seed` is set
  // for a fresh id that is a recorded seed (still unvisited until now)
  __device__ bool test_and_set(bool want, uint32_t id, int lane, bool &seed) {
    const unsigned wm = __ballot_sync(FULL, want);
    if (!spill && inserted + __popc(wm) > limit) spill = true;
    bool fresh = false, newword = false, added = false, to_bits = false;
    seed = false;
    if (want) {
      if (!spill) {
        const int r = insert(id, false, seed);
        fresh = r == 1;
        added = r == 1 && !seed;
        to_bits = r < 0;
      } else {
        to_bits = find(id, seed) == 0;
        fresh = seed;
      }
      if (to_bits) {
        const uint32_t bit = 1u << (id & 31);
        const uint32_t old = atomicOr(bits + (id >> 5), bit);
        fresh = (old & bit) == 0;
        newword = old == 0;
      }
    }
    if (__any_sync(FULL, to_bits)) spill = true;  // an overflow keeps later lookups exact
    inserted += __popc(__ballot_sync(FULL, added));
    const unsigned nwm = __ballot_sync(FULL, newword);
    if (newword) touched[ntouch + __popc(nwm & ((1u << lane) - 1u))] = id >> 5;
    ntouch += __popc(nwm);
    return fresh;
  }
};

// distances of `cnt` rows (ids in lanes 0..cnt-1 of `my`) to the query.
// INTS: warp-cooperative coalesced rows (any summation order is exact);
// else one lane per row in the reference's order.
template <bool INTS>
__device__ __forceinline__ float batch_dist(const float *__restrict__ base, uint32_t d, uint32_t my, int cnt,
                                            const float *qv, int lane, float qn = 0.f,
                                            const float *__restrict__ xnorm = nullptr) {
  float out = 0.f;
  const uint32_t d4 = d >> 2;
  if (INTS) {
    // with row norms (d <= 128): |q|^2 + |x|^2 - 2 q.x, integers below 2^24
    // throughout (|q|^2 + |x|^2 <= 2 * 128 * 255^2), so exact; else the
    // difference form, exact in any order for d <= 256
    const bool dot = xnorm != nullptr;
    const float xn = (dot && lane < cnt) ? __ldg(xnorm + my) : 0.f;
    const float4 *q4 = reinterpret_cast<const float4 *>(qv);
    constexpr int G = 8;
    for (int c0 = 0; c0 < cnt; c0 += G) {
      float part[G];
      unsigned long long pacc[G];  // packed accumulators of the dot form
      const float4 *row[G];
#pragma unroll
      for (int g = 0; g < G; g++) {
        const int c = c0 + g;
        const uint32_t id = __shfl_sync(FULL, my, c & 31);
        part[g] = 0.f;
        pacc[g] = 0ull;
        // rows past cnt read row 0 (in bounds) and are ignored: no branch
        // keeps the G loads from issuing together
        row[g] = reinterpret_cast<const float4 *>(base + (size_t)(c < cnt ? id : 0u) * d);
      }
      // chunk-major: all G rows' loads of one step are issued before any math
      for (uint32_t k = lane; k < d4; k += 32) {
        const float4 qk = q4[k];
        float4 x[G];
#pragma unroll
        for (int g = 0; g < G; g++) x[g] = __ldg(row[g] + k);
        if (dot) {
          // packed FMAs: two dimensions per instruction (integer sums: exact)
#pragma unroll
          for (int g = 0; g < G; g++) {
            fma2(pacc[g], x[g].x, x[g].y, qk.x, qk.y);
            fma2(pacc[g], x[g].z, x[g].w, qk.z, qk.w);
          }
        } else {
#pragma unroll
          for (int g = 0; g < G; g++) part[g] += group4(x[g], qk);
        }
      }
      if (dot) {
#pragma unroll
        for (int g = 0; g < G; g++) part[g] = sum2(pacc[g]);
      }
      // transpose-reduce the 8 rows' dot products over the warp (10
      // shuffles, not 40): lanes exchange halves at distances 16, 8, 4 so
      // that each lane keeps one row, then finish over distances 2, 1.  Lane
      // l ends with row 4*bit4(l) + 2*bit3(l) + bit2(l).
      const bool b16 = lane & 16, b8 = lane & 8, b4 = lane & 4;
      float w[4];
#pragma unroll
      for (int j = 0; j < 4; j++) {
        const float send = b16 ? part[j] : part[j + 4];
        w[j] = (b16 ? part[j + 4] : part[j]) + __shfl_xor_sync(FULL, send, 16);
      }
      float x2[2];
#pragma unroll
      for (int j = 0; j < 2; j++) {
        const float send = b8 ? w[j] : w[j + 2];
        x2[j] = (b8 ? w[j + 2] : w[j]) + __shfl_xor_sync(FULL, send, 8);
      }
      float y = (b4 ? x2[1] : x2[0]) + __shfl_xor_sync(FULL, b4 ? x2[0] : x2[1], 4);
      y += __shfl_xor_sync(FULL, y, 2);
      y += __shfl_xor_sync(FULL, y, 1);
      // lane c0 + g takes row g from a lane that holds it
      const int g = (lane - c0) & 7;
      const float t = __shfl_sync(FULL, y, ((g >> 2) << 4) | (((g >> 1) & 1) << 3) | ((g & 1) << 2));
      if (lane >= c0 && lane < c0 + G) out = dot ? qn + xn - 2.f * t : t;
    }
  } else if (lane < cnt) {
    const float4 *row = reinterpret_cast<const float4 *>(base + (size_t)my * d);
    const float4 *q4 = reinterpret_cast<const float4 *>(qv);
#pragma unroll 8
    for (uint32_t g = 0; g < d4; g++) out = __fadd_rn(out, group4(__ldg(row + g), q4[g]));
  }
  return out;
}

}  // namespace
}  // namespace wv
