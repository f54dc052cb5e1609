#include "wv_host.h"

#include <algorithm>
#include <cstring>

namespace wv {

void GlibcRand::seed_with(uint32_t seed) {
  if (seed == 0) seed = 1;
  int32_t w = (int32_t)seed;
  r_[0] = (uint32_t)w;
  for (int k = 1; k < 31; k++) {
    // 16807 * w mod (2^31 - 1) without overflow (Schrage)
    int32_t hi = w / 127773, lo = w % 127773;
    w = 16807 * lo - 2836 * hi;
    if (w < 0) w += 2147483647;
    r_[k] = (uint32_t)w;
  }
  for (int k = 31; k < 34; k++) r_[k] = r_[k - 31];
  i_ = 0;
  // r_[i_] is the oldest word; the next word is r[n-31] + r[n-3], which sit
  // 3 and 31 slots after i_ in the ring of 34
  for (int k = 0; k < 310; k++) step();
}

void gen_random(std::mt19937 &rng, uint32_t *addr, uint32_t size, uint32_t N) {
  for (uint32_t i = 0; i < size; ++i) addr[i] = (uint32_t)(rng() % (N - size));
  std::sort(addr, addr + size);
  for (uint32_t i = 1; i < size; ++i)
    if (addr[i] <= addr[i - 1]) addr[i] = addr[i - 1] + 1;
  uint32_t off = (uint32_t)(rng() % N);
  for (uint32_t i = 0; i < size; ++i) addr[i] = (addr[i] + off) % N;
}

void draw_seeds_rand(RandSource &rnd, uint32_t nq, uint32_t L, uint32_t N, uint32_t *seeds, uint32_t stride) {
  std::vector<uint32_t> sv(nq);
  for (uint32_t q = 0; q < nq; q++) sv[q] = (uint32_t)rnd.next();
#pragma omp parallel for schedule(static)
  for (int64_t q = 0; q < (int64_t)nq; q++) {
    std::mt19937 rng(sv[q]);
    gen_random(rng, seeds + (size_t)q * stride, L, N);
  }
}

namespace {
// small open-addressing id set (ids < 2^32 - 1)
struct IdSet {
  std::vector<uint32_t> slot;
  uint32_t mask;
  explicit IdSet(uint32_t expect) {
    uint32_t cap = 16;
    while (cap < 2 * expect + 2) cap <<= 1;
    slot.assign(cap, 0xffffffffu);
    mask = cap - 1;
  }
  // returns true if inserted (was absent)
  bool insert(uint32_t id) {
    uint32_t h = (id * 2654435761u) & mask;
    while (slot[h] != 0xffffffffu) {
      if (slot[h] == id) return false;
      h = (h + 1) & mask;
    }
    slot[h] = id;
    return true;
  }
};
}  // namespace

void draw_seeds_row(RandSource &rnd, uint32_t L, uint32_t N, const uint32_t *row, uint32_t deg, uint32_t *out) {
  IdSet set(L);
  uint32_t t = 0;
  for (; t < L && t < deg; t++) {
    out[t] = row[t];
    set.insert(row[t]);
  }
  while (t < L) {
    uint32_t id = (uint32_t)rnd.next() % N;
    if (!set.insert(id)) continue;
    out[t++] = id;
  }
}

void draw_seeds_centroid(RandSource &rnd, uint32_t nq, uint32_t L, uint32_t N, const uint32_t *ep_row,
                         uint32_t ep_deg, uint32_t *seeds, uint32_t stride) {
  for (uint32_t q = 0; q < nq; q++) draw_seeds_row(rnd, L, N, ep_row, ep_deg, seeds + (size_t)q * stride);
}

}  // namespace wv
