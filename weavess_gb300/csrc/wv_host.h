// Host-side pieces of the drop-in: the rand() stream the reference draws from,
// GenRandom, and the seed draws of the search-entry components.  These are
// sequential by nature (one shared stream), cheap, and run on the host exactly
// as the reference runs them; everything per-vector runs on the GPU.
#pragma once
#include <cstdint>
#include <random>
#include <vector>

namespace wv {

// glibc's rand(): the TYPE_3 additive feedback generator (r[i] = r[i-3] +
// r[i-31] mod 2^32, output r[i] >> 1) seeded by a 16807 Lehmer sequence with
// 310 discarded outputs.  Reproduces the stream a fresh process sees (seed 1).
class GlibcRand {
 public:
  explicit GlibcRand(uint32_t seed = 1) { seed_with(seed); }
  void seed_with(uint32_t seed);
  int next() { return (int)(step() >> 1); }

 private:
  uint32_t step() {
    uint32_t v = r_[(i_ + 3) % 34] + r_[(i_ + 31) % 34];
    r_[i_] = v;
    i_ = (i_ + 1) % 34;
    return v;
  }
  uint32_t r_[34];
  int i_ = 0;
};

// The rand() source a context draws from: its own glibc-compatible stream or
// a caller function (the process's rand when embedded in a reference process).
struct RandSource {
  GlibcRand own;
  int (*fn)(void) = nullptr;
  unsigned long long drawn = 0;  // values handed out
  int next() {
    drawn++;
    return fn ? fn() : own.next();
  }
};

// GenRandom (include/weavess/util.h:13-27): `size` distinct ids in [0, N)
void gen_random(std::mt19937 &rng, uint32_t *addr, uint32_t size, uint32_t N);

// SearchEntryRand seeds (component_search_entry.cpp:9-30): per query one
// rand() seeds an mt19937 that draws L ids.  The rand() values are drawn in
// query order; the per-query mt19937 work then runs on host threads.
void draw_seeds_rand(RandSource &rnd, uint32_t nq, uint32_t L, uint32_t N, uint32_t *seeds, uint32_t stride);

// SearchEntryCentroid seeds (component_search_entry.cpp:33-67): the first L
// ids of the entry point's row, then rand() % N draws that skip taken ids.
void draw_seeds_centroid(RandSource &rnd, uint32_t nq, uint32_t L, uint32_t N, const uint32_t *ep_row,
                         uint32_t ep_deg, uint32_t *seeds, uint32_t stride);

// Seeds for the build-time greedy searches (CandidateNSG / entry centroid /
// conn findroot, component_candidate.cpp:17-31): first L ids of `row`, then
// rand() % N draws skipping taken ids.  One set per call.
void draw_seeds_row(RandSource &rnd, uint32_t L, uint32_t N, const uint32_t *row, uint32_t deg, uint32_t *out);

}  // namespace wv
