// Graph construction on the GPU: INIT_RANDOM, INIT_RAND, REFINE_NN_DESCENT and REFINE_EFANNA.
#pragma once
#include <cstdint>

#include "wv_ctx.h"

namespace wv {

struct NndParams {
  uint32_t S, K, L, ITER, R;
  // ComponentRefineEFANNA's init (random nn_new, sorted de-duplicated pools)
  // instead of ComponentRefineNNDescent's
  bool efanna = false;
};

struct NndStats {
  unsigned long long overflow_events = 0;  // reverse-list overwrites (rand() draws)
  unsigned long long offers = 0;           // offers that reached the per-target merge
  unsigned long long pairs = 0;            // local-join distance evaluations
  unsigned chunks = 0;                     // join chunks over all iterations
  float ms_join = 0, ms_update = 0;
};

// ComponentInitRandom::InitInner: rows of width S into ctx->fg_*
int init_random_gpu(wv_ctx *c, uint32_t S);
// ComponentInitRand::InitInner (the Vamana init): rows of width L into ctx->fg_*
int init_rand_gpu(wv_ctx *c, uint32_t L);
// ComponentRefineNNDescent::RefineInner / ComponentRefineEFANNA::RefineInner:
// ctx->fg_* (init graph) -> ctx->fg_* (width K)
int nndescent_gpu(wv_ctx *c, const NndParams &p, NndStats *st);
// mt19937 outputs [0, count) for `seed` (tests)
int mt19937_gpu(wv_ctx *c, uint32_t seed, uint32_t *d_out, size_t count);

}  // namespace wv
