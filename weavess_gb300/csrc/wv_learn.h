// Learned entry point / beam width (wv_learn.cu).
#pragma once
#include <cstdint>

#include "wv_ctx.h"

namespace wv {

struct LearnParams {
  uint32_t clusters = 64;      // entry clusters (k-means on the base)
  uint32_t kmeans_iters = 8;
  uint32_t list_len = 512;     // seeds kept per cluster
  uint32_t L_trace = 512;      // beam of the plain search that labels the traces
  uint32_t epochs = 6, batch = 1024;
  float lr = 1e-3f, lam = 0.5f;  // Adam step, weight of the beam regressor
  uint32_t L_min = 16, L_max = 512;
  float target_agreement = 0.97f;  // held-out agreement with the plain answers
  float fallback_p = 0.f;          // top-1 probability under which the plain search runs
  uint32_t seed = 1234;
};

struct LearnReport {
  float loss_ce = 0, loss_mse = 0, margin = 0, val_agreement = 0, ms = 0, mean_label_L = 0;
  uint32_t steps = 0, labelled = 0;
};

int learn_fit(wv_ctx *c, const float *train_q, uint32_t nt, const LearnParams &p, LearnReport *rep);
// learned search of nq device queries; d_plain_seeds: nq x L_trace rand seeds
// (fallback and fill), or null
int learn_search(wv_ctx *c, const float *dq, uint32_t nq, uint32_t K, uint32_t *dout, float *ddist,
                 wv_counters *counters, const uint32_t *d_plain_seeds, uint32_t *d_Lq_out);
// the same without synchronizing, for a captured plan: work buffers named
// with `pfx` for nq_max queries (learn_prepare, before the capture; *Lcap the
// beam the search kernel is sized for, *stride the seed row stride), then
// the forward pass, the seed kernel and the search of the first *d_nq
// queries (per-query K optional, capped by K) on the caller's visited
// scratch; ev0 / ev1 (nullable) are recorded around the search kernel
int learn_prepare(wv_ctx *c, const char *pfx, uint32_t nq_max, uint32_t *Lcap, uint32_t *stride);
int learn_enqueue(wv_ctx *c, const char *pfx, const float *dq, uint32_t nq_max, const uint32_t *d_nq, uint32_t K,
                  const uint32_t *d_K, uint32_t *dout, float *ddist, uint32_t out_stride,
                  const uint32_t *d_plain_seeds, SearchShape shape, int blocks, const SearchScratch &scr,
                  cudaEvent_t ev0 = nullptr, cudaEvent_t ev1 = nullptr);
// loss and gradients of a batch for given parameters (gradient check)
int learn_grad(wv_ctx *c, const float *x, const uint32_t *yc, const float *yr, uint32_t B, uint32_t C,
               const float *params, float lam, float *grad, float *loss);
size_t learn_param_count(uint32_t d, uint32_t C);
int learn_set_margin(wv_ctx *c, float margin);
int learn_set_fallback(wv_ctx *c, float p, uint32_t L_plain);
int learn_predict(wv_ctx *c, const float *q, uint32_t nq, uint32_t *cluster, float *prob, float *log2L);
int learn_assign(wv_ctx *c, const uint32_t *ids, uint32_t n, uint32_t *cluster);
// plain seeds per query the learned search may read (the trace beam), or 0
// when no query can read one (no fallback, every entry list covers L_max)
uint32_t learn_plain_beam(wv_ctx *c);
void learn_free(wv_ctx *c);

}  // namespace wv
