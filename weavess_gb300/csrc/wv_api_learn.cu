// C ABI of the learned entry point / beam width (wv_learn.cu).
#include <vector>

#include "wv_ctx.h"
#include "wv_learn.h"
#include "wv_seeds.h"

using namespace wv;

extern "C" {

void wv_learn_default_params(wv_learn_params *p) {
  if (!p) return;
  LearnParams d;
  *p = wv_learn_params{d.clusters, d.kmeans_iters, d.list_len, d.L_trace, d.epochs, d.batch, d.lr, d.lam,
                       d.L_min,    d.L_max,        d.target_agreement,      d.fallback_p, d.seed};
}

int wv_learn_fit(wv_ctx *c, const float *train_q, uint32_t nt, const wv_learn_params *p, wv_learn_report *rep) {
  if (!c || !train_q || !p) return WV_ERR_ARG;
  WV_CUDA(c, cudaSetDevice(c->device));
  LearnParams lp;
  lp.clusters = p->clusters;
  lp.kmeans_iters = p->kmeans_iters;
  lp.list_len = p->list_len;
  lp.L_trace = p->L_trace;
  lp.epochs = p->epochs;
  lp.batch = p->batch;
  lp.lr = p->lr;
  lp.lam = p->lam;
  lp.L_min = p->L_min;
  lp.L_max = p->L_max;
  lp.target_agreement = p->target_agreement;
  lp.fallback_p = p->fallback_p;
  lp.seed = p->seed;
  WV_CHECK(c, lp.batch >= 32 && lp.batch < nt, WV_ERR_ARG, "batch must be in [32, nt)");
  WV_CHECK(c, lp.L_trace >= 10 && lp.L_trace < c->n && lp.L_max < c->n && lp.L_min >= 10, WV_ERR_ARG,
           "beam limits out of range");
  LearnReport r;
  c->generation++;
  int rc = learn_fit(c, train_q, nt, lp, &r);
  if (rep) *rep = wv_learn_report{r.loss_ce, r.loss_mse, r.margin, r.val_agreement, r.ms, r.mean_label_L, r.steps,
                                  r.labelled};
  return rc;
}

int wv_search_learned_device(wv_ctx *c, const float *d_queries, uint32_t nq, uint32_t K, const uint32_t *d_plain_seeds,
                             uint32_t *d_out_ids, float *d_out_dist, wv_counters *counters) {
  if (!c || !d_queries || !d_out_ids) return WV_ERR_ARG;
  if (nq == 0) return WV_OK;
  WV_CUDA(c, cudaSetDevice(c->device));
  return learn_search(c, d_queries, nq, K, d_out_ids, d_out_dist, counters, d_plain_seeds, nullptr);
}

int wv_search_learned(wv_ctx *c, const float *queries, uint32_t nq, uint32_t K, uint32_t *out_ids, float *out_dist,
                      wv_counters *counters, uint32_t *out_L) {
  if (!c || !queries || !out_ids) return WV_ERR_ARG;
  if (nq == 0) return WV_OK;
  WV_CUDA(c, cudaSetDevice(c->device));
  WV_CHECK(c, c->learn, WV_ERR_STATE, "no trained model (call wv_learn_fit)");
  // the plain seeds of the fallback (and of short entry lists), drawn as
  // SearchEntryRand draws them; skipped when the model can read none
  const uint32_t Lp = learn_plain_beam(c);
  cudaError_t e = cudaSuccess;
  float *dq = c->buf<float>("sl_q", (size_t)nq * c->d, &e);
  uint32_t *ds = Lp ? c->buf<uint32_t>("sl_s", (size_t)nq * Lp, &e) : nullptr;
  uint32_t *dout = c->buf<uint32_t>("sl_o", (size_t)nq * K, &e);
  float *dd = out_dist ? c->buf<float>("sl_d", (size_t)nq * K, &e) : nullptr;
  uint32_t *dL = c->buf<uint32_t>("sl_L", nq, &e);
  WV_CUDA(c, e);
  WV_CUDA(c, cudaMemcpyAsync(dq, queries, (size_t)nq * c->d * 4, cudaMemcpyHostToDevice, c->stream));
  if (Lp) {
    const int rc = draw_seeds_rand_device(c, nq, nullptr, Lp, Lp, ds, Lp);
    if (rc) return rc;
  }
  int rc = learn_search(c, dq, nq, K, dout, dd, counters, ds, dL);
  if (rc) return rc;
  WV_CUDA(c, cudaMemcpyAsync(out_ids, dout, (size_t)nq * K * 4, cudaMemcpyDeviceToHost, c->stream));
  if (out_dist) WV_CUDA(c, cudaMemcpyAsync(out_dist, dd, (size_t)nq * K * 4, cudaMemcpyDeviceToHost, c->stream));
  if (out_L) WV_CUDA(c, cudaMemcpyAsync(out_L, dL, (size_t)nq * 4, cudaMemcpyDeviceToHost, c->stream));
  WV_CUDA(c, cudaStreamSynchronize(c->stream));
  return WV_OK;
}

int wv_learn_predict(wv_ctx *c, const float *q, uint32_t nq, uint32_t *cluster, float *prob, float *log2L) {
  if (!c || !q) return WV_ERR_ARG;
  WV_CUDA(c, cudaSetDevice(c->device));
  return learn_predict(c, q, nq, cluster, prob, log2L);
}

int wv_learn_assign(wv_ctx *c, const uint32_t *ids, uint32_t n, uint32_t *cluster) {
  if (!c || !ids || !cluster) return WV_ERR_ARG;
  return learn_assign(c, ids, n, cluster);
}

int wv_learn_set_margin(wv_ctx *c, float margin) {
  if (!c || !(margin > 0.f)) return WV_ERR_ARG;
  WV_CHECK(c, c->learn, WV_ERR_STATE, "no trained model");
  c->generation++;
  return learn_set_margin(c, margin);
}

int wv_learn_set_fallback(wv_ctx *c, float p, uint32_t L_plain) {
  if (!c || !(p >= 0.f && p <= 1.f)) return WV_ERR_ARG;
  WV_CHECK(c, c->learn, WV_ERR_STATE, "no trained model");
  WV_CHECK(c, L_plain >= 1 && L_plain < c->n && L_plain <= SEARCH_MAX_L, WV_ERR_ARG,
           "fallback beam %u (1..min(n - 1, %u))", L_plain, SEARCH_MAX_L);
  c->generation++;
  return learn_set_fallback(c, p, L_plain);
}

int wv_learn_plain_beam(wv_ctx *c, uint32_t *L) {
  if (!c || !L) return WV_ERR_ARG;
  WV_CHECK(c, c->learn, WV_ERR_STATE, "no trained model");
  *L = learn_plain_beam(c);
  return WV_OK;
}

int wv_learn_param_count(uint32_t d, uint32_t clusters, unsigned long long *count) {
  if (!count || d == 0 || clusters < 2) return WV_ERR_ARG;
  *count = learn_param_count(d, clusters);
  return WV_OK;
}

int wv_learn_grad(wv_ctx *c, const float *x, const uint32_t *yc, const float *yr, uint32_t B, uint32_t clusters,
                  const float *params, float lam, float *grad, float *loss) {
  if (!c || !x || !yc || !yr || !params || !grad || !loss || B == 0) return WV_ERR_ARG;
  WV_CHECK(c, c->d > 0, WV_ERR_STATE, "upload a base first (it sets the input width)");
  for (uint32_t i = 0; i < B; i++) WV_CHECK(c, yc[i] < clusters, WV_ERR_ARG, "label %u >= clusters", yc[i]);
  WV_CUDA(c, cudaSetDevice(c->device));
  c->generation++;
  return learn_grad(c, x, yc, yr, B, clusters, params, lam, grad, loss);
}

}  // extern "C"
