// C ABI: build components and the graph passed between them.
#include <algorithm>
#include <chrono>
#include <vector>

#include "wv_ctx.h"
#include "wv_link.h"
#include "wv_nnd.h"
#include "wv_search.h"

using namespace wv;

extern "C" {

int wv_set_graph(wv_ctx *c, const uint32_t *ids, const float *dist, const uint32_t *deg, uint32_t n, uint32_t width,
                 uint32_t ep) {
  if (!c) return WV_ERR_ARG;
  WV_CHECK(c, ids && deg && n > 0 && width > 0, WV_ERR_ARG, "empty graph");
  WV_CHECK(c, n == c->n, WV_ERR_ARG, "graph has %u rows, base has %u", n, c->n);
  for (uint32_t i = 0; i < n; i++)
    WV_CHECK(c, deg[i] <= width, WV_ERR_ARG, "row %u has degree %u > width %u", i, deg[i], width);
  WV_CUDA(c, cudaSetDevice(c->device));
  WV_CUDA(c, c->fg_ids.ensure((size_t)n * width * 4));
  WV_CUDA(c, c->fg_dist.ensure((size_t)n * width * 4));
  WV_CUDA(c, c->fg_deg.ensure((size_t)n * 4));
  WV_CUDA(c, cudaMemcpyAsync(c->fg_ids.p, ids, (size_t)n * width * 4, cudaMemcpyHostToDevice, c->stream));
  if (dist) WV_CUDA(c, cudaMemcpyAsync(c->fg_dist.p, dist, (size_t)n * width * 4, cudaMemcpyHostToDevice, c->stream));
  else WV_CUDA(c, cudaMemsetAsync(c->fg_dist.p, 0, (size_t)n * width * 4, c->stream));
  WV_CUDA(c, cudaMemcpyAsync(c->fg_deg.p, deg, (size_t)n * 4, cudaMemcpyHostToDevice, c->stream));
  WV_CUDA(c, cudaStreamSynchronize(c->stream));
  c->fg_n = n;
  c->fg_w = width;
  c->fg_ep = ep;
  c->fg_has_ep = true;
  c->fg_eps.clear();
  return WV_OK;
}

int wv_graph_width(wv_ctx *c, uint32_t *width, uint32_t *ep) {
  if (!c || !width) return WV_ERR_ARG;
  WV_CHECK(c, c->fg_n > 0, WV_ERR_STATE, "no graph built");
  *width = c->fg_w;
  if (ep) *ep = c->fg_ep;
  return WV_OK;
}

int wv_get_graph(wv_ctx *c, uint32_t *ids, float *dist, uint32_t *deg, uint32_t width) {
  if (!c) return WV_ERR_ARG;
  WV_CHECK(c, c->fg_n > 0, WV_ERR_STATE, "no graph built");
  WV_CHECK(c, width >= c->fg_w, WV_ERR_ARG, "width %u < graph width %u", width, c->fg_w);
  WV_CUDA(c, cudaSetDevice(c->device));
  const size_t n = c->fg_n, w = c->fg_w;
  if (ids)
    WV_CUDA(c, cudaMemcpy2DAsync(ids, width * 4, c->fg_ids.p, w * 4, w * 4, n, cudaMemcpyDeviceToHost, c->stream));
  if (dist)
    WV_CUDA(c, cudaMemcpy2DAsync(dist, width * 4, c->fg_dist.p, w * 4, w * 4, n, cudaMemcpyDeviceToHost, c->stream));
  if (deg) WV_CUDA(c, cudaMemcpyAsync(deg, c->fg_deg.p, n * 4, cudaMemcpyDeviceToHost, c->stream));
  WV_CUDA(c, cudaStreamSynchronize(c->stream));
  return WV_OK;
}

int wv_load_built_graph(wv_ctx *c) {
  if (!c) return WV_ERR_ARG;
  WV_CHECK(c, c->fg_n > 0 && c->fg_n == c->n, WV_ERR_STATE, "no graph built for the uploaded base");
  WV_CHECK(c, c->fg_w <= SEARCH_MAX_WIDTH, WV_ERR_LIMIT, "graph width %u above %u", c->fg_w, SEARCH_MAX_WIDTH);
  WV_CUDA(c, cudaSetDevice(c->device));
  const size_t n = c->fg_n, w = c->fg_w;
  WV_CUDA(c, c->gids.ensure(n * w * 4));
  WV_CUDA(c, c->gdeg.ensure(n * 4));
  WV_CUDA(c, cudaMemcpyAsync(c->gids.p, c->fg_ids.p, n * w * 4, cudaMemcpyDeviceToDevice, c->stream));
  WV_CUDA(c, cudaMemcpyAsync(c->gdeg.p, c->fg_deg.p, n * 4, cudaMemcpyDeviceToDevice, c->stream));
  const uint32_t ep = c->fg_has_ep ? c->fg_ep : 0;
  uint32_t dep = 0;
  WV_CUDA(c, cudaMemcpyAsync(&dep, c->fg_deg.as<uint32_t>() + ep, 4, cudaMemcpyDeviceToHost, c->stream));
  WV_CUDA(c, cudaStreamSynchronize(c->stream));
  c->ep_row.resize(dep);
  if (dep)
    WV_CUDA(c, cudaMemcpy(c->ep_row.data(), c->fg_ids.as<uint32_t>() + (size_t)ep * w, dep * 4,
                          cudaMemcpyDeviceToHost));
  c->generation++;
  c->gn = (uint32_t)n;
  c->gw = (uint32_t)w;
  c->ep = ep;
  c->eps = c->fg_eps;
  if (c->vis_words != (n + 31) / 32) c->vis_slots = 0;
  return WV_OK;
}

int wv_init_random(wv_ctx *c, uint32_t S, wv_build_stats *stats) {
  if (!c) return WV_ERR_ARG;
  WV_CUDA(c, cudaSetDevice(c->device));
  auto t0 = std::chrono::steady_clock::now();
  int rc = init_random_gpu(c, S);
  if (stats) {
    *stats = wv_build_stats{};
    stats->rand_draws = 1;
    stats->ms_total = std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t0).count();
  }
  return rc;
}

int wv_init_rand(wv_ctx *c, uint32_t L, wv_build_stats *stats) {
  if (!c) return WV_ERR_ARG;
  WV_CUDA(c, cudaSetDevice(c->device));
  auto t0 = std::chrono::steady_clock::now();
  int rc = init_rand_gpu(c, L);
  if (stats) {
    *stats = wv_build_stats{};
    stats->rand_draws = 1;
    stats->ms_total = std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t0).count();
  }
  return rc;
}

int wv_init_kdt(wv_ctx *c, uint32_t nTrees, uint32_t K, uint32_t mLevel, wv_build_stats *stats) {
  if (!c) return WV_ERR_ARG;
  WV_CUDA(c, cudaSetDevice(c->device));
  auto t0 = std::chrono::steady_clock::now();
  const unsigned long long d0 = c->rnd.drawn;
  int rc = init_kdt_gpu(c, nTrees, K, mLevel);
  if (stats) {
    *stats = wv_build_stats{};
    stats->rand_draws = c->rnd.drawn - d0;
    stats->ms_total = std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t0).count();
  }
  return rc;
}

int wv_nnd_refine(wv_ctx *c, uint32_t S, uint32_t K, uint32_t L, uint32_t ITER, uint32_t R, wv_build_stats *stats) {
  if (!c) return WV_ERR_ARG;
  WV_CUDA(c, cudaSetDevice(c->device));
  auto t0 = std::chrono::steady_clock::now();
  NndStats st;
  int rc = nndescent_gpu(c, NndParams{S, K, L, ITER, R}, &st);
  if (stats) {
    *stats = wv_build_stats{};
    stats->rand_draws = st.overflow_events;
    stats->offers = st.offers;
    stats->pairs = st.pairs;
    stats->chunks = st.chunks;
    stats->ms_join = st.ms_join;
    stats->ms_update = st.ms_update;
    stats->ms_total = std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t0).count();
  }
  return rc;
}

int wv_efanna_refine(wv_ctx *c, uint32_t S, uint32_t K, uint32_t L, uint32_t ITER, uint32_t R,
                     wv_build_stats *stats) {
  if (!c) return WV_ERR_ARG;
  WV_CUDA(c, cudaSetDevice(c->device));
  auto t0 = std::chrono::steady_clock::now();
  const unsigned long long d0 = c->rnd.drawn;
  NndStats st;
  NndParams np{S, K, L, ITER, R};
  np.efanna = true;
  int rc = nndescent_gpu(c, np, &st);
  if (stats) {
    *stats = wv_build_stats{};
    stats->rand_draws = c->rnd.drawn - d0;
    stats->offers = st.offers;
    stats->pairs = st.pairs;
    stats->chunks = st.chunks;
    stats->ms_join = st.ms_join;
    stats->ms_update = st.ms_update;
    stats->ms_total = std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t0).count();
  }
  return rc;
}

int wv_vamana_refine(wv_ctx *c, uint32_t L_refine, uint32_t R_refine, float alpha, uint32_t entry_L,
                     wv_build_stats *stats) {
  if (!c) return WV_ERR_ARG;
  WV_CUDA(c, cudaSetDevice(c->device));
  auto t0 = std::chrono::steady_clock::now();
  const unsigned long long d0 = c->rnd.drawn;
  LinkStats st;
  LinkParams lp{L_refine, R_refine, 0, alpha, entry_L, LinkMode::VAMANA};
  lp.clean = c->build_clean != 0;
  // clean mode: the entry point is the centroid search the link intends
  // (the reference's Vamana refine never sets the L_refine it reads)
  if (lp.clean && lp.entry_L == 0) lp.entry_L = L_refine;
  int rc = link_gpu(c, lp, &st);
  if (stats) {
    *stats = wv_build_stats{};
    stats->rand_draws = c->rnd.drawn - d0;
    stats->levels = st.levels;
    stats->ep = st.ep;
    stats->ms_total = std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t0).count();
  }
  return rc;
}

int wv_set_build_mode(wv_ctx *c, int mode) {
  if (!c) return WV_ERR_ARG;
  WV_CHECK(c, mode == WV_BUILD_COMPAT || mode == WV_BUILD_CLEAN, WV_ERR_ARG, "unknown build mode %d", mode);
  c->build_clean = mode == WV_BUILD_CLEAN ? 1 : 0;
  return WV_OK;
}

int wv_nsg_refine(wv_ctx *c, uint32_t L_refine, uint32_t R_refine, uint32_t C_refine, wv_build_stats *stats) {
  if (!c) return WV_ERR_ARG;
  WV_CUDA(c, cudaSetDevice(c->device));
  auto t0 = std::chrono::steady_clock::now();
  const unsigned long long d0 = c->rnd.drawn;
  LinkStats st;
  int rc = link_gpu(c, LinkParams{L_refine, R_refine, C_refine, 1.0f, L_refine, LinkMode::NSG}, &st);
  uint32_t added = 0;
  if (rc == WV_OK) rc = conn_dfs_gpu(c, L_refine, &added);
  if (stats) {
    *stats = wv_build_stats{};
    stats->rand_draws = c->rnd.drawn - d0;
    stats->levels = st.levels;
    stats->ep = st.ep;
    stats->conn_added = added;
    stats->ms_total = std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t0).count();
  }
  return rc;
}

int wv_ssg_refine(wv_ctx *c, uint32_t L_refine, uint32_t R_refine, float A, uint32_t n_try, uint32_t *eps,
                  wv_build_stats *stats) {
  if (!c) return WV_ERR_ARG;
  WV_CUDA(c, cudaSetDevice(c->device));
  WV_CHECK(c, n_try >= 1 && n_try <= c->n, WV_ERR_ARG, "n_try=%u out of range (n=%u)", n_try, c->n);
  auto t0 = std::chrono::steady_clock::now();
  const unsigned long long d0 = c->rnd.drawn;
  LinkStats st;
  LinkParams lp{L_refine, R_refine, 0, 1.0f, 0, LinkMode::SSG};
  lp.A = A;
  int rc = link_gpu(c, lp, &st);
  uint32_t added = 0;
  std::vector<uint32_t> roots;
  if (rc == WV_OK) rc = conn_ssg_gpu(c, n_try, R_refine, roots, &added);
  if (rc == WV_OK) {
    c->fg_eps = roots;
    if (eps) std::copy(roots.begin(), roots.end(), eps);
  }
  if (stats) {
    *stats = wv_build_stats{};
    stats->rand_draws = c->rnd.drawn - d0;
    stats->levels = st.levels;
    stats->conn_added = added;
    stats->ms_total = std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t0).count();
  }
  return rc;
}

}  // extern "C"
