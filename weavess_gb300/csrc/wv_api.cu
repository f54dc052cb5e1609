// C ABI: context, data upload and search entry points (include/weavess_gpu.h).
#include <algorithm>
#include <cstring>

#include "wv_ctx.h"
#include "wv_learn.h"
#include "wv_search.h"
#include "wv_seeds.h"

using namespace wv;

namespace wv {

int check_device_status(wv_ctx *c, const char *what) {
  int st = 0;
  WV_CUDA(c, cudaMemcpyAsync(&st, c->d_status(), sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  WV_CUDA(c, cudaStreamSynchronize(c->stream));
  if (st != 0) {
    WV_CUDA(c, cudaMemsetAsync(c->d_status(), 0, sizeof(int), c->stream));
    const char *why = st == 1 ? "an id >= n or a row longer than the graph width"
                      : st == 2 ? "a bounded device buffer overflowed"
                                : "a bounded wait timed out";
    return fail(c, WV_ERR_DEVICE, "%s: kernel reported %s (code %d)", what, why, st);
  }
  return WV_OK;
}

}  // namespace wv

namespace {

__global__ void k_check_int(const float *x, size_t count, int *ok) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < count; i += (size_t)gridDim.x * blockDim.x) {
    const float v = x[i];
    if (!(v >= 0.f && v <= 255.f && v == rintf(v))) {
      *ok = 0;
      return;
    }
  }
}

// status code; *out_blocks = the persistent grid of the shape
// squared norm of every row (warp per row; on integer data any order is exact)
__global__ void k_row_norms(const float *x, uint32_t n, uint32_t d, float *out) {
  const int lane = threadIdx.x & 31;
  const uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t r = w; r < n; r += nw) {
    float a = 0.f;
    for (uint32_t k = lane; k < d; k += 32) a = fmaf(x[(size_t)r * d + k], x[(size_t)r * d + k], a);
    for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(FULL, a, o);
    if (lane == 0) out[r] = a;
  }
}

int ensure_search_scratch(wv_ctx *c, uint32_t Lmax, SearchShape sh, int *out_blocks) {
  int blocks = route_grid(c, Lmax, sh);
  WV_CHECK(c, blocks > 0, WV_ERR_LIMIT, "search kernel cannot run with d=%u L=%u width=%u (shared memory)", c->d,
           Lmax, c->gw);
  size_t slots = (size_t)blocks * sh.wpb;
  size_t words = (c->n + 31) / 32;
  if (slots > c->vis_slots || words != c->vis_words) {
    c->visited.release();
    c->touched.release();
    WV_CUDA(c, c->visited.ensure(slots * words * 4));
    WV_CUDA(c, c->touched.ensure(slots * words * 4));
    WV_CUDA(c, cudaMemsetAsync(c->visited.p, 0, slots * words * 4, c->stream));
    c->vis_slots = slots;
    c->vis_words = words;
  }
  *out_blocks = blocks;
  return WV_OK;
}

}  // namespace

int wv::search_prepare(wv_ctx *c, uint32_t Lmax, SearchShape shape, int *blocks) {
  return ensure_search_scratch(c, Lmax, shape, blocks);
}

SearchArgs wv::search_args(wv_ctx *c, const float *d_q, uint32_t nq, const uint32_t *nq_dev, const uint32_t *d_seeds,
                           uint32_t seed_stride, const uint32_t *d_L, const uint32_t *d_K, uint32_t L, uint32_t K,
                           uint32_t Lmax, uint32_t *d_out, float *d_dist, uint32_t out_stride) {
  SearchArgs a{};
  a.base = c->base.as<float>();
  a.n = c->n;
  a.d = c->d;
  a.gids = c->gids.as<uint32_t>();
  a.gdeg = c->gdeg.as<uint32_t>();
  a.gw = c->gw;
  a.queries = d_q;
  a.nq = nq;
  a.nq_dev = nq_dev;
  a.seeds = d_seeds;
  a.seed_stride = seed_stride;
  a.Lq = d_L;
  a.Kq = d_K;
  a.L = L;
  a.K = K;
  a.Lmax = Lmax;
  a.out_ids = d_out;
  a.out_dist = d_dist;
  a.out_stride = out_stride;
  a.counters = c->d_counters();
  a.visited = c->visited.as<uint32_t>();
  a.touched = c->touched.as<uint32_t>();
  a.words = (uint32_t)c->vis_words;
  a.cap = c->gw + 32;
  a.next_query = c->d_next();
  a.status = c->d_status();
  a.int_exact = c->base_int;
  a.xnorm = c->xnorm.as<float>();
  a.storage = c->storage;
  a.qbase = c->qbase.p;
  a.qscale = c->qscale.as<float>();
  a.qnorm = c->qnorm.as<float>();
  a.rerank = c->rerank == 0 ? Lmax : c->rerank;
  a.parents = c->parents;
  return a;
}

int wv::route_grid(wv_ctx *c, uint32_t Lmax, SearchShape sh) {
  return c->parents > 0 ? beam_grid(c->d, Lmax, c->gw, c->parents, c->device, sh)
                        : search_grid(c->d, Lmax, c->gw + 32, c->device, sh);
}

int wv::search_enqueue(wv_ctx *c, const SearchArgs &a, SearchShape shape, int blocks) {
  WV_CUDA(c, cudaMemsetAsync(c->misc.p, 0, 32, c->stream));
  WV_CUDA(c, launch_search(a, shape, blocks, c->stream));
  return WV_OK;
}

// runs the kernel on device-resident queries / seeds / outputs
int wv::run_search_device(wv_ctx *c, const float *d_q, uint32_t nq, const uint32_t *d_seeds, uint32_t seed_stride,
               const uint32_t *d_L, const uint32_t *d_K, uint32_t L, uint32_t K, uint32_t Lmax, uint32_t *d_out,
               float *d_dist, uint32_t out_stride, wv_counters *counters, bool shift_seeds) {
  const SearchShape sh{};
  int blocks = 0;
  int rc = search_prepare(c, Lmax, sh, &blocks);
  if (rc) return rc;
  SearchArgs a =
      search_args(c, d_q, nq, nullptr, d_seeds, seed_stride, d_L, d_K, L, K, Lmax, d_out, d_dist, out_stride);
  a.seed_shift = shift_seeds ? 1 : 0;
  if (d_L) {
    cudaError_t e = cudaSuccess;
    a.order = c->buf<uint32_t>("search_order", nq, &e);
    WV_CUDA(c, e);
  }
  int nb = std::min<long>(blocks, ((long)nq + sh.wpb - 1) / sh.wpb);
  if (nb < 1) nb = 1;
  rc = search_enqueue(c, a, sh, nb);
  if (rc) return rc;
  if (counters) {
    unsigned long long h[2];
    WV_CUDA(c, cudaMemcpyAsync(h, c->d_counters(), 16, cudaMemcpyDeviceToHost, c->stream));
    WV_CUDA(c, cudaStreamSynchronize(c->stream));
    counters->dist_count = h[0];
    counters->hop_count = h[1];
  }
  return check_device_status(c, "search");
}

namespace {

int check_search_args(wv_ctx *c, uint32_t nq, uint32_t L, uint32_t K) {
  WV_CHECK(c, c->n > 0, WV_ERR_STATE, "no base uploaded");
  WV_CHECK(c, c->gn == c->n, WV_ERR_STATE, "no search graph for the uploaded base (graph n=%u, base n=%u)", c->gn,
           c->n);
  WV_CHECK(c, c->d % 4 == 0, WV_ERR_LIMIT, "dimension %u is not a multiple of 4", c->d);
  WV_CHECK(c, K >= 1 && L >= K, WV_ERR_ARG, "search_L cannot be smaller than search_K (L=%u K=%u)", L, K);
  WV_CHECK(c, L < c->n, WV_ERR_ARG, "L=%u must be smaller than n=%u", L, c->n);
  WV_CHECK(c, L <= SEARCH_MAX_L, WV_ERR_LIMIT, "L=%u above the supported maximum %u", L, SEARCH_MAX_L);
  (void)nq;
  return WV_OK;
}

// SearchEntrySubCentroid overwrites the first eps_.size() of L seeds
// (component_search_entry.cpp:77-80; the reference asserts they fit)
int check_roots(wv_ctx *c, uint32_t L) {
  WV_CHECK(c, !c->eps.empty(), WV_ERR_STATE, "sub-centroid entry needs the search graph's SSG roots");
  WV_CHECK(c, c->eps.size() <= L, WV_ERR_ARG, "%zu SSG roots do not fit L=%u", c->eps.size(), L);
  return WV_OK;
}

int draw(wv_ctx *c, uint32_t nq, int entry, uint32_t L, uint32_t *seeds, uint32_t stride) {
  if (entry == WV_ENTRY_RAND) {
    draw_seeds_rand(c->rnd, nq, L, c->n, seeds, stride);
  } else if (entry == WV_ENTRY_CENTROID) {
    WV_CHECK(c, c->gn == c->n, WV_ERR_STATE, "centroid entry needs the search graph");
    draw_seeds_centroid(c->rnd, nq, L, c->n, c->ep_row.data(), (uint32_t)c->ep_row.size(), seeds, stride);
  } else if (entry == WV_ENTRY_KDT) {
    return fail(c, WV_ERR_ARG, "the KD-tree entry takes the host queries of wv_search");
  } else if (entry == WV_ENTRY_SUB_CENTROID) {
    int rc = check_roots(c, L);
    if (rc) return rc;
    draw_seeds_rand(c->rnd, nq, L, c->n, seeds, stride);
    for (uint32_t q = 0; q < nq; q++) std::copy(c->eps.begin(), c->eps.end(), seeds + (size_t)q * stride);
  } else {
    return fail(c, WV_ERR_ARG, "unknown entry %d", entry);
  }
  return WV_OK;
}

}  // namespace

extern "C" {

int wv_ctx_create(wv_ctx **out, int device) {
  if (!out) return WV_ERR_ARG;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) return WV_ERR_STATE;
  wv_ctx *c = new wv_ctx();
  c->device = device;
  if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) !=
                                                  cudaSuccess) {
    delete c;
    return WV_ERR_CUDA;
  }
  c->own_stream = c->stream;
  cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, device);
  if (c->misc.ensure(64) != cudaSuccess) {
    cudaStreamDestroy(c->stream);
    delete c;
    return WV_ERR_NOMEM;
  }
  cudaMemset(c->misc.p, 0, 64);
  *out = c;
  return WV_OK;
}

int wv_ctx_destroy(wv_ctx *c) {
  if (!c) return WV_ERR_ARG;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  for (DevBuf *b : {&c->base, &c->gids, &c->gdeg, &c->visited, &c->touched, &c->misc, &c->q_buf, &c->seed_buf,
                    &c->out_ids_buf, &c->out_dist_buf, &c->lq_buf, &c->kq_buf, &c->fg_ids, &c->fg_dist,
                    &c->fg_deg, &c->qbase, &c->qscale})
    b->release();
  c->release_work();
  learn_free(c);
  cudaStreamDestroy(c->own_stream);
  delete c;
  return WV_OK;
}

const char *wv_last_error(const wv_ctx *c) { return c ? c->err.c_str() : "null context"; }

int wv_srand(wv_ctx *c, unsigned seed) {
  if (!c) return WV_ERR_ARG;
  c->rnd.own.seed_with(seed);
  return WV_OK;
}

int wv_set_rand_source(wv_ctx *c, int (*fn)(void)) {
  if (!c) return WV_ERR_ARG;
  c->rnd.fn = fn;
  return WV_OK;
}

int wv_set_stream(wv_ctx *c, void *stream) {
  if (!c) return WV_ERR_ARG;
  WV_CUDA(c, cudaStreamSynchronize(c->stream));
  c->stream = stream ? (cudaStream_t)stream : c->own_stream;
  return WV_OK;
}

int wv_rand(wv_ctx *c, int *out) {
  if (!c || !out) return WV_ERR_ARG;
  *out = c->rnd.next();
  return WV_OK;
}

int wv_upload_base(wv_ctx *c, const float *base, uint32_t n, uint32_t d) {
  if (!c) return WV_ERR_ARG;
  WV_CHECK(c, base && n > 0 && d > 0, WV_ERR_ARG, "empty base");
  WV_CHECK(c, (uint64_t)n * d < (1ull << 32), WV_ERR_LIMIT, "n*d=%llu overflows the reference's 32-bit offsets",
           (unsigned long long)n * d);
  WV_CUDA(c, cudaSetDevice(c->device));
  // a zero float follows the last row: SearchEntrySubCentroid reads the row
  // shifted by one float (component_search_entry.cpp:84-86)
  WV_CUDA(c, c->base.ensure((size_t)n * d * 4 + 16));
  WV_CUDA(c, cudaMemcpyAsync(c->base.p, base, (size_t)n * d * 4, cudaMemcpyHostToDevice, c->stream));
  WV_CUDA(c, cudaMemsetAsync(c->base.as<char>() + (size_t)n * d * 4, 0, 16, c->stream));
  WV_CUDA(c, cudaStreamSynchronize(c->stream));
  c->generation++;
  if (c->n != n) c->gn = 0;  // the old graph no longer matches
  c->storage = 0;            // a low-precision copy no longer matches
  c->kdt = wv::KdtForest{};  // nor do KD-trees of the old base
  c->n = n;
  c->d = d;
  int *ok = c->d_status() + 4;
  int one = 1, hok = 0;
  WV_CUDA(c, cudaMemcpyAsync(ok, &one, 4, cudaMemcpyHostToDevice, c->stream));
  k_check_int<<<c->sms * 8, 256, 0, c->stream>>>(c->base.as<float>(), (size_t)n * d, ok);
  WV_CUDA(c, cudaGetLastError());
  WV_CUDA(c, cudaMemcpyAsync(&hok, ok, 4, cudaMemcpyDeviceToHost, c->stream));
  WV_CUDA(c, cudaStreamSynchronize(c->stream));
  c->base_int = hok == 1;
  if (c->base_int) {
    // the distance kernels use |q|^2 + |x|^2 - 2 q.x on integer data (exact)
    WV_CUDA(c, c->xnorm.ensure((size_t)n * 4));
    k_row_norms<<<c->sms * 8, 256, 0, c->stream>>>(c->base.as<float>(), n, d, c->xnorm.as<float>());
    WV_CUDA(c, cudaGetLastError());
    WV_CUDA(c, cudaStreamSynchronize(c->stream));
  }
  return WV_OK;
}

int wv_upload_graph(wv_ctx *c, const uint32_t *ids, const uint32_t *deg, uint32_t n, uint32_t width, uint32_t ep) {
  if (!c) return WV_ERR_ARG;
  WV_CHECK(c, ids && deg && n > 0 && width > 0, WV_ERR_ARG, "empty graph");
  WV_CHECK(c, width <= SEARCH_MAX_WIDTH, WV_ERR_LIMIT, "graph width %u above %u", width, SEARCH_MAX_WIDTH);
  WV_CHECK(c, ep < n, WV_ERR_ARG, "entry point %u >= n=%u", ep, n);
  for (uint32_t i = 0; i < n; i++) WV_CHECK(c, deg[i] <= width, WV_ERR_ARG, "row %u has degree %u > width %u", i, deg[i], width);
  WV_CUDA(c, cudaSetDevice(c->device));
  WV_CUDA(c, c->gids.ensure((size_t)n * width * 4));
  WV_CUDA(c, c->gdeg.ensure((size_t)n * 4));
  WV_CUDA(c, cudaMemcpyAsync(c->gids.p, ids, (size_t)n * width * 4, cudaMemcpyHostToDevice, c->stream));
  WV_CUDA(c, cudaMemcpyAsync(c->gdeg.p, deg, (size_t)n * 4, cudaMemcpyHostToDevice, c->stream));
  WV_CUDA(c, cudaStreamSynchronize(c->stream));
  c->generation++;
  c->gn = n;
  c->gw = width;
  c->ep = ep;
  c->ep_row.assign(ids + (size_t)ep * width, ids + (size_t)ep * width + deg[ep]);
  c->eps.clear();
  if (c->vis_words != (n + 31) / 32) c->vis_slots = 0;
  return WV_OK;
}

int wv_set_eps(wv_ctx *c, const uint32_t *eps, uint32_t n_eps) {
  if (!c) return WV_ERR_ARG;
  WV_CHECK(c, c->gn == c->n && c->n > 0, WV_ERR_STATE, "upload the search graph first");
  WV_CHECK(c, n_eps == 0 || eps, WV_ERR_ARG, "null roots");
  for (uint32_t i = 0; i < n_eps; i++) WV_CHECK(c, eps[i] < c->n, WV_ERR_ARG, "root %u >= n=%u", eps[i], c->n);
  c->eps.assign(eps, eps + n_eps);
  c->generation++;
  return WV_OK;
}

int wv_get_eps(wv_ctx *c, int built, uint32_t *eps, uint32_t cap, uint32_t *n_eps) {
  if (!c || !n_eps) return WV_ERR_ARG;
  const std::vector<uint32_t> &v = built ? c->fg_eps : c->eps;
  *n_eps = (uint32_t)v.size();
  if (eps) std::copy(v.begin(), v.begin() + std::min<size_t>(cap, v.size()), eps);
  return WV_OK;
}

int wv_draw_seeds(wv_ctx *c, uint32_t nq, int entry, uint32_t L, uint32_t *seeds) {
  if (!c || !seeds) return WV_ERR_ARG;
  WV_CHECK(c, c->n > 0 && L < c->n, WV_ERR_ARG, "L=%u must be smaller than n=%u", L, c->n);
  return draw(c, nq, entry, L, seeds, L);
}

int wv_draw_seeds_device(wv_ctx *c, uint32_t nq, uint32_t L, uint32_t *d_seeds, uint32_t stride) {
  if (!c || !d_seeds) return WV_ERR_ARG;
  WV_CHECK(c, c->n > 0 && L < c->n, WV_ERR_ARG, "L=%u must be smaller than n=%u", L, c->n);
  WV_CHECK(c, stride >= L, WV_ERR_ARG, "stride %u < L=%u", stride, L);
  if (nq == 0) return WV_OK;
  WV_CUDA(c, cudaSetDevice(c->device));
  return draw_seeds_rand_device(c, nq, nullptr, L, L, d_seeds, stride);
}

int wv_search(wv_ctx *c, const float *queries, uint32_t nq, int entry, uint32_t L, uint32_t K,
              const uint32_t *seeds, uint32_t *out_ids, float *out_dist, wv_counters *counters) {
  if (!c) return WV_ERR_ARG;
  WV_CHECK(c, queries && out_ids, WV_ERR_ARG, "null buffer");
  int rc = check_search_args(c, nq, L, K);
  if (rc) return rc;
  if (counters) *counters = wv_counters{0, 0};
  if (nq == 0) return WV_OK;
  WV_CUDA(c, cudaSetDevice(c->device));
  WV_CUDA(c, c->q_buf.ensure((size_t)nq * c->d * 4));
  WV_CUDA(c, c->seed_buf.ensure((size_t)nq * L * 4));
  WV_CUDA(c, c->out_ids_buf.ensure((size_t)nq * K * 4));
  if (out_dist) WV_CUDA(c, c->out_dist_buf.ensure((size_t)nq * K * 4));
  WV_CUDA(c, cudaMemcpyAsync(c->q_buf.p, queries, (size_t)nq * c->d * 4, cudaMemcpyHostToDevice, c->stream));
  std::vector<uint32_t> hs;
  if (entry == WV_ENTRY_SEEDS) {
    WV_CHECK(c, seeds != nullptr, WV_ERR_ARG, "WV_ENTRY_SEEDS needs seeds");
    for (size_t i = 0; i < (size_t)nq * L; i++) WV_CHECK(c, seeds[i] < c->n, WV_ERR_ARG, "seed id %u >= n", seeds[i]);
  } else if (entry == WV_ENTRY_RAND || entry == WV_ENTRY_SUB_CENTROID) {
    // one rand() per query on the host, the mt19937 draws on the device
    if (entry == WV_ENTRY_SUB_CENTROID) {
      rc = check_roots(c, L);
      if (rc) return rc;
    }
    rc = draw_seeds_rand_device(c, nq, nullptr, L, L, c->seed_buf.as<uint32_t>(), L);
    if (rc) return rc;
    if (entry == WV_ENTRY_SUB_CENTROID) {
      rc = put_roots_device(c, nq, nullptr, c->seed_buf.as<uint32_t>(), L);
      if (rc) return rc;
    }
  } else if (entry == WV_ENTRY_KDT) {
    hs.resize((size_t)nq * L);
    rc = draw_seeds_kdt(c, queries, nq, L, hs.data(), L);
    if (rc) return rc;
    seeds = hs.data();
  } else {
    hs.resize((size_t)nq * L);
    rc = draw(c, nq, entry, L, hs.data(), L);
    if (rc) return rc;
    seeds = hs.data();
  }
  if (seeds)
    WV_CUDA(c, cudaMemcpyAsync(c->seed_buf.p, seeds, (size_t)nq * L * 4, cudaMemcpyHostToDevice, c->stream));
  rc = run_search_device(c, c->q_buf.as<float>(), nq, c->seed_buf.as<uint32_t>(), L, nullptr, nullptr, L, K, L,
                         c->out_ids_buf.as<uint32_t>(), out_dist ? c->out_dist_buf.as<float>() : nullptr, K, counters,
                         entry == WV_ENTRY_SUB_CENTROID);
  if (rc) return rc;
  WV_CUDA(c, cudaMemcpyAsync(out_ids, c->out_ids_buf.p, (size_t)nq * K * 4, cudaMemcpyDeviceToHost, c->stream));
  if (out_dist)
    WV_CUDA(c, cudaMemcpyAsync(out_dist, c->out_dist_buf.p, (size_t)nq * K * 4, cudaMemcpyDeviceToHost, c->stream));
  WV_CUDA(c, cudaStreamSynchronize(c->stream));
  return WV_OK;
}

int wv_search_batch(wv_ctx *c, const float *queries, uint32_t nq, int entry, const uint32_t *L, const uint32_t *K,
                    uint32_t out_stride, uint32_t *out_ids, float *out_dist, wv_counters *counters) {
  if (!c) return WV_ERR_ARG;
  WV_CHECK(c, queries && L && K && out_ids, WV_ERR_ARG, "null buffer");
  WV_CHECK(c, entry == WV_ENTRY_RAND || entry == WV_ENTRY_CENTROID || entry == WV_ENTRY_SUB_CENTROID, WV_ERR_ARG,
           "batch search draws its seeds");
  if (counters) *counters = wv_counters{0, 0};
  if (nq == 0) return WV_OK;
  uint32_t Lmax = 0;
  for (uint32_t q = 0; q < nq; q++) {
    int rc = check_search_args(c, nq, L[q], K[q]);
    if (rc) return rc;
    WV_CHECK(c, K[q] <= out_stride, WV_ERR_ARG, "K[%u]=%u > out_stride", q, K[q]);
    if (entry == WV_ENTRY_SUB_CENTROID) {
      rc = check_roots(c, L[q]);
      if (rc) return rc;
    }
    Lmax = std::max(Lmax, L[q]);
  }
  WV_CUDA(c, cudaSetDevice(c->device));
  WV_CUDA(c, c->q_buf.ensure((size_t)nq * c->d * 4));
  WV_CUDA(c, c->seed_buf.ensure((size_t)nq * Lmax * 4));
  WV_CUDA(c, c->out_ids_buf.ensure((size_t)nq * out_stride * 4));
  WV_CUDA(c, c->lq_buf.ensure((size_t)nq * 4));
  WV_CUDA(c, c->kq_buf.ensure((size_t)nq * 4));
  if (out_dist) WV_CUDA(c, c->out_dist_buf.ensure((size_t)nq * out_stride * 4));
  WV_CUDA(c, cudaMemcpyAsync(c->q_buf.p, queries, (size_t)nq * c->d * 4, cudaMemcpyHostToDevice, c->stream));
  WV_CUDA(c, cudaMemcpyAsync(c->lq_buf.p, L, (size_t)nq * 4, cudaMemcpyHostToDevice, c->stream));
  WV_CUDA(c, cudaMemcpyAsync(c->kq_buf.p, K, (size_t)nq * 4, cudaMemcpyHostToDevice, c->stream));
  // seeds drawn query by query with each query's own L, as the reference's
  // loop would draw them (Rand: one rand() per query, the rest on the device)
  std::vector<uint32_t> hs;
  if (entry == WV_ENTRY_RAND || entry == WV_ENTRY_SUB_CENTROID) {
    int rc = draw_seeds_rand_device(c, nq, c->lq_buf.as<uint32_t>(), 0, Lmax, c->seed_buf.as<uint32_t>(), Lmax);
    if (rc) return rc;
    if (entry == WV_ENTRY_SUB_CENTROID) {
      rc = put_roots_device(c, nq, nullptr, c->seed_buf.as<uint32_t>(), Lmax);
      if (rc) return rc;
    }
  } else {
    hs.resize((size_t)nq * Lmax);
    for (uint32_t q = 0; q < nq; q++) {
      int rc = draw(c, 1, entry, L[q], hs.data() + (size_t)q * Lmax, Lmax);
      if (rc) return rc;
    }
    WV_CUDA(c, cudaMemcpyAsync(c->seed_buf.p, hs.data(), hs.size() * 4, cudaMemcpyHostToDevice, c->stream));
  }
  int rc = run_search_device(c, c->q_buf.as<float>(), nq, c->seed_buf.as<uint32_t>(), Lmax, c->lq_buf.as<uint32_t>(),
                      c->kq_buf.as<uint32_t>(), 0, 0, Lmax, c->out_ids_buf.as<uint32_t>(),
                      out_dist ? c->out_dist_buf.as<float>() : nullptr, out_stride, counters,
                      entry == WV_ENTRY_SUB_CENTROID);
  if (rc) return rc;
  WV_CUDA(c, cudaMemcpyAsync(out_ids, c->out_ids_buf.p, (size_t)nq * out_stride * 4, cudaMemcpyDeviceToHost,
                             c->stream));
  if (out_dist)
    WV_CUDA(c, cudaMemcpyAsync(out_dist, c->out_dist_buf.p, (size_t)nq * out_stride * 4, cudaMemcpyDeviceToHost,
                               c->stream));
  WV_CUDA(c, cudaStreamSynchronize(c->stream));
  return WV_OK;
}

int wv_search_device(wv_ctx *c, const float *d_queries, uint32_t nq, uint32_t L, uint32_t K, const uint32_t *d_seeds,
                     uint32_t *d_out_ids, float *d_out_dist, wv_counters *counters) {
  if (!c) return WV_ERR_ARG;
  WV_CHECK(c, d_queries && d_seeds && d_out_ids, WV_ERR_ARG, "null buffer");
  int rc = check_search_args(c, nq, L, K);
  if (rc) return rc;
  if (counters) *counters = wv_counters{0, 0};
  if (nq == 0) return WV_OK;
  WV_CUDA(c, cudaSetDevice(c->device));
  return run_search_device(c, d_queries, nq, d_seeds, L, nullptr, nullptr, L, K, L, d_out_ids, d_out_dist, K, counters);
}

}  // extern "C"
