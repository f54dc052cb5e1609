// Batched search plans: one batch of queries with uneven beam widths L and
// result sizes K served by one persistent launch, bound to caller-owned
// device buffers, its launch shape picked by measurement, and the whole step
// (seed draws or the learned model's forward pass, the counter reset and the
// search) captured once as a CUDA graph that each batch replays.
//
// No counterpart in the reference, whose IndexBuilder::search loops over
// queries one at a time (src/builder.cpp:445-454); the plan is the batched
// form of that loop.  Seeds follow SearchEntryRand exactly: each replay draws
// one rand() per query from the context's stream, in query order, into
// pinned memory the graph copies from.
//
// Tuning (wv_plan_tune): the search kernel alone is timed with CUDA events on
// the current inputs for every shape that fits -- warps per block 1, 2, 4, 8
// and the default or a doubled visited hash -- and the fastest is captured.
// Results do not depend on the shape (each warp runs the same exact search
// for whichever query it takes).
//
// A plan owns everything its graph points at that the context could
// reallocate (visited scratch, seed and model work buffers under its own
// names); the base, graph, precision and model are the context's, so a plan
// refuses to run once any of them changed (the context's generation).
#include <algorithm>
#include <cstdio>
#include <string>
#include <vector>

#include "wv_ctx.h"
#include "wv_learn.h"
#include "wv_seeds.h"

using namespace wv;

struct wv_plan {
  wv_ctx *c = nullptr;
  wv_plan_params p{};
  unsigned long long gen = 0;  // context generation the plan was made for
  std::string pfx;             // names of its learned work buffers
  const float *d_q = nullptr;
  const uint32_t *d_L = nullptr, *d_K = nullptr, *d_seeds_in = nullptr;
  uint32_t *d_out = nullptr;
  float *d_dist = nullptr;
  DevBuf seeds, sv, nqd, vis, touch;  // plan-owned device buffers
  size_t vis_slots = 0, words = 0;
  uint32_t *h_sv = nullptr;  // pinned: rand() values of the replay
  uint32_t *h_nq = nullptr;  // pinned: query count of the replay
  uint32_t plain_L = 0;      // learned mode: plain seeds per query (0: none)
  uint32_t Lcap = 0;         // the beam the kernel is sized for
  uint32_t lstride = 0;      // learned mode: seed row stride
  SearchShape shape{};
  int blocks = 0;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaEvent_t done = nullptr;
  cudaEvent_t s0 = nullptr, s1 = nullptr;  // around the search kernel (recorded inside the graph)
  bool pending = false;
};

namespace {

bool draws_seeds(const wv_plan *p) {
  return p->p.mode == WV_PLAN_RAND || (p->p.mode == WV_PLAN_LEARNED && p->plain_L);
}

// visited scratch for `slots` warps (all-zero bitsets)
int ensure_scratch(wv_plan *p, size_t slots) {
  wv_ctx *c = p->c;
  if (slots <= p->vis_slots) return WV_OK;
  p->vis.release();
  p->touch.release();
  p->vis_slots = 0;
  WV_CUDA(c, p->vis.ensure(slots * p->words * 4));
  WV_CUDA(c, p->touch.ensure(slots * p->words * 4));
  WV_CUDA(c, cudaMemsetAsync(p->vis.p, 0, slots * p->words * 4, c->stream));
  p->vis_slots = slots;
  return WV_OK;
}

SearchScratch scratch(const wv_plan *p) {
  SearchScratch s;
  s.visited = p->vis.as<uint32_t>();
  s.touched = p->touch.as<uint32_t>();
  s.words = (uint32_t)p->words;
  return s;
}

// the search arguments of the staged batch (seeds and beams from the plan)
SearchArgs plan_args(wv_plan *p, uint32_t nq, const uint32_t *nq_dev, int *rc) {
  wv_ctx *c = p->c;
  SearchArgs a;
  *rc = WV_OK;
  if (p->p.mode == WV_PLAN_LEARNED) {
    cudaError_t e = cudaSuccess;
    uint32_t *seeds = c->buf<uint32_t>((p->pfx + "seeds").c_str(), (size_t)p->p.nq_max * p->lstride, &e);
    uint32_t *Lq = c->buf<uint32_t>((p->pfx + "Lq").c_str(), p->p.nq_max, &e);
    if (e != cudaSuccess) *rc = fail(c, WV_ERR_NOMEM, "plan work buffers");
    a = search_args(c, p->d_q, nq, nq_dev, seeds, p->lstride, Lq, p->d_K, 0, p->p.K_max, p->Lcap, p->d_out,
                    p->d_dist, p->p.out_stride);
  } else {
    const uint32_t *seeds = p->p.mode == WV_PLAN_RAND ? p->seeds.as<uint32_t>() : p->d_seeds_in;
    a = search_args(c, p->d_q, nq, nq_dev, seeds, p->p.L_max, p->d_L, p->d_K, p->p.L_max, p->p.K_max, p->p.L_max,
                    p->d_out, p->d_dist, p->p.out_stride);
  }
  if (a.Lq) {
    cudaError_t e = cudaSuccess;
    a.order = c->buf<uint32_t>((p->pfx + "order").c_str(), p->p.nq_max, &e);
    if (e != cudaSuccess) *rc = fail(c, WV_ERR_NOMEM, "plan work buffers");
  }
  const SearchScratch s = scratch(p);
  a.visited = s.visited;
  a.touched = s.touched;
  a.words = s.words;
  return a;
}

// the work of one replay, issued on the context stream
int enqueue(wv_plan *p) {
  wv_ctx *c = p->c;
  const uint32_t nqm = p->p.nq_max;
  WV_CUDA(c, cudaMemcpyAsync(p->nqd.p, p->h_nq, 4, cudaMemcpyHostToDevice, c->stream));
  const uint32_t *nq_dev = p->nqd.as<uint32_t>();
  if (draws_seeds(p)) {
    const bool rand_mode = p->p.mode == WV_PLAN_RAND;
    const uint32_t Ls = rand_mode ? p->p.L_max : p->plain_L;
    WV_CUDA(c, cudaMemcpyAsync(p->sv.p, p->h_sv, (size_t)nqm * 4, cudaMemcpyHostToDevice, c->stream));
    WV_CUDA(c, seeds_rand_launch(p->sv.as<uint32_t>(), nqm, nq_dev, rand_mode ? p->d_L : nullptr, Ls, Ls, c->n,
                                 p->seeds.as<uint32_t>(), Ls, c->d_status(), c->stream));
  }
  if (p->p.mode == WV_PLAN_LEARNED)
    return learn_enqueue(c, p->pfx.c_str(), p->d_q, nqm, nq_dev, p->p.K_max, p->d_K, p->d_out, p->d_dist,
                         p->p.out_stride, p->plain_L ? p->seeds.as<uint32_t>() : nullptr, p->shape, p->blocks,
                         scratch(p), p->s0, p->s1);
  int rc = WV_OK;
  const SearchArgs a = plan_args(p, nqm, nq_dev, &rc);
  if (rc) return rc;
  WV_CUDA(c, record_event(p->s0, c->stream));
  rc = search_enqueue(c, a, p->shape, p->blocks);
  if (rc) return rc;
  WV_CUDA(c, record_event(p->s1, c->stream));
  return WV_OK;
}

// sizes, grid and scratch for the current shape
int prepare(wv_plan *p) {
  wv_ctx *c = p->c;
  if (p->p.mode == WV_PLAN_LEARNED) {
    int rc = learn_prepare(c, p->pfx.c_str(), p->p.nq_max, &p->Lcap, &p->lstride);
    if (rc) return rc;
  } else {
    p->Lcap = p->p.L_max;
  }
  const int grid = route_grid(c, p->Lcap, p->shape);
  WV_CHECK(c, grid > 0, WV_ERR_LIMIT, "search kernel cannot run with d=%u L=%u width=%u", c->d, p->Lcap, c->gw);
  p->blocks = std::min<int>(grid, (int)((p->p.nq_max + p->shape.wpb - 1) / p->shape.wpb));
  return ensure_scratch(p, (size_t)p->blocks * p->shape.wpb);
}

void drop_graph(wv_plan *p) {
  if (p->exec) cudaGraphExecDestroy(p->exec);
  if (p->graph) cudaGraphDestroy(p->graph);
  p->exec = nullptr;
  p->graph = nullptr;
}

int capture(wv_plan *p) {
  wv_ctx *c = p->c;
  drop_graph(p);
  int rc = prepare(p);
  if (rc) return rc;
  // one uncaptured pass first: first-use allocations and attributes happen
  // outside the capture (with zero queries nothing is searched)
  *p->h_nq = 0;
  rc = enqueue(p);
  if (rc) return rc;
  WV_CUDA(c, cudaStreamSynchronize(c->stream));
  WV_CUDA(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
  rc = enqueue(p);
  cudaGraph_t g = nullptr;
  const cudaError_t ce = cudaStreamEndCapture(c->stream, &g);
  if (rc) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  WV_CUDA(c, ce);
  p->graph = g;
  WV_CUDA(c, cudaGraphInstantiate(&p->exec, p->graph, 0));
  return WV_OK;
}

int wait_pending(wv_plan *p) {
  if (p->pending) {
    p->pending = false;
    WV_CUDA(p->c, cudaEventSynchronize(p->done));
  }
  return WV_OK;
}

int check_usable(wv_plan *p) {
  WV_CHECK(p->c, p->exec, WV_ERR_STATE, "the plan has no captured graph");
  WV_CHECK(p->c, p->gen == p->c->generation, WV_ERR_STATE,
           "the base, graph, precision or model changed since the plan was made: create it again");
  return WV_OK;
}

// host side of a replay: the query count and the rand() values
int stage(wv_plan *p, uint32_t nq) {
  int rc = wait_pending(p);
  if (rc) return rc;
  *p->h_nq = nq;
  if (draws_seeds(p))
    for (uint32_t q = 0; q < nq; q++) p->h_sv[q] = (uint32_t)p->c->rnd.next();
  return WV_OK;
}

// times the search of the staged batch with one shape (best of 3)
int time_shape(wv_plan *p, uint32_t nq, SearchShape sh, cudaEvent_t e0, cudaEvent_t e1, float *ms, int *blocks) {
  wv_ctx *c = p->c;
  const int grid = route_grid(c, p->Lcap, sh);
  if (grid <= 0) return WV_ERR_LIMIT;
  *blocks = std::min<int>(grid, (int)((nq + sh.wpb - 1) / sh.wpb));
  int rc = ensure_scratch(p, (size_t)*blocks * sh.wpb);
  if (rc) return rc;
  const SearchArgs a = plan_args(p, nq, nullptr, &rc);
  if (rc) return rc;
  *ms = 3.4e38f;
  for (int it = 0; it < 3; it++) {
    WV_CUDA(c, cudaEventRecord(e0, c->stream));
    rc = search_enqueue(c, a, sh, *blocks);
    if (rc) return rc;
    WV_CUDA(c, cudaEventRecord(e1, c->stream));
    WV_CUDA(c, cudaEventSynchronize(e1));
    float t = 0.f;
    WV_CUDA(c, cudaEventElapsedTime(&t, e0, e1));
    *ms = std::min(*ms, t);
  }
  return check_device_status(c, "plan tuning");
}

}  // namespace

extern "C" {

int wv_plan_create(wv_ctx *c, const wv_plan_params *prm, const float *d_queries, const uint32_t *d_L,
                   const uint32_t *d_K, const uint32_t *d_seeds, uint32_t *d_out_ids, float *d_out_dist,
                   wv_plan **out) {
  if (!c || !prm || !out || !d_queries || !d_out_ids) return WV_ERR_ARG;
  *out = nullptr;
  const wv_plan_params &q = *prm;
  WV_CHECK(c, c->n > 0 && c->gn == c->n, WV_ERR_STATE, "a plan needs the base and its search graph");
  WV_CHECK(c, c->d % 4 == 0, WV_ERR_LIMIT, "dimension %u is not a multiple of 4", c->d);
  WV_CHECK(c, q.nq_max > 0 && q.K_max >= 1 && q.out_stride >= q.K_max, WV_ERR_ARG,
           "bad plan sizes (nq_max > 0, K_max >= 1, out_stride >= K_max)");
  WV_CHECK(c, q.mode == WV_PLAN_RAND || q.mode == WV_PLAN_SEEDS || q.mode == WV_PLAN_LEARNED, WV_ERR_ARG,
           "unknown plan mode %d", q.mode);
  if (q.mode == WV_PLAN_LEARNED) {
    WV_CHECK(c, c->learn, WV_ERR_STATE, "learned plan without a trained model (call wv_learn_fit)");
    WV_CHECK(c, d_L == nullptr, WV_ERR_ARG, "the learned plan picks each query's L itself (d_L must be null)");
  } else {
    WV_CHECK(c, q.L_max >= q.K_max && q.L_max < c->n && q.L_max <= SEARCH_MAX_L, WV_ERR_ARG,
             "L_max=%u must lie in [K_max, min(n - 1, %u)]", q.L_max, SEARCH_MAX_L);
  }
  WV_CHECK(c, q.mode != WV_PLAN_SEEDS || d_seeds, WV_ERR_ARG, "WV_PLAN_SEEDS needs d_seeds (nq_max x L_max)");
  WV_CUDA(c, cudaSetDevice(c->device));
  wv_plan *p = new wv_plan;
  p->c = c;
  p->p = q;
  p->gen = c->generation;
  char tag[48];
  snprintf(tag, sizeof(tag), "plan%p_", (void *)p);
  p->pfx = tag;
  p->d_q = d_queries;
  p->d_L = d_L;
  p->d_K = d_K;
  p->d_seeds_in = d_seeds;
  p->d_out = d_out_ids;
  p->d_dist = d_out_dist;
  p->words = (c->n + 31) / 32;
  if (q.mode == WV_PLAN_LEARNED) p->plain_L = learn_plain_beam(c);
  const uint32_t seed_L = q.mode == WV_PLAN_RAND ? q.L_max : p->plain_L;
  if (cudaMallocHost(&p->h_nq, 4) != cudaSuccess || cudaMallocHost(&p->h_sv, (size_t)q.nq_max * 4) != cudaSuccess ||
      p->nqd.ensure(16) != cudaSuccess || p->sv.ensure((size_t)q.nq_max * 4) != cudaSuccess ||
      (seed_L && p->seeds.ensure((size_t)q.nq_max * seed_L * 4) != cudaSuccess) ||
      cudaEventCreateWithFlags(&p->done, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreate(&p->s0) != cudaSuccess || cudaEventCreate(&p->s1) != cudaSuccess) {
    wv_plan_destroy(p);
    return fail(c, WV_ERR_NOMEM, "plan buffers");
  }
  const int rc = capture(p);
  if (rc) {
    const std::string msg = c->err;
    wv_plan_destroy(p);
    c->err = msg;
    return rc;
  }
  *out = p;
  return WV_OK;
}

int wv_plan_run(wv_plan *p, uint32_t nq) {
  if (!p) return WV_ERR_ARG;
  wv_ctx *c = p->c;
  int rc = check_usable(p);
  if (rc) return rc;
  WV_CHECK(c, nq <= p->p.nq_max, WV_ERR_ARG, "nq=%u above the plan's nq_max=%u", nq, p->p.nq_max);
  rc = stage(p, nq);
  if (rc) return rc;
  WV_CUDA(c, cudaGraphLaunch(p->exec, c->stream));
  WV_CUDA(c, cudaEventRecord(p->done, c->stream));
  p->pending = true;
  return WV_OK;
}

int wv_plan_wait(wv_plan *p, wv_counters *counters) {
  if (!p) return WV_ERR_ARG;
  wv_ctx *c = p->c;
  int rc = wait_pending(p);
  if (rc) return rc;
  if (counters) {
    unsigned long long h[2];
    WV_CUDA(c, cudaMemcpyAsync(h, c->d_counters(), 16, cudaMemcpyDeviceToHost, c->stream));
    WV_CUDA(c, cudaStreamSynchronize(c->stream));
    counters->dist_count = h[0];
    counters->hop_count = h[1];
  }
  return check_device_status(c, "plan");
}

int wv_plan_tune(wv_plan *p, uint32_t nq, wv_tune_report *rep) {
  if (!p) return WV_ERR_ARG;
  wv_ctx *c = p->c;
  int rc = check_usable(p);
  if (rc) return rc;
  WV_CHECK(c, nq >= 1 && nq <= p->p.nq_max, WV_ERR_ARG, "tune needs 1 <= nq <= nq_max");
  // one replay makes the seeds (and the learned beams) of these inputs
  rc = wv_plan_run(p, nq);
  if (rc) return rc;
  rc = wv_plan_wait(p, nullptr);
  if (rc) return rc;
  // areas: the least the beam allows, the default, twice the default
  const uint32_t h0 = search_hash_slots(p->Lcap, 0), hmin = search_hash_min(p->Lcap, c->n);
  std::vector<uint32_t> areas;
  if (hmin < h0) areas.push_back(hmin);
  if (hmin < h0 / 2) areas.push_back(h0 / 2);
  areas.push_back(0u);
  areas.push_back(2 * h0);
  std::vector<SearchShape> cand;
  for (int w : {1, 2, 4, 8})
    for (uint32_t h : areas) cand.push_back(SearchShape{w, h});
  // the throughput form also tries 32-bit visited-hash entries (half the
  // slots in the same bytes, but a native compare-and-swap per probe) and
  // 2 or 4 warps per query (the query's shared memory serving more rows in
  // flight)
  if (c->parents > 0) {
    for (int w : {1, 2, 4, 8})
      for (uint32_t h : {0u, 2 * h0}) cand.push_back(SearchShape{w, h, true});
    for (int qw : {2, 4}) {  // one query per block
      SearchShape sh{qw, 0u};
      sh.qw = qw;
      cand.push_back(sh);
      SearchShape sh2{qw, 2 * h0};
      sh2.qw = qw;
      cand.push_back(sh2);
    }
  }
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  WV_CUDA(c, cudaEventCreate(&e0));
  WV_CUDA(c, cudaEventCreate(&e1));
  wv_tune_report r{};
  r.chosen = -1;
  float best = 3.4e38f;
  SearchShape chosen = p->shape;
  for (const SearchShape &sh : cand) {
    float ms = 0.f;
    int blocks = 0;
    const int trc = time_shape(p, nq, sh, e0, e1, &ms, &blocks);
    if (trc == WV_ERR_LIMIT) {  // the shape does not fit: skip it
      c->err.clear();
      continue;
    }
    if (trc) {
      rc = trc;
      break;
    }
    if (r.n < WV_TUNE_MAX) {
      r.tried[r.n] = wv_plan_shape{sh.wpb, search_hash_slots(p->Lcap, sh.hcap), sh.wide ? 1 : 0, blocks, ms, sh.qw};
      if (ms < best) {
        best = ms;
        chosen = sh;
        r.chosen = r.n;
      }
      r.n++;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  // always recapture: the trials may have moved the scratch the old graph used
  if (rc == WV_OK) p->shape = chosen;
  const std::string msg = c->err;
  const int crc = capture(p);
  if (rc) {
    c->err = msg;
    return rc;
  }
  if (crc) return crc;
  if (rep) *rep = r;
  return WV_OK;
}

int wv_plan_search_ms(wv_plan *p, float *ms) {
  if (!p || !ms) return WV_ERR_ARG;
  int rc = wait_pending(p);
  if (rc) return rc;
  WV_CUDA(p->c, cudaEventElapsedTime(ms, p->s0, p->s1));
  return WV_OK;
}

int wv_plan_shape_of(wv_plan *p, wv_plan_shape *out) {
  if (!p || !out) return WV_ERR_ARG;
  *out = wv_plan_shape{p->shape.wpb, search_hash_slots(p->Lcap, p->shape.hcap), p->shape.wide ? 1 : 0, p->blocks,
                       0.f, p->shape.qw};
  return WV_OK;
}

int wv_plan_set_shape(wv_plan *p, const wv_plan_shape *sh) {
  if (!p || !sh) return WV_ERR_ARG;
  wv_ctx *c = p->c;
  int rc = check_usable(p);
  if (rc) return rc;
  WV_CHECK(c, sh->warps_per_block == 1 || sh->warps_per_block == 2 || sh->warps_per_block == 4 ||
                  sh->warps_per_block == 8,
           WV_ERR_ARG, "warps_per_block must be 1, 2, 4 or 8");
  WV_CHECK(c, sh->hash_words == 0 || (sh->hash_words & (sh->hash_words - 1)) == 0, WV_ERR_ARG,
           "hash_words must be 0 or a power of two");
  WV_CHECK(c, sh->query_warps <= 1 || (c->parents > 0 && (sh->query_warps == 2 || sh->query_warps == 4) &&
                                       sh->warps_per_block == sh->query_warps),
           WV_ERR_ARG, "query_warps %d: 1, or 2 / 4 equal to warps_per_block with the throughput form",
           sh->query_warps);
  WV_CHECK(c, sh->hash_words == 0 || sh->hash_words >= search_hash_min(p->Lcap, c->n), WV_ERR_ARG,
           "hash_words=%u below the least area %u for L=%u, n=%u", sh->hash_words, search_hash_min(p->Lcap, c->n),
           p->Lcap, c->n);
  rc = wait_pending(p);
  if (rc) return rc;
  const SearchShape old = p->shape;
  p->shape = SearchShape{sh->warps_per_block, sh->hash_words, sh->wide_hash != 0};
  p->shape.qw = sh->query_warps > 0 ? sh->query_warps : 1;
  rc = capture(p);
  if (rc) {
    const std::string msg = c->err;
    p->shape = old;
    capture(p);
    c->err = msg;
  }
  return rc;
}

int wv_plan_destroy(wv_plan *p) {
  if (!p) return WV_OK;
  if (p->pending && p->done) cudaEventSynchronize(p->done);
  drop_graph(p);
  if (p->done) cudaEventDestroy(p->done);
  if (p->s0) cudaEventDestroy(p->s0);
  if (p->s1) cudaEventDestroy(p->s1);
  if (p->h_nq) cudaFreeHost(p->h_nq);
  if (p->h_sv) cudaFreeHost(p->h_sv);
  p->seeds.release();
  p->sv.release();
  p->nqd.release();
  p->vis.release();
  p->touch.release();
  if (p->c && !p->pfx.empty()) {
    for (auto it = p->c->work.begin(); it != p->c->work.end();) {
      if (it->first.compare(0, p->pfx.size(), p->pfx) == 0) {
        it->second.release();
        it = p->c->work.erase(it);
      } else {
        ++it;
      }
    }
  }
  delete p;
  return WV_OK;
}

}  // extern "C"
