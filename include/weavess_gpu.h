/* weavess_gpu.h -- C ABI of the GB300 implementation of the WEAVESS hot path.
 *
 * The reference exposes this path as per-item C++ virtuals called from
 * OpenMP loops inside IndexBuilder (include/weavess/component.h).  A GPU
 * wants whole batches, so each entry point below replaces one of those
 * components for ALL items at once, reading and writing the reference's own
 * layouts (row-major float base, per-node adjacency rows with distances).
 *
 * Conventions: every call returns a wv_status; wv_last_error() describes the
 * last failure.  No exception crosses the ABI.  Host buffers are owned by the
 * caller.  A context owns one GPU's device memory and stream; calls on one
 * context must not overlap (one context per thread).  Random draws come from
 * a per-context stream that reproduces glibc rand() (seeded 1 like a fresh
 * process), or from a caller-supplied rand function (wv_set_rand_source),
 * consumed in the same order as the reference consumes rand().
 */
#ifndef WEAVESS_GPU_H
#define WEAVESS_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  WV_OK = 0,
  WV_ERR_ARG = 1,      /* invalid argument (sizes, NULL, L < K ...) */
  WV_ERR_CUDA = 2,     /* a CUDA call failed */
  WV_ERR_STATE = 3,    /* missing base/graph, or no device */
  WV_ERR_NOMEM = 4,    /* device allocation failed */
  WV_ERR_LIMIT = 5,    /* a size beyond what this build supports */
  WV_ERR_DEVICE = 6    /* a kernel reported corrupt input or a bounded wait ran out */
} wv_status;

typedef enum {
  WV_ENTRY_RAND = 0,     /* ComponentSearchEntryRand (component_search_entry.cpp:9-30) */
  WV_ENTRY_CENTROID = 1, /* ComponentSearchEntryCentroid (component_search_entry.cpp:33-67) */
  WV_ENTRY_SEEDS = 2,    /* caller-supplied seed ids (nq x L) */
  /* ComponentSearchEntrySubCentroid (component_search_entry.cpp:70-99), the
   * SSG search entry: the Rand draw with its first ids replaced by the
   * search graph's SSG roots, seed distances taken -- as the reference
   * takes them -- to each row shifted by one float (a zero follows the last
   * row) */
  WV_ENTRY_SUB_CENTROID = 3,
  /* ComponentSearchEntryKDT (component_search_entry.cpp:102-170), the EFANNA
   * search entry: the ids of L / (nTrees * 10) + 1 leaves per tree of the
   * last wv_init_kdt, found depth first on the query's side of each cut,
   * then rand() % n fills; the base id equal to the query's number in the
   * batch is skipped, as the reference flags it.  wv_search only (the
   * leaves are walked on the device; the rand() fills follow on the host in
   * query order). */
  WV_ENTRY_KDT = 4
} wv_entry;

typedef struct wv_ctx wv_ctx;

typedef struct {
  unsigned long long dist_count; /* Index::addDistCount calls (entry + route) */
  unsigned long long hop_count;  /* Index::addHopCount calls (expansions) */
} wv_counters;

/* ---- context ---------------------------------------------------------- */
int wv_ctx_create(wv_ctx **ctx, int device);
int wv_ctx_destroy(wv_ctx *ctx);
const char *wv_last_error(const wv_ctx *ctx);
/* glibc-compatible rand() stream of the context (srand semantics) */
int wv_srand(wv_ctx *ctx, unsigned seed);
/* draw from `fn` instead (e.g. the process's own rand, to share its stream
 * with the rest of a reference process); NULL restores the context stream */
int wv_set_rand_source(wv_ctx *ctx, int (*fn)(void));
/* next value of the context's rand stream (for callers that interleave) */
int wv_rand(wv_ctx *ctx, int *out);
/* run the context's work on `stream` (a cudaStream_t of the same device);
 * NULL restores the context's own stream */
int wv_set_stream(wv_ctx *ctx, void *stream);

/* ---- data --------------------------------------------------------------- */
/* Replaces the base arrays ComponentLoad::LoadInner hands to the index
 * (component_load.cpp:67-104): n x d float32, row-major. */
int wv_upload_base(wv_ctx *ctx, const float *base, uint32_t n, uint32_t d);
/* Replaces IndexBuilder::load_graph (builder.cpp:1083-1311): the search graph
 * (load_graph_) as fixed-width rows, ids[n*width], deg[n], entry point ep_. */
int wv_upload_graph(wv_ctx *ctx, const uint32_t *ids, const uint32_t *deg, uint32_t n, uint32_t width,
                    uint32_t ep);
/* The SSG roots eps_ of the search graph (load_graph of INDEX_SSG,
 * builder.cpp:1091-1095); uploading a graph clears them. */
int wv_set_eps(wv_ctx *ctx, const uint32_t *eps, uint32_t n_eps);
/* Reads the roots of the built graph (built != 0) or of the search graph:
 * *n_eps = their count, the first min(cap, count) copied to eps (nullable). */
int wv_get_eps(wv_ctx *ctx, int built, uint32_t *eps, uint32_t cap, uint32_t *n_eps);

/* ---- build ------------------------------------------------------------- */
typedef struct {
  unsigned long long rand_draws; /* values taken from the rand stream */
  unsigned long long offers;     /* join offers that reached the per-node merge */
  unsigned long long pairs;      /* local-join distance evaluations */
  unsigned chunks;               /* join chunks over all iterations */
  float ms_join, ms_update, ms_total;
  unsigned levels;               /* InterInsert dependency levels (link) */
  unsigned ep;                   /* entry point chosen (link) */
  unsigned conn_added;           /* edges added by the NSG connectivity pass */
} wv_build_stats;

/* The graph the build components hand to each other (final_graph_ of the
 * reference's Index, include/weavess/index.h:1658): fixed-width rows of ids
 * and distances, deg[n] entries each.  Set it from the host, or read back the
 * result of the last build step.  out arrays are n x width (width >= the
 * current row width, see wv_graph_width). */
int wv_set_graph(wv_ctx *ctx, const uint32_t *ids, const float *dist, const uint32_t *deg, uint32_t n,
                 uint32_t width, uint32_t ep);
int wv_graph_width(wv_ctx *ctx, uint32_t *width, uint32_t *ep);
int wv_get_graph(wv_ctx *ctx, uint32_t *ids, float *dist, uint32_t *deg, uint32_t width);
/* IndexBuilder::save_graph + load_graph (builder.cpp:918-1311) without the
 * host round trip: the current build graph becomes the search graph. */
int wv_load_built_graph(wv_ctx *ctx);

/* ComponentInitRandom::InitInner (component_init.cpp:11-45): S random
 * neighbours per node from one mt19937 seeded by one rand() draw, sorted by
 * distance.  Result: the current graph (width S). */
int wv_init_random(wv_ctx *ctx, uint32_t S, wv_build_stats *stats);
/* ComponentInitRand::InitInner (component_init.cpp:979-1025), the init of the
 * reference's Vamana pipeline: L random neighbours per node from one mt19937
 * seeded by one rand() draw (GenRandom, node order; the node itself
 * skipped), each pool make_heap'd then sorted by distance as the reference
 * does.  Result: the current graph (width L, 1 <= L <= 1024). */
int wv_init_rand(wv_ctx *ctx, uint32_t L, wv_build_stats *stats);

/* INIT_KDT: replaces ComponentInitKDT::InitInner (component_init.cpp:500-640).
 * nTrees randomised KD-trees (ids shuffled with rand(), cuts at the mean of
 * one of the 5 highest-variance dimensions of 101 sampled ids, leaves of at
 * most 10 ids), leaves merged below depth mLevel into per-point sets of K
 * nearest candidates; the current graph becomes those rows (K each,
 * ascending; rows short of K filled from mt19937(1998) % n).  The trees are
 * kept for WV_ENTRY_KDT.  Identical to the reference run on one thread.
 * K <= 1024. */
int wv_init_kdt(wv_ctx *ctx, uint32_t nTrees, uint32_t K, uint32_t mLevel, wv_build_stats *stats);

/* ComponentRefineNNDescent::RefineInner (component_refine.cpp:12-239) on the
 * current graph: ITER rounds of join + update with pool size L, sample S,
 * reverse cap R, then sorted rows truncated to K (PruneNaive).  Result: the
 * current graph (width K). */
int wv_nnd_refine(wv_ctx *ctx, uint32_t S, uint32_t K, uint32_t L, uint32_t ITER, uint32_t R,
                  wv_build_stats *stats);

/* ComponentRefineEFANNA::RefineInner (component_refine.cpp:959-1178) on the
 * current graph (the KD-tree graph in the reference's EFANNA pipeline; any
 * graph whose rows hold at most L entries): REFINE_NN_DESCENT's join /
 * update / PruneNaive, with EFANNA's init -- one rand() seeds an mt19937
 * from which every node draws 2S random ids as its first nn_new (GenRandom,
 * node order), and the pools take each row sorted by distance without the
 * node itself or repeated ids -- so the first join does work.  Result: the
 * current graph (width K).  Bit-exact with the reference run on one thread;
 * stats->rand_draws counts the values taken from the rand stream. */
int wv_efanna_refine(wv_ctx *ctx, uint32_t S, uint32_t K, uint32_t L, uint32_t ITER, uint32_t R,
                     wv_build_stats *stats);

/* ComponentRefineVAMANA::RefineInner (component_refine.cpp:794-950) on the
 * current graph: entry point (ComponentRefineEntryCentroid), a greedy
 * candidate search of L_refine per node (ComponentCandidateNSG), the alpha
 * prune to R_refine (ComponentPruneVAMANA) and InterInsert.  entry_L is the
 * index's L_refine member the entry search reads: the Vamana refine never
 * sets it, so in a NN-Descent -> Vamana pipeline it is 0 and the entry point
 * is node 0.  The reference sets alpha = 2 after a link; pass alpha for each
 * call.  Result: the current graph (width R_refine) with its entry point. */
int wv_vamana_refine(wv_ctx *ctx, uint32_t L_refine, uint32_t R_refine, float alpha, uint32_t entry_L,
                     wv_build_stats *stats);
/* Build behaviour.  No counterpart in the reference.  WV_BUILD_COMPAT (the
 * default) reproduces the reference bit for bit, defects included.
 * WV_BUILD_CLEAN fixes the Vamana link's three: the entry point is the
 * centroid search with L_refine (entry_L = 0 reads as L_refine; the
 * reference's entry is node 0, component_refine.cpp:831-833 never sets the
 * L_refine that component_entry.cpp:32 reads); PruneVAMANA sorts short pools
 * too (component_prune.cpp:281-285 copies them unsorted); and the overflow
 * re-prune of InterInsert walks the sorted row closest first, testing each
 * candidate against its own distance (component_refine.cpp:905-907 walks
 * farthest first against temp_pool[i], the outer index). */
typedef enum { WV_BUILD_COMPAT = 0, WV_BUILD_CLEAN = 1 } wv_build_mode;
int wv_set_build_mode(wv_ctx *ctx, int mode);

/* ComponentRefineNSG::RefineInner (component_refine.cpp:393-541) on the
 * current graph: centroid entry point with L_refine, candidate search, the
 * RNG prune (ComponentPruneNSG, C_refine candidates), InterInsert, then
 * ComponentConnNSGDFS.  Result: the current graph (rows may exceed R_refine
 * after the connectivity pass) with its entry point. */
int wv_nsg_refine(wv_ctx *ctx, uint32_t L_refine, uint32_t R_refine, uint32_t C_refine, wv_build_stats *stats);
/* ComponentRefineSSG::RefineInner (component_refine.cpp:550-720): candidates
 * by ComponentCandidatePropagation2 (component_candidate.cpp:90-109, the
 * first L_refine unseen neighbours of neighbours), ComponentPruneSSG's angle
 * rule (component_prune.cpp:71-122, angle A in degrees, rows of at most
 * R_refine), InterInsert with the same rule, then ComponentConnSSGDFS
 * (component_conn.cpp:169-225): n_try roots from std::random_shuffle on the
 * rand stream, every node linked from them.  eps (nullable) receives the
 * n_try roots; the built graph keeps them for save / load.  Bit-exact with
 * the reference run on one thread. */
int wv_ssg_refine(wv_ctx *ctx, uint32_t L_refine, uint32_t R_refine, float A, uint32_t n_try, uint32_t *eps,
                  wv_build_stats *stats);

/* ---- search ------------------------------------------------------------- */
/* Replaces the query loop of IndexBuilder::search with L_SEARCH_ASSIGN
 * (builder.cpp:430-454): SearchEntryInner (entry) + ComponentSearchRouteGreedy
 * ::RouteInner (component_route.cpp:9-53) for every query, K_search = K.
 * queries: nq x d host floats; out_ids: nq x K; out_dist (nullable): nq x K.
 * seeds: nq x L ids when entry == WV_ENTRY_SEEDS, else NULL. */
int wv_search(wv_ctx *ctx, const float *queries, uint32_t nq, int entry, uint32_t L, uint32_t K,
              const uint32_t *seeds, uint32_t *out_ids, float *out_dist, wv_counters *counters);

/* Mixed beam widths in one launch: per-query L[q] and K[q]; results at
 * out_ids[q*out_stride + j], j < K[q]. */
int wv_search_batch(wv_ctx *ctx, const float *queries, uint32_t nq, int entry, const uint32_t *L,
                    const uint32_t *K, uint32_t out_stride, uint32_t *out_ids, float *out_dist,
                    wv_counters *counters);

/* Same as wv_search, with queries / seeds / outputs already in device memory
 * (d_seeds required: the caller drew them, e.g. with wv_draw_seeds). */
int wv_search_device(wv_ctx *ctx, const float *d_queries, uint32_t nq, uint32_t L, uint32_t K,
                     const uint32_t *d_seeds, uint32_t *d_out_ids, float *d_out_dist, wv_counters *counters);

/* Low-precision candidate distances (not in the reference).  Builds a copy of
 * the uploaded base in bf16, or in fp8 e4m3 with one FP32 scale per row
 * (max |x| / 448), and makes every later search compute candidate distances
 * from it (FP32 accumulation), then re-score the first `rerank` entries of
 * each final pool exactly in FP32 (0 = the whole pool) and re-sort them before
 * the top K are returned.  WV_STORE_FP32 restores the plain form. */
typedef enum { WV_STORE_FP32 = 0, WV_STORE_BF16 = 1, WV_STORE_FP8 = 2 } wv_storage;
int wv_set_search_precision(wv_ctx *ctx, int storage, uint32_t rerank);
/* Traversal of the route searches (wv_search*, plans, the learned search).
 * No counterpart in the reference, whose RouteInner
 * (src/component_route.cpp:9-53) expands one pool entry at a time.
 * parents = 0 (the default): the exact traversal, the reference's expansion
 * order, ids and DistCount/HopCount equal to RouteInner's.  parents = E in
 * 1..4: the throughput form -- each step expands the E best unexpanded pool
 * entries together, seeds are marked visited when pooled, and candidate
 * distances of bf16 rows (d = 96, 128) and of FP32 rows of integer data
 * (d = 128) run on the tensor cores; results are a best-first beam search of
 * the same graph but not the reference's traversal order.  Build-time
 * candidate searches and the sub-centroid entry always use the exact form. */
int wv_set_search_expansion(wv_ctx *ctx, uint32_t parents);
/* Candidate distances of the current precision for nq host queries against
 * m base ids each (ids nq x m): out nq x m (to measure the error). */
int wv_candidate_distances(wv_ctx *ctx, const float *queries, uint32_t nq, const uint32_t *ids, uint32_t m,
                           float *out);

/* ---- learned entry point and beam width (not in the reference) ----------- */
/* A small MLP (d -> 256 -> 256 -> `clusters` entry logits + 1 beam
 * regressor, BF16 with FP32 accumulation) trained on the GPU by this
 * library's own forward / backward kernels, on traces of the plain search:
 * the cluster (k-means on the base) of each training query's plain answer is
 * its entry label, and the smallest beam whose cluster-seeded answer keeps 9
 * of the 10 plain ids its beam label.  The beam margin is calibrated on 10%
 * of the training queries held out, to keep `target_agreement` of the plain
 * answers.  Needs the base and the search graph. */
typedef struct {
  uint32_t clusters, kmeans_iters, list_len, L_trace, epochs, batch;
  float lr, lam;
  uint32_t L_min, L_max;
  float target_agreement, fallback_p;
  uint32_t seed;
} wv_learn_params;
typedef struct {
  float loss_ce, loss_mse, margin, val_agreement, ms, mean_label_L;
  uint32_t steps, labelled;
} wv_learn_report;
void wv_learn_default_params(wv_learn_params *p);
int wv_learn_fit(wv_ctx *ctx, const float *train_queries, uint32_t nt, const wv_learn_params *p,
                 wv_learn_report *report);
/* Learned search: entry cluster(s) and beam per query from the model, the
 * plain random-entry search (beam L_trace) for queries below fallback_p, all
 * queries in one mixed-beam launch.  out_L (nullable): the beam each query
 * used. */
int wv_search_learned(wv_ctx *ctx, const float *queries, uint32_t nq, uint32_t K, uint32_t *out_ids, float *out_dist,
                      wv_counters *counters, uint32_t *out_L);
/* Same with device buffers; d_plain_seeds (nq x L_trace, drawn with
 * wv_draw_seeds at L_trace) serve the fallback and fill short lists. */
int wv_search_learned_device(wv_ctx *ctx, const float *d_queries, uint32_t nq, uint32_t K,
                             const uint32_t *d_plain_seeds, uint32_t *d_out_ids, float *d_out_dist,
                             wv_counters *counters);
/* The model's entry cluster (argmax), its probability and the beam
 * regressor output (log2 L) for nq host queries. */
int wv_learn_predict(wv_ctx *ctx, const float *queries, uint32_t nq, uint32_t *cluster, float *prob, float *log2L);
/* The k-means cluster of base ids (as the entry lists were built). */
int wv_learn_assign(wv_ctx *ctx, const uint32_t *ids, uint32_t n, uint32_t *cluster);
/* Overrides the calibrated beam margin (beam = margin * 2^regressor). */
int wv_learn_set_margin(wv_ctx *ctx, float margin);
/* The fallback: queries whose top entry-cluster probability is below p take
 * the plain search instead (SearchEntryRand seeds, beam L_plain, drawn in
 * query order as the plain search draws them); L_plain also sizes the plain
 * seeds that fill short entry lists.  p = 0 turns the fallback off. */
int wv_learn_set_fallback(wv_ctx *ctx, float p, uint32_t L_plain);
/* Plain (SearchEntryRand) seeds per query that wv_search_learned draws on the
 * host and copies to the device: the trace beam, or 0 when no query can read
 * one (no fallback and every entry list covers the largest beam). */
int wv_learn_plain_beam(wv_ctx *ctx, uint32_t *L);
/* Loss (ce, mse) and gradients of one batch for given parameters, for the
 * gradient check; parameters packed as W1 (d x 256), b1, W2 (256 x 256), b2,
 * W3 (256 x (clusters + 1)), b3.  Overwrites (and unsets) a trained model. */
int wv_learn_param_count(uint32_t d, uint32_t clusters, unsigned long long *count);
int wv_learn_grad(wv_ctx *ctx, const float *x, const uint32_t *y_cluster, const float *y_log2L, uint32_t B,
                  uint32_t clusters, const float *params, float lam, float *grad, float *loss);

/* The seed ids SearchEntryInner would draw for nq queries (host nq x L),
 * consuming the context's rand stream exactly as the reference does. */
int wv_draw_seeds(wv_ctx *ctx, uint32_t nq, int entry, uint32_t L, uint32_t *seeds);
/* The same SEARCH_ENTRY_RAND seeds written to device memory (row q at
 * d_seeds + q * stride): one rand() per query on the host, the mt19937 /
 * GenRandom draws on the device; asynchronous on the context's stream. */
int wv_draw_seeds_device(wv_ctx *ctx, uint32_t nq, uint32_t L, uint32_t *d_seeds, uint32_t stride);

/* ---- graph files and index statistics ------------------------------------ */
/* Header forms of a graph file (the `with_ep` / `use_ep` arguments below) */
#define WV_GRAPH_PLAIN 0 /* no header (KGraph, ...) */
#define WV_GRAPH_EP 1    /* one entry point ep_ (INDEX_NSG, INDEX_VAMANA) */
#define WV_GRAPH_EPS 2   /* root count, then the roots eps_ (INDEX_SSG) */
#define WV_GRAPH_HNSW 3  /* the INDEX_HNSW file (load only, into the HNSW search graph) */
#define WV_GRAPH_NSW 4   /* the INDEX_NSW file (load only: a one-layer HNSW graph, node 0 first) */
/* The per-node graph file of IndexBuilder::save_graph / load_graph
 * (src/builder.cpp:918-1095): the header (WV_GRAPH_*), then, per node, its
 * degree and ids (u32 each).  Save writes the built graph (final_graph_);
 * load reads into the search graph (load_graph_) and must hold exactly n rows
 * for the uploaded base. */
int wv_save_graph(wv_ctx *ctx, const char *path, int with_ep);
int wv_load_graph(wv_ctx *ctx, const char *path, int with_ep);
/* IndexBuilder::print_index_info (builder.cpp:501-600, 714-780) on the search
 * graph: out-degree statistics, conn (traversal passes: the first from the
 * roots -- the entry point (WV_GRAPH_EP), the SSG roots (WV_GRAPH_EPS) or
 * node 0 (WV_GRAPH_PLAIN) -- then each from the smallest unreached id, until
 * every node is reached) and, given an exact KNN graph (n rows of
 * exact_width ids, exact_deg valid), the mean share of each node's first 10
 * exact neighbours in its row (-1 when no exact graph is given; an FP32 sum
 * in node order, as the reference takes it).  WV_GRAPH_HNSW reports on the
 * HNSW graph: layer-0 degrees and quality, conn walked over every layer from
 * the enterpoint. */
typedef struct {
  uint32_t max_out, min_out;
  double avg_out;
  uint32_t conn;
  double quality;
} wv_index_stats;
int wv_index_info(wv_ctx *ctx, int use_ep, const uint32_t *exact_ids, const uint32_t *exact_deg,
                  uint32_t exact_width, wv_index_stats *out);

/* ---- HNSW / NSW routing --------------------------------------------------- */
/* The HNSW search graph, given as the words of the reference's INDEX_HNSW
 * file (IndexBuilder::save_graph / load_graph, builder.cpp:925-944,
 * 1096-1124): enterpoint id, max level, then per node its id, its layer
 * count and per layer the friend count and ids.  Every node of the uploaded
 * base appears once.  wv_load_graph(ctx, path, WV_GRAPH_HNSW) reads the
 * file into it. */
int wv_load_hnsw(wv_ctx *ctx, const uint32_t *words, size_t count);
/* ComponentSearchRouteHNSW::RouteInner (router 0: greedy descent through
 * every layer from the enterpoint, then SearchAtLayer on layer 0 from the
 * path element before the last -- the enterpoint when the path holds only
 * it, where the reference reads before its path vector) or
 * ComponentSearchRouteNSW::RouteInner (router 1: SearchAtLayer on layer 0
 * from node 0), src/component_route.cpp:56-260, for every query, with L as
 * L_search (L >= K) and K as K_search.  Results equal the reference's,
 * DistCount / HopCount included (its priority queues are reproduced). */
int wv_search_hnsw(wv_ctx *ctx, const float *queries, uint32_t nq, int router, uint32_t L, uint32_t K,
                   uint32_t *out_ids, float *out_dist, wv_counters *counters);

/* ---- batched search plans (CUDA graphs, tuned launch shape) -------------- */
/* No counterpart in the reference (IndexBuilder::search loops over queries,
 * src/builder.cpp:445-454).  A plan binds one batch layout to caller-owned
 * device buffers -- queries (nq_max x d), per-query L and K (nullable: L_max,
 * K_max for every query), caller seeds (WV_PLAN_SEEDS: nq_max x L_max),
 * result ids and distances (nq_max x out_stride) -- and captures the whole
 * step as a CUDA graph: WV_PLAN_RAND draws SearchEntryRand seeds (one rand()
 * per query from the context's stream, the mt19937 draws on the device),
 * WV_PLAN_LEARNED runs the learned model's forward pass and picks each
 * query's entry and L; then the search of the first nq queries (nq given at
 * run time, <= nq_max) in one persistent launch.  Results equal
 * wv_search_batch / wv_search_learned on the same inputs and rand stream.
 * The caller rewrites its buffers between runs (after wv_plan_wait).  A plan
 * refuses to run after the base, graph, precision or model changed; destroy
 * plans before their context. */
enum { WV_PLAN_RAND = 0, WV_PLAN_SEEDS = 1, WV_PLAN_LEARNED = 2 };
typedef struct {
  uint32_t nq_max, L_max, K_max, out_stride;
  int mode;
} wv_plan_params;
typedef struct {
  int warps_per_block;
  uint32_t hash_words; /* visited-hash area per warp (32-bit words) */
  int wide_hash;       /* 1: 32-bit entries; 0: 16-bit entries where n allows (twice the slots) */
  int blocks;
  float ms;        /* measured search time (tuning) */
  int query_warps; /* throughput form (wv_set_search_expansion > 0): warps per query, 1, or 2 / 4 equal to
                      warps_per_block (one query per block); 0 reads as 1 */
} wv_plan_shape;
#define WV_TUNE_MAX 32
typedef struct {
  int n, chosen;
  wv_plan_shape tried[WV_TUNE_MAX];
} wv_tune_report;
typedef struct wv_plan wv_plan;
int wv_plan_create(wv_ctx *ctx, const wv_plan_params *p, const float *d_queries, const uint32_t *d_L,
                   const uint32_t *d_K, const uint32_t *d_seeds, uint32_t *d_out_ids, float *d_out_dist,
                   wv_plan **out);
/* Enqueues one replay on the context's stream for the first nq queries
 * (asynchronous; waits for the previous replay of this plan first). */
int wv_plan_run(wv_plan *plan, uint32_t nq);
/* Waits for the last replay; device-reported errors; counters (nullable). */
int wv_plan_wait(wv_plan *plan, wv_counters *counters);
/* Times the search of the current inputs (first nq queries) in every launch
 * shape that fits, recaptures with the fastest; consumes one replay's rand()
 * draws.  The report lists every shape tried. */
int wv_plan_tune(wv_plan *plan, uint32_t nq, wv_tune_report *report);
int wv_plan_shape_of(wv_plan *plan, wv_plan_shape *shape);
/* Pins a launch shape (warps_per_block 1/2/4/8, hash_words 0 for the default
 * or a power of two, wide_hash) and recaptures, e.g. one found by an earlier
 * wv_plan_tune; blocks and ms are ignored. */
int wv_plan_set_shape(wv_plan *plan, const wv_plan_shape *shape);
/* Device time of the search kernel in the last replay (CUDA events captured
 * around it in the graph); waits for the replay. */
int wv_plan_search_ms(wv_plan *plan, float *ms);
int wv_plan_destroy(wv_plan *plan);

/* ---- allocation-free search ---------------------------------------------- */
/* No counterpart in the reference: an extra entry point for callers that
 * cannot call cudaMalloc -- a process whose GPU memory belongs to another
 * allocator that forbids driver allocations once it is running, or a
 * latency-critical thread where cudaMalloc / cudaFree would synchronize the
 * device.  It runs the same greedy search as wv_search_device with every
 * input and output in caller-owned device memory (base n x d, graph rows
 * n x width with degrees, queries nq x d, seeds nq x L, out_ids nq x K,
 * out_dist nq x K or NULL) on `stream` (a cudaStream_t, NULL = default).
 * It needs no context and allocates nothing: its working memory is a fixed
 * 64 MiB device array inside this library, shared by every call, so calls
 * that overlap on the GPU race on it.  The first call on a device looks that
 * array's address up and keeps it for later calls; make that first call
 * before any stream capture, and after a cudaDeviceReset the kept address is
 * stale (the library must then be reloaded).  The call returns once the
 * search has finished on `stream` (it reads the kernel's status back), so
 * it is synchronous and cannot itself be captured into a CUDA graph.
 * Returns WV_ERR_LIMIT when n is too large for the fixed array (n / 16
 * words per warp slot, four slots at least: about 67 million nodes) or L /
 * width exceed the search limits, WV_ERR_DEVICE if the kernel saw an id >= n. */
int wv_search_noalloc(const float *d_base, uint32_t n, uint32_t d, const uint32_t *d_graph_ids,
                      const uint32_t *d_graph_deg, uint32_t width, const float *d_queries, uint32_t nq,
                      const uint32_t *d_seeds, uint32_t L, uint32_t K, uint32_t *d_out_ids, float *d_out_dist,
                      void *stream);

/* ---- diagnostics -------------------------------------------------------- */
/* Sorts narr arrays of (key, value) pairs, array i being
 * [offsets[i], offsets[i+1]), with the device replica of std::sort (mode 0:
 * warp-parallel, mode 1: one thread), in place, so a test can compare the
 * order of tied keys with the host's std::sort.  Arrays of up to 4096. */
int wv_debug_sort(wv_ctx *ctx, float *keys, uint32_t *vals, const uint32_t *offsets, uint32_t narr, int mode);
/* C (M x N, FP32, row-major) = A B with bf16 operands (bit patterns) at
 * element strides A(m, k) = A[m * sam + k * sak], B(k, n) = B[k * sbk + n * sbn];
 * impl 0: the mma.sync kernel, 1: the tcgen05 kernel (the MLP's GEMMs). */
int wv_debug_gemm(wv_ctx *ctx, int impl, uint32_t M, uint32_t N, uint32_t K, const uint16_t *A, long long sam,
                  long long sak, const uint16_t *B, long long sbk, long long sbn, float *C);

#ifdef __cplusplus
}
#endif

#endif /* WEAVESS_GPU_H */
