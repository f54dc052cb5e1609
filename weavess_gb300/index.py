"""Host-side API over the C ABI.

`Context` is one GPU's view of an index: base vectors, the current graph and
the rand() stream, with one method per reference component it replaces.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib

ENTRY = {"rand": 0, "centroid": 1, "seeds": 2, "sub_centroid": 3, "kdt": 4}
RAND_FN = C.CFUNCTYPE(C.c_int)


def _u32(x):
    return np.ascontiguousarray(x, dtype=np.uint32)


def _f32(x):
    return np.ascontiguousarray(x, dtype=np.float32)


class Context:
    def __init__(self, device: int = 0):
        self.L = _lib.load()
        h = C.c_void_p()
        rc = self.L.wv_ctx_create(C.byref(h), device)
        if rc != 0:
            raise _lib.WeavessError(rc, f"wv_ctx_create(device={device}) failed")
        self.h = h
        self.n = self.d = 0

    # -- plumbing
    def _check(self, rc):
        if rc != 0:
            raise _lib.WeavessError(rc, self.L.wv_last_error(self.h).decode())

    def close(self):
        if getattr(self, "h", None):
            self.L.wv_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream_ptr: int = 0):
        """Issue all work on this CUDA stream (e.g. torch.cuda.current_stream().cuda_stream)."""
        self._check(self.L.wv_set_stream(self.h, C.c_void_p(stream_ptr or None)))

    # -- rand stream
    def srand(self, seed: int):
        self._check(self.L.wv_srand(self.h, seed))

    def set_rand_source(self, fn=None):
        """Draw rand() values from the callable `fn` (None: the context's own
        glibc-compatible stream), e.g. to share a process-wide stream."""
        self._rand_cb = RAND_FN(fn) if fn is not None else None
        self._check(self.L.wv_set_rand_source(self.h, C.cast(self._rand_cb, C.c_void_p) if fn else None))

    def rand(self) -> int:
        v = C.c_int()
        self._check(self.L.wv_rand(self.h, C.byref(v)))
        return v.value

    # -- data
    def upload_base(self, base: np.ndarray):
        base = _f32(base)
        self._check(self.L.wv_upload_base(self.h, base, base.shape[0], base.shape[1]))
        self.n, self.d = base.shape

    def upload_graph(self, ids: np.ndarray, deg: np.ndarray, ep: int = 0, eps=None):
        """The search graph; `eps` are its SSG roots (the sub-centroid entry)."""
        ids = _u32(ids)
        self._check(self.L.wv_upload_graph(self.h, ids, _u32(deg), ids.shape[0], ids.shape[1], int(ep or 0)))
        if eps is not None:
            e = _u32(eps)
            self._check(self.L.wv_set_eps(self.h, e.ctypes.data, len(e)))

    # -- IndexBuilder::search with its L policy (builder.cpp:187-487)
    def search_policy(self, queries, gt, policy: str = "set_recall", entry: str = "rand", L: int = 0,
                      router: str = "greedy"):
        """The reference's search loop around this context's searches:
        policy "set_recall" (L_SEARCH_SET_RECALL; returns (steps, L_min)),
        "ascend" (L_SEARCH_ASCEND) or "assign" (L_SEARCH_ASSIGN with L);
        router "greedy" (with `entry`) or "hnsw" / "nsw".  Each step records
        L, the reference's 10-NN accuracy, DistCount, HopCount and seconds."""
        from . import policy as P
        if router == "greedy":
            def fn(Lq):
                return self.search(queries, Lq, P.K_SEARCH, entry=entry)
        else:
            def fn(Lq):
                return self.search_hnsw(queries, Lq, P.K_SEARCH, router=router)
        if policy == "set_recall":
            return P.set_recall(fn, gt)
        if policy == "ascend":
            return P.ascend(fn, gt)
        return P.assign(fn, L, gt)

    # -- HNSW / NSW routing over the reference's INDEX_HNSW graph
    def load_hnsw(self, words: np.ndarray):
        """The HNSW search graph from the words of an INDEX_HNSW file."""
        w = _u32(np.asarray(words).reshape(-1))
        self._check(self.L.wv_load_hnsw(self.h, w, w.size))

    def search_hnsw(self, queries, L: int, K: int = 10, router: str = "hnsw", return_dist=False):
        """ROUTER_HNSW / ROUTER_NSW; returns (ids nq x K, dist_count, hop_count)
        (and the distances when return_dist)."""
        q = _f32(queries)
        nq = q.shape[0]
        out = np.zeros((nq, K), np.uint32)
        dist = np.zeros((nq, K), np.float32) if return_dist else None
        cnt = _lib.Counters()
        self._check(self.L.wv_search_hnsw(self.h, q, nq, {"hnsw": 0, "nsw": 1}[router], L, K, out,
                                          None if dist is None else dist.ctypes.data, C.byref(cnt)))
        if return_dist:
            return out, dist, int(cnt.dist_count), int(cnt.hop_count)
        return out, int(cnt.dist_count), int(cnt.hop_count)

    def get_eps(self, built: bool = False) -> np.ndarray:
        """SSG roots of the built graph (built=True) or of the search graph."""
        n = C.c_uint32()
        self._check(self.L.wv_get_eps(self.h, int(built), None, 0, C.byref(n)))
        out = np.zeros(n.value, np.uint32)
        self._check(self.L.wv_get_eps(self.h, int(built), out.ctypes.data, n.value, C.byref(n)))
        return out

    # -- build graph (final_graph_)
    def set_graph(self, ids, deg, dist=None, ep=0):
        ids = _u32(ids)
        d = None if dist is None else _f32(dist)
        self._check(self.L.wv_set_graph(self.h, ids, None if d is None else d.ctypes.data, _u32(deg), ids.shape[0],
                                        ids.shape[1], int(ep or 0)))

    def get_graph(self):
        """(ids [n, w], dist [n, w], deg [n], ep) of the current build graph."""
        w, ep = C.c_uint32(), C.c_uint32()
        self._check(self.L.wv_graph_width(self.h, C.byref(w), C.byref(ep)))
        ids = np.zeros((self.n, w.value), np.uint32)
        dist = np.zeros((self.n, w.value), np.float32)
        deg = np.zeros(self.n, np.uint32)
        self._check(self.L.wv_get_graph(self.h, ids.ctypes.data, dist.ctypes.data, deg.ctypes.data, w.value))
        return ids, dist, deg, int(ep.value)

    def load_built_graph(self):
        self._check(self.L.wv_load_built_graph(self.h))

    def init_random(self, S: int):
        st = _lib.BuildStats()
        self._check(self.L.wv_init_random(self.h, S, C.byref(st)))
        return st.as_dict()

    def init_rand(self, L: int):
        """INIT_RAND (the Vamana pipeline's init): L random neighbours per node."""
        st = _lib.BuildStats()
        self._check(self.L.wv_init_rand(self.h, L, C.byref(st)))
        return st.as_dict()

    def init_kdt(self, nTrees: int, K: int, mLevel: int):
        """INIT_KDT (the EFANNA pipeline's init): nTrees randomised KD-trees,
        leaves merged below depth mLevel into rows of K; the trees are kept
        for the "kdt" search entry."""
        st = _lib.BuildStats()
        self._check(self.L.wv_init_kdt(self.h, nTrees, K, mLevel, C.byref(st)))
        return st.as_dict()

    def nnd_refine(self, S: int, K: int, L: int, ITER: int, R: int):
        st = _lib.BuildStats()
        self._check(self.L.wv_nnd_refine(self.h, S, K, L, ITER, R, C.byref(st)))
        return st.as_dict()

    def efanna_refine(self, S: int, K: int, L: int, ITER: int, R: int):
        st = _lib.BuildStats()
        self._check(self.L.wv_efanna_refine(self.h, S, K, L, ITER, R, C.byref(st)))
        return st.as_dict()

    def vamana_refine(self, L_refine: int, R_refine: int, alpha: float, entry_L: int = 0):
        st = _lib.BuildStats()
        self._check(self.L.wv_vamana_refine(self.h, L_refine, R_refine, alpha, entry_L, C.byref(st)))
        return st.as_dict()

    def set_build_mode(self, mode: str = "compat"):
        """"compat": the reference's behaviour bit for bit (the default);
        "clean": the Vamana link's defects fixed (entry point, short-pool
        order, InterInsert re-prune)."""
        self._check(self.L.wv_set_build_mode(self.h, {"compat": 0, "clean": 1}[mode]))

    def nsg_refine(self, L_refine: int, R_refine: int, C_refine: int):
        st = _lib.BuildStats()
        self._check(self.L.wv_nsg_refine(self.h, L_refine, R_refine, C_refine, C.byref(st)))
        return st.as_dict()

    def ssg_refine(self, L_refine: int, R_refine: int, A: float, n_try: int):
        """REFINE_SSG; returns the build stats with the n_try roots under "eps"."""
        st = _lib.BuildStats()
        eps = np.zeros(n_try, np.uint32)
        self._check(self.L.wv_ssg_refine(self.h, L_refine, R_refine, A, n_try, eps.ctypes.data, C.byref(st)))
        out = st.as_dict()
        out["eps"] = eps
        return out

    # -- search (IndexBuilder::search, L_SEARCH_ASSIGN)
    def search(self, queries, L: int, K: int = 10, entry="rand", return_dist=False):
        q = _f32(queries)
        nq = q.shape[0]
        out = np.zeros((nq, K), np.uint32)
        dist = np.zeros((nq, K), np.float32) if return_dist else None
        cnt = _lib.Counters()
        if isinstance(entry, np.ndarray):
            seeds = _u32(entry)
            assert seeds.shape == (nq, L)
            rc = self.L.wv_search(self.h, q, nq, ENTRY["seeds"], L, K, seeds.ctypes.data, out,
                                  None if dist is None else dist.ctypes.data, C.byref(cnt))
        else:
            rc = self.L.wv_search(self.h, q, nq, ENTRY[entry], L, K, None, out,
                                  None if dist is None else dist.ctypes.data, C.byref(cnt))
        self._check(rc)
        res = (out, int(cnt.dist_count), int(cnt.hop_count))
        return res + (dist,) if return_dist else res

    def search_batch(self, queries, L, K, entry="rand"):
        q = _f32(queries)
        nq = q.shape[0]
        L, K = _u32(L), _u32(K)
        stride = int(K.max())
        out = np.zeros((nq, stride), np.uint32)
        cnt = _lib.Counters()
        self._check(self.L.wv_search_batch(self.h, q, nq, ENTRY[entry], L, K, stride, out, None, C.byref(cnt)))
        return out, int(cnt.dist_count), int(cnt.hop_count)

    STORAGE = {"fp32": 0, "bf16": 1, "fp8": 2}

    def set_precision(self, storage: str = "fp32", rerank: int = 0):
        """Candidate distances from a bf16 / fp8 copy of the base, exact FP32
        rerank of the first `rerank` pool entries (0 = whole pool)."""
        self._check(self.L.wv_set_search_precision(self.h, self.STORAGE[storage], rerank))

    def set_expansion(self, parents: int = 0):
        """Route-search traversal: 0 the exact form (the reference's order);
        E in 1..4 the throughput form, E pool entries expanded per step."""
        self._check(self.L.wv_set_search_expansion(self.h, int(parents)))

    def candidate_distances(self, queries, ids):
        q = _f32(queries)
        ids = _u32(ids)
        out = np.zeros(ids.shape, np.float32)
        self._check(self.L.wv_candidate_distances(self.h, q, q.shape[0], ids, ids.shape[1], out))
        return out

    # -- learned entry point / beam width
    def learn_fit(self, train_queries, **kw):
        p = _lib.LearnParams()
        self.L.wv_learn_default_params(C.byref(p))
        for k, v in kw.items():
            setattr(p, k, v)
        rep = _lib.LearnReport()
        tq = _f32(train_queries)
        self._check(self.L.wv_learn_fit(self.h, tq, tq.shape[0], C.byref(p), C.byref(rep)))
        return rep.as_dict()

    def learn_predict(self, queries):
        q = _f32(queries)
        c = np.zeros(q.shape[0], np.uint32)
        p = np.zeros(q.shape[0], np.float32)
        l2 = np.zeros(q.shape[0], np.float32)
        self._check(self.L.wv_learn_predict(self.h, q, q.shape[0], c, p, l2))
        return c, p, l2

    def learn_assign(self, ids):
        ids = _u32(ids)
        out = np.zeros(ids.shape, np.uint32)
        self._check(self.L.wv_learn_assign(self.h, ids.reshape(-1), ids.size, out.reshape(-1)))
        return out

    def learn_set_margin(self, margin: float):
        self._check(self.L.wv_learn_set_margin(self.h, margin))

    def learn_set_fallback(self, p: float, L_plain: int):
        """Queries whose top entry-cluster probability is below p take the
        plain search at beam L_plain (p = 0: no fallback)."""
        self._check(self.L.wv_learn_set_fallback(self.h, float(p), int(L_plain)))

    def learn_plain_beam(self) -> int:
        v = C.c_uint32()
        self._check(self.L.wv_learn_plain_beam(self.h, C.byref(v)))
        return int(v.value)

    def search_learned(self, queries, K: int = 10, return_L=False):
        q = _f32(queries)
        nq = q.shape[0]
        out = np.zeros((nq, K), np.uint32)
        Ls = np.zeros(nq, np.uint32)
        cnt = _lib.Counters()
        self._check(self.L.wv_search_learned(self.h, q, nq, K, out, None, C.byref(cnt), Ls.ctypes.data))
        res = (out, int(cnt.dist_count), int(cnt.hop_count))
        return res + (Ls,) if return_L else res

    def search_learned_device(self, d_queries_ptr, nq, K, d_plain_seeds_ptr, d_out_ptr, counters=False):
        cnt = _lib.Counters() if counters else None
        self._check(self.L.wv_search_learned_device(self.h, C.c_void_p(d_queries_ptr), nq, K,
                                                    C.c_void_p(d_plain_seeds_ptr), C.c_void_p(d_out_ptr), None,
                                                    C.byref(cnt) if counters else None))
        return (int(cnt.dist_count), int(cnt.hop_count)) if counters else None

    def learn_grad(self, x, yc, yr, clusters, params, lam=0.5):
        x = _f32(x)
        grad = np.zeros_like(_f32(params))
        loss = np.zeros(2, np.float32)
        self._check(self.L.wv_learn_grad(self.h, x, _u32(yc), _f32(yr), x.shape[0], clusters, _f32(params), lam,
                                         grad, loss))
        return grad, loss

    def draw_seeds(self, nq: int, L: int, entry="rand"):
        out = np.zeros((nq, L), np.uint32)
        self._check(self.L.wv_draw_seeds(self.h, nq, ENTRY[entry], L, out))
        return out

    # -- graph files and statistics (IndexBuilder::save_graph / load_graph / print_index_info)
    # graph-file headers: False / "plain" (none), True / "ep" (ep_), "eps" (SSG roots)
    @staticmethod
    def _hdr(with_ep):
        return {False: 0, True: 1, "plain": 0, "ep": 1, "eps": 2, "hnsw": 3, "nsw": 4}[with_ep]

    def save_graph(self, path: str, with_ep=False):
        self._check(self.L.wv_save_graph(self.h, path.encode(), self._hdr(with_ep)))

    def load_graph(self, path: str, with_ep=False):
        self._check(self.L.wv_load_graph(self.h, path.encode(), self._hdr(with_ep)))

    def index_info(self, use_ep=False, exact_ids=None, exact_deg=None):
        r = _lib.IndexInfo()
        h = self._hdr(use_ep)
        if exact_ids is not None:
            ex = _u32(exact_ids)
            exd = _u32(exact_deg if exact_deg is not None else np.full(ex.shape[0], ex.shape[1], np.uint32))
            self._check(self.L.wv_index_info(self.h, h, ex.ctypes.data, exd.ctypes.data, ex.shape[1], C.byref(r)))
        else:
            self._check(self.L.wv_index_info(self.h, h, None, None, 0, C.byref(r)))
        return {"max_out": r.max_out, "min_out": r.min_out, "avg_out": r.avg_out, "conn": r.conn,
                "quality": r.quality}

    def plan(self, nq_max: int, K_max: int, d_queries: int, d_out_ids: int, L_max: int = 0, mode: str = "rand",
             d_L: int = 0, d_K: int = 0, d_seeds: int = 0, d_out_dist: int = 0, out_stride: int = 0):
        """A captured batch search on device buffers (pointers); see Plan."""
        return Plan(self, nq_max, K_max, d_queries, d_out_ids, L_max, mode, d_L, d_K, d_seeds, d_out_dist,
                    out_stride)

    def draw_seeds_device(self, nq: int, L: int, d_seeds_ptr: int, stride: int = 0):
        """SEARCH_ENTRY_RAND seeds into device memory (asynchronous)."""
        self._check(self.L.wv_draw_seeds_device(self.h, nq, L, C.c_void_p(d_seeds_ptr), stride or L))

    def search_device(self, d_queries_ptr: int, nq: int, L: int, K: int, d_seeds_ptr: int, d_out_ptr: int,
                      d_dist_ptr: int = 0, counters: bool = False):
        cnt = _lib.Counters() if counters else None
        self._check(self.L.wv_search_device(self.h, C.c_void_p(d_queries_ptr), nq, L, K, C.c_void_p(d_seeds_ptr),
                                            C.c_void_p(d_out_ptr), C.c_void_p(d_dist_ptr or None),
                                            C.byref(cnt) if counters else None))
        return (int(cnt.dist_count), int(cnt.hop_count)) if counters else None


PLAN_MODE = {"rand": 0, "seeds": 1, "learned": 2}


class Plan:
    """wv_plan_*: one batch layout (queries, per-query L and K, results) on
    caller-owned device buffers, captured as a CUDA graph; `run(nq)` replays it
    for the first nq queries, `wait()` returns (dist_count, hop_count), `tune(nq)`
    picks the launch shape by timing the current inputs."""

    def __init__(self, ctx, nq_max, K_max, d_queries, d_out_ids, L_max=0, mode="rand", d_L=0, d_K=0, d_seeds=0,
                 d_out_dist=0, out_stride=0):
        self.ctx, self.L = ctx, ctx.L
        p = _lib.PlanParams(nq_max, L_max, K_max, out_stride or K_max, PLAN_MODE[mode])
        h = C.c_void_p()
        vp = lambda x: C.c_void_p(x or None)
        ctx._check(self.L.wv_plan_create(ctx.h, C.byref(p), vp(d_queries), vp(d_L), vp(d_K), vp(d_seeds),
                                         vp(d_out_ids), vp(d_out_dist), C.byref(h)))
        self.h = h

    def run(self, nq: int):
        self.ctx._check(self.L.wv_plan_run(self.h, nq))

    def wait(self):
        cnt = _lib.Counters()
        self.ctx._check(self.L.wv_plan_wait(self.h, C.byref(cnt)))
        return int(cnt.dist_count), int(cnt.hop_count)

    def tune(self, nq: int):
        r = _lib.TuneReport()
        self.ctx._check(self.L.wv_plan_tune(self.h, nq, C.byref(r)))
        tried = [{"warps_per_block": t.warps_per_block, "hash_words": t.hash_words, "wide_hash": t.wide_hash,
                  "blocks": t.blocks, "ms": round(t.ms, 4), "query_warps": t.query_warps} for t in r.tried[:r.n]]
        return {"tried": tried, "chosen": tried[r.chosen] if r.chosen >= 0 else None}

    def search_ms(self) -> float:
        """Device time of the search kernel in the last replay (waits for it)."""
        v = C.c_float()
        self.ctx._check(self.L.wv_plan_search_ms(self.h, C.byref(v)))
        return float(v.value)

    def shape(self):
        sh = _lib.PlanShape()
        self.ctx._check(self.L.wv_plan_shape_of(self.h, C.byref(sh)))
        return {"warps_per_block": sh.warps_per_block, "hash_words": sh.hash_words, "wide_hash": sh.wide_hash,
                "blocks": sh.blocks, "query_warps": sh.query_warps}

    def set_shape(self, warps_per_block=4, hash_words=0, wide_hash=False, query_warps=1):
        sh = _lib.PlanShape(warps_per_block, hash_words, 1 if wide_hash else 0, 0, 0.0, query_warps)
        self.ctx._check(self.L.wv_plan_set_shape(self.h, C.byref(sh)))

    def close(self):
        if getattr(self, "h", None):
            self.L.wv_plan_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
