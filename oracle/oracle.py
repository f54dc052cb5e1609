"""ORACLE -- test infrastructure only.

ctypes bindings for oracle/_build/liboracle.so (the C++ restatement of the
reference path in weavess_oracle.cpp) and readers for the reference driver's
dump files.  Imported only by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
REF_DRIVER = os.path.join(HERE, "_ref", "ref_driver")

_lib = None

u32p = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")
f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
u8p = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")
u64p = np.ctypeslib.ndpointer(np.uint64, flags="C_CONTIGUOUS")
i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")


def build(force: bool = False) -> str:
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(
            os.path.join(HERE, "weavess_oracle.cpp")):
        subprocess.check_call(["make", "-s", "-C", HERE, "port"])
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        L.orc_rand_create.restype = C.c_void_p
        L.orc_rand_create.argtypes = [C.c_uint]
        L.orc_rand_destroy.argtypes = [C.c_void_p]
        L.orc_rand_next.argtypes = [C.c_void_p]
        L.orc_rand_fill.argtypes = [C.c_void_p, i32p, C.c_uint]
        L.orc_l2_rows.argtypes = [f32p, f32p, C.c_uint, C.c_uint, f32p]
        L.orc_init_random.argtypes = [f32p, C.c_uint, C.c_uint, C.c_uint, C.c_void_p, u32p, f32p, u32p]
        L.orc_init_rand.argtypes = [f32p, C.c_uint, C.c_uint, C.c_uint, C.c_void_p, u32p, f32p, u32p]
        L.orc_nndescent.argtypes = [f32p, C.c_uint, C.c_uint, u32p, f32p, u32p, C.c_uint, C.c_uint, C.c_uint,
                                    C.c_uint, C.c_uint, C.c_uint, C.c_void_p, C.c_int, u32p, f32p, u32p, u64p]
        L.orc_efanna.argtypes = L.orc_nndescent.argtypes[:12] + [C.c_void_p, u32p, f32p, u32p, u64p]
        L.orc_search_hnsw.argtypes = [f32p, C.c_uint, C.c_uint, f32p, C.c_uint, u32p, C.c_size_t, C.c_int, C.c_uint,
                                      C.c_uint, u32p, u64p]
        L.orc_nndescent_pools.argtypes = [f32p, C.c_uint, C.c_uint, u32p, f32p, u32p, C.c_uint, C.c_uint,
                                          C.c_uint, C.c_uint, C.c_uint, C.c_void_p, u32p, f32p, u8p, u32p, u32p]
        L.orc_vamana.argtypes = [f32p, C.c_uint, C.c_uint, u32p, f32p, u32p, C.c_uint, C.c_uint, C.c_uint,
                                 C.c_float, C.c_uint, C.c_void_p, C.c_int, u32p, f32p, u32p, u32p, C.c_int]
        L.orc_nsg.argtypes = [f32p, C.c_uint, C.c_uint, u32p, f32p, u32p, C.c_uint, C.c_uint, C.c_uint, C.c_uint,
                              C.c_void_p, C.c_int, u32p, f32p, u32p, C.c_uint, u32p, u32p]
        L.orc_ssg.argtypes = [f32p, C.c_uint, C.c_uint, u32p, f32p, u32p, C.c_uint, C.c_uint, C.c_uint, C.c_float,
                              C.c_uint, C.c_void_p, u32p, f32p, u32p, C.c_uint, u32p, u32p]
        L.orc_search.argtypes = [f32p, C.c_uint, C.c_uint, f32p, C.c_uint, u32p, u32p, C.c_uint, C.c_uint,
                                 C.c_int, C.c_uint, C.c_uint, C.c_void_p, C.c_int, u32p, u64p, u32p, C.c_uint]
        i32p_ = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
        L.orc_init_kdt.argtypes = [f32p, C.c_uint, C.c_uint, C.c_uint, C.c_uint, C.c_uint, C.c_void_p, u32p, f32p,
                                   u32p, C.c_uint, i32p_, u32p, u32p]
        L.orc_search_kdt.argtypes = [f32p, C.c_uint, C.c_uint, f32p, C.c_uint, u32p, u32p, C.c_uint, C.c_uint,
                                     C.c_uint, i32p_, u32p, u32p, C.c_uint, C.c_uint, C.c_void_p, u32p, u64p, u32p]
        L.orc_search_seeds.argtypes = [C.c_uint, C.c_uint, u32p, u32p, C.c_uint, C.c_uint, C.c_int, C.c_uint,
                                       C.c_void_p, u32p, u32p, C.c_uint]
        _lib = L
    return _lib


class Rand:
    """glibc-compatible rand() stream (default seed 1, as a fresh process)."""

    def __init__(self, seed: int = 1):
        self.h = lib().orc_rand_create(seed)

    def next(self) -> int:
        return lib().orc_rand_next(self.h)

    def take(self, n: int) -> np.ndarray:
        out = np.empty(n, dtype=np.int32)
        lib().orc_rand_fill(self.h, out, n)
        return out

    def __del__(self):
        try:
            lib().orc_rand_destroy(self.h)
        except Exception:
            pass


class Graph:
    """Fixed-width adjacency: ids[n, w], dist[n, w], deg[n] (+ entry point)."""

    def __init__(self, ids, dist, deg, ep=None):
        self.ids, self.dist, self.deg, self.ep = ids, dist, deg, ep

    @property
    def n(self):
        return self.ids.shape[0]

    @property
    def width(self):
        return self.ids.shape[1]

    def rows(self):
        return [list(zip(self.ids[i, : self.deg[i]].tolist(), self.dist[i, : self.deg[i]].tolist()))
                for i in range(self.n)]


def _c(x, dt):
    return np.ascontiguousarray(x, dtype=dt)


def l2_rows(a, b):
    a, b = _c(a, np.float32), _c(b, np.float32)
    out = np.empty(a.shape[0], dtype=np.float32)
    lib().orc_l2_rows(a, b, a.shape[0], a.shape[1], out)
    return out


def init_rand(base, L, rnd: Rand) -> Graph:
    """INIT_RAND (the Vamana init): L random neighbours per node, sorted."""
    base = _c(base, np.float32)
    n, d = base.shape
    ids = np.zeros((n, L), np.uint32)
    dist = np.zeros((n, L), np.float32)
    deg = np.zeros(n, np.uint32)
    assert lib().orc_init_rand(base, n, d, L, rnd.h, ids, dist, deg) == 0
    return Graph(ids, dist, deg)


def init_random(base, S, rnd: Rand) -> Graph:
    base = _c(base, np.float32)
    n, d = base.shape
    ids = np.zeros((n, S), np.uint32)
    dist = np.zeros((n, S), np.float32)
    deg = np.zeros(n, np.uint32)
    assert lib().orc_init_random(base, n, d, S, rnd.h, ids, dist, deg) == 0
    return Graph(ids, dist, deg)


def nndescent(base, init: Graph, S, K, L, ITER, R, rnd: Rand, threads=1):
    base = _c(base, np.float32)
    n, d = base.shape
    ids = np.zeros((n, K), np.uint32)
    dist = np.zeros((n, K), np.float32)
    deg = np.zeros(n, np.uint32)
    stats = np.zeros(2, np.uint64)
    assert lib().orc_nndescent(base, n, d, _c(init.ids, np.uint32), _c(init.dist, np.float32),
                               _c(init.deg, np.uint32), init.width, S, K, L, ITER, R, rnd.h, threads,
                               ids, dist, deg, stats) == 0
    g = Graph(ids, dist, deg)
    g.overflow_events = int(stats[0])
    return g


def efanna(base, init: Graph, S, K, L, ITER, R, rnd: Rand):
    """REFINE_EFANNA on `init` (its rows are the KD-tree graph in the
    reference's pipeline; any graph with rows of at most L entries here)."""
    base = _c(base, np.float32)
    n, d = base.shape
    ids = np.zeros((n, K), np.uint32)
    dist = np.zeros((n, K), np.float32)
    deg = np.zeros(n, np.uint32)
    stats = np.zeros(2, np.uint64)
    assert lib().orc_efanna(base, n, d, _c(init.ids, np.uint32), _c(init.dist, np.float32), _c(init.deg, np.uint32),
                            init.width, S, K, L, ITER, R, rnd.h, ids, dist, deg, stats) == 0
    g = Graph(ids, dist, deg)
    g.overflow_events = int(stats[0])
    return g


class KdtForest:
    """The trees of INIT_KDT: nodes[t, j] = (div_dim, div_val bits, start, end,
    left, right) for j < cnt[t] (node 0 the root; -1 children: a leaf), and
    the shuffled id lists leaf[t, :]."""

    def __init__(self, n, T, ncap):
        self.n, self.T, self.ncap = n, T, ncap
        self.nodes = np.zeros((T, ncap, 6), np.int32)
        self.cnt = np.zeros(T, np.uint32)
        self.leaf = np.zeros((T, n), np.uint32)


def init_kdt(base, nTrees, K, mLevel, rnd: Rand):
    """INIT_KDT: (graph with rows of K ascending, KdtForest)."""
    base = _c(base, np.float32)
    n, d = base.shape
    F = KdtForest(n, nTrees, 2 * n)
    ids = np.zeros((n, K), np.uint32)
    dist = np.zeros((n, K), np.float32)
    deg = np.zeros(n, np.uint32)
    rc = lib().orc_init_kdt(base, n, d, nTrees, K, mLevel, rnd.h, ids, dist, deg, F.ncap, F.nodes, F.cnt, F.leaf)
    assert rc == 0, rc
    return Graph(ids, dist, deg), F


def search_kdt(base, query, g: Graph, F: KdtForest, L, rnd: Rand, K=10, return_seeds=False):
    """SEARCH_ENTRY_KDT + ROUTER_GREEDY (queries in order)."""
    base, query = _c(base, np.float32), _c(query, np.float32)
    n, d = base.shape
    nq = query.shape[0]
    res = np.zeros((nq, K), np.uint32)
    cnt = np.zeros(2, np.uint64)
    seeds = np.zeros((nq, L), np.uint32)
    rc = lib().orc_search_kdt(base, n, d, query, nq, _c(g.ids, np.uint32), _c(g.deg, np.uint32), g.width, F.T,
                              F.ncap, F.nodes, F.cnt, F.leaf, L, K, rnd.h, res, cnt, seeds)
    assert rc == 0, rc
    if return_seeds:
        return res, int(cnt[0]), int(cnt[1]), seeds
    return res, int(cnt[0]), int(cnt[1])


def nndescent_pools(base, init: Graph, S, L, iters, R, rnd: Rand):
    base = _c(base, np.float32)
    n, d = base.shape
    ids = np.zeros((n, L), np.uint32)
    dist = np.zeros((n, L), np.float32)
    flag = np.zeros((n, L), np.uint8)
    deg = np.zeros(n, np.uint32)
    M = np.zeros(n, np.uint32)
    lib().orc_nndescent_pools(base, n, d, _c(init.ids, np.uint32), _c(init.dist, np.float32),
                              _c(init.deg, np.uint32), init.width, S, L, iters, R, rnd.h, ids, dist, flag, deg, M)
    return ids, dist, flag, deg, M


def vamana(base, g: Graph, L_refine, R_refine, alpha, rnd: Rand, entry_L=0, threads=1, clean=False) -> Graph:
    """REFINE_VAMANA; clean=True: this library's clean build mode (the
    link's defects fixed), not the reference."""
    base = _c(base, np.float32)
    n, d = base.shape
    ids = np.zeros((n, R_refine), np.uint32)
    dist = np.zeros((n, R_refine), np.float32)
    deg = np.zeros(n, np.uint32)
    ep = np.zeros(1, np.uint32)
    assert lib().orc_vamana(base, n, d, _c(g.ids, np.uint32), _c(g.dist, np.float32), _c(g.deg, np.uint32),
                            g.width, L_refine, R_refine, alpha, entry_L, rnd.h, threads, ids, dist, deg, ep,
                            1 if clean else 0) == 0
    return Graph(ids, dist, deg, int(ep[0]))


def nsg(base, g: Graph, L_refine, R_refine, C_refine, rnd: Rand, threads=1, out_w=None) -> Graph:
    base = _c(base, np.float32)
    n, d = base.shape
    out_w = out_w or R_refine + 32
    ids = np.zeros((n, out_w), np.uint32)
    dist = np.zeros((n, out_w), np.float32)
    deg = np.zeros(n, np.uint32)
    ep = np.zeros(1, np.uint32)
    added = np.zeros(1, np.uint32)
    assert lib().orc_nsg(base, n, d, _c(g.ids, np.uint32), _c(g.dist, np.float32), _c(g.deg, np.uint32),
                         g.width, L_refine, R_refine, C_refine, rnd.h, threads, ids, dist, deg, out_w, ep,
                         added) == 0
    out = Graph(ids, dist, deg, int(ep[0]))
    out.conn_added = int(added[0])
    return out


def ssg(base, g: Graph, L_refine, R_refine, A, n_try, rnd: Rand, out_w=None) -> Graph:
    """REFINE_SSG: Propagation2 candidates, SSG prune, InterInsert, DFS-expand
    conn; the returned graph carries `eps` (the n_try roots)."""
    base = _c(base, np.float32)
    n, d = base.shape
    out_w = out_w or R_refine
    ids = np.zeros((n, out_w), np.uint32)
    dist = np.zeros((n, out_w), np.float32)
    deg = np.zeros(n, np.uint32)
    eps = np.zeros(max(1, n_try), np.uint32)
    added = np.zeros(1, np.uint32)
    assert lib().orc_ssg(base, n, d, _c(g.ids, np.uint32), _c(g.dist, np.float32), _c(g.deg, np.uint32), g.width,
                         L_refine, R_refine, A, n_try, rnd.h, ids, dist, deg, out_w, eps, added) == 0
    out = Graph(ids, dist, deg, None)
    out.eps = eps[:n_try].copy()
    out.conn_added = int(added[0])
    return out


ENTRIES = {"rand": 0, "centroid": 1, "sub_centroid": 2}


def _eps(g: Graph, entry):
    eps = getattr(g, "eps", None) if entry == "sub_centroid" else None
    eps = np.zeros(1, np.uint32) if eps is None else _c(eps, np.uint32)
    return eps, (len(eps) if entry == "sub_centroid" else 0)


def search(base, query, g: Graph, L, rnd: Rand, entry="rand", K=10, threads=1):
    """IndexBuilder::search (L_SEARCH_ASSIGN): entry "rand", "centroid" (the
    graph's ep) or "sub_centroid" (the graph's SSG roots, g.eps)."""
    base, query = _c(base, np.float32), _c(query, np.float32)
    n, d = base.shape
    nq = query.shape[0]
    res = np.zeros((nq, K), np.uint32)
    cnt = np.zeros(2, np.uint64)
    eps, ne = _eps(g, entry)
    rc = lib().orc_search(base, n, d, query, nq, _c(g.ids, np.uint32), _c(g.deg, np.uint32), g.width,
                          int(g.ep or 0), ENTRIES[entry], L, K, rnd.h, threads, res, cnt, eps, ne)
    assert rc == 0
    return res, int(cnt[0]), int(cnt[1])


def search_hnsw(base, query, words, L, K=10, router="hnsw"):
    """ROUTER_HNSW / ROUTER_NSW over a graph in the INDEX_HNSW file layout
    (a uint32 array); returns (ids nq x K, dist_count, hop_count)."""
    base, query = _c(base, np.float32), _c(query, np.float32)
    n, d = base.shape
    nq = query.shape[0]
    w = _c(words, np.uint32)
    res = np.zeros((nq, K), np.uint32)
    cnt = np.zeros(2, np.uint64)
    rc = lib().orc_search_hnsw(base, n, d, query, nq, w, w.size, 0 if router == "hnsw" else 1, L, K, res, cnt)
    assert rc == 0, rc
    return res, int(cnt[0]), int(cnt[1])


def nsw_to_hnsw_words(words, n):
    """An INDEX_NSW file's words (records of node id, count, ids; a node's
    friends appended in file order, builder.cpp:1171-1189) as a one-layer
    INDEX_HNSW graph with node 0 as its enterpoint (where ROUTER_NSW starts)."""
    w = np.asarray(words, np.uint32)
    fr = [[] for _ in range(n)]
    p = 0
    while p + 2 <= w.size:
        v, k = int(w[p]), int(w[p + 1])
        fr[v] += w[p + 2:p + 2 + k].tolist()
        p += 2 + k
    out = [0, 0]
    for v in range(n):
        out += [v, 1, len(fr[v])] + fr[v]
    return np.array(out, np.uint32)


def search_seeds(n, nq, g: Graph, L, rnd: Rand, entry="rand"):
    seeds = np.zeros((nq, L), np.uint32)
    eps, ne = _eps(g, entry)
    lib().orc_search_seeds(n, nq, _c(g.ids, np.uint32), _c(g.deg, np.uint32), g.width, int(g.ep or 0),
                           ENTRIES[entry], L, rnd.h, seeds, eps, ne)
    return seeds


# ---------------------------------------------------------------- ref dumps
def read_graph_dump(path: str) -> Graph:
    """Read a ref_driver graph dump: u32 n, u32 ep, then per node u32 deg and
    deg x (u32 id, f32 dist)."""
    raw = np.fromfile(path, dtype=np.uint32)
    n, ep = int(raw[0]), int(raw[1])
    pos = 2
    rows = []
    for _ in range(n):
        deg = int(raw[pos])
        pos += 1
        rows.append(raw[pos: pos + 2 * deg].reshape(deg, 2))
        pos += 2 * deg
    w = max(1, max(r.shape[0] for r in rows))
    ids = np.zeros((n, w), np.uint32)
    dist = np.zeros((n, w), np.float32)
    deg = np.zeros(n, np.uint32)
    for i, r in enumerate(rows):
        deg[i] = r.shape[0]
        ids[i, : r.shape[0]] = r[:, 0]
        dist[i, : r.shape[0]] = r[:, 1].view(np.float32)
    return Graph(ids, dist, deg, None if ep == 0xFFFFFFFF else ep)


def read_search_dump(path: str):
    raw = np.fromfile(path, dtype=np.uint32)
    nq, k = int(raw[0]), int(raw[1])
    res = raw[2: 2 + nq * k].reshape(nq, k)
    dc, hc = int(raw[2 + nq * k]), int(raw[3 + nq * k])
    return res, dc, hc


def graphs_equal(a: Graph, b: Graph, check_dist=True) -> bool:
    if a.n != b.n or not np.array_equal(a.deg, b.deg):
        return False
    for i in range(a.n):
        k = int(a.deg[i])
        if not np.array_equal(a.ids[i, :k], b.ids[i, :k]):
            return False
        if check_dist and not np.array_equal(a.dist[i, :k].view(np.uint32), b.dist[i, :k].view(np.uint32)):
            return False
    return True


def row_mismatches(a: Graph, b: Graph) -> int:
    bad = 0
    for i in range(a.n):
        k = int(a.deg[i])
        if a.deg[i] != b.deg[i] or not np.array_equal(a.ids[i, :k], b.ids[i, :k]):
            bad += 1
    return bad
