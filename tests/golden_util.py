"""Replays the pipelines recorded in tests/golden/*.npz (see make_golden.py)
with a pluggable implementation, so the same replay checks the oracle against
the reference's dumps and the GPU path against the same dumps."""
from __future__ import annotations

import ast
import glob
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def cases():
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz")))


def load(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    f = {k: z[k] for k in z.files}
    f["base"] = f["base"].astype(np.float32)
    f["query"] = f["query"].astype(np.float32)
    f["params"] = ast.literal_eval(str(f["params"]))
    f["pipelines"] = ast.literal_eval(str(f["pipelines"]))
    return f


def graph_of(f, key):
    ep = f.get(key + ".ep")
    return f[key + ".ids"], f[key + ".dist"], f[key + ".deg"], (None if ep is None else int(ep))


def rows_equal(ids_a, dist_a, deg_a, ids_b, dist_b, deg_b, check_dist=True):
    """Number of rows that differ (ids in order, and distance bits)."""
    bad = 0
    n = len(deg_b)
    for i in range(n):
        k = int(deg_b[i])
        if int(deg_a[i]) != k or not np.array_equal(ids_a[i, :k], ids_b[i, :k]):
            bad += 1
        elif check_dist and not np.array_equal(np.asarray(dist_a[i, :k], np.float32).view(np.uint32),
                                               np.asarray(dist_b[i, :k], np.float32).view(np.uint32)):
            bad += 1
    return bad


def replay_oracle(f, pi, on_search=None, on_graph=None):
    """Replays pipeline `pi` of fixture `f` with the oracle (single thread,
    glibc rand stream seeded 1).  For each search step, on_search(kind, L,
    graph, rnd) may return (res, dc, hc) from the implementation under test
    (default: the oracle).  For each graph step, on_graph(kind, graph, rnd)
    may return a graph to continue with.  Yields (step, expected_key, got)."""
    import oracle as O
    p = f["params"]
    base, query = f["base"], f["query"]
    steps = f["pipelines"][pi]
    rnd = O.Rand(1)
    g = loaded = None
    entry_L = 0
    alpha = p["alpha"]
    vam_pass = 0
    for s in steps:
        kind, _, arg = s.partition(":")
        key = f"p{pi}."
        if kind == "init_random":
            g = O.init_random(base, p["S"], rnd)
            exp = key + "init"
        elif kind == "init_rand":
            g = O.init_rand(base, p["L"], rnd)
            exp = key + "initrand"
        elif kind == "init_kdt":
            g, forest = O.init_kdt(base, p["nTrees"], p["K"], p["mLevel"], rnd)
            exp = key + "initkdt"
        elif kind == "nndescent":
            g = O.nndescent(base, g, p["S"], p["K"], p["L"], p["ITER"], p["R"], rnd)
            exp = key + "nnd"
        elif kind == "vamana":
            vam_pass += 1
            g = O.vamana(base, g, p["L_refine"], p["R_refine"], alpha, rnd, entry_L=entry_L)
            alpha = 2.0
            exp = key + ("vamana" if vam_pass == steps.count("vamana") else f"vamana{vam_pass}")
        elif kind == "nsg":
            g = O.nsg(base, g, p["L_refine"], p["R_refine"], p["C_refine"], rnd)
            entry_L = p["L_refine"]
            exp = key + "nsg"
        elif kind == "efanna":
            g = O.efanna(base, g, p["S"], p["K"], p["L"], p["ITER"], p["R"], rnd)
            exp = key + "efanna"
        elif kind == "ssg":
            g = O.ssg(base, g, p["L_refine"], p["R_refine"], float(p["A"]), p["n_try"], rnd)
            exp = key + "ssg"
        elif kind == "load":
            loaded = g
            continue
        elif kind == "hnsw":
            hwords = f[key + "hnsw.words"]
            continue
        elif kind == "policy":
            # IndexBuilder::search's L policy around the search of `loaded`
            from weavess_gb300 import policy as P
            entry, _, pol = arg.partition("_")
            fn = ((lambda L: on_search(entry, L, loaded, rnd)) if on_search
                  else (lambda L: O.search(base, query, loaded, L, rnd, entry=entry)))
            got = P.set_recall(fn, f["gt"])[0] if pol == "set_recall" else P.ascend(fn, f["gt"])
            yield s, f"{key}policy_{arg}", got
            continue
        elif kind == "nsw":
            hwords = O.nsw_to_hnsw_words(f[key + "nsw.words"], base.shape[0])
            continue
        elif kind in ("search_hnsw", "search_nsw", "search_nswidx"):
            router, L = ("hnsw" if kind == "search_hnsw" else "nsw"), int(arg)
            got = (on_search(router, L, hwords, rnd) if on_search
                   else O.search_hnsw(base, query, hwords, L, router=router))
            yield s, f"{key}{kind}_{arg}", got
            continue
        elif kind == "search_kdt":
            L = int(arg)
            got = on_search("kdt", L, loaded, rnd) if on_search else O.search_kdt(base, query, loaded, forest, L, rnd)
            yield s, f"{key}{kind}_{arg}", got
            continue
        else:
            entry = {"search_rand": "rand", "search_centroid": "centroid", "search_sub": "sub_centroid"}[kind]
            L = int(arg)
            got = on_search(entry, L, loaded, rnd) if on_search else O.search(base, query, loaded, L, rnd,
                                                                              entry=entry)
            yield s, f"{key}{kind}_{arg}", got
            continue
        if on_graph is not None:
            g2 = on_graph(kind, g, rnd)
            if g2 is not None:
                g = g2
        yield s, exp, g
