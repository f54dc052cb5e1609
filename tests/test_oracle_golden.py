"""The oracle (C++ restatement, oracle/weavess_oracle.cpp) against fixtures
produced by the unmodified reference: every graph row, entry point, search
result id and DistCount/HopCount must be identical."""
import ctypes

import numpy as np
import pytest

import oracle as O
from golden_util import cases, load, graph_of, rows_equal


def check_policy(steps, f, key, where):
    """The widths, DistCount and HopCount of every step equal the reference's
    (its accuracy was printed with six significant digits)."""
    want = f[key + ".steps"]
    got = np.array([[st["L"], st["dist_count"], st["hop_count"]] for st in steps], np.uint64)
    assert got.shape == want.shape and np.array_equal(got, want.astype(np.uint64)), (where, got, want)
    acc = np.array([st["accuracy"] for st in steps])
    assert np.allclose(acc, f[key + ".acc"], rtol=0, atol=5e-6), where


def test_rand_stream_matches_glibc():
    libc = ctypes.CDLL("libc.so.6")
    libc.srand(1)
    r = O.Rand(1)
    assert all(r.next() == libc.rand() for _ in range(20000))
    libc.srand(12345)
    r = O.Rand(12345)
    assert all(r.next() == libc.rand() for _ in range(20000))


@pytest.mark.parametrize("name", cases())
def test_oracle_replays_reference(name):
    f = load(name)
    p = f["params"]
    base, query = f["base"], f["query"]
    for pi, steps in enumerate(f["pipelines"]):
        rnd = O.Rand(1)
        g = None
        loaded = None
        entry_L = 0
        alpha = p["alpha"]
        vam_pass = 0
        for s in steps:
            kind, _, arg = s.partition(":")
            key = f"p{pi}."
            if kind == "init_random":
                g = O.init_random(base, p["S"], rnd)
                exp = graph_of(f, key + "init")
            elif kind == "init_rand":
                g = O.init_rand(base, p["L"], rnd)
                exp = graph_of(f, key + "initrand")
            elif kind == "init_kdt":
                g, forest = O.init_kdt(base, p["nTrees"], p["K"], p["mLevel"], rnd)
                assert np.array_equal(forest.leaf, f[key + "kdtleaf"]), (name, s)
                exp = graph_of(f, key + "initkdt")
            elif kind == "nndescent":
                g = O.nndescent(base, g, p["S"], p["K"], p["L"], p["ITER"], p["R"], rnd)
                exp = graph_of(f, key + "nnd")
            elif kind == "vamana":
                vam_pass += 1
                g = O.vamana(base, g, p["L_refine"], p["R_refine"], alpha, rnd, entry_L=entry_L)
                alpha = 2.0  # the reference sets alpha = 2 after a Vamana link
                last = vam_pass == steps.count("vamana")
                exp = graph_of(f, key + ("vamana" if last else f"vamana{vam_pass}"))
            elif kind == "nsg":
                g = O.nsg(base, g, p["L_refine"], p["R_refine"], p["C_refine"], rnd)
                entry_L = p["L_refine"]
                exp = graph_of(f, key + "nsg")
            elif kind == "efanna":
                g = O.efanna(base, g, p["S"], p["K"], p["L"], p["ITER"], p["R"], rnd)
                exp = graph_of(f, key + "efanna")
            elif kind == "ssg":
                g = O.ssg(base, g, p["L_refine"], p["R_refine"], float(p["A"]), p["n_try"], rnd)
                exp = graph_of(f, key + "ssg")
                assert np.array_equal(g.eps, f[key + "ssg.eps"]), (name, s)
            elif kind == "load":
                loaded = g
                continue
            elif kind == "hnsw":
                hwords = f[key + "hnsw.words"]
                continue
            elif kind == "nsw":
                hwords = O.nsw_to_hnsw_words(f[key + "nsw.words"], base.shape[0])
                continue
            elif kind in ("search_hnsw", "search_nsw", "search_nswidx"):
                router = "hnsw" if kind == "search_hnsw" else "nsw"
                res, dc, hc = O.search_hnsw(base, query, hwords, int(arg), router=router)
                k = f"{key}{kind}_{arg}"
                assert np.array_equal(res, f[k + ".res"]), (name, s)
                assert [dc, hc] == f[k + ".counts"].tolist(), (name, s)
                continue
            elif kind == "policy":
                from weavess_gb300 import policy as P
                entry, _, pol = arg.partition("_")
                fn = lambda L: O.search(base, query, loaded, L, rnd, entry=entry)  # noqa: E731
                steps = P.set_recall(fn, f["gt"])[0] if pol == "set_recall" else P.ascend(fn, f["gt"])
                check_policy(steps, f, f"{key}policy_{arg}", (name, s))
                continue
            elif kind == "search_kdt":
                res, dc, hc = O.search_kdt(base, query, loaded, forest, int(arg), rnd)
                k = f"{key}{kind}_{arg}"
                assert np.array_equal(res, f[k + ".res"]), (name, s)
                assert [dc, hc] == f[k + ".counts"].tolist(), (name, s)
                continue
            elif kind.startswith("search"):
                entry = {"search_rand": "rand", "search_centroid": "centroid", "search_sub": "sub_centroid"}[kind]
                res, dc, hc = O.search(base, query, loaded, int(arg), rnd, entry=entry)
                k = f"{key}{kind}_{arg}"
                assert np.array_equal(res, f[k + ".res"]), (name, s)
                assert [dc, hc] == f[k + ".counts"].tolist(), (name, s)
                continue
            ids, dist, deg, ep = exp
            assert rows_equal(g.ids, g.dist, g.deg, ids, dist, deg) == 0, (name, s)
            if ep is not None:
                assert g.ep == ep, (name, s)
