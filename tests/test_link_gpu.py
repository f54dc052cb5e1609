"""GPU Vamana / NSG / SSG link (candidates, prune, InterInsert, entry point,
connectivity) against the reference: every row, the entry point (the SSG
roots) and the searches that follow must be identical."""
import numpy as np
import pytest

import oracle as O
from golden_util import cases, load, graph_of, rows_equal
from weavess_gb300 import datasets as ds

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from weavess_gb300 import Context
    return Context(0)


def _replay(ctx, f, pi):
    """Runs pipeline pi of a golden case on the GPU; checks every graph and
    search step against the reference's dumps."""
    p = f["params"]
    base, query = f["base"], f["query"]
    steps = f["pipelines"][pi]
    ctx.upload_base(base)
    ctx.srand(1)
    alpha = p["alpha"]
    entry_L = 0
    vam = 0
    checked = []
    for s in steps:
        kind, _, arg = s.partition(":")
        key = f"p{pi}."
        if kind == "init_random":
            ctx.init_random(p["S"])
            exp = key + "init"
        elif kind == "init_rand":
            ctx.init_rand(p["L"])
            exp = key + "initrand"
        elif kind == "nndescent":
            ctx.nnd_refine(p["S"], p["K"], p["L"], p["ITER"], p["R"])
            exp = key + "nnd"
        elif kind == "vamana":
            vam += 1
            ctx.vamana_refine(p["L_refine"], p["R_refine"], alpha, entry_L)
            alpha = 2.0
            exp = key + ("vamana" if vam == steps.count("vamana") else f"vamana{vam}")
        elif kind == "nsg":
            ctx.nsg_refine(p["L_refine"], p["R_refine"], p["C_refine"])
            entry_L = p["L_refine"]
            exp = key + "nsg"
        elif kind == "efanna":
            ctx.efanna_refine(p["S"], p["K"], p["L"], p["ITER"], p["R"])
            exp = key + "efanna"
        elif kind == "ssg":
            st = ctx.ssg_refine(p["L_refine"], p["R_refine"], float(p["A"]), p["n_try"])
            exp = key + "ssg"
            assert np.array_equal(st["eps"], f[exp + ".eps"]), s
        elif kind == "load":
            ctx.load_built_graph()
            continue
        elif kind == "policy":  # IndexBuilder::search with its L policy, on the context's rand stream
            entry, _, pol = arg.partition("_")
            got = ctx.search_policy(query, f["gt"], policy=pol, entry=entry)
            steps = got[0] if pol == "set_recall" else got
            k = f"{key}policy_{arg}"
            have = np.array([[st["L"], st["dist_count"], st["hop_count"]] for st in steps], np.uint64)
            assert np.array_equal(have, f[k + ".steps"].astype(np.uint64)), s
            assert np.allclose([st["accuracy"] for st in steps], f[k + ".acc"], rtol=0, atol=5e-6), s
            checked.append(s)
            continue
        else:
            entry = {"search_rand": "rand", "search_centroid": "centroid", "search_sub": "sub_centroid"}[kind]
            res, dc, hc = ctx.search(query, int(arg), 10, entry=entry)
            k = f"{key}{kind}_{arg}"
            assert np.array_equal(res, f[k + ".res"]), s
            assert [dc, hc] == f[k + ".counts"].tolist(), s
            checked.append(s)
            continue
        ids, dist, deg, ep = ctx.get_graph()
        e = graph_of(f, exp)
        assert rows_equal(ids, dist, deg, *e[:3]) == 0, s
        if e[3] is not None:
            assert ep == e[3], s
        checked.append(s)
    return checked


@pytest.mark.parametrize("name", cases())
def test_full_pipelines_match_reference_golden(ctx, name):
    f = load(name)
    for pi, steps in enumerate(f["pipelines"]):
        if steps[0] in ("hnsw", "nsw"):
            continue  # HNSW / NSW routing over the reference's graphs: tests/test_hnsw_gpu.py
        if steps[0] == "init_kdt":
            continue  # INIT_KDT -> EFANNA -> KD-tree entry: tests/test_kdt_gpu.py
        assert _replay(ctx, f, pi)


@pytest.fixture(scope="module")
def mix20k():
    base, query = ds.int_mixture(20000, 128, 32, seed=21, n_query=200)
    return base, query, None


@pytest.mark.parametrize("alpha,L_refine", [(1.2, 24), (1.2, 48), (2.0, 24)])
def test_vamana_matches_oracle_20k(ctx, mix20k, alpha, L_refine):
    base, query, g = mix20k
    # the GPU and the oracle each run the whole pipeline from rand seed 1
    ctx.upload_base(base)
    ctx.srand(1)
    ctx.init_random(10)
    ctx.nnd_refine(10, 24, 40, 6, 50)
    ro = O.Rand(1)
    go = O.nndescent(base, O.init_random(base, 10, ro), 10, 24, 40, 6, 50, ro)
    gv = O.vamana(base, go, L_refine, 32, alpha, ro)
    st = ctx.vamana_refine(L_refine, 32, alpha, 0)
    ids, dist, deg, ep = ctx.get_graph()
    assert ep == gv.ep
    assert rows_equal(ids, dist, deg, gv.ids, gv.dist, gv.deg) == 0, st


@pytest.mark.parametrize("alpha,L_refine", [(1.2, 24), (1.2, 48), (2.0, 32)])
def test_vamana_clean_mode_matches_oracle_20k(ctx, mix20k, alpha, L_refine):
    """The clean build mode (the Vamana link's defects fixed: centroid entry
    search, sorted short pools, closest-first re-prune) against the oracle's
    clean mode, row for row and entry point; compat stays the default."""
    base, query, g = mix20k
    ctx.upload_base(base)
    ctx.srand(1)
    ctx.init_random(10)
    ctx.nnd_refine(10, 24, 40, 6, 50)
    ro = O.Rand(1)
    go = O.nndescent(base, O.init_random(base, 10, ro), 10, 24, 40, 6, 50, ro)
    gv = O.vamana(base, go, L_refine, 32, alpha, ro, clean=True)
    ctx.set_build_mode("clean")
    try:
        st = ctx.vamana_refine(L_refine, 32, alpha, 0)
    finally:
        ctx.set_build_mode("compat")
    ids, dist, deg, ep = ctx.get_graph()
    assert ep == gv.ep and ep != 0  # the centroid search, not node 0
    assert rows_equal(ids, dist, deg, gv.ids, gv.dist, gv.deg) == 0, st


@pytest.mark.parametrize("prune", ["gram", "fp32"])
def test_nsg_matches_oracle_20k(ctx, mix20k, prune, monkeypatch):
    # integer rows: the prune's pair distances come from BF16 Gram tiles by
    # default, from ordered FP32 sums with WV_LINK_PRUNE=fp32; both must give
    # the reference's graph
    if prune == "fp32":
        monkeypatch.setenv("WV_LINK_PRUNE", "fp32")
    base, query, g = mix20k
    ctx.upload_base(base)
    ctx.srand(1)
    ctx.init_random(10)
    ctx.nnd_refine(10, 24, 40, 6, 50)
    ro = O.Rand(1)
    go = O.nndescent(base, O.init_random(base, 10, ro), 10, 24, 40, 6, 50, ro)
    gn = O.nsg(base, go, 40, 24, 200, ro)
    st = ctx.nsg_refine(40, 24, 200)
    ids, dist, deg, ep = ctx.get_graph()
    assert ep == gn.ep
    assert st["conn_added"] == gn.conn_added
    assert rows_equal(ids, dist, deg, gn.ids, gn.dist, gn.deg) == 0, st


@pytest.mark.parametrize("L_refine,R_refine,A,n_try", [(100, 50, 60.0, 10), (200, 32, 30.0, 4), (40, 24, 75.0, 1)])
def test_ssg_matches_oracle_20k(ctx, mix20k, L_refine, R_refine, A, n_try):
    base, query, g = mix20k
    ctx.upload_base(base)
    ctx.srand(1)
    ctx.init_random(10)
    ctx.nnd_refine(10, 24, 40, 6, 50)
    ro = O.Rand(1)
    go = O.nndescent(base, O.init_random(base, 10, ro), 10, 24, 40, 6, 50, ro)
    gs = O.ssg(base, go, L_refine, R_refine, A, n_try, ro)
    st = ctx.ssg_refine(L_refine, R_refine, A, n_try)
    assert np.array_equal(st["eps"], gs.eps)
    assert st["conn_added"] == gs.conn_added
    ids, dist, deg, _ = ctx.get_graph()
    assert rows_equal(ids, dist, deg, gs.ids, gs.dist, gs.deg) == 0, st
    # the rand stream continues where the reference's would
    assert ctx.rand() == ro.next()
    # the SSG search (sub-centroid entry over the roots), per call and batched
    ctx.load_built_graph()
    assert np.array_equal(ctx.get_eps(), gs.eps)
    L = max(50, n_try)
    res, dc, hc = ctx.search(query, L, 10, entry="sub_centroid")
    eres, edc, ehc = O.search(base, query, gs, L, ro, entry="sub_centroid")
    assert np.array_equal(res, eres) and (dc, hc) == (edc, ehc)
    Ls = np.full(query.shape[0], L, np.uint32)
    Ks = np.full(query.shape[0], 10, np.uint32)
    bres, bdc, bhc = ctx.search_batch(query, Ls, Ks, entry="sub_centroid")
    eres, edc, ehc = O.search(base, query, gs, L, ro, entry="sub_centroid")
    assert np.array_equal(bres[:, :10], eres) and (bdc, bhc) == (edc, ehc)


def test_ssg_graph_file_and_conn(ctx, mix20k, tmp_path):
    """The INDEX_SSG file (root count, roots, rows) round-trips, and
    print_index_info's conn, walked from all the roots, is one pass."""
    base, query, g = mix20k
    ctx.upload_base(base)
    ctx.srand(1)
    ctx.init_random(10)
    ctx.nnd_refine(10, 24, 40, 6, 50)
    st = ctx.ssg_refine(100, 50, 60.0, 10)
    path = str(tmp_path / "g.ssg")
    ctx.save_graph(path, with_ep="eps")
    raw = np.fromfile(path, dtype=np.uint32)
    assert raw[0] == 10 and np.array_equal(raw[1:11], st["eps"])
    ids, dist, deg, _ = ctx.get_graph()
    ctx.load_graph(path, with_ep="eps")
    info = ctx.index_info(use_ep="eps")
    assert info["conn"] == 1
    assert info["max_out"] == int(deg.max()) and info["min_out"] == int(deg.min())


@pytest.mark.parametrize("L", [64])
def test_vamana_pipeline_matches_oracle_20k(ctx, mix20k, L):
    """The reference's Vamana build (test/main.cpp:168-172): INIT_RAND, then
    REFINE_VAMANA twice (alpha 1.2, then 2 as the reference leaves it), then
    a centroid-entry search."""
    base, query, _ = mix20k
    ctx.upload_base(base)
    ctx.srand(1)
    st = ctx.init_rand(L)
    ro = O.Rand(1)
    g = O.init_rand(base, L, ro)
    ids, dist, deg, _ = ctx.get_graph()
    assert rows_equal(ids, dist, deg, g.ids, g.dist, g.deg) == 0, st
    for alpha in (1.2, 2.0):
        ctx.vamana_refine(40, 32, alpha, 0)
        g = O.vamana(base, g, 40, 32, alpha, ro)
        ids, dist, deg, ep = ctx.get_graph()
        assert ep == g.ep and rows_equal(ids, dist, deg, g.ids, g.dist, g.deg) == 0
    ctx.load_built_graph()
    res, dc, hc = ctx.search(query, 64, 10, entry="centroid")
    eres, edc, ehc = O.search(base, query, g, 64, ro, entry="centroid")
    assert np.array_equal(res, eres) and (dc, hc) == (edc, ehc)


def test_nsg_conn_batched_equals_serial(ctx, monkeypatch):
    """ConnNSGDFS's greedy searches run in batches that the host takes in
    repair order; with one search at a time (WV_CONN_BATCH=1), a small batch
    and the default, the rows, the repairs and the rand() draws must agree."""
    base, _ = ds.int_mixture(100_000, 128, 64, seed=5)
    out = {}
    for batch in ("1", "7", "4096"):
        monkeypatch.setenv("WV_CONN_BATCH", batch)
        ctx.upload_base(base)
        ctx.srand(1)
        ctx.init_random(10)
        ctx.nnd_refine(10, 24, 40, 6, 50)
        st = ctx.nsg_refine(32, 32, 500)
        out[batch] = (st, ctx.get_graph())
    s1, (i1, d1, g1, e1) = out["1"]
    assert s1["conn_added"] >= 10, s1
    for batch in ("7", "4096"):
        s, (i, d, g, e) = out[batch]
        assert s["conn_added"] == s1["conn_added"] and s["rand_draws"] == s1["rand_draws"], (batch, s, s1)
        assert e == e1 and rows_equal(i, d, g, i1, d1, g1) == 0, batch
