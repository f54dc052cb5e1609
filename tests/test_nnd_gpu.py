"""GPU INIT_RANDOM + NN-Descent against the reference: every row of every
graph (ids in order and distance bits) must be identical."""
import os

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


@pytest.mark.parametrize("name", cases())
def test_init_and_nndescent_match_reference_golden(ctx, name):
    f = load(name)
    p = f["params"]
    ctx.upload_base(f["base"])
    ctx.srand(1)
    ctx.init_random(p["S"])
    ids, dist, deg, _ = ctx.get_graph()
    assert rows_equal(ids, dist, deg, *graph_of(f, "p0.init")[:3]) == 0
    st = ctx.nnd_refine(p["S"], p["K"], p["L"], p["ITER"], p["R"])
    ids, dist, deg, _ = ctx.get_graph()
    e = graph_of(f, "p0.nnd")
    assert rows_equal(ids, dist, deg, *e[:3]) == 0, st
    # the rand stream advanced exactly as in the reference (checked through the
    # next search, which draws from it)
    r = O.Rand(1)
    g0 = O.init_random(f["base"], p["S"], r)
    O.nndescent(f["base"], g0, p["S"], p["K"], p["L"], p["ITER"], p["R"], r)
    assert ctx.rand() == r.next()


@pytest.fixture(scope="module")
def mix20k():
    base, _ = ds.int_mixture(20000, 128, 32, seed=21)
    r = O.Rand(1)
    g0 = O.init_random(base, 10, r)
    g = O.nndescent(base, g0, 10, 20, 40, 6, 60, r)
    return base, g


@pytest.mark.parametrize("offer_cap", [None, "16384"])
def test_nndescent_matches_oracle_20k(ctx, mix20k, offer_cap, monkeypatch):
    base, g = mix20k
    if offer_cap:
        monkeypatch.setenv("WV_NND_OFFER_CAP", offer_cap)  # many small join chunks
    ctx.upload_base(base)
    ctx.srand(1)
    ctx.init_random(10)
    st = ctx.nnd_refine(10, 20, 40, 6, 60)
    ids, dist, deg, _ = ctx.get_graph()
    assert rows_equal(ids, dist, deg, g.ids, g.dist, g.deg) == 0, st
    if offer_cap:
        assert st["chunks"] > 20


def test_nndescent_unit_vectors_exact_fp32(ctx):
    """Real-valued data: distances must carry the reference's FP32 rounding."""
    base, _ = ds.unit_mixture(3000, 96, 30, seed=4)
    r = O.Rand(1)
    g = O.nndescent(base, O.init_random(base, 12, r), 12, 16, 32, 5, 24, r)
    ctx.upload_base(base)
    ctx.srand(1)
    ctx.init_random(12)
    ctx.nnd_refine(12, 16, 32, 5, 24)
    ids, dist, deg, _ = ctx.get_graph()
    assert rows_equal(ids, dist, deg, g.ids, g.dist, g.deg) == 0


@pytest.mark.parametrize("S,L,R", [(10, 40, 50), (16, 48, 12), (4, 24, 100)])
def test_efanna_matches_oracle_20k(ctx, mix20k, S, L, R):
    """REFINE_EFANNA (random first nn_new, sorted de-duplicated pools, live
    first join) on an INIT_RANDOM graph: every row and the rand stream."""
    base, _ = mix20k
    ctx.upload_base(base)
    ctx.srand(1)
    ctx.init_random(S)
    st = ctx.efanna_refine(S, 24, L, 6, R)
    ro = O.Rand(1)
    ge = O.efanna(base, O.init_random(base, S, ro), S, 24, L, 6, R, ro)
    ids, dist, deg, _ = ctx.get_graph()
    assert rows_equal(ids, dist, deg, ge.ids, ge.dist, ge.deg) == 0, st
    assert st["rand_draws"] == 1 + ge.overflow_events
    assert ctx.rand() == ro.next()


@pytest.mark.parametrize("d,S,R", [(128, 10, 60), (64, 20, 100), (16, 8, 30)])
def test_tensor_core_join_equals_fp32_join(ctx, d, S, R, monkeypatch):
    """The local join's Gram tiles on the tensor cores (integer data, d a
    multiple of 16, new lists of at most 128 ids) give the offers of the FP32
    pair kernel: the graphs, the pair and offer counts and the rand() stream
    are identical, and both equal the single-threaded oracle."""
    base, _ = ds.int_mixture(12000, d, 24, seed=50 + d)
    out = {}
    for path in ("tc", "fp32"):
        if path == "fp32":
            monkeypatch.setenv("WV_NND_JOIN", "fp32")
        else:
            monkeypatch.delenv("WV_NND_JOIN", raising=False)
        ctx.upload_base(base)
        ctx.srand(1)
        ctx.init_random(S)
        st = ctx.nnd_refine(S, 24, 40, 6, R)
        out[path] = (ctx.get_graph(), st, ctx.rand())
    (g1, st1, r1), (g2, st2, r2) = out["tc"], out["fp32"]
    assert rows_equal(g1[0], g1[1], g1[2], g2[0], g2[1], g2[2]) == 0
    assert (st1["pairs"], st1["offers"], st1["rand_draws"], r1) == (st2["pairs"], st2["offers"], st2["rand_draws"], r2)
    ro = O.Rand(1)
    g = O.nndescent(base, O.init_random(base, S, ro), S, 24, 40, 6, R, ro)
    assert rows_equal(g1[0], g1[1], g1[2], g.ids, g.dist, g.deg) == 0
