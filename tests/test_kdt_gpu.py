"""GPU INIT_KDT and SEARCH_ENTRY_KDT against the reference: the EFANNA
pipeline of the golden fixtures (INIT_KDT -> REFINE_EFANNA -> save / load ->
SEARCH_ENTRY_KDT + ROUTER_GREEDY, as test/main.cpp:190-210 runs it) row for
row (ids and distance bits), result ids and DistCount / HopCount; and against
the oracle at sizes beyond the fixtures."""
import numpy as np
import pytest

import oracle as O
from golden_util import cases, graph_of, load, rows_equal
from weavess_gb300 import datasets as ds

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from weavess_gb300 import Context
    return Context(0)


@pytest.mark.parametrize("name", cases())
def test_kdt_efanna_pipeline_matches_reference_golden(ctx, name):
    f = load(name)
    p = f["params"]
    pis = [i for i, s in enumerate(f["pipelines"]) if s[0] == "init_kdt"]
    assert pis
    pi = pis[0]
    key = f"p{pi}."
    ctx.upload_base(f["base"])
    ctx.srand(1)
    ctx.init_kdt(p["nTrees"], p["K"], p["mLevel"])
    ids, dist, deg, _ = ctx.get_graph()
    assert rows_equal(ids, dist, deg, *graph_of(f, key + "initkdt")[:3]) == 0
    ctx.efanna_refine(p["S"], p["K"], p["L"], p["ITER"], p["R"])
    ids, dist, deg, _ = ctx.get_graph()
    assert rows_equal(ids, dist, deg, *graph_of(f, key + "efanna")[:3]) == 0
    ctx.load_built_graph()
    query = f["query"].astype(np.float32)
    n_search = 0
    for s in f["pipelines"][pi]:
        kind, _, arg = s.partition(":")
        if kind != "search_kdt":
            continue
        res, dc, hc = ctx.search(query, int(arg), 10, entry="kdt")
        assert np.array_equal(res, f[f"{key}{kind}_{arg}.res"]), (name, s)
        assert [dc, hc] == f[f"{key}{kind}_{arg}.counts"].tolist(), (name, s)
        n_search += 1
    assert n_search > 0


@pytest.mark.parametrize("kind,n,d,T,K,ml,L", [
    ("int", 20000, 128, 8, 30, 4, 64),
    ("int", 12000, 64, 3, 17, 0, 40),
    ("unit", 10000, 96, 4, 20, 2, 48),
    ("int", 60000, 16, 2, 12, 6, 30),  # id lists beyond shared memory: shuffled in global memory
])
def test_init_kdt_matches_oracle(ctx, kind, n, d, T, K, ml, L):
    if kind == "int":
        base, query = ds.int_mixture(n, d, 24, seed=31, n_query=200)
    else:
        base, query = ds.unit_mixture(n, d, 40, seed=31, n_query=200)
    ctx.upload_base(base)
    ctx.srand(1)
    st = ctx.init_kdt(T, K, ml)
    r = O.Rand(1)
    g, forest = O.init_kdt(base, T, K, ml, r)
    assert st["rand_draws"] == T * (n - 1)
    ids, dist, deg, _ = ctx.get_graph()
    assert rows_equal(ids, dist, deg, g.ids, g.dist, g.deg) == 0
    # the KD-tree entry over the KD-tree graph itself
    ctx.load_built_graph()
    ctx.srand(77)
    res, dc, hc = ctx.search(query, L, 10, entry="kdt")
    eres, edc, ehc = O.search_kdt(base, query, g, forest, L, O.Rand(77))
    assert np.array_equal(res, eres)
    assert (dc, hc) == (edc, ehc)


def test_init_kdt_short_rows_and_errors(ctx):
    """Rows short of K (no merges above a deep mLevel) take the reference's
    mt19937 fill; the KD-tree entry needs trees of the current base and the
    host-query call."""
    base, query = ds.int_mixture(3000, 16, 6, seed=4, n_query=20)
    ctx.upload_base(base)
    with pytest.raises(RuntimeError):
        ctx.search(query, 20, 10, entry="kdt")  # no trees yet
    ctx.srand(1)
    ctx.init_kdt(2, 12, 30)  # mLevel deeper than the trees: every row is filled
    g, forest = O.init_kdt(base, 2, 12, 30, O.Rand(1))
    ids, dist, deg, _ = ctx.get_graph()
    assert rows_equal(ids, dist, deg, g.ids, g.dist, g.deg) == 0
    ctx.load_built_graph()
    with pytest.raises(RuntimeError):
        ctx.search_batch(query, np.full(20, 20, np.uint32), np.full(20, 10, np.uint32), entry="kdt")


def test_failed_init_kdt_clears_the_forest(ctx):
    """An INIT_KDT that is refused part way through rewrites the forest's work
    buffers, so the trees of the earlier init on the same base are gone: the
    KD-tree entry must refuse instead of walking a partial forest."""
    rng = np.random.default_rng(9)
    # five distinct rows repeated: every point sees at most five distinct
    # distances, so K = 3 fills its rows and K = 8 cannot
    base = np.repeat(rng.integers(0, 256, (5, 16)).astype(np.float32), 40, axis=0)
    query = base[::37].copy()
    ctx.upload_base(base)
    ctx.srand(1)
    ctx.init_kdt(2, 3, 30)
    ctx.load_built_graph()
    ctx.search(query, 8, 3, entry="kdt")  # the forest of the completed init
    with pytest.raises(RuntimeError):
        ctx.init_kdt(2, 8, 30)  # refused by the K fill
    with pytest.raises(RuntimeError):
        ctx.search(query, 8, 3, entry="kdt")
