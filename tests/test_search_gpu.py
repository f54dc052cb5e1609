"""GPU greedy beam search (ROUTER_GREEDY) against the reference: result ids
and DistCount / HopCount must be identical."""
import numpy as np
import pytest

import oracle as O
from golden_util import cases, load, replay_oracle
from weavess_gb300 import datasets as ds

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from weavess_gb300 import Context
    return Context(0)


@pytest.mark.parametrize("name", cases())
def test_search_matches_reference_golden(ctx, name):
    f = load(name)
    ctx.upload_base(f["base"])
    query = f["query"]
    checked = 0

    def on_search(entry, L, g, rnd):
        if entry in ("hnsw", "nsw"):  # g: the reference's INDEX_HNSW file, as words
            ctx.load_hnsw(g)
            return ctx.search_hnsw(query, L, 10, router=entry)
        if entry == "sub_centroid":
            # the GPU draws from the oracle's rand stream (its seed distances
            # are not those of plain seeds)
            ctx.upload_graph(g.ids, g.deg, 0, eps=g.eps)
            ctx.set_rand_source(rnd.next)
            try:
                return ctx.search(query, L, 10, entry="sub_centroid")
            finally:
                ctx.set_rand_source(None)
        seeds = O.search_seeds(g.n, query.shape[0], g, L, rnd, entry=entry)
        ctx.upload_graph(g.ids, g.deg, g.ep or 0)
        return ctx.search(query, L, 10, entry=seeds)

    for pi in range(len(f["pipelines"])):
        if f["pipelines"][pi][0] == "init_kdt":
            continue  # the EFANNA pipeline (KD-tree entry): tests/test_kdt_gpu.py
        for step, key, got in replay_oracle(f, pi, on_search=on_search):
            if step.startswith("policy"):  # IndexBuilder::search's L loop around the GPU search
                want = f[key + ".steps"].astype(np.uint64)
                have = np.array([[st["L"], st["dist_count"], st["hop_count"]] for st in got], np.uint64)
                assert have.shape == want.shape and np.array_equal(have, want), (name, step)
                checked += 1
                continue
            if "search" not in step:
                continue
            res, dc, hc = got
            assert np.array_equal(res, f[key + ".res"]), (name, step)
            assert [dc, hc] == f[key + ".counts"].tolist(), (name, step)
            checked += 1
    assert checked > 0


@pytest.mark.parametrize("entry", ["rand", "centroid"])
def test_seed_draws_match_oracle(ctx, entry):
    base, q = ds.int_mixture(3000, 16, 4, seed=3, n_query=20)
    rnd = O.Rand(1)
    g = O.init_random(base, 20, rnd)
    g.ep = 17
    ctx.upload_base(base)
    ctx.upload_graph(g.ids, g.deg, g.ep)
    for L in (10, 20, 64, 300):
        ctx.srand(77)
        r2 = O.Rand(77)
        a = ctx.draw_seeds(50, L, entry)
        b = O.search_seeds(3000, 50, g, L, r2, entry=entry)
        assert np.array_equal(a, b)
        assert ctx.rand() == r2.next()  # both streams advanced alike


@pytest.mark.parametrize("n", [3000, 1601])
def test_device_seed_draws_match_oracle(ctx, n):
    """SEARCH_ENTRY_RAND seeds drawn on the device (one host rand() per query,
    mt19937 + GenRandom per warp) equal the oracle's host draws, including
    beams that need several mt19937 twists and N - L small."""
    import torch
    base, _ = ds.int_mixture(n, 16, 4, seed=3, n_query=0)
    ctx.upload_base(base)
    dummy = O.Graph(np.zeros((n, 1), np.uint32), np.zeros((n, 1), np.float32), np.zeros(n, np.uint32), 0)
    for L in (1, 10, 17, 623, 624, 1000, 1536 if n > 1536 else n - 1):
        ctx.srand(91)
        r2 = O.Rand(91)
        stride = L + 3
        d = torch.full((37, stride), -1, dtype=torch.int32, device="cuda")
        ctx.draw_seeds_device(37, L, d.data_ptr(), stride)
        torch.cuda.synchronize()
        got = d.cpu().numpy().view(np.uint32)
        want = O.search_seeds(n, 37, dummy, L, r2, entry="rand")
        assert np.array_equal(got[:, :L], want), L
        assert np.all(got[:, L:] == 0xFFFFFFFF)
        assert ctx.rand() == r2.next()


@pytest.fixture(scope="module")
def kgraph20k():
    base, query = ds.int_mixture(20000, 128, 32, seed=21, n_query=300)
    rnd = O.Rand(1)
    g = O.init_random(base, 10, rnd)
    g = O.nndescent(base, g, 10, 20, 40, 6, 60, rnd)
    return base, query, g


@pytest.mark.parametrize("L", [10, 16, 17, 50, 100, 300])
@pytest.mark.parametrize("entry", ["rand", "centroid"])
def test_search_matches_oracle_20k(ctx, kgraph20k, L, entry):
    base, query, g = kgraph20k
    g.ep = 123
    ctx.upload_base(base)
    ctx.upload_graph(g.ids, g.deg, g.ep)
    ctx.srand(5)
    res, dc, hc = ctx.search(query, L, 10, entry=entry)
    eres, edc, ehc = O.search(base, query, g, L, O.Rand(5), entry=entry)
    assert np.array_equal(res, eres)
    assert (dc, hc) == (edc, ehc)


def test_search_batch_mixed_L_K(ctx, kgraph20k):
    base, query, g = kgraph20k
    ctx.upload_base(base)
    ctx.upload_graph(g.ids, g.deg, 0)
    rng = np.random.default_rng(0)
    nq = 120
    K = rng.choice([1, 10, 50, 100], size=nq).astype(np.uint32)
    L = np.maximum(K, rng.integers(10, 400, size=nq)).astype(np.uint32)
    ctx.srand(9)
    out, dc, hc = ctx.search_batch(query[:nq], L, K)
    r = O.Rand(9)
    tdc = thc = 0
    for i in range(nq):
        e, c1, c2 = O.search(base, query[i:i + 1], g, int(L[i]), r, K=int(K[i]))
        assert np.array_equal(out[i, :K[i]], e[0]), i
        tdc += c1
        thc += c2
    assert (dc, hc) == (tdc, thc)


def test_search_batch_widest_first_many_rounds(ctx, kgraph20k):
    """Per-query beams dispatch the widest queries first (a counting sort on
    the device): with more queries than resident warps, every query's ids and
    the summed counters still equal the oracle's per-query searches."""
    base, _, g = kgraph20k
    b2, query = ds.int_mixture(20000, 128, 32, seed=21, n_query=3000)
    assert np.array_equal(b2, base)
    ctx.upload_base(base)
    ctx.upload_graph(g.ids, g.deg, 0)
    rng = np.random.default_rng(3)
    nq = query.shape[0]
    L = rng.integers(10, 200, size=nq).astype(np.uint32)
    K = np.full(nq, 10, np.uint32)
    ctx.srand(12)
    out, dc, hc = ctx.search_batch(query, L, K)
    r = O.Rand(12)
    tdc = thc = 0
    for i in range(nq):
        e, c1, c2 = O.search(base, query[i:i + 1], g, int(L[i]), r, K=10)
        assert np.array_equal(out[i], e[0]), i
        tdc += c1
        thc += c2
    assert (dc, hc) == (tdc, thc)


def test_search_edge_rows(ctx):
    """Duplicate ids inside a row, empty rows, a self loop and the widest rows."""
    rng = np.random.default_rng(4)
    n, d, w = 700, 32, 256
    base = rng.integers(0, 4, size=(n, d)).astype(np.float32)  # many ties
    query = rng.integers(0, 4, size=(40, d)).astype(np.float32)
    deg = rng.integers(0, w + 1, size=n).astype(np.uint32)
    deg[:5] = 0
    deg[5:10] = w
    ids = rng.integers(0, n, size=(n, w)).astype(np.uint32)
    ids[:, 1] = ids[:, 0]  # duplicates
    ids[7, 3] = 7
    g = O.Graph(ids, np.zeros((n, w), np.float32), deg, 3)
    ctx.upload_base(base)
    ctx.upload_graph(ids, deg, 3)
    for L, entry in ((10, "rand"), (40, "rand"), (33, "centroid"), (200, "rand")):
        ctx.srand(11)
        res, dc, hc = ctx.search(query, L, 10, entry=entry)
        e, edc, ehc = O.search(base, query, g, L, O.Rand(11), entry=entry)
        assert np.array_equal(res, e), (L, entry)
        assert (dc, hc) == (edc, ehc)


def test_search_rejects_bad_args(ctx, kgraph20k):
    from weavess_gb300._lib import WeavessError
    base, query, g = kgraph20k
    ctx.upload_base(base)
    ctx.upload_graph(g.ids, g.deg, 0)
    with pytest.raises(WeavessError):
        ctx.search(query, 5, 10)  # L < K
    with pytest.raises(WeavessError):
        ctx.search(query, 20000, 10)  # L >= n
    bad = g.ids.copy()
    bad[0, 0] = 10 ** 6
    with pytest.raises(WeavessError):
        ctx.upload_graph(bad, np.full(g.n, 25, np.uint32), 0)  # deg > width
