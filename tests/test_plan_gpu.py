"""Batched search plans (wv_plan_*): uneven L and K in one launch, captured as
a CUDA graph and replayed, tuned launch shapes -- results equal to the
per-call entry points (and so to the reference) on the same rand stream."""
import numpy as np
import pytest

import oracle as O
from weavess_gb300 import datasets as ds
from weavess_gb300._lib import WeavessError

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def setup():
    import torch
    from weavess_gb300 import Context
    base, query = ds.int_mixture(20000, 128, 32, seed=21, n_query=400)
    ctx = Context(0)
    ctx.upload_base(base)
    ctx.srand(1)
    ctx.init_random(10)
    ctx.nnd_refine(10, 20, 40, 6, 60)
    ctx.load_built_graph()
    rng = np.random.default_rng(4)
    nq = query.shape[0]
    K = rng.choice([1, 10, 50, 100], size=nq).astype(np.uint32)
    L = np.maximum(K, rng.integers(10, 501, size=nq)).astype(np.uint32)
    dev = torch.device("cuda:0")
    t = {"q": torch.from_numpy(query).to(dev),
         "L": torch.from_numpy(L.astype(np.int32)).to(dev),
         "K": torch.from_numpy(K.astype(np.int32)).to(dev),
         "out": torch.full((nq, 100), -1, dtype=torch.int32, device=dev)}
    return ctx, base, query, L, K, t


def rand_plan(ctx, t, nq):
    return ctx.plan(nq, 100, t["q"].data_ptr(), t["out"].data_ptr(), L_max=500, mode="rand",
                    d_L=t["L"].data_ptr(), d_K=t["K"].data_ptr(), out_stride=100)


def check_rows(out, ref, K, n):
    for i in range(n):
        assert np.array_equal(out[i, :K[i]], ref[i, :K[i]]), i


def test_plan_matches_search_batch(setup):
    ctx, base, query, L, K, t = setup
    nq = query.shape[0]
    ctx.srand(9)
    ref, dc, hc = ctx.search_batch(query, L, K)
    plan = rand_plan(ctx, t, nq)
    ctx.srand(9)
    t["out"].fill_(-1)
    plan.run(nq)
    got_counts = plan.wait()
    out = t["out"].cpu().numpy().view(np.uint32)
    check_rows(out, ref, K, nq)
    assert got_counts == (dc, hc)
    plan.close()


def test_plan_replays_smaller_batches(setup):
    ctx, base, query, L, K, t = setup
    plan = rand_plan(ctx, t, query.shape[0])
    ctx.srand(31)
    refs = []
    for nq in (400, 150, 7):
        refs.append(ctx.search_batch(query[:nq], L[:nq], K[:nq]))
    ctx.srand(31)
    for nq, (ref, dc, hc) in zip((400, 150, 7), refs):
        t["out"].fill_(-1)
        plan.run(nq)
        assert plan.wait() == (dc, hc)
        out = t["out"].cpu().numpy().view(np.uint32)
        check_rows(out, ref, K, nq)
        assert np.all(out[nq:] == 0xFFFFFFFF)  # rows past nq untouched
    plan.close()


def test_plan_tune_keeps_results(setup):
    ctx, base, query, L, K, t = setup
    nq = query.shape[0]
    plan = rand_plan(ctx, t, nq)
    rep = plan.tune(nq)
    assert len(rep["tried"]) >= 4 and rep["chosen"] is not None
    assert {s["warps_per_block"] for s in rep["tried"]} >= {1, 2, 4, 8}
    assert plan.shape()["warps_per_block"] == rep["chosen"]["warps_per_block"]
    assert plan.shape()["hash_words"] == rep["chosen"]["hash_words"]
    ctx.srand(12)
    ref, dc, hc = ctx.search_batch(query, L, K)
    ctx.srand(12)
    plan.run(nq)
    assert plan.wait() == (dc, hc)
    check_rows(t["out"].cpu().numpy().view(np.uint32), ref, K, nq)
    plan.close()


@pytest.mark.parametrize("shape", [dict(warps_per_block=1, wide_hash=True), dict(warps_per_block=8, wide_hash=False),
                                   dict(warps_per_block=2, hash_words=4096, wide_hash=True)])
def test_plan_shapes_agree(setup, shape):
    """Pinned launch shapes, 16-bit and 32-bit visited-hash entries included,
    give the per-call results and counters."""
    ctx, base, query, L, K, t = setup
    nq = query.shape[0]
    plan = rand_plan(ctx, t, nq)
    plan.set_shape(**shape)
    got = plan.shape()
    assert got["warps_per_block"] == shape["warps_per_block"] and got["wide_hash"] == int(shape["wide_hash"])
    ctx.srand(17)
    ref, dc, hc = ctx.search_batch(query, L, K)
    ctx.srand(17)
    plan.run(nq)
    assert plan.wait() == (dc, hc)
    check_rows(t["out"].cpu().numpy().view(np.uint32), ref, K, nq)
    plan.close()


def test_plan_caller_seeds_match_oracle(setup):
    import torch
    ctx, base, query, L, K, t = setup
    nq, Lm = 64, 200
    r = O.Rand(3)
    g = O.Graph(*[np.asarray(x) for x in ctx.get_graph()[:3]], 0)
    seeds = O.search_seeds(base.shape[0], nq, g, Lm, r, entry="rand")
    ds_ = torch.from_numpy(seeds.astype(np.int32)).cuda()
    out = torch.full((nq, 10), -1, dtype=torch.int32, device="cuda")
    plan = ctx.plan(nq, 10, t["q"].data_ptr(), out.data_ptr(), L_max=Lm, mode="seeds", d_seeds=ds_.data_ptr())
    plan.run(nq)
    dc, hc = plan.wait()
    exp, edc, ehc = O.search(base, query[:nq], g, Lm, O.Rand(3), K=10)
    assert np.array_equal(out.cpu().numpy().view(np.uint32), exp)
    assert (dc, hc) == (edc, ehc)
    plan.close()


def test_plan_learned_matches_search_learned(setup):
    import torch
    ctx, base, query, L, K, t = setup
    _, train = ds.int_mixture(0, 128, 32, seed=21, n_query=8000, query_stream=3)
    ctx.learn_fit(train, clusters=16, L_trace=128, L_max=128, list_len=128, epochs=4, batch=512)
    nq = query.shape[0]
    ref, dc, hc = ctx.search_learned(query, 10)
    out = torch.full((nq, 10), -1, dtype=torch.int32, device="cuda")
    plan = ctx.plan(nq, 10, t["q"].data_ptr(), out.data_ptr(), mode="learned")
    plan.run(nq)
    assert plan.wait() == (dc, hc)
    assert np.array_equal(out.cpu().numpy().view(np.uint32), ref)
    plan.tune(nq)
    plan.run(nq)
    assert plan.wait() == (dc, hc)
    assert np.array_equal(out.cpu().numpy().view(np.uint32), ref)
    # the plan refuses to run once the model changed
    ctx.learn_set_margin(3.0)
    with pytest.raises(WeavessError):
        plan.run(nq)
    plan.close()


def test_plan_rejects_out_of_range_beams(setup):
    """Per-query L above the plan's L_max, sitting in device memory the host
    never reads, is caught by the kernels' own checks and reported."""
    import torch
    ctx, base, query, L, K, t = setup
    nq = 32
    bad = torch.from_numpy(np.full(nq, 600, np.int32)).cuda()
    kk = torch.from_numpy(np.full(nq, 10, np.int32)).cuda()
    out = torch.full((nq, 10), -1, dtype=torch.int32, device="cuda")
    plan = ctx.plan(nq, 10, t["q"].data_ptr(), out.data_ptr(), L_max=500, mode="rand", d_L=bad.data_ptr(),
                    d_K=kk.data_ptr())
    plan.run(nq)
    with pytest.raises(WeavessError):
        plan.wait()
    assert np.all(out.cpu().numpy() == -1)
    plan.close()
