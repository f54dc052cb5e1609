"""Low-precision candidate distances (bf16, fp8 e4m3 + per-row scale) with an
exact FP32 rerank: error against FP64, exact returned distances, and bf16 on
integer data being lossless."""
import numpy as np
import pytest

import oracle as O
from weavess_gb300 import datasets as ds

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def setup():
    from weavess_gb300 import Context
    base, query = ds.int_mixture(20000, 128, 32, seed=31, n_query=200)
    ctx = Context(0)
    ctx.upload_base(base)
    ctx.srand(1)
    ctx.init_random(12)
    ctx.nnd_refine(12, 32, 48, 6, 64)
    ctx.vamana_refine(48, 32, 1.2, 0)
    ctx.load_built_graph()
    return ctx, base, query


def test_bf16_is_lossless_on_integer_data(setup):
    ctx, base, query = setup
    ctx.set_precision("fp32")
    ctx.srand(3)
    r32, dc32, hc32 = ctx.search(query, 64, 10)
    ctx.set_precision("bf16", rerank=0)
    ctx.srand(3)
    r16, dc16, hc16 = ctx.search(query, 64, 10)
    ctx.set_precision("fp32")
    assert np.array_equal(r32, r16)
    assert hc16 == hc32 and dc16 == dc32 + 64 * query.shape[0]  # + the rerank


@pytest.mark.parametrize("storage", ["bf16", "fp8"])
def test_candidate_distance_error_vs_fp64(setup, storage):
    ctx, base, query = setup
    rng = np.random.default_rng(0)
    ids = rng.integers(0, base.shape[0], size=(query.shape[0], 64)).astype(np.uint32)
    exact = ((query[:, None, :].astype(np.float64) - base[ids].astype(np.float64)) ** 2).sum(2)
    ctx.set_precision(storage)
    got = ctx.candidate_distances(query, ids).astype(np.float64)
    ctx.set_precision("fp32")
    rel = np.abs(got - exact) / np.maximum(exact, 1.0)
    if storage == "bf16":
        assert rel.max() < 1e-6  # integers up to 255 are exact in bf16
    else:
        assert rel.mean() < 0.02 and rel.max() < 0.1, (rel.mean(), rel.max())


@pytest.mark.parametrize("storage", ["bf16", "fp8"])
def test_rerank_returns_exact_fp32_distances(setup, storage):
    ctx, base, query = setup
    ctx.set_precision(storage, rerank=0)
    ctx.srand(5)
    res, _, _, dist = ctx.search(query, 80, 10, return_dist=True)
    ctx.set_precision("fp32")
    exact = O.l2_rows(np.repeat(query, 10, axis=0), base[res.reshape(-1)]).reshape(res.shape)
    assert np.array_equal(dist.view(np.uint32), exact.view(np.uint32))
    assert np.all(np.diff(dist, axis=1) >= 0)


def test_fp8_recall_close_to_plain(setup):
    from weavess_gb300.datasets import groundtruth_fp64, recall_at
    ctx, base, query = setup
    gt = groundtruth_fp64(base, query, 10)
    ctx.srand(7)
    r32, _, _ = ctx.search(query, 64, 10)
    ctx.set_precision("fp8", rerank=0)
    ctx.srand(7)
    r8, _, _ = ctx.search(query, 64, 10)
    ctx.set_precision("fp32")
    assert recall_at(r8, gt) >= recall_at(r32, gt) - 0.02


def test_real_valued_bf16_error(setup):
    from weavess_gb300 import Context
    base, query = ds.unit_mixture(5000, 96, 40, seed=8, n_query=100)
    c2 = Context(0)
    c2.upload_base(base)
    rng = np.random.default_rng(1)
    ids = rng.integers(0, 5000, size=(100, 32)).astype(np.uint32)
    exact = ((query[:, None, :].astype(np.float64) - base[ids].astype(np.float64)) ** 2).sum(2)
    for storage, tol in (("bf16", 0.02), ("fp8", 0.15)):
        c2.set_precision(storage)
        got = c2.candidate_distances(query, ids).astype(np.float64)
        err = np.abs(got - exact)
        assert err.max() / exact.mean() < tol, (storage, err.max(), exact.mean())
