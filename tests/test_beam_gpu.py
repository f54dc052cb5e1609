"""The throughput form of the route search (wv_set_search_expansion(E > 0),
weavess_gb300/csrc/wv_beam.cu): tensor-core row distances and E parents per
step.

On integer data every distance path of the kernel is exact, so the kernel
must equal its plain-Python statement (tests/beam_model.py) id for id,
distance for distance, DistCount / HopCount included, for every distance path
(FP32 rows of integer data on the tensor cores at d = 128, bf16 rows at
d = 128 and d = 96, the warp-cooperative rows at other d) and E = 1, 2, 4.
On real-valued data the bf16 candidates carry the query as a hi + lo bf16
pair: distances after the FP32 rerank are the exact FP32 values, and recall
stays with the exact traversal's."""
import numpy as np
import pytest

import oracle as O
from beam_model import beam_search, int_dist
from weavess_gb300 import datasets as ds

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from weavess_gb300 import Context
    c = Context(0)
    yield c
    c.set_expansion(0)


_graphs = {}


def graph_for(ctx, d):
    """A KNN graph (GPU NN-Descent) on a 6,000-point integer mixture."""
    if d not in _graphs:
        base, query = ds.int_mixture(6000, d, 16, seed=40 + d, n_query=120)
        ctx.upload_base(base)
        ctx.set_precision("fp32")
        ctx.srand(1)
        ctx.init_random(12)
        ctx.nnd_refine(12, 24, 40, 6, 60)
        ids, _, deg, _ = ctx.get_graph()
        _graphs[d] = (base, query, ids, deg)
    base, query, ids, deg = _graphs[d]
    ctx.upload_base(base)
    ctx.upload_graph(ids, deg, 0)
    return base, query, ids, deg


@pytest.mark.parametrize("d,storage", [(128, "fp32"), (128, "bf16"), (96, "bf16"), (64, "fp32"), (64, "bf16")])
@pytest.mark.parametrize("E", [1, 2, 4])
def test_throughput_form_matches_its_statement(ctx, d, storage, E):
    base, query, ids, deg = graph_for(ctx, d)
    ctx.set_precision(storage)
    ctx.set_expansion(E)
    try:
        for L in (16, 64, 200):
            ctx.srand(7 + L)
            seeds = ctx.draw_seeds(query.shape[0], L, "rand")
            res, dc, hc, dist = ctx.search(query, L, 10, entry=seeds, return_dist=True)
            # bf16 candidates of integer data are exact: re-ranked only above d = 128
            rerank = L if (storage != "fp32" and d > 128) else 0
            eres, edist, edc, ehc = beam_search(base, query, ids, deg, seeds, L, 10, E, rerank=rerank,
                                                exact=int_dist)
            assert int(np.sum(np.any(res != eres, axis=1))) == 0, (L, "queries whose ids differ")
            assert np.array_equal(dist.view(np.uint32), edist.view(np.uint32)), L
            assert (dc, hc) == (edc, ehc), L
    finally:
        ctx.set_expansion(0)
        ctx.set_precision("fp32")


def test_throughput_form_batch_and_plan(ctx):
    """Per-query L and K in one launch (widest first), and the captured plan
    in rand mode, equal the statement query by query."""
    import torch
    base, query, ids, deg = graph_for(ctx, 128)
    ctx.set_precision("bf16")
    ctx.set_expansion(2)
    try:
        rng = np.random.default_rng(5)
        nq = query.shape[0]
        K = rng.choice([1, 10, 50], size=nq).astype(np.uint32)
        L = np.maximum(K, rng.integers(10, 300, size=nq)).astype(np.uint32)
        ctx.srand(21)
        out, dc, hc = ctx.search_batch(query, L, K)
        r = O.Rand(21)
        tdc = thc = 0
        for i in range(nq):
            s = O.search_seeds(base.shape[0], 1, O.Graph(ids, np.zeros(ids.shape, np.float32), deg, 0), int(L[i]), r)
            e, _, c1, c2 = beam_search(base, query[i:i + 1], ids, deg, s, int(L[i]), int(K[i]), 2)
            assert np.array_equal(out[i, :K[i]], e[0]), i
            tdc += c1
            thc += c2
        assert (dc, hc) == (tdc, thc)
        # the plan (seeds drawn on the device from one host rand() per query)
        dq = torch.from_numpy(query).cuda()
        dout = torch.zeros((nq, 10), dtype=torch.int32, device="cuda")
        plan = ctx.plan(nq, 10, dq.data_ptr(), dout.data_ptr(), L_max=64, mode="rand")
        ctx.srand(33)
        plan.run(nq)
        pdc, phc = plan.wait()
        got = dout.cpu().numpy().view(np.uint32)
        ctx.srand(33)
        seeds = ctx.draw_seeds(nq, 64, "rand")
        e, _, edc, ehc = beam_search(base, query, ids, deg, seeds, 64, 10, 2)
        assert np.array_equal(got, e)
        assert (pdc, phc) == (edc, ehc)
        plan.close()
    finally:
        ctx.set_expansion(0)
        ctx.set_precision("fp32")


def test_throughput_form_real_valued(ctx):
    """Unit vectors, bf16 candidates with the hi + lo query: the reranked
    distances are the exact FP32 distances of the returned ids, and recall
    stays within 0.02 of the exact traversal at the same beam."""
    base, query = ds.unit_mixture(8000, 96, 40, seed=3, n_query=200)
    ctx.upload_base(base)
    ctx.set_precision("fp32")
    ctx.srand(1)
    ctx.init_random(12)
    ctx.nnd_refine(12, 24, 40, 6, 60)
    ctx.load_built_graph()
    from weavess_gb300.groundtruth import knn_fp64
    gt = knn_fp64(base, query, k=10)

    def recall(res):
        return float(np.mean([len(set(a.tolist()) & set(b.tolist())) / 10 for a, b in zip(res, gt)]))

    ctx.srand(9)
    seeds = ctx.draw_seeds(query.shape[0], 64, "rand")
    exact, _, _ = ctx.search(query, 64, 10, entry=seeds)
    ctx.set_precision("bf16")
    for E in (1, 2, 4):
        ctx.set_expansion(E)
        res, dc, hc, dist = ctx.search(query, 64, 10, entry=seeds, return_dist=True)
        want = np.stack([O.l2_rows(base[res[i]], np.repeat(query[i:i + 1], 10, 0)) for i in range(len(res))])
        assert np.array_equal(dist.view(np.uint32), want.view(np.uint32)), E
        assert recall(res) >= recall(exact) - 0.02, E
    ctx.set_expansion(0)
    ctx.set_precision("fp32")


def test_expansion_setting_is_checked(ctx):
    from weavess_gb300._lib import WeavessError
    with pytest.raises(WeavessError):
        ctx.set_expansion(5)
    ctx.set_expansion(0)


@pytest.mark.parametrize("kind", ["int128_bf16", "unit96_bf16", "int64_fp32"])
@pytest.mark.parametrize("wpb,qw", [(2, 2), (4, 4)])
def test_query_warps_do_not_change_results(ctx, kind, wpb, qw):
    """2 or 4 warps sharing each query's distance passes (seeds, fresh rows,
    the FP32 rerank) return the ids, distances and counters of one warp per
    query, mixed beams included."""
    import torch
    if kind == "int128_bf16":
        base, query, ids, deg = graph_for(ctx, 128)
        storage = "bf16"
    elif kind == "int64_fp32":
        base, query, ids, deg = graph_for(ctx, 64)
        storage = "fp32"
    else:
        base, query = ds.unit_mixture(6000, 96, 24, seed=8, n_query=150)
        ctx.upload_base(base)
        ctx.set_precision("fp32")
        ctx.srand(1)
        ctx.init_random(12)
        ctx.nnd_refine(12, 24, 40, 5, 40)
        ctx.load_built_graph()
        storage = "bf16"  # real-valued: the final pool is re-ranked in FP32
    ctx.set_precision(storage)
    ctx.set_expansion(2)
    try:
        nq = query.shape[0]
        rng = np.random.default_rng(2)
        L = rng.integers(10, 200, size=nq).astype(np.int32)
        dq = torch.from_numpy(query).cuda()
        dL = torch.from_numpy(L).cuda()
        dout = torch.zeros((nq, 10), dtype=torch.int32, device="cuda")
        ddist = torch.zeros((nq, 10), dtype=torch.float32, device="cuda")
        plan = ctx.plan(nq, 10, dq.data_ptr(), dout.data_ptr(), L_max=200, mode="rand", d_L=dL.data_ptr(),
                        d_out_dist=ddist.data_ptr())
        res = []
        for shape in ((1, 1), (wpb, qw)):
            plan.set_shape(shape[0], 0, False, shape[1])
            assert plan.shape()["query_warps"] == shape[1]
            ctx.srand(33)
            plan.run(nq)
            counters = plan.wait()
            res.append((dout.cpu().numpy().copy(), ddist.cpu().numpy().copy(), counters))
        plan.close()
        assert np.array_equal(res[0][0], res[1][0])
        assert np.array_equal(res[0][1].view(np.uint32), res[1][1].view(np.uint32))
        assert res[0][2] == res[1][2]
    finally:
        ctx.set_expansion(0)
        ctx.set_precision("fp32")
