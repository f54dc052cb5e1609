"""wv_search_noalloc: the allocation-free search, for callers that cannot call
cudaMalloc (their GPU memory is owned by another allocator, or cudaMalloc
would stall a latency-critical thread).  Called through the C ABI with
caller-owned device buffers, it must return exactly what the existing
wv_search_device returns, on two calls in a row (its fixed scratch array is
reused, so the second call checks that the first left nothing behind).
This file is collected last on purpose."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kind", ["int", "unit"])
def test_noalloc_search_matches_search_device(kind):
    """Integer data (any summation order exact) and real-valued unit
    vectors (distances folded in the reference's order)."""
    import torch
    from weavess_gb300 import Context, datasets as ds

    if kind == "int":
        base, query = ds.int_mixture(6000, 64, 8, seed=17, n_query=300)
    else:
        base, query = ds.unit_mixture(6000, 96, 12, seed=17, n_query=300)
    ctx = Context(0)
    ctx.upload_base(base)
    ctx.srand(1)
    ctx.init_random(12)
    ctx.nnd_refine(12, 24, 40, 5, 40)
    ctx.load_built_graph()
    ids, _, deg, _ = ctx.get_graph()
    L, K = 64, 10
    seeds = ctx.draw_seeds(query.shape[0], L, "rand")
    dev = torch.device("cuda:0")
    d_base = torch.from_numpy(base).to(dev)
    d_ids = torch.from_numpy(ids.astype(np.int32)).to(dev)
    d_deg = torch.from_numpy(deg.astype(np.int32)).to(dev)
    d_q = torch.from_numpy(query).to(dev)
    d_seeds = torch.from_numpy(seeds.astype(np.int32)).to(dev)
    nq = query.shape[0]
    # the existing entry point
    ref_ids = torch.zeros((nq, K), dtype=torch.int32, device=dev)
    ref_dist = torch.zeros((nq, K), dtype=torch.float32, device=dev)
    ctx.search_device(d_q.data_ptr(), nq, L, K, d_seeds.data_ptr(), ref_ids.data_ptr(), ref_dist.data_ptr())
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):
        out_ids = torch.full((nq, K), -1, dtype=torch.int32, device=dev)
        out_dist = torch.full((nq, K), -1.0, dtype=torch.float32, device=dev)
        rc = ctx.L.wv_search_noalloc(C.c_void_p(d_base.data_ptr()), base.shape[0], base.shape[1],
                                     C.c_void_p(d_ids.data_ptr()), C.c_void_p(d_deg.data_ptr()), ids.shape[1],
                                     C.c_void_p(d_q.data_ptr()), nq, C.c_void_p(d_seeds.data_ptr()), L, K,
                                     C.c_void_p(out_ids.data_ptr()), C.c_void_p(out_dist.data_ptr()),
                                     C.c_void_p(stream))
        assert rc == 0, (call, rc)
        torch.cuda.synchronize()
        assert torch.equal(out_ids, ref_ids), call
        assert torch.equal(out_dist, ref_dist), call
    # sizes beyond the fixed scratch or the search limits are refused
    assert ctx.L.wv_search_noalloc(C.c_void_p(d_base.data_ptr()), base.shape[0], base.shape[1],
                                   C.c_void_p(d_ids.data_ptr()), C.c_void_p(d_deg.data_ptr()), ids.shape[1],
                                   C.c_void_p(d_q.data_ptr()), nq, C.c_void_p(d_seeds.data_ptr()), 5000, K,
                                   C.c_void_p(out_ids.data_ptr()), None, C.c_void_p(stream)) != 0
    # a base too large for the fixed scratch (n / 16 words per warp slot,
    # four slots at least) is refused before anything is launched: n is
    # only compared, the buffers are never read
    n_big = 67_200_000
    assert ctx.L.wv_search_noalloc(C.c_void_p(d_base.data_ptr()), n_big, base.shape[1],
                                   C.c_void_p(d_ids.data_ptr()), C.c_void_p(d_deg.data_ptr()), ids.shape[1],
                                   C.c_void_p(d_q.data_ptr()), nq, C.c_void_p(d_seeds.data_ptr()), L, K,
                                   C.c_void_p(out_ids.data_ptr()), None, C.c_void_p(stream)) == 5  # WV_ERR_LIMIT
