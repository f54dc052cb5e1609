"""GPU HNSW / NSW routing (ROUTER_HNSW, ROUTER_NSW) against the reference:
result ids and DistCount / HopCount over the reference's own INDEX_HNSW
graphs (golden fixtures), and against the oracle on larger synthetic layered
graphs in the same file layout."""
import numpy as np
import pytest

import oracle as O
from golden_util import cases, load
from weavess_gb300 import datasets as ds

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from weavess_gb300 import Context
    return Context(0)


def _hnsw_cases(first="hnsw"):
    out = []
    for name in cases():
        f = load(name)
        for pi, steps in enumerate(f["pipelines"]):
            if steps[0] == first:
                out.append((name, pi))
    return out


@pytest.mark.parametrize("name,pi", _hnsw_cases("nsw"))
def test_nsw_index_matches_reference_golden(ctx, name, pi, tmp_path):
    """INIT_NSW graphs in the reference's INDEX_NSW file, read by the library,
    routed by ROUTER_NSW."""
    f = load(name)
    ctx.upload_base(f["base"])
    path = str(tmp_path / "g.nsw")
    f[f"p{pi}.nsw.words"].astype(np.uint32).tofile(path)
    ctx.load_graph(path, with_ep="nsw")
    for s in f["pipelines"][pi][1:]:
        kind, _, arg = s.partition(":")
        res, dc, hc = ctx.search_hnsw(f["query"], int(arg), 10, router="nsw")
        k = f"p{pi}.{kind}_{arg}"
        assert np.array_equal(res, f[k + ".res"]), (name, s)
        assert [dc, hc] == f[k + ".counts"].tolist(), (name, s)


@pytest.mark.parametrize("name,pi", _hnsw_cases())
def test_routes_match_reference_golden(ctx, name, pi, tmp_path):
    f = load(name)
    words = f[f"p{pi}.hnsw.words"]
    ctx.upload_base(f["base"])
    path = str(tmp_path / "g.hnsw")
    words.astype(np.uint32).tofile(path)
    ctx.load_graph(path, with_ep="hnsw")  # the reference's file, read by the library
    for s in f["pipelines"][pi][1:]:
        kind, _, arg = s.partition(":")
        router = kind[len("search_"):]
        res, dc, hc = ctx.search_hnsw(f["query"], int(arg), 10, router=router)
        k = f"p{pi}.{kind}_{arg}"
        assert np.array_equal(res, f[k + ".res"]), (name, s)
        assert [dc, hc] == f[k + ".counts"].tolist(), (name, s)


def layered_graph(base, m, m0, seed):
    """A hierarchical graph in the INDEX_HNSW file layout: levels drawn
    geometrically, every layer the m (layer 0: m0) nearest nodes of that
    layer (exact, numpy), the enterpoint on the top layer."""
    rng = np.random.default_rng(seed)
    n = base.shape[0]
    level = np.minimum(rng.geometric(1 - 1 / m, size=n) - 1, 6)
    top = int(level.max())
    ep = int(np.flatnonzero(level == top)[0])
    x = base.astype(np.float64)
    friends = [[None] * (level[v] + 1) for v in range(n)]
    for lv in range(top + 1):
        ids = np.flatnonzero(level >= lv)
        k = min(m0 if lv == 0 else m, len(ids) - 1)
        xs = x[ids]
        sq = (xs * xs).sum(1)
        for c0 in range(0, len(ids), 2048):
            blk = slice(c0, c0 + 2048)
            d2 = sq[blk, None] + sq[None, :] - 2 * xs[blk] @ xs.T
            d2[np.arange(d2.shape[0]), np.arange(c0, c0 + d2.shape[0])] = np.inf
            nn = np.argpartition(d2, k, axis=1)[:, :k]
            for r, row in enumerate(nn):
                friends[ids[c0 + r]][lv] = ids[row]
    words = [ep, top]
    for v in range(n):
        words += [v, level[v] + 1]
        for lv in range(level[v] + 1):
            words += [len(friends[v][lv])] + [int(t) for t in friends[v][lv]]
    return np.array(words, np.uint32)


@pytest.fixture(scope="module")
def layered20k():
    base, query = ds.int_mixture(20000, 128, 32, seed=21, n_query=300)
    return base, query, layered_graph(base, 8, 16, seed=3)


@pytest.mark.parametrize("router", ["hnsw", "nsw"])
@pytest.mark.parametrize("L", [10, 64, 200])
def test_routes_match_oracle_20k(ctx, layered20k, router, L):
    base, query, words = layered20k
    ctx.upload_base(base)
    ctx.load_hnsw(words)
    res, dist, dc, hc = ctx.search_hnsw(query, L, 10, router=router, return_dist=True)
    eres, edc, ehc = O.search_hnsw(base, query, words, L, router=router)
    assert np.array_equal(res, eres)
    assert (dc, hc) == (edc, ehc)
    # distances are the exact FP32 ones of the returned ids, ascending
    ex = ((base[res.astype(np.int64)].astype(np.float64) - query[:, None, :]) ** 2).sum(-1)
    assert np.allclose(dist, ex, rtol=0, atol=0)
    assert np.all(np.diff(dist, axis=1) >= 0)


def test_rejects_bad_graphs(ctx):
    from weavess_gb300._lib import WeavessError
    base, _ = ds.int_mixture(100, 8, 2, seed=1, n_query=1)
    ctx.upload_base(base)
    with pytest.raises(WeavessError):
        ctx.load_hnsw(np.array([0, 0, 0, 1, 1, 5], np.uint32))  # truncated: 99 nodes missing
    words = [0, 0] + sum(([v, 1, 1, (v + 1) % 100] for v in range(100)), [])
    bad = np.array(words, np.uint32)
    bad[5] = 100  # an id >= n
    with pytest.raises(WeavessError):
        ctx.load_hnsw(bad)
    ctx.load_hnsw(np.array(words, np.uint32))  # a ring: valid
    with pytest.raises(WeavessError):
        ctx.search_hnsw(base[:2], 5, 10)  # L < K


def test_index_info_over_the_layers(ctx, layered20k):
    """print_index_info for INDEX_HNSW: layer-0 degrees and quality, conn by a
    walk over every layer from the enterpoint."""
    from test_graph_io_gpu import host_quality
    base, query, words = layered20k
    n = base.shape[0]
    ctx.upload_base(base)
    ctx.load_hnsw(words)
    # parse the words on the host
    ep, p = int(words[0]), 2
    fr = [None] * n
    for _ in range(n):
        v, t = int(words[p]), int(words[p + 1])
        p += 2
        fr[v] = []
        for _l in range(t):
            k = int(words[p])
            fr[v].append(words[p + 1:p + 1 + k].astype(np.int64))
            p += 1 + k
    deg0 = np.array([len(f[0]) for f in fr])
    w0 = int(deg0.max())
    ids0 = np.zeros((n, w0), np.int64)
    for v in range(n):
        ids0[v, :deg0[v]] = fr[v][0]
    # conn: passes from the enterpoint, then the smallest unreached id
    seen = np.zeros(n, bool)
    conn, root = 0, ep
    while True:
        conn += 1
        stack = [root]
        seen[root] = True
        while stack:
            u = stack.pop()
            for lay in fr[u]:
                for x in lay:
                    if not seen[x]:
                        seen[x] = True
                        stack.append(int(x))
        left = np.nonzero(~seen)[0]
        if left.size == 0:
            break
        root = int(left[0])
    exact = ds.groundtruth_fp64(base, base, 11)
    info = ctx.index_info(use_ep="hnsw", exact_ids=exact)
    assert info["max_out"] == deg0.max() and info["min_out"] == deg0.min()
    assert abs(info["avg_out"] - deg0.mean()) < 1e-9
    assert info["conn"] == conn
    assert info["quality"] == host_quality(ids0, deg0, exact)
