"""Graph files (the reference's per-node format, IndexBuilder::save_graph /
load_graph) and print_index_info statistics against host computations."""
import os
import struct

import numpy as np
import pytest

import oracle as O
from weavess_gb300 import datasets as ds

pytestmark = pytest.mark.gpu


def write_reference_format(path, ids, deg, ep=None):
    """The byte layout builder.cpp:918-1089 writes: [ep] then per node GK + ids."""
    with open(path, "wb") as f:
        if ep is not None:
            f.write(struct.pack("<I", ep))
        for i in range(ids.shape[0]):
            f.write(struct.pack("<I", int(deg[i])))
            f.write(ids[i, :deg[i]].astype("<u4").tobytes())


def host_conn(ids, deg, root):
    """DFS restarts from `root`, then from the smallest unreached id."""
    n = ids.shape[0]
    seen = np.zeros(n, bool)
    conn = 0
    while True:
        conn += 1
        stack = [root]
        seen[root] = True
        while stack:
            u = stack.pop()
            for v in ids[u, :deg[u]]:
                if not seen[v]:
                    seen[v] = True
                    stack.append(int(v))
        left = np.nonzero(~seen)[0]
        if left.size == 0:
            return conn
        root = int(left[0])


def host_quality(ids, deg, exact):
    """graph_quality (builder.cpp:716-775): per node hits / min(10, degree,
    exact-list length) in FP32, summed in FP32 in node order, over n."""
    s = np.float32(0)
    for i in range(ids.shape[0]):
        v = list(exact[i])
        if v and v[0] == i:
            v = v[1:]
        row = set(ids[i, :deg[i]].tolist())
        hits = sum(1 for j in range(min(10, len(v))) if v[j] in row)
        den = min(10, int(deg[i]), len(v))
        s = np.float32(s + (np.float32(hits) / np.float32(den) if den else np.float32("nan")))
    return float(np.float32(s / np.float32(ids.shape[0])))


@pytest.fixture(scope="module")
def built():
    from weavess_gb300 import Context
    base, _ = ds.int_mixture(6000, 32, 12, seed=5, n_query=0)
    ctx = Context(0)
    ctx.upload_base(base)
    ctx.srand(1)
    ctx.init_random(10)
    ctx.nnd_refine(10, 16, 24, 5, 40)
    ctx.nsg_refine(24, 16, 200)
    ctx.load_built_graph()
    ids, _, deg, ep = ctx.get_graph()
    return ctx, base, np.asarray(ids), np.asarray(deg), int(ep)


def test_save_is_byte_compatible(built, tmp_path):
    ctx, base, ids, deg, ep = built
    for with_ep in (False, True):
        a, b = str(tmp_path / f"ours{with_ep}.graph"), str(tmp_path / f"ref{with_ep}.graph")
        ctx.save_graph(a, with_ep=with_ep)
        write_reference_format(b, ids, deg, ep if with_ep else None)
        assert open(a, "rb").read() == open(b, "rb").read()


def test_load_round_trip_and_search(built, tmp_path):
    ctx, base, ids, deg, ep = built
    p = str(tmp_path / "g.graph")
    write_reference_format(p, ids, deg, ep)
    ctx.load_graph(p, with_ep=True)
    q = base[:50] + 1.0
    ctx.srand(3)
    got, dc, hc = ctx.search(q, 40, 10)
    g = O.Graph(ids, np.zeros(ids.shape, np.float32), deg, ep)
    exp, edc, ehc = O.search(base, q, g, 40, O.Rand(3))
    assert np.array_equal(got, exp) and (dc, hc) == (edc, ehc)


def test_index_info_matches_host(built, tmp_path):
    ctx, base, ids, deg, ep = built
    ctx.load_built_graph()
    exact = ds.groundtruth_fp64(base, base, 11)  # includes the node itself first
    info = ctx.index_info(use_ep=True, exact_ids=exact)
    assert info["max_out"] == deg.max() and info["min_out"] == deg.min()
    assert abs(info["avg_out"] - deg.mean()) < 1e-9
    assert info["conn"] == host_conn(ids, deg, ep)
    assert info["quality"] == host_quality(ids, deg, exact)
    # a graph cut in two pieces needs two traversals from node 0
    cut, deg = ids.copy(), deg.copy()
    half = ids.shape[0] // 2
    for i in range(ids.shape[0]):
        keep = [v for v in ids[i, :deg[i]] if (v < half) == (i < half)] or [i]
        cut[i, :len(keep)] = keep
        cut[i, len(keep):] = 0
        deg[i] = len(keep)
    ctx.upload_graph(cut, deg.copy(), 0)
    assert ctx.index_info(use_ep=False)["conn"] == host_conn(cut, deg, 0)
