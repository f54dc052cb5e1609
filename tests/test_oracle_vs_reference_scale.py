"""The oracle against the unmodified reference at a larger size than the
committed fixtures: 10,000 x 64 integer mixture, the reference driver
(oracle/_ref, built from the reference sources) run live.  Runs where the
driver exists (the fixture machine); skipped elsewhere."""
import os
import subprocess

import numpy as np
import pytest

import oracle as O
from golden_util import rows_equal
from weavess_gb300 import datasets as ds

pytestmark = pytest.mark.skipif(not os.path.exists(O.REF_DRIVER), reason="reference driver not built")


def test_kgraph_nsg_ssg_and_searches_at_10k(tmp_path):
    base, query = ds.int_mixture(10000, 64, 24, seed=13, n_query=100)
    gt = ds.groundtruth_fp64(base, query, 20)
    bf, qf, gf = (str(tmp_path / x) for x in ("b.fvecs", "q.fvecs", "g.ivecs"))
    ds.write_vecs(bf, base)
    ds.write_vecs(qf, query)
    ds.write_vecs(gf, gt)
    p = dict(S=12, K=24, L=48, ITER=6, R=60, L_refine=48, R_refine=24, C_refine=300, A=60, n_try=6)
    kv = [f"{k}={v}" for k, v in p.items()]
    runs = {
        "a": ["init_random", "nndescent", "nsg", "load:nsg", "search_centroid:48", "search_rand:64"],
        "b": ["init_random", "nndescent", "ssg", "load:ssg", "search_rand:40"],
    }
    for tag, steps in runs.items():
        prefix = str(tmp_path / tag)
        subprocess.run([O.REF_DRIVER, bf, qf, gf, prefix] + kv + ["--"] + steps, check=True, capture_output=True,
                       timeout=900)
        r = O.Rand(1)
        g = O.nndescent(base, O.init_random(base, p["S"], r), p["S"], p["K"], p["L"], p["ITER"], p["R"], r)
        want = O.read_graph_dump(prefix + ".nnd.bin")
        assert rows_equal(g.ids, g.dist, g.deg, want.ids, want.dist, want.deg) == 0
        if tag == "a":
            g = O.nsg(base, g, p["L_refine"], p["R_refine"], p["C_refine"], r)
            want = O.read_graph_dump(prefix + ".nsg.bin")
            assert want.ep == g.ep
            searches = [("centroid", 48), ("rand", 64)]
        else:
            g = O.ssg(base, g, p["L_refine"], p["R_refine"], float(p["A"]), p["n_try"], r)
            want = O.read_graph_dump(prefix + ".ssg.bin")
            eps = np.fromfile(prefix + ".ssgeps.bin", np.uint32)[1:]
            assert np.array_equal(g.eps, eps)
            searches = [("rand", 40)]
        assert rows_equal(g.ids, g.dist, g.deg, want.ids, want.dist, want.deg) == 0
        for entry, L in searches:
            res, dc, hc = O.search(base, query, g, L, r, entry=entry)
            wres, wdc, whc = O.read_search_dump(f"{prefix}.search_{entry}_{L}.bin")
            assert np.array_equal(res, wres) and (dc, hc) == (wdc, whc), (tag, entry, L)


def test_init_kdt_and_kdt_search_at_10k(tmp_path):
    base, query = ds.int_mixture(10000, 64, 24, seed=17, n_query=100)
    gt = ds.groundtruth_fp64(base, query, 20)
    bf, qf, gf = (str(tmp_path / x) for x in ("b.fvecs", "q.fvecs", "g.ivecs"))
    ds.write_vecs(bf, base)
    ds.write_vecs(qf, query)
    ds.write_vecs(gf, gt)
    p = dict(nTrees=6, mLevel=5, K=25, S=10, L=40, ITER=4, R=60)
    prefix = str(tmp_path / "k")
    subprocess.run([O.REF_DRIVER, bf, qf, gf, prefix] + [f"{k}={v}" for k, v in p.items()] +
                   ["--", "init_kdt", "efanna", "load:efanna", "search_kdt:48"], check=True, capture_output=True,
                   timeout=900)
    r = O.Rand(1)
    g, forest = O.init_kdt(base, p["nTrees"], p["K"], p["mLevel"], r)
    lf = np.fromfile(prefix + ".kdtleaf.bin", np.uint32)[2:].reshape(p["nTrees"], -1)
    assert np.array_equal(lf, forest.leaf)
    want = O.read_graph_dump(prefix + ".initkdt.bin")
    assert rows_equal(g.ids, g.dist, g.deg, want.ids, want.dist, want.deg) == 0
    g = O.efanna(base, g, p["S"], p["K"], p["L"], p["ITER"], p["R"], r)
    want = O.read_graph_dump(prefix + ".efanna.bin")
    assert rows_equal(g.ids, g.dist, g.deg, want.ids, want.dist, want.deg) == 0
    res, dc, hc = O.search_kdt(base, query, g, forest, 48, r)
    wres, wdc, whc = O.read_search_dump(prefix + ".search_kdt_48.bin")
    assert np.array_equal(res, wres) and (dc, hc) == (wdc, whc)
