"""The C++ builder facade (include/weavess_gpu_builder.hpp) driven the way the
reference's test/main.cpp drives weavess::IndexBuilder: a native program
(tests/native/builder_pipeline.cpp) runs whole pipelines -- KGraph -> NSG,
INIT_RAND -> Vamana x2, KGraph -> SSG -- with saves, loads, searches and the
L policies, and its graph files, result ids and DistCount / HopCount must
equal the reference's own (golden fixtures)."""
import os
import re
import shutil
import subprocess

import numpy as np
import pytest

from golden_util import load
from weavess_gb300 import build as wbuild
from weavess_gb300 import datasets as ds

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def program(tmp_path_factory):
    if not shutil.which("g++"):
        pytest.skip("no host C++ compiler")
    lib = wbuild.build()
    out = str(tmp_path_factory.mktemp("native") / "builder_pipeline")
    src = os.path.join(ROOT, "tests", "native", "builder_pipeline.cpp")
    cmd = ["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), src, "-o", out,
           "-L", os.path.dirname(lib), "-lweavess_gpu", "-Wl,-rpath," + os.path.dirname(lib)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


def run(program, f, tmp_path, steps):
    bf, qf, gf = (str(tmp_path / x) for x in ("b.fvecs", "q.fvecs", "g.ivecs"))
    ds.write_vecs(bf, f["base"].astype(np.float32))
    ds.write_vecs(qf, f["query"].astype(np.float32))
    ds.write_vecs(gf, f["gt"].astype(np.int32))
    prefix = str(tmp_path / "out")
    kv = [f"{k}={v}" for k, v in f["params"].items()]
    r = subprocess.run([program, bf, qf, gf, prefix] + kv + ["--"] + steps, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    counts = list(zip(map(int, re.findall(r"DistCount: (\d+)", r.stdout)),
                      map(int, re.findall(r"HopCount: (\d+)", r.stdout))))
    return prefix, counts, r.stdout


def graph_bytes(ids, deg, head=()):
    words = list(head)
    for i in range(len(deg)):
        k = int(deg[i])
        words += [k] + [int(x) for x in ids[i, :k]]
    return np.array(words, np.uint32).tobytes()


def test_kgraph_nsg_pipeline(program, tmp_path):
    f = load("int_n2000")
    prefix, counts, _ = run(program, f, tmp_path, ["init_random", "nndescent", "nsg", "save:nsg", "load:nsg",
                                                   "search:centroid:30", "search:rand:40", "policy:centroid:ascend"])
    want = graph_bytes(f["p1.nsg.ids"], f["p1.nsg.deg"], head=[int(f["p1.nsg.ep"])])
    assert open(prefix + ".nsg.graph", "rb").read() == want
    res = np.fromfile(prefix + ".s0.bin", np.uint32).reshape(-1, 10)
    assert np.array_equal(res, f["p1.search_centroid_30.res"])
    assert counts[0] == tuple(f["p1.search_centroid_30.counts"].tolist())
    assert counts[1] == tuple(f["p1.search_rand_40.counts"].tolist())
    steps = f["p1.policy_centroid_ascend.steps"]
    assert counts[2:] == [tuple(x) for x in steps[:, 1:].tolist()]


def test_vamana_pipeline(program, tmp_path):
    f = load("int_n2000")
    prefix, counts, out = run(program, f, tmp_path, ["init_rand", "vamana", "vamana", "save:vamana", "load:vamana",
                                                     "search:centroid:30", "policy:centroid:set_recall"])
    want = graph_bytes(f["p5.vamana.ids"], f["p5.vamana.deg"], head=[int(f["p5.vamana.ep"])])
    assert open(prefix + ".vamana.graph", "rb").read() == want
    res = np.fromfile(prefix + ".s0.bin", np.uint32).reshape(-1, 10)
    assert np.array_equal(res, f["p5.search_centroid_30.res"])
    assert counts[0] == tuple(f["p5.search_centroid_30.counts"].tolist())
    steps = f["p5.policy_centroid_set_recall.steps"]
    assert counts[1:] == [tuple(x) for x in steps[:, 1:].tolist()]
    assert [int(x) for x in re.findall(r"SEARCH_L : (\d+)", out)][1:] == steps[:, 0].tolist()


def test_ssg_pipeline_and_index_info(program, tmp_path):
    f = load("int_n2000")
    prefix, counts, out = run(program, f, tmp_path, ["init_random", "nndescent", "ssg", "save:ssg", "load:ssg",
                                                     "search:rand:30", "search:sub:30", "info:ssg"])
    eps = f["p2.ssg.eps"]
    want = graph_bytes(f["p2.ssg.ids"], f["p2.ssg.deg"], head=[len(eps)] + [int(x) for x in eps])
    assert open(prefix + ".ssg.graph", "rb").read() == want
    assert counts[0] == tuple(f["p2.search_rand_30.counts"].tolist())
    assert counts[1] == tuple(f["p2.search_sub_30.counts"].tolist())
    for i, k in enumerate(("p2.search_rand_30", "p2.search_sub_30")):
        res = np.fromfile(prefix + f".s{i}.bin", np.uint32).reshape(-1, 10)
        assert np.array_equal(res, f[k + ".res"])
    deg = f["p2.ssg.deg"]
    m = re.search(r"Max out degree = (\d+), Min out degree= (\d+), Avg out degree = ([0-9.]+)", out)
    assert m and int(m.group(1)) == deg.max() and int(m.group(2)) == deg.min()
    assert "Conn Statistics: conn = 1" in out


def test_efanna_pipeline_kdt(program, tmp_path):
    """INIT_KDT -> REFINE_EFANNA -> save / load -> SEARCH_ENTRY_KDT, as the
    reference's EFANNA test (test/main.cpp:190-210) drives it."""
    f = load("int_n2000")
    pi = [i for i, s in enumerate(f["pipelines"]) if s[0] == "init_kdt"][0]
    key = f"p{pi}."
    prefix, counts, _ = run(program, f, tmp_path, ["init_kdt", "efanna", "save:efanna", "load:efanna",
                                                   "search:kdt:30", "search:kdt:64"])
    assert open(prefix + ".efanna.graph", "rb").read() == graph_bytes(f[key + "efanna.ids"], f[key + "efanna.deg"])
    for i, L in enumerate((30, 64)):
        res = np.fromfile(prefix + f".s{i}.bin", np.uint32).reshape(-1, 10)
        assert np.array_equal(res, f[f"{key}search_kdt_{L}.res"])
        assert counts[i] == tuple(f[f"{key}search_kdt_{L}.counts"].tolist())
