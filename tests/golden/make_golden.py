"""Generate the golden fixtures in this folder by running the UNMODIFIED
reference (compiled by `make -C oracle ref` from the reference tree) on small
seeded inputs.  Run from the repository root:

    make -C oracle ref && python tests/golden/make_golden.py

Each fixture is an .npz holding the inputs (base / query vectors) and every
output the reference driver dumped: the INIT_RANDOM graph, the NN-Descent
graph, the EFANNA-refined graph, the Vamana / NSG graphs (with entry point), the SSG graph (with its
random roots), the HNSW graph (the reference's INDEX_HNSW file, as words) and search result
ids plus DistCount / HopCount for the listed beam widths.  The oracle is
checked against these by tests/test_oracle_golden.py, and the GPU path
against the oracle by the gpu tests.
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import oracle as O  # noqa: E402
from weavess_gb300 import datasets as ds  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def tie_heavy(n, d, levels, seed, nq):
    r = np.random.default_rng(seed)
    return (r.integers(0, levels, size=(n, d)).astype(np.float32),
            r.integers(0, levels, size=(nq, d)).astype(np.float32))


CASES = {
    # integer mixture (exact FP32 distances), KGraph + Vamana + NSG, reverse-list
    # overflow active (R=100 < in-degree of hubs)
    "int_n2000": dict(data=lambda: ds.int_mixture(2000, 128, 8, seed=1, n_query=50),
                      params=dict(S=10, K=20, L=40, ITER=8, R=100, L_refine=40, R_refine=16, C_refine=200,
                                  alpha=1.2, A=60, n_try=5, max_m=8, max_m0=16, ef_construction=40, mult=0,
                                  n_threads=1, NN=10, nTrees=4, mLevel=2),
                      pipelines=[["init_random", "nndescent", "load:kgraph", "search_rand:20", "search_rand:50",
                                  "vamana", "load:vamana", "search_centroid:30", "search_rand:17",
                                  "policy:rand_set_recall"],
                                 ["init_random", "nndescent", "nsg", "load:nsg", "search_centroid:30",
                                  "search_rand:40", "policy:centroid_ascend"],
                                 ["init_random", "nndescent", "ssg", "load:ssg", "search_rand:30", "search_sub:30"],
                                 ["init_random", "efanna", "load:efanna", "search_rand:30"],
                                 ["hnsw", "search_hnsw:20", "search_hnsw:50", "search_nsw:30"],
                                 ["init_rand", "vamana", "vamana", "load:vamana", "search_centroid:30",
                                  "policy:centroid_set_recall"],
                                 ["nsw", "search_nswidx:20", "search_nswidx:50"],
                                 ["init_kdt", "efanna", "load:efanna", "search_kdt:30", "search_kdt:64"]]),
    # S > 16 and L_refine > K: introsort on ties, rand() seed fill in the
    # candidate search, heavy reverse-list overflow (R=12)
    "int_n1500_s20": dict(data=lambda: ds.int_mixture(1500, 128, 4, seed=3, n_query=40),
                          params=dict(S=20, K=24, L=48, ITER=6, R=12, L_refine=64, R_refine=20, C_refine=100,
                                      alpha=1.2, A=30, n_try=8, nTrees=8, mLevel=4),
                          pipelines=[["init_random", "nndescent", "load:kgraph", "search_rand:33",
                                      "vamana", "load:vamana", "search_centroid:64", "vamana", "load:vamana",
                                      "search_rand:25"],
                                     ["init_random", "nndescent", "ssg", "load:ssg", "search_sub:40"],
                                     ["init_kdt", "efanna", "load:efanna", "search_kdt:40"]]),
    # massive distance ties (values in {0,1,2}, d=16)
    "ties_n1000": dict(data=lambda: tie_heavy(1000, 16, 3, seed=5, nq=40),
                       params=dict(S=12, K=16, L=30, ITER=5, R=20, L_refine=30, R_refine=12, C_refine=60,
                                   alpha=1.2, A=60, n_try=4, max_m=6, max_m0=12, ef_construction=30, mult=0,
                                   n_threads=1, nTrees=2, mLevel=3),
                       pipelines=[["init_random", "nndescent", "load:kgraph", "search_rand:20", "search_rand:40",
                                   "vamana", "load:vamana", "search_centroid:24"],
                                  ["init_random", "nndescent", "nsg", "load:nsg", "search_centroid:20",
                                   "policy:rand_ascend"],
                                  ["init_random", "nndescent", "ssg", "load:ssg", "search_sub:20"],
                                  ["init_random", "efanna"],
                                  ["hnsw", "search_hnsw:16", "search_nsw:24"],
                                  ["init_rand", "vamana", "load:vamana", "search_centroid:20"],
                                  ["init_kdt", "efanna", "load:efanna", "search_kdt:24"]]),
    # real-valued unit vectors (FP32 summation order matters), d=32
    "unit_n1200": dict(data=lambda: ds.unit_mixture(1200, 32, 20, seed=2, n_query=40),
                       params=dict(S=10, K=20, L=40, ITER=6, R=50, L_refine=40, R_refine=16, C_refine=120,
                                   alpha=1.2, A=60, n_try=10, max_m=8, max_m0=16, ef_construction=40, mult=0,
                                   n_threads=1, nTrees=3, mLevel=1),
                       pipelines=[["init_random", "nndescent", "load:kgraph", "search_rand:30",
                                   "vamana", "load:vamana", "search_centroid:30"],
                                  ["init_random", "nndescent", "ssg", "load:ssg", "search_rand:24", "search_sub:24"],
                                  ["init_random", "efanna", "load:efanna", "search_rand:20"],
                                  ["hnsw", "search_hnsw:24", "search_nsw:24"],
                                  ["init_rand", "vamana", "vamana", "load:vamana", "search_centroid:24"],
                                  ["init_kdt", "efanna", "load:efanna", "search_kdt:24"]]),
    # tiny graph: GenRandom wrap-around, self hits, L = N-1 style edges
    "tiny_n60": dict(data=lambda: ds.int_mixture(60, 8, 3, seed=9, n_query=10),
                     params=dict(S=10, K=8, L=16, ITER=4, R=6, L_refine=12, R_refine=6, C_refine=30, alpha=1.2,
                                 A=60, n_try=3, max_m=4, max_m0=8, ef_construction=16, mult=0, n_threads=1, NN=5,
                                 nTrees=1, mLevel=3),
                     pipelines=[["init_random", "nndescent", "load:kgraph", "search_rand:10", "search_rand:20",
                                 "vamana", "load:vamana", "search_centroid:12"],
                                ["init_random", "nndescent", "ssg", "load:ssg", "search_rand:10", "search_sub:10"],
                                ["init_random", "efanna"],
                                ["hnsw", "search_hnsw:10", "search_hnsw:30", "search_nsw:12"],
                                ["init_rand", "vamana", "vamana", "load:vamana", "search_centroid:12"],
                                ["nsw", "search_nswidx:10", "search_nswidx:30"],
                                ["init_kdt", "efanna", "load:efanna", "search_kdt:12"]]),
}


def run_case(name, spec):
    base, query = spec["data"]()
    gt = ds.groundtruth_fp64(base, query, 20)
    out = {"base": base, "query": query, "gt": gt.astype(np.uint32)}
    with tempfile.TemporaryDirectory() as tmp:
        bf, qf, gf = (os.path.join(tmp, x) for x in ("b.fvecs", "q.fvecs", "g.ivecs"))
        ds.write_vecs(bf, base)
        ds.write_vecs(qf, query)
        ds.write_vecs(gf, gt)
        params = [f"{k}={v}" for k, v in spec["params"].items()]
        for pi, steps in enumerate(spec["pipelines"]):
            prefix = os.path.join(tmp, f"p{pi}")
            # repeated steps overwrite their dump, so run prefixes step by step
            log = subprocess.run([O.REF_DRIVER, bf, qf, gf, prefix] + params + ["--"] + steps,
                                 check=True, capture_output=True, text=True).stdout
            del log
            seen = {}
            for s in steps:
                seen[s] = seen.get(s, 0) + 1
            # rerun with unique dumps for steps that repeat (vamana twice)
            if any(v > 1 for v in seen.values()):
                cut = []
                counts = {}
                for s in steps:
                    counts[s] = counts.get(s, 0) + 1
                    cut.append(s)
                    if s in ("vamana",) and counts[s] == 1:
                        subprocess.run([O.REF_DRIVER, bf, qf, gf, prefix + "a"] + params + ["--"] + cut,
                                       check=True, capture_output=True)
                        g = O.read_graph_dump(prefix + "a.vamana.bin")
                        out[f"p{pi}.vamana1.ids"], out[f"p{pi}.vamana1.dist"] = g.ids, g.dist
                        out[f"p{pi}.vamana1.deg"], out[f"p{pi}.vamana1.ep"] = g.deg, np.uint32(g.ep)
            for f in sorted(os.listdir(tmp)):
                if not f.startswith(f"p{pi}.") or not f.endswith(".bin"):
                    continue
                key = f[: -len(".bin")]
                if ".policy_" in key:
                    raw = np.fromfile(os.path.join(tmp, f), np.uint32)
                    rec = raw[1:].reshape(int(raw[0]), 4)
                    out[key + ".steps"] = rec[:, :3].copy()
                    out[key + ".acc"] = rec[:, 3].copy().view(np.float32)
                elif key.endswith(".hnswgraph"):
                    out[f"p{pi}.hnsw.words"] = np.fromfile(os.path.join(tmp, f), np.uint32)
                elif key.endswith(".nswgraph"):
                    out[f"p{pi}.nsw.words"] = np.fromfile(os.path.join(tmp, f), np.uint32)
                elif key.endswith(".kdtleaf"):
                    raw = np.fromfile(os.path.join(tmp, f), np.uint32)
                    out[key] = raw[2:].reshape(int(raw[0]), int(raw[1]))
                elif key.endswith(".ssgeps"):
                    out[key[: -len("eps")] + ".eps"] = np.fromfile(os.path.join(tmp, f), np.uint32)[1:]
                elif "search" in key:
                    res, dc, hc = O.read_search_dump(os.path.join(tmp, f))
                    out[key + ".res"] = res
                    out[key + ".counts"] = np.array([dc, hc], np.uint64)
                else:
                    g = O.read_graph_dump(os.path.join(tmp, f))
                    out[key + ".ids"], out[key + ".dist"], out[key + ".deg"] = g.ids, g.dist, g.deg
                    if g.ep is not None:
                        out[key + ".ep"] = np.uint32(g.ep)
    out["params"] = np.array(repr(spec["params"]))
    out["pipelines"] = np.array(repr(spec["pipelines"]))
    is_int = bool(np.all(base == np.rint(base)) and base.max() <= 255 and base.min() >= 0)
    if is_int:
        out["base"] = base.astype(np.uint8)
        out["query"] = query.astype(np.uint8)
    np.savez_compressed(os.path.join(OUT, name + ".npz"), **out)
    print(name, sorted(k for k in out if k not in ("base", "query")))


if __name__ == "__main__":
    if not os.path.exists(O.REF_DRIVER):
        sys.exit("build the reference driver first: make -C oracle ref")
    for name, spec in CASES.items():
        run_case(name, spec)
