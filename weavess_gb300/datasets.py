"""Seeded synthetic stand-ins for the workloads the hot path is measured on, and
the fvecs / ivecs file formats the reference loader reads.

File formats follow the reference loader (src/component_load.cpp:9-28): every
record is a 4-byte little-endian dimension followed by `dim` 4-byte values;
the record count is file_size / ((dim + 1) * 4).

Workloads (public datasets are not available; these keep the shapes, sizes
and value distributions of the measured configurations):

* ``int_mixture``  -- integer-valued Gaussian mixture: centres uniform in
  [0, 255]^d, sigma 20, values rounded to integers and clipped to [0, 255]
  (N=1e5 / 64 centres, N=1e6 / 256 centres, N=1e7 / 1024 centres; d=128).
  Squared L2 distances on these vectors are exact in FP32 (max 128*255^2 < 2^24).
* ``unit_mixture`` -- d=96 unit-norm vectors: an isotropic Gaussian part plus
  points around 1,000 random unit directions (cosine ~0.7 to the nearest one).
* ``simplex_mixture`` -- d=960 non-negative vectors: 512-component Gaussian
  mixture, ReLU-clipped, each row scaled to sum 1.
"""
from __future__ import annotations

import os
import numpy as np


# ---------------------------------------------------------------- generators
def int_mixture(n: int, d: int = 128, n_centers: int = 64, sigma: float = 20.0,
                seed: int = 7, n_query: int = 0, query_stream: int = 2):
    """Integer-valued Gaussian mixture (float32).  Returns (base, query);
    `query_stream` selects an independent stream of queries from the same
    mixture (2: the evaluation queries; other values: e.g. training queries)."""
    rng = np.random.default_rng(seed)
    centers = rng.uniform(0.0, 255.0, size=(n_centers, d))

    def draw(count, sub):
        r = np.random.default_rng([seed, sub])
        out = np.empty((count, d), dtype=np.float32)
        step = 1 << 18
        for s in range(0, count, step):
            c = min(step, count - s)
            lab = r.integers(0, n_centers, size=c)
            x = centers[lab] + r.normal(0.0, sigma, size=(c, d))
            out[s:s + c] = np.clip(np.rint(x), 0.0, 255.0)
        return out

    return draw(n, 1), draw(n_query, query_stream)


def unit_mixture(n: int, d: int = 96, n_dirs: int = 1000, cos: float = 0.7,
                 iso_frac: float = 0.1, seed: int = 11, n_query: int = 0):
    """Unit-norm vectors: `iso_frac` isotropic, the rest clustered around
    `n_dirs` random unit directions with cosine ~`cos` to their direction."""
    rng = np.random.default_rng(seed)
    dirs = rng.normal(size=(n_dirs, d))
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    # a unit vector at angle theta from u: cos(theta) u + sin(theta) v, v _|_ u
    sin = np.sqrt(1.0 - cos * cos)

    def draw(count, sub):
        r = np.random.default_rng([seed, sub])
        out = np.empty((count, d), dtype=np.float32)
        step = 1 << 18
        for s in range(0, count, step):
            c = min(step, count - s)
            g = r.normal(size=(c, d))
            lab = r.integers(0, n_dirs, size=c)
            u = dirs[lab]
            v = g - (g * u).sum(1, keepdims=True) * u
            v /= np.linalg.norm(v, axis=1, keepdims=True)
            x = cos * u + sin * v
            iso = r.random(c) < iso_frac
            x[iso] = g[iso] / np.linalg.norm(g[iso], axis=1, keepdims=True)
            x /= np.linalg.norm(x, axis=1, keepdims=True)
            out[s:s + c] = x
        return out

    return draw(n, 1), draw(n_query, 2)


def simplex_mixture(n: int, d: int = 960, n_comp: int = 512, seed: int = 13,
                    n_query: int = 0):
    """Non-negative rows summing to 1 (ReLU-clipped Gaussian mixture)."""
    rng = np.random.default_rng(seed)
    centers = rng.normal(0.0, 1.0, size=(n_comp, d))

    def draw(count, sub):
        r = np.random.default_rng([seed, sub])
        out = np.empty((count, d), dtype=np.float32)
        step = 1 << 16
        for s in range(0, count, step):
            c = min(step, count - s)
            lab = r.integers(0, n_comp, size=c)
            x = np.maximum(centers[lab] + r.normal(0.0, 0.5, size=(c, d)), 0.0)
            x /= np.maximum(x.sum(1, keepdims=True), 1e-12)
            out[s:s + c] = x
        return out

    return draw(n, 1), draw(n_query, 2)


# -------------------------------------------------------------- file formats
def write_vecs(path: str, x: np.ndarray) -> None:
    """Write float32 (fvecs) or uint32/int32 (ivecs) rows with a dim header."""
    x = np.ascontiguousarray(x)
    n, d = x.shape
    rec = np.empty((n, d + 1), dtype=np.uint32)
    rec[:, 0] = d
    rec[:, 1:] = x.view(np.uint32) if x.dtype.itemsize == 4 else x.astype(np.uint32)
    rec.tofile(path)


def read_vecs(path: str, dtype=np.float32) -> np.ndarray:
    """Read an fvecs/ivecs file as the reference loader does
    (component_load.cpp:9-28): num = file_size / (dim + 1) / 4."""
    raw = np.fromfile(path, dtype=np.uint32)
    if raw.size == 0:
        return np.zeros((0, 0), dtype=dtype)
    d = int(raw[0])
    n = raw.size // (d + 1)
    rec = raw[: n * (d + 1)].reshape(n, d + 1)
    return np.ascontiguousarray(rec[:, 1:]).view(dtype)


# -------------------------------------------------------------- ground truth
def groundtruth_fp64(base: np.ndarray, query: np.ndarray, k: int = 100,
                     chunk: int = 256) -> np.ndarray:
    """Exact top-k by FP64 squared L2 (ties broken by smaller id).  CPU, for
    sizes up to ~1e5 x 1e3."""
    b = base.astype(np.float64)
    bn = (b * b).sum(1)
    out = np.empty((query.shape[0], k), dtype=np.uint32)
    for s in range(0, query.shape[0], chunk):
        q = query[s:s + chunk].astype(np.float64)
        d = (q * q).sum(1)[:, None] + bn[None, :] - 2.0 * q @ b.T
        # exact rerank of a generous candidate set in the direct form
        cand = np.argpartition(d, min(k + 64, d.shape[1] - 1), axis=1)[:, : k + 64]
        for r in range(q.shape[0]):
            c = cand[r]
            dd = ((b[c] - q[r]) ** 2).sum(1)
            o = np.lexsort((c, dd))[:k]
            out[s + r] = c[o]
    return out


def recall_at(res: np.ndarray, gt: np.ndarray, k: int = 10) -> float:
    """recall@k as the reference computes it (src/builder.cpp:466-480):
    1 - misses / (nq * k), a miss being a returned id not among gt[:, :k]."""
    nq = res.shape[0]
    miss = 0
    for i in range(nq):
        g = set(int(v) for v in gt[i, :k])
        miss += sum(1 for v in res[i, :k] if int(v) not in g)
    return 1.0 - miss / float(nq * k)


def cache_dir() -> str:
    d = os.environ.get("WEAVESS_DATA_CACHE", os.path.join(os.path.dirname(__file__), "..", "_data"))
    os.makedirs(d, exist_ok=True)
    return d
