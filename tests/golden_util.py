"""Replays the pipelines recorded in tests/golden/*.npz (see make_golden.py)
with a pluggable implementation, so the same replay checks the oracle against
the reference's dumps and the GPU path against the same dumps."""
from __future__ import annotations

import ast
import glob
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def cases():
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz")))


def load(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    f = {k: z[k] for k in z.files}
    f["base"] = f["base"].astype(np.float32)
    f["query"] = f["query"].astype(np.float32)
    f["params"] = ast.literal_eval(str(f["params"]))
    f["pipelines"] = ast.literal_eval(str(f["pipelines"]))
    return f


def graph_of(f, key):
    ep = f.get(key + ".ep")
    return f[key + ".ids"], f[key + ".dist"], f[key + ".deg"], (None if ep is None else int(ep))


def rows_equal(ids_a, dist_a, deg_a, ids_b, dist_b, deg_b, check_dist=True):
    """Number of rows that differ (ids in order, and distance bits)."""
    bad = 0
    n = len(deg_b)
    for i in range(n):
        k = int(deg_b[i])
        if int(deg_a[i]) != k or not np.array_equal(ids_a[i, :k], ids_b[i, :k]):
            bad += 1
        elif check_dist and not np.array_equal(np.asarray(dist_a[i, :k], np.float32).view(np.uint32),
                                               np.asarray(dist_b[i, :k], np.float32).view(np.uint32)):
            bad += 1
    return bad
