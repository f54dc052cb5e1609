"""The device replicas of std::sort (warp-parallel and one-lane) order tied
keys exactly as the host's libstdc++ std::sort does."""
import ctypes
import os
import subprocess
import tempfile

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))

HOST_SORT = r"""
#include <algorithm>
#include <cstdint>
struct E { float d; uint32_t i; bool operator<(const E &o) const { return d < o.d; } };
extern "C" void host_sort(float *k, uint32_t *v, const uint32_t *off, uint32_t narr) {
  for (uint32_t a = 0; a < narr; a++) {
    uint32_t f = off[a], n = off[a + 1] - f;
    E *e = new E[n];
    for (uint32_t j = 0; j < n; j++) e[j] = E{k[f + j], v[f + j]};
    std::sort(e, e + n);
    for (uint32_t j = 0; j < n; j++) { k[f + j] = e[j].d; v[f + j] = e[j].i; }
    delete[] e;
  }
}
"""


@pytest.fixture(scope="module")
def host_sort():
    tmp = tempfile.mkdtemp()
    src = os.path.join(tmp, "hs.cpp")
    so = os.path.join(tmp, "hs.so")
    open(src, "w").write(HOST_SORT)
    subprocess.check_call(["g++", "-O2", "-shared", "-fPIC", "-o", so, src])
    lib = ctypes.CDLL(so)
    f32 = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
    u32 = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")
    lib.host_sort.argtypes = [f32, u32, u32, ctypes.c_uint32]
    return lib


@pytest.mark.parametrize("mode", [0, 1])
def test_device_sort_matches_std_sort(host_sort, mode):
    from weavess_gb300 import Context
    ctx = Context(0)
    rng = np.random.default_rng(mode)
    sizes = np.concatenate([rng.integers(0, 40, 300), rng.integers(40, 4097, 200), [16, 17, 33, 4096, 1, 0]])
    off = np.zeros(len(sizes) + 1, np.uint32)
    off[1:] = np.cumsum(sizes)
    n = int(off[-1])
    keys = np.empty(n, np.float32)
    for a in range(len(sizes)):
        lv = [1, 2, 3, 10, 100, 100000][a % 6]
        f, l = off[a], off[a + 1]
        if a % 11 == 0:
            keys[f:l] = np.arange(l - f)[::-1] % (lv + 1)  # descending runs (deep recursions)
        else:
            keys[f:l] = rng.integers(0, lv, l - f)
    vals = np.arange(n, dtype=np.uint32)
    hk, hv = keys.copy(), vals.copy()
    host_sort.host_sort(hk, hv, off, len(sizes))
    dk, dv = keys.copy(), vals.copy()
    ctx._check(ctx.L.wv_debug_sort(ctx.h, dk, dv, off, len(sizes), mode))
    assert np.array_equal(hk, dk)
    assert np.array_equal(hv, dv)
