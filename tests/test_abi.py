"""The C-ABI library builds, loads and exports every function the header
declares (no GPU needed)."""
import ctypes

from weavess_gb300 import _lib, build


def test_library_exports_header_symbols():
    path = build.build()
    lib = ctypes.CDLL(path)
    names = _lib.declared_functions()
    assert len(names) >= 10
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_ctx_create_without_gpu_fails_cleanly():
    import torch
    if torch.cuda.is_available():
        return
    lib = _lib.load()
    h = ctypes.c_void_p()
    assert lib.wv_ctx_create(ctypes.byref(h), 0) != 0


def test_library_has_no_unresolved_own_symbols():
    import subprocess
    path = build.build()
    out = subprocess.run(["nm", "-D", "--undefined-only", path], capture_output=True, text=True).stdout
    own = [l.split()[-1] for l in out.splitlines() if "wv" in l.split()[-1].lower() or "learn" in l]
    assert not own, own
