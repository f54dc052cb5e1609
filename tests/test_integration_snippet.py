"""The reference-side binding shown in INTEGRATION.md (GPU component
subclasses over the C ABI) compiles against the reference's own headers.
Runs where the reference tree is present (the fixture machine); skipped
elsewhere."""
import os
import re
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _reference_tree() -> str:
    """WEAVESS_REF, else the tree the oracle's reference build recorded."""
    if os.environ.get("WEAVESS_REF"):
        return os.environ["WEAVESS_REF"]
    rec = os.path.join(ROOT, "oracle", "_ref", "REF_PATH")
    return open(rec).read().strip() if os.path.exists(rec) else ""


REF = _reference_tree()


@pytest.mark.skipif(not REF or not os.path.isdir(os.path.join(REF, "include", "weavess")) or not shutil.which("g++"),
                    reason="reference headers not present")
def test_component_subclasses_compile_against_reference_headers(tmp_path):
    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    code = re.findall(r"```cpp\n(.*?)```", text, re.S)[0]
    src = tmp_path / "components_gpu.cpp"
    src.write_text("#include <algorithm>\n#include <vector>\n" + code)
    # the flags the oracle's Makefile builds the reference with (C++11, OpenMP,
    # the standard headers its sources use without including them)
    inc = ["climits", "typeinfo", "set", "map", "unordered_map", "tuple", "cmath", "list", "unistd.h"]
    cmd = ["g++", "-std=gnu++11", "-fsyntax-only", "-fopenmp", "-w"] + sum((["-include", h] for h in inc), []) + [
        "-I", os.path.join(REF, "include"), "-I", os.path.join(ROOT, "oracle", "shim"),
        "-I", os.path.join(ROOT, "include"), str(src)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
