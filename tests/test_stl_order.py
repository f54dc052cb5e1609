"""The device-side restatement of libstdc++'s sort / heap algorithms
(weavess_gb300/csrc/stl_order.cuh) must leave tied elements in exactly the
order the host's std::sort / std::*_heap leave them."""
import os
import subprocess
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))


def test_stl_order_matches_libstdcxx():
    with tempfile.TemporaryDirectory() as tmp:
        exe = os.path.join(tmp, "chk")
        subprocess.check_call(["g++", "-O2", "-std=c++17", "-o", exe,
                               os.path.join(HERE, "native", "stl_order_check.cpp")])
        out = subprocess.run([exe], capture_output=True, text=True, timeout=300)
        assert out.returncode == 0 and out.stdout.startswith("OK"), out.stdout + out.stderr
