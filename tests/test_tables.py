"""Host planning of the preparation kernel (usgb_tables.h), on the CPU: the
mixed-radix plan chosen by the shared-memory wavefront model and the Hilbert
pair table in digit-reversed position order, over a sweep of A-scan lengths
(tests/tables/tables_check.cpp)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _cuda_include():
    nvcc = shutil.which("nvcc")
    for d in ([os.path.join(os.path.dirname(os.path.dirname(nvcc)), "include")] if nvcc else []) + \
             ["/usr/local/cuda/include"]:
        if os.path.exists(os.path.join(d, "cuda_runtime.h")):
            return d
    return None


@pytest.mark.skipif(_cuda_include() is None, reason="CUDA headers not found")
def test_fft_plan_and_hilbert_table(tmp_path):
    exe = str(tmp_path / "tables_check")
    cmd = ["g++", "-std=c++17", "-O2", "-I" + _cuda_include(), "-I" + os.path.join(ROOT, "us_lab4a_gb300", "csrc"),
           os.path.join(ROOT, "tests", "tables", "tables_check.cpp"), "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    out = subprocess.run([exe, "1", "70000", "97"], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout[-3000:]
    assert "bad 0" in out.stdout
