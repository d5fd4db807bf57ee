"""The C++ drop-in processors (include/usgb_sta_processor.hpp) compile against
stand-ins of the reference's interface types (tests/adapter/standin/) and map
a library error to the reference's exception type before any device work:
a negative dead zone is InvalidValueException "Invalid dead zone: ..." (the
frames themselves run in test_gpu_adapter_standin.py)."""
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_dropin_compiles_against_standins_and_maps_errors(tmp_path):
    from us_lab4a_gb300 import build
    lib = build.build()
    exe = str(tmp_path / "adapter_gpu")
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", "-Werror", "-I", os.path.join(ROOT, "tests", "adapter", "standin"),
           "-I", os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "adapter", "adapter_gpu.cpp"),
           lib, "-Wl,-rpath," + os.path.dirname(lib), "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    n, ns, ncols, nrows = 8, 256, 4, 4
    head = np.array([0, n, 0, n - 1, ns, 4, ncols, nrows, 1], np.uint32)
    vals = np.array([0.3e-3, 40e6, 1540.0, 5e6, -1e-3, 0.0, 1.0, 1.0], np.float32)   # dead zone -1 mm
    fin = tmp_path / "frame.bin"
    with open(fin, "wb") as f:
        f.write(head.tobytes())
        f.write(vals.tobytes())
        f.write(np.zeros((n, n, ns), np.float32).tobytes())
        f.write(np.zeros((ncols, nrows, 3), np.float32).tobytes())
        f.write(np.ones(n, np.float32).tobytes())
    out = subprocess.run([exe, str(fin), str(tmp_path / "image.bin")], capture_output=True, text=True, timeout=60)
    assert out.stdout.startswith("InvalidValueException Invalid dead zone: -0.001"), out.stdout + out.stderr
