"""The C++ drop-in processors (include/usgb_sta_processor.hpp) run whole frames
on the GPU through the reference's plugin interface (prepare / process on a
Matrix<XYZValueFactor<float>> grid), compiled against stand-ins of the
reference's interface types (tests/adapter/standin/reference_standin.h), since
the reference sources are not present where the GPU is. Each frame's image
equals the C-ABI path's bit for bit and the FP32 oracle's within the parity
tolerances: value within 1e-5 of the image maximum, PCF within 1e-3, SCF
within 1e-4.

Cases: VectorialSTAGB300Processor (analytic path, sub-aperture transmit
elements 2-13 of 16, Blackman receive apodization, dead zone, with and
without PCF) and DefaultSTAGB300Processor (real-RF path, with and without
SCF)."""
import os
import subprocess

import numpy as np
import pytest

from helpers import oracle_spec, rel_err, run_device

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
FIRST_TX, LAST_TX = 2, 13


@pytest.fixture(scope="module")
def adapter_exe(cuda, tmp_path_factory):
    from us_lab4a_gb300 import build
    lib = build.build()
    exe = str(tmp_path_factory.mktemp("adapter") / "adapter_gpu")
    cmd = ["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "tests", "adapter", "standin"),
           "-I", os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "adapter", "adapter_gpu.cpp"),
           lib, "-Wl,-rpath," + os.path.dirname(lib), "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return exe


def _frame(case):
    """A 16-element frame (the small cf2d scene) and the spec the drop-in
    derives from its configuration: transmit elements 2-13, positions from
    ArrayGeometry::getElementXCentered2D."""
    from us_lab4a_gb300 import workloads
    from us_lab4a_gb300.config import element_x_centered_2d
    from us_lab4a_gb300.engine import FrameSpec
    fr = workloads.cf2d(small=True)
    s = fr.spec
    n = s.num_rx
    x = element_x_centered_2d(n, 0.3e-3)
    xy = np.stack([x, np.zeros(n, np.float32)], axis=1).astype(np.float32)
    real = case.endswith("_real")
    cf = case.split("_")[0]
    spec = FrameSpec(tx_xy=xy[FIRST_TX:LAST_TX + 1].copy(), rx_xy=xy, num_samples=s.num_samples,
                     upsampling=4 if real else s.upsampling, sampling_frequency=s.sampling_frequency,
                     propagation_speed=s.propagation_speed, center_frequency=s.center_frequency,
                     peak_offset=1.5, dead_zone_m=0.4e-3, rx_apod=None if real else s.rx_apod,
                     coherence=cf, pcf_gamma=1.0, scf_p=1.0, real_path=real)
    rf = np.ascontiguousarray(fr.make_rf_numpy()[FIRST_TX:LAST_TX + 1], np.float32)
    return spec, rf, np.ascontiguousarray(fr.grid_xyz, np.float32)


def _write_frame(path, case, spec, rf, grid):
    real = case.endswith("_real")
    head = np.array([1 if real else 0, spec.num_rx, FIRST_TX, LAST_TX, spec.num_samples, spec.upsampling,
                     grid.shape[0], grid.shape[1], 0 if spec.coherence == "none" else 1], np.uint32)
    vals = np.array([0.3e-3, spec.sampling_frequency, spec.propagation_speed, spec.center_frequency,
                     spec.dead_zone_m, spec.peak_offset, spec.pcf_gamma, spec.scf_p], np.float32)
    with open(path, "wb") as f:
        f.write(head.tobytes())
        f.write(vals.tobytes())
        f.write(rf.tobytes())
        f.write(grid.tobytes())
        if not real:
            f.write(np.asarray(spec.rx_apod, np.float32).tobytes())


@pytest.mark.parametrize("case", ["pcf", "none", "scf_real", "none_real"])
def test_dropin_processor_frame_on_gpu(adapter_exe, tmp_path, oracle_lib, case):
    spec, rf, grid = _frame(case)
    fin, fout = str(tmp_path / "frame.bin"), str(tmp_path / "image.bin")
    _write_frame(fin, case, spec, rf, grid)
    out = subprocess.run([adapter_exe, fin, fout], capture_output=True, text=True, timeout=120)
    assert out.stdout.strip() == "ok", out.stdout + out.stderr
    img = np.fromfile(fout, np.float32).reshape(2, grid.shape[0], grid.shape[1])
    v, f = img[0], img[1]
    # The C-ABI path on the same frame: the same kernels, bit for bit.
    vd, fd = run_device(spec, rf, grid)
    assert np.array_equal(v, vd) and np.array_equal(f, fd)
    # The FP32 oracle.
    vo, fo, _ = oracle_lib.process(oracle_spec(oracle_lib, spec), rf, grid, dtype=np.float32)
    assert rel_err(v, vo) <= 1e-5, rel_err(v, vo)
    tol = {"pcf": 1e-3, "scf": 1e-4, "none": 0.0}[spec.coherence]
    assert np.abs(f - fo).max() <= tol
