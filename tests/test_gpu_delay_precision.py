"""Delay precision of the staged delay-and-sum kernel.

FP32 delays of d samples carry an error of up to about 8 * 2^-24 * d samples;
beyond d = 32768 that can exceed 1/64 sample. Tiles whose delays go past that
switch to FP64 geometry (usgb_set_delay_precision, mode "auto"), and their
image moves towards the FP64 oracle; shallow frames are untouched."""
import numpy as np
import pytest

from helpers import db_err, oracle_spec

pytestmark = pytest.mark.gpu


def _deep_frame():
    """16-element linear array, 5000 samples at 40 MHz, 8x upsampling (L =
    40000), a 32 x 24 grid at z 88-93 mm: delays up to ~38 600 samples."""
    from us_lab4a_gb300 import synth, workloads
    from us_lab4a_gb300.config import window
    from us_lab4a_gb300.engine import FrameSpec
    rng = np.random.default_rng(77)
    scat = synth.point_scatterers(rng, 6, (-1.5e-3, 1.5e-3), (88.5e-3, 92.5e-3))
    el = workloads.linear_array(16)
    spec = FrameSpec(tx_xy=el, rx_xy=el, num_samples=5000, upsampling=8, sampling_frequency=40e6,
                     propagation_speed=workloads.C_SOUND, center_frequency=5e6, rx_apod=window("blackman", 16),
                     coherence="pcf")
    g = workloads.grid_xz(-2e-3, 2e-3, 32, 88e-3, 93e-3, 24)
    return workloads.Frame("deep2d", spec, g, scat, 77)


def _image(spec, rf, grid, mode, device="cuda:0"):
    import torch
    from us_lab4a_gb300 import StaEngine
    with StaEngine(spec) as eng:
        s = torch.cuda.current_stream()
        eng.set_stream(s)
        eng.set_das_variant(1)
        eng.set_delay_precision(mode)
        eng.set_grid_device(torch.as_tensor(grid, device=device))
        v = torch.empty(grid.shape[:2], device=device)
        f = torch.empty_like(v)
        eng.process_device(torch.as_tensor(rf, device=device), v, f)
        eng.synchronize()
        return v.cpu().numpy(), f.cpu().numpy()


def test_deep_grid_fp64_delays_track_the_fp64_oracle(cuda, oracle_lib):
    fr = _deep_frame()
    rf = fr.make_rf_numpy()
    v64, _, _ = oracle_lib.process(oracle_spec(oracle_lib, fr.spec), rf, fr.grid_xyz, dtype=np.float64)
    v32o, _, _ = oracle_lib.process(oracle_spec(oracle_lib, fr.spec), rf, fr.grid_xyz, dtype=np.float32)
    v_auto, f_auto = _image(fr.spec, rf, fr.grid_xyz, "auto")
    v_fp32, _ = _image(fr.spec, rf, fr.grid_xyz, "fp32")
    v_fp64, f_fp64 = _image(fr.spec, rf, fr.grid_xyz, "fp64")
    e_auto, e_fp32, e_oracle32 = db_err(v_auto, v64), db_err(v_fp32, v64), db_err(v32o, v64)
    # Every tile of this grid is deep: auto and forced FP64 are the same launch.
    assert np.array_equal(v_auto, v_fp64) and np.array_equal(f_auto, f_fp64)
    # FP32 delays at ~38 600 samples: the reference's own FP32 arithmetic (and
    # the FP32 mode, the same delays) sits near -90 dB from the FP64 oracle;
    # FP64 delays bring the image down to the FP32 accumulation noise.
    assert abs(e_fp32 - e_oracle32) < 6.0, (e_fp32, e_oracle32)
    assert e_auto <= -110.0 and e_auto < e_fp32 - 20.0, (e_auto, e_fp32)


def test_shallow_grid_auto_is_fp32(cuda):
    """No tile of a shallow frame reaches 32768 samples: "auto" and "fp32"
    give bit-identical images."""
    from us_lab4a_gb300 import workloads
    fr = workloads.cf2d(small=True)
    rf = fr.make_rf_numpy()
    va, fa = _image(fr.spec, rf, fr.grid_xyz, "auto")
    vf, ff = _image(fr.spec, rf, fr.grid_xyz, "fp32")
    assert np.array_equal(va, vf) and np.array_equal(fa, ff)


def test_delay_precision_rejects_unknown_mode(cuda):
    from us_lab4a_gb300 import StaEngine, native, workloads
    from us_lab4a_gb300.errors import InvalidParameterException
    fr = workloads.plain2d(tiny=True)
    with StaEngine(fr.spec) as eng:
        with pytest.raises(InvalidParameterException):
            eng._check(native.load().usgb_set_delay_precision(eng._h, 3))
