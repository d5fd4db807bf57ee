"""The saved-acquisition flow of the reference's sta_*_saved tasks on the GPU:
RF saved as signals-base####-tx####.h5, read back by SavedSTAAcquisition,
imaged by the drop-in processor, the image written as image_value.h5 /
image_factor.h5 and read back; against the FP32 oracle on the same RF."""
import os

import numpy as np
import pytest

from helpers import oracle_spec, rel_err

pytestmark = pytest.mark.gpu


def test_saved_acquisition_to_saved_image(cuda, oracle_lib, tmp_path):
    from us_lab4a_gb300 import (AnalyticSignalCoherenceFactorProcessor, STAConfiguration, VectorialSTAGB300Processor,
                                h5, make_grid, workloads)
    fr = workloads.cf2d(small=True, seed=91)
    rf = fr.make_rf_numpy()
    n = fr.spec.num_tx
    acq_dir = str(tmp_path / "acq")
    for tx in range(n):
        h5.save_tx_elem_signals(rf[tx], acq_dir, 0, tx)
    cfg = STAConfiguration(num_elements=n, pitch=0.3e-3, center_frequency=fr.spec.center_frequency,
                           sampling_frequency=fr.spec.sampling_frequency, propagation_speed=fr.spec.propagation_speed)
    cf = AnalyticSignalCoherenceFactorProcessor("phase_coherence_factor", 1.0)
    proc = VectorialSTAGB300Processor(cfg, h5.SavedSTAAcquisition(n, acq_dir), fr.spec.upsampling, cf, 0.0,
                                      fr.spec.rx_apod)
    g = fr.grid_xyz
    grid = make_grid(g.shape[0], g.shape[1])
    grid["x"], grid["y"], grid["z"] = g[..., 0], g[..., 1], g[..., 2]
    proc.prepare(0)
    proc.process(grid)
    proc.close()
    out = str(tmp_path / "img")
    h5.save_image(grid, out)
    value, factor = h5.load_image(out)
    spec = oracle_spec(oracle_lib, fr.spec)
    vo, fo, _ = oracle_lib.process(spec, rf, g, dtype=np.float32)
    assert rel_err(value, vo) <= 1e-5
    assert np.abs(factor - fo).max() <= 1e-3
    assert os.path.exists(os.path.join(out, "image_x.h5"))
