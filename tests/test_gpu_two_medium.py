"""GPU parity of two-medium imaging (usgb_two_medium_*, the drop-in for
VectorialCombinedTwoMediumImagingProcessor) against the reference processor's
outputs (golden fixtures) and the CPU oracle.

Tolerances: the complex image within 1e-5 of its maximum magnitude without a
coherence factor; with PCF within 1e-3 (each step's sum is weighted by its
PCF, which follows atan2 of the receive terms: a last-bit difference there
moves the factor by up to ~1e-3); FP16 / BF16 storage within -60 dB of the
FP64 oracle. Delays are rounded as the reference's float arithmetic, so the
interface search picks the same points and the points above the interface
(exactly 0) are the same."""
import numpy as np
import pytest

from helpers import TWO_MEDIUM_CASE_NAMES, db_err, rel_err, two_medium_case

pytestmark = pytest.mark.gpu

VALUE_TOL = 1e-5
PCF_VALUE_TOL = 1e-3


def _engine(spec, num_acq, num_tx, storage="f32"):
    from us_lab4a_gb300 import TwoMediumEngine, TwoMediumSTAConfiguration
    cfg = TwoMediumSTAConfiguration(num_elements=spec.num_elements, num_elements_mux=spec.num_elements_mux,
                                    pitch=spec.pitch, center_frequency=spec.center_frequency,
                                    propagation_speed_1=spec.propagation_speed_1,
                                    propagation_speed_2=spec.propagation_speed_2,
                                    sampling_frequency=spec.sampling_frequency)
    return TwoMediumEngine(cfg, num_acq, num_tx, spec.num_samples, spec.upsampling,
                           coherence={0: "none", 1: "pcf", 2: "scf", 3: "mf"}[spec.cf], pcf_gamma=spec.pcf_gamma,
                           max_fermat_block_size=spec.max_fermat_block_size, peak_offset=spec.peak_offset,
                           signal_start_offset=spec.signal_start_offset, storage=storage)


def _run(spec, rf, grid, storage="f32"):
    with _engine(spec, rf.shape[0], rf.shape[1], storage) as eng:
        return eng.process(rf, spec.steps, spec.interface_xz, spec.rx_apod, grid)


@pytest.mark.parametrize("name", TWO_MEDIUM_CASE_NAMES)
def test_two_medium_matches_reference_golden(cuda, oracle_lib, golden_two_medium, name):
    """The GPU image equals VectorialCombinedTwoMediumImagingProcessor<float>'s."""
    spec, rf, grid = two_medium_case(oracle_lib, golden_two_medium, name)
    img = _run(spec, rf, grid)
    ref = golden_two_medium[name + "/image"]
    tol = PCF_VALUE_TOL if spec.cf else VALUE_TOL
    assert rel_err(img, ref) <= tol
    assert np.array_equal(img == 0, ref == 0)


@pytest.mark.parametrize("name", TWO_MEDIUM_CASE_NAMES)
def test_two_medium_processor_class(cuda, oracle_lib, golden_two_medium, name):
    """The Python drop-in with the reference's constructor and process()."""
    from us_lab4a_gb300 import (AnalyticSignalCoherenceFactorProcessor, TwoMediumSTAConfiguration,
                                VectorialCombinedTwoMediumGB300Processor)
    spec, rf, grid = two_medium_case(oracle_lib, golden_two_medium, name)
    cfg = TwoMediumSTAConfiguration(num_elements=spec.num_elements, num_elements_mux=spec.num_elements_mux,
                                    pitch=spec.pitch, center_frequency=spec.center_frequency,
                                    propagation_speed_1=spec.propagation_speed_1,
                                    propagation_speed_2=spec.propagation_speed_2,
                                    sampling_frequency=spec.sampling_frequency)
    cf = AnalyticSignalCoherenceFactorProcessor("phase_coherence_factor" if spec.cf else "none", spec.pcf_gamma)
    proc = VectorialCombinedTwoMediumGB300Processor(cfg, list(rf), spec.upsampling, cf, spec.max_fermat_block_size,
                                                    spec.peak_offset, spec.signal_start_offset)
    img = proc.process(spec.steps, spec.interface_xz, spec.rx_apod, grid)
    proc.close()
    ref = golden_two_medium[name + "/image"]
    assert rel_err(img, ref) <= (PCF_VALUE_TOL if spec.cf else VALUE_TOL)


def _scene_spec(oracle_lib, one_tx, cf, **kw):
    from us_lab4a_gb300 import workloads
    sc = workloads.two_medium_scene(one_tx, **kw)
    spec = oracle_lib.TwoMediumSpec(
        num_elements=sc.num_elements, num_elements_mux=sc.num_elements_mux, pitch=sc.pitch,
        center_frequency=sc.center_frequency, propagation_speed_1=sc.propagation_speed_1,
        propagation_speed_2=sc.propagation_speed_2, sampling_frequency=sc.sampling_frequency,
        num_samples=sc.num_samples, upsampling=sc.upsampling, steps=sc.steps, interface_xz=sc.interface_xz,
        rx_apod=sc.rx_apod, max_fermat_block_size=sc.max_fermat_block_size, peak_offset=sc.peak_offset,
        signal_start_offset=sc.signal_start_offset, cf=cf, pcf_gamma=1.0)
    return spec, sc.rf, sc.grid_xz


@pytest.mark.parametrize("one_tx,cf", [(True, 0), (True, 1), (False, 0), (False, 1)])
def test_two_medium_matches_oracle_larger_scene(cuda, oracle_lib, one_tx, cf):
    """A 64-element array, 32-element sub-aperture in 5 steps, 64 x 160 grid,
    against the FP32 oracle."""
    spec, rf, grid = _scene_spec(oracle_lib, one_tx, cf, num_steps=5, num_samples=1500, grid=(64, 160),
                                 tx_element=7, seed=77)
    img = _run(spec, rf, grid)
    ref = oracle_lib.two_medium(spec, rf, grid, dtype=np.float32)
    assert np.abs(ref).max() > 0
    assert rel_err(img, ref) <= (PCF_VALUE_TOL if cf else VALUE_TOL)
    assert np.array_equal(img == 0, ref == 0)


@pytest.mark.parametrize("storage", ["f16", "bf16"])
def test_two_medium_storage_error_against_fp64_oracle(cuda, oracle_lib, storage):
    spec, rf, grid = _scene_spec(oracle_lib, False, 0, num_steps=3, num_samples=1500, grid=(48, 128), seed=78)
    img = _run(spec, rf, grid, storage)
    ref = oracle_lib.two_medium(spec, rf, grid, dtype=np.float64)
    assert db_err(img, ref) <= -60.0


def test_two_medium_device_path_equals_host_path(cuda, oracle_lib, golden_two_medium):
    import torch
    spec, rf, grid = two_medium_case(oracle_lib, golden_two_medium, "sta_pcf")
    with _engine(spec, rf.shape[0], rf.shape[1]) as eng:
        host = eng.process(rf, spec.steps, spec.interface_xz, spec.rx_apod, grid)
        s = torch.cuda.Stream()
        eng.set_stream(s)
        t = lambda a: torch.as_tensor(np.ascontiguousarray(a, np.float32), device=cuda)
        out = torch.empty((grid.shape[0], grid.shape[1], 2), device=cuda)
        eng.process_device(t(rf), spec.steps, t(spec.interface_xz), t(spec.rx_apod), t(grid), out)
        eng.synchronize()
        dev = out.cpu().numpy().view(np.complex64)[..., 0]
    assert np.array_equal(dev, host)


def test_two_medium_rejects_invalid_steps(cuda, oracle_lib, golden_two_medium):
    """Steps the reference would index out of bounds are rejected with
    InvalidParameterException before any device work."""
    from us_lab4a_gb300 import InvalidParameterException
    spec, rf, grid = two_medium_case(oracle_lib, golden_two_medium, "sta_plain")
    with _engine(spec, rf.shape[0], rf.shape[1]) as eng:
        bad = [
            ([], "empty"),
            ([[0, 9, 0, 7]], "base element"),
            ([[5, 0, 0, 7]], "acquisition"),
            ([[0, 0, 3, 9]], "transmit elements"),
        ]
        for steps, what in bad:
            with pytest.raises(InvalidParameterException):
                eng.process(rf, steps, spec.interface_xz, spec.rx_apod, grid)
        with pytest.raises(InvalidParameterException, match="two points"):
            eng.process(rf, spec.steps, spec.interface_xz[:1], spec.rx_apod, grid)
