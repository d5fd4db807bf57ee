"""GPU parity of the single-term 3D processors (T1R1 SAFT, TnRn, synthetic-y
TnRn) through the C ABI, against the reference processors' outputs (golden
fixtures) and the FP32 / FP64 CPU oracle.

Tolerances as for the STA processors: value within 1e-5 of the image maximum,
coherence factor within 1e-4 (PCF within 1e-3: atan2 of the terms differs in
the last bits between the GPU and the host library); FP16 / BF16 storage
within -60 dB of the FP64 oracle. Delays are rounded as the reference rounds
them, so the grid points where every term falls outside the signal (value
exactly 0) are the same on both sides."""
import numpy as np
import pytest

from helpers import SINGLE_CASE_NAMES, db_err, rel_err, single_case

pytestmark = pytest.mark.gpu

VALUE_TOL = 1e-5
FACTOR_TOL = 1e-4
PCF_TOL = 1e-3


class _SaftAcquisition:
    """STAAcquisition of a T1R1 scan: execute(element) -> (1, ns) rows."""

    def __init__(self, rf, active):
        self.rows = {int(e): rf[i:i + 1] for i, e in enumerate(active)}

    def prepare(self, base_element):
        pass

    def execute(self, element):
        return self.rows[int(element)]


class _TnRnAcquisition:
    def __init__(self, rf):
        self.rf = list(rf) if rf.ndim == 3 else [rf]
        self.next = 0

    def prepare(self, base_element, tx_delays):
        self.delays = tx_delays

    def execute(self):
        r = self.rf[self.next % len(self.rf)]
        self.next += 1
        return r


def _grid(g):
    from us_lab4a_gb300 import make_grid
    grid = make_grid(g.shape[0], g.shape[1])
    grid["x"], grid["y"], grid["z"] = g[..., 0], g[..., 1], g[..., 2]
    return grid


def _run_golden_processor(d, name, storage="f32"):
    from us_lab4a_gb300 import (AnalyticSignalCoherenceFactorProcessor, SA3DConfiguration,
                                SynthYVectorial3DTnRnGB300Processor, TnRnConfiguration,
                                Vectorial3DT1R1SAFTGB300Processor, Vectorial3DTnRnGB300Processor,
                                element_positions_matrix)
    g = lambda k: d[name + "/" + k]
    mode = int(g("mode"))
    el = element_positions_matrix(0.3e-3, 6, 0.0, 0.3e-3, 5, 0.0, np.float32)
    rf = g("rf").astype(np.float32)
    grid = _grid(g("grid"))
    cf = AnalyticSignalCoherenceFactorProcessor("phase_coherence_factor" if int(g("cf")) == 1 else "none",
                                                float(g("pcf_gamma")))
    U, po = int(g("upsampling")), float(g("peak_offset"))
    if mode == 0:
        act = [int(x) for x in g("active")]
        cfg = SA3DConfiguration(tx_elem_pos=el, rx_elem_pos=el, active_tx_elem=act, active_rx_elem=act,
                                center_frequency=float(g("fc")), sampling_frequency=float(g("fs")),
                                propagation_speed=float(g("c")), dead_zone_m=float(g("dead_zone_m")))
        proc = Vectorial3DT1R1SAFTGB300Processor(cfg, _SaftAcquisition(rf, act), U, cf, po, storage=storage)
        proc.prepare(0)
        proc.process(grid)
        return proc, grid
    n, b = int(g("rx_apod").size), int(g("base_element"))
    cfg = TnRnConfiguration(num_elements=n, tx_elem_pos=el, rx_elem_pos=el, center_frequency=float(g("fc")),
                            sampling_frequency=float(g("fs")), propagation_speed=float(g("c")),
                            dead_zone_m=float(g("dead_zone_m")), num_elements_mux=30)
    fx, fy, fz = (float(x) for x in g("focus"))
    if mode == 1:
        proc = Vectorial3DTnRnGB300Processor(cfg, _TnRnAcquisition(rf), U, cf, po, g("rx_apod"), storage=storage)
        proc.set_tx_delays(fx, fy, fz, g("tx_delays"))
        proc.prepare(b)
        proc.process(grid)
        return proc, grid
    proc = SynthYVectorial3DTnRnGB300Processor(cfg, _TnRnAcquisition(rf), U, cf, po, g("rx_apod"), storage=storage,
                                               max_acquisitions=8)
    proc.set_tx_delays(fx, fy, fz, g("tx_delays"))
    proc.prepare(b)
    for y in g("acq_y"):
        proc.get_acq_data(float(y))
    proc.process(int(g("first_acq")), int(g("last_acq")), grid)
    return proc, grid


@pytest.mark.parametrize("name", SINGLE_CASE_NAMES)
def test_single_processor_matches_reference_golden(cuda, golden_single, name):
    """The drop-in processors reproduce Vectorial3DT1R1SAFTProcessor,
    Vectorial3DTnRnProcessor and SynthYVectorial3DTnRnProcessor<float>."""
    proc, grid = _run_golden_processor(golden_single, name)
    vr, fr = golden_single[name + "/value"], golden_single[name + "/factor"]
    assert rel_err(grid["value"], vr) <= VALUE_TOL
    tol = PCF_TOL if "pcf" in name else FACTOR_TOL
    assert np.abs(grid["factor"] - fr).max() <= tol
    assert np.array_equal(grid["value"] == 0, vr == 0)
    if name.startswith("synthy"):
        # process() writes the window's center y into every point, as the reference.
        a, b = int(golden_single[name + "/first_acq"]), int(golden_single[name + "/last_acq"])
        assert np.all(grid["y"] == np.float32(golden_single[name + "/acq_y"][(a + b) // 2]))
    else:
        v1 = grid["value"].copy()
        proc.process(grid)
        assert np.array_equal(grid["value"], v1)
    proc.close()


@pytest.mark.parametrize("name", SINGLE_CASE_NAMES)
def test_single_engine_matches_fp32_oracle(cuda, oracle_lib, golden_single, name):
    """Same frames against the FP32 oracle restatement (host entry points)."""
    spec, rf, grid = single_case(oracle_lib, golden_single, name)
    vo, fo, _ = oracle_lib.single(spec, rf, grid, dtype=np.float32)
    eng = _engine(spec, max_acq=rf.shape[0] if spec.mode == 2 else 0)
    eng.set_grid(grid)
    if spec.mode == 2:
        for r, y in zip(rf, spec.acq_y):
            eng.add_acquisition(r, float(y))
        v, f = eng.process_window(0, rf.shape[0] - 1)
    else:
        v, f = eng.process(rf)
    eng.close()
    assert rel_err(v, vo) <= VALUE_TOL
    assert np.abs(f - fo).max() <= (PCF_TOL if spec.cf == 1 else FACTOR_TOL)
    assert np.array_equal(v == 0, vo == 0)


def _engine(spec, storage="f32", max_acq=0, coherence=None):
    from us_lab4a_gb300 import SingleEngine
    cf = coherence or {0: "none", 1: "pcf", 2: "scf", 3: "mf"}[spec.cf]
    eng = SingleEngine(spec.mode, spec.tx_xy, spec.rx_xy, spec.num_samples, spec.upsampling, spec.sampling_frequency,
                       spec.propagation_speed, spec.center_frequency, spec.peak_offset, spec.dead_zone_m,
                       rx_apod=spec.rx_apod, coherence=cf, pcf_gamma=spec.pcf_gamma, scf_p=spec.scf_p,
                       storage=storage, max_acquisitions=max_acq)
    if spec.mode != 0:
        eng.set_tx_delays(spec.focus[0], spec.focus[1], spec.focus[2], [spec.first_tx_delay])
    return eng


def _saft_volume(oracle_lib, cf=1, nx=16, seed=11):
    """A 16 x 16 matrix array T1R1 scan of a 3D volume (24 x 24 x 96 points)."""
    from us_lab4a_gb300 import synth
    from us_lab4a_gb300.config import element_positions_matrix
    from us_lab4a_gb300.workloads import grid_xyz3
    fs, c, fc, ns = 40e6, 1540.0, 5e6, 1024
    el = element_positions_matrix(0.3e-3, nx, 0.0, 0.3e-3, nx, 0.0, np.float32)
    rng = np.random.default_rng(seed)
    scat = synth.point_scatterers(rng, 12, (-2e-3, 2e-3), (6e-3, 14e-3), y_range=(-2e-3, 2e-3))
    rf = np.stack([synth.synth_rf_numpy(el[i:i + 1], el[i:i + 1], scat, fs, c, fc, ns, rng)[0, 0]
                   for i in range(el.shape[0])])
    grid = grid_xyz3(-3e-3, 3e-3, 24, -3e-3, 3e-3, 24, 5e-3, 15e-3, 96).astype(np.float32).reshape(576, 96, 3)
    spec = oracle_lib.SingleSpec(mode=0, tx_xy=el, rx_xy=el, num_samples=ns, upsampling=4, sampling_frequency=fs,
                                 propagation_speed=c, center_frequency=fc, peak_offset=1.5, cf=cf, pcf_gamma=1.0)
    return spec, rf, grid


@pytest.mark.parametrize("storage,limit_db", [("f32", -100.0), ("f16", -60.0), ("bf16", -60.0)])
def test_single_storage_error_against_fp64_oracle(cuda, oracle_lib, storage, limit_db):
    """FP16 / BF16 signal storage with FP32 accumulation on a 256-element T1R1
    volume: peak-relative image error in dB against the FP64 oracle."""
    spec, rf, grid = _saft_volume(oracle_lib)
    v64, _, _ = oracle_lib.single(spec, rf, grid, dtype=np.float64)
    eng = _engine(spec, storage=storage)
    eng.set_grid(grid)
    v, f = eng.process(rf)
    eng.close()
    assert db_err(v, v64) <= limit_db
    if storage == "f32":
        # The factor follows the FP32 arithmetic (FP64 delays pick other
        # interpolation weights, which moves the phases of weak terms). PCF
        # is discontinuous where a term's phase sits at +-pi: a last-bit
        # difference flips it by 2 pi, which moves the factor by ~1e-3 when
        # the phi branch has the smaller deviation. Over 14 M terms a few
        # points meet that; all others agree within 1e-4.
        _, f32, _ = oracle_lib.single(spec, rf, grid, dtype=np.float32)
        d = np.abs(f - f32)
        assert np.mean(d > FACTOR_TOL) <= 1e-3
        assert d.max() <= 1e-2


def test_single_device_path_equals_host_path(cuda, oracle_lib):
    """process_device on resident tensors gives the host path's bits; two runs
    are bit-identical."""
    import torch
    spec, rf, grid = _saft_volume(oracle_lib, cf=1)
    eng = _engine(spec)
    eng.set_grid(grid)
    vh, fh = eng.process(rf)
    s = torch.cuda.Stream()
    eng.set_stream(s)
    g = torch.as_tensor(grid, device=cuda)
    r = torch.as_tensor(rf, device=cuda)
    v = torch.empty(grid.shape[:2], device=cuda)
    f = torch.empty_like(v)
    eng.set_grid_device(g)
    eng.process_device(r, v, f)
    eng.synchronize()
    assert np.array_equal(v.cpu().numpy(), vh) and np.array_equal(f.cpu().numpy(), fh)
    eng.process_device(r, v, f)
    eng.synchronize()
    assert np.array_equal(v.cpu().numpy(), vh)
    eng.close()


def test_single_separate_tx_positions_and_other_factors(cuda, oracle_lib, golden_single):
    """T1R1 with tx positions different from the rx positions (two distances
    per term), and the SCF / Mallart-Fink factors over the single terms."""
    spec, rf, grid = single_case(oracle_lib, golden_single, "t1r1_plain")
    spec.tx_xy = spec.tx_xy + np.float32(0.05e-3)
    for cf in (0, 2, 3):
        spec.cf, spec.scf_p = cf, 1.5
        vo, fo, _ = oracle_lib.single(spec, rf, grid, dtype=np.float32)
        eng = _engine(spec)
        eng.set_grid(grid)
        v, f = eng.process(rf)
        eng.close()
        assert rel_err(v, vo) <= VALUE_TOL
        assert np.abs(f - fo).max() <= FACTOR_TOL


def test_synthy_ring_keeps_the_last_acquisitions(cuda, oracle_lib, golden_single):
    """With a ring of 3 acquisitions, the 5-acquisition scan keeps the last 3:
    an older window is rejected, a resident one matches the oracle."""
    from us_lab4a_gb300 import InvalidParameterException
    spec, rf, grid = single_case(oracle_lib, golden_single, "synthy_all")
    all_rf, all_y = rf, spec.acq_y
    eng = _engine(spec, max_acq=3)
    eng.set_grid(grid)
    for r, y in zip(all_rf, all_y):
        eng.add_acquisition(r, float(y))
    assert eng.num_acquisitions == 5
    with pytest.raises(InvalidParameterException, match="no longer on the device"):
        eng.process_window(1, 3)
    with pytest.raises(InvalidParameterException, match="has not been added"):
        eng.process_window(3, 5)
    v, f = eng.process_window(2, 4)
    eng.close()
    spec.acq_y = all_y[2:5]
    vo, fo, _ = oracle_lib.single(spec, all_rf[2:5], grid, dtype=np.float32)
    assert rel_err(v, vo) <= VALUE_TOL


def test_single_grid_outside_the_signal_is_zero(cuda, oracle_lib, golden_single):
    """Points whose every delay is past the end of the signal: value 0 and the
    coherence factor of all-zero terms, as the reference (idx + 1 < L test)."""
    spec, rf, grid = single_case(oracle_lib, golden_single, "t1r1_pcf")
    far = grid.copy()
    far[..., 2] += 0.5  # 50 cm deep
    vo, fo, _ = oracle_lib.single(spec, rf, far, dtype=np.float32)
    eng = _engine(spec)
    eng.set_grid(far)
    v, f = eng.process(rf)
    eng.close()
    assert np.all(v == 0) and np.all(vo == 0)
    assert np.array_equal(f, fo.astype(np.float32))
