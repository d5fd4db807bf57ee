"""GPU parity: the CUDA path (through the C ABI) against the reference
processors' outputs (golden fixtures) and the FP32 CPU oracle.

Tolerances: value within 1e-5 of the image maximum (before log compression);
coherence factor within 1e-4 absolute (PCF within 1e-3: its phases come from
atan2 of sums accumulated in a different order)."""
import math
import os

import numpy as np
import pytest

from helpers import oracle_spec, rel_err, run_device, run_host

pytestmark = pytest.mark.gpu

VALUE_TOL = 1e-5
FACTOR_TOL = 1e-4
PCF_TOL = 1e-3


def _golden_processor_case(golden_frames, prefix):
    from us_lab4a_gb300 import (AnalyticSignalCoherenceFactorProcessor, CoherenceFactorProcessor,
                                DefaultSTAGB300Processor, InMemorySTAAcquisition, SA3DConfiguration,
                                STAConfiguration, Vectorial3DSTAGB300Processor, VectorialSTAGB300Processor,
                                element_positions_matrix, make_grid)
    d = golden_frames
    rf = d[prefix + "/rf"].astype(np.float32)
    g = d[prefix + "/grid"]
    grid = make_grid(g.shape[0], g.shape[1])
    grid["x"], grid["y"], grid["z"] = g[..., 0], g[..., 1], g[..., 2]
    apod = d[prefix + "/apod"]
    if prefix == "vectorial3d_pcf":
        nx = int(d[prefix + "/nx"])
        el = element_positions_matrix(0.3e-3, nx, 0.0, 0.3e-3, nx, 0.0)
        cfg = SA3DConfiguration(tx_elem_pos=el, rx_elem_pos=el, active_tx_elem=list(range(nx * nx)),
                                active_rx_elem=list(range(nx * nx)), center_frequency=3e6,
                                sampling_frequency=24e6, propagation_speed=1540.0)
        proc = Vectorial3DSTAGB300Processor(cfg, InMemorySTAAcquisition(rf), 4,
                                            AnalyticSignalCoherenceFactorProcessor("phase_coherence_factor", 1.0),
                                            0.0, apod)
        return proc, grid
    n = int(d[prefix + "/num_elements"])
    if prefix == "default_scf":
        cfg = STAConfiguration(num_elements=n, pitch=0.3e-3, center_frequency=5e6, sampling_frequency=40e6,
                               propagation_speed=1540.0)
        return DefaultSTAGB300Processor(cfg, InMemorySTAAcquisition(rf), CoherenceFactorProcessor("sign_coherence_factor", 2.0), 0.0), grid
    if prefix == "vectorial_subtx":
        cfg = STAConfiguration(num_elements=n, pitch=0.3e-3, center_frequency=5e6, sampling_frequency=40e6,
                               propagation_speed=1540.0, first_tx_elem=3, last_tx_elem=8)
        cf = AnalyticSignalCoherenceFactorProcessor("phase_coherence_factor", 2.0)
        return VectorialSTAGB300Processor(cfg, InMemorySTAAcquisition(rf, first_tx=3), 1, cf, 0.0, apod), grid
    if prefix == "vectorial_pcf":
        cfg = STAConfiguration(num_elements=n, pitch=0.3e-3, center_frequency=5e6, sampling_frequency=40e6,
                               propagation_speed=1540.0, dead_zone_m=0.5e-3)
        cf = AnalyticSignalCoherenceFactorProcessor("phase_coherence_factor", 1.0)
        return VectorialSTAGB300Processor(cfg, InMemorySTAAcquisition(rf), int(d[prefix + "/upsampling"]), cf, 1.5, apod), grid
    cfg = STAConfiguration(num_elements=n, pitch=0.3e-3, center_frequency=5e6, sampling_frequency=40e6,
                           propagation_speed=1540.0)
    return VectorialSTAGB300Processor(cfg, InMemorySTAAcquisition(rf), int(d[prefix + "/upsampling"]),
                                      AnalyticSignalCoherenceFactorProcessor(), 0.0, apod), grid


@pytest.mark.parametrize("prefix", ["vectorial_plain", "vectorial_pcf", "vectorial_subtx", "default_scf",
                                    "vectorial3d_pcf"])
def test_processor_matches_reference_golden(cuda, golden_frames, prefix):
    """The drop-in processors reproduce the reference processors' images."""
    proc, grid = _golden_processor_case(golden_frames, prefix)
    proc.prepare(0)
    proc.process(grid)
    vr, fr = golden_frames[prefix + "/value"], golden_frames[prefix + "/factor"]
    assert rel_err(grid["value"], vr) <= VALUE_TOL
    tol = PCF_TOL if "pcf" in prefix or prefix == "vectorial_subtx" else FACTOR_TOL
    assert np.abs(grid["factor"] - fr).max() <= tol
    # A second process() call on the same object gives the same image.
    v1 = grid["value"].copy()
    proc.process(grid)
    assert np.array_equal(grid["value"], v1)
    proc.close()


def _small_frames():
    from us_lab4a_gb300 import workloads
    out = [("plain2d", workloads.plain2d(small=True))]
    for cf in ("pcf", "scf", "mf", "none"):
        out.append(("cf2d-" + cf, workloads.cf2d(small=True, coherence=cf)))
    out.append(("matrix3d", workloads.with_storage(workloads.matrix3d(small=True), "f32")))
    real = workloads.plain2d(small=True, seed=5)
    real.spec.real_path, real.spec.coherence = True, "scf"
    out.append(("real-scf", real))
    return out


@pytest.mark.parametrize("name,frame", _small_frames(), ids=[n for n, _ in _small_frames()])
def test_gpu_matches_oracle_fp32(cuda, oracle_lib, name, frame):
    rf = frame.make_rf_numpy()
    v, f = run_host(frame.spec, rf, frame.grid_xyz)
    vo, fo, _ = oracle_lib.process(oracle_spec(oracle_lib, frame.spec), rf, frame.grid_xyz, dtype=np.float32)
    assert rel_err(v, vo) <= VALUE_TOL
    tol = PCF_TOL if frame.spec.coherence == "pcf" else FACTOR_TOL
    assert np.abs(f - fo).max() <= tol


def test_host_and_device_paths_agree(cuda):
    from us_lab4a_gb300 import workloads
    fr = workloads.cf2d(small=True)
    rf = fr.make_rf_numpy()
    vh, fh = run_host(fr.spec, rf, fr.grid_xyz)
    vd, fd = run_device(fr.spec, rf, fr.grid_xyz)
    assert np.array_equal(vh, vd) and np.array_equal(fh, fd)


def test_whole_frame_host_entry_point_paths_agree(cuda):
    """usgb_process_rf reading the host RF in place (where the device reaches
    pageable host memory) or through a copy, and the reference data flow
    (usgb_submit_rf per transmit event + usgb_process), give the same image."""
    from us_lab4a_gb300 import StaEngine, workloads
    fr = workloads.cf2d(small=True)
    rf = fr.make_rf_numpy()
    with StaEngine(fr.spec) as eng:
        eng.set_grid(fr.grid_xyz)
        available, enabled = eng.host_direct()
        assert enabled == available
        vs, fs = eng.process_submitted(rf)
        vd, fd = eng.process_host(rf)
        eng.set_host_direct(False)
        vc, fc = eng.process_host(rf)
        vs2, fs2 = eng.process_submitted(rf)   # the submitted rows are still the frame's
    for v, f in ((vd, fd), (vc, fc), (vs2, fs2)):
        assert np.array_equal(v, vs) and np.array_equal(f, fs)


@pytest.mark.parametrize("U,ns", [(1, 333), (4, 512), (8, 640), (3, 500)])
def test_analytic_signal_matches_oracle(cuda, oracle_lib, U, ns):
    """The prepared tensor (upsampling, DC removal, Hilbert) against the oracle."""
    import torch
    from us_lab4a_gb300 import StaEngine, workloads
    fr = workloads.plain2d(small=True, seed=11)
    spec = fr.spec
    spec.upsampling, spec.num_samples, spec.dead_zone_m = U, ns, 0.2e-3
    fr.rf = None
    rf = fr.make_rf_numpy()
    with StaEngine(spec) as eng:
        info = eng.signal_info()
        stride, L = info["signal_stride"], info["signal_length"]
        eng.set_stream(torch.cuda.current_stream())
        sig = torch.zeros(info["signal_bytes"] // 4, dtype=torch.float32, device=cuda)
        eng.prepare_signals_device(torch.as_tensor(rf, device=cuda), sig)
        eng.synchronize()
    n_sig = spec.num_tx * spec.num_rx
    got = sig[: n_sig * stride * 2].view(n_sig, stride, 2).cpu().numpy()[:, :L]
    got = (got[..., 0] + 1j * got[..., 1]).reshape(spec.num_tx, spec.num_rx, L)
    _, _, ref = oracle_lib.process(oracle_spec(oracle_lib, spec), rf, None, dtype=np.float64, want_signals=True)
    assert np.abs(got - ref).max() <= 2e-6 * np.abs(ref).max()


def test_edge_cases(cuda, oracle_lib):
    """Single column / single row grids, points beyond the last sample,
    a one-element array, no upsampling."""
    from us_lab4a_gb300 import workloads
    from us_lab4a_gb300.engine import FrameSpec
    fr = workloads.plain2d(small=True, seed=21)
    rf = fr.make_rf_numpy()
    for g in (fr.grid_xyz[:1], fr.grid_xyz[:, :1], fr.grid_xyz[:1, :1]):
        g = np.ascontiguousarray(g)
        v, f = run_host(fr.spec, rf, g)
        vo, fo, _ = oracle_lib.process(oracle_spec(oracle_lib, fr.spec), rf, g, dtype=np.float32)
        assert np.allclose(v, vo, rtol=0, atol=VALUE_TOL * max(np.abs(vo).max(), 1e-30))
    # Points far beyond the acquisition: every gather is skipped, value 0.
    far = fr.grid_xyz.copy()
    far[..., 2] = 1.0
    v, _ = run_host(fr.spec, rf, far)
    assert np.all(v == 0)
    # One element, PCF over a single receiver is 1.
    one = FrameSpec(tx_xy=fr.spec.tx_xy[:1], rx_xy=fr.spec.rx_xy[:1], num_samples=fr.spec.num_samples,
                    upsampling=1, sampling_frequency=40e6, propagation_speed=1540.0, center_frequency=5e6,
                    coherence="pcf")
    v, f = run_host(one, rf[:1, :1], fr.grid_xyz)
    vo, fo, _ = oracle_lib.process(oracle_spec(oracle_lib, one), rf[:1, :1], fr.grid_xyz, dtype=np.float32)
    assert rel_err(v, vo) <= VALUE_TOL
    assert np.allclose(f, 1.0) and np.allclose(fo, 1.0)


def test_errors_follow_reference_semantics(cuda):
    from us_lab4a_gb300 import (InvalidParameterException, InvalidStateException, InvalidValueException,
                                StaEngine, workloads)
    fr = workloads.plain2d(small=True)
    with StaEngine(fr.spec) as eng:
        with pytest.raises(InvalidStateException):
            eng.process()  # nothing submitted, no grid
        with pytest.raises(InvalidParameterException, match="Data size mismatch"):
            eng.submit_rf(0, np.zeros((fr.spec.num_rx, fr.spec.num_samples + 1), np.float32))
        with pytest.raises(InvalidValueException, match="Zero columns"):
            eng.set_grid(np.zeros((0, 4, 3), np.float32))


def test_native_library_is_loaded(cuda):
    """The CUDA path runs from the in-tree libusgb.so (no fallback)."""
    from us_lab4a_gb300 import native
    run_host(*_tiny_case())
    maps = open("/proc/self/maps").read()
    assert os.path.realpath(native.LIB_PATH) in maps


def _tiny_case():
    from us_lab4a_gb300 import workloads
    fr = workloads.plain2d(tiny=True)
    return fr.spec, fr.make_rf_numpy(), fr.grid_xyz


@pytest.mark.slow
def test_full_size_cf2d_properties(cuda, oracle_lib):
    """The 64-element, 4096-sample, 8x, 512 x 512 PCF frame at full size:
    random A-scans of the GPU tensor against the oracle's preparation, and
    random grid points of the GPU image against the oracle's delay-and-sum on
    the GPU's own tensor."""
    import torch
    from us_lab4a_gb300 import StaEngine, workloads
    fr = workloads.cf2d(num_speckle=2000)
    spec = fr.spec
    rf = fr.make_rf_torch(cuda)
    rng = np.random.default_rng(0)
    with StaEngine(spec) as eng:
        info = eng.signal_info()
        stride, L = info["signal_stride"], info["signal_length"]
        eng.set_stream(torch.cuda.current_stream())
        sig = torch.zeros(info["signal_bytes"] // 4, dtype=torch.float32, device=cuda)
        eng.prepare_signals_device(rf, sig)
        g = torch.as_tensor(fr.grid_xyz, device=cuda)
        eng.set_grid_device(g)
        v = torch.empty(fr.grid_xyz.shape[:2], device=cuda)
        f = torch.empty_like(v)
        eng.delay_and_sum_device(sig, v, f)
        eng.synchronize()
    n_sig = spec.num_tx * spec.num_rx
    tensor = sig[: n_sig * stride * 2].view(n_sig, stride, 2)[:, :L].cpu().numpy()
    tensor = (tensor[..., 0] + 1j * tensor[..., 1]).astype(np.complex64).reshape(spec.num_tx, spec.num_rx, L)
    rf_h = rf.cpu().numpy()
    # Preparation on 6 random (tx, rx) A-scans.
    for _ in range(6):
        t, r = int(rng.integers(spec.num_tx)), int(rng.integers(spec.num_rx))
        sub = oracle_spec(oracle_lib, spec)
        sub.tx_xy, sub.rx_xy, sub.rx_apod = spec.tx_xy[t:t + 1], spec.rx_xy[r:r + 1], np.ones(1, np.float32)
        _, _, ref = oracle_lib.process(sub, rf_h[t:t + 1, r:r + 1], None, dtype=np.float64, want_signals=True)
        assert np.abs(tensor[t, r] - ref[0, 0]).max() <= 2e-6 * np.abs(ref).max()
    # Delay-and-sum on 512 random points.
    idx = rng.choice(fr.npix, 512, replace=False)
    pts = fr.grid_xyz.reshape(-1, 3)[idx][:, None, :]
    vo, fo = oracle_lib.das(oracle_spec(oracle_lib, spec), tensor, pts, dtype=np.float32)
    vg = v.cpu().numpy().reshape(-1)[idx]
    fg = f.cpu().numpy().reshape(-1)[idx]
    assert np.abs(vg - vo[:, 0]).max() <= VALUE_TOL * np.abs(v.cpu().numpy()).max()
    assert np.abs(fg - fo[:, 0]).max() <= PCF_TOL


def _staged_cases():
    from us_lab4a_gb300 import workloads
    real = workloads.plain2d(small=True, seed=5)
    real.spec.real_path, real.spec.coherence = True, "scf"
    return [("cf2d-pcf", workloads.cf2d(small=True)), ("cf2d-mf", workloads.cf2d(small=True, coherence="mf")),
            ("plain2d", workloads.plain2d(small=True)), ("real-scf", real),
            ("matrix3d-f16", workloads.matrix3d(small=True)),
            ("cf2d-bf16", workloads.with_storage(workloads.cf2d(small=True, coherence="scf"), "bf16")),
            ("plain2d-12el", workloads.plain2d(tiny=True))]


@pytest.mark.parametrize("rows,stage_bytes", [(8, 16384), (4, 4096), (16, 1024)])
@pytest.mark.parametrize("name,frame", _staged_cases(), ids=[n for n, _ in _staged_cases()])
def test_staged_kernel_equals_plain_kernel(cuda, name, frame, rows, stage_bytes):
    """The shared-memory staged kernel and the receiver-group kernel (32- and
    64-column tiles) read the same samples with the same weights in the same
    order as the plain kernel: the images are identical, also when windows
    overflow a stage (small stages force the global-memory path), for partial
    tiles and for a receiver count that leaves a partial receiver group (12
    elements)."""
    import torch
    from us_lab4a_gb300 import StaEngine
    rf = torch.as_tensor(frame.make_rf_numpy(), device=cuda)
    g = torch.as_tensor(frame.grid_xyz, device=cuda)
    out = []
    for variant in (0, 1, 2, 3, 4):
        with StaEngine(frame.spec) as eng:
            eng.set_stream(torch.cuda.current_stream())
            eng.set_das_variant(variant, min(rows, 8) if variant >= 3 else rows, stage_bytes)
            eng.set_grid_device(g)
            v = torch.empty(frame.grid_xyz.shape[:2], device=cuda)
            f = torch.empty_like(v)
            eng.process_device(rf, v, f)
            eng.synchronize()
            out.append((v.cpu().numpy(), f.cpu().numpy()))
    for variant in (1, 2, 3, 4):
        assert np.array_equal(out[0][0], out[variant][0]), variant
        assert np.array_equal(out[0][1], out[variant][1]), variant


def test_grid_selects_tile_width(cuda):
    """Without an explicit choice, a grid of at least 1.5 tiles of 64 x 16 per
    SM selects the two-points-per-thread kernel on 64 x 2R tiles (512 rows on
    152 SMs: R = 7, 296 tiles in two waves), one of at
    least two 64 x 8 tiles per SM the receiver-group kernel on 64-column
    tiles, a small grid keeps 32-column tiles, and a variant set explicitly
    survives a new grid."""
    import torch
    from us_lab4a_gb300 import StaEngine, workloads
    frame = workloads.cf2d(small=True)
    with StaEngine(frame.spec) as eng:
        eng.set_grid_device(torch.zeros((32, 32, 3), device=cuda))
        assert eng.das_config()["variant"] == 2
        eng.set_grid_device(torch.zeros((512, 512, 3), device=cuda))
        sms = torch.cuda.get_device_properties(cuda).multi_processor_count
        cost = {r: math.ceil(8 * math.ceil(512 / (2 * r)) / sms) * (r + 0.6) for r in (8, 7, 6, 5)}
        best = min(cost, key=lambda r: (cost[r], -r))
        assert eng.das_config() == {"variant": 4, "tile_rows": best, "stage_bytes": 102400, "stages": 2}
        eng.set_grid_device(torch.zeros((256, 512, 3), device=cuda))
        cfg = eng.das_config()
        assert cfg["variant"] == 3 and (cfg["tile_rows"], cfg["stage_bytes"]) in ((8, 102400), (8, 98304), (4, 49152),
                                                                                   (4, 32768))
        eng.set_das_variant(2, 8, 16384, 2)
        eng.set_grid_device(torch.zeros((512, 512, 3), device=cuda))
        assert eng.das_config() == {"variant": 2, "tile_rows": 8, "stage_bytes": 16384, "stages": 2}


@pytest.mark.parametrize("cfg", [(3, 8, 102400, 2), (3, 8, 98304, 2), (3, 4, 65536, 2), (2, 16, 98304, 2),
                                 (4, 8, 102400, 2), (4, 8, 65536, 2), (4, 4, 102400, 2), (4, 8, 16384, 3),
                                 (4, 7, 102400, 2), (4, 5, 102400, 2), (4, 3, 65536, 2), (3, 6, 98304, 2),
                                 (3, 1, 32768, 2)])
def test_large_stages_equal_plain_kernel(cuda, cfg):
    """Stages of 64-96 KiB (several units each, one block per SM) give the
    plain kernel's images bit for bit (PCF, partial tiles, FP32 and FP16),
    also with tiles of fewer thread rows than the block holds (the other
    consumer warps idle)."""
    import torch
    from us_lab4a_gb300 import StaEngine, workloads
    for frame in (workloads.cf2d(small=True), workloads.with_storage(workloads.cf2d(small=True, coherence="mf"), "f16")):
        rf = torch.as_tensor(frame.make_rf_numpy(), device=cuda)
        g = torch.as_tensor(frame.grid_xyz, device=cuda)
        out = []
        for variant_cfg in ((0,), cfg):
            with StaEngine(frame.spec) as eng:
                eng.set_stream(torch.cuda.current_stream())
                eng.set_das_variant(*variant_cfg)
                eng.set_grid_device(g)
                v = torch.empty(frame.grid_xyz.shape[:2], device=cuda)
                f = torch.empty_like(v)
                eng.process_device(rf, v, f)
                eng.synchronize()
                out.append((v.cpu().numpy(), f.cpu().numpy()))
        assert np.array_equal(out[0][0], out[1][0])
        assert np.array_equal(out[0][1], out[1][1])
