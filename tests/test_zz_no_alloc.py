"""The no-allocation entry point, usgb_process_frame_noalloc.

Some callers cannot let the library allocate device memory while they run
(a host that already handed nearly all GPU memory to its own pool, an
acquisition loop with a fixed latency budget). This entry point takes the RF,
the grid and the outputs from the caller and keeps its tables and prepared
signal tensor in a fixed 64 MiB array inside the library. These tests call it
through the C ABI twice in a row and compare each image with the one the
regular entry point (usgb_create + usgb_process_device) forms from the same
frame, within the parity tolerances of the other GPU tests. The file is named
so that pytest collects it last."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

USGB_ERR_INVALID_VALUE = 2
VALUE_TOL = 1e-5     # of the image maximum
FACTOR_TOL = 1e-3    # PCF


def _params(spec):
    from us_lab4a_gb300 import native
    from us_lab4a_gb300.engine import COHERENCE, STORAGE
    tx = np.ascontiguousarray(spec.tx_xy, np.float32)
    rx = np.ascontiguousarray(spec.rx_xy, np.float32)
    apod = np.ascontiguousarray(spec.rx_apod, np.float32)
    p = native.StaParams()
    p.num_tx, p.num_rx = tx.shape[0], rx.shape[0]
    p.num_samples, p.upsampling = spec.num_samples, spec.upsampling
    p.signal_path = native.USGB_PATH_ANALYTIC
    p.sampling_frequency, p.propagation_speed = spec.sampling_frequency, spec.propagation_speed
    p.center_frequency, p.peak_offset, p.dead_zone_m = spec.center_frequency, spec.peak_offset, spec.dead_zone_m
    p.tx_xy = tx.ctypes.data_as(C.POINTER(C.c_float))
    p.rx_xy = rx.ctypes.data_as(C.POINTER(C.c_float))
    p.rx_apod = apod.ctypes.data_as(C.POINTER(C.c_float))
    p.coherence = COHERENCE[spec.coherence]
    p.pcf_gamma, p.scf_p = spec.pcf_gamma, spec.scf_p
    p.storage, p.storage_scale = STORAGE[spec.storage], spec.storage_scale
    return p, (tx, rx, apod)


def _noalloc(lib, spec, rf, grid, stream):
    import torch
    p, keep = _params(spec)
    v = torch.full(grid.shape[:2], -1.0, device=rf.device)
    f = torch.full(grid.shape[:2], -1.0, device=rf.device)
    err = C.create_string_buffer(512)
    rc = lib.usgb_process_frame_noalloc(C.byref(p), C.c_void_p(rf.data_ptr()), C.c_void_p(grid.data_ptr()),
                                        grid.shape[0], grid.shape[1], C.c_void_p(v.data_ptr()),
                                        C.c_void_p(f.data_ptr()), C.c_void_p(stream.cuda_stream), err, 512)
    return rc, err.value.decode(), v, f


def test_noalloc_matches_regular_entry_point_twice(cuda):
    import torch
    from us_lab4a_gb300 import StaEngine, native, workloads
    lib = native.load()
    fr = workloads.cf2d(small=True)  # 16 x 16 A-scans of 5120 samples, PCF
    rf = torch.as_tensor(fr.make_rf_numpy(), device=cuda)
    grid = torch.as_tensor(fr.grid_xyz, device=cuda)
    stream = torch.cuda.current_stream()
    with StaEngine(fr.spec) as eng:
        eng.set_stream(stream)
        eng.set_das_variant(1)
        eng.set_grid_device(grid)
        v_ref = torch.empty(fr.grid_xyz.shape[:2], device=cuda)
        f_ref = torch.empty_like(v_ref)
        eng.process_device(rf, v_ref, f_ref)
        eng.synchronize()
    v_ref, f_ref = v_ref.cpu().numpy(), f_ref.cpu().numpy()
    for _ in range(2):
        rc, msg, v, f = _noalloc(lib, fr.spec, rf, grid, stream)
        assert rc == 0, msg
        torch.cuda.synchronize()
        v, f = v.cpu().numpy(), f.cpu().numpy()
        assert np.abs(v - v_ref).max() <= VALUE_TOL * np.abs(v_ref).max()
        assert np.abs(f - f_ref).max() <= FACTOR_TOL


def test_noalloc_other_frame_after_first(cuda):
    """A second, differently shaped frame reuses the array: its image still
    matches the regular entry point (nothing left over from the previous call)."""
    import torch
    from us_lab4a_gb300 import StaEngine, native, workloads
    lib = native.load()
    stream = torch.cuda.current_stream()
    for fr in (workloads.plain2d(small=True), workloads.cf2d(small=True, coherence="mf")):
        rf = torch.as_tensor(fr.make_rf_numpy(), device=cuda)
        grid = torch.as_tensor(fr.grid_xyz, device=cuda)
        rc, msg, v, f = _noalloc(lib, fr.spec, rf, grid, stream)
        assert rc == 0, msg
        with StaEngine(fr.spec) as eng:
            eng.set_stream(stream)
            eng.set_das_variant(1)
            eng.set_grid_device(grid)
            v_ref = torch.empty(fr.grid_xyz.shape[:2], device=cuda)
            f_ref = torch.empty_like(v_ref)
            eng.process_device(rf, v_ref, f_ref)
            eng.synchronize()
        v_ref = v_ref.cpu().numpy()
        assert np.abs(v.cpu().numpy() - v_ref).max() <= VALUE_TOL * np.abs(v_ref).max()
        assert np.abs(f.cpu().numpy() - f_ref.cpu().numpy()).max() <= FACTOR_TOL


def test_noalloc_rejects_frames_beyond_its_array(cuda):
    import torch
    from us_lab4a_gb300 import native, workloads
    lib = native.load()
    fr = workloads.cf2d(small=True)
    fr.spec.num_samples = 40000  # 16 x 16 x 320000 complex samples: far beyond 64 MiB
    rf = torch.zeros((16, 16, 8), device=cuda)
    grid = torch.as_tensor(fr.grid_xyz, device=cuda)
    rc, msg, v, _ = _noalloc(lib, fr.spec, rf, grid, torch.cuda.current_stream())
    assert rc == USGB_ERR_INVALID_VALUE
    assert "too large" in msg and "67108864" in msg
    torch.cuda.synchronize()
    assert bool((v == -1.0).all())  # nothing was launched
