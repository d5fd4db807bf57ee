"""The no-allocation entry point, usgb_process_frame_noalloc.

Some callers cannot let the library allocate device memory while they run
(a host that already handed nearly all GPU memory to its own pool, an
acquisition loop with a fixed latency budget). This entry point takes the RF,
the grid and the outputs from the caller and keeps its tables and prepared
signal tensor in a fixed 64 MiB array inside the library. These tests call it
through the C ABI twice in a row and compare each image with the one the
regular entry point (usgb_create + usgb_process_device) forms from the same
frame and with the CPU oracle, within the parity tolerances of the other GPU
tests, for every storage type and for the real-RF (sign coherence factor)
path; the device status word must stay 0 on these clean frames. The file is
named so that pytest collects it last."""
import ctypes as C
from dataclasses import replace

import numpy as np
import pytest

from helpers import db_err, oracle_spec, rel_err

pytestmark = pytest.mark.gpu

USGB_ERR_INVALID_VALUE = 2
VALUE_TOL = 1e-5     # of the image maximum (FP32 storage, against the FP32 oracle)
FACTOR_TOL = 1e-3    # PCF; SCF and MF are within this too
STORAGE_DB = -60.0   # FP16 / BF16 storage against the FP64 oracle, peak-relative


def _params(spec):
    from us_lab4a_gb300 import native
    from us_lab4a_gb300.engine import COHERENCE, STORAGE
    tx = np.ascontiguousarray(spec.tx_xy, np.float32)
    rx = np.ascontiguousarray(spec.rx_xy, np.float32)
    apod = np.ascontiguousarray(spec.rx_apod if spec.rx_apod is not None else np.ones(rx.shape[0]), np.float32)
    p = native.StaParams()
    p.num_tx, p.num_rx = tx.shape[0], rx.shape[0]
    p.num_samples, p.upsampling = spec.num_samples, spec.upsampling
    p.signal_path = native.USGB_PATH_REAL if spec.real_path else native.USGB_PATH_ANALYTIC
    p.sampling_frequency, p.propagation_speed = spec.sampling_frequency, spec.propagation_speed
    p.center_frequency, p.peak_offset, p.dead_zone_m = spec.center_frequency, spec.peak_offset, spec.dead_zone_m
    p.tx_xy = tx.ctypes.data_as(C.POINTER(C.c_float))
    p.rx_xy = rx.ctypes.data_as(C.POINTER(C.c_float))
    p.rx_apod = apod.ctypes.data_as(C.POINTER(C.c_float))
    p.coherence = COHERENCE[spec.coherence]
    p.pcf_gamma, p.scf_p = spec.pcf_gamma, spec.scf_p
    p.storage, p.storage_scale = STORAGE[spec.storage], spec.storage_scale
    return p, (tx, rx, apod)


def _noalloc(lib, spec, rf, grid, stream, status=None):
    """One call; `status` is a device int32 tensor of one element or None."""
    import torch
    p, keep = _params(spec)
    v = torch.full(grid.shape[:2], -1.0, device=rf.device)
    f = torch.full(grid.shape[:2], -1.0, device=rf.device)
    err = C.create_string_buffer(512)
    st = C.c_void_p(status.data_ptr()) if status is not None else None
    rc = lib.usgb_process_frame_noalloc(C.byref(p), C.c_void_p(rf.data_ptr()), C.c_void_p(grid.data_ptr()),
                                        grid.shape[0], grid.shape[1], C.c_void_p(v.data_ptr()),
                                        C.c_void_p(f.data_ptr()), st, C.c_void_p(stream.cuda_stream), err, 512)
    return rc, err.value.decode(), v, f


def _regular(spec, rf, grid, stream):
    """The same frame through usgb_create + usgb_process_device (staged kernel)."""
    import torch
    from us_lab4a_gb300 import StaEngine
    with StaEngine(spec) as eng:
        eng.set_stream(stream)
        eng.set_das_variant(1)
        eng.set_grid_device(grid)
        v = torch.empty(grid.shape[:2], device=rf.device)
        f = torch.empty_like(v)
        eng.process_device(rf, v, f)
        eng.synchronize()
    return v.cpu().numpy(), f.cpu().numpy()


def _frame(kind):
    from us_lab4a_gb300 import workloads
    if kind == "real-scf":
        fr = workloads.plain2d(small=True)
        fr.spec = replace(fr.spec, real_path=True, upsampling=4, coherence="scf", scf_p=1.5)
        return fr, "f32"
    fr = workloads.cf2d(small=True)  # 16 x 16 A-scans of 5120 samples, PCF
    fr.spec = replace(fr.spec, storage=kind)
    return fr, kind


@pytest.mark.parametrize("kind", ["f32", "f16", "bf16", "real-scf"])
def test_noalloc_matches_regular_entry_point_and_oracle_twice(cuda, oracle_lib, kind):
    import torch
    from us_lab4a_gb300 import native
    lib = native.load()
    fr, storage = _frame(kind)
    rf_np = fr.make_rf_numpy()
    rf = torch.as_tensor(rf_np, device=cuda)
    grid = torch.as_tensor(fr.grid_xyz, device=cuda)
    stream = torch.cuda.current_stream()
    v_reg, f_reg = _regular(fr.spec, rf, grid, stream)
    ospec = oracle_spec(oracle_lib, fr.spec)
    if storage == "f32":
        v_orc, f_orc, _ = oracle_lib.process(ospec, rf_np, fr.grid_xyz, dtype=np.float32)
    else:
        v_orc, f_orc, _ = oracle_lib.process(ospec, rf_np, fr.grid_xyz, dtype=np.float64)
    status = torch.full((1,), 7, dtype=torch.int32, device=cuda)
    for call in range(2):
        rc, msg, v, f = _noalloc(lib, fr.spec, rf, grid, stream, status)
        assert rc == 0, msg
        torch.cuda.synchronize()
        assert int(status.item()) == 0, f"call {call}: device status {int(status.item())}"
        v, f = v.cpu().numpy(), f.cpu().numpy()
        assert rel_err(v, v_reg) <= VALUE_TOL, (call, rel_err(v, v_reg))
        assert np.abs(f - f_reg).max() <= FACTOR_TOL
        if storage == "f32":
            assert rel_err(v, v_orc) <= VALUE_TOL, (call, rel_err(v, v_orc))
            assert np.abs(f - f_orc).max() <= FACTOR_TOL
        else:
            assert db_err(v, v_orc) <= STORAGE_DB, (call, db_err(v, v_orc))
        status.fill_(7)  # the next call must clear it again


def test_noalloc_without_status_word_waits_and_reports(cuda, oracle_lib):
    """With no status word the call waits for its frame and returns the
    device status itself: 0 here, and the image is complete on return."""
    import torch
    from us_lab4a_gb300 import native, workloads
    lib = native.load()
    fr = workloads.cf2d(small=True, coherence="mf")
    rf_np = fr.make_rf_numpy()
    rf = torch.as_tensor(rf_np, device=cuda)
    grid = torch.as_tensor(fr.grid_xyz, device=cuda)
    rc, msg, v, f = _noalloc(lib, fr.spec, rf, grid, torch.cuda.current_stream(), None)
    assert rc == 0, msg
    v_orc, f_orc, _ = oracle_lib.process(oracle_spec(oracle_lib, fr.spec), rf_np, fr.grid_xyz, dtype=np.float32)
    assert rel_err(v.cpu().numpy(), v_orc) <= VALUE_TOL
    assert np.abs(f.cpu().numpy() - f_orc).max() <= FACTOR_TOL


def test_noalloc_other_frame_after_first(cuda):
    """A second, differently shaped frame reuses the array: its image still
    matches the regular entry point (nothing left over from the previous call)."""
    import torch
    from us_lab4a_gb300 import native, workloads
    lib = native.load()
    stream = torch.cuda.current_stream()
    for fr in (workloads.plain2d(small=True), workloads.cf2d(small=True, coherence="mf")):
        rf = torch.as_tensor(fr.make_rf_numpy(), device=cuda)
        grid = torch.as_tensor(fr.grid_xyz, device=cuda)
        rc, msg, v, f = _noalloc(lib, fr.spec, rf, grid, stream)
        assert rc == 0, msg
        v_ref, f_ref = _regular(fr.spec, rf, grid, stream)
        assert rel_err(v.cpu().numpy(), v_ref) <= VALUE_TOL
        assert np.abs(f.cpu().numpy() - f_ref).max() <= FACTOR_TOL


def test_noalloc_rejects_frames_beyond_its_array(cuda):
    import torch
    from us_lab4a_gb300 import native, workloads
    lib = native.load()
    fr = workloads.cf2d(small=True)
    fr.spec = replace(fr.spec, num_samples=40000)  # 16 x 16 x 320000 complex samples: far beyond 64 MiB
    rf = torch.zeros((16, 16, 8), device=cuda)
    grid = torch.as_tensor(fr.grid_xyz, device=cuda)
    rc, msg, v, _ = _noalloc(lib, fr.spec, rf, grid, torch.cuda.current_stream())
    assert rc == USGB_ERR_INVALID_VALUE
    assert "too large" in msg and "67108864" in msg
    torch.cuda.synchronize()
    assert bool((v == -1.0).all())  # nothing was launched
