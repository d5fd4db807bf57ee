"""The C-ABI library: it loads, exports every symbol include/usgb.h declares,
and rejects invalid frames with the reference's error semantics before any
device work (so these checks run without a GPU)."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "usgb.h")


def _declared():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:int|void|const char\s*\*)\s+(usgb_\w+)\s*\(", text, re.M)))


@pytest.fixture(scope="module")
def lib():
    from us_lab4a_gb300 import build, native
    build.build()
    return native.load()


def test_header_declares_entry_points():
    names = _declared()
    for n in ("usgb_create", "usgb_destroy", "usgb_last_error", "usgb_set_grid", "usgb_submit_rf", "usgb_process",
              "usgb_process_device", "usgb_prepare_signals_device", "usgb_delay_and_sum_device"):
        assert n in names


def test_library_exports_every_declared_symbol(lib):
    from us_lab4a_gb300 import native
    out = subprocess.run(["nm", "-D", "--defined-only", native.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT\s+(usgb_\w+)", out))
    for name in _declared():
        assert name in exported, name
        assert hasattr(lib, name)
        assert name in native.SIGNATURES, name


def test_header_compiles_as_c():
    src = '#include "usgb.h"\nint main(void){ usgb_sta_params p = {0}; (void)p; return 0; }\n'
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-I" + os.path.dirname(HEADER), "-x", "c", "-",
                        "-fsyntax-only"], input=src, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_version_and_error_strings(lib):
    assert lib.usgb_version().startswith(b"usgb")
    assert lib.usgb_last_error(None) is not None


def _params(**kw):
    from us_lab4a_gb300 import native
    from us_lab4a_gb300.workloads import linear_array
    el = linear_array(8)
    keep = {"el": el}
    p = native.StaParams()
    p.num_tx = p.num_rx = 8
    p.num_samples, p.upsampling = 256, 4
    p.sampling_frequency, p.propagation_speed, p.center_frequency = 40e6, 1540.0, 5e6
    p.tx_xy = p.rx_xy = el.ctypes.data_as(C.POINTER(C.c_float))
    for k, v in kw.items():
        setattr(p, k, v)
    return p, keep


@pytest.mark.parametrize("field,value,status,msg", [
    ("num_tx", 0, 1, "number of elements is zero"),
    ("num_samples", 0, 1, "number of samples is zero"),
    ("upsampling", 0, 2, "Invalid upsampling factor"),
    ("upsampling", 65, 2, "Invalid upsampling factor"),
    ("dead_zone_m", 0.1, 2, "Invalid dead zone"),
    ("coherence", 9, 1, "Invalid coherence factor"),
    ("storage", 7, 1, "Invalid storage"),
    ("num_samples", 300000, 1, "greater than 1048576"),
    ("signal_path", 1, 2, "upsamples by 4"),
])
def test_create_rejects_invalid_frames(lib, field, value, status, msg):
    p, keep = _params(**{field: value})
    if field == "signal_path":
        p.upsampling = 8
    h = C.c_void_p()
    rc = lib.usgb_create(C.byref(p), C.byref(h))
    assert rc == status
    assert msg in lib.usgb_last_error(None).decode()
    assert not h.value


_NOALLOC_CASES = [
    ("num_tx", 0, 1, "number of elements is zero"),
    ("upsampling", 65, 2, "Invalid upsampling factor"),
    ("dead_zone_m", 0.1, 2, "Invalid dead zone"),
    ("coherence", 9, 1, "Invalid coherence factor"),
    ("num_samples", 300000, 1, "greater than 1048576"),
    ("pcf_gamma", float("nan"), 2, "Invalid phase_coherence_factor_gamma"),
    ("pcf_gamma", 101.0, 2, "Invalid phase_coherence_factor_gamma"),
    ("scf_p", -1.0, 2, "Invalid sign_coherence_factor_p"),
]


@pytest.mark.parametrize("field,value,status,msg", _NOALLOC_CASES)
def test_noalloc_checks_like_create(lib, field, value, status, msg):
    """usgb_process_frame_noalloc applies usgb_create's checks (one shared
    function): same status, same message, before any device work."""
    kw = {field: value}
    if field == "pcf_gamma":
        kw["coherence"] = 1
    if field == "scf_p":
        kw["coherence"] = 2
    p, keep = _params(**kw)
    h = C.c_void_p()
    assert lib.usgb_create(C.byref(p), C.byref(h)) == status
    create_msg = lib.usgb_last_error(None).decode()
    assert msg in create_msg
    err = C.create_string_buffer(256)
    fake = C.c_void_p(0x1000)  # never dereferenced: the call fails before any device work
    rc = lib.usgb_process_frame_noalloc(C.byref(p), fake, fake, 16, 16, fake, fake, None, None, err, 256)
    assert rc == status
    assert err.value.decode() == create_msg


def test_noalloc_rejects_oversized_grid(lib):
    p, keep = _params()
    err = C.create_string_buffer(256)
    fake = C.c_void_p(0x1000)
    rc = lib.usgb_process_frame_noalloc(C.byref(p), fake, fake, 65536, 65537, fake, fake, None, None, err, 256)
    assert rc == 2 and err.value == b"Grid too large."
    rc = lib.usgb_process_frame_noalloc(C.byref(p), fake, fake, 0, 16, fake, fake, None, None, err, 256)
    assert rc == 2 and err.value == b"Zero columns in the grid."
    rc = lib.usgb_process_frame_noalloc(C.byref(p), None, fake, 16, 16, fake, fake, None, None, err, 256)
    assert rc == 1 and err.value == b"null device pointer"


def test_real_path_rejects_pcf(lib):
    p, keep = _params(signal_path=1, coherence=1)
    h = C.c_void_p()
    assert lib.usgb_create(C.byref(p), C.byref(h)) == 1
    assert b"sign coherence factor" in lib.usgb_last_error(None)


def test_python_exceptions_map_status(lib):
    from us_lab4a_gb300 import InvalidValueException, StaEngine, workloads
    fr = workloads.plain2d(tiny=True)
    fr.spec.dead_zone_m = 1.0
    with pytest.raises(InvalidValueException, match="Invalid dead zone"):
        StaEngine(fr.spec)


def _single_params(**kw):
    from us_lab4a_gb300 import native
    from us_lab4a_gb300.config import element_positions_matrix
    el = element_positions_matrix(0.3e-3, 4, 0.0, 0.3e-3, 4, 0.0, np.float32)
    apod = np.ones(16, np.float32)
    keep = {"el": el, "apod": apod}
    p = native.SingleParams()
    p.mode = native.USGB_SINGLE_TNRN
    p.num_signals, p.num_samples, p.upsampling = 16, 256, 4
    p.sampling_frequency, p.propagation_speed, p.center_frequency = 40e6, 1540.0, 5e6
    p.tx_xy = p.rx_xy = el.ctypes.data_as(C.POINTER(C.c_float))
    p.rx_apod = apod.ctypes.data_as(C.POINTER(C.c_float))
    for k, v in kw.items():
        setattr(p, k, v)
    return p, keep


@pytest.mark.parametrize("field,value,status,msg", [
    ("mode", 3, 1, "Invalid processor mode"),
    ("num_signals", 0, 1, "number of elements is zero"),
    ("num_signals", 1025, 1, "More than 1024 elements"),
    ("num_samples", 0, 1, "number of samples is zero"),
    ("upsampling", 65, 2, "Invalid upsampling factor"),
    ("dead_zone_m", 0.1, 2, "Invalid dead zone: deadZoneSamplesUp_"),
    ("coherence", 9, 1, "Invalid coherence factor"),
    ("pcf_gamma", -1.0, 2, "Invalid phase_coherence_factor_gamma"),
    ("storage", 7, 1, "Invalid storage"),
    ("max_acquisitions", 4, 1, "Only the synthetic-y array"),
    ("rx_apod", None, 2, "Wrong rx apodization size: 0 (should be 16)"),
])
def test_single_create_rejects_invalid_frames(lib, field, value, status, msg):
    """usgb_single_create checks the frame on the host with the reference's
    messages (Vectorial3DTnRnProcessor.h:131-134, :182-186) before any device work."""
    if field == "rx_apod":
        p, keep = _single_params()
        p.rx_apod = C.cast(None, C.POINTER(C.c_float))
    else:
        p, keep = _single_params(**{field: value})
    if field == "pcf_gamma":
        p.coherence = 1
    h = C.c_void_p()
    rc = lib.usgb_single_create(C.byref(p), C.byref(h))
    assert rc == status
    assert msg in lib.usgb_single_last_error(None).decode()
    assert not h.value


def test_single_t1r1_rejects_apodization_and_synthy_needs_a_ring(lib):
    from us_lab4a_gb300 import native
    p, keep = _single_params(mode=native.USGB_SINGLE_T1R1_SAFT)
    h = C.c_void_p()
    assert lib.usgb_single_create(C.byref(p), C.byref(h)) == 1
    assert b"no rx apodization" in lib.usgb_single_last_error(None)
    p, keep = _single_params(mode=native.USGB_SINGLE_SYNTH_Y_TNRN, max_acquisitions=0)
    assert lib.usgb_single_create(C.byref(p), C.byref(h)) == 1
    assert b"max_acquisitions" in lib.usgb_single_last_error(None)


def test_single_processor_mirrors_reference_checks():
    """Constructor and prepare() checks of the TnRn processors, raised before
    any device work (Vectorial3DTnRnProcessor.h:131-134, 152-157)."""
    from us_lab4a_gb300 import (AnalyticSignalCoherenceFactorProcessor, InvalidParameterException,
                                InvalidStateException, InvalidValueException, TnRnConfiguration,
                                Vectorial3DTnRnGB300Processor)
    from us_lab4a_gb300.config import element_positions_matrix
    el = element_positions_matrix(0.3e-3, 4, 0.0, 0.3e-3, 4, 0.0, np.float32)
    cfg = TnRnConfiguration(num_elements=8, tx_elem_pos=el, rx_elem_pos=el, center_frequency=5e6,
                            sampling_frequency=40e6, propagation_speed=1540.0, num_elements_mux=16)
    cf = AnalyticSignalCoherenceFactorProcessor(method="none")

    class Acq:
        def prepare(self, base, delays):
            pass

        def execute(self):
            return np.zeros((8, 64), np.float32)

    with pytest.raises(InvalidValueException, match="Wrong rx apodization size: 7"):
        Vectorial3DTnRnGB300Processor(cfg, Acq(), 4, cf, 0.0, np.ones(7))
    proc = Vectorial3DTnRnGB300Processor(cfg, Acq(), 4, cf, 0.0, np.ones(8))
    with pytest.raises(InvalidStateException, match="Empty tx delay list"):
        proc.prepare(0)
    proc.set_tx_delays(0.0, 0.0, 0.01, np.zeros(8))
    with pytest.raises(InvalidParameterException, match="Invalid base element: 9"):
        proc.prepare(9)


def _tm_params(**kw):
    from us_lab4a_gb300 import native
    p = native.TwoMediumParams()
    p.num_elements, p.num_elements_mux, p.pitch = 16, 32, 0.6e-3
    p.center_frequency, p.propagation_speed_1, p.propagation_speed_2 = 5e6, 1480.0, 2700.0
    p.sampling_frequency, p.num_samples, p.upsampling = 40e6, 1000, 4
    p.max_fermat_block_size, p.num_acquisitions, p.num_tx = 2.0, 3, 1
    for k, v in kw.items():
        setattr(p, k, v)
    return p


@pytest.mark.parametrize("field,value,status,msg", [
    ("num_elements", 0, 1, "number of elements is zero"),
    ("num_elements", 33, 1, "num_elements (33) > num_elements_mux (32)"),
    ("num_elements_mux", 2000, 1, "More than 1024 elements"),
    ("num_samples", 1, 1, "number of samples (1) is < 2"),
    ("num_acquisitions", 0, 1, "No acquisition data"),
    ("upsampling", 0, 2, "Invalid upsampling factor"),
    ("propagation_speed_2", 0.0, 2, "must be > 0"),
    ("coherence", 7, 1, "Invalid coherence factor"),
    ("storage", 5, 1, "Invalid storage"),
    ("num_samples", 300000, 1, "greater than 1048576"),
])
def test_two_medium_create_rejects_invalid_frames(lib, field, value, status, msg):
    """usgb_two_medium_create checks the parameters on the host before any
    device work."""
    p = _tm_params(**{field: value})
    h = C.c_void_p()
    assert lib.usgb_two_medium_create(C.byref(p), C.byref(h)) == status
    assert msg in lib.usgb_two_medium_last_error(None).decode()
    assert not h.value
