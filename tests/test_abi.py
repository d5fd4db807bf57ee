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
