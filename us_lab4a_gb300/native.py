"""ctypes binding of libusgb.so (the C ABI declared in include/usgb.h).

The library is built in-tree (``us_lab4a_gb300/build.py``). There is no CPU
fallback: if the library is missing or fails to load, every entry point
raises.
"""
from __future__ import annotations

import ctypes as C
import os

from . import errors

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "libusgb.so")

USGB_PATH_ANALYTIC, USGB_PATH_REAL = 0, 1
USGB_CF_NONE, USGB_CF_PCF, USGB_CF_SCF, USGB_CF_MF = 0, 1, 2, 3
USGB_STORE_F32, USGB_STORE_F16, USGB_STORE_BF16 = 0, 1, 2
USGB_DELAY_AUTO, USGB_DELAY_FP32, USGB_DELAY_FP64 = 0, 1, 2
USGB_SINGLE_T1R1_SAFT, USGB_SINGLE_TNRN, USGB_SINGLE_SYNTH_Y_TNRN = 0, 1, 2

_FP = C.POINTER(C.c_float)


class StaParams(C.Structure):
    """Mirror of ``usgb_sta_params``."""
    _fields_ = [
        ("num_tx", C.c_uint32), ("num_rx", C.c_uint32), ("num_samples", C.c_uint32),
        ("upsampling", C.c_uint32), ("signal_path", C.c_uint32),
        ("sampling_frequency", C.c_float), ("propagation_speed", C.c_float),
        ("center_frequency", C.c_float), ("peak_offset", C.c_float), ("dead_zone_m", C.c_float),
        ("tx_xy", _FP), ("rx_xy", _FP), ("rx_apod", _FP),
        ("coherence", C.c_uint32), ("pcf_gamma", C.c_float), ("scf_p", C.c_float),
        ("storage", C.c_uint32), ("storage_scale", C.c_float),
    ]


class SingleParams(C.Structure):
    """Mirror of ``usgb_single_params``."""
    _fields_ = [
        ("mode", C.c_uint32), ("num_signals", C.c_uint32), ("num_samples", C.c_uint32), ("upsampling", C.c_uint32),
        ("sampling_frequency", C.c_float), ("propagation_speed", C.c_float),
        ("center_frequency", C.c_float), ("peak_offset", C.c_float), ("dead_zone_m", C.c_float),
        ("tx_xy", _FP), ("rx_xy", _FP), ("rx_apod", _FP),
        ("coherence", C.c_uint32), ("pcf_gamma", C.c_float), ("scf_p", C.c_float),
        ("storage", C.c_uint32), ("storage_scale", C.c_float), ("max_acquisitions", C.c_uint32),
    ]


class TwoMediumParams(C.Structure):
    """Mirror of ``usgb_two_medium_params``."""
    _fields_ = [
        ("num_elements", C.c_uint32), ("num_elements_mux", C.c_uint32), ("pitch", C.c_float),
        ("center_frequency", C.c_float), ("propagation_speed_1", C.c_float), ("propagation_speed_2", C.c_float),
        ("sampling_frequency", C.c_float), ("num_samples", C.c_uint32), ("upsampling", C.c_uint32),
        ("max_fermat_block_size", C.c_float), ("peak_offset", C.c_float), ("signal_start_offset", C.c_uint32),
        ("num_acquisitions", C.c_uint32), ("num_tx", C.c_uint32), ("coherence", C.c_uint32),
        ("pcf_gamma", C.c_float), ("scf_p", C.c_float), ("storage", C.c_uint32), ("storage_scale", C.c_float),
    ]


class TwoMediumStep(C.Structure):
    """Mirror of ``usgb_two_medium_step``."""
    _fields_ = [("base_elem_idx", C.c_uint32), ("base_elem", C.c_uint32), ("first_tx_elem", C.c_uint32),
                ("last_tx_elem", C.c_uint32)]


class BatchItem(C.Structure):
    """Mirror of ``usgb_batch_item``."""
    _fields_ = [("ctx", C.c_void_p), ("d_rf", C.c_void_p), ("d_value", C.c_void_p), ("d_factor", C.c_void_p)]


# Every symbol include/usgb.h declares, with (restype, argtypes).
SIGNATURES = {
    "usgb_create": (C.c_int, [C.POINTER(StaParams), C.POINTER(C.c_void_p)]),
    "usgb_destroy": (None, [C.c_void_p]),
    "usgb_last_error": (C.c_char_p, [C.c_void_p]),
    "usgb_set_grid": (C.c_int, [C.c_void_p, _FP, C.c_uint32, C.c_uint32]),
    "usgb_submit_rf": (C.c_int, [C.c_void_p, C.c_uint32, _FP, C.c_uint32, C.c_uint32]),
    "usgb_process": (C.c_int, [C.c_void_p, _FP, _FP]),
    "usgb_set_stream": (C.c_int, [C.c_void_p, C.c_void_p]),
    "usgb_set_grid_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32]),
    "usgb_process_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "usgb_prepare_signals_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "usgb_delay_and_sum_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "usgb_signal_info": (C.c_int, [C.c_void_p, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32),
                                   C.POINTER(C.c_uint32), C.POINTER(C.c_size_t)]),
    "usgb_set_das_variant": (C.c_int, [C.c_void_p, C.c_int, C.c_uint32, C.c_uint32, C.c_uint32]),
    "usgb_set_delay_precision": (C.c_int, [C.c_void_p, C.c_uint32]),
    "usgb_batch_set_das_variant": (C.c_int, [C.c_void_p, C.c_int]),
    "usgb_single_create": (C.c_int, [C.POINTER(SingleParams), C.POINTER(C.c_void_p)]),
    "usgb_single_destroy": (None, [C.c_void_p]),
    "usgb_single_last_error": (C.c_char_p, [C.c_void_p]),
    "usgb_single_set_stream": (C.c_int, [C.c_void_p, C.c_void_p]),
    "usgb_single_set_tx_delays": (C.c_int, [C.c_void_p, C.c_float, C.c_float, C.c_float, _FP, C.c_uint32]),
    "usgb_single_set_grid": (C.c_int, [C.c_void_p, _FP, C.c_uint32, C.c_uint32]),
    "usgb_single_set_grid_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32]),
    "usgb_single_process": (C.c_int, [C.c_void_p, _FP, _FP, _FP]),
    "usgb_single_process_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "usgb_single_add_acquisition": (C.c_int, [C.c_void_p, _FP, C.c_float]),
    "usgb_single_add_acquisition_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_float]),
    "usgb_single_num_acquisitions": (C.c_int, [C.c_void_p, C.POINTER(C.c_uint32)]),
    "usgb_single_process_window": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, _FP, _FP]),
    "usgb_single_process_window_device": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p, C.c_void_p]),
    "usgb_single_synchronize": (C.c_int, [C.c_void_p]),
    "usgb_two_medium_create": (C.c_int, [C.POINTER(TwoMediumParams), C.POINTER(C.c_void_p)]),
    "usgb_two_medium_destroy": (None, [C.c_void_p]),
    "usgb_two_medium_last_error": (C.c_char_p, [C.c_void_p]),
    "usgb_two_medium_set_stream": (C.c_int, [C.c_void_p, C.c_void_p]),
    "usgb_two_medium_process": (C.c_int, [C.c_void_p, _FP, C.POINTER(TwoMediumStep), C.c_uint32, _FP, C.c_uint32,
                                          _FP, _FP, C.c_uint32, C.c_uint32, _FP]),
    "usgb_two_medium_process_device": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(TwoMediumStep), C.c_uint32,
                                                 C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p, C.c_uint32,
                                                 C.c_uint32, C.c_void_p]),
    "usgb_two_medium_synchronize": (C.c_int, [C.c_void_p]),
    "usgb_h5_last_error": (C.c_char_p, []),
    "usgb_h5_dataset_info": (C.c_int, [C.c_char_p, C.c_char_p, C.POINTER(C.c_uint32), C.POINTER(C.c_uint64),
                                       C.POINTER(C.c_uint64)]),
    "usgb_h5_read_f64": (C.c_int, [C.c_char_p, C.c_char_p, C.POINTER(C.c_double), C.c_size_t,
                                   C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]),
    "usgb_h5_write_f64": (C.c_int, [C.c_char_p, C.c_char_p, C.POINTER(C.c_double), C.c_uint64, C.c_uint64]),
    "usgb_post_create": (C.c_int, [C.c_uint32, C.POINTER(C.c_void_p)]),
    "usgb_post_destroy": (None, [C.c_void_p]),
    "usgb_post_last_error": (C.c_char_p, [C.c_void_p]),
    "usgb_post_envelope_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p]),
    "usgb_post_decibels_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t, C.c_float, C.c_void_p]),
    "usgb_process_rf": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "usgb_set_host_direct": (C.c_int, [C.c_void_p, C.c_int]),
    "usgb_get_host_direct": (C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "usgb_get_das_config": (C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32),
                                      C.POINTER(C.c_uint32)]),
    "usgb_autotune_das": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32,
                                    C.POINTER(C.c_float)]),
    "usgb_synchronize": (C.c_int, [C.c_void_p]),
    "usgb_set_wait_test": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32]),
    "usgb_version": (C.c_char_p, []),
    "usgb_batch_create": (C.c_int, [C.c_uint32, C.c_uint32, C.c_uint32, C.POINTER(C.c_void_p)]),
    "usgb_batch_destroy": (None, [C.c_void_p]),
    "usgb_batch_last_error": (C.c_char_p, [C.c_void_p]),
    "usgb_batch_set_das_config": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32]),
    "usgb_batch_run": (C.c_int, [C.c_void_p, C.POINTER(BatchItem), C.c_uint32, C.c_void_p, C.c_int]),
    "usgb_batch_synchronize": (C.c_int, [C.c_void_p]),
    "usgb_process_frame_noalloc": (C.c_int, [C.POINTER(StaParams), C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32,
                                             C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_char_p, C.c_size_t]),
}

_lib = None


def load(build_if_missing: bool = True):
    """Load libusgb.so (building it first if it is absent and nvcc exists)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        if not build_if_missing:
            raise errors.NativeLibraryError(f"{LIB_PATH} is missing; run us_lab4a_gb300.build.build()")
        from .build import build
        build()
    try:
        lib = C.CDLL(LIB_PATH)
    except OSError as e:
        raise errors.NativeLibraryError(f"cannot load {LIB_PATH}: {e}") from e
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def check(rc: int, ctx=None) -> None:
    """Raise the exception that matches a usgb_status."""
    if rc == 0:
        return
    lib = load()
    msg = lib.usgb_last_error(ctx).decode(errors="replace")
    raise errors.from_status(rc, msg)


def fptr(addr: int):
    return C.cast(C.c_void_p(addr), _FP)
