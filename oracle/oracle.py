"""ctypes wrapper of the CPU oracle (``liboracle.so``, built from sta_oracle_capi.cpp).

Test infrastructure only: the parity checker of the CUDA library and the CPU
baseline of bench.py. The arithmetic lives in sta_oracle.hpp, which cites the
reference file:line of every step.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass, field
from typing import Optional

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None

CF_NONE, CF_PCF, CF_SCF, CF_MF = 0, 1, 2, 3


def lib_path() -> str:
    return os.path.join(_HERE, "liboracle.so")


def build(force: bool = False) -> str:
    """Compile liboracle.so with the Makefile beside this file."""
    if force or not os.path.exists(lib_path()) or _stale():
        subprocess.run(["make", "-s", "-C", _HERE, "liboracle.so"], check=True)
    return lib_path()


def _stale() -> bool:
    so = lib_path()
    t = os.path.getmtime(so)
    for f in ("sta_oracle_capi.cpp", "sta_oracle.hpp"):
        if os.path.getmtime(os.path.join(_HERE, f)) > t:
            return True
    return False


def available() -> bool:
    return os.path.exists(lib_path())


def _desc_type(ct):
    class Desc(C.Structure):
        _fields_ = [
            ("num_tx", C.c_uint), ("num_rx", C.c_uint), ("num_samples", C.c_uint), ("upsampling", C.c_uint),
            ("sampling_frequency", ct), ("propagation_speed", ct), ("center_frequency", ct),
            ("peak_offset", ct), ("dead_zone_m", ct),
            ("tx_xy", C.POINTER(ct)), ("rx_xy", C.POINTER(ct)), ("rx_apod", C.POINTER(ct)),
            ("cf", C.c_int), ("pcf_gamma", ct), ("scf_p", ct),
            ("real_path", C.c_int), ("nthreads", C.c_int),
        ]
    return Desc


_Desc32 = _desc_type(C.c_float)
_Desc64 = _desc_type(C.c_double)


def _lib():
    global _LIB
    if _LIB is None:
        if not available():
            build()
        lib = C.CDLL(lib_path())
        lib.orc_last_error.restype = C.c_char_p
        lib.orc_next_fast_even_size.restype = C.c_uint
        lib.orc_next_fast_even_size.argtypes = [C.c_uint]
        lib.orc_hilbert_fft_size.restype = C.c_uint
        lib.orc_hilbert_fft_size.argtypes = [C.c_uint]
        for name, ct, desc in (("f32", C.c_float, _Desc32), ("f64", C.c_double, _Desc64)):
            p = C.POINTER(ct)
            f = getattr(lib, "orc_process_" + name)
            f.restype = C.c_int
            f.argtypes = [C.POINTER(desc), p, p, C.c_size_t, p, p, p]
            f = getattr(lib, "orc_das_" + name)
            f.restype = C.c_int
            f.argtypes = [C.POINTER(desc), p, p, C.c_size_t, p, p]
        lib.orc_scf_f64.restype = C.c_double
        lib.orc_scf_f64.argtypes = [C.POINTER(C.c_double), C.c_uint, C.c_double]
        lib.orc_pcf_f64.restype = C.c_double
        lib.orc_pcf_f64.argtypes = [C.POINTER(C.c_double), C.c_uint, C.c_double]
        _LIB = lib
    return _LIB


def _ptr(a: Optional[np.ndarray], ct):
    if a is None:
        return C.cast(None, C.POINTER(ct))
    return a.ctypes.data_as(C.POINTER(ct))


def _err(rc: int):
    if rc != 0:
        raise ValueError(_lib().orc_last_error().decode())


@dataclass
class OracleSpec:
    """One STA frame: geometry, acquisition parameters and processing choices.

    Field meaning follows STAConfiguration / SA3DConfiguration and the
    VectorialSTAProcessor constructor arguments of the reference.
    """
    tx_xy: np.ndarray                  # (num_tx, 2) active transmit element centres, m
    rx_xy: np.ndarray                  # (num_rx, 2) receive element centres, m
    num_samples: int
    upsampling: int
    sampling_frequency: float
    propagation_speed: float
    center_frequency: float
    peak_offset: float = 0.0
    dead_zone_m: float = 0.0
    rx_apod: Optional[np.ndarray] = None
    cf: int = CF_NONE
    pcf_gamma: float = 1.0
    scf_p: float = 1.0
    real_path: bool = False
    nthreads: int = field(default_factory=lambda: os.cpu_count() or 1)

    @property
    def num_tx(self) -> int:
        return int(self.tx_xy.shape[0])

    @property
    def num_rx(self) -> int:
        return int(self.rx_xy.shape[0])

    @property
    def signal_length(self) -> int:
        return self.num_samples * (4 if self.real_path else self.upsampling)


def _make_desc(spec: OracleSpec, dtype):
    desc_t, ct = (_Desc32, C.c_float) if dtype == np.float32 else (_Desc64, C.c_double)
    keep = {
        "tx": np.ascontiguousarray(spec.tx_xy, dtype=dtype),
        "rx": np.ascontiguousarray(spec.rx_xy, dtype=dtype),
        "apod": np.ascontiguousarray(spec.rx_apod if spec.rx_apod is not None else np.ones(spec.num_rx), dtype=dtype),
    }
    d = desc_t(
        spec.num_tx, spec.num_rx, spec.num_samples, spec.upsampling,
        spec.sampling_frequency, spec.propagation_speed, spec.center_frequency,
        spec.peak_offset, spec.dead_zone_m,
        _ptr(keep["tx"], ct), _ptr(keep["rx"], ct), _ptr(keep["apod"], ct),
        spec.cf, spec.pcf_gamma, spec.scf_p, int(spec.real_path), int(spec.nthreads),
    )
    return d, keep, ct


def process(spec: OracleSpec, rf: np.ndarray, grid_xyz: Optional[np.ndarray], dtype=np.float64,
            want_signals: bool = False):
    """Run the whole processor. rf: (num_tx, num_rx, num_samples). grid_xyz: (..., 3).

    Returns (value, factor, signals); value/factor have grid_xyz.shape[:-1];
    signals is the analytic tensor (complex, (num_tx, num_rx, L)) or the real
    tensor for the real path, when want_signals.
    """
    d, keep, ct = _make_desc(spec, dtype)
    rf = np.ascontiguousarray(rf, dtype=dtype)
    assert rf.shape == (spec.num_tx, spec.num_rx, spec.num_samples), rf.shape
    L = spec.signal_length
    npix = 0
    g = None
    if grid_xyz is not None:
        g = np.ascontiguousarray(grid_xyz, dtype=dtype).reshape(-1, 3)
        npix = g.shape[0]
    value = np.zeros(max(npix, 1), dtype=dtype)
    factor = np.ones(max(npix, 1), dtype=dtype)
    sig = None
    if want_signals:
        width = 1 if spec.real_path else 2
        sig = np.zeros(spec.num_tx * spec.num_rx * L * width, dtype=dtype)
    f = getattr(_lib(), "orc_process_" + ("f32" if dtype == np.float32 else "f64"))
    _err(f(C.byref(d), _ptr(rf, ct), _ptr(g, ct), npix, _ptr(value, ct), _ptr(factor, ct), _ptr(sig, ct)))
    if sig is not None:
        if spec.real_path:
            sig = sig.reshape(spec.num_tx, spec.num_rx, L)
        else:
            sig = sig.view(np.complex64 if dtype == np.float32 else np.complex128).reshape(spec.num_tx, spec.num_rx, L)
    shape = grid_xyz.shape[:-1] if grid_xyz is not None else (0,)
    return value[:npix].reshape(shape), factor[:npix].reshape(shape), sig


def das(spec: OracleSpec, signals: np.ndarray, grid_xyz: np.ndarray, dtype=np.float64):
    """Delay-and-sum only, on prepared signals (complex analytic or real tensor)."""
    d, keep, ct = _make_desc(spec, dtype)
    if spec.real_path:
        s = np.ascontiguousarray(signals, dtype=dtype)
    else:
        s = np.ascontiguousarray(signals, dtype=np.complex64 if dtype == np.float32 else np.complex128).view(dtype)
    g = np.ascontiguousarray(grid_xyz, dtype=dtype).reshape(-1, 3)
    npix = g.shape[0]
    value = np.zeros(npix, dtype=dtype)
    factor = np.ones(npix, dtype=dtype)
    f = getattr(_lib(), "orc_das_" + ("f32" if dtype == np.float32 else "f64"))
    _err(f(C.byref(d), _ptr(s, ct), _ptr(g, ct), npix, _ptr(value, ct), _ptr(factor, ct)))
    return value.reshape(grid_xyz.shape[:-1]), factor.reshape(grid_xyz.shape[:-1])


SINGLE_T1R1_SAFT, SINGLE_TNRN, SINGLE_SYNTH_Y_TNRN = 0, 1, 2


def _single_desc_type(ct):
    class SingleDesc(C.Structure):
        _fields_ = [
            ("mode", C.c_int), ("num_signals", C.c_uint), ("num_samples", C.c_uint), ("upsampling", C.c_uint),
            ("sampling_frequency", ct), ("propagation_speed", ct), ("center_frequency", ct),
            ("peak_offset", ct), ("dead_zone_m", ct),
            ("tx_xy", C.POINTER(ct)), ("rx_xy", C.POINTER(ct)), ("rx_apod", C.POINTER(ct)),
            ("focus_x", ct), ("focus_y", ct), ("focus_z", ct), ("first_tx_delay", ct),
            ("num_acq", C.c_uint), ("acq_y", C.POINTER(ct)),
            ("cf", C.c_int), ("pcf_gamma", ct), ("scf_p", ct), ("nthreads", C.c_int),
        ]
    return SingleDesc


_Single32 = _single_desc_type(C.c_float)
_Single64 = _single_desc_type(C.c_double)


@dataclass
class SingleSpec:
    """One frame of a single-term 3D processor (Vectorial3DT1R1SAFTProcessor,
    Vectorial3DTnRnProcessor or SynthYVectorial3DTnRnProcessor).

    tx_xy: T1R1 -- (num_signals, 2) positions of the active transmit elements;
    TnRn -- (>= 1, 2), row 0 = the first element of the group (txElemPos[base]).
    rx_xy: (num_signals, 2). rx_apod: TnRn weights (num_signals).
    first_tx_delay: txDelays[0] in s. acq_y: synthetic y, the y of each
    acquisition of the window (num_acq)."""
    mode: int
    tx_xy: np.ndarray
    rx_xy: np.ndarray
    num_samples: int
    upsampling: int
    sampling_frequency: float
    propagation_speed: float
    center_frequency: float
    peak_offset: float = 0.0
    dead_zone_m: float = 0.0
    rx_apod: Optional[np.ndarray] = None
    focus: tuple = (0.0, 0.0, 0.0)
    first_tx_delay: float = 0.0
    acq_y: Optional[np.ndarray] = None
    cf: int = CF_NONE
    pcf_gamma: float = 1.0
    scf_p: float = 1.0
    nthreads: int = field(default_factory=lambda: os.cpu_count() or 1)

    @property
    def num_signals(self) -> int:
        return int(self.rx_xy.shape[0])

    @property
    def num_acq(self) -> int:
        return int(len(self.acq_y)) if self.mode == SINGLE_SYNTH_Y_TNRN else 1


def single(spec: SingleSpec, rf: np.ndarray, grid_xyz: np.ndarray, dtype=np.float64, want_signals: bool = False):
    """Run a single-term processor. rf: (num_acq, num_signals, num_samples) or
    (num_signals, num_samples). Returns (value, factor, signals)."""
    desc_t, ct = (_Single32, C.c_float) if dtype == np.float32 else (_Single64, C.c_double)
    lib = _lib()
    f = getattr(lib, "orc_single_" + ("f32" if dtype == np.float32 else "f64"))
    p = C.POINTER(ct)
    f.restype = C.c_int
    f.argtypes = [C.POINTER(desc_t), p, p, C.c_size_t, p, p, p]
    n = spec.num_signals
    keep = {
        "tx": np.ascontiguousarray(spec.tx_xy, dtype=dtype),
        "rx": np.ascontiguousarray(spec.rx_xy, dtype=dtype),
        "apod": None if spec.rx_apod is None else np.ascontiguousarray(spec.rx_apod, dtype=dtype),
        "y": None if spec.acq_y is None else np.ascontiguousarray(spec.acq_y, dtype=dtype),
    }
    d = desc_t(spec.mode, n, spec.num_samples, spec.upsampling, spec.sampling_frequency, spec.propagation_speed,
               spec.center_frequency, spec.peak_offset, spec.dead_zone_m,
               _ptr(keep["tx"], ct), _ptr(keep["rx"], ct), _ptr(keep["apod"], ct),
               spec.focus[0], spec.focus[1], spec.focus[2], spec.first_tx_delay,
               spec.num_acq, _ptr(keep["y"], ct), spec.cf, spec.pcf_gamma, spec.scf_p, int(spec.nthreads))
    rf = np.ascontiguousarray(rf, dtype=dtype)
    assert rf.size == spec.num_acq * n * spec.num_samples, rf.shape
    g = np.ascontiguousarray(grid_xyz, dtype=dtype).reshape(-1, 3)
    npix = g.shape[0]
    value = np.zeros(max(npix, 1), dtype=dtype)
    factor = np.ones(max(npix, 1), dtype=dtype)
    L = spec.num_samples * spec.upsampling
    sig = np.zeros(spec.num_acq * n * L * 2, dtype=dtype) if want_signals else None
    _err(f(C.byref(d), _ptr(rf, ct), _ptr(g, ct), npix, _ptr(value, ct), _ptr(factor, ct), _ptr(sig, ct)))
    if sig is not None:
        sig = sig.view(np.complex64 if dtype == np.float32 else np.complex128).reshape(spec.num_acq, n, L)
    shape = grid_xyz.shape[:-1]
    return value[:npix].reshape(shape), factor[:npix].reshape(shape), sig


def _two_medium_desc_type(ct):
    class TwoMediumDesc(C.Structure):
        _fields_ = [
            ("num_elements", C.c_uint), ("num_elements_mux", C.c_uint),
            ("pitch", ct), ("center_frequency", ct), ("propagation_speed_1", ct), ("propagation_speed_2", ct),
            ("sampling_frequency", ct), ("num_samples", C.c_uint), ("upsampling", C.c_uint),
            ("max_fermat_block_size", ct), ("peak_offset", ct), ("signal_start_offset", C.c_uint),
            ("num_acq", C.c_uint), ("num_tx", C.c_uint), ("num_steps", C.c_uint), ("steps", C.POINTER(C.c_uint)),
            ("num_interface", C.c_uint), ("interface_xz", C.POINTER(ct)), ("rx_apod", C.POINTER(ct)),
            ("cf", C.c_int), ("pcf_gamma", ct), ("nthreads", C.c_int),
        ]
    return TwoMediumDesc


_TwoMedium32 = _two_medium_desc_type(C.c_float)
_TwoMedium64 = _two_medium_desc_type(C.c_double)


@dataclass
class TwoMediumSpec:
    """TwoMediumSTAConfiguration fields plus the processor's constructor and
    process() arguments (VectorialCombinedTwoMediumImagingProcessor).
    steps: (n, 4) (baseElemIdx, baseElem, firstTxElem, lastTxElem);
    interface_xz: (m, 2); rx_apod: (num_elements,)."""
    num_elements: int
    num_elements_mux: int
    pitch: float
    center_frequency: float
    propagation_speed_1: float
    propagation_speed_2: float
    sampling_frequency: float
    num_samples: int
    upsampling: int
    steps: np.ndarray
    interface_xz: np.ndarray
    rx_apod: np.ndarray
    max_fermat_block_size: float = 2.0
    peak_offset: float = 0.0
    signal_start_offset: int = 0
    cf: int = CF_NONE
    pcf_gamma: float = 1.0
    nthreads: int = field(default_factory=lambda: os.cpu_count() or 1)


def two_medium(spec: TwoMediumSpec, rf: np.ndarray, grid_xz: np.ndarray, dtype=np.float64) -> np.ndarray:
    """rf: (num_acq, num_tx, num_elements, num_samples); grid_xz: (ncols, nrows, 2).
    Returns the complex image (ncols, nrows)."""
    desc_t, ct = (_TwoMedium32, C.c_float) if dtype == np.float32 else (_TwoMedium64, C.c_double)
    lib = _lib()
    f = getattr(lib, "orc_two_medium_" + ("f32" if dtype == np.float32 else "f64"))
    p = C.POINTER(ct)
    f.restype = C.c_int
    f.argtypes = [C.POINTER(desc_t), p, p, C.c_uint, C.c_uint, p]
    rf = np.ascontiguousarray(rf, dtype=dtype)
    steps = np.ascontiguousarray(spec.steps, dtype=np.uint32).reshape(-1, 4)
    ifxz = np.ascontiguousarray(spec.interface_xz, dtype=dtype).reshape(-1, 2)
    apod = np.ascontiguousarray(spec.rx_apod, dtype=dtype)
    d = desc_t(spec.num_elements, spec.num_elements_mux, spec.pitch, spec.center_frequency,
               spec.propagation_speed_1, spec.propagation_speed_2, spec.sampling_frequency, spec.num_samples,
               spec.upsampling, spec.max_fermat_block_size, spec.peak_offset, spec.signal_start_offset,
               rf.shape[0], rf.shape[1], steps.shape[0], steps.ctypes.data_as(C.POINTER(C.c_uint)),
               ifxz.shape[0], _ptr(ifxz, ct), _ptr(apod, ct), spec.cf, spec.pcf_gamma, int(spec.nthreads))
    g = np.ascontiguousarray(grid_xz, dtype=dtype)
    out = np.zeros(g.shape[0] * g.shape[1] * 2, dtype=dtype)
    _err(f(C.byref(d), _ptr(rf, ct), _ptr(g, ct), g.shape[0], g.shape[1], _ptr(out, ct)))
    return out.view(np.complex64 if dtype == np.float32 else np.complex128).reshape(g.shape[0], g.shape[1])


def interp_taps(U: int, half_transition: float = 0.2, dtype=np.float64) -> np.ndarray:
    cap = 8192
    ct = C.c_float if dtype == np.float32 else C.c_double
    out = np.zeros(cap, dtype=dtype)
    n = C.c_uint(0)
    f = _lib().orc_interp_taps_f32 if dtype == np.float32 else _lib().orc_interp_taps_f64
    f.argtypes = [C.c_uint, ct, C.POINTER(ct), C.c_uint, C.POINTER(C.c_uint)]
    _err(f(U, half_transition, _ptr(out, ct), cap, C.byref(n)))
    return out[: n.value].copy()


def interp4x_taps() -> np.ndarray:
    out = np.zeros(81, dtype=np.float64)
    f = _lib().orc_interp4x_taps_f64
    f.argtypes = [C.POINTER(C.c_double)]
    n = f(_ptr(out, C.c_double))
    return out[:n]


def upsample(x: np.ndarray, U: int, taps: np.ndarray) -> np.ndarray:
    dtype = taps.dtype
    ct = C.c_float if dtype == np.float32 else C.c_double
    x = np.ascontiguousarray(x, dtype=dtype)
    taps = np.ascontiguousarray(taps)
    out = np.zeros(x.size * U, dtype=dtype)
    f = _lib().orc_upsample_f32 if dtype == np.float32 else _lib().orc_upsample_f64
    f.argtypes = [C.POINTER(ct), C.c_uint, C.c_uint, C.POINTER(ct), C.c_uint, C.POINTER(ct)]
    f(_ptr(x, ct), x.size, U, _ptr(taps, ct), taps.size, _ptr(out, ct))
    return out


def hilbert(x: np.ndarray, dtype=np.float64) -> np.ndarray:
    ct = C.c_float if dtype == np.float32 else C.c_double
    x = np.ascontiguousarray(x, dtype=dtype)
    out = np.zeros(2 * x.size, dtype=dtype)
    f = _lib().orc_hilbert_f32 if dtype == np.float32 else _lib().orc_hilbert_f64
    f.argtypes = [C.POINTER(ct), C.c_uint, C.POINTER(ct)]
    _err(f(_ptr(x, ct), x.size, _ptr(out, ct)))
    return out.view(np.complex64 if dtype == np.float32 else np.complex128)


def envelope(x: np.ndarray, dtype=np.float64) -> np.ndarray:
    """HilbertEnvelope::calculate along the last axis (every row of x)."""
    ct = C.c_float if dtype == np.float32 else C.c_double
    x = np.ascontiguousarray(x, dtype=dtype)
    n = x.shape[-1]
    out = np.zeros_like(x)
    f = _lib().orc_envelope_f32 if dtype == np.float32 else _lib().orc_envelope_f64
    f.argtypes = [C.POINTER(ct), C.c_uint, C.c_uint, C.POINTER(ct)]
    _err(f(_ptr(x, ct), n, x.size // n, _ptr(out, ct)))
    return out


def linear_to_decibels(x: np.ndarray, min_db: float, dtype=np.float32) -> np.ndarray:
    """Util::linearToDecibels(vector, minDecibels) over all of x (a copy)."""
    ct = C.c_float if dtype == np.float32 else C.c_double
    out = np.array(x, dtype=dtype, copy=True, order="C")
    f = _lib().orc_linear_to_decibels_f32 if dtype == np.float32 else _lib().orc_linear_to_decibels_f64
    f.argtypes = [C.POINTER(ct), C.c_size_t, ct]
    _err(f(_ptr(out, ct), out.size, min_db))
    return out


def fft(x: np.ndarray, sign: int = -1) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.complex128)
    out = np.zeros_like(x)
    f = _lib().orc_fft_f64
    f.argtypes = [C.POINTER(C.c_double), C.c_uint, C.c_int, C.POINTER(C.c_double)]
    f(_ptr(x.view(np.float64), C.c_double), x.size, sign, _ptr(out.view(np.float64), C.c_double))
    return out


def remove_dc(x: np.ndarray, begin: int) -> np.ndarray:
    y = np.ascontiguousarray(x, dtype=np.float64).copy()
    f = _lib().orc_remove_dc_f64
    f.argtypes = [C.POINTER(C.c_double), C.c_uint, C.c_uint]
    _err(f(_ptr(y, C.c_double), y.size, begin))
    return y


def scf(values: np.ndarray, p: float) -> float:
    v = np.ascontiguousarray(values, dtype=np.float64)
    return float(_lib().orc_scf_f64(_ptr(v, C.c_double), v.size, p))


def pcf(values: np.ndarray, gamma: float) -> float:
    v = np.ascontiguousarray(values, dtype=np.complex128)
    return float(_lib().orc_pcf_f64(_ptr(v.view(np.float64), C.c_double), v.size, gamma))


def kaiser_beta(tol_db: float) -> float:
    f = _lib().orc_kaiser_beta_f64
    f.restype, f.argtypes = C.c_double, [C.c_double]
    return float(f(tol_db))


def kaiser_size(tol_db: float, transition_width: float) -> int:
    f = _lib().orc_kaiser_size_f64
    f.restype, f.argtypes = C.c_int, [C.c_double, C.c_double]
    return int(f(tol_db, transition_width))


def hilbert_fft_size(n: int) -> int:
    return int(_lib().orc_hilbert_fft_size(n))


def next_fast_even_size(n: int) -> int:
    return int(_lib().orc_next_fast_even_size(n))
