"""ctypes wrapper of oracle/_ref/libref.so: the reference's own STA processors
compiled from their sources with the shim headers of oracle/refbuild/.

Test infrastructure only. The library exists only where the reference sources
were present at build time (this container), so every user checks
``available()`` first.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(_HERE, "_ref", "libref.so")
# The reference project's root: the environment variable US_LAB4A_REFERENCE,
# else the read-only checkout this recipe was written against. Every user of
# the reference sources (the refbuild Makefile, the fixture script, the tests
# that read its test files or compile inside its headers) takes it from here.
REF_ROOT = os.environ.get("US_LAB4A_REFERENCE") or "/root/reference"
REF_SRC = os.path.join(REF_ROOT, "src")
REF_TEST = os.path.join(REF_ROOT, "test")
_lib = None


def build(force: bool = False) -> bool:
    """Compile libref.so when the reference sources are present."""
    if not os.path.isdir(REF_SRC):
        return False
    cmd = ["make", "-s", "-C", os.path.join(_HERE, "refbuild"), "REF=" + REF_ROOT]
    if force:
        cmd.append("-B")
    subprocess.run(cmd, check=True)
    return os.path.exists(LIB)


def available() -> bool:
    return os.path.exists(LIB)


def _desc(ct):
    class RefDesc(C.Structure):
        _fields_ = [
            ("num_elements", C.c_uint), ("first_tx_elem", C.c_uint), ("last_tx_elem", C.c_uint), ("pitch", ct),
            ("is_3d", C.c_int), ("tx_nx", C.c_uint), ("tx_ny", C.c_uint), ("rx_nx", C.c_uint), ("rx_ny", C.c_uint),
            ("tx_pitch_x", ct), ("tx_pitch_y", ct), ("rx_pitch_x", ct), ("rx_pitch_y", ct),
            ("num_samples", C.c_uint), ("upsampling", C.c_uint),
            ("sampling_frequency", ct), ("propagation_speed", ct), ("center_frequency", ct),
            ("peak_offset", ct), ("dead_zone_m", ct), ("rx_apod", C.POINTER(ct)),
            ("cf", C.c_int), ("pcf_gamma", ct), ("scf_p", ct), ("real_path", C.c_int),
        ]
    return RefDesc


_D32, _D64 = _desc(C.c_float), _desc(C.c_double)


def _load():
    global _lib
    if _lib is None:
        _lib = C.CDLL(LIB)
        _lib.ref_last_error.restype = C.c_char_p
        for name, ct, d in (("f32", C.c_float, _D32), ("f64", C.c_double, _D64)):
            f = getattr(_lib, "ref_process_" + name)
            p = C.POINTER(ct)
            f.argtypes = [C.POINTER(d), p, p, C.c_uint, C.c_uint, p, p]
            f.restype = C.c_int
    return _lib


def process(*, rf: np.ndarray, grid_xyz: np.ndarray, num_samples: int, upsampling: int, fs: float, c: float,
            fc: float, peak_offset: float = 0.0, dead_zone_m: float = 0.0, rx_apod=None, cf: int = 0,
            pcf_gamma: float = 1.0, scf_p: float = 1.0, real_path: bool = False,
            num_elements: int = 0, first_tx: int = 0, last_tx: int = 0, pitch: float = 0.0,
            matrix=None, dtype=np.float32, threads: int = 0):
    """Run the reference processor. 2D: num_elements/first_tx/last_tx/pitch.
    3D: matrix = (nx, ny, pitch_x, pitch_y) for both tx and rx arrays.
    cf: 0 none, 1 PCF (analytic path), 2 SCF (real path).
    Returns (value, factor) with grid_xyz.shape[:2]."""
    lib = _load()
    if threads:
        os.environ["USGB_REF_THREADS"] = str(threads)
    ct = C.c_float if dtype == np.float32 else C.c_double
    D = _D32 if dtype == np.float32 else _D64
    nrx = num_elements if matrix is None else matrix[0] * matrix[1]
    apod = np.ascontiguousarray(np.ones(nrx) if rx_apod is None else rx_apod, dtype=dtype)
    d = D()
    d.num_elements, d.first_tx_elem, d.last_tx_elem, d.pitch = num_elements, first_tx, last_tx, pitch
    if matrix is not None:
        d.is_3d = 1
        d.tx_nx = d.rx_nx = matrix[0]
        d.tx_ny = d.rx_ny = matrix[1]
        d.tx_pitch_x = d.rx_pitch_x = matrix[2]
        d.tx_pitch_y = d.rx_pitch_y = matrix[3]
    d.num_samples, d.upsampling = num_samples, upsampling
    d.sampling_frequency, d.propagation_speed, d.center_frequency = fs, c, fc
    d.peak_offset, d.dead_zone_m = peak_offset, dead_zone_m
    d.rx_apod = apod.ctypes.data_as(C.POINTER(ct))
    d.cf, d.pcf_gamma, d.scf_p, d.real_path = cf, pcf_gamma, scf_p, int(real_path)
    rf = np.ascontiguousarray(rf, dtype=dtype)
    g = np.ascontiguousarray(grid_xyz, dtype=dtype)
    n1, n2 = g.shape[0], g.shape[1]
    value = np.zeros((n1, n2), dtype)
    factor = np.zeros((n1, n2), dtype)
    f = lib.ref_process_f32 if dtype == np.float32 else lib.ref_process_f64
    rc = f(C.byref(d), rf.ctypes.data_as(C.POINTER(ct)), g.ctypes.data_as(C.POINTER(ct)), n1, n2,
           value.ctypes.data_as(C.POINTER(ct)), factor.ctypes.data_as(C.POINTER(ct)))
    if rc != 0:
        raise RuntimeError(lib.ref_last_error().decode())
    return value, factor


def _single_desc(ct):
    class RefSingleDesc(C.Structure):
        _fields_ = [
            ("mode", C.c_int), ("nx", C.c_uint), ("ny", C.c_uint), ("pitch_x", ct), ("pitch_y", ct),
            ("num_active", C.c_uint), ("active", C.POINTER(C.c_uint)),
            ("base_element", C.c_uint), ("num_elements", C.c_uint),
            ("num_samples", C.c_uint), ("upsampling", C.c_uint),
            ("sampling_frequency", ct), ("propagation_speed", ct), ("center_frequency", ct),
            ("peak_offset", ct), ("dead_zone_m", ct), ("rx_apod", C.POINTER(ct)),
            ("focus_x", ct), ("focus_y", ct), ("focus_z", ct),
            ("num_acq", C.c_uint), ("acq_y", C.POINTER(ct)), ("first_acq", C.c_uint), ("last_acq", C.c_uint),
            ("cf", C.c_int), ("pcf_gamma", ct), ("tx_delays_out", C.POINTER(ct)),
        ]
    return RefSingleDesc


_S32, _S64 = _single_desc(C.c_float), _single_desc(C.c_double)


def single(*, mode: int, rf: np.ndarray, grid_xyz: np.ndarray, matrix, num_samples: int, upsampling: int,
           fs: float, c: float, fc: float, peak_offset: float = 0.0, dead_zone_m: float = 0.0,
           active=None, base_element: int = 0, num_elements: int = 0, rx_apod=None, focus=(0.0, 0.0, 0.0),
           acq_y=None, first_acq: int = 0, last_acq: int = 0, cf: int = 0, pcf_gamma: float = 1.0,
           dtype=np.float32):
    """Run the reference's Vectorial3DT1R1SAFTProcessor (mode 0),
    Vectorial3DTnRnProcessor (1) or SynthYVectorial3DTnRnProcessor (2) on a
    matrix array = (nx, ny, pitch_x, pitch_y) (tx = rx positions).
    T1R1: rf (len(active), num_samples). TnRn: rf (num_elements, num_samples);
    synthetic y: rf (len(acq_y), num_elements, num_samples), window
    [first_acq, last_acq]. Returns (value, factor, tx_delays)."""
    lib = _load()
    ct = C.c_float if dtype == np.float32 else C.c_double
    D = _S32 if dtype == np.float32 else _S64
    f = lib.ref_single_f32 if dtype == np.float32 else lib.ref_single_f64
    p = C.POINTER(ct)
    f.argtypes = [C.POINTER(D), p, p, C.c_uint, C.c_uint, p, p]
    f.restype = C.c_int
    d = D()
    d.mode = mode
    d.nx, d.ny, d.pitch_x, d.pitch_y = matrix
    act = np.ascontiguousarray(np.arange(matrix[0] * matrix[1]) if active is None else active, dtype=np.uint32)
    d.num_active = act.size
    d.active = act.ctypes.data_as(C.POINTER(C.c_uint))
    d.base_element, d.num_elements = base_element, num_elements
    d.num_samples, d.upsampling = num_samples, upsampling
    d.sampling_frequency, d.propagation_speed, d.center_frequency = fs, c, fc
    d.peak_offset, d.dead_zone_m = peak_offset, dead_zone_m
    apod = np.ascontiguousarray(np.ones(max(num_elements, 1)) if rx_apod is None else rx_apod, dtype=dtype)
    d.rx_apod = apod.ctypes.data_as(p)
    d.focus_x, d.focus_y, d.focus_z = focus
    ys = np.ascontiguousarray(np.zeros(1) if acq_y is None else acq_y, dtype=dtype)
    d.num_acq = ys.size if acq_y is not None else 0
    d.acq_y = ys.ctypes.data_as(p)
    d.first_acq, d.last_acq = first_acq, last_acq
    d.cf, d.pcf_gamma = cf, pcf_gamma
    txd = np.zeros(max(num_elements, 1), dtype)
    d.tx_delays_out = txd.ctypes.data_as(p)
    rf = np.ascontiguousarray(rf, dtype=dtype)
    g = np.ascontiguousarray(grid_xyz, dtype=dtype)
    n1, n2 = g.shape[0], g.shape[1]
    value = np.zeros((n1, n2), dtype)
    factor = np.zeros((n1, n2), dtype)
    rc = f(C.byref(d), rf.ctypes.data_as(p), g.ctypes.data_as(p), n1, n2, value.ctypes.data_as(p),
           factor.ctypes.data_as(p))
    if rc != 0:
        raise RuntimeError(lib.ref_last_error().decode())
    return value, factor, txd[:num_elements]


def _two_medium_desc(ct):
    class RefTwoMediumDesc(C.Structure):
        _fields_ = [
            ("num_elements", C.c_uint), ("num_elements_mux", C.c_uint),
            ("pitch", ct), ("center_frequency", ct), ("propagation_speed_1", ct), ("propagation_speed_2", ct),
            ("sampling_frequency", ct), ("num_samples", C.c_uint), ("upsampling", C.c_uint),
            ("max_fermat_block_size", ct), ("peak_offset", ct), ("signal_start_offset", C.c_uint),
            ("num_acq", C.c_uint), ("num_tx", C.c_uint), ("num_steps", C.c_uint), ("steps", C.POINTER(C.c_uint)),
            ("num_interface", C.c_uint), ("interface_xz", C.POINTER(ct)), ("rx_apod", C.POINTER(ct)),
            ("cf", C.c_int), ("pcf_gamma", ct),
        ]
    return RefTwoMediumDesc


_TM32, _TM64 = _two_medium_desc(C.c_float), _two_medium_desc(C.c_double)


def two_medium(spec, rf: np.ndarray, grid_xz: np.ndarray, dtype=np.float32) -> np.ndarray:
    """Run the reference's VectorialCombinedTwoMediumImagingProcessor on an
    oracle.TwoMediumSpec; rf (num_acq, num_tx, num_elements, num_samples),
    grid_xz (ncols, nrows, 2). Returns the complex image (ncols, nrows)."""
    lib = _load()
    ct = C.c_float if dtype == np.float32 else C.c_double
    D = _TM32 if dtype == np.float32 else _TM64
    f = lib.ref_two_medium_f32 if dtype == np.float32 else lib.ref_two_medium_f64
    p = C.POINTER(ct)
    f.argtypes = [C.POINTER(D), p, p, C.c_uint, C.c_uint, p]
    f.restype = C.c_int
    rf = np.ascontiguousarray(rf, dtype=dtype)
    steps = np.ascontiguousarray(spec.steps, dtype=np.uint32).reshape(-1, 4)
    ifxz = np.ascontiguousarray(spec.interface_xz, dtype=dtype).reshape(-1, 2)
    apod = np.ascontiguousarray(spec.rx_apod, dtype=dtype)
    d = D(spec.num_elements, spec.num_elements_mux, spec.pitch, spec.center_frequency, spec.propagation_speed_1,
          spec.propagation_speed_2, spec.sampling_frequency, spec.num_samples, spec.upsampling,
          spec.max_fermat_block_size, spec.peak_offset, spec.signal_start_offset, rf.shape[0], rf.shape[1],
          steps.shape[0], steps.ctypes.data_as(C.POINTER(C.c_uint)), ifxz.shape[0], ifxz.ctypes.data_as(p),
          apod.ctypes.data_as(p), spec.cf, spec.pcf_gamma)
    g = np.ascontiguousarray(grid_xz, dtype=dtype)
    out = np.zeros(g.shape[0] * g.shape[1] * 2, dtype=dtype)
    rc = f(C.byref(d), rf.ctypes.data_as(p), g.ctypes.data_as(p), g.shape[0], g.shape[1], out.ctypes.data_as(p))
    if rc != 0:
        raise RuntimeError(lib.ref_last_error().decode())
    return out.view(np.complex64 if dtype == np.float32 else np.complex128).reshape(g.shape[0], g.shape[1])


def window(description: str, size: int) -> np.ndarray:
    """The reference's WindowFunction::get<float>(description, size)
    (src/util/WindowFunction.h:237-289), from the compiled reference."""
    lib = _load()
    f = lib.ref_window_f32
    f.argtypes = [C.c_char_p, C.c_uint, C.POINTER(C.c_float)]
    f.restype = C.c_int
    out = np.zeros(max(size, 1), np.float32)
    if f(description.encode(), size, out.ctypes.data_as(C.POINTER(C.c_float))) != 0:
        raise ValueError(lib.ref_last_error().decode())
    return out[:size]
