"""Python handle of one libusgb context (one frame geometry + processing choice).

``StaEngine`` owns a ``usgb_ctx``: host entry points (``submit_rf`` +
``process``: host RF in, host image out, the reference processor's data flow)
and device entry points taking torch CUDA tensors (resident RF, asynchronous on
the engine's stream).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from typing import Optional

import numpy as np

from . import native
from .errors import InvalidParameterException

STORAGE = {"f32": native.USGB_STORE_F32, "f16": native.USGB_STORE_F16, "bf16": native.USGB_STORE_BF16}
COHERENCE = {"none": native.USGB_CF_NONE, "pcf": native.USGB_CF_PCF, "scf": native.USGB_CF_SCF,
             "mf": native.USGB_CF_MF}


@dataclass
class FrameSpec:
    """Everything one context needs (fields of usgb_sta_params)."""
    tx_xy: np.ndarray                 # (num_tx, 2) float32, m
    rx_xy: np.ndarray                 # (num_rx, 2) float32, m
    num_samples: int
    upsampling: int
    sampling_frequency: float
    propagation_speed: float
    center_frequency: float
    peak_offset: float = 0.0
    dead_zone_m: float = 0.0
    rx_apod: Optional[np.ndarray] = None
    coherence: str = "none"          # none | pcf | scf | mf
    pcf_gamma: float = 1.0
    scf_p: float = 1.0
    real_path: bool = False           # DefaultSTAProcessor arithmetic
    storage: str = "f32"              # f32 | f16 | bf16
    storage_scale: float = 1.0

    @property
    def num_tx(self) -> int:
        return int(self.tx_xy.shape[0])

    @property
    def num_rx(self) -> int:
        return int(self.rx_xy.shape[0])

    @property
    def signal_length(self) -> int:
        return self.num_samples * self.upsampling


class StaEngine:
    def __init__(self, spec: FrameSpec):
        self.spec = spec
        self._lib = native.load()
        if spec.coherence not in COHERENCE:
            raise InvalidParameterException(f"Invalid coherence factor method: {spec.coherence}.")
        if spec.storage not in STORAGE:
            raise InvalidParameterException(f"Invalid storage type: {spec.storage}.")
        self._tx = np.ascontiguousarray(spec.tx_xy, np.float32)
        self._rx = np.ascontiguousarray(spec.rx_xy, np.float32)
        self._apod = None if spec.rx_apod is None else np.ascontiguousarray(spec.rx_apod, np.float32)
        p = native.StaParams()
        p.num_tx, p.num_rx = self._tx.shape[0], self._rx.shape[0]
        p.num_samples, p.upsampling = spec.num_samples, spec.upsampling
        p.signal_path = native.USGB_PATH_REAL if spec.real_path else native.USGB_PATH_ANALYTIC
        p.sampling_frequency, p.propagation_speed = spec.sampling_frequency, spec.propagation_speed
        p.center_frequency, p.peak_offset, p.dead_zone_m = spec.center_frequency, spec.peak_offset, spec.dead_zone_m
        p.tx_xy = self._tx.ctypes.data_as(C.POINTER(C.c_float))
        p.rx_xy = self._rx.ctypes.data_as(C.POINTER(C.c_float))
        p.rx_apod = None if self._apod is None else self._apod.ctypes.data_as(C.POINTER(C.c_float))
        p.coherence = COHERENCE[spec.coherence]
        p.pcf_gamma, p.scf_p = spec.pcf_gamma, spec.scf_p
        p.storage, p.storage_scale = STORAGE[spec.storage], spec.storage_scale
        h = C.c_void_p()
        native.check(self._lib.usgb_create(C.byref(p), C.byref(h)), None)
        self._h = h
        self.ncols = self.nrows = 0

    # -- lifetime ---------------------------------------------------------
    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.usgb_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _check(self, rc: int) -> None:
        native.check(rc, self._h)

    # -- info -------------------------------------------------------------
    def signal_info(self):
        L, N, stride = C.c_uint32(), C.c_uint32(), C.c_uint32()
        nbytes = C.c_size_t()
        self._check(self._lib.usgb_signal_info(self._h, C.byref(L), C.byref(N), C.byref(stride), C.byref(nbytes)))
        return {"signal_length": L.value, "fft_size": N.value, "signal_stride": stride.value,
                "signal_bytes": nbytes.value}

    def set_das_variant(self, variant: int, tile_rows: int = 0, stage_bytes: int = 0, stages: int = 0) -> None:
        """0: plain kernel; 1: staged kernel; 2: receiver-group kernel on
        32-column tiles (tile_rows in {4, 8, 16}); 3: receiver-group kernel on
        64-column tiles (tile_rows 1 to 8); 4: the same with two grid rows per
        thread row (64 x 2 * tile_rows tiles); stages in [2, 16]."""
        self._check(self._lib.usgb_set_das_variant(self._h, variant, tile_rows, stage_bytes, stages))

    DELAY_PRECISION = {"auto": 0, "fp32": 1, "fp64": 2}

    def set_delay_precision(self, mode: str) -> None:
        """"auto" (FP64 geometry only for tiles whose delays exceed 32768
        samples), "fp32" (as the reference) or "fp64"; staged kernel only."""
        self._check(self._lib.usgb_set_delay_precision(self._h, self.DELAY_PRECISION[mode]))

    def das_config(self):
        v, r, b, n = C.c_int(), C.c_uint32(), C.c_uint32(), C.c_uint32()
        self._check(self._lib.usgb_get_das_config(self._h, C.byref(v), C.byref(r), C.byref(b), C.byref(n)))
        return {"variant": v.value, "tile_rows": r.value, "stage_bytes": b.value, "stages": n.value}

    def autotune_das(self, signals, value, factor, iterations: int = 3) -> float:
        """Times the delay-and-sum configurations on these prepared signals and
        keeps the fastest; returns its time in ms."""
        ms = C.c_float()
        self._check(self._lib.usgb_autotune_das(self._h, C.c_void_p(signals.data_ptr()), C.c_void_p(value.data_ptr()),
                                                C.c_void_p(factor.data_ptr()), iterations, C.byref(ms)))
        return ms.value

    # -- host path (reference data flow) -----------------------------------
    def set_grid(self, xyz: np.ndarray) -> None:
        """xyz: (ncols, nrows, 3) float32."""
        xyz = np.ascontiguousarray(xyz, np.float32)
        ncols, nrows = xyz.shape[0], xyz.shape[1]
        self._check(self._lib.usgb_set_grid(self._h, xyz.ctypes.data_as(C.POINTER(C.c_float)), ncols, nrows))
        self.ncols, self.nrows = ncols, nrows

    def submit_rf(self, tx: int, rf_rows: np.ndarray) -> None:
        rf_rows = np.ascontiguousarray(rf_rows, np.float32)
        nrx, ns = rf_rows.shape
        self._check(self._lib.usgb_submit_rf(self._h, tx, rf_rows.ctypes.data_as(C.POINTER(C.c_float)), nrx, ns))

    def process(self):
        """Returns (value, factor), each (ncols, nrows) float32."""
        value = np.empty((self.ncols, self.nrows), np.float32)
        factor = np.empty((self.ncols, self.nrows), np.float32)
        self._check(self._lib.usgb_process(self._h, value.ctypes.data_as(C.POINTER(C.c_float)),
                                           factor.ctypes.data_as(C.POINTER(C.c_float))))
        return value, factor

    def process_submitted(self, rf: np.ndarray):
        """Whole frame through the reference's data flow: one usgb_submit_rf per
        transmit event, then usgb_process."""
        for t in range(rf.shape[0]):
            self.submit_rf(t, rf[t])
        return self.process()

    def process_host(self, rf: np.ndarray):
        """Whole frame from a (num_tx, num_rx, ns) host array (usgb_process_rf:
        read in place where the device reaches host memory directly)."""
        rf = np.ascontiguousarray(rf, np.float32)
        value = np.empty((self.ncols, self.nrows), np.float32)
        factor = np.empty((self.ncols, self.nrows), np.float32)
        self._check(self._lib.usgb_process_rf(self._h, C.c_void_p(rf.ctypes.data), C.c_void_p(value.ctypes.data),
                                              C.c_void_p(factor.ctypes.data)))
        return value, factor

    def set_host_direct(self, enable: bool) -> None:
        self._check(self._lib.usgb_set_host_direct(self._h, int(enable)))

    def host_direct(self):
        """(available, enabled) for direct host-memory access."""
        a, e = C.c_int(), C.c_int()
        self._check(self._lib.usgb_get_host_direct(self._h, C.byref(a), C.byref(e)))
        return bool(a.value), bool(e.value)

    # -- device path (torch CUDA tensors) ---------------------------------
    def set_stream(self, stream) -> None:
        """stream: torch.cuda.Stream (or raw cudaStream_t int)."""
        ptr = getattr(stream, "cuda_stream", stream)
        self._check(self._lib.usgb_set_stream(self._h, C.c_void_p(ptr)))

    def set_grid_device(self, xyz) -> None:
        assert xyz.is_cuda and xyz.dtype.is_floating_point and xyz.is_contiguous()
        ncols, nrows = int(xyz.shape[0]), int(xyz.shape[1])
        self._check(self._lib.usgb_set_grid_device(self._h, C.c_void_p(xyz.data_ptr()), ncols, nrows))
        self.ncols, self.nrows = ncols, nrows

    def process_device(self, rf, value, factor) -> None:
        for t in (rf, value, factor):
            assert t.is_cuda and t.is_contiguous()
        self._check(self._lib.usgb_process_device(self._h, C.c_void_p(rf.data_ptr()), C.c_void_p(value.data_ptr()),
                                                  C.c_void_p(factor.data_ptr())))

    def prepare_signals_device(self, rf, signals) -> None:
        self._check(self._lib.usgb_prepare_signals_device(self._h, C.c_void_p(rf.data_ptr()),
                                                          C.c_void_p(signals.data_ptr())))

    def delay_and_sum_device(self, signals, value, factor) -> None:
        self._check(self._lib.usgb_delay_and_sum_device(self._h, C.c_void_p(signals.data_ptr()),
                                                        C.c_void_p(value.data_ptr()), C.c_void_p(factor.data_ptr())))

    def synchronize(self) -> None:
        self._check(self._lib.usgb_synchronize(self._h))

    def set_wait_test(self, wait_limit_us: int = 0, skip_stage: int = 0) -> None:
        """Test hook of the timeout path (usgb_set_wait_test): the staged
        delay-and-sum's bounded waits give up after wait_limit_us (0: 2 s), and
        skip_stage = k > 0 leaves every tile's k-th stage unarmed."""
        self._check(self._lib.usgb_set_wait_test(self._h, int(wait_limit_us), int(skip_stage)))
