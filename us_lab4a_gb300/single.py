"""Single-term 3D processors on libusgb (usgb_single_* of include/usgb.h).

Each class mirrors one reference processor: constructor arguments,
``setTxDelays`` / ``prepare`` / ``process`` (and ``getAcqData`` for the
synthetic-y array) with the same meaning and the same exception types:

  Vectorial3DT1R1SAFTGB300Processor  <- Vectorial3DT1R1SAFTProcessor<float>
                                        (src/user/processor/Vectorial3DT1R1SAFTProcessor.h:51-236)
  Vectorial3DTnRnGB300Processor      <- Vectorial3DTnRnProcessor<float>
                                        (src/user/processor/Vectorial3DTnRnProcessor.h:51-282)
  SynthYVectorial3DTnRnGB300Processor <- SynthYVectorial3DTnRnProcessor<float>
                                        (src/user/processor/SynthYVectorial3DTnRnProcessor.h:51-305)

``gridData`` is the structured (n1, n2) array of config.GRID_DTYPE, as for
the STA processors. Acquisitions: T1R1 follows STAAcquisition
(``prepare(baseElement)``, ``execute(txElement)`` -> rows, of which row 0 is
used, as the reference's processor uses it); TnRn follows TnRnAcquisition
(``prepare(baseElement, txDelays)``, ``execute()`` -> (numElements,
numSamples)).
"""
from __future__ import annotations

import ctypes as C
from typing import Optional, Sequence

import numpy as np

from . import native
from .config import (AnalyticSignalCoherenceFactorProcessor, SA3DConfiguration, TnRnConfiguration, grid_xyz)
from .errors import InvalidParameterException, InvalidStateException, InvalidValueException

_CF = {"none": native.USGB_CF_NONE, "phase_coherence_factor": native.USGB_CF_PCF,
       "sign_coherence_factor": native.USGB_CF_SCF, "mallart_fink_coherence_factor": native.USGB_CF_MF,
       "pcf": native.USGB_CF_PCF, "scf": native.USGB_CF_SCF, "mf": native.USGB_CF_MF}
_STORE = {"f32": native.USGB_STORE_F32, "f16": native.USGB_STORE_F16, "bf16": native.USGB_STORE_BF16}


def _fp(a: Optional[np.ndarray]):
    if a is None:
        return C.cast(None, native._FP)
    return a.ctypes.data_as(native._FP)


class SingleEngine:
    """One single-term processor context (geometry, tables, signal ring, grid).

    mode: native.USGB_SINGLE_T1R1_SAFT / _TNRN / _SYNTH_Y_TNRN. tx_xy: T1R1
    (num_signals, 2) transmit positions; TnRn (>= 1, 2), row 0 = the first
    element of the group. rx_xy: (num_signals, 2). rx_apod: TnRn weights."""

    def __init__(self, mode: int, tx_xy, rx_xy, num_samples: int, upsampling: int, sampling_frequency: float,
                 propagation_speed: float, center_frequency: float, peak_offset: float = 0.0,
                 dead_zone_m: float = 0.0, rx_apod=None, coherence: str = "none", pcf_gamma: float = 1.0,
                 scf_p: float = 1.0, storage: str = "f32", storage_scale: float = 0.0, max_acquisitions: int = 0):
        self._lib = native.load()
        self._tx = np.ascontiguousarray(tx_xy, np.float32).reshape(-1, 2)
        self._rx = np.ascontiguousarray(rx_xy, np.float32).reshape(-1, 2)
        self._apod = None if rx_apod is None else np.ascontiguousarray(rx_apod, np.float32)
        p = native.SingleParams()
        p.mode, p.num_signals, p.num_samples, p.upsampling = mode, self._rx.shape[0], num_samples, upsampling
        p.sampling_frequency, p.propagation_speed, p.center_frequency = (sampling_frequency, propagation_speed,
                                                                         center_frequency)
        p.peak_offset, p.dead_zone_m = peak_offset, dead_zone_m
        p.tx_xy, p.rx_xy, p.rx_apod = _fp(self._tx), _fp(self._rx), _fp(self._apod)
        p.coherence, p.pcf_gamma, p.scf_p = _CF[coherence], pcf_gamma, scf_p
        p.storage, p.storage_scale, p.max_acquisitions = _STORE[storage], storage_scale, max_acquisitions
        h = C.c_void_p()
        rc = self._lib.usgb_single_create(C.byref(p), C.byref(h))
        if rc != 0:
            from .errors import from_status
            raise from_status(rc, self._lib.usgb_single_last_error(None).decode())
        self._h = h
        self.mode = mode
        self.num_signals = int(self._rx.shape[0])
        self.num_samples = int(num_samples)
        self._grid_shape = None

    def _check(self, rc: int) -> None:
        if rc != 0:
            from .errors import from_status
            raise from_status(rc, self._lib.usgb_single_last_error(self._h).decode())

    def set_stream(self, stream) -> None:
        self._check(self._lib.usgb_single_set_stream(self._h, C.c_void_p(getattr(stream, "cuda_stream", stream))))

    def set_tx_delays(self, focus_x: float, focus_y: float, focus_z: float, tx_delays: Sequence[float]) -> None:
        d = np.ascontiguousarray(tx_delays, np.float32)
        self._check(self._lib.usgb_single_set_tx_delays(self._h, focus_x, focus_y, focus_z, _fp(d), d.size))

    def set_grid(self, xyz: np.ndarray) -> None:
        """xyz: (ncols, nrows, 3) host coordinates."""
        g = np.ascontiguousarray(xyz, np.float32)
        self._check(self._lib.usgb_single_set_grid(self._h, _fp(g), g.shape[0], g.shape[1]))
        self._grid_shape = g.shape[:2]

    def set_grid_device(self, xyz) -> None:
        """xyz: torch CUDA float32 (ncols, nrows, 3)."""
        assert xyz.is_cuda and xyz.is_contiguous()
        self._check(self._lib.usgb_single_set_grid_device(self._h, C.c_void_p(xyz.data_ptr()), xyz.shape[0],
                                                          xyz.shape[1]))
        self._grid_shape = tuple(xyz.shape[:2])

    def _outputs(self):
        if self._grid_shape is None:
            raise InvalidStateException("The grid has not been set.")
        return np.empty(self._grid_shape, np.float32), np.empty(self._grid_shape, np.float32)

    def process(self, rf: np.ndarray):
        """T1R1 / TnRn: rf (num_signals, num_samples) host -> (value, factor)."""
        r = np.ascontiguousarray(rf, np.float32)
        if r.shape != (self.num_signals, self.num_samples):
            raise InvalidParameterException(f"RF shape {r.shape} != {(self.num_signals, self.num_samples)}.")
        v, f = self._outputs()
        self._check(self._lib.usgb_single_process(self._h, _fp(r), _fp(v), _fp(f)))
        return v, f

    def process_device(self, rf, value, factor) -> None:
        """T1R1 / TnRn on device tensors (asynchronous on the context's stream)."""
        self._check(self._lib.usgb_single_process_device(self._h, C.c_void_p(rf.data_ptr()), C.c_void_p(value.data_ptr()),
                                                         C.c_void_p(factor.data_ptr())))

    def add_acquisition(self, rf: np.ndarray, y: float) -> None:
        r = np.ascontiguousarray(rf, np.float32)
        if r.shape != (self.num_signals, self.num_samples):
            raise InvalidParameterException(f"RF shape {r.shape} != {(self.num_signals, self.num_samples)}.")
        self._check(self._lib.usgb_single_add_acquisition(self._h, _fp(r), float(y)))

    def add_acquisition_device(self, rf, y: float) -> None:
        self._check(self._lib.usgb_single_add_acquisition_device(self._h, C.c_void_p(rf.data_ptr()), float(y)))

    @property
    def num_acquisitions(self) -> int:
        n = C.c_uint32()
        self._check(self._lib.usgb_single_num_acquisitions(self._h, C.byref(n)))
        return int(n.value)

    def process_window(self, first_acq: int, last_acq: int):
        v, f = self._outputs()
        self._check(self._lib.usgb_single_process_window(self._h, first_acq, last_acq, _fp(v), _fp(f)))
        return v, f

    def process_window_device(self, first_acq: int, last_acq: int, value, factor) -> None:
        self._check(self._lib.usgb_single_process_window_device(self._h, first_acq, last_acq,
                                                                C.c_void_p(value.data_ptr()),
                                                                C.c_void_p(factor.data_ptr())))

    def synchronize(self) -> None:
        self._check(self._lib.usgb_single_synchronize(self._h))

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.usgb_single_destroy(self._h)
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


def _check_grid(grid: np.ndarray) -> None:
    if grid.ndim != 2:
        raise InvalidParameterException("gridData must be a 2-D matrix of points.")
    if grid.shape[0] == 0 or grid.shape[1] == 0:
        raise InvalidValueException("Empty grid.")


class _SingleBase:
    _engine: Optional[SingleEngine] = None
    _grid_xyz = None

    def _set_grid(self, grid: np.ndarray) -> None:
        xyz = grid_xyz(grid)
        if self._grid_xyz is None or xyz.shape != self._grid_xyz.shape or not np.array_equal(xyz, self._grid_xyz):
            self._engine.set_grid(xyz)
            self._grid_xyz = xyz

    def close(self) -> None:
        if self._engine is not None:
            self._engine.close()
            self._engine = None


class Vectorial3DT1R1SAFTGB300Processor(_SingleBase):
    def __init__(self, config: SA3DConfiguration, acquisition, upsampling_factor: int,
                 coherence_factor: AnalyticSignalCoherenceFactorProcessor, peak_offset: float, storage: str = "f32"):
        if len(config.active_tx_elem) != len(config.active_rx_elem):
            raise InvalidParameterException("The T1R1 SAFT processor needs as many active rx as tx elements.")
        self.config = config
        self.acquisition = acquisition
        self.upsampling_factor = int(upsampling_factor)
        self.coherence_factor = coherence_factor
        self.peak_offset = float(peak_offset)
        self.storage = storage
        self.base_element = 0

    def prepare(self, base_element: int) -> None:
        if base_element != self.base_element:
            self.close()
        self.base_element = base_element
        self.acquisition.prepare(base_element)

    def process(self, grid: np.ndarray) -> None:
        _check_grid(grid)
        c = self.config
        grid["value"] = 0.0
        grid["factor"] = 1.0
        rf = np.stack([np.atleast_2d(np.asarray(self.acquisition.execute(t), np.float32))[0]
                       for t in c.active_tx_elem])
        if self._engine is None or self._engine.num_samples != rf.shape[1]:
            self.close()
            b = self.base_element
            tx = np.asarray([c.tx_elem_pos[b + e] for e in c.active_tx_elem], np.float32)
            rx = np.asarray([c.rx_elem_pos[b + e] for e in c.active_rx_elem], np.float32)
            cf = self.coherence_factor
            self._engine = SingleEngine(native.USGB_SINGLE_T1R1_SAFT, tx, rx, rf.shape[1], self.upsampling_factor,
                                        c.sampling_frequency, c.propagation_speed, c.center_frequency,
                                        self.peak_offset, c.dead_zone_m, coherence=cf.method, pcf_gamma=cf.gamma, scf_p=cf.p,
                                        storage=self.storage)
            self._grid_xyz = None
        self._set_grid(grid)
        v, f = self._engine.process(rf)
        grid["value"] = v
        grid["factor"] = f


class _TnRnBase(_SingleBase):
    _mode = native.USGB_SINGLE_TNRN

    def __init__(self, config: TnRnConfiguration, acquisition, upsampling_factor: int,
                 coherence_factor: AnalyticSignalCoherenceFactorProcessor, peak_offset: float,
                 rx_apod: Sequence[float], storage: str = "f32", max_acquisitions: int = 0):
        self.config = config
        self.acquisition = acquisition
        self.upsampling_factor = int(upsampling_factor)
        self.coherence_factor = coherence_factor
        self.peak_offset = float(peak_offset)
        self.rx_apod = np.asarray(rx_apod, np.float32).copy()
        self.storage = storage
        self.max_acquisitions = max_acquisitions
        self.base_element = 0
        self.focus = (0.0, 0.0, 0.0)
        self.tx_delays: list = []
        if self.rx_apod.size != config.num_elements:
            raise InvalidValueException(f"Wrong rx apodization size: {self.rx_apod.size} "
                                        f"(should be {config.num_elements}).")

    def set_tx_delays(self, focus_x: float, focus_y: float, focus_z: float, tx_delays: Sequence[float]) -> None:
        self.focus = (float(focus_x), float(focus_y), float(focus_z))
        self.tx_delays = list(np.asarray(tx_delays, np.float32))
        if self._engine is not None and self.tx_delays:
            self._engine.set_tx_delays(*self.focus, self.tx_delays)

    def prepare(self, base_element: int) -> None:
        c = self.config
        if base_element + c.num_elements > c.num_elements_mux:
            raise InvalidParameterException(f"Invalid base element: {base_element}.")
        if not self.tx_delays:
            raise InvalidStateException("Empty tx delay list.")
        if base_element != self.base_element:
            self.close()
        self.base_element = base_element
        self.acquisition.prepare(base_element, self.tx_delays)

    def _ensure_engine(self, ns: int) -> None:
        if self._engine is not None and self._engine.num_samples == ns:
            return
        self.close()
        c, b, n = self.config, self.base_element, self.config.num_elements
        tx = np.asarray(c.tx_elem_pos[b:b + 1], np.float32)
        rx = np.asarray(c.rx_elem_pos[b:b + n], np.float32)
        cf = self.coherence_factor
        self._engine = SingleEngine(self._mode, tx, rx, ns, self.upsampling_factor, c.sampling_frequency,
                                    c.propagation_speed, c.center_frequency, self.peak_offset, c.dead_zone_m,
                                    rx_apod=self.rx_apod, coherence=cf.method, pcf_gamma=cf.gamma, scf_p=cf.p,
                                    storage=self.storage, max_acquisitions=self.max_acquisitions)
        self._engine.set_tx_delays(*self.focus, self.tx_delays)
        self._grid_xyz = None


class Vectorial3DTnRnGB300Processor(_TnRnBase):
    def process(self, grid: np.ndarray) -> None:
        _check_grid(grid)
        grid["value"] = 0.0
        grid["factor"] = 1.0
        rf = np.asarray(self.acquisition.execute(), np.float32)
        if rf.shape[0] != self.config.num_elements:
            raise InvalidValueException("Wrong number of signals in the acquisition.")
        self._ensure_engine(rf.shape[1])
        self._set_grid(grid)
        v, f = self._engine.process(rf)
        grid["value"] = v
        grid["factor"] = f


class SynthYVectorial3DTnRnGB300Processor(_TnRnBase):
    """Keeps the last `max_acquisitions` prepared acquisitions on the device
    (the reference keeps every acquisition in host memory)."""
    _mode = native.USGB_SINGLE_SYNTH_Y_TNRN

    def __init__(self, config: TnRnConfiguration, acquisition, upsampling_factor: int,
                 coherence_factor: AnalyticSignalCoherenceFactorProcessor, peak_offset: float,
                 rx_apod: Sequence[float], storage: str = "f32", max_acquisitions: int = 64):
        super().__init__(config, acquisition, upsampling_factor, coherence_factor, peak_offset, rx_apod, storage,
                         max_acquisitions)
        self._y: list = []

    def get_acq_data(self, y: float) -> None:
        rf = np.asarray(self.acquisition.execute(), np.float32)
        if rf.shape[0] != self.config.num_elements:
            raise InvalidValueException("Wrong number of signals in the acquisition.")
        if self._engine is None:
            self._ensure_engine(rf.shape[1])
        elif rf.shape[1] != self._engine.num_samples:
            raise InvalidValueException("All acquisitions must have the same number of samples.")
        self._engine.add_acquisition(rf, y)
        self._y.append(np.float32(y))

    # The reference's name.
    getAcqData = get_acq_data

    def process(self, first_acq: int, last_acq: int, grid: np.ndarray) -> None:
        _check_grid(grid)
        if not self.tx_delays:
            raise InvalidStateException("Empty tx delay list.")
        if self._engine is None:
            raise InvalidStateException("No acquisition has been added.")
        grid["value"] = 0.0
        grid["factor"] = 1.0
        self._set_grid(grid)
        v, f = self._engine.process_window(first_acq, last_acq)
        grid["value"] = v
        grid["factor"] = f
        grid["y"] = self._y[(first_acq + last_acq) // 2]
