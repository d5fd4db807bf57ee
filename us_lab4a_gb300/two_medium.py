"""Two-medium imaging on libusgb (usgb_two_medium_* of include/usgb.h).

VectorialCombinedTwoMediumGB300Processor mirrors
VectorialCombinedTwoMediumImagingProcessor<float>
(src/user/processor/VectorialCombinedTwoMediumImagingProcessor.h:59-401):
the constructor takes the configuration, the list of acquisitions (one
(num_tx, num_elements, num_samples) array per base-element step), the
upsampling factor, the coherence factor, maxFermatBlockSize, peakOffset and
signalStartOffset; process(step_config_list, interface_point_list, rx_apod,
grid_xz) returns the complex image (ncols, nrows), 0 above the interface.
"""
from __future__ import annotations

import ctypes as C
from typing import Sequence

import numpy as np

from . import native
from .config import AnalyticSignalCoherenceFactorProcessor, TwoMediumSTAConfiguration
from .errors import InvalidParameterException

_CF = {"none": native.USGB_CF_NONE, "phase_coherence_factor": native.USGB_CF_PCF,
       "sign_coherence_factor": native.USGB_CF_SCF, "mallart_fink_coherence_factor": native.USGB_CF_MF,
       "pcf": native.USGB_CF_PCF, "scf": native.USGB_CF_SCF, "mf": native.USGB_CF_MF}
_STORE = {"f32": native.USGB_STORE_F32, "f16": native.USGB_STORE_F16, "bf16": native.USGB_STORE_BF16}


def _fp(a):
    return a.ctypes.data_as(native._FP)


def _steps(step_config_list) -> "C.Array":
    """StepConfiguration list: objects with base_elem_idx, base_elem,
    first_tx_elem, last_tx_elem, or 4-sequences in that order."""
    arr = (native.TwoMediumStep * len(step_config_list))()
    for i, s in enumerate(step_config_list):
        v = (s.base_elem_idx, s.base_elem, s.first_tx_elem, s.last_tx_elem) if hasattr(s, "base_elem") else tuple(s)
        arr[i].base_elem_idx, arr[i].base_elem, arr[i].first_tx_elem, arr[i].last_tx_elem = (int(x) for x in v)
    return arr


class TwoMediumEngine:
    """One usgb_two_medium context: the acquisitions' shape and the processing
    parameters; process() / process_device() form images."""

    def __init__(self, config: TwoMediumSTAConfiguration, num_acquisitions: int, num_tx: int, num_samples: int,
                 upsampling: int, coherence: str = "none", pcf_gamma: float = 1.0, scf_p: float = 1.0,
                 max_fermat_block_size: float = 2.0, peak_offset: float = 0.0, signal_start_offset: int = 0,
                 storage: str = "f32", storage_scale: float = 0.0):
        self._lib = native.load()
        p = native.TwoMediumParams()
        p.num_elements, p.num_elements_mux, p.pitch = config.num_elements, config.num_elements_mux, config.pitch
        p.center_frequency = config.center_frequency
        p.propagation_speed_1, p.propagation_speed_2 = config.propagation_speed_1, config.propagation_speed_2
        p.sampling_frequency, p.num_samples, p.upsampling = config.sampling_frequency, num_samples, upsampling
        p.max_fermat_block_size, p.peak_offset, p.signal_start_offset = (max_fermat_block_size, peak_offset,
                                                                         signal_start_offset)
        p.num_acquisitions, p.num_tx = num_acquisitions, num_tx
        p.coherence, p.pcf_gamma, p.scf_p = _CF[coherence], pcf_gamma, scf_p
        p.storage, p.storage_scale = _STORE[storage], storage_scale
        h = C.c_void_p()
        rc = self._lib.usgb_two_medium_create(C.byref(p), C.byref(h))
        if rc != 0:
            from .errors import from_status
            raise from_status(rc, self._lib.usgb_two_medium_last_error(None).decode())
        self._h = h
        self.shape = (num_acquisitions, num_tx, config.num_elements, num_samples)

    def _check(self, rc: int) -> None:
        if rc != 0:
            from .errors import from_status
            raise from_status(rc, self._lib.usgb_two_medium_last_error(self._h).decode())

    def set_stream(self, stream) -> None:
        self._check(self._lib.usgb_two_medium_set_stream(self._h, C.c_void_p(getattr(stream, "cuda_stream", stream))))

    def process(self, rf: np.ndarray, steps, interface_xz: np.ndarray, rx_apod: np.ndarray,
                grid_xz: np.ndarray) -> np.ndarray:
        """Host arrays: rf (num_acquisitions, num_tx, num_elements, num_samples),
        interface_xz (m, 2), rx_apod (num_elements,), grid_xz (ncols, nrows, 2).
        Returns the complex64 image (ncols, nrows)."""
        r = np.ascontiguousarray(rf, np.float32)
        if r.shape != self.shape:
            raise InvalidParameterException(f"Acquisition shape {r.shape} != {self.shape}.")
        ifxz = np.ascontiguousarray(interface_xz, np.float32).reshape(-1, 2)
        apod = np.ascontiguousarray(rx_apod, np.float32)
        if apod.size != self.shape[2]:
            raise InvalidParameterException(f"Wrong rx apodization size: {apod.size} (should be {self.shape[2]}).")
        g = np.ascontiguousarray(grid_xz, np.float32)
        out = np.zeros(g.shape[0] * g.shape[1] * 2, np.float32)
        st = _steps(steps)
        self._check(self._lib.usgb_two_medium_process(self._h, _fp(r), st, len(st), _fp(ifxz), ifxz.shape[0], _fp(apod),
                                                      _fp(g), g.shape[0], g.shape[1], _fp(out)))
        return out.view(np.complex64).reshape(g.shape[0], g.shape[1])

    def process_device(self, rf, steps, interface_xz, rx_apod, grid_xz, value) -> None:
        """Device tensors (float32, contiguous); value: (ncols, nrows, 2) or
        complex64 (ncols, nrows). Asynchronous on the context's stream."""
        st = _steps(steps)
        self._check(self._lib.usgb_two_medium_process_device(
            self._h, C.c_void_p(rf.data_ptr()), st, len(st), C.c_void_p(interface_xz.data_ptr()),
            interface_xz.numel() // 2, C.c_void_p(rx_apod.data_ptr()), C.c_void_p(grid_xz.data_ptr()),
            grid_xz.shape[0], grid_xz.shape[1], C.c_void_p(value.data_ptr())))

    def synchronize(self) -> None:
        self._check(self._lib.usgb_two_medium_synchronize(self._h))

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.usgb_two_medium_destroy(self._h)
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


class VectorialCombinedTwoMediumGB300Processor:
    def __init__(self, config: TwoMediumSTAConfiguration, acq_data_list: Sequence[np.ndarray], upsampling_factor: int,
                 coherence_factor: AnalyticSignalCoherenceFactorProcessor, max_fermat_block_size: float,
                 peak_offset: float, signal_start_offset: int, storage: str = "f32"):
        if not acq_data_list:
            raise InvalidParameterException("Empty acquisition list.")
        self.config = config
        self.acq_data_list = acq_data_list
        shape = np.shape(acq_data_list[0])
        if any(np.shape(a) != shape for a in acq_data_list):
            raise InvalidParameterException("The acquisitions differ in size.")
        cf = coherence_factor
        self._engine = TwoMediumEngine(config, len(acq_data_list), shape[0], shape[2], int(upsampling_factor),
                                       coherence=cf.method, pcf_gamma=cf.gamma, scf_p=cf.p,
                                       max_fermat_block_size=max_fermat_block_size, peak_offset=peak_offset,
                                       signal_start_offset=signal_start_offset, storage=storage)

    def process(self, step_config_list, interface_point_list, rx_apod, grid_xz: np.ndarray) -> np.ndarray:
        """interface_point_list: (m, 2) (x, z); grid_xz: (ncols, nrows, 2).
        Returns the complex image (ncols, nrows)."""
        rf = np.stack([np.asarray(a, np.float32) for a in self.acq_data_list])
        return self._engine.process(rf, step_config_list, interface_point_list, rx_apod, grid_xz)

    def close(self) -> None:
        self._engine.close()
