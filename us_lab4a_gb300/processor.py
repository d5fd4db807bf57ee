"""Processors with the reference's plugin interface, running on libusgb.

Each class mirrors one reference processor: constructor arguments,
``prepare(baseElement)`` and ``process(gridData)`` with the same meaning, and
the same exception types:

  VectorialSTAGB300Processor   <- VectorialSTAProcessor<float, XYZValueFactor<float>>
                                  (src/user/processor/VectorialSTAProcessor.h:58-341) and
                                  VectorialSTACUDAProcessor (src/user/processor/VectorialSTACUDAProcessor.h:63-127)
  Vectorial3DSTAGB300Processor <- Vectorial3DSTAProcessor<float> (src/user/processor/Vectorial3DSTAProcessor.h:51-253)
  DefaultSTAGB300Processor     <- DefaultSTAProcessor<float, XYZValueFactor<float>>
                                  (src/user/processor/DefaultSTAProcessor.h:50-227)

``gridData`` is the numpy form of Matrix<XYZValueFactor<float>>: a structured
array of shape (n1, n2) with fields x, y, z, value, factor (config.GRID_DTYPE);
process() reads x, y, z and writes value and factor, like the reference.
Acquisitions follow STAAcquisition: ``prepare(baseElement)`` and
``execute(txElement) -> (numRx, numSamples) array``.
"""
from __future__ import annotations

from typing import Optional, Sequence

import numpy as np

from .config import (AnalyticSignalCoherenceFactorProcessor, CoherenceFactorProcessor, SA3DConfiguration,
                     STAConfiguration, element_x_centered_2d, grid_xyz)
from .engine import FrameSpec, StaEngine
from .errors import InvalidParameterException, InvalidValueException

_CF_NAMES = {"none": "none", "phase_coherence_factor": "pcf", "sign_coherence_factor": "scf",
             "mallart_fink_coherence_factor": "mf"}


class InMemorySTAAcquisition:
    """STAAcquisition over an in-memory (numTx, numRx, numSamples) RF block;
    execute(tx) returns the rows of transmit element tx (absolute index,
    counted from first_tx)."""

    def __init__(self, rf: np.ndarray, first_tx: int = 0):
        self.rf = np.asarray(rf, np.float32)
        self.first_tx = first_tx
        self.base_element = 0

    def prepare(self, base_element: int) -> None:
        self.base_element = base_element

    def execute(self, tx_element: int) -> np.ndarray:
        return self.rf[tx_element - self.first_tx]


class _GB300ProcessorBase:
    _engine: Optional[StaEngine] = None
    _grid_shape = None
    _grid_xyz = None

    def _run(self, grid: np.ndarray, spec_factory, tx_list: Sequence[int]) -> None:
        if grid.ndim != 2:
            raise InvalidParameterException("gridData must be a 2-D matrix of points.")
        if grid.shape[0] == 0:
            raise InvalidValueException("Zero columns in the grid.")
        # Util::resetValueFactor (src/util/Util.h:990-997).
        grid["value"] = 0.0
        grid["factor"] = 1.0
        rows = []
        for t in tx_list:
            rows.append(np.asarray(self.acquisition.execute(t), np.float32))
        ns = rows[0].shape[1]
        if self._engine is None:
            self._engine = StaEngine(spec_factory(ns))
            self._ns = ns
        elif ns != self._ns:
            raise InvalidParameterException("Data size mismatch.")
        for i, r in enumerate(rows):
            self._engine.submit_rf(i, r)
        xyz = grid_xyz(grid)
        if self._grid_xyz is None or xyz.shape != self._grid_xyz.shape or not np.array_equal(xyz, self._grid_xyz):
            self._engine.set_grid(xyz)
            self._grid_xyz = xyz
        value, factor = self._engine.process()
        grid["value"] = value
        grid["factor"] = factor

    def close(self) -> None:
        if self._engine is not None:
            self._engine.close()
            self._engine = None


class VectorialSTAGB300Processor(_GB300ProcessorBase):
    def __init__(self, config: STAConfiguration, acquisition, upsampling_factor: int,
                 coherence_factor: AnalyticSignalCoherenceFactorProcessor, peak_offset: float,
                 rx_apod: Sequence[float], storage: str = "f32"):
        self.config = config
        self.acquisition = acquisition
        self.upsampling_factor = int(upsampling_factor)
        self.coherence_factor = coherence_factor
        self.peak_offset = float(peak_offset)
        self.rx_apod = np.asarray(rx_apod, np.float32).copy()
        self.storage = storage
        if self.rx_apod.size != config.num_elements:
            raise InvalidValueException(f"Wrong rx apodization size: {self.rx_apod.size} "
                                        f"(should be {config.num_elements}).")

    def prepare(self, base_element: int) -> None:
        self.acquisition.prepare(base_element)

    def _spec(self, ns: int) -> FrameSpec:
        c = self.config
        x = element_x_centered_2d(c.num_elements, c.pitch, np.float32)
        rx = np.stack([x, np.zeros_like(x)], axis=1)
        tx = rx[c.first_tx_elem:c.last_tx_elem + 1]
        cf = self.coherence_factor
        return FrameSpec(tx_xy=tx, rx_xy=rx, num_samples=ns, upsampling=self.upsampling_factor,
                         sampling_frequency=c.sampling_frequency, propagation_speed=c.propagation_speed,
                         center_frequency=c.center_frequency, peak_offset=self.peak_offset,
                         dead_zone_m=c.dead_zone_m, rx_apod=self.rx_apod,
                         coherence=_CF_NAMES[cf.method], pcf_gamma=cf.gamma, scf_p=cf.p, storage=self.storage)

    def process(self, grid: np.ndarray) -> None:
        c = self.config
        self._run(grid, self._spec, range(c.first_tx_elem, c.last_tx_elem + 1))


class Vectorial3DSTAGB300Processor(_GB300ProcessorBase):
    def __init__(self, config: SA3DConfiguration, acquisition, upsampling_factor: int,
                 coherence_factor: AnalyticSignalCoherenceFactorProcessor, peak_offset: float,
                 rx_apod: Sequence[float], storage: str = "f32"):
        self.config = config
        self.acquisition = acquisition
        self.upsampling_factor = int(upsampling_factor)
        self.coherence_factor = coherence_factor
        self.peak_offset = float(peak_offset)
        self.rx_apod = np.asarray(rx_apod, np.float32).copy()
        self.storage = storage
        self.base_element = 0
        if self.rx_apod.size != len(config.active_rx_elem):
            raise InvalidValueException(f"Wrong rx apodization size: {self.rx_apod.size} "
                                        f"(should be {len(config.active_rx_elem)}).")

    def prepare(self, base_element: int) -> None:
        if base_element != self.base_element and self._engine is not None:
            self.close()
        self.base_element = base_element
        self.acquisition.prepare(base_element)

    def _spec(self, ns: int) -> FrameSpec:
        c = self.config
        b = self.base_element
        tx = np.asarray([c.tx_elem_pos[b + e] for e in c.active_tx_elem], np.float32)
        rx = np.asarray([c.rx_elem_pos[b + e] for e in c.active_rx_elem], np.float32)
        cf = self.coherence_factor
        return FrameSpec(tx_xy=tx, rx_xy=rx, num_samples=ns, upsampling=self.upsampling_factor,
                         sampling_frequency=c.sampling_frequency, propagation_speed=c.propagation_speed,
                         center_frequency=c.center_frequency, peak_offset=self.peak_offset,
                         dead_zone_m=c.dead_zone_m, rx_apod=self.rx_apod,
                         coherence=_CF_NAMES[cf.method], pcf_gamma=cf.gamma, scf_p=cf.p, storage=self.storage)

    def process(self, grid: np.ndarray) -> None:
        self._run(grid, self._spec, list(self.config.active_tx_elem))


class DefaultSTAGB300Processor(_GB300ProcessorBase):
    """Real-RF STA with the fixed 4x interpolator and the sign coherence factor;
    value is the signed sum (the envelope is taken afterwards by the caller)."""

    upsampling_factor = 4

    def __init__(self, config: STAConfiguration, acquisition, coherence_factor: CoherenceFactorProcessor,
                 peak_offset: float, storage: str = "f32"):
        self.config = config
        self.acquisition = acquisition
        self.coherence_factor = coherence_factor
        self.peak_offset = float(peak_offset)
        self.storage = storage

    def prepare(self, base_element: int) -> None:
        self.acquisition.prepare(base_element)

    def _spec(self, ns: int) -> FrameSpec:
        c = self.config
        x = element_x_centered_2d(c.num_elements, c.pitch, np.float32)
        rx = np.stack([x, np.zeros_like(x)], axis=1)
        tx = rx[c.first_tx_elem:c.last_tx_elem + 1]
        return FrameSpec(tx_xy=tx, rx_xy=rx, num_samples=ns, upsampling=4,
                         sampling_frequency=c.sampling_frequency, propagation_speed=c.propagation_speed,
                         center_frequency=c.center_frequency, peak_offset=self.peak_offset,
                         dead_zone_m=c.dead_zone_m, coherence="scf" if self.coherence_factor.enabled() else "none",
                         scf_p=self.coherence_factor.p, real_path=True, storage=self.storage)

    def process(self, grid: np.ndarray) -> None:
        c = self.config
        self._run(grid, self._spec, range(c.first_tx_elem, c.last_tx_elem + 1))
