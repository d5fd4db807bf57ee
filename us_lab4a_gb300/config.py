"""Host-side configuration objects of the STA/TFM processors.

Mirrors the reference's parameter contract so that a project's files drive
this library unchanged:
  ParameterMap                         src/util/ParameterMap.h:30-120 (key = value files, range checks)
  STAConfiguration                     src/user/configuration/STAConfiguration.h:29-75
  SA3DConfiguration                    src/user/configuration/SA3DConfiguration.h:33-135
  TnRnConfiguration                    src/user/configuration/TnRnConfiguration.h:32-81
  TwoMediumSTAConfiguration            src/user/configuration/TwoMediumSTAConfiguration.h:29-67
  ArrayUtil::calculateTx3DFocusDelay   src/util/ArrayUtil.h:100-144
  ArrayGeometry::getElementXCentered2D src/util/ArrayGeometry.h:37-49
  ArrayUtil::calculateElementPositions src/util/ArrayUtil.h:51-70
  WindowFunction::get                  src/util/WindowFunction.h:237-289
  (Analytic)CoherenceFactorProcessor   src/util/CoherenceFactor.h:63-76, 139-152
Element positions are computed in the processor's float type with the
reference's evaluation order, so they are bit-identical to the reference's.
"""
from __future__ import annotations

import math
import os
from dataclasses import dataclass, field
from typing import Dict, List, Optional

import numpy as np

from .errors import InvalidParameterException, InvalidValueException, MissingValueException

PI = math.pi


# ---------------------------------------------------------------------------
# ParameterMap
# ---------------------------------------------------------------------------
class ParameterMap:
    """key = value file reader with typed, range-checked access."""

    def __init__(self, file_path: Optional[str] = None, text: Optional[str] = None):
        self.file_path = file_path or "<memory>"
        self._map: Dict[str, str] = {}
        if text is None:
            try:
                with open(file_path, "r") as f:
                    text = f.read()
            except OSError as e:
                raise InvalidValueException(f"Could not open the file {file_path}.") from e
        for n, raw in enumerate(text.splitlines(), 1):
            line = raw.strip()
            if not line or line.startswith("#"):
                continue
            if "=" not in line:
                raise InvalidValueException(f"Missing '=' separator at line {n} of file {self.file_path}.")
            k, v = line.split("=", 1)
            k, v = k.strip(), v.strip()
            if not k:
                raise InvalidValueException(f"Missing key at line {n} of file {self.file_path}.")
            if not v:
                raise InvalidValueException(f"Missing value at line {n} of file {self.file_path}.")
            if any(c.isspace() for c in k):
                raise InvalidValueException(f"Key has space at line {n} of file {self.file_path}.")
            if k in self._map:
                raise InvalidValueException(f"Duplicate key '{k}' at line {n} of file {self.file_path}.")
            self._map[k] = v

    @classmethod
    def from_dict(cls, d: Dict[str, object]) -> "ParameterMap":
        return cls(text="\n".join(f"{k} = {v}" for k, v in d.items()))

    def contains(self, key: str) -> bool:
        return key in self._map

    def value(self, key: str, typ=str, min_value=None, max_value=None):
        if key not in self._map:
            raise InvalidValueException(f"Key '{key}' not found in file {self.file_path}.")
        s = self._map[key]
        try:
            if typ is bool:
                if s not in ("true", "false"):
                    raise ValueError(s)
                v = s == "true"
            elif typ is int:
                v = int(s)
            elif typ is float:
                v = float(s)
            else:
                v = s
        except ValueError as e:
            raise InvalidValueException(f"Invalid value for key '{key}' in file {self.file_path}: {e}") from e
        if max_value is not None and v > max_value:
            raise InvalidValueException(f"The value for key '{key}' must be <= {max_value} in file {self.file_path}.")
        if min_value is not None and v < min_value:
            raise InvalidValueException(f"The value for key '{key}' must be >= {min_value} in file {self.file_path}.")
        return v


# ---------------------------------------------------------------------------
# Configurations
# ---------------------------------------------------------------------------
@dataclass
class STAConfiguration:
    """Synthetic transmit aperture, one medium, linear array."""
    num_elements: int
    pitch: float
    center_frequency: float
    sampling_frequency: float
    propagation_speed: float
    first_tx_elem: int = 0
    last_tx_elem: Optional[int] = None
    num_elements_mux: Optional[int] = None
    num_pulses: int = 1
    max_frequency: Optional[float] = None
    acquisition_time: float = 1e-4
    min_gain: float = 0.0
    max_gain: float = 0.0
    acquisition_delay: float = 0.0
    dead_zone_m: float = 0.0
    value_scale: float = 1.0

    def __post_init__(self):
        if self.last_tx_elem is None:
            self.last_tx_elem = self.num_elements - 1
        if self.num_elements_mux is None:
            self.num_elements_mux = self.num_elements
        if self.max_frequency is None:
            self.max_frequency = 2.0 * self.center_frequency
        if self.num_elements < 1:
            raise InvalidParameterException("The number of elements is zero.")
        if not (0 <= self.first_tx_elem <= self.last_tx_elem <= self.num_elements - 1):
            raise InvalidValueException("Invalid first_tx_elem / last_tx_elem.")

    @classmethod
    def from_parameter_map(cls, pm: ParameterMap) -> "STAConfiguration":
        """STAConfiguration::load (src/user/configuration/STAConfiguration.h:55-75)."""
        mux = pm.value("num_elements_mux", int, 1, 1024)
        n = pm.value("num_elements", int, 1, mux)
        first = pm.value("first_tx_elem", int, 0, n - 1)
        last = pm.value("last_tx_elem", int, first, n - 1)
        min_gain = pm.value("min_gain", float, -2000.0, 2000.0)
        return cls(
            num_elements_mux=mux, num_elements=n, first_tx_elem=first, last_tx_elem=last,
            num_pulses=pm.value("num_pulses", int, 1, 100),
            pitch=pm.value("pitch", float, 1.0e-6, 1000.0),
            center_frequency=pm.value("center_frequency", float, 100.0, 100.0e6),
            max_frequency=pm.value("max_frequency", float, 100.0, 100.0e6),
            acquisition_time=pm.value("acquisition_time", float, 1.0e-6, 1.0),
            min_gain=min_gain, max_gain=pm.value("max_gain", float, min_gain, 2000.0),
            propagation_speed=pm.value("propagation_speed_1", float, 100.0, 10000.0),
            acquisition_delay=pm.value("acquisition_delay", float, 0.0, 1.0),
            sampling_frequency=pm.value("sampling_frequency", float, 100.0, 200.0e6),
            dead_zone_m=pm.value("dead_zone_m", float, 0.0, 50.0e-3),
            value_scale=pm.value("value_scale", float, 0.0, 1.0e30),
        )

    @property
    def num_tx(self) -> int:
        return self.last_tx_elem - self.first_tx_elem + 1


def element_x_centered_2d(num_elements: int, pitch: float, dtype=np.float32) -> np.ndarray:
    """ArrayGeometry::getElementXCentered2D in TFloat = dtype:
    xCenter = ((N - 1) * pitch) / 2; x[e] = e * pitch - xCenter."""
    if num_elements == 0:
        raise InvalidParameterException("The number of elements is zero.")
    t = np.dtype(dtype).type
    p = t(pitch)
    x_center = t(t(num_elements - 1) * p) / t(2)
    return np.array([t(t(e) * p) - x_center for e in range(num_elements)], dtype=dtype)


def element_positions_matrix(pitch_x: float, num_x: int, offset_x: float,
                             pitch_y: float, num_y: int, offset_y: float, dtype=np.float32) -> np.ndarray:
    """ArrayUtil::calculateElementPositions: element iy*numX+ix at
    (ix*pitchX - halfW + offsetX, iy*pitchY - halfH + offsetY); halfW is
    evaluated as (numX - 1) * 0.5 * pitchX in double and stored as TFloat."""
    t = np.dtype(dtype).type
    px, py, ox, oy = t(pitch_x), t(pitch_y), t(offset_x), t(offset_y)
    half_w = t((num_x - 1) * 0.5 * float(px))
    half_h = t((num_y - 1) * 0.5 * float(py))
    out = np.empty((num_x * num_y, 2), dtype=dtype)
    for iy in range(num_y):
        for ix in range(num_x):
            out[iy * num_x + ix, 0] = t(t(t(ix) * px) - half_w) + ox
            out[iy * num_x + ix, 1] = t(t(t(iy) * py) - half_h) + oy
    return out


@dataclass
class SA3DConfiguration:
    """3D synthetic aperture with a 2D matrix array (element positions lists
    and active element lists)."""
    tx_elem_pos: np.ndarray          # (n, 2)
    rx_elem_pos: np.ndarray          # (n, 2)
    active_tx_elem: List[int]
    active_rx_elem: List[int]
    center_frequency: float
    sampling_frequency: float
    propagation_speed: float
    dead_zone_m: float = 0.0
    num_elements_mux: int = 1024
    max_frequency: Optional[float] = None
    value_scale: float = 1.0

    @staticmethod
    def parse_active_list(text: str, max_elem: int) -> List[int]:
        """SA3DConfiguration::fillActiveElem: "a b c:d ..." with ranges."""
        out: List[int] = []
        for item in text.split():
            if ":" in item:
                a, b = item.split(":", 1)
                try:
                    e1, e2 = int(a), int(b)
                except ValueError as e:
                    raise InvalidValueException("Missing element in the list of active elements.") from e
                if e1 > max_elem or e2 > max_elem:
                    raise InvalidValueException("Invalid element in the list of active elements.")
                out.extend(range(e1, e2 + 1))
            else:
                try:
                    e = int(item)
                except ValueError as ex:
                    raise InvalidValueException("Missing element in the list of active elements.") from ex
                if e > max_elem:
                    raise InvalidValueException("Invalid element in the list of active elements.")
                out.append(e)
        if not out:
            raise InvalidValueException("Empty list of active elements.")
        return out

    @classmethod
    def from_parameter_maps(cls, sa_pm: ParameterMap, array_pm: ParameterMap, dtype=np.float32) -> "SA3DConfiguration":
        def pos(prefix):
            return element_positions_matrix(
                array_pm.value(prefix + "_pitch_x", float, 1.0e-6, 1000.0),
                int(array_pm.value(prefix + "_num_elem_x", float, 1, 1024)),
                array_pm.value(prefix + "_offset_x", float, -1000.0, 1000.0),
                array_pm.value(prefix + "_pitch_y", float, 1.0e-6, 1000.0),
                int(array_pm.value(prefix + "_num_elem_y", float, 1, 1024)),
                array_pm.value(prefix + "_offset_y", float, -1000.0, 1000.0), dtype)
        tx, rx = pos("tx"), pos("rx")
        mux = sa_pm.value("num_elements_mux", int, 1, 1024)
        if tx.shape[0] > mux or rx.shape[0] > mux:
            raise InvalidParameterException("Error: numElementsMux is less than the number of array elements.")
        return cls(
            tx_elem_pos=tx, rx_elem_pos=rx,
            active_tx_elem=cls.parse_active_list(sa_pm.value("active_tx_elem"), tx.shape[0] - 1),
            active_rx_elem=cls.parse_active_list(sa_pm.value("active_rx_elem"), rx.shape[0] - 1),
            center_frequency=sa_pm.value("center_frequency", float, 100.0, 100.0e6),
            sampling_frequency=sa_pm.value("sampling_frequency", float, 100.0, 200.0e6),
            propagation_speed=sa_pm.value("propagation_speed_1", float, 100.0, 10000.0),
            dead_zone_m=sa_pm.value("dead_zone_m", float, 0.0, 50.0e-3),
            num_elements_mux=mux,
        )


@dataclass
class TnRnConfiguration:
    """Imaging with every element of the active group in transmission and
    reception (one medium): group size, element positions of the whole array."""
    num_elements: int
    tx_elem_pos: np.ndarray          # (n, 2)
    rx_elem_pos: np.ndarray          # (n, 2)
    center_frequency: float
    sampling_frequency: float
    propagation_speed: float
    dead_zone_m: float = 0.0
    num_elements_mux: int = 1024
    max_frequency: Optional[float] = None
    value_scale: float = 1.0

    @classmethod
    def from_parameter_maps(cls, img_pm: ParameterMap, array_pm: ParameterMap, dtype=np.float32) -> "TnRnConfiguration":
        def pos(prefix):
            return element_positions_matrix(
                array_pm.value(prefix + "_pitch_x", float, 1.0e-6, 1000.0),
                int(array_pm.value(prefix + "_num_elem_x", float, 1, 1024)),
                array_pm.value(prefix + "_offset_x", float, -1000.0, 1000.0),
                array_pm.value(prefix + "_pitch_y", float, 1.0e-6, 1000.0),
                int(array_pm.value(prefix + "_num_elem_y", float, 1, 1024)),
                array_pm.value(prefix + "_offset_y", float, -1000.0, 1000.0), dtype)
        tx, rx = pos("tx"), pos("rx")
        mux = img_pm.value("num_elements_mux", int, 1, 1024)
        if tx.shape[0] > mux or rx.shape[0] > mux:
            raise InvalidParameterException("Error: numElementsMux is less than the number of array elements.")
        return cls(
            num_elements=img_pm.value("num_elements", int, 1, mux),
            tx_elem_pos=tx, rx_elem_pos=rx,
            center_frequency=img_pm.value("center_frequency", float, 100.0, 100.0e6),
            sampling_frequency=img_pm.value("sampling_frequency", float, 100.0, 200.0e6),
            propagation_speed=img_pm.value("propagation_speed_1", float, 100.0, 10000.0),
            dead_zone_m=img_pm.value("dead_zone_m", float, 0.0, 50.0e-3),
            num_elements_mux=mux,
        )


@dataclass
class TwoMediumSTAConfiguration:
    """STA through an interface into a second medium (linear array)."""
    num_elements: int
    num_elements_mux: int
    pitch: float
    center_frequency: float
    propagation_speed_1: float
    propagation_speed_2: float
    sampling_frequency: float
    acquisition_time: float = 1e-4
    min_gain: float = 0.0
    max_gain: float = 0.0
    acquisition_delay: float = 0.0
    dead_zone_m: float = 0.0

    @classmethod
    def from_parameter_map(cls, pm: ParameterMap) -> "TwoMediumSTAConfiguration":
        mux = pm.value("num_elements_mux", int, 1, 1024)
        return cls(
            num_elements_mux=mux,
            num_elements=pm.value("num_elements", int, 1, mux),
            pitch=pm.value("pitch", float, 0.01e-3, 10.0e-3),
            center_frequency=pm.value("center_frequency", float, 100.0, 100.0e6),
            acquisition_time=pm.value("acquisition_time", float, 1.0e-6, 1.0),
            min_gain=pm.value("min_gain", float, 0.0, 48.0),
            max_gain=pm.value("max_gain", float, 0.0, 48.0),
            propagation_speed_1=pm.value("propagation_speed_1", float, 100.0, 10000.0),
            propagation_speed_2=pm.value("propagation_speed_2", float, 100.0, 10000.0),
            acquisition_delay=pm.value("acquisition_delay", float, 0.0, 1.0),
            sampling_frequency=pm.value("sampling_frequency", float, 100.0, 200.0e6),
            dead_zone_m=pm.value("dead_zone_m", float, 0.0, 50.0e-3),
        )


def tx_3d_focus_delay(focus_x: float, focus_y: float, focus_z: float, propagation_speed: float,
                      elem_pos: np.ndarray, base_element: int = 0, num_group_elements: Optional[int] = None,
                      dtype=np.float32) -> np.ndarray:
    """Transmit delays (s) of the group elements for a focus (focus_z > 0) or
    a virtual source behind the array (focus_z <= 0): the element farthest
    from the focus fires first (delay 0), resp. the nearest one; evaluated in
    `dtype` in the reference's order (distance3DZ0(pos, focus) * (1 / c))."""
    t = np.dtype(dtype).type
    pos = np.asarray(elem_pos, dtype)
    n = pos.shape[0] - base_element if num_group_elements is None else int(num_group_elements)
    if base_element + n > pos.shape[0]:
        raise InvalidParameterException(
            f"Error: baseElement + numGroupElements > elemPos.size() ( baseElement={base_element} "
            f"numGroupElements={n} elemPos.size()={pos.shape[0]}).")
    grp = pos[base_element:base_element + n]
    inv_c = t(t(1) / t(propagation_speed))
    dx = t(focus_x) - grp[:, 0]
    dy = t(focus_y) - grp[:, 1]
    fz = t(focus_z)
    dt = np.sqrt(dx * dx + dy * dy + fz * fz).astype(dtype) * inv_c
    if focus_z > 0.0:
        return (max(t(0), dt.max()) - dt).astype(dtype)
    return (dt - dt.min()).astype(dtype)


# ---------------------------------------------------------------------------
# Apodization windows (src/util/WindowFunction.h:100-289), evaluated in double.
# ---------------------------------------------------------------------------
def _fade(n: float, out: np.ndarray, at: int, second: bool, fade_out: bool) -> None:
    """WindowFunction::fadeIn/fadeIn2/fadeOut/fadeOut2 (src/util/WindowFunction.h:59-99):
    i runs over 0 <= i < n (n may be non-integer); fadeIn writes i/n,
    fadeIn2 (i+1)/(n+1); the fade-outs write the same ramps mirrored over
    ceil(n) elements."""
    if n <= 0:  # the reference's loop runs no iteration (its 1 / n is then inf, unused)
        return
    c1 = 1.0 / (n + 1.0) if second else 1.0 / n
    m = int(math.ceil(n))
    i = 0
    while i < n:
        v = (i + 1.0) * c1 if second else i * c1
        out[at + (m - i - 1 if fade_out else i)] = v
        i += 1


def window(description: str, size: int, dtype=np.float32) -> np.ndarray:
    """WindowFunction::get (src/util/WindowFunction.h:237-289): rectangular,
    triangular(2), hanning(2), hamming, blackman(2), trapezoidal(2)
    "name nFadeIn nTop nFadeOut"; evaluated in double, stored as dtype."""
    parts = description.split()
    if not parts:
        raise MissingValueException("Missing window function name.")
    name = parts[0]
    n = int(size)
    i = np.arange(n, dtype=np.float64)
    if name in ("trapezoidal", "trapezoidal2"):
        for k, what in enumerate(("fade in", "top", "fade out")):
            if len(parts) < 2 + k:
                raise InvalidParameterException(f"Missing {what} size for the trapezoidal window function.")
        nin, ntop, nout = (int(x) for x in parts[1:4])
        if size != nin + ntop + nout:
            raise InvalidParameterException("Invalid total size for the trapezoidal window function.")
        if n < 2:
            raise InvalidParameterException("The window function size must be >= 2.")
        second = name == "trapezoidal2"
        w = np.zeros(n)
        _fade(nin, w, 0, second, False)
        w[nin:nin + ntop] = 1.0
        _fade(nout, w, nin + ntop, second, True)
        return w.astype(dtype)
    if n < 2:
        raise InvalidParameterException("The window function size must be >= 2.")
    if name == "rectangular":
        w = np.ones(n)
    elif name in ("hanning", "hamming", "blackman"):
        c2 = i * (1.0 / (n - 1.0))
        if name == "hanning":
            w = 0.5 - 0.5 * np.cos(2.0 * PI * c2)
        elif name == "hamming":
            w = 0.54 - 0.46 * np.cos(2.0 * PI * c2)
        else:
            w = 0.42 - 0.5 * np.cos(2.0 * PI * c2) + 0.08 * np.cos(4.0 * PI * c2)
    elif name in ("hanning2", "blackman2"):
        c2 = (i + 1.0) * (1.0 / (n + 1.0))
        if name == "hanning2":
            w = 0.5 - 0.5 * np.cos(2.0 * PI * c2)
        else:
            w = 0.42 - 0.5 * np.cos(2.0 * PI * c2) + 0.08 * np.cos(4.0 * PI * c2)
    elif name in ("triangular", "triangular2"):
        second = name == "triangular2"
        w = np.zeros(n)
        half = 0.5 * (n - 1.0)
        if n % 2 == 0:
            _fade(half, w, 0, second, False)
            _fade(half, w, n // 2, second, True)
        else:
            _fade(half, w, 0, second, False)
            n2 = (n - 1) // 2
            w[n2] = 1.0
            _fade(half, w, n2 + 1, second, True)
    else:
        raise InvalidParameterException(f"Invalid window function name: {name}.")
    return w.astype(dtype)


# ---------------------------------------------------------------------------
# Coherence factor selection.
# ---------------------------------------------------------------------------
@dataclass
class AnalyticSignalCoherenceFactorProcessor:
    """Analytic-path coherence factor: "none", "phase_coherence_factor"
    (reference), plus the library's "sign_coherence_factor" (on the real parts)
    and "mallart_fink_coherence_factor" (no reference counterpart)."""
    method: str = "none"
    gamma: float = 1.0
    p: float = 1.0

    @classmethod
    def from_parameter_map(cls, pm: ParameterMap) -> "AnalyticSignalCoherenceFactorProcessor":
        m = pm.value("analytic_signal_coherence_factor_method")
        if m == "none":
            return cls("none")
        if m == "phase_coherence_factor":
            return cls(m, gamma=pm.value("phase_coherence_factor_gamma", float, 0.0, 100.0))
        if m == "sign_coherence_factor":
            return cls(m, p=pm.value("sign_coherence_factor_p", float, 0.0, 100.0))
        if m == "mallart_fink_coherence_factor":
            return cls(m)
        raise InvalidParameterException(f"Invalid coherence factor method: {m}.")

    def enabled(self) -> bool:
        return self.method != "none"

    def get_constants(self) -> List[float]:
        """PhaseCoherenceFactor::getConstants: [gamma, sigma0, gamma/sigma0] in float."""
        sigma0 = np.float32(PI / math.sqrt(3.0))
        g = np.float32(self.gamma)
        return [float(g), float(sigma0), float(np.float32(g / sigma0))]


@dataclass
class CoherenceFactorProcessor:
    """Real-path coherence factor: "none" or "sign_coherence_factor"."""
    method: str = "none"
    p: float = 1.0

    @classmethod
    def from_parameter_map(cls, pm: ParameterMap) -> "CoherenceFactorProcessor":
        m = pm.value("coherence_factor_method")
        if m == "none":
            return cls("none")
        if m == "sign_coherence_factor":
            return cls(m, p=pm.value("sign_coherence_factor_p", float, 0.0, 100.0))
        raise InvalidParameterException(f"Invalid coherence factor method: {m}.")

    def enabled(self) -> bool:
        return self.method != "none"


# ---------------------------------------------------------------------------
# Grids
# ---------------------------------------------------------------------------
GRID_DTYPE = np.dtype([("x", np.float32), ("y", np.float32), ("z", np.float32),
                       ("value", np.float32), ("factor", np.float32)])


def make_grid(ncols: int, nrows: int) -> np.ndarray:
    """Matrix<XYZValueFactor<float>>(ncols, nrows): value 0, factor 1."""
    g = np.zeros((ncols, nrows), dtype=GRID_DTYPE)
    g["factor"] = 1.0
    return g


def rectangular_grid_xz(x_min: float, x_max: float, ncols: int, z_min: float, z_max: float, nrows: int) -> np.ndarray:
    """x-z rectangular grid, point(col, row) = (x[col], 0, z[row])."""
    g = make_grid(ncols, nrows)
    xs = np.linspace(x_min, x_max, ncols) if ncols > 1 else np.array([x_min])
    zs = np.linspace(z_min, z_max, nrows) if nrows > 1 else np.array([z_min])
    g["x"] = xs[:, None].astype(np.float32)
    g["z"] = zs[None, :].astype(np.float32)
    return g


def rectangular_grid_xyz(x: np.ndarray, y: np.ndarray, z: np.ndarray) -> np.ndarray:
    """3D voxel grid as a (len(x)*len(y)) x len(z) matrix: column index
    ix*len(y)+iy, row index iz."""
    g = make_grid(len(x) * len(y), len(z))
    xx, yy = np.meshgrid(np.asarray(x, np.float32), np.asarray(y, np.float32), indexing="ij")
    g["x"] = xx.reshape(-1)[:, None]
    g["y"] = yy.reshape(-1)[:, None]
    g["z"] = np.asarray(z, np.float32)[None, :]
    return g


def grid_xyz(grid: np.ndarray) -> np.ndarray:
    """(ncols, nrows, 3) float32 coordinates of a grid matrix."""
    return np.ascontiguousarray(np.stack([grid["x"], grid["y"], grid["z"]], axis=-1).astype(np.float32))
