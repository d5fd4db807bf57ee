"""Saved acquisitions and images in the reference's HDF5 files (usgb_h5_* of
include/usgb.h, host code in libusgb.so; no GPU needed).

  read / write               HDF5Util::load / HDF5Util::save (src/util/HDF5Util.h:181-287)
  tx_elem_signals_path       FileUtil::txElemSignalsPath (src/util/FileUtil.cpp:58-65)
  SavedSTAAcquisition        SavedSTAAcquisition<float> (src/user/acquisition/SavedSTAAcquisition.h:30-90)
  save_image / load_image    Project::saveImageToHDF5 / saveFactorToHDF5 / saveXYZToHDF5 and
                             loadImageFromHDF5 (src/Project.h:106-118): image_value.h5 "value",
                             image_factor.h5 "factor", image_x / image_y / image_z.h5
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import native
from .errors import InvalidParameterException, from_status

FILE_SUFFIX = ".h5"


def _check(rc: int) -> None:
    if rc != 0:
        raise from_status(rc, native.load().usgb_h5_last_error().decode())


def info(path: str, dataset: str):
    """(rank, n1, n2) of a dataset (rank-1 datasets: n1 = 1)."""
    lib = native.load()
    r, a, b = C.c_uint32(), C.c_uint64(), C.c_uint64()
    _check(lib.usgb_h5_dataset_info(path.encode(), dataset.encode(), C.byref(r), C.byref(a), C.byref(b)))
    return int(r.value), int(a.value), int(b.value)


def read(path: str, dataset: str) -> np.ndarray:
    """float64 array: (n1, n2) for rank 2, (n,) for rank 1."""
    lib = native.load()
    rank, n1, n2 = info(path, dataset)
    out = np.empty(n1 * n2, np.float64)
    a, b = C.c_uint64(), C.c_uint64()
    _check(lib.usgb_h5_read_f64(path.encode(), dataset.encode(), out.ctypes.data_as(C.POINTER(C.c_double)), out.size,
                                C.byref(a), C.byref(b)))
    return out.reshape(n1, n2) if rank == 2 else out


def write(path: str, dataset: str, data) -> None:
    """One rank-2 IEEE 64-bit little-endian dataset (a 1-D array is stored as
    one row, as HDF5Util::save stores a std::vector)."""
    a = np.ascontiguousarray(data, np.float64)
    if a.ndim == 1:
        a = a.reshape(1, -1)
    if a.ndim != 2:
        raise InvalidParameterException("Only rank-1 and rank-2 arrays are written.")
    _check(native.load().usgb_h5_write_f64(path.encode(), dataset.encode(), a.ctypes.data_as(C.POINTER(C.c_double)),
                                           a.shape[0], a.shape[1]))


def tx_elem_signals_path(base_dir: str, base_element: int, tx_element: int) -> str:
    return f"{base_dir}/signals-base{base_element:04d}-tx{tx_element:04d}"


class SavedSTAAcquisition:
    """Reads the RF of one transmit event from <data_dir>/signals-base####-tx####.h5
    (dataset "signal", num_rx rows of samples)."""

    def __init__(self, num_rx_elements: int, data_dir: str):
        self.num_rx_elements = int(num_rx_elements)
        self.data_dir = data_dir
        self.base_element = 0

    def set_data_dir(self, data_dir: str) -> None:
        self.data_dir = data_dir

    def prepare(self, base_element: int) -> None:
        self.base_element = int(base_element)

    def execute(self, tx_element: int) -> np.ndarray:
        from .errors import InvalidValueException
        path = tx_elem_signals_path(self.data_dir, self.base_element, tx_element) + FILE_SUFFIX
        m = read(path, "signal")
        if m.ndim == 1:
            m = m.reshape(1, -1)
        if m.shape[0] != self.num_rx_elements:
            raise InvalidValueException(f"Invalid number of rx elements ({m.shape[0]}) in file {path}, should be "
                                        f"{self.num_rx_elements}.")
        return m.astype(np.float32)


def save_tx_elem_signals(rf_rows, output_dir: str, base_element: int, tx_element: int) -> None:
    """Project::saveTxElemSignalsToHDF5: one transmit event's rows."""
    os.makedirs(output_dir, exist_ok=True)
    write(tx_elem_signals_path(output_dir, base_element, tx_element) + FILE_SUFFIX, "signal", rf_rows)


def save_image(grid: np.ndarray, output_dir: str, save_xyz: bool = True) -> None:
    """gridData (config.GRID_DTYPE, (n1, n2)) -> image_value.h5 ("value"),
    image_factor.h5 ("factor") and, with save_xyz, image_x/y/z.h5."""
    os.makedirs(output_dir, exist_ok=True)
    write(os.path.join(output_dir, "image_value" + FILE_SUFFIX), "value", grid["value"])
    write(os.path.join(output_dir, "image_factor" + FILE_SUFFIX), "factor", grid["factor"])
    if save_xyz:
        for k in ("x", "y", "z"):
            write(os.path.join(output_dir, "image_" + k + FILE_SUFFIX), k, grid[k])


def load_image(input_dir: str):
    """(value, factor) of a saved image."""
    return (read(os.path.join(input_dir, "image_value" + FILE_SUFFIX), "value"),
            read(os.path.join(input_dir, "image_factor" + FILE_SUFFIX), "factor"))
