"""Apodization windows: config.window (the library's WindowFunction::get)
against the reference's own WindowFunction::get<float> output
(src/util/WindowFunction.h:100-289), compiled from the reference sources and
stored in tests/golden/reference_windows.npz. Bit for bit in float: both
evaluate the window in double and round once to float. CPU only."""
import os

import numpy as np
import pytest

from conftest import GOLDEN


@pytest.fixture(scope="module")
def windows():
    return np.load(os.path.join(GOLDEN, "reference_windows.npz"))


def test_every_window_matches_reference_bit_for_bit(windows):
    from us_lab4a_gb300.config import window
    assert len(windows.files) >= 120
    for key in windows.files:
        desc, size = key.rsplit("/", 1)
        got = window(desc, int(size), np.float32)
        ref = windows[key]
        assert got.dtype == np.float32 and got.shape == ref.shape, key
        assert np.array_equal(got.view(np.uint32), ref.view(np.uint32)), (key, np.abs(got - ref).max())


@pytest.mark.parametrize("desc,size,exc,msg", [
    ("", 8, "MissingValueException", "Missing window function name."),
    ("kaiser", 8, "InvalidParameterException", "Invalid window function name: kaiser."),
    ("blackman", 1, "InvalidParameterException", "The window function size must be >= 2."),
    ("trapezoidal", 12, "InvalidParameterException", "Missing fade in size for the trapezoidal window function."),
    ("trapezoidal 3", 12, "InvalidParameterException", "Missing top size for the trapezoidal window function."),
    ("trapezoidal 3 4", 12, "InvalidParameterException", "Missing fade out size for the trapezoidal window function."),
    ("trapezoidal 3 4 5", 11, "InvalidParameterException", "Invalid total size for the trapezoidal window function."),
    ("trapezoidal 1 0 0", 1, "InvalidParameterException", "The window function size must be >= 2."),
])
def test_invalid_windows_rejected_like_reference(desc, size, exc, msg):
    """The reference's exception type and message (WindowFunction.h:237-289)."""
    from us_lab4a_gb300 import errors
    from us_lab4a_gb300.config import window
    with pytest.raises(getattr(errors, exc)) as ei:
        window(desc, size, np.float32)
    assert str(ei.value) == msg
