"""us_lab4a_gb300: GB300-native (sm_103a) STA/TFM delay-and-sum imaging.

A drop-in for the STA/TFM processors of us_lab4a (VectorialSTAProcessor,
VectorialSTACUDAProcessor, Vectorial3DSTAProcessor, DefaultSTAProcessor):
the hot path runs in hand-written CUDA kernels in libusgb.so, reached through
the C ABI of include/usgb.h.
"""
from .config import (  # noqa: F401
    GRID_DTYPE, AnalyticSignalCoherenceFactorProcessor, CoherenceFactorProcessor, ParameterMap,
    SA3DConfiguration, STAConfiguration, element_positions_matrix, element_x_centered_2d, grid_xyz,
    make_grid, rectangular_grid_xyz, rectangular_grid_xz, window,
)
from .errors import (  # noqa: F401
    CUDAException, DeviceTimeoutException, InvalidParameterException, InvalidStateException,
    InvalidValueException, NativeLibraryError, UnsupportedException,
)
from .engine import FrameSpec, StaEngine  # noqa: F401
from .processor import (  # noqa: F401
    DefaultSTAGB300Processor, InMemorySTAAcquisition, Vectorial3DSTAGB300Processor, VectorialSTAGB300Processor,
)

__version__ = "0.1.0"
