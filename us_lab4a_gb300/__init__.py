"""us_lab4a_gb300: GB300-native (sm_103a) STA/TFM delay-and-sum imaging.

A drop-in for the STA/TFM processors of us_lab4a (VectorialSTAProcessor,
VectorialSTACUDAProcessor, Vectorial3DSTAProcessor, DefaultSTAProcessor) and
for its single-term 3D processors (Vectorial3DT1R1SAFTProcessor,
Vectorial3DTnRnProcessor, SynthYVectorial3DTnRnProcessor) and its two-medium
imaging (VectorialCombinedTwoMediumImagingProcessor): the hot path runs
in hand-written CUDA kernels in libusgb.so, reached through the C ABI of
include/usgb.h.
"""
from .config import (  # noqa: F401
    GRID_DTYPE, AnalyticSignalCoherenceFactorProcessor, CoherenceFactorProcessor, ParameterMap,
    SA3DConfiguration, STAConfiguration, TnRnConfiguration, TwoMediumSTAConfiguration, element_positions_matrix,
    element_x_centered_2d,
    grid_xyz, make_grid, rectangular_grid_xyz, rectangular_grid_xz, tx_3d_focus_delay, window,
)
from .errors import (  # noqa: F401
    CUDAException, DeviceTimeoutException, InvalidParameterException, InvalidStateException,
    InvalidValueException, NativeLibraryError, UnsupportedException,
)
from .engine import FrameSpec, StaEngine  # noqa: F401
from .processor import (  # noqa: F401
    DefaultSTAGB300Processor, InMemorySTAAcquisition, Vectorial3DSTAGB300Processor, VectorialSTAGB300Processor,
)

from .single import (  # noqa: F401
    SingleEngine, SynthYVectorial3DTnRnGB300Processor, Vectorial3DT1R1SAFTGB300Processor,
    Vectorial3DTnRnGB300Processor,
)

from .two_medium import TwoMediumEngine, VectorialCombinedTwoMediumGB300Processor  # noqa: F401

__version__ = "0.1.0"
