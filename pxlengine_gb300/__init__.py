"""pxlengine_gb300 — GB300-native (sm_103a) FLIP liquid substep for pxlengine scenes.

The product is libpxlflip.so (CUDA kernels + C++ host engine behind the C ABI in
include/pxlflip.h). This package builds it (build.build()) and mirrors the reference's liquid
interface on top of it (fluid.FluidState, fluid.Fluid, fluid.Batch).
"""
from .serve import Server  # noqa: F401
from .fluid import (Batch, Fluid, FluidBlock, FluidError, FluidState, HostBuffer, Snapshot,  # noqa: F401
                    make_options, steps_for_frame)
