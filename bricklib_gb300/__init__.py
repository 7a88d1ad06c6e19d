"""GB300 brick stencil engine: bricklib's single-node brick stencil sweep as
hand-written sm_103a CUDA behind a C ABI (include/bricklib_gb300.h).

The package is the host side: ctypes binding of the ABI (_abi), the reference-named
brick API (bricks), stencil shapes (stencils) and the reference drivers' single-node
setup (domain).  Importing it does not touch the GPU; the first call that needs the
library loads bricklib_gb300/lib/libbrick_gb300.so and fails loudly if it is missing.
"""
from ._abi import (BK_ACC_COMPENSATED, BK_ACC_FLOATFLOAT, BK_ACC_NATIVE, BK_BF16, BK_F32, BK_F64,
                   BkError, lib)
from .bricks import (Brick, BrickInfo, BrickList, BrickStorage, DeviceBuffer, GhostPlan, Layout,
                     PinnedBuffer, brickSweep, compareBrick, copyFromBrick, copyToBrick, error_flags,
                     ghostFill, init_grid, movBrickInfo, movBrickStorage, synchronize, timeSteps)
from .domain import GridDomain
from . import stencils

__all__ = [
    "BK_ACC_COMPENSATED", "BK_ACC_FLOATFLOAT", "BK_ACC_NATIVE", "BK_BF16", "BK_F32", "BK_F64", "BkError",
    "Brick", "BrickInfo", "BrickList", "BrickStorage", "DeviceBuffer", "GhostPlan", "GridDomain", "Layout",
    "PinnedBuffer", "brickSweep", "compareBrick", "copyFromBrick", "copyToBrick", "error_flags",
    "ghostFill", "init_grid", "lib", "movBrickInfo", "movBrickStorage", "stencils", "synchronize",
    "timeSteps",
]
