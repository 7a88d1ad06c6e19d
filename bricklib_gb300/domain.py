"""The reference drivers' single-node setup as one object.

stencils/stencils.h:11-26 and stencils/3axis.cu:77-125 build the same thing every
time: an N^3 interior with a ghost zone of one brick (GZ = 8 cells) and array
padding (PADDING = 8), a dense brick grid over interior + ghost (init_grid), two
interleaved fields bIn / bOut in one BrickStorage, and the list of interior bricks
the kernel visits.  GridDomain owns those pieces, on the host and on the device.
"""
from __future__ import annotations

from typing import Optional, Sequence

import numpy as np

from . import bricks as B
from ._abi import BK_F64


class GridDomain:
    def __init__(self, n, layout: B.Layout = B.DEFAULT_LAYOUT, ghost=None, pad: int = 8,
                 dtype=BK_F64, nfields: int = 2, device: bool = True):
        n = (int(n),) * 3 if np.isscalar(n) else tuple(int(x) for x in n)  # (k, j, i)
        # ghost zone per axis (k, j, i): one brick, at least 8 cells (stencils.h:14)
        if ghost is None:
            ghost = tuple(max(8, b) for b in layout.bdim)
        elif np.isscalar(ghost):
            ghost = (int(ghost),) * 3
        ghost = tuple(int(g) for g in ghost)
        for d in range(3):
            if n[d] % layout.bdim[d] or ghost[d] % layout.bdim[d]:
                raise ValueError("interior and ghost zone must be multiples of the brick dims")
        self.n, self.layout, self.ghost, self.pad = n, layout, ghost, pad
        self.dtype = B.dtype_of(dtype)
        self.nfields = nfields
        self.adims = tuple(x + 2 * (g + pad) for x, g in zip(n, ghost))   # array dims (k, j, i)
        self.org = tuple(g + pad for g in ghost)                         # first interior cell
        self.gdims = tuple((x + 2 * g) // b for x, g, b in zip(n, ghost, layout.bdim))
        self.nb = tuple(x // b for x, b in zip(n, layout.bdim))          # interior bricks per axis
        self.gb = tuple(g // b for g, b in zip(ghost, layout.bdim))      # ghost bricks per side
        self.grid, self.bInfo = B.init_grid(list(reversed(self.gdims)))
        self.nbricks = self.bInfo.nbricks
        self.bsize = layout.size
        self.step = self.bsize * nfields
        g3 = self.grid.reshape(self.gdims)
        gb, nb = self.gb, self.nb
        self.interior = np.ascontiguousarray(
            g3[gb[0]:gb[0] + nb[0], gb[1]:gb[1] + nb[1], gb[2]:gb[2] + nb[2]].reshape(-1))
        self.all_bricks = np.ascontiguousarray(self.grid)
        self.storage = B.BrickStorage.allocate(self.nbricks, self.step, self.dtype)
        self.dev_info = self.dev_storage = None
        self.dev_interior = self.dev_plan = None
        if device:
            self.to_device()

    # ---------------------------------------------------------------- fields
    def brick(self, field: int, on_device: bool = True) -> B.Brick:
        info = self.dev_info if on_device else self.bInfo
        st = self.dev_storage if on_device else self.storage
        return B.Brick(info, st, field * self.bsize, self.layout)

    @property
    def points(self) -> int:
        return int(np.prod(self.n))

    # ---------------------------------------------------------------- host <-> bricks
    def set_field(self, field: int, arr: np.ndarray) -> None:
        """copyToBrick of interior + ghost from a padded (k, j, i) array into host storage."""
        g = [x + 2 * gz for x, gz in zip(reversed(self.n), reversed(self.ghost))]
        B.copyToBrick(g, [self.pad] * 3, [0] * 3, arr, self.grid, self.brick(field, on_device=False))

    def get_field(self, field: int) -> np.ndarray:
        """copyFromBrick of the interior into a fresh padded float64 array."""
        arr = np.zeros(self.adims, dtype=np.float64)
        B.copyFromBrick(list(reversed(self.n)), [self.pad] * 3, list(reversed(self.ghost)), arr, self.grid,
                        self.brick(field, on_device=False))
        return arr

    def interior_view(self, arr: np.ndarray) -> np.ndarray:
        o = self.org
        return arr[o[0]:o[0] + self.n[0], o[1]:o[1] + self.n[1], o[2]:o[2] + self.n[2]]

    # ---------------------------------------------------------------- device
    def to_device(self) -> None:
        self.dev_info = B.movBrickInfo(self.bInfo)
        self.dev_storage = B.movBrickStorage(self.storage)
        self.dev_interior = B.BrickList(self.interior)

    def upload(self) -> None:
        self.dev_storage.device.upload(self.storage.host)

    def download(self) -> None:
        self.dev_storage.device.download(self.storage.host)

    def periodic_plan(self) -> B.GhostPlan:
        if self.dev_plan is None:
            self.dev_plan = B.GhostPlan.periodic(self.grid, self.nb, self.gb)
        return self.dev_plan
