"""Four-dimensional bricks (weak/main-4d.cpp): Brick<Dim<4,4,4,4>, Dim<fold>> layouts,
init_grid<4> adjacency, copyToBrick<4> / copyFromBrick<4> on the host and the device sweep
bk_sweep4.  Tuples are (l, k, j, i), outermost first; dimension lists passed to init_grid and
the copies are contiguous first, as in the reference.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import Sequence, Tuple

import numpy as np

from . import _abi, bricks as B, stencils
from ._abi import bk_layout4, bk_stencil4, call


@dataclass(frozen=True)
class Layout4:
    """bdim and fold (l, k, j, i); the folds of main-4d.cpp are (1,1,2,4) for AVX512,
    (1,1,2,2) for AVX2 and (1,1,1,1) for the scalar build."""
    bdim: Tuple[int, int, int, int] = (4, 4, 4, 4)
    fold: Tuple[int, int, int, int] = (1, 1, 2, 4)

    @property
    def size(self) -> int:
        return int(np.prod(self.bdim))

    def offsets(self) -> np.ndarray:
        """Element offset of (l, k, j, i) in row-major (l, k, j, i) order."""
        b, f = self.bdim, self.fold
        l, k, j, i = np.indices(b).reshape(4, -1)
        vl = int(np.prod(f))
        vec = (((l // f[0]) * (b[1] // f[1]) + k // f[1]) * (b[2] // f[2]) + j // f[2]) * (b[3] // f[3]) + i // f[3]
        lane = (((l % f[0]) * f[1] + k % f[1]) * f[2] + j % f[2]) * f[3] + i % f[3]
        return vec * vl + lane

    def to_c(self) -> bk_layout4:
        return bk_layout4((C.c_int * 4)(*self.bdim), (C.c_int * 4)(*self.fold))


def init_grid(dimlist: Sequence[int]) -> Tuple[np.ndarray, np.ndarray]:
    """init_grid<D> (bricksetup.h:73-90) for any D: grid[p] = p; adjacency slot s (outermost
    offset most significant) is the brick at linear position p + sum o_d * stride_d, or 0
    when that position is outside the whole grid (bricksetup.h:44-47)."""
    dims = [int(x) for x in dimlist]  # contiguous first
    D = len(dims)
    size = int(np.prod(dims))
    strides = np.cumprod([1] + dims[:-1])
    grid = np.arange(size, dtype=np.uint32)
    p = np.arange(size, dtype=np.int64)
    adj = np.empty((size, 3 ** D), np.uint32)
    for s in range(3 ** D):
        # digit of the outermost dimension is the most significant
        offs = [(s // 3 ** (D - 1 - d)) % 3 - 1 for d in range(D)]  # outermost first
        q = p + sum(o * int(strides[D - 1 - d]) for d, o in enumerate(offs))
        adj[:, s] = np.where((q >= 0) & (q < size), grid[np.clip(q, 0, size - 1)], 0)
    return grid, adj


def copy_to_bricks(arr: np.ndarray, grid: np.ndarray, gdims: Sequence[int], org: Sequence[int],
                   storage: np.ndarray, step: int, offset: int, lay: Layout4) -> None:
    """copyToBrick<4>: the region arr[org : org + gdims * bdim] (l, k, j, i) into the bricks
    grid[...] (gdims bricks per dimension, outermost first) of a flat host storage."""
    b = lay.bdim
    sub = arr[tuple(slice(o, o + g * bb) for o, g, bb in zip(org, gdims, b))]
    blk = sub.reshape(gdims[0], b[0], gdims[1], b[1], gdims[2], b[2], gdims[3], b[3]).transpose(0, 2, 4, 6, 1, 3, 5, 7)
    blk = blk.reshape(-1, lay.size)
    view = storage.reshape(-1, step)
    view[grid.reshape(-1)[:, None], offset + lay.offsets()[None, :]] = blk


def copy_from_bricks(arr: np.ndarray, grid: np.ndarray, gdims: Sequence[int], org: Sequence[int],
                     storage: np.ndarray, step: int, offset: int, lay: Layout4) -> None:
    """copyFromBrick<4>: the inverse of copy_to_bricks."""
    b = lay.bdim
    view = storage.reshape(-1, step)
    blk = view[grid.reshape(-1)[:, None], offset + lay.offsets()[None, :]]
    blk = blk.reshape(gdims[0], gdims[1], gdims[2], gdims[3], b[0], b[1], b[2], b[3]).transpose(0, 4, 1, 5, 2, 6, 3, 7)
    arr[tuple(slice(o, o + g * bb) for o, g, bb in zip(org, gdims, b))] = blk.reshape(
        tuple(g * bb for g, bb in zip(gdims, b)))


def mpi9pt(alpha: float = 0.2, beta: float = 0.1) -> stencils.Stencil:
    """The 9-point 4-D star of stencils/mpi9pt.py in its tap order, (dl, dk, dj, di)."""
    taps = [(0, 0, 0, 0), (0, 0, 0, 1), (0, 0, 0, -1), (0, 0, 1, 0), (0, 0, -1, 0), (0, 1, 0, 0), (0, -1, 0, 0),
            (1, 0, 0, 0), (-1, 0, 0, 0)]
    return stencils.Stencil("mpi9pt", taps, np.array([alpha] + [beta] * 8), list(range(9)))


def to_c_stencil4(st: stencils.Stencil) -> bk_stencil4:
    if not 1 <= st.npoints <= _abi.BK_MAX_TAPS4:
        raise ValueError("4-D stencils take 1 to 81 taps")
    c = bk_stencil4()
    c.npoints = st.npoints
    for t, (tap, v) in enumerate(zip(st.taps, st.coeff)):
        if len(tap) != 4:
            raise ValueError("4-D taps are (dl, dk, dj, di)")
        for d in range(4):
            c.offsets[t][d] = int(tap[d])
        c.coeff[t] = float(v)
    return c


def sweep4(adj_dev: B.DeviceBuffer, nbricks: int, storage: B.BrickStorage, in_off: int, out_off: int,
           blist: B.BrickList, st, lay: Layout4 = Layout4(), stream=None, out_storage: B.BrickStorage = None) -> None:
    """One 4-D sweep of `st` over the bricks in `blist` (bk_sweep4)."""
    cst = st if isinstance(st, bk_stencil4) else to_c_stencil4(st)
    so = out_storage or storage
    fin = _abi.bk_field(C.c_void_p(storage.ptr), storage.chunks, storage.step, in_off, storage.dtype)
    fout = _abi.bk_field(C.c_void_p(so.ptr), so.chunks, so.step, out_off, so.dtype)
    call("bk_sweep4", C.c_void_p(adj_dev.ptr), nbricks, C.byref(fin), C.byref(fout), C.c_void_p(blist.ptr),
         blist.n, C.byref(cst), C.byref(lay.to_c()), B.stream_ptr(stream))
