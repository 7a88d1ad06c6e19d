"""BrickDecomp without MPI: the reference's brick layout producer (include/brick-mpi.h:178-464)
over the bk_decomp_* C ABI, and its exchange on one GPU with periodic boundaries.

    dec = BrickDecomp([64, 64, 64], 8, bdim=(8, 8, 8), numfield=2)   # dims: contiguous first
    dec.initialize(SKIN3D_GOOD)
    info = dec.getBrickInfo()           # BrickInfo with the decomposition's adjacency
    dec[k][j][i]                        # grid access (brick index), grid_access of brick-mpi.h
    dec.exchange(device_storage)        # ghost[i] <- skin[i] for every region: a periodic wrap

A region or neighbour is a set of signed dimension numbers (+d / -d: high / low side of
dimension d-1, dimension 0 contiguous), carried as the reference's BitSet bit field.
"""
from __future__ import annotations

import ctypes as C
from typing import Iterable, List, Sequence

import numpy as np

from . import _abi, bricks as B
from ._abi import call


def bitset(sides: Iterable[int]) -> int:
    """BitSet of bitset.h: side +p is bit p, side -p is bit 31 + p."""
    s = 0
    for p in sides:
        s ^= 1 << (p if p > 0 else 31 - p)
    return s


def sides(bits: int) -> List[int]:
    return [b if b < 32 else 31 - b for b in range(64) if (bits >> b) & 1]


# Skin orders of src/brick-mpi.cpp:25-112 (the layouts a decomposition is tuned with; data,
# kept identical so that storages and exchanges match the reference's).
SKIN3D_GOOD = [bitset(s) for s in (
    (1,), (1, -3), (1, 2, -3), (1, 2), (1, 2, 3), (2, 3), (2,), (2, -3), (-1, 2, -3), (-1, 2), (-1, 2, 3),
    (-1, 3), (-1,), (-3,), (-1, -3), (-1, -2, -3), (-1, -2), (-1, -2, 3), (-2, 3), (-2,), (-2, -3),
    (1, -2, -3), (1, -2), (1, -2, 3), (1, 3), (3,))]
SKIN3D_NORMAL = [bitset(s) for s in (
    (-1, -2, -3), (-2, -3), (1, -2, -3), (-1, -3), (-3,), (1, -3), (-1, 2, -3), (2, -3), (1, 2, -3),
    (-1, -2), (-2,), (1, -2), (-1,), (), (1,), (-1, 2), (2,), (1, 2), (-1, -2, 3), (-2, 3), (1, -2, 3),
    (-1, 3), (3,), (1, 3), (-1, 2, 3), (2, 3), (1, 2, 3))]


def all_regions(dim: int) -> List[int]:
    """Every non-empty region of `dim` dimensions in the neighbour order of brick-mpi.cpp:9-23."""
    out: List[int] = []

    def rec(cur, idx):
        if idx > dim:
            out.append(cur)
            return
        rec(cur ^ bitset([idx]), idx + 1)
        rec(cur, idx + 1)
        rec(cur ^ bitset([-idx]), idx + 1)

    rec(0, 1)
    return [r for r in out if r]


class _GridAccess:
    def __init__(self, dec: "BrickDecomp", ref: int, d: int):
        self.dec, self.ref, self.d = dec, ref, d

    def __getitem__(self, i: int):
        ref = self.ref + i * int(self.dec.stride[self.d - 1])
        if self.d == 1:
            return int(self.dec.grid[ref])
        return _GridAccess(self.dec, ref, self.d - 1)


class BrickDecomp:
    def __init__(self, dims: Sequence[int], depth: int, bdim: Sequence[int] = (8, 8, 8), numfield: int = 1,
                 dtype: int = _abi.BK_F64, pagesize: int = 4096):
        """dims and bdim contiguous dimension first (the reference's vector order)."""
        self.dim = len(dims)
        if len(bdim) != self.dim:
            raise ValueError("bdim needs one entry per dimension")
        self.dims_el = [int(x) for x in dims]
        self.bdim = [int(x) for x in bdim]
        self.depth, self.numfield, self.dtype, self.pagesize = int(depth), int(numfield), dtype, int(pagesize)
        self.h = None

    def initialize(self, skinlist: Sequence[int]) -> None:
        self.close()
        n = self.dim
        U = C.c_uint * n
        sk = (C.c_uint64 * max(1, len(skinlist)))(*[int(x) for x in skinlist])
        h = C.c_void_p()
        call("bk_decomp_create", n, U(*self.dims_el), U(*self.bdim), self.depth, self.numfield,
             B.ELEM_SIZE[self.dtype], self.pagesize, sk, len(skinlist), C.byref(h))
        self.h = h
        self.skinlist = [int(x) for x in skinlist]
        nb, gs, nr = C.c_uint(), C.c_size_t(), C.c_uint()
        sep = (C.c_uint * 3)()
        call("bk_decomp_info", h, C.byref(nb), C.byref(gs), C.byref(nr), sep)
        self.nbricks, self.nregions, self.sep_pos = nb.value, nr.value, list(sep)
        self.grid = np.zeros(gs.value, np.uint32)
        call("bk_decomp_grid", h, self.grid.ctypes.data_as(C.POINTER(C.c_uint)))
        self.adj = np.zeros((self.nbricks, 3 ** n), np.uint32)
        call("bk_decomp_adjacency", h, self.adj.ctypes.data_as(C.POINTER(C.c_uint)))
        g = (_abi.bk_decomp_region * max(1, nr.value))()
        s = (_abi.bk_decomp_region * max(1, nr.value))()
        ss = (C.c_long * max(1, len(skinlist)))()
        call("bk_decomp_regions", h, g, s, ss)
        f = [x for x, _ in _abi.bk_decomp_region._fields_]
        self.ghost = [{k: getattr(g[q], k) for k in f} for q in range(nr.value)]
        self.skin = [{k: getattr(s[q], k) for k in f} for q in range(nr.value)]
        self.skin_size = list(ss)[:len(skinlist)]
        self.t_dims = [x // b + 2 * (self.depth // b) for x, b in zip(self.dims_el, self.bdim)]
        self.stride = np.cumprod([1] + self.t_dims[:-1]).tolist()
        self._links = {}

    def grid_array(self) -> np.ndarray:
        """The grid as an array indexed [last dim] ... [first dim] (e.g. [k][j][i])."""
        return self.grid.reshape(tuple(reversed(self.t_dims)))

    def __getitem__(self, i: int):
        return _GridAccess(self, 0, self.dim)[i]

    def getBrickInfo(self) -> B.BrickInfo:
        if self.dim != 3:
            raise ValueError("BrickInfo of this package is three-dimensional")
        return B.BrickInfo(self.nbricks, self.adj)

    def exchange_links(self, storage_ptr: int, step_bytes: int) -> np.ndarray:
        links = np.zeros(3 * max(1, self.nregions), np.uint64)
        call("bk_decomp_exchange_links", self.h, C.c_void_p(storage_ptr), step_bytes,
             links.ctypes.data_as(C.POINTER(C.c_uint64)))
        return links[:3 * self.nregions].reshape(-1, 3)

    def exchange(self, storage: B.BrickStorage, stream=None) -> None:
        """Periodic exchange on the device: one bk_region_copy over the ghost / skin pairs."""
        key = (storage.ptr, storage.step)
        if key not in self._links:
            host = self.exchange_links(storage.ptr, storage.step * B.ELEM_SIZE[storage.dtype])
            buf = B.DeviceBuffer(max(8, host.nbytes))
            if host.size:
                buf.upload(np.ascontiguousarray(host))
            self._links[key] = buf
        call("bk_region_copy", C.c_void_p(self._links[key].ptr), self.nregions, B.stream_ptr(stream))

    def close(self) -> None:
        if self.h:
            _abi.lib().bk_decomp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
