"""Host-side mirror of bricklib's brick API over the C ABI.

Names and argument meaning follow the reference (include/brick.h, include/bricksetup.h,
include/brick-gpu.h) so that driver code reads like stencils/3axis.cu:

    grid, bInfo = init_grid([STRIDEB] * 3)                 # bricksetup.h:73-90
    bStorage = BrickStorage.allocate(bInfo.nbricks, 512 * 2)
    bIn, bOut = Brick(bInfo, bStorage, 0), Brick(bInfo, bStorage, 512)
    copyToBrick([STRIDEG] * 3, [PADDING] * 3, [0] * 3, in_arr, grid, bIn)
    bInfo_dev = movBrickInfo(bInfo)                         # brick-gpu.h:42-55
    bStorage_dev = movBrickStorage(bStorage)                # brick-gpu.h:84-103
    brickSweep(Brick(bInfo_dev, bStorage_dev, 0), Brick(bInfo_dev, bStorage_dev, 512), blist, st)

Dimension lists passed to init_grid / copyToBrick / copyFromBrick are contiguous-first
(i, j, k) as in the reference; numpy arrays are indexed [k][j][i].
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import Optional, Sequence, Tuple

import numpy as np

from . import _abi
from ._abi import BK_BF16, BK_F32, BK_F64, call, lib
from .stencils import Stencil

NP_DTYPE = {BK_F64: np.float64, BK_F32: np.float32, BK_BF16: np.uint16}
ELEM_SIZE = {BK_F64: 8, BK_F32: 4, BK_BF16: 2}
DTYPE_NAMES = {"f64": BK_F64, "f32": BK_F32, "bf16": BK_BF16}


def dtype_of(x) -> int:
    if isinstance(x, str):
        return DTYPE_NAMES[x]
    return int(x)


# ------------------------------------------------------------------ bf16 helpers

def f32_to_bf16(a: np.ndarray) -> np.ndarray:
    """Round-to-nearest-even float32 -> bfloat16 bit patterns (uint16)."""
    u = np.ascontiguousarray(a, dtype=np.float32).view(np.uint32)
    rounding = ((u >> np.uint32(16)) & np.uint32(1)) + np.uint32(0x7FFF)
    out = ((u + rounding) >> np.uint32(16)).astype(np.uint16)
    nan = np.isnan(a)
    if nan.any():
        out[nan] = 0x7FC0
    return out


def bf16_to_f32(a: np.ndarray) -> np.ndarray:
    return (np.asarray(a, dtype=np.uint16).astype(np.uint32) << np.uint32(16)).view(np.float32)


def to_storage_dtype(a: np.ndarray, dtype: int) -> np.ndarray:
    if dtype == BK_F64:
        return np.asarray(a, dtype=np.float64)
    if dtype == BK_F32:
        return np.asarray(a, dtype=np.float32)
    return f32_to_bf16(np.asarray(a, dtype=np.float32))


def from_storage_dtype(a: np.ndarray, dtype: int) -> np.ndarray:
    if dtype == BK_BF16:
        return bf16_to_f32(a).astype(np.float64)
    return np.asarray(a, dtype=np.float64)


# ------------------------------------------------------------------ memory

def stream_ptr(stream) -> Optional[int]:
    """Accepts None, an int handle, or an object with a `cuda_stream` attribute."""
    if stream is None:
        return None
    if hasattr(stream, "cuda_stream"):
        return int(stream.cuda_stream) or None
    return int(stream) or None


class DeviceBuffer:
    """Device memory from bk_device_malloc, released by bk_device_free."""

    def __init__(self, nbytes: int):
        self.nbytes = int(nbytes)
        p = C.c_void_p()
        call("bk_device_malloc", C.byref(p), self.nbytes)
        self.ptr = p.value or 0

    def free(self) -> None:
        if self.ptr:
            call("bk_device_free", C.c_void_p(self.ptr))
            self.ptr = 0

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass

    def upload(self, host: np.ndarray, stream=None, offset: int = 0) -> None:
        host = np.ascontiguousarray(host)
        if host.nbytes + offset > self.nbytes:
            raise ValueError("upload larger than the buffer")
        call("bk_memcpy", C.c_void_p(self.ptr + offset), host.ctypes.data_as(C.c_void_p), host.nbytes, 0,
             stream_ptr(stream))
        if stream is None:
            call("bk_stream_synchronize", None)

    def download(self, host: np.ndarray, stream=None, offset: int = 0) -> np.ndarray:
        if not host.flags.c_contiguous:
            raise ValueError("host array must be contiguous")
        call("bk_memcpy", host.ctypes.data_as(C.c_void_p), C.c_void_p(self.ptr + offset), host.nbytes, 1,
             stream_ptr(stream))
        if stream is None:
            call("bk_stream_synchronize", None)
        return host


class PinnedBuffer:
    """Page-locked host memory with a numpy view (for copies timed end to end)."""

    def __init__(self, nbytes: int):
        self.nbytes = int(nbytes)
        p = C.c_void_p()
        call("bk_host_malloc", C.byref(p), self.nbytes)
        self.ptr = p.value or 0

    def view(self, dtype, count: Optional[int] = None) -> np.ndarray:
        dt = np.dtype(dtype)
        n = self.nbytes // dt.itemsize if count is None else count
        buf = (C.c_char * (n * dt.itemsize)).from_address(self.ptr)
        return np.frombuffer(buf, dtype=dt, count=n)

    def free(self) -> None:
        if self.ptr:
            call("bk_host_free", C.c_void_p(self.ptr))
            self.ptr = 0

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def memcpy(dst: int, src: int, nbytes: int, kind: int, stream=None) -> None:
    call("bk_memcpy", C.c_void_p(dst), C.c_void_p(src), nbytes, kind, stream_ptr(stream))


def synchronize(stream=None) -> None:
    call("bk_stream_synchronize", stream_ptr(stream))


def error_flags(stream=None) -> int:
    f = C.c_int()
    call("bk_error_flags", stream_ptr(stream), C.byref(f))
    return f.value


def check_device(stream=None) -> None:
    """Reads and clears the device error flags; raises BkError with BK_ERR_TIMEOUT when a
    bounded device wait gave up (the launch stopped early and its output is incomplete) and
    with BK_ERR_BOUNDS when an out-of-range brick index was clamped or skipped."""
    f = error_flags(stream)
    if f & 2:
        raise _abi.BkError(_abi.BK_ERR_TIMEOUT, "a bounded device wait gave up; the launch stopped early")
    if f & 1:
        raise _abi.BkError(_abi.BK_ERR_BOUNDS, "an out-of-range brick index was clamped or skipped")


# ------------------------------------------------------------------ layout

@dataclass(frozen=True)
class Layout:
    """Brick dims and vector fold, (k, j, i).  Brick<Dim<8,8,8>, Dim<4,8>> is
    Layout((8, 8, 8), (1, 4, 8))."""
    bdim: Tuple[int, int, int] = (8, 8, 8)
    fold: Tuple[int, int, int] = (1, 4, 8)

    @property
    def size(self) -> int:
        return int(np.prod(self.bdim))

    def to_c(self) -> _abi.bk_layout:
        return _abi.bk_layout((C.c_int * 3)(*self.bdim), (C.c_int * 3)(*self.fold))

    def offsets(self) -> np.ndarray:
        """layout(k, j, i) for every element in row-major (k, j, i) order
        (_BrickAccessor, brick.h:213-327)."""
        bk, bj, bi = self.bdim
        fk, fj, fi = self.fold
        k, j, i = np.meshgrid(np.arange(bk), np.arange(bj), np.arange(bi), indexing="ij")
        vec = ((k // fk) * (bj // fj) + j // fj) * (bi // fi) + i // fi
        lane = ((k % fk) * fj + j % fj) * fi + i % fi
        return (vec * (fk * fj * fi) + lane).reshape(-1)

    def row_major(self) -> bool:
        """Whether every element sits at its row-major (k, j, i) offset (the layouts the
        pipelined and TMA-fed kernels take)."""
        return bool(np.array_equal(self.offsets(), np.arange(self.size)))


DEFAULT_LAYOUT = Layout()


# ------------------------------------------------------------------ BrickInfo / BrickStorage / Brick

class BrickInfo:
    """Adjacency list: adj[nbricks][27] (brick.h:96-127).  Host arrays are numpy;
    a device copy (movBrickInfo) holds a DeviceBuffer instead."""

    def __init__(self, nbricks: int, adj: Optional[np.ndarray] = None, device: Optional[DeviceBuffer] = None):
        self.nbricks = int(nbricks)
        self.adj = adj if adj is not None or device is not None else np.zeros((nbricks, 27), np.uint32)
        self.device = device

    @property
    def on_device(self) -> bool:
        return self.device is not None

    @property
    def ptr(self) -> int:
        if not self.device:
            raise ValueError("BrickInfo is on the host; use movBrickInfo first")
        return self.device.ptr


def init_grid(dimlist: Sequence[int]) -> Tuple[np.ndarray, BrickInfo]:
    """init_grid<3>(grid_ptr, dimlist) (bricksetup.h:73-90): dimlist contiguous-first;
    returns (grid_ptr as a flat array, BrickInfo).  grid[p] = p; the neighbour at
    (dk, dj, di) is the brick at linear position p + (dk*gj + dj)*gi + di, or brick 0
    when that position is outside the whole grid (bricksetup.h:44-47)."""
    gi, gj, gk = (int(x) for x in dimlist)
    size = gk * gj * gi
    grid = np.arange(size, dtype=np.uint32)
    adj = np.empty((size, 27), dtype=np.uint32)
    p = np.arange(size, dtype=np.int64)
    s = 0
    for dk in (-1, 0, 1):
        for dj in (-1, 0, 1):
            for di in (-1, 0, 1):
                q = p + (dk * gj + dj) * gi + di
                ok = (q >= 0) & (q < size)
                adj[:, s] = np.where(ok, grid[np.clip(q, 0, size - 1)], 0)
                s += 1
    return grid, BrickInfo(size, adj)


class DeviceView(DeviceBuffer):
    """`nbytes` of another device buffer from byte `offset` on (not owned: the parent stays
    alive as long as the view)."""

    def __init__(self, parent: DeviceBuffer, offset: int, nbytes: int):
        if offset < 0 or offset + nbytes > parent.nbytes:
            raise ValueError("view outside its buffer")
        self.parent, self.nbytes, self.ptr = parent, int(nbytes), parent.ptr + int(offset)

    def free(self) -> None:
        self.ptr = 0


class BrickStorage:
    """`chunks` chunks of `step` elements (brick.h:53-82).  Host storage is a numpy
    array; device storage (movBrickStorage) a DeviceBuffer."""

    def __init__(self, chunks: int, step: int, dtype: int = BK_F64, host: Optional[np.ndarray] = None,
                 device: Optional[DeviceBuffer] = None):
        self.chunks, self.step, self.dtype = int(chunks), int(step), dtype_of(dtype)
        self.host = host
        self.device = device

    @staticmethod
    def allocate(chunks: int, step: int, dtype=BK_F64) -> "BrickStorage":
        dt = dtype_of(dtype)
        return BrickStorage(chunks, step, dt, host=np.zeros(int(chunks) * int(step), dtype=NP_DTYPE[dt]))

    @staticmethod
    def allocate_device(chunks: int, step: int, dtype=BK_F64) -> "BrickStorage":
        dt = dtype_of(dtype)
        buf = DeviceBuffer(int(chunks) * int(step) * ELEM_SIZE[dt])
        call("bk_memset", C.c_void_p(buf.ptr), 0, buf.nbytes, None)
        return BrickStorage(chunks, step, dt, device=buf)

    @staticmethod
    def allocate_pinned(chunks: int, step: int, dtype=BK_F64) -> "BrickStorage":
        """Storage in page-locked host memory mapped into the device (bk_host_malloc): `host` is
        its numpy view and kernels use it at the same address, e.g. as a sweep's output field,
        whose results then arrive in host memory without a separate copy."""
        dt = dtype_of(dtype)
        buf = PinnedBuffer(int(chunks) * int(step) * ELEM_SIZE[dt])
        st = BrickStorage(chunks, step, dt, host=buf.view(NP_DTYPE[dt]), device=buf)
        return st

    @property
    def nbytes(self) -> int:
        return self.chunks * self.step * ELEM_SIZE[self.dtype]

    @property
    def ptr(self) -> int:
        if not self.device:
            raise ValueError("BrickStorage is on the host; use movBrickStorage first")
        return self.device.ptr


def movBrickInfo(info: BrickInfo) -> BrickInfo:
    """movBrickInfo(bInfo, cudaMemcpyHostToDevice) (brick-gpu.h:42-55)."""
    adj = np.ascontiguousarray(info.adj, dtype=np.uint32)
    p = C.c_void_p()
    call("bk_info_to_device", adj.ctypes.data_as(C.c_void_p), info.nbricks, C.byref(p))
    buf = DeviceBuffer.__new__(DeviceBuffer)
    buf.nbytes, buf.ptr = adj.nbytes, p.value
    return BrickInfo(info.nbricks, device=buf)


def movBrickStorage(st: BrickStorage, to_device: bool = True) -> BrickStorage:
    """movBrickStorage(bStorage, HostToDevice / DeviceToHost) (brick-gpu.h:84-103)."""
    if to_device:
        host = np.ascontiguousarray(st.host)
        p = C.c_void_p()
        call("bk_storage_to_device", host.ctypes.data_as(C.c_void_p), st.chunks, st.step, st.dtype, C.byref(p))
        buf = DeviceBuffer.__new__(DeviceBuffer)
        buf.nbytes, buf.ptr = st.nbytes, p.value
        return BrickStorage(st.chunks, st.step, st.dtype, device=buf)
    host = np.empty(st.chunks * st.step, dtype=NP_DTYPE[st.dtype])
    call("bk_storage_to_host", C.c_void_p(st.ptr), st.chunks, st.step, st.dtype, host.ctypes.data_as(C.c_void_p))
    return BrickStorage(st.chunks, st.step, st.dtype, host=host)


class Brick:
    """Brick<Dim<BDims...>, Dim<Folds...>>(bInfo, bStorage, offset) (brick.h:353-395)."""

    def __init__(self, info: BrickInfo, storage: BrickStorage, offset: int, layout: Layout = DEFAULT_LAYOUT):
        if offset + layout.size > storage.step:
            raise ValueError("offset + brick size exceeds the storage step")
        self.bInfo, self.bStorage, self.offset, self.layout = info, storage, int(offset), layout

    @property
    def step(self) -> int:
        return self.bStorage.step

    def field(self) -> _abi.bk_field:
        s = self.bStorage
        return _abi.bk_field(C.c_void_p(s.ptr), s.chunks, s.step, self.offset, s.dtype)

    def host_bricks(self) -> np.ndarray:
        """[chunks, BRICKSIZE] view of this field in host storage, layout order."""
        s = self.bStorage
        return s.host.reshape(s.chunks, s.step)[:, self.offset:self.offset + self.layout.size]


def _iter_grid_blocks(dimlist, padding, ghost, bdim_kji):
    """(array slices, grid slices) covered by iter_grid (bricksetup.h:139-159)."""
    dim = [int(x) for x in reversed(dimlist)]  # -> (k, j, i)
    pad = [int(x) for x in reversed(padding)]
    gh = [int(x) for x in reversed(ghost)]
    asl, gsl, gdims = [], [], []
    for d in range(3):
        b = bdim_kji[d]
        s0, s1 = gh[d] // b, (dim[d] + gh[d]) // b
        asl.append(slice(pad[d] + s0 * b, pad[d] + s1 * b))
        gsl.append(slice(s0, s1))
        gdims.append((dim[d] + 2 * gh[d]) // b)
    return tuple(asl), tuple(gsl), tuple(gdims)


def _bricks_of_array(block: np.ndarray, bdim) -> np.ndarray:
    bk, bj, bi = bdim
    nk, nj, ni = block.shape[0] // bk, block.shape[1] // bj, block.shape[2] // bi
    return block.reshape(nk, bk, nj, bj, ni, bi).transpose(0, 2, 4, 1, 3, 5).reshape(nk * nj * ni, bk * bj * bi)


def copyToBrick(dimlist, padding, ghost, arr: np.ndarray, grid: np.ndarray, brick: Brick) -> None:
    """copyToBrick<3> (bricksetup.h:172-181) into host storage."""
    lay = brick.layout
    asl, gsl, gdims = _iter_grid_blocks(dimlist, padding, ghost, lay.bdim)
    rows = _bricks_of_array(arr[asl], lay.bdim)
    ids = grid.reshape(gdims)[gsl].reshape(-1)
    view = brick.bStorage.host.reshape(brick.bStorage.chunks, brick.bStorage.step)
    cols = brick.offset + lay.offsets()
    view[ids[:, None], cols[None, :]] = to_storage_dtype(rows, brick.bStorage.dtype)


def copyFromBrick(dimlist, padding, ghost, arr: np.ndarray, grid: np.ndarray, brick: Brick) -> None:
    """copyFromBrick<3> (bricksetup.h:213-221) from host storage."""
    lay = brick.layout
    asl, gsl, gdims = _iter_grid_blocks(dimlist, padding, ghost, lay.bdim)
    ids = grid.reshape(gdims)[gsl].reshape(-1)
    view = brick.bStorage.host.reshape(brick.bStorage.chunks, brick.bStorage.step)
    cols = brick.offset + lay.offsets()
    rows = from_storage_dtype(view[ids[:, None], cols[None, :]], brick.bStorage.dtype)
    bk, bj, bi = lay.bdim
    nk, nj, ni = (s.stop - s.start for s in gsl)
    block = rows.reshape(nk, nj, ni, bk, bj, bi).transpose(0, 3, 1, 4, 2, 5).reshape(nk * bk, nj * bj, ni * bi)
    arr[asl] = block


def compareBrick(dimlist, padding, ghost, arr: np.ndarray, grid: np.ndarray, brick: Brick,
                 tol: float = 1e-6) -> Tuple[bool, float]:
    """compareBrick<3> (brickcompare.h:30-57): passes when every element has
    diff < tol or diff < (|a|+|b|)*tol.  Returns (passed, max |diff|)."""
    got = np.zeros_like(arr, dtype=np.float64)
    copyFromBrick(dimlist, padding, ghost, got, grid, brick)
    asl, _, _ = _iter_grid_blocks(dimlist, padding, ghost, brick.layout.bdim)
    a, b = got[asl], np.asarray(arr[asl], dtype=np.float64)
    diff = np.abs(a - b)
    ok = (diff < tol) | (diff < (np.abs(a) + np.abs(b)) * tol)
    return bool(ok.all()), float(diff.max(initial=0.0))


# ------------------------------------------------------------------ stencil descriptor

def to_c_stencil(st: Stencil) -> _abi.bk_stencil:
    if st.npoints > _abi.BK_MAX_TAPS:
        raise ValueError("too many taps")
    s = _abi.bk_stencil()
    s.npoints = st.npoints
    for t, (tap, c) in enumerate(zip(st.taps, st.coeff)):
        s.offsets[t][0], s.offsets[t][1], s.offsets[t][2] = tap
        s.coeff[t] = float(c)
    s.pre_op, s.post_op = int(st.pre_op), int(st.post_op)
    return s


def stencil_family(st: Stencil, layout: Layout = DEFAULT_LAYOUT) -> Tuple[int, int]:
    r, f = C.c_int(), C.c_int()
    call("bk_stencil_check", C.byref(to_c_stencil(st)), C.byref(layout.to_c()), C.byref(r), C.byref(f))
    return r.value, f.value


# ------------------------------------------------------------------ device operations

class BrickList:
    """A device array of brick indices (the bricks one sweep computes)."""

    def __init__(self, ids: np.ndarray):
        ids = np.ascontiguousarray(ids, dtype=np.uint32)
        self.n = len(ids)
        self.host = ids
        self.buf = DeviceBuffer(max(4, ids.nbytes))
        if self.n:
            self.buf.upload(ids)

    @property
    def ptr(self) -> int:
        return self.buf.ptr


def brickSweep(bIn: Brick, bOut: Brick, blist: BrickList, st, acc: int = _abi.BK_ACC_NATIVE,
               stream=None) -> None:
    """One sweep of stencil `st` over the bricks in `blist` (bk_sweep)."""
    cst = st if isinstance(st, _abi.bk_stencil) else to_c_stencil(st)
    info = bIn.bInfo
    call("bk_sweep", C.c_void_p(info.ptr), info.nbricks, C.byref(bIn.field()), C.byref(bOut.field()),
         C.c_void_p(blist.ptr), blist.n, C.byref(cst), C.byref(bIn.layout.to_c()), acc, stream_ptr(stream))


def sweepKernel(bIn: Brick, bOut: Brick, st, acc: int = _abi.BK_ACC_NATIVE) -> str:
    """Name of the kernel brickSweep would launch for these bricks and stencil (bk_sweep_kernel)."""
    cst = st if isinstance(st, _abi.bk_stencil) else to_c_stencil(st)
    name = C.c_char_p()
    call("bk_sweep_kernel", C.byref(bIn.field()), C.byref(bOut.field()), C.byref(cst),
         C.byref(bIn.layout.to_c()), acc, C.byref(name))
    return name.value.decode()


class GhostPlan:
    """(dst, src) brick pairs on the device for bk_ghost_fill."""

    def __init__(self, pairs: np.ndarray):
        pairs = np.ascontiguousarray(pairs, dtype=np.uint32).reshape(-1, 2)
        self.n = len(pairs)
        self.host = pairs
        self.buf = DeviceBuffer(max(8, pairs.nbytes))
        if self.n:
            self.buf.upload(pairs)

    @property
    def ptr(self) -> int:
        return self.buf.ptr

    @staticmethod
    def periodic(grid: np.ndarray, nb, gb) -> "GhostPlan":
        nb_c, gb_c = (C.c_long * 3)(*nb), (C.c_long * 3)(*gb)
        g = np.ascontiguousarray(grid, dtype=np.uint32)
        cnt = C.c_long()
        call("bk_periodic_plan", g.ctypes.data_as(C.c_void_p), nb_c, gb_c, None, 0, C.byref(cnt))
        pairs = np.empty((cnt.value, 2), dtype=np.uint32)
        call("bk_periodic_plan", g.ctypes.data_as(C.c_void_p), nb_c, gb_c, pairs.ctypes.data_as(C.c_void_p),
             cnt.value, C.byref(cnt))
        return GhostPlan(pairs)


def ghostFill(plan: GhostPlan, brick: Brick, stream=None) -> None:
    call("bk_ghost_fill", C.c_void_p(plan.ptr), plan.n, C.byref(brick.field()), C.byref(brick.layout.to_c()),
         stream_ptr(stream))


def timeSteps(a: Brick, b: Brick, blist: BrickList, st, steps: int, plan: Optional[GhostPlan] = None,
              fill_every: int = 1, acc: int = _abi.BK_ACC_NATIVE, use_graph: bool = False, stream=None) -> Brick:
    """`steps` ping-pong sweeps (weak/main.cu:277-282) with the ghost plan applied to the
    current input every `fill_every` steps; returns the Brick holding the newest values."""
    cst = st if isinstance(st, _abi.bk_stencil) else to_c_stencil(st)
    info = a.bInfo
    call("bk_steps", C.c_void_p(info.ptr), info.nbricks, C.byref(a.field()), C.byref(b.field()),
         C.c_void_p(blist.ptr), blist.n, C.c_void_p(plan.ptr if plan else 0), plan.n if plan else 0,
         C.byref(cst), C.byref(a.layout.to_c()), acc, steps, fill_every if plan else 0, 1 if use_graph else 0,
         stream_ptr(stream))
    return a if steps % 2 == 0 else b


# ------------------------------------------------------------------ precision form

def convertField(src: Brick, dst: Brick, blist: BrickList, stream=None) -> None:
    """Element-wise storage-type conversion of the listed bricks (bk_convert)."""
    call("bk_convert", C.byref(src.field()), C.byref(dst.field()), C.c_void_p(blist.ptr), blist.n,
         C.byref(src.layout.to_c()), stream_ptr(stream))


def fieldNorms(a: Brick, ref: Brick, blist: BrickList, stream=None) -> dict:
    """FP64 device reduction of the error of field a against ref (bk_field_norms)."""
    out = (C.c_double * 4)()
    call("bk_field_norms", C.byref(a.field()), C.byref(ref.field()), C.c_void_p(blist.ptr), blist.n,
         C.byref(a.layout.to_c()), stream_ptr(stream), out)
    n = blist.n * a.layout.size
    return {"max_abs": out[0], "sum_sq": out[1], "max_ref": out[2], "sum_sq_ref": out[3],
            "rms": (out[1] / n) ** 0.5 if n else 0.0,
            "max_rel": out[0] / out[2] if out[2] else 0.0,
            "rms_rel": (out[1] / out[3]) ** 0.5 if out[3] else 0.0}


def fillSines(brick: Brick, grid_bricks, ghost_bricks, nwaves: int = 8, seed: int = 0, noise: float = 1e-3,
              stream=None) -> None:
    """The seeded sum-of-sines initial field on every brick of an init_grid layout."""
    call("bk_fill_sines", C.byref(brick.field()), C.byref(brick.layout.to_c()), (C.c_long * 3)(*grid_bricks),
         (C.c_long * 3)(*ghost_bricks), nwaves, seed, noise, stream_ptr(stream))


# ------------------------------------------------------------------ array <-> bricks on the device

def copyToBrickDevice(dimlist, padding, ghost, arr_dev: int, grid_dev: int, brick: Brick, stream=None) -> None:
    """copyToBrick with the array and grid on the device (bk_copy_to_bricks); lists are
    contiguous-first like the host copyToBrick."""
    L3 = C.c_long * 3
    call("bk_copy_to_bricks", C.c_void_p(arr_dev), L3(*reversed(dimlist)), L3(*reversed(padding)),
         L3(*reversed(ghost)), C.c_void_p(grid_dev), C.byref(brick.field()), C.byref(brick.layout.to_c()),
         stream_ptr(stream))


def copyFromBrickDevice(dimlist, padding, ghost, arr_dev: int, grid_dev: int, brick: Brick, stream=None) -> None:
    """copyFromBrick on the device (bk_copy_from_bricks)."""
    L3 = C.c_long * 3
    call("bk_copy_from_bricks", C.c_void_p(arr_dev), L3(*reversed(dimlist)), L3(*reversed(padding)),
         L3(*reversed(ghost)), C.c_void_p(grid_dev), C.byref(brick.field()), C.byref(brick.layout.to_c()),
         stream_ptr(stream))
