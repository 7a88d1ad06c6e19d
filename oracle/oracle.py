"""ctypes wrapper of the CPU oracle (brick_oracle.c) and, where it was built, of
the reference-compiled checker in ``_ref/``.

TEST INFRASTRUCTURE ONLY: imported by ``tests/``, ``__graft_entry__.smoke()`` and
the CPU-baseline leg of ``bench.py``.  The product path never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from typing import Optional, Sequence, Tuple

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
TIMED_PATH = os.path.join(HERE, "liboracle_timed.so")
REF_PATH = os.path.join(HERE, "_ref", "libbrickref.so")

_u32p = np.ctypeslib.ndpointer(dtype=np.uint32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_f32p = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_i64p = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")
_u64p = np.ctypeslib.ndpointer(dtype=np.uint64, flags="C_CONTIGUOUS")
_l3 = C.c_long * 3
_i3 = C.c_int * 3


def reference_tree() -> Optional[str]:
    """The bricklib source tree the ``ref`` recipe compiles: $BRICKLIB_REF, else the
    Makefile's default; None where that tree is absent (e.g. on a machine that only runs
    the prebuilt files)."""
    path = os.environ.get("BRICKLIB_REF")
    if not path:
        try:
            path = subprocess.run(["make", "-s", "-C", HERE, "print-ref"], capture_output=True, text=True,
                                  check=True).stdout.strip()
        except (OSError, subprocess.CalledProcessError):
            return None
    return path if path and os.path.isdir(os.path.join(path, "include")) else None


def build(force: bool = False) -> None:
    """Compile liboracle.so (and _ref/ when the reference tree is present)."""
    if force or not os.path.exists(LIB_PATH) or not os.path.exists(TIMED_PATH):
        subprocess.check_call(["make", "-s", "-C", HERE, "all", "timed"])
    tree = reference_tree()
    if tree and (force or not os.path.exists(REF_PATH)):
        subprocess.check_call(["make", "-s", "-C", HERE, "ref", f"REF={tree}"])


_lib = None
_timed = None
_ref = None


def lib():
    """The parity build (-ffp-contract=off): every check runs on this one."""
    global _lib
    if _lib is None:
        _lib = _load(LIB_PATH)
    return _lib


def timed_lib():
    """The same source built as the reference builds its CPU path (-O2, multiply-adds fused):
    only the timed CPU baseline runs on it."""
    global _timed
    if _timed is None:
        _timed = _load(TIMED_PATH)
    return _timed


def _load(path):
    if not os.path.exists(path):
        build()
    L = C.CDLL(path)
    L.orc_fill_uniform.argtypes = [_f64p, C.c_long, C.c_uint64, C.c_double, C.c_double]
    L.orc_fill_sines.argtypes = [_f64p, _l3, _l3, _l3, C.c_int, C.c_uint64, C.c_double]
    L.orc_init_grid.argtypes = [_u32p, _u32p, C.c_long, C.c_long, C.c_long]
    L.orc_brick_offset.argtypes = [_i3, _i3, C.c_int, C.c_int, C.c_int]
    L.orc_brick_offset.restype = C.c_long
    L.orc_copy_brick.argtypes = [C.c_int, _l3, _l3, _l3, _f64p, _u32p, _f64p, C.c_long, C.c_long, _i3, _i3]
    L.orc_brick_sweep.argtypes = [_u32p, _f64p, C.c_long, C.c_long, _f64p, C.c_long, C.c_long,
                                  _u32p, C.c_long, _i3, _i3, C.c_int, _i32p, _f64p, C.c_int]
    L.orc_brick_sweep_f32.argtypes = [_u32p, _f32p, C.c_long, C.c_long, _f32p, C.c_long, C.c_long,
                                      _u32p, C.c_long, _i3, _i3, C.c_int, _i32p, _f64p, C.c_int]
    L.orc_array_sweep.argtypes = [_f64p, _f64p, _l3, _l3, _l3, C.c_int, _i32p, _f64p, C.c_int]
    L.orc_brick_sweep_ops.argtypes = [_u32p, _f64p, C.c_long, C.c_long, _f64p, C.c_long, C.c_long,
                                      _u32p, C.c_long, _i3, _i3, C.c_int, _i32p, _f64p, C.c_int, C.c_int,
                                      C.c_int]
    L.orc_array_sweep_ops.argtypes = [_f64p, _f64p, _l3, _l3, _l3, C.c_int, _i32p, _f64p, C.c_int, C.c_int,
                                      C.c_int]
    L.orc_array_periodic_fill.argtypes = [_f64p, _l3, _l3, _l3, _l3]
    L.orc_periodic_plan.argtypes = [_u32p, _l3, _l3, C.c_void_p]
    L.orc_periodic_plan.restype = C.c_long
    L.orc_apply_plan.argtypes = [_f64p, C.c_long, C.c_long, C.c_long, _u32p, C.c_long]
    L.orc_compare_brick.argtypes = [_l3, _l3, _l3, _f64p, _u32p, _f64p, C.c_long, C.c_long,
                                    _i3, _i3, C.c_double, _f64p]
    L.orc_compare_brick.restype = C.c_long
    L.orc_max_threads.restype = C.c_int
    return L


def ref() -> Optional[C.CDLL]:
    """The reference-compiled checker, or None where it was not built."""
    global _ref
    if _ref is None and os.path.exists(REF_PATH):
        R = C.CDLL(REF_PATH)
        R.ref_layout_offsets.argtypes = [C.c_int, _i64p]
        R.ref_init_grid.argtypes = [C.c_long, C.c_long, C.c_long, _u32p, _u32p]
        R.ref_sweep.argtypes = [C.c_int, C.c_long, _f64p, C.c_int, _i32p, _f64p, _f64p, _f64p]
        R.ref_cond.argtypes = [C.c_long, _f64p, _f64p, _f64p, _f64p]
        R.ref_layout_offsets4.argtypes = [C.c_int, _i64p]
        R.ref_init_grid4.argtypes = [C.c_long, C.c_long, C.c_long, C.c_long, _u32p, _u32p]
        R.ref_sweep4.argtypes = [C.c_int, C.c_long, _f64p, C.c_int, _i32p, _f64p, _f64p, _f64p]
        R.ref_skin_list.argtypes = [C.c_int, C.c_void_p]
        R.ref_allneighbors.argtypes = [C.c_int, C.c_void_p]
        R.ref_decomp.argtypes = [C.c_int, _u32p, C.c_uint, C.c_uint, C.c_long, C.c_long, _u64p, C.c_uint, _i64p,
                                 C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        _ref = R
    return _ref


# ---------------------------------------------------------------- helpers

def fill_uniform(n: int, seed: int, lo: float = -1.0, hi: float = 1.0) -> np.ndarray:
    a = np.empty(n, dtype=np.float64)
    lib().orc_fill_uniform(a, n, seed, lo, hi)
    return a


def fill_sines(dims, org, n, nw: int, seed: int, noise: float) -> np.ndarray:
    a = np.empty(int(np.prod(dims)), dtype=np.float64)
    lib().orc_fill_sines(a, _l3(*dims), _l3(*org), _l3(*n), nw, seed, noise)
    return a.reshape(dims)


def init_grid(gk: int, gj: int, gi: int) -> Tuple[np.ndarray, np.ndarray]:
    grid = np.empty(gk * gj * gi, dtype=np.uint32)
    adj = np.empty(gk * gj * gi * 27, dtype=np.uint32)
    lib().orc_init_grid(grid, adj, gk, gj, gi)
    return grid, adj


def brick_offset(bdim, fold, k, j, i) -> int:
    return lib().orc_brick_offset(_i3(*bdim), _i3(*fold), k, j, i)


def copy_brick(to_brick: bool, dim, pad, ghost, arr: np.ndarray, grid: np.ndarray,
               dat: np.ndarray, step: int, off: int, bdim, fold) -> None:
    lib().orc_copy_brick(1 if to_brick else 0, _l3(*dim), _l3(*pad), _l3(*ghost), arr.reshape(-1),
                         grid, dat.reshape(-1), step, off, _i3(*bdim), _i3(*fold))


def brick_sweep(adj, inp, in_step, in_off, out, out_step, out_off, blist, bdim, fold,
                offs: np.ndarray, coeff: np.ndarray, nthreads: int = 0, pre: int = 0, post: int = 0,
                timed: bool = False) -> None:
    """The brick sweep on the parity build, or with `timed` on the timed build (CPU baseline)."""
    offs = np.ascontiguousarray(offs, dtype=np.int32).reshape(-1)
    coeff = np.ascontiguousarray(coeff, dtype=np.float64)
    L = timed_lib() if timed else lib()
    if pre or post:
        L.orc_brick_sweep_ops(adj, inp.reshape(-1), in_step, in_off, out.reshape(-1), out_step, out_off,
                                  blist, len(blist), _i3(*bdim), _i3(*fold), len(coeff), offs, coeff, pre, post,
                                  nthreads)
        return
    fn = L.orc_brick_sweep if inp.dtype == np.float64 else L.orc_brick_sweep_f32
    fn(adj, inp.reshape(-1), in_step, in_off, out.reshape(-1), out_step, out_off,
       blist, len(blist), _i3(*bdim), _i3(*fold), len(coeff), offs, coeff, nthreads)


def array_sweep(inp: np.ndarray, out: np.ndarray, lo, hi, offs, coeff, nthreads: int = 0,
                pre: int = 0, post: int = 0) -> None:
    offs = np.ascontiguousarray(offs, dtype=np.int32).reshape(-1)
    coeff = np.ascontiguousarray(coeff, dtype=np.float64)
    lib().orc_array_sweep_ops(inp.reshape(-1), out.reshape(-1), _l3(*inp.shape), _l3(*lo), _l3(*hi),
                              len(coeff), offs, coeff, pre, post, nthreads)


def array_periodic_fill(a: np.ndarray, org, n, ghost) -> None:
    lib().orc_array_periodic_fill(a.reshape(-1), _l3(*a.shape), _l3(*org), _l3(*n), _l3(*ghost))


def periodic_plan(grid: np.ndarray, nb, gb) -> np.ndarray:
    cnt = lib().orc_periodic_plan(grid, _l3(*nb), _l3(*gb), None)
    pairs = np.empty(2 * cnt, dtype=np.uint32)
    lib().orc_periodic_plan(grid, _l3(*nb), _l3(*gb), pairs.ctypes.data)
    return pairs.reshape(-1, 2)


def apply_plan(dat: np.ndarray, step: int, off: int, belems: int, pairs: np.ndarray) -> None:
    p = np.ascontiguousarray(pairs, dtype=np.uint32).reshape(-1)
    lib().orc_apply_plan(dat.reshape(-1), step, off, belems, p, len(p) // 2)


def compare_brick(dim, pad, ghost, arr, grid, dat, step, off, bdim, fold, tol) -> Tuple[int, float, float]:
    stats = np.zeros(2, dtype=np.float64)
    bad = lib().orc_compare_brick(_l3(*dim), _l3(*pad), _l3(*ghost), arr.reshape(-1), grid,
                                  dat.reshape(-1), step, off, _i3(*bdim), _i3(*fold), tol, stats)
    return int(bad), float(stats[0]), float(stats[1])


def max_threads() -> int:
    return int(lib().orc_max_threads())


# ------------------------------------------------- the reference's single-node setup

class Domain:
    """The reference's single-node layout (stencils/stencils.h:11-26): an n^3
    interior, a ghost zone of one brick (GZ = 8) and array padding (PADDING = 8);
    the brick grid covers interior + ghost with init_grid."""

    def __init__(self, n, bdim=(8, 8, 8), fold=(1, 4, 8), ghost=8, pad=8, nfields=2):
        n = (n, n, n) if np.isscalar(n) else tuple(n)
        self.n, self.bdim, self.fold = n, tuple(bdim), tuple(fold)
        self.ghost, self.pad = ghost, pad
        self.adims = tuple(x + 2 * (ghost + pad) for x in n)
        self.gdims = tuple((x + 2 * ghost) // b for x, b in zip(n, bdim))
        self.gb = tuple(ghost // b for b in bdim)
        self.nb = tuple(x // b for x, b in zip(n, bdim))
        self.grid, self.adj = init_grid(*self.gdims)
        self.nbricks = len(self.grid)
        self.bsize = int(np.prod(bdim))
        self.step = self.bsize * nfields
        g3 = self.grid.reshape(self.gdims)
        gb = self.gb
        self.interior = np.ascontiguousarray(
            g3[gb[0]:gb[0] + self.nb[0], gb[1]:gb[1] + self.nb[1], gb[2]:gb[2] + self.nb[2]].reshape(-1))

    def alloc(self, dtype=np.float64) -> np.ndarray:
        return np.zeros(self.nbricks * self.step, dtype=dtype)

    def to_bricks(self, arr: np.ndarray, dat: np.ndarray, off: int) -> None:
        """copyToBrick over interior + ghost (3axis.cpp:26-30 call shape)."""
        g = tuple(x + 2 * self.ghost for x in self.n)
        copy_brick(True, g, (self.pad,) * 3, (0, 0, 0), arr, self.grid, dat, self.step, off,
                   self.bdim, self.fold)

    def from_bricks(self, dat: np.ndarray, off: int) -> np.ndarray:
        """copyFromBrick of the interior into a fresh padded array."""
        arr = np.zeros(self.adims, dtype=np.float64)
        copy_brick(False, self.n, (self.pad,) * 3, (self.ghost,) * 3, arr, self.grid, dat,
                   self.step, off, self.bdim, self.fold)
        return arr

    def interior_view(self, arr: np.ndarray) -> np.ndarray:
        o = self.ghost + self.pad
        return arr[o:o + self.n[0], o:o + self.n[1], o:o + self.n[2]]

    def compare(self, arr, dat, off, tol) -> Tuple[int, float, float]:
        return compare_brick(self.n, (self.pad,) * 3, (self.ghost,) * 3, arr, self.grid, dat,
                             self.step, off, self.bdim, self.fold, tol)
