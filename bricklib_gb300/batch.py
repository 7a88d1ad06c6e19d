"""Batched form: many uneven periodic domains advanced together by one persistent launch
per step over a global brick work list, T steps replayed from a captured CUDA graph
(bk_batch_*), and the autotuner that picks the brick dims, vector fold and CTA count.

Workload: 256 domains, each edge log-uniform on [16, 192] rounded to a multiple of 8
(anisotropic), stencil drawn uniformly from {7pt, 13pt, 27pt, 125pt}, FP32 storage, 10 steps,
periodic boundaries (through the adjacency, or ghost bricks refreshed before every step).
"""
from __future__ import annotations

import ctypes as C
import hashlib
import json
import os
import time
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

from . import _abi, bricks as B, stencils
from ._abi import BK_ACC_NATIVE, BK_F32, BK_F64, call

BATCH_SHAPES = ("star7", "star13", "cube27", "cube125")
CANDIDATES = [  # (bdim, fold)
    ((8, 8, 8), (1, 4, 8)), ((8, 8, 8), (1, 1, 8)), ((8, 8, 8), (2, 4, 4)),
    ((4, 4, 4), (1, 4, 4)), ((16, 8, 8), (1, 4, 8)), ((8, 8, 32), (1, 1, 32)),
]
CACHE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "lib", "autotune_cache.json")


@dataclass
class DomainSpec:
    n: Tuple[int, int, int]  # interior (k, j, i)
    stencil: int             # index into the workload's stencil list
    seed: int


@dataclass
class Workload:
    domains: List[DomainSpec]
    stencils: List[stencils.Stencil]

    @property
    def points(self) -> int:
        return int(sum(np.prod(d.n) for d in self.domains))

    def signature(self) -> str:
        h = hashlib.sha1()
        for d in self.domains:
            h.update(f"{d.n}:{d.stencil};".encode())
        return h.hexdigest()[:16]


def make_workload(ndom: int = 256, seed: int = 4, lo: int = 16, hi: int = 192, multiple: int = 8,
                  shapes: Sequence[str] = BATCH_SHAPES) -> Workload:
    u = stencils.uniform01(seed, ndom * 4)
    doms = []
    for d in range(ndom):
        edges = []
        for a in range(3):
            e = np.exp(np.log(lo) + (np.log(hi) - np.log(lo)) * u[4 * d + a])
            edges.append(int(max(multiple, round(e / multiple) * multiple)))
        doms.append(DomainSpec(tuple(edges), int(u[4 * d + 3] * len(shapes)) % len(shapes), seed * 100003 + d))
    return Workload(doms, [stencils.make(s, seed) for s in shapes])


def periodic_adjacency(adj: np.ndarray, pairs: np.ndarray) -> np.ndarray:
    """The adjacency with the periodic boundary in it: every entry that names a ghost brick
    (a `dst` of the periodic plan `pairs`) names the interior brick the fill copies into it
    (its `src`) instead."""
    src = np.arange(len(adj), dtype=np.uint32)
    pairs = np.asarray(pairs, dtype=np.uint32).reshape(-1, 2)
    src[pairs[:, 0]] = pairs[:, 1]
    return np.ascontiguousarray(src[np.asarray(adj, dtype=np.uint32)])


def layout_valid(w: Workload, lay: B.Layout) -> bool:
    """Every domain fits the brick dims: edges that are not whole bricks are padded to whole
    bricks (the periodic boundary then runs as a cell-level wrap fill), which needs every
    stencil radius within one brick and within the domain."""
    rmax = max(s.radius for s in w.stencils)
    return all(rmax <= lay.bdim[a] and rmax <= d.n[a] for d in w.domains for a in range(3))


def partial(spec: DomainSpec, lay: B.Layout) -> bool:
    """Whether some edge of the domain is not a whole number of bricks."""
    return any(spec.n[a] % lay.bdim[a] for a in range(3))


class DomainStorage:
    """One periodic domain on the device: init_grid over interior + one ghost brick per side,
    two interleaved fields, interior list and periodic plan (host arrays for the batch).

    wrap=False keeps the reference's layout: ghost bricks, refreshed from the periodic plan
    before a step.  wrap=True applies the periodic boundary through the adjacency instead:
    every reference to a ghost brick points at the interior brick the fill would copy into it,
    so the sweep reads the same values and no fill runs (the ghost bricks stay unused)."""

    @staticmethod
    def bricks(spec: DomainSpec, lay: B.Layout) -> int:
        return int(np.prod([-(-spec.n[a] // lay.bdim[a]) + 2 for a in range(3)]))

    def __init__(self, spec: DomainSpec, lay: B.Layout, dtype: int, wrap: bool = False,
                 storage: Optional[B.BrickStorage] = None):
        self.spec, self.lay, self.dtype = spec, lay, dtype
        # a domain whose edges are not whole bricks is padded to whole bricks; its periodic
        # boundary is then the batch's cell-level wrap fill (the ghost bricks hold the wrapped
        # cells), not the adjacency or a brick-pair plan
        self.partial = partial(spec, lay)
        nb = tuple(-(-spec.n[a] // lay.bdim[a]) for a in range(3))
        self.gdims = tuple(x + 2 for x in nb)
        self.grid, info = B.init_grid(list(reversed(self.gdims)))
        self.nbricks = info.nbricks
        g3 = self.grid.reshape(self.gdims)
        self.interior = np.ascontiguousarray(g3[1:-1, 1:-1, 1:-1].reshape(-1))
        if self.partial:
            pairs = np.zeros((0, 2), dtype=np.uint32)
            wrap = False
        else:
            pairs = B.GhostPlan.periodic(self.grid, nb, (1, 1, 1)).host
        if wrap:
            info = B.BrickInfo(self.nbricks, periodic_adjacency(info.adj, pairs))
            pairs = np.zeros((0, 2), dtype=np.uint32)
        self.wrap = wrap
        self.pairs = pairs
        self.info = B.movBrickInfo(info)
        self.storage = storage if storage is not None else B.BrickStorage.allocate_device(self.nbricks, 2 * lay.size,
                                                                                         dtype)

    def field(self, which: int) -> B.Brick:
        return B.Brick(self.info, self.storage, which * self.lay.size, self.lay)

    def desc(self, stencil: int) -> _abi.bk_batch_domain:
        d = _abi.bk_batch_domain()
        d.adj, d.nbricks = self.info.ptr, self.nbricks
        d.dat, d.chunks, d.step = self.storage.ptr, self.nbricks, 2 * self.lay.size
        d.off0, d.off1 = 0, self.lay.size
        d.blist, d.nlist = self.interior.ctypes.data, len(self.interior)
        d.pairs, d.npairs = self.pairs.ctypes.data, len(self.pairs)
        d.stencil = stencil
        if self.partial:
            d.n = (C.c_long * 3)(*self.spec.n)
            d.gdims = (C.c_long * 3)(*self.gdims)
            d.grid = self.grid.ctypes.data
        return d

    def cells(self, which: int) -> np.ndarray:
        """Field `which` of the domain as an array of its cells (k, j, i), read back to the host."""
        host = B.movBrickStorage(self.storage, to_device=False).host.reshape(self.nbricks, -1)
        lay = self.lay
        f = host[:, which * lay.size:(which + 1) * lay.size]
        off = lay.offsets().reshape(lay.bdim)  # element offset of (k, j, i) in a brick
        nb = [g - 2 for g in self.gdims]
        g3 = self.grid.reshape(self.gdims)[1:-1, 1:-1, 1:-1]
        full = f[g3.reshape(-1)][:, off.reshape(-1)].reshape(nb + list(lay.bdim))
        full = full.transpose(0, 3, 1, 4, 2, 5).reshape([nb[a] * lay.bdim[a] for a in range(3)])
        n = self.spec.n
        return full[:n[0], :n[1], :n[2]]


class Batch:
    """A bk_batch over freshly allocated domain storages, initialised with seeded uniform
    values (generated in FP64 and converted, so every storage type starts equal).  The
    periodic boundary goes through the adjacency (wrap=True, no ghost fill per step) unless
    wrap=False asks for ghost bricks refreshed by a batched fill before every step."""

    def __init__(self, w: Workload, lay: B.Layout, dtype: int = BK_F32, acc: int = BK_ACC_NATIVE,
                 grid_cap: int = 0, stream=None, init: bool = True, wrap: bool = True, arena: bool = True):
        self.w, self.lay, self.dtype = w, lay, dtype
        if arena:
            # every domain a range of bricks of one storage: bk_batch then sweeps the batch as
            # one brick set through the plain kernels (stars take the TMA-fed ones)
            step = 2 * lay.size
            counts = [DomainStorage.bricks(d, lay) for d in w.domains]
            bb = step * B.ELEM_SIZE[B.dtype_of(dtype)]
            self.arena = B.DeviceBuffer(sum(counts) * bb)
            call("bk_memset", C.c_void_p(self.arena.ptr), 0, self.arena.nbytes, None)
            firsts = np.concatenate([[0], np.cumsum(counts)[:-1]]).astype(int)
            views = [B.BrickStorage(c, step, dtype, device=B.DeviceView(self.arena, f * bb, c * bb))
                     for c, f in zip(counts, firsts)]
            self.doms = [DomainStorage(d, lay, dtype, wrap=wrap, storage=v) for d, v in zip(w.domains, views)]
        else:
            self.arena = None
            self.doms = [DomainStorage(d, lay, dtype, wrap=wrap) for d in w.domains]
        if init:
            for ds in self.doms:
                init_domain(ds, stream)
        descs = (_abi.bk_batch_domain * len(self.doms))(*[ds.desc(d.stencil) for ds, d in zip(self.doms, w.domains)])
        sts = (_abi.bk_stencil * len(w.stencils))(*[B.to_c_stencil(s) for s in w.stencils])
        h = C.c_void_p()
        call("bk_batch_create", C.byref(h), descs, len(self.doms), sts, len(w.stencils), C.byref(lay.to_c()), dtype, acc)
        self.h = h
        if grid_cap:
            call("bk_batch_set_grid", self.h, grid_cap)

    def run(self, steps: int, use_graph: bool = True, fill_every: int = 1, stream=None) -> None:
        call("bk_batch_run", self.h, steps, fill_every, 1 if use_graph else 0, B.stream_ptr(stream))

    @property
    def parity(self) -> int:
        return lib_parity(self.h)

    def close(self) -> None:
        if self.h:
            call("bk_batch_destroy", self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def lib_parity(h) -> int:
    return int(_abi.lib().bk_batch_parity(h))


def init_domain(ds: DomainStorage, stream=None) -> None:
    """Seeded uniform[-1, 1) values in field 0 (generated in FP64, converted to the storage type)."""
    if ds.dtype == BK_F64:
        call("bk_fill_uniform", C.c_void_p(ds.storage.ptr), ds.nbricks * 2 * ds.lay.size, BK_F64, ds.spec.seed,
             -1.0, 1.0, B.stream_ptr(stream))
        return
    tmp = B.BrickStorage.allocate_device(ds.nbricks, 2 * ds.lay.size, BK_F64)
    call("bk_fill_uniform", C.c_void_p(tmp.ptr), ds.nbricks * 2 * ds.lay.size, BK_F64, ds.spec.seed, -1.0, 1.0,
         B.stream_ptr(stream))
    allb = B.BrickList(ds.grid)
    B.convertField(B.Brick(ds.info, tmp, 0, ds.lay), ds.field(0), allb, stream)
    B.synchronize(stream)


def time_batch(b: Batch, steps: int, reps: int = 3, stream=None) -> float:
    """Seconds per `steps`-step run (graph replay), best of `reps`, CUDA-event timed."""
    import torch
    s = torch.cuda.current_stream() if stream is None else stream
    b.run(steps, stream=s.cuda_stream)  # capture + warm-up
    torch.cuda.synchronize()
    best = 1e30
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        b.run(steps, stream=s.cuda_stream)
        e1.record(s)
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1) * 1e-3)
    return best


def autotune(w: Workload, dtype: int = BK_F32, acc: int = BK_ACC_NATIVE, steps: int = 10,
             candidates=CANDIDATES, grid_caps=(0,), concurrency=(1, 0), stages=(0, 2, 3),
             use_cache: bool = True) -> Dict:
    """Time every (brick dims, fold) candidate -- domains whose edges are not whole bricks
    padded to whole bricks with the cell-level wrap fill -- with the stencil segments of a step
    as parallel graph branches or one after another, and, on the layouts whose stars run the
    TMA-fed kernels (8^3 row-major bricks), each pipeline depth in `stages` (0: the kernels'
    defaults); any CTA caps given bound the batch-mode kernels of domains in storages of their
    own.  Return the best with the full table.  Results are cached per (workload, dtype, acc,
    GPU)."""
    import torch
    key = f"{w.signature()}:{dtype}:{acc}:{torch.cuda.get_device_name()}"
    cache = {}
    if use_cache and os.path.exists(CACHE):
        try:
            cache = json.load(open(CACHE))
        except Exception:
            cache = {}
        if key in cache:
            return cache[key]
    table = []
    for bdim, fold in candidates:
        lay = B.Layout(bdim, fold)
        if not layout_valid(w, lay):
            table.append({"bdim": bdim, "fold": fold, "skipped": "a stencil radius exceeds a brick or a domain edge"})
            continue
        b = Batch(w, lay, dtype, acc)
        npart = sum(1 for ds in b.doms if ds.partial)
        tma = tuple(bdim) == (8, 8, 8) and lay.row_major()
        for conc in concurrency:
            call("bk_batch_set_concurrent", b.h, conc)
            for stg in (stages if tma else (0,)):
                call("bk_batch_set_stages", b.h, stg)
                for cap in grid_caps:
                    call("bk_batch_set_grid", b.h, cap)
                    t = time_batch(b, steps)
                    table.append({"bdim": bdim, "fold": fold, "concurrent": conc, "stages": stg, "grid_cap": cap,
                                  "partial_domains": npart, "s_per_run": t,
                                  "gstencil_s": w.points * steps / t / 1e9})
        b.close()
        del b
    best = max((r for r in table if "gstencil_s" in r), key=lambda r: r["gstencil_s"])
    res = {"best": best, "table": table}
    if use_cache:
        cache[key] = res
        os.makedirs(os.path.dirname(CACHE), exist_ok=True)
        json.dump(cache, open(CACHE, "w"), indent=1)
    return res
