"""Precision form: the same time-stepped problem stored in FP64, FP32 and BF16 (FP32
accumulation, compensated for the 125-point cube), with the error of every lower-precision
run measured on the device in FP64 against the FP64 run.

Problem: a periodic n^3 interior with an 8-cell ghost zone, initial
field = sum of 8 seeded random-phase sines + 1e-3 uniform noise (bk_fill_sines); the
7-point explicit heat step (centre 0.4, axes 0.1 = dt*alpha/h^2, stencils/mpi7pt.py with
fake.h:11-12) and the 125-point cube; ghost bricks refreshed from the periodic plan before
every step.  The FP64 run is the device's native FP64 path, itself checked against the CPU
oracle in the tests.
"""
from __future__ import annotations

import time
from typing import Dict, Iterable, List, Optional

import numpy as np

from . import bricks as B
from . import stencils
from ._abi import BK_ACC_COMPENSATED, BK_ACC_FLOATFLOAT, BK_ACC_NATIVE, BK_BF16, BK_F32, BK_F64

VARIANTS = {  # name: (storage, accumulation for star / for cube)
    "f64": (BK_F64, BK_ACC_NATIVE, BK_ACC_NATIVE),
    "f64-floatfloat": (BK_F64, BK_ACC_FLOATFLOAT, BK_ACC_FLOATFLOAT),
    "f32": (BK_F32, BK_ACC_NATIVE, BK_ACC_COMPENSATED),
    "bf16": (BK_BF16, BK_ACC_NATIVE, BK_ACC_COMPENSATED),
}


class PeriodicProblem:
    """Device storage for one storage type: two interleaved fields (ping-pong) on an
    init_grid layout of (n/8 + 2)^3 bricks."""

    def __init__(self, n: int, dtype: int, layout: B.Layout = B.DEFAULT_LAYOUT):
        self.n, self.dtype, self.layout = n, dtype, layout
        g = (n + 16) // 8
        self.gdims = (g, g, g)
        self.grid, info = B.init_grid([g, g, g])
        self.info = B.movBrickInfo(info)
        self.nbricks = info.nbricks
        g3 = self.grid.reshape(g, g, g)
        self.interior = B.BrickList(np.ascontiguousarray(g3[1:-1, 1:-1, 1:-1].reshape(-1)))
        self.all = B.BrickList(self.grid)
        self.plan = B.GhostPlan.periodic(self.grid, (g - 2,) * 3, (1, 1, 1))
        self.storage = B.BrickStorage.allocate_device(self.nbricks, 2 * layout.size, dtype)

    def field(self, which: int) -> B.Brick:
        return B.Brick(self.info, self.storage, which * self.layout.size, self.layout)


def run_study(n: int = 512, shapes: Iterable[str] = ("heat7", "cube125"),
              variants: Iterable[str] = ("f32", "bf16", "f64-floatfloat"), steps: Iterable[int] = (1, 10, 100),
              seed: int = 20261203, stream=None, timing: bool = True) -> List[Dict]:
    """Run every (shape, variant) for max(steps) steps, measuring the error against the FP64
    run at each checkpoint in `steps`.  Returns one record per (shape, variant, steps)."""
    steps = sorted(set(int(s) for s in steps))
    ref = PeriodicProblem(n, BK_F64)
    out: List[Dict] = []
    for shape in shapes:
        st = B.to_c_stencil(stencils.make(shape, 5))
        cube = stencils.make(shape, 5).npoints > 13 and not stencils.make(shape, 5).is_star()
        runs = {}
        for v in variants:
            dt, acc_star, acc_cube = VARIANTS[v]
            runs[v] = (PeriodicProblem(n, dt), acc_cube if cube else acc_star)
        # identical initial values: generated in FP64, converted into every storage type
        B.fillSines(ref.field(0), ref.gdims, (1, 1, 1), 8, seed, 1e-3, stream)
        for v, (p, _) in runs.items():
            B.convertField(ref.field(0), p.field(0), ref.all, stream)
        done = 0
        for t in steps:
            todo = t - done
            B.timeSteps(ref.field(done % 2), ref.field((done + 1) % 2), ref.interior, st, todo, plan=ref.plan,
                        acc=BK_ACC_NATIVE, stream=stream)
            newest = t % 2
            B.synchronize(stream)
            for v, (p, acc) in runs.items():
                t0 = time.perf_counter()
                B.timeSteps(p.field(done % 2), p.field((done + 1) % 2), p.interior, st, todo, plan=p.plan, acc=acc,
                            stream=stream)
                B.synchronize(stream)
                dt_s = time.perf_counter() - t0
                nrm = B.fieldNorms(p.field(newest), ref.field(newest), p.interior, stream)
                rec = {"stencil": shape, "variant": v, "steps": t, "max_abs_err": nrm["max_abs"],
                       "rms_err": nrm["rms"], "max_rel_err": nrm["max_rel"], "rms_rel_err": nrm["rms_rel"],
                       "max_ref": nrm["max_ref"]}
                if timing:
                    rec["gstencil_s_incl_fill"] = round(todo * n ** 3 / dt_s / 1e9, 2)
                out.append(rec)
            done = t
    return out
