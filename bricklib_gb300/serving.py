"""Serving form: Python client of the continuous-batching server (bk_server_*), the mixed
job set and a Poisson load generator.

Jobs: a periodic domain drawn as in the batched form (each edge log-uniform on [16, 192],
rounded to a multiple of 8), a stencil from the five plain shapes, a step count uniform on
[1, 200], FP64 or FP32 storage with equal probability; admission against a 150 GB HBM
budget.  Latency is submission to result-in-host-memory; throughput is completed
point-steps over the span from first submission to last completion.
"""
from __future__ import annotations

import ctypes as C
import threading
import time
from dataclasses import dataclass
from typing import Dict, List, Optional, Sequence

import numpy as np

from . import _abi, bricks as B, stencils
from ._abi import BK_ACC_NATIVE, BK_F32, BK_F64, call


class Server:
    def __init__(self, budget_bytes: float = 150e9, layout: B.Layout = B.DEFAULT_LAYOUT, max_active: int = 1024):
        h = C.c_void_p()
        call("bk_server_create", C.byref(h), int(budget_bytes), C.byref(layout.to_c()), max_active)
        self.h, self.layout = h, layout
        self._keep: Dict[int, tuple] = {}
        self._mu = threading.Lock()

    def submit(self, n, stencil, steps: int, dtype: int, acc: int, inp: np.ndarray, out: np.ndarray) -> int:
        cst = stencil if isinstance(stencil, _abi.bk_stencil) else B.to_c_stencil(stencil)
        d = _abi.bk_job_desc()
        d.n[0], d.n[1], d.n[2] = n
        d.stencil = C.pointer(cst)
        d.steps, d.dtype, d.acc = steps, dtype, acc
        d.input, d.output = inp.ctypes.data, out.ctypes.data
        jid = C.c_ulonglong()
        call("bk_server_submit", self.h, C.byref(d), C.byref(jid))
        with self._mu:
            self._keep[jid.value] = (cst, inp, out)
        return jid.value

    def wait(self, jid: int, timeout: float = 60.0) -> float:
        lat = C.c_double()
        call("bk_server_wait", self.h, jid, timeout, C.byref(lat))
        with self._mu:
            self._keep.pop(jid, None)
        return lat.value

    def drain(self, timeout: float = 600.0) -> None:
        call("bk_server_drain", self.h, timeout)

    def stats(self) -> dict:
        s = _abi.bk_server_report()
        call("bk_server_stats", self.h, C.byref(s))
        return {f: getattr(s, f) for f, _ in _abi.bk_server_report._fields_}

    def close(self) -> None:
        if self.h:
            call("bk_server_destroy", self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


@dataclass
class JobSpec:
    n: tuple
    shape: str
    steps: int
    dtype: int
    seed: int

    @property
    def points(self) -> int:
        return int(np.prod(self.n))


def make_jobs(njobs: int, seed: int = 11, lo: int = 16, hi: int = 192, max_steps: int = 200,
              shapes: Sequence[str] = stencils.PLAIN_SHAPES, fp64_frac: float = 0.5) -> List[JobSpec]:
    """Seeded jobs: edges log-uniform on [lo, hi] (multiples of 8), a shape, steps uniform on
    [1, max_steps], FP64 storage with probability fp64_frac, else FP32."""
    u = stencils.uniform01(seed, njobs * 6)
    jobs = []
    for q in range(njobs):
        e = [int(max(8, round(np.exp(np.log(lo) + (np.log(hi) - np.log(lo)) * u[6 * q + a]) / 8) * 8))
             for a in range(3)]
        shape = shapes[int(u[6 * q + 3] * len(shapes)) % len(shapes)]
        steps = 1 + int(u[6 * q + 4] * max_steps) % max_steps
        dtype = BK_F64 if u[6 * q + 5] < fp64_frac else BK_F32
        jobs.append(JobSpec(tuple(e), shape, steps, dtype, seed * 7919 + q))
    return jobs


def job_arrays(jobs: Sequence[JobSpec], pinned: bool = True):
    """Input (seeded uniform[-1, 1)) and output arrays for every job, carved from one
    page-locked arena when `pinned`."""
    sizes = [j.points * (8 if j.dtype == BK_F64 else 4) for j in jobs]
    arena = B.PinnedBuffer(2 * sum(sizes) + 64) if pinned else None
    off = 0
    ins, outs = [], []
    for j, sz in zip(jobs, sizes):
        dt = np.float64 if j.dtype == BK_F64 else np.float32
        if arena is not None:
            a = arena.view(np.uint8)[off:off + sz].view(dt).reshape(j.n)
            off += sz
            o = arena.view(np.uint8)[off:off + sz].view(dt).reshape(j.n)
            off += sz
        else:
            a, o = np.empty(j.n, dt), np.empty(j.n, dt)
        a[...] = stencils.uniform(j.seed, j.points).reshape(j.n).astype(dt)
        ins.append(a)
        outs.append(o)
    return arena, ins, outs


def run_load(rate: float, njobs: int, seed: int = 11, budget: float = 150e9, fp64_acc: int = BK_ACC_NATIVE,
             max_active: int = 1024, fp64_frac: float = 0.5) -> dict:
    """Poisson arrivals at `rate` jobs/s of `njobs` jobs; returns the server statistics."""
    jobs = make_jobs(njobs, seed, fp64_frac=fp64_frac)
    arena, ins, outs = job_arrays(jobs)
    sts = {s: B.to_c_stencil(stencils.make(s, 5)) for s in stencils.PLAIN_SHAPES}
    srv = Server(budget, max_active=max_active)
    gaps = -np.log(np.maximum(stencils.uniform01(seed ^ 0xABC, njobs), 1e-12)) / rate
    t0 = time.perf_counter()
    due = t0
    ids = []
    for j, a, o, g in zip(jobs, ins, outs, gaps):
        due += g
        while True:
            now = time.perf_counter()
            if now >= due:
                break
            time.sleep(min(due - now, 0.002))
        acc = fp64_acc if j.dtype == BK_F64 else BK_ACC_NATIVE
        ids.append(srv.submit(j.n, sts[j.shape], j.steps, j.dtype, acc, a, o))
    submit_span = time.perf_counter() - t0
    srv.drain(3600.0)
    st = srv.stats()
    srv.close()
    st.update({"rate": rate, "njobs": njobs, "submit_span_s": submit_span,
               "offered_point_steps": float(sum(j.points * j.steps for j in jobs))})
    del arena
    return st


def plain_rate(njobs: int, seed: int = 11, fp64_frac: float = 0.5, dtype: int = BK_F64, stream=None) -> dict:
    """The jobs of run_load(njobs, seed, fp64_frac=...) run one after another through the plain
    drop-in path instead (each its own 8^3-brick domain with ghost bricks, a periodic ghost fill
    before every step, `dtype` storage): device time of the steps (CUDA events; set-up and copies
    excluded) and the aggregate GStencil/s, the comparator of the served rate."""
    import torch
    from . import batch as BT
    jobs = make_jobs(njobs, seed, fp64_frac=fp64_frac)
    s = torch.cuda.current_stream() if stream is None else stream
    w_st = [stencils.make(x, 5) for x in stencils.PLAIN_SHAPES]
    tot, work = 0.0, 0.0
    for j in jobs:
        ds = BT.DomainStorage(BT.DomainSpec(j.n, stencils.PLAIN_SHAPES.index(j.shape), j.seed), B.DEFAULT_LAYOUT, dtype)
        BT.init_domain(ds, s.cuda_stream)
        plan, lst = B.GhostPlan(ds.pairs), B.BrickList(ds.interior)
        st = B.to_c_stencil(w_st[stencils.PLAIN_SHAPES.index(j.shape)])
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        B.timeSteps(ds.field(0), ds.field(1), lst, st, j.steps, plan=plan, stream=s.cuda_stream)
        e1.record(s)
        torch.cuda.synchronize()
        tot += e0.elapsed_time(e1) * 1e-3
        work += float(j.points * j.steps)
        del ds
    return {"jobs": njobs, "seconds": tot, "point_steps": work, "gstencil_s": work / tot / 1e9}
