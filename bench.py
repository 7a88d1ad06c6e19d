"""Benchmark of the brick stencil sweep on one GB300 (or N independent replicas).

Workload (default): the plain FP64 drop-in at 512^3 interior + an 8-cell ghost zone,
8x8x8 bricks with the CUDA vector fold (4,8), one sweep each of the 7-point star (r=1),
13-point star (r=2), 25-point star (r=4), 27-point cube (r=1) and 125-point cube (r=2),
seeded uniform[-1,1) input and seeded coefficients normalised to sum 1.  One step = one
sweep of every shape.  GStencil/s = interior points x sweeps / seconds (the reference's
tot_elems * 1e-9 / time, weak/main.cu:315-317).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Under torchrun every rank runs the same workload on its own GPU (replicas: the sweep
has no exchange step on one node); the step time is the max over ranks.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

SHAPES = ("star7", "star13", "star25", "cube27", "cube125")
SEED_IN, SEED_COEFF = 20261203, 7
PEAKS_PATH = os.path.join(ROOT, "MEASURED_PEAKS.json")
TRAFFIC_PATH = os.path.join(ROOT, "profiles", "traffic.json")


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--n", type=int, default=512)
    p.add_argument("--dtype", default="f64", choices=["f64", "f32", "bf16"])
    p.add_argument("--acc", default="native", choices=["native", "compensated", "floatfloat"])
    p.add_argument("--shapes", default=",".join(SHAPES))
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--no-alt", action="store_true")
    p.add_argument("--no-forms", action="store_true")
    p.add_argument("--ndom", type=int, default=256)
    p.add_argument("--rates", default="200,2000")
    p.add_argument("--njobs", type=int, default=400)
    p.add_argument("--form", default="plain", choices=["plain", "precision", "batched", "serving", "next"],
                   help="plain: the FP64 drop-in bench line; precision: the precision-form error study; "
                        "next: array<->brick copies, ghost fill, BrickDecomp exchange and 4-D sweeps")
    return p.parse_args()


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(x: float) -> float:
    """The largest value of x over the ranks of the job (the slowest replica's time); x itself
    when the job has one rank.  Works on NCCL (device tensor) and gloo (host tensor) groups."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return x
    t = torch.tensor([float(x)], dtype=torch.float64, device="cuda" if dist.get_backend() == "nccl" else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def peaks():
    try:
        with open(PEAKS_PATH) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def traffic_table():
    try:
        with open(TRAFFIC_PATH) as f:
            return json.load(f)
    except Exception:
        return {}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device, self.proc, self.lines = device, None, []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                          "-lms", "100", "-i", str(self.device)],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            time.sleep(0.3)
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.15)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": mx, "reasons": ["unavailable"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------- our arm

def run_ours(args):
    import torch
    from bricklib_gb300 import _abi, bricks as B, stencils
    from bricklib_gb300._abi import call

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    call("bk_set_device", local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream
    dtype = B.DTYPE_NAMES[args.dtype]
    acc = {"native": _abi.BK_ACC_NATIVE, "compensated": _abi.BK_ACC_COMPENSATED,
           "floatfloat": _abi.BK_ACC_FLOATFLOAT}[args.acc]
    esize = B.ELEM_SIZE[dtype]
    shapes = args.shapes.split(",")

    n = args.n
    lay = B.DEFAULT_LAYOUT
    g = (n + 16) // 8
    grid, info = B.init_grid([g, g, g])
    nbricks = info.nbricks
    g3 = grid.reshape(g, g, g)
    interior = np.ascontiguousarray(g3[1:-1, 1:-1, 1:-1].reshape(-1))
    dinfo = B.movBrickInfo(info)
    blist = B.BrickList(interior)
    bsize = lay.size
    s_in = B.BrickStorage.allocate_device(nbricks, bsize, dtype)
    s_out = B.BrickStorage.allocate_device(nbricks, bsize, dtype)
    b_in, b_out = B.Brick(dinfo, s_in, 0, lay), B.Brick(dinfo, s_out, 0, lay)
    call("bk_fill_uniform", C.c_void_p(s_in.ptr), nbricks * bsize, dtype, SEED_IN, -1.0, 1.0, sp)
    sts = {name: stencils.make(name, SEED_COEFF) for name in shapes}
    csts = {name: B.to_c_stencil(st) for name, st in sts.items()}
    points = n ** 3

    def sweep(name):
        B.brickSweep(b_in, b_out, blist, csts[name], acc, stream=sp)

    # warm-up
    for _ in range(args.warmup):
        for name in shapes:
            sweep(name)
    torch.cuda.synchronize()
    if B.error_flags(sp) != 0:
        raise RuntimeError("device error flags raised during warm-up")

    K = args.steps
    ev = {name: [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(K)]
          for name in shapes}
    t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        t0.record(stream)
        for k in range(K):
            for name in shapes:
                ev[name][k][0].record(stream)
                sweep(name)
                ev[name][k][1].record(stream)
        t1.record(stream)
        torch.cuda.synchronize()
    if ws > 1:
        torch.distributed.barrier()
    total_ms = max_over_ranks(t0.elapsed_time(t1))
    per_shape_ms = {name: sum(a.elapsed_time(b) for a, b in ev[name]) / K for name in shapes}
    ms_per_step = total_ms / K
    value = ws * len(shapes) * points / (ms_per_step * 1e-3) / 1e9

    hbm, peak_kind = peaks()
    fp64_rate = C.c_double()
    call("bk_measure_fma_rate", _abi.BK_F64 if dtype == _abi.BK_F64 else _abi.BK_F32, sp, C.byref(fp64_rate))
    bytes_pt = 2 * esize
    per_shape = {}
    for name in shapes:
        ms = per_shape_ms[name]
        gst = points / (ms * 1e-3) / 1e9
        flops = sts[name].flops_per_point * points / (ms * 1e-3)
        per_shape[name] = {"ms": round(ms, 4), "gstencil_s": round(gst, 2),
                           "hbm_frac": round(gst * 1e9 * bytes_pt / (hbm * 1e9), 4),
                           "compute_frac": round(flops / fp64_rate.value, 4)}
    dom = max(shapes, key=lambda s: per_shape_ms[s])
    dom_ms = per_shape_ms[dom]
    achieved = points * bytes_pt / (dom_ms * 1e-3) / 1e9
    tr = traffic_table().get(f"{args.dtype}:{args.acc}:{dom}:{n}")
    instr = fp_instructions_per_point(sts[dom], acc, dtype)
    roofline = {"bound": "hbm", "achieved": round(achieved, 1), "peak": hbm, "unit": "GB/s",
                "frac": round(achieved / hbm, 4), "traffic": tr,
                "kernel": f"{B.sweepKernel(b_in, b_out, csts[dom], acc)} {dom}",
                "peak_source": f"{peak_kind} hbm_gbs",
                "compute": {"unit": "TFLOP/s", "achieved": round(sts[dom].flops_per_point * points / (dom_ms * 1e-3) / 1e12, 3),
                            "peak": round(fp64_rate.value / 1e12, 3),
                            "peak_source": f"measured {'FP64' if dtype == _abi.BK_F64 else 'FP32'} FMA rate (bk_measure_fma_rate)",
                            "fp_instructions_per_point": instr,
                            "pipe_frac": round(points / (dom_ms * 1e-3) * instr / (fp64_rate.value / 2), 4),
                            "note": "achieved counts 2 x taps flop per point; pipe_frac counts the floating-point "
                                    "instructions the kernel executes per point (mirror-symmetric cubes run on "
                                    "pair sums) against the measured FMA instruction rate"}}
    pipe_frac = roofline["compute"]["pipe_frac"]
    roofline["binding"] = (("fp64 pipe" if dtype == _abi.BK_F64 and acc != _abi.BK_ACC_FLOATFLOAT else "fp32 pipe")
                           if pipe_frac > roofline["frac"] else "hbm")

    # end to end through the public API, every result in host memory.  Per step: the input is
    # copied from page-locked memory (on a copy stream, into one of two device buffers, while the
    # previous step sweeps); each sweep writes its own device buffer, whose device-to-host copy runs
    # on a second copy stream under the following sweeps (one buffer per stencil, so no sweep waits
    # for an earlier result to leave its buffer, and the last results of a step leave under the
    # next step's first sweeps).  The link carries the input and the results in opposite
    # directions; the results (five fields per step) keep the device-to-host direction busy.
    e2e = None
    if not args.no_e2e:
        nbytes = nbricks * bsize * esize
        h_in = B.PinnedBuffer(nbytes)
        s_in2 = B.BrickStorage.allocate_device(nbricks, bsize, dtype)
        ins = [B.Brick(dinfo, s_in, 0, lay), B.Brick(dinfo, s_in2, 0, lay)]
        s_out2 = B.BrickStorage.allocate_device(nbricks, bsize, dtype)
        nbuf = max(2, len(shapes))
        s_outs = [s_out, s_out2] + [B.BrickStorage.allocate_device(nbricks, bsize, dtype) for _ in range(nbuf - 2)]
        outs = [B.Brick(dinfo, so, 0, lay) for so in s_outs]
        h_outs = {}
        for name in shapes:
            h_outs[name] = B.BrickStorage.allocate_pinned(nbricks, bsize, dtype)
            h_outs[name].host[:] = 0
        B.memcpy(h_in.ptr, s_in.ptr, nbytes, 1, sp)
        torch.cuda.synchronize()
        cin, cout = torch.cuda.Stream(), torch.cuda.Stream()
        arrived = [torch.cuda.Event(), torch.cuda.Event()]
        consumed = [torch.cuda.Event(), torch.cuda.Event()]
        swept = [torch.cuda.Event() for _ in range(nbuf)]
        copied = [torch.cuda.Event() for _ in range(nbuf)]
        Ke = max(1, min(K, 10))

        def h2d(buf):
            cin.wait_event(consumed[buf])
            B.memcpy(ins[buf].bStorage.ptr, h_in.ptr, nbytes, 0, cin.cuda_stream)
            arrived[buf].record(cin)

        def e2e_trial():
            """Ke timed steps after one untimed step; ms per step."""
            for q in range(2):
                consumed[q].record(stream)
            for q in range(nbuf):
                copied[q].record(stream)
            h2d(0)
            for it in range(Ke + 1):
                cur = it % 2
                if it == 1:
                    torch.cuda.synchronize()
                    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                    e0.record(stream)
                if it < Ke:
                    h2d(1 - cur)  # the next step's input, while this step sweeps
                stream.wait_event(arrived[cur])
                for q, name in enumerate(shapes):
                    ob = q % nbuf
                    stream.wait_event(copied[ob])  # its previous result has left the buffer
                    B.brickSweep(ins[cur], outs[ob], blist, csts[name], acc, stream=sp)
                    swept[ob].record(stream)
                    cout.wait_event(swept[ob])
                    B.memcpy(h_outs[name].ptr, outs[ob].bStorage.ptr, nbytes, 1, cout.cuda_stream)
                    copied[ob].record(cout)
                consumed[cur].record(stream)
            for q in range(nbuf):
                stream.wait_event(copied[q])
            e1.record(stream)
            torch.cuda.synchronize()
            return max_over_ranks(e0.elapsed_time(e1) / Ke)

        # five trials, the median reported (all are listed): the host link and host memory are
        # shared with other work on the node, and single trials on one box ranged 31-52 ms per step
        trials = [e2e_trial() for _ in range(5)]
        e_ms = statistics.median(trials)
        # the link rates this box gives alone (after the timed region): one copy each way
        link = {}
        for key, dst, src, kind in (("h2d_gbs", s_in2.ptr, h_in.ptr, 0),
                                    ("d2h_gbs", h_in.ptr, s_out2.ptr, 1)):
            la, lb = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            la.record(stream)
            B.memcpy(dst, src, nbytes, kind, sp)
            lb.record(stream)
            torch.cuda.synchronize()
            link[key] = round(nbytes / (la.elapsed_time(lb) * 1e-3) / 1e9, 1)
        # every host result equals the device sweep's
        dev_out = np.empty(nbricks * bsize, dtype=B.NP_DTYPE[dtype])
        for name in shapes:
            sweep(name)
            B.memcpy(dev_out.ctypes.data, s_out.ptr, nbytes, 1, sp)
            B.synchronize(sp)
            if not np.array_equal(dev_out.view(np.uint8), h_outs[name].host.view(np.uint8)):
                raise RuntimeError(f"{name}: the result in host memory differs from the device sweep")
        e2e = {"value": round(ws * len(shapes) * points / (e_ms * 1e-3) / 1e9, 3), "unit": "GStencil/s",
               "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes * len(shapes), "ms_per_step": round(e_ms, 3),
               "trials_ms_per_step": [round(x, 3) for x in trials],
               "link_alone": link,
               "path": "input: cudaMemcpyAsync from page-locked memory into one of two device buffers on a copy "
                       "stream under the previous step's sweeps; results: device-to-host copies into page-locked "
                       "memory on a second stream under the following sweeps (one device buffer per stencil, the "
                       "last results of a step leaving under the next step's first sweeps); one host buffer per "
                       "stencil"}

    # the other FP64 arithmetic mode on the same data: per-stencil rate and its normwise
    # error against the first mode's output
    alt = None
    if dtype == _abi.BK_F64 and not args.no_alt:
        alt_acc = _abi.BK_ACC_FLOATFLOAT if acc == _abi.BK_ACC_NATIVE else _abi.BK_ACC_NATIVE
        alt = {"accumulation": "floatfloat" if alt_acc == _abi.BK_ACC_FLOATFLOAT else "native", "per_stencil": {}}
        nb = nbricks * bsize
        ref_out, alt_out = np.empty(nb), np.empty(nb)
        for name in shapes:
            sweep(name)
            B.memcpy(ref_out.ctypes.data, s_out.ptr, ref_out.nbytes, 1, sp)
            B.brickSweep(b_in, b_out, blist, csts[name], alt_acc, stream=sp)
            torch.cuda.synchronize()
            ea, eb = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            ea.record(stream)
            for _ in range(K):
                B.brickSweep(b_in, b_out, blist, csts[name], alt_acc, stream=sp)
            eb.record(stream)
            torch.cuda.synchronize()
            ms = ea.elapsed_time(eb) / K
            B.memcpy(alt_out.ctypes.data, s_out.ptr, alt_out.nbytes, 1, sp)
            B.synchronize(sp)
            live = np.concatenate([np.arange(int(b) * bsize, int(b) * bsize + bsize) for b in interior[:4096]])
            err = float(np.abs(alt_out[live] - ref_out[live]).max() / np.abs(ref_out[live]).max())
            gst = points / (ms * 1e-3) / 1e9
            alt["per_stencil"][name] = {"ms": round(ms, 4), "gstencil_s": round(gst, 2),
                                        "hbm_frac": round(gst * 1e9 * bytes_pt / (hbm * 1e9), 4),
                                        "normwise_err_vs_main": err}
        tot = sum(v["ms"] for v in alt["per_stencil"].values())
        alt["value"] = round(len(shapes) * points / (tot * 1e-3) / 1e9, 3)

    # CPU baseline: the oracle's OpenMP brick sweep on a sample of the same bricks,
    # also used as a spot check of the GPU output on those bricks
    cpu = None
    if not args.no_cpu and rank == 0 and dtype == _abi.BK_F64:
        cpu = cpu_baseline_on_device_data(B, s_in, s_out, info, interior, sts, shapes, lay, nbricks, bsize, sp,
                                          lambda name: (sweep(name), torch.cuda.synchronize()))

    forms = None
    if rank == 0 and not args.no_forms and args.n == 512 and dtype == _abi.BK_F64:
        forms = forms_record(args)

    if rank == 0:
        line = {"metric": "GStencil/s", "value": round(value, 3), "unit": "GStencil/s", "n_gpus": ws,
                "steps": K, "warmup": args.warmup, "ms_per_step": round(ms_per_step, 4),
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": {"f64": "f64", "f32": "f32", "bf16": "bf16"}[args.dtype],
                "data": "synthetic: seeded uniform[-1,1) input, seeded coefficients normalised to sum 1",
                "config": plain_config(args, shapes, nbricks, esize, ws),
                "per_stencil": per_shape, "alt_mode": alt, "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e,
                "forms": forms,
                "gpu_launches": K * len(shapes), "clocks": clk.summary()}
        print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()


def fp_instructions_per_point(st, acc, dtype=None) -> float:
    """Floating-point operations per point of the kernel that runs `st` on 8x8x8 row-major bricks:
    a multiply-add per tap, except mirror-symmetric cubes, which stream class sums along i
    (sweep2_kernel.cuh sym_cube_istream, FP64, and sym_cube_istream4, FP32 / BF16 storage): per
    point (R+1)R additions for the j pair sums H, R(R+1) for the k pair sums Q, R(R+1)/2 more
    when the coefficients are also symmetric under k <-> j, one operation per class and i
    distance for the W sums, 2R for the i taps (37 for the 125-point cube with k <-> j symmetry,
    43 without).  Compensated FP32 runs each W sum as Dot2 (ten operations per term after the
    first) and the output sum Neumaier-compensated.  Float-float and the other accumulation
    modes take a multiply-add per tap."""
    from bricklib_gb300 import _abi
    taps = [tuple(t) for t in st.taps]
    r = st.radius
    cube = len(taps) == (2 * r + 1) ** 3 and len(set(taps)) == len(taps) and r in (1, 2)
    comp = acc == _abi.BK_ACC_COMPENSATED and dtype in (_abi.BK_F32, _abi.BK_BF16)
    if not cube or not (acc == _abi.BK_ACC_NATIVE or comp):
        return float(len(taps))
    c = {t: v for t, v in zip(taps, st.coeff)}
    if any(c[t] != c[tuple(abs(a) for a in t)] for t in taps):
        return float(len(taps))
    kj = all(c[(k, j, i)] == c[(j, k, i)] for (k, j, i) in taps)
    ncls = (r + 1) * (r + 2) // 2 if kj else (r + 1) ** 2
    sums = (r + 1) * r + r * (r + 1) + (r * (r + 1) // 2 if kj else 0)
    if comp:
        return float(sums + (r + 1) * (2 + 10 * (ncls - 1)) + 10 * r + 2)
    return float(sums + (r + 1) * ncls + 2 * r)


def cpu_info(threads: int) -> dict:
    """The host the CPU leg ran on: core counts, CPU model and the OpenMP settings."""
    model = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                model = line.split(":", 1)[1].strip()
                break
    except (OSError, subprocess.SubprocessError):
        pass
    if not model:
        try:
            for line in open("/proc/cpuinfo"):
                if line.lower().startswith(("model name", "cpu part")):
                    model = line.split(":", 1)[1].strip()
                    break
        except OSError:
            pass
    try:
        affinity = len(os.sched_getaffinity(0))
    except AttributeError:
        affinity = os.cpu_count()
    return {"nproc": os.cpu_count(), "affinity": affinity, "threads_used": threads, "model": model or "unknown",
            "OMP_NUM_THREADS": os.environ.get("OMP_NUM_THREADS", "unset"),
            "OMP_PROC_BIND": os.environ.get("OMP_PROC_BIND", "unset")}


def plain_config(args, shapes, nbricks: int, esize: int, ws: int) -> dict:
    """The plain-form workload, identical in both arms' lines."""
    n = args.n
    return {"workload": f"plain {args.dtype} brick sweep, {n}^3 interior + 8-cell ghost, 8x8x8 bricks fold (4,8), "
                        f"one sweep each of {'/'.join(shapes)}",
            "interior_points": n ** 3, "bricks": nbricks, "accumulation": args.acc,
            "l2": (f"no flush: inputs {nbricks * 512 * esize / 1e9:.2f} GB per field > 129 MB L2"
                   if nbricks * 512 * esize > 129e6 else
                   f"inputs {nbricks * 512 * esize / 1e6:.1f} MB per field fit in L2: a small case, not a bench value"),
            "parallelism": f"replicas x{ws}"}


CPU_BUILD = ("the oracle's OpenMP brick sweep (gather of the rows the taps read, then taps in order per row), "
             "built as the reference builds its CPU path: gcc -O2 -fopenmp with default floating-point "
             "contraction (oracle/Makefile, target timed)")


def cpu_plain_steps(oracle, adj, host_in, out, interior, sts, shapes, steps: int, warmup: int, threads: int):
    """`warmup` then `steps` CPU steps of the plain workload (one sweep of each shape over every
    interior brick, separate input and output storages, as the GPU arm runs it); per-shape
    mean seconds and mean seconds per step."""
    per = {name: 0.0 for name in shapes}
    for it in range(warmup + steps):
        for name in shapes:
            st = sts[name]
            t = time.perf_counter()
            oracle.brick_sweep(adj, host_in, 512, 0, out, 512, 0, interior, (8, 8, 8), (1, 4, 8), st.offsets(),
                               st.coeff, threads, timed=True)
            if it >= warmup:
                per[name] += time.perf_counter() - t
    per = {k: v / steps for k, v in per.items()}
    return per, sum(per.values())


def cpu_baseline_on_device_data(B, s_in, s_out, info, interior, sts, shapes, lay, nbricks, bsize, sp, run_one):
    """The CPU leg of this arm: the same workload on the host cores (one untimed and two timed
    steps, ~10 s on 16 cores), from the device input; every interior point of every GPU result
    is then compared with the CPU result (normwise)."""
    from oracle import oracle
    host_in = np.empty(nbricks * bsize, dtype=np.float64)
    B.memcpy(host_in.ctypes.data, s_in.ptr, host_in.nbytes, 1, sp)
    B.synchronize(sp)
    adj = np.ascontiguousarray(info.adj.reshape(-1))
    threads = oracle.max_threads()
    out = np.zeros(nbricks * bsize, dtype=np.float64)
    per, step_s = cpu_plain_steps(oracle, adj, host_in, out, interior, sts, shapes, 2, 1, threads)
    points = len(interior) * bsize
    max_err = 0.0
    gpu = np.empty(nbricks * bsize, dtype=np.float64)
    rows = interior.astype(np.int64)
    for name in shapes:
        st = sts[name]
        oracle.brick_sweep(adj, host_in, bsize, 0, out, bsize, 0, interior, lay.bdim, lay.fold, st.offsets(),
                           st.coeff, threads, timed=True)
        run_one(name)
        B.memcpy(gpu.ctypes.data, s_out.ptr, gpu.nbytes, 1, sp)
        B.synchronize(sp)
        a, b = gpu.reshape(-1, bsize)[rows], out.reshape(-1, bsize)[rows]
        max_err = max(max_err, float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)))
    return {"value": round(len(shapes) * points / step_s / 1e9, 4), "unit": "GStencil/s", "cores": threads,
            "kind": "port",
            "sample": f"the whole workload ({len(shapes)} sweeps of {points} interior points per step), one untimed "
                      f"and two timed steps, {step_s:.2f} s per step; {CPU_BUILD}",
            "per_stencil": {k: round(points / v / 1e9, 4) for k, v in per.items()},
            "host": cpu_info(threads), "gpu_vs_cpu_max_normwise_err": max_err}


# ---------------------------------------------------------------------------- reference arm

def run_reference(args):
    """The reference's CPU brick path on the host cores, on this arm's workload and config: the
    same 512^3 input (the splitmix64 stream the device fill writes), the same bricks, fold, taps
    and separate input / output storages; each step one sweep of each shape."""
    ws, rank, local = dist_env()
    if rank != 0:
        return
    from bricklib_gb300 import stencils
    from oracle import oracle
    oracle.build()
    shapes = args.shapes.split(",")
    n = args.n
    g = n // 8 + 2
    grid, adj = oracle.init_grid(g, g, g)
    nbricks = g ** 3
    interior = np.ascontiguousarray(grid.reshape(g, g, g)[1:-1, 1:-1, 1:-1].reshape(-1))
    host_in = oracle.fill_uniform(nbricks * 512, SEED_IN)
    out = np.zeros(nbricks * 512)
    threads = oracle.max_threads()
    sts = {name: stencils.make(name, SEED_COEFF) for name in shapes}
    per, step_s = cpu_plain_steps(oracle, adj, host_in, out, interior, sts, shapes, args.steps, args.warmup, threads)
    value = len(shapes) * n ** 3 / step_s / 1e9
    cpu = {"value": round(value, 4), "unit": "GStencil/s", "cores": threads, "kind": "port",
           "sample": f"the whole workload, {args.warmup} untimed and {args.steps} timed steps; {CPU_BUILD}",
           "per_stencil": {k: round(n ** 3 / v / 1e9, 4) for k, v in per.items()}, "host": cpu_info(threads)}
    line = {"impl": "reference", "metric": "GStencil/s", "value": round(value, 4), "unit": "GStencil/s",
            "n_gpus": ws, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(step_s * 1e3, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic: seeded uniform[-1,1) input, seeded coefficients normalised to sum 1",
            "config": plain_config(args, shapes, nbricks, 8, ws),
            "cpu_baseline": cpu,
            "e2e": {"value": round(value, 4), "unit": "GStencil/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_precision(args):
    """The precision form (FP64 / FP32 / BF16 storage, 1, 10, 100 steps): one JSON line with
    the max and RMS error of every run against the FP64 run, per stencil and step count."""
    import torch
    from bricklib_gb300 import precision
    from bricklib_gb300._abi import call
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    call("bk_set_device", local)
    t = time.perf_counter()
    recs = precision.run_study(n=args.n, shapes=("heat7", "cube125"), variants=("f32", "bf16", "f64-floatfloat"),
                               steps=(1, 10, 100), stream=torch.cuda.current_stream().cuda_stream)
    if rank == 0:
        print(json.dumps({"form": "precision", "n": args.n, "seconds": round(time.perf_counter() - t, 1),
                          "reference": "FP64 native run on the device", "records": recs}), flush=True)


def batched_record(ndom: int, tune: bool, reps: int = 5) -> dict:
    """The batched form on `ndom` uneven periodic FP32 domains: 10 steps of all domains from one
    captured graph, against the plain FP64 drop-in run domain by domain and an unbatched FP32
    run of the same domains (both with their ghost fills), and the FP32 error against FP64.
    With `tune` the autotuner picks the layout first, else the default 8^3 bricks run."""
    import torch
    from bricklib_gb300 import _abi, batch as BT, bricks as B
    from bricklib_gb300._abi import call
    stream = torch.cuda.current_stream()
    w = BT.make_workload(ndom=ndom)
    steps = 10
    tune_rec = None
    if tune:
        t0 = time.perf_counter()
        res = BT.autotune(w, _abi.BK_F32, _abi.BK_ACC_NATIVE, steps=steps, use_cache=False)
        best = res["best"]
        lay, cap, conc = B.Layout(tuple(best["bdim"]), tuple(best["fold"])), best["grid_cap"], best["concurrent"]
        stg = best.get("stages", 0)
        tune_rec = {"seconds": round(time.perf_counter() - t0, 1), "table": res["table"]}
    else:
        lay, cap, conc, stg = B.DEFAULT_LAYOUT, 0, 1, 0
    bt = BT.Batch(w, lay, _abi.BK_F32)
    call("bk_batch_set_grid", bt.h, cap)
    call("bk_batch_set_concurrent", bt.h, conc)
    call("bk_batch_set_stages", bt.h, stg)
    t_batch = BT.time_batch(bt, steps, reps=reps)
    gst_batch = w.points * steps / t_batch / 1e9
    npart = sum(1 for ds in bt.doms if ds.partial)
    bt.close()

    def unbatched(dtype, lay_):
        tot = 0.0
        outs = []
        for spec in w.domains:
            ds = BT.DomainStorage(spec, lay_, dtype)
            BT.init_domain(ds, stream.cuda_stream)
            plan, lst = B.GhostPlan(ds.pairs), B.BrickList(ds.interior)
            st = B.to_c_stencil(w.stencils[spec.stencil])
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            B.timeSteps(ds.field(0), ds.field(1), lst, st, steps, plan=plan, stream=stream.cuda_stream)
            e1.record(stream)
            torch.cuda.synchronize()
            tot += e0.elapsed_time(e1) * 1e-3
            outs.append((ds, lst))
        return tot, outs

    # the plain drop-in path domain by domain, on its own 8^3 bricks
    t_plain64, _ = unbatched(_abi.BK_F64, B.DEFAULT_LAYOUT)
    t_plain32, _ = unbatched(_abi.BK_F32, B.DEFAULT_LAYOUT)
    # error of a fresh 10-step batched FP32 run against a batched FP64 run of the same domains
    # on the same layout, domain by domain over the domains' own cells
    chk = BT.Batch(w, lay, _abi.BK_F32)
    ref = BT.Batch(w, lay, _abi.BK_F64)
    chk.run(steps, stream=stream.cuda_stream)
    ref.run(steps, stream=stream.cuda_stream)
    torch.cuda.synchronize()
    worst = 0.0
    for ds32, ds64 in zip(chk.doms, ref.doms):
        if ds32.partial:
            a, r = ds32.cells(chk.parity).astype(np.float64), ds64.cells(ref.parity)
            worst = max(worst, float(np.abs(a - r).max() / np.abs(r).max()))
        else:
            lst = B.BrickList(ds32.interior)
            nrm = B.fieldNorms(ds32.field(chk.parity), ds64.field(ref.parity), lst)
            worst = max(worst, nrm["max_rel"])
    chk.close()
    ref.close()
    rec = {"metric": "GStencil/s", "unit": "GStencil/s", "domains": len(w.domains), "interior_points": w.points,
           "steps": steps,
           "batched_fp32": {"value": round(gst_batch, 2), "ms_per_10_steps": round(t_batch * 1e3, 3),
                            "layout": {"bdim": lay.bdim, "fold": lay.fold, "grid_cap": cap, "stages": stg,
                                       "chosen_by": "autotuner" if tune else "default 8^3 bricks"},
                            "segments": "parallel graph branches" if conc else "one after another",
                            "partial_brick_domains": npart,
                            "graph": True, "periodic": "through the adjacency (no ghost fill)"},
           "plain_fp64_per_domain": {"value": round(w.points * steps / t_plain64 / 1e9, 2),
                                     "ms": round(t_plain64 * 1e3, 2),
                                     "note": "the drop-in run domain by domain, ghost fill before every step"},
           "unbatched_fp32_per_domain": {"value": round(w.points * steps / t_plain32 / 1e9, 2),
                                         "ms": round(t_plain32 * 1e3, 2),
                                         "note": "the same FP32 arithmetic domain by domain, ghost fill every step"},
           "batched_vs_plain_fp64": round(t_plain64 / t_batch, 2),
           "batched_vs_unbatched_fp32": round(t_plain32 / t_batch, 2),
           "fp32_max_normwise_err_vs_fp64": worst,
           "comparators_layout": "plain path: 8^3 bricks, fold (4,8)"}
    if tune_rec:
        rec["autotune"] = tune_rec
    return rec


def run_batched(args):
    """The batched form (256 uneven periodic FP32 domains), the layout chosen by the autotuner."""
    import torch
    from bricklib_gb300._abi import call
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    call("bk_set_device", local)
    rec = batched_record(args.ndom, tune=True)
    if rank == 0:
        print(json.dumps({"form": "batched", **rec}), flush=True)


SERVING_JOBS = "edges log-uniform [16,192] (multiples of 8), 5 shapes, steps U[1,200], 50% FP64 / 50% FP32"


def run_serving(args):
    """The serving form (mixed FP64 / FP32 jobs of up to 256^3): Poisson arrivals of the mixed job set at each rate
    against the continuous-batching server; p50 / p99 latency and aggregate GStencil/s."""
    import torch
    from bricklib_gb300 import _abi, serving
    from bricklib_gb300._abi import call
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    call("bk_set_device", local)
    res = []
    for rate in [float(r) for r in args.rates.split(",")]:
        for acc_name, acc in (("native", _abi.BK_ACC_NATIVE), ("floatfloat", _abi.BK_ACC_FLOATFLOAT)):
            st = serving.run_load(rate, args.njobs, fp64_acc=acc)
            st["fp64_arithmetic"] = acc_name
            res.append(st)
    # the served FP32 form against the plain path on the same mixed-size jobs: all jobs FP32,
    # offered faster than the server completes them (its throughput), and the same jobs run one
    # by one through the plain drop-in path (FP64 storage)
    fp32 = serving.run_load(20000.0, args.njobs, fp64_frac=0.0)
    fp32["job_mix"] = "all FP32, otherwise as above"
    plain = serving.plain_rate(args.njobs, fp64_frac=0.0, dtype=_abi.BK_F64)
    if rank == 0:
        print(json.dumps({"form": "serving", "metric": "p50/p99 latency (s), GStencil/s", "budget_bytes": 150e9,
                          "jobs": SERVING_JOBS, "runs": res, "served_fp32": fp32,
                          "plain_fp64_same_jobs": plain,
                          "served_fp32_vs_plain_fp64": round(fp32["gstencil_s"] / plain["gstencil_s"], 2)}),
              flush=True)


def forms_record(args) -> dict:
    """The three forms in compact runs (about a minute together), for the default line: the
    batched form (default bricks, no autotuning), 200 served jobs at 200 and 2000 jobs/s, the
    precision form's errors after 1 and 10 steps at 512^3; and of the next rows the periodic ghost
    fill at 512^3 and the 4-D sweep."""
    import torch
    from bricklib_gb300 import _abi, precision, serving
    out = {}
    t = time.perf_counter()
    out["batched"] = batched_record(args.ndom, tune=False, reps=3)
    out["batched"]["seconds"] = round(time.perf_counter() - t, 1)
    t = time.perf_counter()
    runs = []
    for rate in (200.0, 2000.0):
        st = serving.run_load(rate, 200, fp64_acc=_abi.BK_ACC_NATIVE)
        runs.append({k: st[k] for k in ("rate", "p50_s", "p99_s", "gstencil_s", "completed") if k in st})
    out["serving"] = {"jobs": 200, "job_mix": SERVING_JOBS, "budget_bytes": 150e9, "fp64_arithmetic": "native",
                      "runs": runs, "seconds": round(time.perf_counter() - t, 1)}
    t = time.perf_counter()
    recs = precision.run_study(n=512, shapes=("heat7", "cube125"), variants=("f32", "bf16"), steps=(1, 10),
                               stream=torch.cuda.current_stream().cuda_stream, timing=False)
    out["precision"] = {"n": 512, "reference": "FP64 native run on the device",
                        "records": [{k: r[k] for k in ("stencil", "variant", "steps", "max_rel_err", "rms_rel_err")}
                                    for r in recs],
                        "seconds": round(time.perf_counter() - t, 1)}
    t = time.perf_counter()
    out["next"] = {"ghost_fill_512": ghost_record(20, 3), "sweep4_mpi9pt": sweep4_record(10, 3), "seconds": None}
    out["next"]["seconds"] = round(time.perf_counter() - t, 1)
    return out


def ghost_record(K: int, warmup: int) -> dict:
    """The periodic ghost fill of the 512^3 FP64 domain with one ghost brick a side (66^3 bricks,
    25,352 ghost bricks, each 4 KiB read from its periodic image and written): CUDA events
    around K fills after `warmup`, on the current stream."""
    import torch
    from bricklib_gb300 import _abi, bricks as B
    from bricklib_gb300._abi import call
    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream
    hbm, _ = peaks()
    gb = 512 // 8 + 2
    grid, info = B.init_grid([gb] * 3)
    st = B.BrickStorage.allocate_device(info.nbricks, 512, _abi.BK_F64)
    call("bk_fill_uniform", C.c_void_p(st.ptr), info.nbricks * 512, _abi.BK_F64, 3, -1.0, 1.0, sp)
    dinfo = B.movBrickInfo(info)
    brick = B.Brick(dinfo, st, 0)
    plan = B.GhostPlan.periodic(grid, (gb - 2,) * 3, (1, 1, 1))
    for _ in range(warmup):
        B.ghostFill(plan, brick, sp)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(K):
        B.ghostFill(plan, brick, sp)
    e1.record(stream)
    torch.cuda.synchronize()
    sec = e0.elapsed_time(e1) / K * 1e-3
    nbytes = 2 * plan.n * 512 * 8
    if B.error_flags() != 0:
        raise RuntimeError("ghost fill raised device error flags")
    return {"ghost_bricks": plan.n, "steps": K, "warmup": warmup, "ms": round(sec * 1e3, 4),
            "gb_s": round(nbytes / sec / 1e9, 1), "hbm_frac": round(nbytes / sec / 1e9 / hbm, 4)}


def sweep4_record(K: int, warmup: int) -> dict:
    """The 4-D 9-point star (stencils/mpi9pt.py) on 64^4 points, 4^4 bricks with one ghost brick
    per side, in and out interleaved in one storage (weak/main-4d.cpp's layout), FP64 and FP32
    storage: CUDA events around K launches after `warmup`, on the current stream."""
    import torch
    from bricklib_gb300 import _abi, bricks as B, bricks4 as B4
    from bricklib_gb300._abi import call
    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream
    hbm, _ = peaks()
    n4 = 64
    gb4 = n4 // 4 + 2
    grid4, adj4 = B4.init_grid([gb4] * 4)
    adj_dev = B.DeviceBuffer(adj4.nbytes)
    adj_dev.upload(np.ascontiguousarray(adj4))
    g4 = grid4.reshape((gb4,) * 4)
    inner = B.BrickList(np.ascontiguousarray(g4[1:-1, 1:-1, 1:-1, 1:-1].reshape(-1)))
    st4 = B4.mpi9pt()
    rec = {"points": n4 ** 4, "bricks": int(len(grid4)), "steps": K, "warmup": warmup}
    for name, dt in (("f64", _abi.BK_F64), ("f32", _abi.BK_F32)):
        s4 = B.BrickStorage.allocate_device(len(grid4), 512, dt)
        call("bk_fill_uniform", C.c_void_p(s4.ptr), len(grid4) * 512, dt, 5, -1.0, 1.0, sp)
        for _ in range(warmup):
            B4.sweep4(adj_dev, len(grid4), s4, 0, 256, inner, st4, stream=sp)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(K):
            B4.sweep4(adj_dev, len(grid4), s4, 0, 256, inner, st4, stream=sp)
        e1.record(stream)
        torch.cuda.synchronize()
        sec = e0.elapsed_time(e1) / K * 1e-3
        nbytes = 2 * B.ELEM_SIZE[dt] * n4 ** 4
        rec[name] = {"ms": round(sec * 1e3, 4), "gstencil_s": round(n4 ** 4 / sec / 1e9, 2),
                     "gb_s": round(nbytes / sec / 1e9, 1), "hbm_frac": round(nbytes / sec / 1e9 / hbm, 4)}
        del s4
    if B.error_flags() != 0:
        raise RuntimeError("4-D sweep raised device error flags")
    return rec


def run_next(args):
    """The rows beside the sweep, each timed on the device against the measured copy bandwidth:
    device copyToBrick / copyFromBrick and a plain array copy (what stencils/copy.cpp times,
    at 512^3 + 8 ghost + 8 padding, FP64), the periodic ghost fill of that domain, the periodic
    exchange of a BrickDecomp of it, and the 4-D 9-point sweep (mpi9pt) on 64^4 bricks of 4^4."""
    import torch
    from bricklib_gb300 import _abi, bricks as B, bricks4 as B4, decomp as D
    from bricklib_gb300._abi import call
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    call("bk_set_device", local)
    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream
    hbm, peak_kind = peaks()
    K = max(3, args.steps)

    def timed(fn):
        for _ in range(args.warmup):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(K):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / K * 1e-3

    def rate(nbytes, sec):
        return {"ms": round(sec * 1e3, 4), "gb_s": round(nbytes / sec / 1e9, 1), "hbm_frac": round(nbytes / sec / 1e9 / hbm, 4),
                "bytes": int(nbytes)}

    out = {"form": "next", "peak_hbm_gbs": hbm, "peak_source": f"{peak_kind} hbm_gbs", "steps": K, "warmup": args.warmup}
    n, gz, pad = 512, 8, 8
    g = n + 2 * gz
    adim = g + 2 * pad
    gb = g // 8
    grid, info = B.init_grid([gb, gb, gb])
    nb = info.nbricks
    f64 = _abi.BK_F64
    arr_in = B.DeviceBuffer(adim ** 3 * 8)
    arr_out = B.DeviceBuffer(adim ** 3 * 8)
    call("bk_fill_uniform", C.c_void_p(arr_in.ptr), adim ** 3, f64, 3, -1.0, 1.0, sp)
    grid_dev = B.DeviceBuffer(grid.nbytes)
    grid_dev.upload(np.ascontiguousarray(grid, dtype=np.uint32))
    dinfo = B.movBrickInfo(info)
    st = B.BrickStorage.allocate_device(nb, 512, f64)
    brick = B.Brick(dinfo, st, 0)
    moved = 2 * 8 * g ** 3  # every element of interior + ghost read once and written once
    out["copy_to_bricks"] = rate(moved, timed(lambda: B.copyToBrickDevice([g] * 3, [pad] * 3, [0] * 3, arr_in.ptr,
                                                                          grid_dev.ptr, brick, sp)))
    out["copy_from_bricks"] = rate(moved, timed(lambda: B.copyFromBrickDevice([g] * 3, [pad] * 3, [0] * 3, arr_out.ptr,
                                                                              grid_dev.ptr, brick, sp)))
    out["array_copy"] = rate(2 * 8 * adim ** 3, timed(lambda: B.memcpy(arr_out.ptr, arr_in.ptr, adim ** 3 * 8, 2, sp)))
    # the round trip is exact
    back = np.empty(adim ** 3, np.float64)
    ref = np.empty(adim ** 3, np.float64)
    B.memcpy(back.ctypes.data, arr_out.ptr, back.nbytes, 1, sp)
    B.memcpy(ref.ctypes.data, arr_in.ptr, ref.nbytes, 1, sp)
    B.synchronize(sp)
    sl = (slice(pad, pad + g),) * 3
    out["copy_round_trip_exact"] = bool(np.array_equal(back.reshape((adim,) * 3)[sl], ref.reshape((adim,) * 3)[sl]))
    del arr_in, arr_out, back, ref
    # periodic ghost fill of the 512^3 + one-brick ghost domain
    plan = B.GhostPlan.periodic(grid, (n // 8,) * 3, (1, 1, 1))
    out["ghost_fill"] = rate(2 * plan.n * 512 * 8, timed(lambda: B.ghostFill(plan, brick, sp)))
    out["ghost_fill"]["ghost_bricks"] = plan.n
    del st, brick, dinfo, plan
    # BrickDecomp of the same domain (skin3d_good), its periodic exchange
    dec = D.BrickDecomp([n] * 3, gz, (8, 8, 8), numfield=1)
    dec.initialize(D.SKIN3D_GOOD)
    dst = B.BrickStorage.allocate_device(dec.nbricks, 512, f64)
    links = dec.exchange_links(dst.ptr, 512 * 8)
    out["decomp_exchange"] = rate(2 * int(links[:, 2].sum()), timed(lambda: dec.exchange(dst, sp)))
    out["decomp_exchange"]["regions"] = dec.nregions
    dec.close()
    del dst
    out["sweep4_mpi9pt"] = sweep4_record(K, args.warmup)
    assert B.error_flags() == 0
    if rank == 0:
        print(json.dumps(out), flush=True)


if __name__ == "__main__":
    a = parse()
    if a.impl == "reference":
        run_reference(a)
    elif a.form == "precision":
        run_precision(a)
    elif a.form == "batched":
        run_batched(a)
    elif a.form == "serving":
        run_serving(a)
    elif a.form == "next":
        run_next(a)
    else:
        run_ours(a)
