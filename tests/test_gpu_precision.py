"""Precision form on the GPU: conversion, FP64 norms and the sines field against numpy /
the oracle, the FP64 multi-step run against the CPU oracle, and error bounds of the FP32 /
BF16 / float-float runs."""
import numpy as np
import pytest

from bricklib_gb300 import bricks as B, precision, stencils
from bricklib_gb300._abi import BK_BF16, BK_F32, BK_F64
from bricklib_gb300.domain import GridDomain
from oracle import oracle

pytestmark = pytest.mark.gpu


def test_convert_and_norms_match_numpy():
    dom = GridDomain(16)
    arr = stencils.uniform(3, int(np.prod(dom.adims))).reshape(dom.adims) * 1e3
    dom.set_field(0, arr)
    dom.upload()
    allb = B.BrickList(dom.grid)
    f32 = B.BrickStorage.allocate_device(dom.nbricks, dom.bsize, BK_F32)
    b16 = B.BrickStorage.allocate_device(dom.nbricks, dom.bsize, BK_BF16)
    B.convertField(dom.brick(0), B.Brick(dom.dev_info, f32, 0), allb)
    B.convertField(dom.brick(0), B.Brick(dom.dev_info, b16, 0), allb)
    h32 = B.movBrickStorage(f32, to_device=False).host
    h16 = B.movBrickStorage(b16, to_device=False).host
    src = dom.storage.host.reshape(dom.nbricks, dom.step)[:, :dom.bsize].reshape(-1)
    np.testing.assert_array_equal(h32, src.astype(np.float32))
    back = B.bf16_to_f32(h16).astype(np.float64)
    assert np.all(np.abs(back - src) <= np.abs(src) * 2.0 ** -8)
    nrm = B.fieldNorms(B.Brick(dom.dev_info, f32, 0), dom.brick(0), dom.dev_interior)
    lst = dom.interior
    s64 = src.reshape(dom.nbricks, dom.bsize)[lst].reshape(-1)
    d = h32.reshape(dom.nbricks, dom.bsize)[lst].reshape(-1).astype(np.float64) - s64
    assert nrm["max_abs"] == np.abs(d).max()
    assert abs(nrm["sum_sq"] - np.sum(d * d)) <= 1e-12 * np.sum(d * d)
    assert nrm["max_ref"] == np.abs(s64).max()
    assert abs(nrm["sum_sq_ref"] - np.sum(s64 * s64)) <= 1e-12 * np.sum(s64 * s64)


def test_sines_field_matches_oracle():
    n = 32
    p = precision.PeriodicProblem(n, BK_F64)
    B.fillSines(p.field(0), p.gdims, (1, 1, 1), 8, 77, 1e-3)
    host = B.movBrickStorage(p.storage, to_device=False).host
    # oracle field on the padded array, copied into bricks the same way
    dom = oracle.Domain(n)
    o = dom.ghost + dom.pad
    arr = oracle.fill_sines(dom.adims, (o,) * 3, (n,) * 3, 8, 77, 1e-3)
    dat = dom.alloc()
    dom.to_bricks(arr, dat, 0)
    got = host.reshape(dom.nbricks, dom.step)[:, :dom.bsize]
    want = dat.reshape(dom.nbricks, dom.step)[:, :dom.bsize]
    assert np.abs(got - want).max() < 1e-5  # FP32 sines on the device, FP64 in the oracle


def test_fp64_run_matches_oracle_multistep():
    n, steps = 32, 10
    rec = precision.run_study(n=n, shapes=("heat7",), variants=("f32",), steps=(steps,), timing=False)
    # independent FP64 device run vs the CPU oracle's array path from the same initial field
    p = precision.PeriodicProblem(n, BK_F64)
    B.fillSines(p.field(0), p.gdims, (1, 1, 1), 8, 20261203, 1e-3)
    host0 = B.movBrickStorage(p.storage, to_device=False).host.copy()
    st = stencils.make("heat7")
    B.timeSteps(p.field(0), p.field(1), p.interior, st, steps, plan=p.plan)
    B.synchronize()
    host = B.movBrickStorage(p.storage, to_device=False).host
    dom = oracle.Domain(n)
    o = dom.ghost + dom.pad
    a = dom.from_bricks(host0, 0)
    b = np.zeros_like(a)
    for _ in range(steps):
        oracle.array_periodic_fill(a, (o,) * 3, (n,) * 3, (8, 8, 8))
        oracle.array_sweep(a, b, (o,) * 3, (o + n,) * 3, st.offsets(), st.coeff)
        a, b = b, a
    got = dom.interior_view(dom.from_bricks(host, 0))
    want = dom.interior_view(a)
    assert np.abs(got - want).max() <= 1e-12 * np.abs(want).max()
    assert rec[0]["max_rel_err"] < 1e-5


def test_precision_error_bounds():
    recs = precision.run_study(n=32, shapes=("heat7", "cube125"), variants=("f32", "bf16", "f64-floatfloat"),
                               steps=(1, 10), timing=False)
    for r in recs:
        # BF16 keeps 8 significant bits per stored value; each step re-rounds the field, so
        # the error relative to a decaying field grows with the step count (stated, not a spec)
        bound = {"f32": 1e-5, "bf16": 5e-2, "f64-floatfloat": 1e-12}[r["variant"]]
        assert r["max_rel_err"] <= bound, r
        assert r["rms_rel_err"] <= r["max_rel_err"] + 1e-300
