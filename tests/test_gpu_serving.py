"""Serving form: continuous batching.  Each job's result is the same alone and in the mix
(bit for bit), an FP64 job matches the CPU oracle, the budget gates admission, and waits
are bounded."""
import numpy as np
import pytest

from bricklib_gb300 import _abi, bricks as B, serving, stencils
from bricklib_gb300._abi import BK_ACC_NATIVE, BK_F32, BK_F64
from oracle import oracle

pytestmark = pytest.mark.gpu


def small_jobs():
    return serving.make_jobs(14, seed=3, lo=8, hi=32, max_steps=12)


def run(jobs, budget=150e9, max_active=64, stagger=False):
    arena, ins, outs = serving.job_arrays(jobs)
    srv = serving.Server(budget, max_active=max_active)
    sts = {s: B.to_c_stencil(stencils.make(s, 5)) for s in stencils.PLAIN_SHAPES}
    ids = []
    for q, (j, a, o) in enumerate(zip(jobs, ins, outs)):
        ids.append(srv.submit(j.n, sts[j.shape], j.steps, j.dtype, BK_ACC_NATIVE, a, o))
        if stagger and q % 3 == 2:
            srv.wait(ids[-1], 60.0)  # later jobs join while earlier ones are running
    for i in ids:
        srv.wait(i, 120.0)
    st = srv.stats()
    srv.close()
    return [o.copy() for o in outs], st, arena


def test_each_result_same_alone_and_in_the_mix():
    jobs = small_jobs()
    assert {j.dtype for j in jobs} == {BK_F64, BK_F32}
    mix, st, _ = run(jobs, stagger=True)
    assert st["completed"] == len(jobs) and st["rejected"] == 0
    for q, j in enumerate(jobs):
        alone, _, _ = run([j])
        np.testing.assert_array_equal(alone[0], mix[q], err_msg=f"job {q}")


def test_fp64_job_matches_oracle():
    j = serving.JobSpec((16, 24, 32), "star13", 7, BK_F64, 99)
    out, st, _ = run([j])
    n = j.n
    dom = oracle.Domain(n)
    o = dom.ghost + dom.pad
    a = np.zeros(dom.adims)
    a[o:o + n[0], o:o + n[1], o:o + n[2]] = stencils.uniform(j.seed, j.points).reshape(n)
    b = np.zeros_like(a)
    stn = stencils.make("star13", 5)
    for _ in range(j.steps):
        oracle.array_periodic_fill(a, (o,) * 3, n, (8, 8, 8))
        oracle.array_sweep(a, b, (o,) * 3, tuple(o + x for x in n), stn.offsets(), stn.coeff)
        a, b = b, a
    want = a[o:o + n[0], o:o + n[1], o:o + n[2]]
    assert np.abs(out[0] - want).max() <= 1e-12 * np.abs(want).max()


def oracle_periodic_steps(j, st, inp):
    """The oracle's array path with periodic fill, FP64, from the job's (rounded) input."""
    n = j.n
    dom = oracle.Domain(n)
    o = dom.ghost + dom.pad
    a = np.zeros(dom.adims)
    a[o:o + n[0], o:o + n[1], o:o + n[2]] = inp
    b = np.zeros_like(a)
    for _ in range(j.steps):
        oracle.array_periodic_fill(a, (o,) * 3, n, (8, 8, 8))
        oracle.array_sweep(a, b, (o,) * 3, tuple(o + x for x in n), st.offsets(), st.coeff)
        a, b = b, a
    return a[o:o + n[0], o:o + n[1], o:o + n[2]]


def test_fp32_jobs_in_a_mix_match_the_fp64_oracle():
    """Served FP32 jobs (FP32 storage, FP32 arithmetic), one of each shape, submitted together with
    FP64 jobs: each result is within 1e-5 normwise (max |d| / max |ref|) of the FP64 oracle run from
    the same FP32-rounded input, and every FP64 job within 1e-12."""
    jobs = [serving.JobSpec((24, 16, 32), "star7", 12, BK_F32, 201),
            serving.JobSpec((16, 32, 24), "star13", 9, BK_F32, 202),
            serving.JobSpec((32, 24, 16), "star25", 6, BK_F32, 203),
            serving.JobSpec((24, 24, 24), "cube27", 8, BK_F32, 204),
            serving.JobSpec((16, 24, 32), "cube125", 5, BK_F32, 205),
            serving.JobSpec((24, 16, 16), "cube125", 4, BK_F64, 206),
            serving.JobSpec((16, 16, 24), "star25", 3, BK_F64, 207)]
    out, st, _ = run(jobs)
    assert st["completed"] == len(jobs)
    for j, got in zip(jobs, out):
        inp = stencils.uniform(j.seed, j.points).reshape(j.n)
        if j.dtype == BK_F32:
            inp = inp.astype(np.float32).astype(np.float64)
        want = oracle_periodic_steps(j, stencils.make(j.shape, 5), inp)
        err = float(np.abs(got.astype(np.float64) - want).max() / np.abs(want).max())
        assert err <= (1e-5 if j.dtype == BK_F32 else 1e-12), (j, err)


def test_budget_gates_admission_and_rejects_oversized_jobs():
    jobs = small_jobs()
    one = max(j.points for j in jobs) * 8 * 6  # room for about one job at a time
    out_tight, st, _ = run(jobs, budget=one * 2, max_active=64)
    assert st["completed"] == len(jobs)
    assert st["hbm_peak"] <= one * 2
    out_free, _, _ = run(jobs)
    for x, y in zip(out_tight, out_free):
        np.testing.assert_array_equal(x, y)
    srv = serving.Server(1e6)
    big = serving.JobSpec((64, 64, 64), "star7", 1, BK_F64, 1)
    _, ins, outs = serving.job_arrays([big])
    with pytest.raises(_abi.BkError) as e:
        srv.submit(big.n, stencils.make("star7", 1), 1, BK_F64, BK_ACC_NATIVE, ins[0], outs[0])
    assert e.value.status == _abi.BK_ERR_BUDGET
    srv.close()


def test_wait_is_bounded():
    j = serving.JobSpec((96, 96, 96), "cube125", 200, BK_F64, 5)
    _, ins, outs = serving.job_arrays([j])
    srv = serving.Server()
    jid = srv.submit(j.n, stencils.make("cube125", 5), j.steps, j.dtype, BK_ACC_NATIVE, ins[0], outs[0])
    with pytest.raises(_abi.BkError) as e:
        srv.wait(jid, 0.001)
    assert e.value.status == _abi.BK_ERR_TIMEOUT
    srv.wait(jid, 300.0)
    srv.close()
