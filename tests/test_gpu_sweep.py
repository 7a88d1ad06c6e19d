"""Parity of the CUDA sweep, ghost fill and time stepping with the oracle and the
golden vectors of bricklib's own CPU brick path.  All calls go through the C ABI.

Tolerances: FP64 uses compareBrick's mixed test (brickcompare.h:37) with tol 1e-12;
FP32 / BF16 storage are held to a normwise bound max|d| / max|ref| against the FP64
oracle (1e-5 for FP32, 2^-7 for BF16, whose inputs and outputs are rounded to 8 bits).
"""
import glob
import os

import numpy as np
import pytest

from bricklib_gb300 import _abi, bricks as B, stencils
from bricklib_gb300._abi import BK_ACC_COMPENSATED, BK_ACC_NATIVE, BK_BF16, BK_F32, BK_F64
from bricklib_gb300.domain import GridDomain
from oracle import oracle

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), "golden")
TOL64 = 1e-12


@pytest.fixture(params=["default", "pipelined", "oneshot"])
def kernel(request, monkeypatch):
    """With no override, star stencils on row-major 8x8x8 bricks run the TMA-fed kernel;
    BK_SWEEP_PIPELINED=1 forces the cp.async pipelined kernel (also where the one-shot
    kernel is preferred); BK_SWEEP_ONESHOT=1 selects the one-shot kernel that also serves
    every other layout.  All must pass."""
    monkeypatch.delenv("BK_SWEEP_ONESHOT", raising=False)
    monkeypatch.delenv("BK_SWEEP_PIPELINED", raising=False)
    if request.param == "oneshot":
        monkeypatch.setenv("BK_SWEEP_ONESHOT", "1")
    elif request.param == "pipelined":
        monkeypatch.setenv("BK_SWEEP_PIPELINED", "1")
    return request.param


def mixed_ok(a, b, tol=TOL64):
    d = np.abs(a - b)
    return bool(np.all((d < tol) | (d < (np.abs(a) + np.abs(b)) * tol))), float(d.max(initial=0))


def normwise(a, ref):
    return float(np.abs(a - ref).max() / max(np.abs(ref).max(), 1e-300))


def device_sweep(n, st, dtype=BK_F64, layout=B.DEFAULT_LAYOUT, acc=BK_ACC_NATIVE, seed=1234, arr=None):
    dom = GridDomain(n, layout=layout, dtype=dtype)
    if arr is None:
        arr = stencils.uniform(seed, int(np.prod(dom.adims))).reshape(dom.adims)
    dom.set_field(0, arr)
    dom.upload()
    B.brickSweep(dom.brick(0), dom.brick(1), dom.dev_interior, st, acc)
    B.synchronize()
    assert B.error_flags() == 0
    dom.download()
    return dom, arr, dom.interior_view(dom.get_field(1))


def oracle_array(dom, arr, st):
    out = np.zeros_like(arr, dtype=np.float64)
    o, n = dom.org, dom.n
    oracle.array_sweep(np.ascontiguousarray(arr, dtype=np.float64), out, o,
                       (o[0] + n[0], o[1] + n[1], o[2] + n[2]), st.offsets(), st.coeff)
    return dom.interior_view(out)


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLD, "sweep_*.npz"))),
                         ids=lambda p: os.path.basename(p)[6:-4])
def test_fp64_matches_reference_golden(path):
    z = np.load(path)
    st = stencils.custom("golden", [tuple(t) for t in z["offsets"]], z["coeff"])
    st.pre_op = int(z["pre_op"]) if "pre_op" in z else 0
    st.post_op = int(z["post_op"]) if "post_op" in z else 0
    lay = B.Layout((8, 8, 8), (1, 4, 8)) if int(z["layout"]) == 0 else B.Layout((4, 4, 4), (1, 4, 4))
    _, _, got = device_sweep(int(z["n"]), st, layout=lay, seed=int(z["seed_in"]))
    ok, md = mixed_ok(got, z["out"])
    assert ok, f"max |diff| {md}"


@pytest.mark.parametrize("name", stencils.PLAIN_SHAPES + ("heat7", "lap7"))
def test_fp64_matches_oracle_64(name, kernel):
    st = stencils.make(name, 7)
    dom, arr, got = device_sweep(64, st, seed=42)
    ok, md = mixed_ok(got, oracle_array(dom, arr, st))
    assert ok, f"{name}: max |diff| {md}"


def test_c1_laplacian_128():
    """The reference's CPU-runnable case: 7-point Laplacian (centre -6/h^2, axes 1/h^2, h = 1/128),
    FP64, 128^3 interior + 8-cell ghost, uniform[-1,1) input, one sweep, checked against the array
    kernel with compareBrick's mixed test."""
    st = stencils.make("lap7")
    dom, arr, got = device_sweep(128, st, seed=20261204)
    ok, md = mixed_ok(got, oracle_array(dom, arr, st))
    assert ok, f"max |diff| {md}"


LAYOUTS = [((8, 8, 8), (1, 1, 8)), ((8, 8, 8), (1, 2, 2)), ((8, 8, 8), (2, 4, 4)), ((4, 4, 4), (1, 4, 4)),
           ((16, 8, 8), (1, 4, 8)), ((8, 8, 32), (1, 1, 32)), ((8, 8, 32), (1, 4, 8))]


@pytest.mark.parametrize("bdim,fold", LAYOUTS, ids=lambda x: "x".join(map(str, x)))
@pytest.mark.parametrize("name", ["star7", "star13", "cube27", "cube125"])
def test_fp64_layouts(bdim, fold, name, kernel):
    st = stencils.make(name, 3)
    if st.radius > min(bdim):
        pytest.skip("radius beyond the brick")
    n = (32, 32, 64) if bdim[2] == 32 else (32, 32, 32)
    dom, arr, got = device_sweep(n, st, layout=B.Layout(bdim, fold), seed=9,
                                 arr=None)
    ok, md = mixed_ok(got, oracle_array(dom, arr, st))
    assert ok, f"max |diff| {md}"


def test_generic_family_19pt(kernel):
    taps = [t for t in stencils.cube_taps(1)[0] if sum(1 for a in t if a) <= 2]
    st = stencils.custom("d3pt19", taps, stencils.uniform(5, len(taps), 0, 1))
    assert B.stencil_family(st)[1] == 0
    dom, arr, got = device_sweep(32, st, seed=3)
    ok, md = mixed_ok(got, oracle_array(dom, arr, st))
    assert ok, f"max |diff| {md}"


@pytest.mark.parametrize("name", stencils.PLAIN_SHAPES)
@pytest.mark.parametrize("acc", [BK_ACC_NATIVE, BK_ACC_COMPENSATED])
def test_fp32_against_fp64_oracle(name, acc, kernel):
    st = stencils.make(name, 11)
    dom, arr, got = device_sweep(64, st, dtype=BK_F32, acc=acc, seed=5)
    ref = oracle_array(dom, arr.astype(np.float32).astype(np.float64), st)
    assert normwise(got, ref) <= 1e-5


def test_compensated_beats_native_on_cube125():
    st = stencils.make("cube125", 2)
    dom, arr, nat = device_sweep(64, st, dtype=BK_F32, acc=BK_ACC_NATIVE, seed=8)
    _, _, comp = device_sweep(64, st, dtype=BK_F32, acc=BK_ACC_COMPENSATED, arr=arr)
    ref = oracle_array(dom, arr.astype(np.float32).astype(np.float64), st)
    # the FP32 output rounding (2^-24 relative) bounds both; compensation removes most of the rest
    assert np.sqrt(np.mean((comp - ref) ** 2)) <= np.sqrt(np.mean((nat - ref) ** 2)) * 1.01


@pytest.mark.parametrize("name", ["star7", "cube125"])
def test_bf16_against_fp64_oracle(name, kernel):
    st = stencils.make(name, 4)
    dom, arr, got = device_sweep(32, st, dtype=BK_BF16, acc=BK_ACC_COMPENSATED, seed=6)
    arr_b = B.bf16_to_f32(B.f32_to_bf16(arr.astype(np.float32))).astype(np.float64)
    ref = oracle_array(dom, arr_b, st)
    assert normwise(got, ref) <= 2.0 ** -7


def test_interleaved_equals_separate_storages():
    st = stencils.make("star13", 1)
    dom, arr, inter = device_sweep(32, st, seed=2)
    # separate storages: in and out each in their own BrickStorage
    d1 = GridDomain(32, nfields=1)
    d1.set_field(0, arr)
    d1.upload()
    out_st = B.BrickStorage.allocate_device(d1.nbricks, d1.step)
    B.brickSweep(d1.brick(0), B.Brick(d1.dev_info, out_st, 0), d1.dev_interior, st)
    host = B.movBrickStorage(out_st, to_device=False)
    d1.storage.host[:] = host.host
    np.testing.assert_array_equal(d1.interior_view(d1.get_field(0)), inter)


def test_ghost_fill_matches_oracle_plan():
    dom = GridDomain(32)
    arr = stencils.uniform(17, int(np.prod(dom.adims))).reshape(dom.adims)
    dom.set_field(0, arr)
    dom.upload()
    plan = dom.periodic_plan()
    B.ghostFill(plan, dom.brick(0))
    B.synchronize()
    dom.download()
    want = oracle.Domain(32)
    dat = want.alloc()
    want.to_bricks(arr, dat, 0)
    oracle.apply_plan(dat, want.step, 0, want.bsize, plan.host)
    np.testing.assert_array_equal(dom.storage.host, dat)


@pytest.mark.parametrize("use_graph", [False, True])
def test_time_steps_with_periodic_fill(use_graph):
    n, steps = 32, 10
    st = stencils.make("heat7")
    dom = GridDomain(n)
    o = dom.org[0]
    arr = oracle.fill_sines(dom.adims, (o,) * 3, (n,) * 3, 8, 123, 1e-3)
    dom.set_field(0, arr)
    dom.upload()
    newest = B.timeSteps(dom.brick(0), dom.brick(1), dom.dev_interior, st, steps, plan=dom.periodic_plan(),
                         fill_every=1, use_graph=use_graph)
    B.synchronize()
    dom.download()
    assert newest.offset == (0 if steps % 2 == 0 else dom.bsize)
    got = dom.interior_view(dom.get_field(0 if steps % 2 == 0 else 1))
    a, b = arr.copy(), np.zeros_like(arr)
    for _ in range(steps):
        oracle.array_periodic_fill(a, (o,) * 3, (n,) * 3, (8, 8, 8))
        oracle.array_sweep(a, b, (o,) * 3, (o + n,) * 3, st.offsets(), st.coeff)
        a, b = b, a
    ok, md = mixed_ok(got, dom.interior_view(a))
    assert ok, f"max |diff| {md}"


def test_graph_and_plain_steps_bitwise_equal():
    res = []
    for g in (False, True):
        dom = GridDomain(32, dtype=BK_F32)
        arr = stencils.uniform(77, int(np.prod(dom.adims))).reshape(dom.adims)
        dom.set_field(0, arr)
        dom.upload()
        B.timeSteps(dom.brick(0), dom.brick(1), dom.dev_interior, stencils.make("cube27", 1), 7,
                    plan=dom.periodic_plan(), use_graph=g)
        B.synchronize()
        dom.download()
        res.append(dom.storage.host.copy())
    np.testing.assert_array_equal(res[0], res[1])


def test_out_of_range_adjacency_is_clamped_and_flagged():
    dom = GridDomain(16, device=False)
    bad = dom.bInfo.adj.copy()
    victim = dom.interior[0]
    bad[victim, 14] = dom.nbricks + 1000  # neighbour (0,0,+1) points past the storage
    dom.bInfo = B.BrickInfo(dom.nbricks, bad)
    arr = stencils.uniform(1, int(np.prod(dom.adims))).reshape(dom.adims)
    dom.set_field(0, arr)
    dom.to_device()
    B.error_flags()  # clear
    B.brickSweep(dom.brick(0), dom.brick(1), dom.dev_interior, stencils.make("star7", 1))
    B.synchronize()
    assert B.error_flags() & 1
    # a list entry past nbricks is skipped and flagged as well
    lst = B.BrickList(np.array([dom.nbricks + 5, dom.interior[1]], dtype=np.uint32))
    B.brickSweep(dom.brick(0), dom.brick(1), lst, stencils.make("star7", 1))
    B.synchronize()
    assert B.error_flags() & 1
    assert B.error_flags() == 0  # reading clears


def _mirror_symmetric_cube(r, seed, ij=False, kj=False):
    """A (2r+1)^3 cube whose coefficient depends on (|dk|, |dj|, |di|) only; with `ij` also
    symmetric under the swap of |dj| and |di|, with `kj` under the swap of |dk| and |dj|."""
    taps, _ = stencils.cube_taps(r)
    per = stencils.uniform01(seed, (r + 1) ** 3).reshape(r + 1, r + 1, r + 1)
    if ij:
        per = per + per.transpose(0, 2, 1)
    if kj:
        per = per + per.transpose(1, 0, 2)
    c = np.array([per[abs(t[0]), abs(t[1]), abs(t[2])] for t in taps])
    return stencils.custom(f"symcube{2 * r + 1}", taps, c / c.sum())


@pytest.mark.parametrize("ij", [False, True])
@pytest.mark.parametrize("r", [1, 2])
@pytest.mark.parametrize("dtype", [BK_F64, BK_F32, BK_BF16])
def test_mirror_symmetric_cubes_against_oracle(r, dtype, ij, kernel):
    """Mirror-symmetric cubes take the pair-sum paths of the pipelined kernel (fewer
    multiply-adds); the result still meets the FP64 / FP32 / BF16 bounds against the oracle."""
    st = _mirror_symmetric_cube(r, 40 + r, ij)
    dom, arr, got = device_sweep(32, st, dtype=dtype, seed=17)
    if dtype == BK_F64:
        ok, md = mixed_ok(got, oracle_array(dom, arr, st))
        assert ok, f"max |diff| {md}"
    elif dtype == BK_F32:
        assert normwise(got, oracle_array(dom, arr.astype(np.float32).astype(np.float64), st)) <= 1e-5
    else:
        arr_b = B.bf16_to_f32(B.f32_to_bf16(arr.astype(np.float32))).astype(np.float64)
        assert normwise(got, oracle_array(dom, arr_b, st)) <= 2.0 ** -7


def _sweep_with(env, monkeypatch, dom, st, acc, lst):
    monkeypatch.delenv("BK_SWEEP_ONESHOT", raising=False)
    monkeypatch.delenv("BK_SWEEP_PIPELINED", raising=False)
    if env:
        monkeypatch.setenv(env, "1")
    # output field = all-ones bytes (NaN in every storage type) before each run
    raw = dom.storage.host.view(np.uint8).reshape(dom.nbricks, dom.nfields, -1)
    raw[:, 1, :] = 0xFF
    dom.upload()
    B.brickSweep(dom.brick(0), dom.brick(1), lst, st, acc)
    B.synchronize()
    assert B.error_flags() == 0
    dom.download()
    return dom.storage.host.copy()


@pytest.mark.parametrize("dtype,acc", [(BK_F64, BK_ACC_NATIVE), (BK_F64, _abi.BK_ACC_FLOATFLOAT),
                                       (BK_F32, BK_ACC_NATIVE), (BK_F32, BK_ACC_COMPENSATED),
                                       (BK_BF16, BK_ACC_NATIVE), (BK_BF16, BK_ACC_COMPENSATED)])
@pytest.mark.parametrize("name", ["star7", "star13", "star25"])
def test_tma_star_kernel_equals_pipelined(dtype, acc, name, monkeypatch):
    """The TMA-fed star kernel sums in the pipelined kernel's order: bit-identical outputs.
    The domain has enough brick groups for every CTA to cycle through its pipeline stages
    several times; the second list is odd-length and shorter than one group per CTA."""
    st = stencils.make(name, 13)
    dom = GridDomain((128, 256, 256), dtype=dtype)  # 16,384 bricks: 8,192 groups of two
    arr = stencils.uniform(31, int(np.prod(dom.adims))).reshape(dom.adims)
    dom.set_field(0, arr)
    dom.upload()
    short = B.BrickList(np.asarray(dom.interior[:77][::-1], dtype=np.uint32))
    for lst, nout in ((dom.dev_interior, len(dom.interior)), (short, 77)):
        got = [_sweep_with(env, monkeypatch, dom, st, acc, lst) for env in (None, "BK_SWEEP_PIPELINED")]
        np.testing.assert_array_equal(got[0].view(np.uint8), got[1].view(np.uint8))
        written = got[0].view(np.uint8).reshape(dom.nbricks, dom.nfields, -1)[:, 1, :]
        assert int(np.count_nonzero((written != 0xFF).any(axis=1))) == nout


@pytest.mark.parametrize("name", ["star7", "star13", "star25"])
def test_fp64_register_operand_stars_equal_the_plain_operations(name, monkeypatch):
    """The native FP64 star kernels that run on register operands (the first product as
    fma(c, x, -0), coefficients in registers, taps outer over a column: the TMA-fed kernel and
    the pipelined one) give the bits of the one-shot kernel, which multiplies and adds with
    the coefficients as constant operands, point by point in the same order."""
    st = stencils.make(name, 29)
    dom = GridDomain((64, 64, 128), dtype=BK_F64)
    arr = stencils.uniform(37, int(np.prod(dom.adims))).reshape(dom.adims)
    # interior runs of signed zeros and of values whose products underflow exercise the -0 addend
    o = dom.org
    arr[o[0] + 3, o[1] + 5:o[1] + 9, o[2]:o[2] + 40] = -0.0
    arr[o[0] + 9, o[1] + 2:o[1] + 6, o[2] + 8:o[2] + 48] = 1e-310
    dom.set_field(0, arr)
    dom.upload()
    plain = _sweep_with("BK_SWEEP_ONESHOT", monkeypatch, dom, st, BK_ACC_NATIVE, dom.dev_interior)
    for env in (None, "BK_SWEEP_PIPELINED"):
        got = _sweep_with(env, monkeypatch, dom, st, BK_ACC_NATIVE, dom.dev_interior)
        np.testing.assert_array_equal(got.view(np.uint8), plain.view(np.uint8), err_msg=str(env))


def _row_lists(dom, seed):
    """Brick lists for the row-run kernel: grid order (full runs), a shuffle (runs of one),
    grid-order pieces of 1..9 bricks in shuffled order (runs cut at every alignment),
    repeated entries, and an odd-length tail."""
    rng = np.random.default_rng(seed)
    it = np.asarray(dom.interior, dtype=np.uint32)
    cuts = np.cumsum(rng.integers(1, 10, size=len(it)))
    pieces = np.split(it, cuts[cuts < len(it)])
    order = rng.permutation(len(pieces))
    lists = {
        "grid": it,
        "shuffled": rng.permutation(it),
        "pieces": np.concatenate([pieces[k] for k in order]),
        "repeats": np.repeat(it[:300], rng.integers(1, 3, size=300)),
        "tail": it[5:5 + 4 * 37 + 3],
    }
    return {k: np.ascontiguousarray(v, dtype=np.uint32) for k, v in lists.items()}


@pytest.mark.parametrize("dtype,acc", [(BK_F32, BK_ACC_NATIVE), (BK_F32, BK_ACC_COMPENSATED),
                                       (BK_BF16, BK_ACC_NATIVE), (BK_BF16, BK_ACC_COMPENSATED)])
@pytest.mark.parametrize("name", ["star7", "star13", "star25"])
def test_row_kernel_equals_per_brick_staging(dtype, acc, name, monkeypatch):
    """The row-run TMA kernel (runs of i-adjacent list entries share their whole-brick i
    faces) writes exactly what per-brick TMA staging and the pipelined kernel write, for
    lists in grid order, shuffled, in grid-order pieces, with repeats and with a ragged tail;
    full runs over consecutive bricks give the same with grouped and brick-by-brick copies."""
    st = stencils.make(name, 17)
    dom = GridDomain((64, 128, 128), dtype=dtype)  # 4,096 interior bricks
    arr = stencils.uniform(37, int(np.prod(dom.adims))).reshape(dom.adims)
    dom.set_field(0, arr)
    dom.upload()
    monkeypatch.delenv("BK_TMA_ROW", raising=False)
    assert B.sweepKernel(dom.brick(0), dom.brick(1), st, acc) == "sweep_star_row_kernel"
    for key, lst in _row_lists(dom, 3).items():
        dl = B.BrickList(lst)
        row = _sweep_with(None, monkeypatch, dom, st, acc, dl)
        monkeypatch.setenv("BK_TMA_ROW", "0")
        per_brick = _sweep_with(None, monkeypatch, dom, st, acc, dl)
        monkeypatch.delenv("BK_TMA_ROW")
        piped = _sweep_with("BK_SWEEP_PIPELINED", monkeypatch, dom, st, acc, dl)
        np.testing.assert_array_equal(row.view(np.uint8), per_brick.view(np.uint8), err_msg=key)
        np.testing.assert_array_equal(row.view(np.uint8), piped.view(np.uint8), err_msg=key)
        if key == "grid":  # full runs over consecutive bricks: grouped and brick-by-brick copies
            for g in ("0", "1"):
                monkeypatch.setenv("BK_TMA_GROUP", g)
                other = _sweep_with(None, monkeypatch, dom, st, acc, dl)
                monkeypatch.delenv("BK_TMA_GROUP")
                np.testing.assert_array_equal(row.view(np.uint8), other.view(np.uint8), err_msg=f"group {g}")
        written = row.view(np.uint8).reshape(dom.nbricks, dom.nfields, -1)[:, 1, :]
        assert int(np.count_nonzero((written != 0xFF).any(axis=1))) == len(np.unique(lst)), key


@pytest.mark.parametrize("dtype", [BK_F32, BK_BF16])
def test_row_kernel_follows_asymmetric_adjacency(dtype, monkeypatch):
    """Runs need both directions: entry n+1 is entry n's i-hi neighbour AND entry n is entry
    n+1's i-lo neighbour.  With one direction broken (i-lo re-pointed elsewhere, or a brick
    whose i-hi is itself, periodic one brick wide) the row kernel still reads exactly the
    adjacency the per-brick kernels read."""
    st = stencils.make("star13", 5)
    dom = GridDomain((32, 64, 64), dtype=dtype, device=False)
    adj = dom.bInfo.adj.copy()
    rng = np.random.default_rng(9)
    it = dom.interior
    victims = rng.choice(it, size=len(it) // 5, replace=False)
    adj[victims, 12] = rng.choice(it, size=len(victims))          # i-lo elsewhere
    selfies = rng.choice(it, size=len(it) // 7, replace=False)
    adj[selfies, 14] = selfies                                       # i-hi is the brick itself
    adj[selfies[::2], 12] = selfies[::2]                             # ... and i-lo too for half
    dom.bInfo = B.BrickInfo(dom.nbricks, adj)
    arr = stencils.uniform(8, int(np.prod(dom.adims))).reshape(dom.adims)
    dom.set_field(0, arr)
    dom.to_device()
    lst = np.concatenate([it, np.repeat(selfies[:50], 2)]).astype(np.uint32)
    dl = B.BrickList(lst)
    monkeypatch.delenv("BK_TMA_ROW", raising=False)
    row = _sweep_with(None, monkeypatch, dom, st, BK_ACC_NATIVE, dl)
    piped = _sweep_with("BK_SWEEP_PIPELINED", monkeypatch, dom, st, BK_ACC_NATIVE, dl)
    np.testing.assert_array_equal(row.view(np.uint8), piped.view(np.uint8))


def test_row_kernel_bounds_are_flagged(monkeypatch):
    """Out-of-range adjacency and list entries on the row kernel: the bricks that can run
    equal the per-brick kernel's output, and the bounds flag is raised."""
    st = stencils.make("star7", 2)
    dom = GridDomain((32, 32, 64), dtype=BK_F32, device=False)
    adj = dom.bInfo.adj.copy()
    it = dom.interior
    adj[it[3], 14] = dom.nbricks + 7
    adj[it[10], 12] = dom.nbricks + 9
    dom.bInfo = B.BrickInfo(dom.nbricks, adj)
    arr = stencils.uniform(6, int(np.prod(dom.adims))).reshape(dom.adims)
    dom.set_field(0, arr)
    dom.to_device()
    lst = B.BrickList(np.concatenate([it[:20], [dom.nbricks + 3], it[20:]]).astype(np.uint32))
    outs = []
    for row in ("1", "0"):
        monkeypatch.setenv("BK_TMA_ROW", row)
        raw = dom.storage.host.view(np.uint8).reshape(dom.nbricks, dom.nfields, -1)
        raw[:, 1, :] = 0xFF
        dom.upload()
        B.error_flags()
        B.brickSweep(dom.brick(0), dom.brick(1), lst, st)
        B.synchronize()
        assert B.error_flags() & 1
        dom.download()
        outs.append(dom.storage.host.copy())
    np.testing.assert_array_equal(outs[0].view(np.uint8), outs[1].view(np.uint8))


def _istream_stencil(shape):
    if shape == "cube125":
        return stencils.make("cube125", 7)  # symmetric under every axis swap
    r, ij, kj = {"sym27": (1, False, False), "sym27kj": (1, False, True),
                 "sym125": (2, False, False), "sym125ij": (2, True, False)}[shape]
    return _mirror_symmetric_cube(r, 50 + r, ij, kj)


ISTREAM_MODES = [(BK_F64, BK_ACC_NATIVE), (BK_F32, BK_ACC_NATIVE), (BK_F32, BK_ACC_COMPENSATED),
                 (BK_BF16, BK_ACC_NATIVE), (BK_BF16, BK_ACC_COMPENSATED)]


def _istream_close(dtype, got, ref_arr, dom, st):
    """FP64: compareBrick's mixed test at 1e-12 against the oracle; FP32 / BF16: the normwise
    bounds of the other reduced-precision tests."""
    if dtype == BK_F64:
        return mixed_ok(got, ref_arr)
    return normwise(got, ref_arr) <= (1e-5 if dtype == BK_F32 else 2.0 ** -7), normwise(got, ref_arr)


def _rounded_input(dtype, arr):
    if dtype == BK_F32:
        return arr.astype(np.float32).astype(np.float64)
    if dtype == BK_BF16:
        return B.bf16_to_f32(B.f32_to_bf16(arr.astype(np.float32))).astype(np.float64)
    return arr


@pytest.mark.parametrize("dtype,acc", ISTREAM_MODES, ids=lambda x: str(x))
@pytest.mark.parametrize("shape", ["cube125", "sym27", "sym27kj", "sym125", "sym125ij"])
def test_istream_cubes_same_bits_for_every_list_order(shape, dtype, acc, monkeypatch):
    """Mirror-symmetric cubes carry per-column class sums from one brick to the next along runs
    of i-adjacent list entries (FP64; FP32 and BF16 storage in native or compensated FP32).
    Every list order -- grid order (long runs), shuffled (none), grid-order pieces, repeated
    entries, a ragged tail -- writes the same bits into every brick it lists; the result meets
    the storage type's bound against the oracle, and agrees with the one-brick-at-a-time
    kernels (BK_SWEEP_ISTREAM=0)."""
    st = _istream_stencil(shape)
    dom = GridDomain((32, 64, 128), dtype=dtype)  # (k, j, i): 4 x 8 x 16 interior bricks, runs of 16
    arr = stencils.uniform(23, int(np.prod(dom.adims))).reshape(dom.adims)
    dom.set_field(0, arr)
    dom.upload()
    monkeypatch.delenv("BK_SWEEP_ISTREAM", raising=False)
    assert B.sweepKernel(dom.brick(0), dom.brick(1), st, acc) == "sweep2_kernel"
    want = oracle_array(dom, _rounded_input(dtype, arr), st)
    full = None
    for key, lst in _row_lists(dom, 5).items():
        got = _sweep_with(None, monkeypatch, dom, st, acc, B.BrickList(lst))
        out = got.reshape(dom.nbricks, dom.nfields, -1)[:, 1, :]
        if full is None:  # grid order: every interior brick
            full = out.copy()
            ok, md = _istream_close(dtype, dom.interior_view(dom.get_field(1)), want, dom, st)
            assert ok, f"vs oracle: {md}"
        listed = np.unique(lst)
        np.testing.assert_array_equal(out[listed].view(np.uint8), full[listed].view(np.uint8), err_msg=key)
        assert int(np.count_nonzero((out.view(np.uint8) != 0xFF).any(axis=1))) == len(listed)
    monkeypatch.setenv("BK_SWEEP_ISTREAM", "0")
    _sweep_with(None, monkeypatch, dom, st, acc, dom.dev_interior)
    per_brick = dom.interior_view(dom.get_field(1))
    dom.storage.host.reshape(dom.nbricks, dom.nfields, -1)[:, 1, :] = full
    streamed = dom.interior_view(dom.get_field(1))
    if dtype == BK_F64:
        ok, md = mixed_ok(streamed, per_brick)
        assert ok, f"vs one brick at a time: max |diff| {md}"
    else:
        assert normwise(streamed, per_brick) <= (2e-6 if dtype == BK_F32 else 2.0 ** -7)


def test_fp32_istream_compensated_beats_native_and_the_one_column_code(monkeypatch):
    """FP32 125-point cube: the class-sum stream in native FP32 is closer to the FP64 oracle than
    the one-column code, and its compensated form (Dot2 W sums, Neumaier output sum) closer
    still, at least as close as the one-column compensated code (RMS over the interior)."""
    st = stencils.make("cube125", 2)
    dom = GridDomain(64, dtype=BK_F32)
    arr = stencils.uniform(8, int(np.prod(dom.adims))).reshape(dom.adims)
    dom.set_field(0, arr)
    dom.upload()
    ref = oracle_array(dom, arr.astype(np.float32).astype(np.float64), st)

    def rms(env_istream, acc):
        monkeypatch.setenv("BK_SWEEP_ISTREAM", env_istream)
        _sweep_with(None, monkeypatch, dom, st, acc, dom.dev_interior)
        return float(np.sqrt(np.mean((dom.interior_view(dom.get_field(1)) - ref) ** 2)))

    nat_stream, comp_stream = rms("1", BK_ACC_NATIVE), rms("1", BK_ACC_COMPENSATED)
    nat_old, comp_old = rms("0", BK_ACC_NATIVE), rms("0", BK_ACC_COMPENSATED)
    assert nat_stream < nat_old
    assert comp_stream < nat_stream
    assert comp_stream <= comp_old * 1.05


@pytest.mark.parametrize("dtype", [BK_F64, BK_F32])
def test_istream_follows_asymmetric_adjacency(dtype, monkeypatch):
    """A run continues only where the next entry's i-lo and centre columns of neighbours are
    this entry's centre and i-hi columns.  With i-lo, diagonal and i-hi entries re-pointed
    (and bricks whose i neighbours are themselves) the streamed sweep reads exactly the
    adjacency the one-brick-at-a-time kernel reads (FP32: the same bits as the stream restarted
    at every brick, i.e. the class sums of a shuffled list)."""
    st = stencils.make("cube125", 11)
    dom = GridDomain((32, 64, 64), device=False, dtype=dtype)
    adj = dom.bInfo.adj.copy()
    rng = np.random.default_rng(12)
    it = dom.interior
    # slots (dk, dj, di): 12 (0, 0, -1), 3 (-1, 0, -1), 23 (+1, 0, +1), 11 (0, -1, +1), 14 (0, 0, +1)
    for slot, frac in ((12, 5), (3, 6), (23, 6), (11, 7), (14, 9)):
        v = rng.choice(it, size=len(it) // frac, replace=False)
        adj[v, slot] = rng.choice(it, size=len(v))
    selfies = rng.choice(it, size=len(it) // 7, replace=False)
    adj[selfies, 14] = selfies
    adj[selfies[::2], 12] = selfies[::2]
    dom.bInfo = B.BrickInfo(dom.nbricks, adj)
    arr = stencils.uniform(8, int(np.prod(dom.adims))).reshape(dom.adims)
    dom.set_field(0, arr)
    dom.to_device()
    dl = B.BrickList(np.concatenate([it, np.repeat(selfies[:50], 2)]).astype(np.uint32))
    monkeypatch.delenv("BK_SWEEP_ISTREAM", raising=False)
    streamed = _sweep_with(None, monkeypatch, dom, st, BK_ACC_NATIVE, dl)
    a = streamed.reshape(dom.nbricks, dom.nfields, -1)[it, 1, :]
    if dtype == BK_F64:
        monkeypatch.setenv("BK_SWEEP_ISTREAM", "0")
        per_brick = _sweep_with(None, monkeypatch, dom, st, BK_ACC_NATIVE, dl)
        b = per_brick.reshape(dom.nbricks, dom.nfields, -1)[it, 1, :]
        ok, md = mixed_ok(a, b)
        assert ok, f"max |diff| {md}"
    else:
        # entries one at a time, shuffled: no run continues, every brick from its own tile
        lone = B.BrickList(np.random.default_rng(3).permutation(it).astype(np.uint32))
        b = _sweep_with(None, monkeypatch, dom, st, BK_ACC_NATIVE, lone).reshape(dom.nbricks, dom.nfields, -1)
        np.testing.assert_array_equal(a.view(np.uint8), b[it, 1, :].view(np.uint8))


@pytest.mark.parametrize("dtype,name", [(BK_F64, "cube125"), (BK_F64, "star7"), (BK_F32, "cube27"),
                                        (BK_F32, "star7"), (BK_BF16, "star13")])
def test_output_field_off_the_pair_boundary(dtype, name):
    """An output field whose bricks start at odd element offsets (step 2 x 512 + 1, offset 1)
    takes kernels that store one element at a time; the results match the oracle."""
    st = stencils.make(name, 3)
    dom = GridDomain(32, dtype=dtype)
    arr = stencils.uniform(19, int(np.prod(dom.adims))).reshape(dom.adims)
    dom.set_field(0, arr)
    dom.upload()
    ost = B.BrickStorage.allocate_device(dom.nbricks, 2 * dom.bsize + 1, dtype)
    bout = B.Brick(dom.dev_info, ost, 1, dom.layout)
    assert B.sweepKernel(dom.brick(0), bout, st) in ("sweep_kernel", "sweep_star_tma_kernel")
    B.brickSweep(dom.brick(0), bout, dom.dev_interior, st)
    B.synchronize()
    assert B.error_flags() == 0
    host = B.movBrickStorage(ost, to_device=False).host.reshape(dom.nbricks, -1)
    dom.storage.host.reshape(dom.nbricks, dom.nfields, -1)[:, 1, :] = host[:, 1:1 + dom.bsize]
    got = dom.interior_view(dom.get_field(1))
    if dtype == BK_F64:
        ok, md = mixed_ok(got, oracle_array(dom, arr, st))
        assert ok, f"max |diff| {md}"
    elif dtype == BK_F32:
        assert normwise(got, oracle_array(dom, arr.astype(np.float32).astype(np.float64), st)) <= 1e-5
    else:
        arr_b = B.bf16_to_f32(B.f32_to_bf16(arr.astype(np.float32))).astype(np.float64)
        assert normwise(got, oracle_array(dom, arr_b, st)) <= 2.0 ** -7


@pytest.mark.parametrize("name,acc", [("star7", BK_ACC_NATIVE), ("cube27", BK_ACC_NATIVE),
                                      ("cube125", _abi.BK_ACC_FLOATFLOAT)])
def test_output_field_in_mapped_host_memory(name, acc, kernel):
    """An output field in page-locked host memory (bk_host_malloc) receives exactly the
    device sweep's results, written by the kernel over the CPU-GPU link."""
    st = stencils.make(name, 5)
    dom, arr, _ = device_sweep(32, st, acc=acc, seed=4)
    hst = B.BrickStorage.allocate_pinned(dom.nbricks, dom.step)
    hst.host[:] = 0
    B.brickSweep(dom.brick(0), B.Brick(dom.dev_info, hst, dom.bsize), dom.dev_interior, st, acc)
    B.synchronize()
    assert B.error_flags() == 0
    want = dom.storage.host.reshape(dom.nbricks, dom.step)[:, dom.bsize:][dom.interior]
    got = hst.host.reshape(dom.nbricks, dom.step)[:, dom.bsize:][dom.interior]
    np.testing.assert_array_equal(got, want)


def test_empty_brick_list_is_a_no_op():
    dom = GridDomain(16)
    B.brickSweep(dom.brick(0), dom.brick(1), B.BrickList(np.zeros(0, np.uint32)), stencils.make("star7", 1))
    B.synchronize()


@pytest.mark.parametrize("name", stencils.PLAIN_SHAPES + ("heat7", "lap7"))
def test_fp64_floatfloat_against_oracle(name, kernel):
    """FP64 storage computed in float-float on the FP32 pipes: normwise error against the
    FP64 oracle within 1e-12 (47-bit inputs and Dot2 accumulation give ~1e-14)."""
    st = stencils.make(name, 7)
    dom, arr, got = device_sweep(64, st, acc=_abi.BK_ACC_FLOATFLOAT, seed=42)
    ref = oracle_array(dom, arr, st)
    err = normwise(got, ref)
    assert err <= 1e-12, err
    assert err <= 1e-13, err


def test_fp64_floatfloat_extreme_magnitudes():
    """Inputs spanning 1e-30 .. 1e30 keep ~1e-14 relative accuracy point by point where
    the result is not a cancellation; zeros stay zero."""
    st = stencils.make("star7", 1)
    dom = GridDomain(16)
    rng = np.random.default_rng(0)
    arr = rng.uniform(-1, 1, dom.adims) * 10.0 ** rng.integers(-30, 30, dom.adims)
    arr[rng.random(dom.adims) < 0.05] = 0.0
    _, _, got = device_sweep(16, st, acc=_abi.BK_ACC_FLOATFLOAT, arr=arr)
    ref = oracle_array(dom, arr, st)
    assert normwise(got, ref) <= 1e-13
    _, _, z = device_sweep(16, st, acc=_abi.BK_ACC_FLOATFLOAT, arr=np.zeros(dom.adims))
    assert np.all(z == 0.0)


def test_floatfloat_rejected_for_fp32():
    dom = GridDomain(16, dtype=BK_F32)
    with pytest.raises(_abi.BkError) as e:
        B.brickSweep(dom.brick(0), dom.brick(1), dom.dev_interior, stencils.make("star7", 1),
                     _abi.BK_ACC_FLOATFLOAT)
    assert e.value.status == _abi.BK_ERR_UNSUPPORTED


@pytest.mark.parametrize("dtype,acc,tol", [(BK_F64, BK_ACC_NATIVE, 1e-14), (BK_F64, _abi.BK_ACC_FLOATFLOAT, 1e-12),
                                           (BK_F32, BK_ACC_NATIVE, 1e-5)])
def test_cond_stencil_against_oracle(dtype, acc, tol):
    """The non-linear cond kernel (|sum c * max(x, 0)|) in every storage / arithmetic mode."""
    st = stencils.make("cond7", 3)
    dom, arr, got = device_sweep(32, st, dtype=dtype, acc=acc, seed=12)
    ref = np.zeros_like(arr)
    o, n = dom.org, dom.n
    src = arr.astype(np.float32).astype(np.float64) if dtype == BK_F32 else arr
    oracle.array_sweep(src, ref, o, tuple(a + b for a, b in zip(o, n)), st.offsets(), st.coeff,
                       pre=st.pre_op, post=st.post_op)
    ref = dom.interior_view(ref)
    assert np.all(got >= 0)
    assert normwise(got, ref) <= tol


def test_dsl_script_runs_on_the_gpu():
    from bricklib_gb300 import dsl
    path = os.path.join(os.path.dirname(__file__), "golden", "dsl", "star13_loops.py")
    st = dsl.load_stencil(path, {"W0": 0.4, "W1": 0.07, "W2": 0.03})
    dom, arr, got = device_sweep(32, st, seed=21)
    ok, md = mixed_ok(got, oracle_array(dom, arr, st))
    assert ok, md


def test_a_bounded_wait_that_runs_out_is_flagged_and_the_device_stays_usable(monkeypatch):
    """The TMA star kernel's waits are bounded.  With the test hook BK_TEST_WITHHOLD_COPY its
    first CTA posts a stage's byte count but withholds one of that stage's copies (so no copy is
    left in flight) and the wait limit drops to 5 ms: the consumers' wait runs out, the CTA sets
    the timeout flag, stops, and its producer drains its stages with bounded waits.  The host
    reads BK_ERR_TIMEOUT from the flags; the next sweep is clean and matches the oracle."""
    monkeypatch.delenv("BK_SWEEP_ONESHOT", raising=False)
    monkeypatch.delenv("BK_SWEEP_PIPELINED", raising=False)
    st = stencils.make("star7", 7)
    dom = GridDomain(64)
    arr = stencils.uniform(77, int(np.prod(dom.adims))).reshape(dom.adims)
    dom.set_field(0, arr)
    dom.upload()
    assert B.sweepKernel(dom.brick(0), dom.brick(1), st) == "sweep_star_tma_kernel"
    B.check_device()
    monkeypatch.setenv("BK_TEST_WITHHOLD_COPY", "1")
    B.brickSweep(dom.brick(0), dom.brick(1), dom.dev_interior, st)
    B.synchronize()
    with pytest.raises(_abi.BkError) as e:
        B.check_device()
    assert e.value.status == _abi.BK_ERR_TIMEOUT
    assert B.error_flags() == 0  # read and cleared
    monkeypatch.delenv("BK_TEST_WITHHOLD_COPY")
    B.brickSweep(dom.brick(0), dom.brick(1), dom.dev_interior, st)
    B.synchronize()
    B.check_device()
    dom.download()
    ok, md = mixed_ok(dom.interior_view(dom.get_field(1)), oracle_array(dom, arr, st))
    assert ok, f"max |diff| {md}"
