"""4-D bricks on the GPU (bk_sweep4): the reference's 4-D brick kernel's golden outputs
(weak/main-4d.cpp layout, stencils/mpi9pt.py), FP32, a radius-2 tap list, bad input, and
periodic steps over a 4-D BrickDecomp layout with its exchange."""
import os

import numpy as np
import pytest

from bricklib_gb300 import _abi, bricks as B, bricks4 as B4, decomp as D, stencils
from oracle import array4

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), "golden")
FOLDS = {0: (1, 1, 2, 4), 2: (1, 1, 1, 1)}


def mixed_ok(a, b, tol=1e-12):
    d = np.abs(a - b)
    return bool(np.all((d < tol) | (d < (np.abs(a) + np.abs(b)) * tol))), float(d.max(initial=0))


def run4(arr, st, n, dtype=_abi.BK_F64, lay=B4.Layout4(), ghost=8, pad=4):
    """One sweep of a (n + 2*(ghost+pad))^4 array's n^4 interior through init_grid<4> bricks."""
    gb = (n + 2 * ghost) // 4
    grid, adj = B4.init_grid([gb] * 4)
    np_dt = B.NP_DTYPE[dtype]
    store = np.zeros(len(grid) * 512, np_dt)
    B4.copy_to_bricks(arr.astype(np_dt), grid, (gb,) * 4, (pad,) * 4, store, 512, 0, lay)
    adj_dev = B.DeviceBuffer(adj.nbytes)
    adj_dev.upload(adj)
    st_dev = B.BrickStorage(len(grid), 512, dtype, device=B.DeviceBuffer(store.nbytes))
    st_dev.device.upload(store)
    g3 = grid.reshape((gb,) * 4)
    q = ghost // 4
    interior = np.ascontiguousarray(g3[q:-q, q:-q, q:-q, q:-q].reshape(-1))
    B4.sweep4(adj_dev, len(grid), st_dev, 0, 256, B.BrickList(interior), st, lay)
    B.synchronize()
    assert B.error_flags() == 0
    st_dev.device.download(store)
    out = np.zeros(arr.shape)
    B4.copy_from_bricks(out, g3[q:-q, q:-q, q:-q, q:-q], (n // 4,) * 4, (pad + ghost,) * 4, store, 512, 256, lay)
    return out[(slice(pad + ghost, pad + ghost + n),) * 4]


@pytest.mark.parametrize("name", ["mpi9pt", "mpi9pt_fold1", "star9"])
def test_sweep4_matches_reference_golden(name):
    z = np.load(os.path.join(GOLD, f"sweep4_{name}.npz"))
    n = int(z["n"])
    S = n + 24
    arr = stencils.uniform(int(z["seed_in"]), S ** 4).reshape((S,) * 4)
    st = stencils.Stencil(name, [tuple(int(a) for a in t) for t in z["offsets"]], z["coeff"])
    got = run4(arr, st, n, lay=B4.Layout4(fold=FOLDS[int(z["fold"])]))
    ok, md = mixed_ok(got, z["out"])
    assert ok, f"max |diff| {md}"


def test_sweep4_fp32_and_radius2():
    n = 8
    S = n + 24
    arr = stencils.uniform(5, S ** 4).reshape((S,) * 4)
    taps = [(0, 0, 0, 0)] + [tuple(d if a == ax else 0 for a in range(4)) for ax in range(4) for d in (1, -1, 2, -2)]
    st = stencils.Stencil("star17_4d", taps, stencils.uniform01(9, len(taps)))
    ref = array4.array_sweep4(arr, st.taps, st.coeff, (12,) * 4, (n,) * 4)
    ok, md = mixed_ok(run4(arr, st, n), ref)
    assert ok, f"max |diff| {md}"
    a32 = arr.astype(np.float32).astype(np.float64)
    ref32 = array4.array_sweep4(a32, st.taps, st.coeff, (12,) * 4, (n,) * 4)
    got32 = run4(arr, st, n, dtype=_abi.BK_F32)
    assert np.abs(got32 - ref32).max() <= 1e-5 * np.abs(ref32).max()


@pytest.mark.parametrize("dtype", [_abi.BK_F64, _abi.BK_F32])
@pytest.mark.parametrize("fold", [(1, 1, 1, 1), (1, 1, 2, 4), (2, 1, 4, 1)])
@pytest.mark.parametrize("radius", [1, 2])
def test_sweep4_box_stencils_match_the_array_oracle(radius, fold, dtype):
    """Box tap lists, for which every tile row and both i halos are gathered, against the array
    loop: the full radius-1 box (81 taps) and 81 taps picked from the radius-2 box, on three
    folds; FP32 storage against the oracle on the FP32-rounded input (1e-5 of the largest)."""
    n = 8
    S = n + 24
    arr = stencils.uniform(6, S ** 4).reshape((S,) * 4)
    box = [tuple(int(a) - radius for a in t) for t in np.ndindex(*(2 * radius + 1,) * 4)]
    if len(box) > 81:
        box = [box[q] for q in np.random.default_rng(5).choice(len(box), size=81, replace=False)]
    st = stencils.Stencil(f"box{radius}", box, stencils.uniform01(7, len(box)))
    lay = B4.Layout4(fold=fold)
    if dtype == _abi.BK_F64:
        ref = array4.array_sweep4(arr, st.taps, st.coeff, (12,) * 4, (n,) * 4)
        ok, md = mixed_ok(run4(arr, st, n, lay=lay), ref)
        assert ok, f"max |diff| {md}"
    else:
        a32 = arr.astype(np.float32).astype(np.float64)
        ref32 = array4.array_sweep4(a32, st.taps, st.coeff, (12,) * 4, (n,) * 4)
        got32 = run4(arr, st, n, dtype=dtype, lay=lay)
        assert np.abs(got32 - ref32).max() <= 1e-5 * np.abs(ref32).max()


@pytest.mark.parametrize("dtype", [_abi.BK_F64, _abi.BK_F32])
def test_sweep4_partial_and_reordered_stars_match_the_array_oracle(dtype):
    """Stars that are not exactly the full star of the kernel's radius take the tap-list path
    (a partial star, one with a repeated tap); the full star listed in a shuffled order is
    summed in the kernel's canonical order: all three against the array oracle."""
    n = 8
    S = n + 24
    arr = stencils.uniform(8, S ** 4).reshape((S,) * 4)
    full = [(0, 0, 0, 0)] + [tuple(d if a == ax else 0 for a in range(4)) for ax in range(4) for d in (1, -1)]
    order = np.random.default_rng(9).permutation(len(full))
    cases = [
        ("partial", [(0, 0, 0, 0), (1, 0, 0, 0), (-1, 0, 0, 0), (0, 0, 0, 1)]),
        ("repeated", [(0, 0, 0, 0), (0, 0, 1, 0), (0, 0, 1, 0), (0, -1, 0, 0), (0, 0, 0, -1)]),
        ("shuffled", [full[q] for q in order]),
    ]
    for name, taps in cases:
        st = stencils.Stencil(name, taps, stencils.uniform01(10, len(taps)))
        if dtype == _abi.BK_F64:
            ref = array4.array_sweep4(arr, st.taps, st.coeff, (12,) * 4, (n,) * 4)
            ok, md = mixed_ok(run4(arr, st, n), ref)
            assert ok, f"{name}: max |diff| {md}"
        else:
            a32 = arr.astype(np.float32).astype(np.float64)
            ref32 = array4.array_sweep4(a32, st.taps, st.coeff, (12,) * 4, (n,) * 4)
            got32 = run4(arr, st, n, dtype=dtype)
            assert np.abs(got32 - ref32).max() <= 1e-5 * np.abs(ref32).max(), name


@pytest.mark.parametrize("dtype", [_abi.BK_F64, _abi.BK_F32])
def test_sweep4_mpi9pt_at_the_bench_size(dtype):
    """mpi9pt over the 64^4 domain the 4-D bench line times (18^4 bricks with one ghost brick a
    side, the default fold): every interior point against the array oracle (FP64: the mixed test
    at 1e-12; FP32 storage: the oracle on the FP32-rounded input, 1e-5 of the largest)."""
    n = 64
    S = n + 8
    arr = stencils.uniform(12, S ** 4).reshape((S,) * 4)
    st = B4.mpi9pt()
    if dtype == _abi.BK_F64:
        ref = array4.array_sweep4(arr, st.taps, st.coeff, (4,) * 4, (n,) * 4)
        ok, md = mixed_ok(run4(arr, st, n, ghost=4, pad=0), ref)
        assert ok, f"max |diff| {md}"
    else:
        a32 = arr.astype(np.float32).astype(np.float64)
        ref32 = array4.array_sweep4(a32, st.taps, st.coeff, (4,) * 4, (n,) * 4)
        got32 = run4(arr, st, n, dtype=dtype, ghost=4, pad=0)
        assert np.abs(got32 - ref32).max() <= 1e-5 * np.abs(ref32).max()


def test_sweep4_rejects_bad_arguments_and_flags_bad_lists():
    st = B4.mpi9pt()
    buf = B.DeviceBuffer(64 * 512 * 8)
    storage = B.BrickStorage(64, 512, _abi.BK_F64, device=buf)
    adj = B.DeviceBuffer(64 * 81 * 4)
    adj.upload(np.zeros(64 * 81, np.uint32))
    with pytest.raises(_abi.BkError):
        B4.sweep4(adj, 64, storage, 0, 256, B.BrickList(np.arange(4, dtype=np.uint32)), st,
                  B4.Layout4(bdim=(8, 4, 4, 2), fold=(1, 1, 1, 1)))
    with pytest.raises(_abi.BkError):
        B4.sweep4(adj, 64, storage, 0, 128, B.BrickList(np.arange(4, dtype=np.uint32)), st)  # fields overlap
    B.error_flags()
    B4.sweep4(adj, 64, storage, 0, 256, B.BrickList(np.array([1000], dtype=np.uint32)), st)
    B.synchronize()
    assert B.error_flags() & 1


def test_sweep4_periodic_steps_over_brickdecomp():
    n, depth, pad, steps = 16, 4, 4, 4
    st = B4.mpi9pt()
    dec = D.BrickDecomp([n] * 4, depth, (4, 4, 4, 4), numfield=2)
    dec.initialize(D.all_regions(4))
    lay = B4.Layout4()
    t = dec.t_dims[::-1]  # outermost first
    S = n + 2 * (depth + pad)
    o = depth + pad
    arr = np.zeros((S,) * 4)
    arr[(slice(o, o + n),) * 4] = stencils.uniform(3, n ** 4).reshape((n,) * 4)
    store = np.zeros(dec.nbricks * 512)
    grid = dec.grid_array()
    B4.copy_to_bricks(arr, grid, t, (pad,) * 4, store, 512, 0, lay)
    adj_dev = B.DeviceBuffer(dec.adj.nbytes)
    adj_dev.upload(np.ascontiguousarray(dec.adj))
    sdev = B.BrickStorage(dec.nbricks, 512, _abi.BK_F64, device=B.DeviceBuffer(store.nbytes))
    sdev.device.upload(store)
    interior = B.BrickList(np.ascontiguousarray(grid[1:-1, 1:-1, 1:-1, 1:-1].reshape(-1)))
    for s in range(steps):
        dec.exchange(sdev)
        B4.sweep4(adj_dev, dec.nbricks, sdev, (s % 2) * 256, ((s + 1) % 2) * 256, interior, st, lay)
    B.synchronize()
    assert B.error_flags() == 0
    sdev.device.download(store)
    out = np.zeros_like(arr)
    B4.copy_from_bricks(out, grid[1:-1, 1:-1, 1:-1, 1:-1], (n // 4,) * 4, (o,) * 4, store, 512,
                        (steps % 2) * 256, lay)
    a = arr.copy()
    for _ in range(steps):
        array4.periodic_fill4(a, (o,) * 4, (n,) * 4, depth)
        nxt = np.zeros_like(a)
        nxt[(slice(o, o + n),) * 4] = array4.array_sweep4(a, st.taps, st.coeff, (o,) * 4, (n,) * 4)
        a = nxt
    sl = (slice(o, o + n),) * 4
    ok, md = mixed_ok(out[sl], a[sl])
    assert ok, f"max |diff| {md}"


@pytest.mark.parametrize("dtype", [_abi.BK_F64, _abi.BK_F32])
@pytest.mark.parametrize("fold", [(1, 1, 2, 4), (1, 1, 2, 2)])
def test_sweep4_element_copies_equal_vector_copies(dtype, fold):
    """Input bricks off the 16-byte boundary (storage step 513) take one copy per element
    instead of 16-byte copies of whole row blocks: the same bits as the aligned storage, for a
    star (centre and faces fetched) and a radius-2 box (every element within the radius)."""
    gb = 6  # 4^4 interior bricks with one ghost brick a side
    grid, adj = B4.init_grid([gb] * 4)
    nb = len(grid)
    np_dt = B.NP_DTYPE[dtype]
    data = stencils.uniform(21, nb * 256).astype(np_dt).reshape(nb, 256)
    adj_dev = B.DeviceBuffer(adj.nbytes)
    adj_dev.upload(adj)
    g4 = grid.reshape((gb,) * 4)
    inner = B.BrickList(np.ascontiguousarray(g4[1:-1, 1:-1, 1:-1, 1:-1].reshape(-1)))
    lay = B4.Layout4(fold=fold)
    box = [tuple(int(a) - 2 for a in t) for t in np.ndindex(5, 5, 5, 5)]
    pick = np.random.default_rng(4).choice(len(box), size=81, replace=False)
    sts = [B4.mpi9pt(), stencils.Stencil("box81", [box[q] for q in pick], stencils.uniform01(4, 81))]
    for st in sts:
        outs = []
        for step in (512, 513):
            store = np.zeros((nb, step), np_dt)
            store[:, :256] = data
            sdev = B.BrickStorage(nb, step, dtype, device=B.DeviceBuffer(store.nbytes))
            sdev.device.upload(store)
            B4.sweep4(adj_dev, nb, sdev, 0, step - 256, inner, st, lay)
            B.synchronize()
            assert B.error_flags() == 0
            sdev.device.download(store)
            outs.append(store[:, step - 256:].copy())
        np.testing.assert_array_equal(outs[0].view(np.uint8), outs[1].view(np.uint8), err_msg=st.name)
