"""A sweep over a BrickDecomp layout (include/brick-mpi.h:178-464) with its exchange as the
periodic ghost refresh, against the oracle's periodic array path."""
import numpy as np
import pytest

from bricklib_gb300 import bricks as B, decomp as D, stencils
from oracle import oracle

pytestmark = pytest.mark.gpu


def mixed_ok(a, b, tol=1e-12):
    d = np.abs(a - b)
    return bool(np.all((d < tol) | (d < (np.abs(a) + np.abs(b)) * tol))), float(d.max(initial=0))


@pytest.mark.parametrize("name,skin", [("heat7", "good"), ("star13", "normal"), ("cube27", "good")])
def test_decomp_steps_with_exchange_match_array_oracle(name, skin):
    n, depth, pad, steps = 32, 8, 8, 6
    st = stencils.make(name, 3)
    dec = D.BrickDecomp([n, n, n], depth, (8, 8, 8), numfield=2)
    dec.initialize(D.SKIN3D_GOOD if skin == "good" else D.SKIN3D_NORMAL)
    info = dec.getBrickInfo()
    bsize = 512
    storage = B.BrickStorage.allocate(dec.nbricks, 2 * bsize)
    g = n + 2 * depth
    adims = (g + 2 * pad,) * 3
    o = depth + pad
    arr = oracle.fill_sines(adims, (o,) * 3, (n,) * 3, 8, 77, 1e-3)
    grid = dec.grid_array()
    B.copyToBrick([g] * 3, [pad] * 3, [0] * 3, arr, grid, B.Brick(info, storage, 0))
    dinfo, dst = B.movBrickInfo(info), B.movBrickStorage(storage)
    gb = depth // 8
    interior = np.ascontiguousarray(grid[gb:-gb, gb:-gb, gb:-gb].reshape(-1))
    blist = B.BrickList(interior)
    bricks = [B.Brick(dinfo, dst, 0), B.Brick(dinfo, dst, bsize)]
    for t in range(steps):
        dec.exchange(dst)
        B.brickSweep(bricks[t % 2], bricks[(t + 1) % 2], blist, st)
    B.synchronize()
    assert B.error_flags() == 0
    host = B.movBrickStorage(dst, to_device=False)
    out = np.zeros(adims)
    B.copyFromBrick([n] * 3, [pad] * 3, [depth] * 3, out, grid, B.Brick(info, host, (steps % 2) * bsize))
    a, b = arr.copy(), np.zeros_like(arr)
    for _ in range(steps):
        oracle.array_periodic_fill(a, (o,) * 3, (n,) * 3, (8, 8, 8))
        oracle.array_sweep(a, b, (o,) * 3, (o + n,) * 3, st.offsets(), st.coeff)
        a, b = b, a
    sl = (slice(o, o + n),) * 3
    ok, md = mixed_ok(out[sl], a[sl])
    assert ok, f"max |diff| {md}"
