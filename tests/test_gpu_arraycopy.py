"""Device copyToBrick / copyFromBrick against the host versions (which the golden
vectors of the reference accessor pin)."""
import numpy as np
import pytest

from bricklib_gb300 import bricks as B, stencils
from bricklib_gb300._abi import BK_BF16, BK_F32, BK_F64

pytestmark = pytest.mark.gpu

LAYOUTS = [((8, 8, 8), (1, 4, 8)), ((8, 8, 8), (2, 4, 4)), ((4, 4, 4), (1, 4, 4)), ((8, 8, 32), (1, 1, 32))]


@pytest.mark.parametrize("bdim,fold", LAYOUTS, ids=lambda x: "x".join(map(str, x)))
@pytest.mark.parametrize("dtype", [BK_F64, BK_F32, BK_BF16])
def test_device_copy_to_and_from_bricks(bdim, fold, dtype):
    lay = B.Layout(bdim, fold)
    n = (16, 24, 64) if bdim[2] == 32 else (16, 24, 32)
    ghost = tuple(bdim)
    pad = (3, 5, 0)
    ext = tuple(x + 2 * (p + g) for x, p, g in zip(n, pad, ghost))
    arr = stencils.uniform(8, int(np.prod(ext))).reshape(ext)
    arr_s = B.to_storage_dtype(arr, dtype)
    gd = [(x + 2 * g) // b for x, g, b in zip(n, ghost, bdim)]
    grid, info = B.init_grid(list(reversed(gd)))
    # host reference copy
    hst = B.BrickStorage.allocate(info.nbricks, lay.size, dtype)
    rev = lambda t: list(reversed(t))
    B.copyToBrick(rev(n), rev(pad), rev(ghost), B.from_storage_dtype(arr_s, dtype), grid, B.Brick(info, hst, 0, lay))
    # device copy
    dst = B.BrickStorage.allocate_device(info.nbricks, lay.size, dtype)
    darr = B.DeviceBuffer(arr_s.nbytes)
    darr.upload(arr_s)
    dgrid = B.BrickList(grid)
    B.copyToBrickDevice(rev(n), rev(pad), rev(ghost), darr.ptr, dgrid.ptr, B.Brick(info, dst, 0, lay))
    B.synchronize()
    got = B.movBrickStorage(dst, to_device=False).host
    np.testing.assert_array_equal(got, hst.host)
    # and back, into an interior-only array (negative padding = -ghost)
    out = B.DeviceBuffer(int(np.prod(n)) * arr_s.itemsize)
    B.copyFromBrickDevice(rev(n), rev(tuple(-g for g in ghost)), rev(ghost), out.ptr, dgrid.ptr,
                          B.Brick(info, dst, 0, lay))
    back = out.download(np.empty(n, dtype=arr_s.dtype))
    o = tuple(p + g for p, g in zip(pad, ghost))
    np.testing.assert_array_equal(back, arr_s[o[0]:o[0] + n[0], o[1]:o[1] + n[1], o[2]:o[2] + n[2]])
