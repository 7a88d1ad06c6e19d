"""A domain past 2^31 elements per field (1536^3 interior, FP32, 15 GB per field): the
sweeps address every brick with 64-bit offsets.  Checked on a sample of bricks that includes
the last ones in storage, each against its neighbourhood computed on the host."""
import ctypes as C

import numpy as np
import pytest

from bricklib_gb300 import _abi, bricks as B, stencils
from bricklib_gb300._abi import call

pytestmark = pytest.mark.gpu


def _brick(ptr, b, bsize, step):
    out = np.empty(bsize, np.float32)
    B.memcpy(out.ctypes.data, ptr + b * step * 4, bsize * 4, 1, None)
    return out


@pytest.mark.parametrize("name", ["star7", "cube27"])
def test_fields_past_two_to_the_31_elements(name):
    n = 1536
    g = n // 8 + 2
    grid, info = B.init_grid([g, g, g])
    nb = info.nbricks
    assert nb * 512 > 2 ** 31
    dinfo = B.movBrickInfo(info)
    s_in = B.BrickStorage.allocate_device(nb, 512, _abi.BK_F32)
    s_out = B.BrickStorage.allocate_device(nb, 512, _abi.BK_F32)
    call("bk_fill_uniform", C.c_void_p(s_in.ptr), nb * 512, _abi.BK_F32, 7, -1.0, 1.0, None)
    g3 = grid.reshape(g, g, g)
    interior = np.ascontiguousarray(g3[1:-1, 1:-1, 1:-1].reshape(-1))
    st = stencils.make(name, 3)
    B.brickSweep(B.Brick(dinfo, s_in, 0), B.Brick(dinfo, s_out, 0), B.BrickList(interior), st)
    B.synchronize()
    assert B.error_flags() == 0
    rng = np.random.default_rng(5)
    sample = np.concatenate([interior[-8:], interior[rng.integers(0, len(interior), 24)]])
    for b in sample.tolist():
        cube = np.zeros((24, 24, 24))
        for s in range(27):
            dk, dj, di = s // 9 - 1, (s // 3) % 3 - 1, s % 3 - 1
            nbr = int(info.adj[b, s])
            cube[(dk + 1) * 8:(dk + 2) * 8, (dj + 1) * 8:(dj + 2) * 8, (di + 1) * 8:(di + 2) * 8] = \
                _brick(s_in.ptr, nbr, 512, 512).reshape(8, 8, 8)
        want = np.zeros((8, 8, 8))
        for (dk, dj, di), c in zip(st.taps, st.coeff):
            want += c * cube[8 + dk:16 + dk, 8 + dj:16 + dj, 8 + di:16 + di]
        got = _brick(s_out.ptr, b, 512, 512).reshape(8, 8, 8)
        assert np.abs(got - want).max() <= 1e-5 * max(np.abs(want).max(), 1e-30), b
