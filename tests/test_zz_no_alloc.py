"""bk_field_norms_noalloc: the FP64 error norms for callers that cannot call cudaMalloc
(a latency-bound serving loop, where cudaMalloc / cudaFree may synchronise the device, or a
process whose device memory another allocator has reserved).  Its scratch is a static
device array of BK_NORMS_NOALLOC_MAX_BRICKS partials shared by every call.

Called through the C ABI and checked against the allocating bk_field_norms on the same
inputs, two calls in a row with different inputs (the shared array keeps the previous
call's contents, which must not leak into the next result).  This file is collected last;
it passes alone in a fresh process and after the other tests.
"""
import ctypes as C

import numpy as np
import pytest

from bricklib_gb300 import _abi, bricks as B, stencils
from bricklib_gb300._abi import BK_F32, BK_F64
from bricklib_gb300.domain import GridDomain

pytestmark = pytest.mark.gpu

MAX_BRICKS = 16384  # BK_NORMS_NOALLOC_MAX_BRICKS


def norms(fn, a, ref, blist):
    out = (C.c_double * 4)()
    status = getattr(_abi.lib(), fn)(C.byref(a.field()), C.byref(ref.field()), C.c_void_p(blist.ptr), blist.n,
                                     C.byref(a.layout.to_c()), None, out)
    return status, list(out)


def close(x, y):
    # max entries are order independent: exact; sums may differ by the order of FP64 adds
    return x[0] == y[0] and x[2] == y[2] and abs(x[1] - y[1]) <= 1e-12 * abs(y[1]) and \
        abs(x[3] - y[3]) <= 1e-12 * abs(y[3])


def test_noalloc_norms_match_allocating_norms_twice():
    dom = GridDomain(64)  # 512 interior bricks
    arr = stencils.uniform(41, int(np.prod(dom.adims))).reshape(dom.adims)
    dom.set_field(0, arr)
    dom.upload()
    allb = B.BrickList(dom.grid)
    low = B.BrickStorage.allocate_device(dom.nbricks, dom.bsize, BK_F32)
    lowb = B.Brick(dom.dev_info, low, 0)
    B.convertField(dom.brick(0), lowb, allb)
    # call 1: FP32 copy against FP64 over every interior brick
    s1, got1 = norms("bk_field_norms_noalloc", lowb, dom.brick(0), dom.dev_interior)
    r1, want1 = norms("bk_field_norms", lowb, dom.brick(0), dom.dev_interior)
    assert s1 == 0 and r1 == 0
    assert got1[0] > 0 and close(got1, want1), (got1, want1)
    # call 2: a different field pair and a shorter list; nothing from call 1 may remain
    B.brickSweep(dom.brick(0), dom.brick(1), dom.dev_interior, stencils.make("star7", 2))
    short = B.BrickList(dom.interior[:37])
    s2, got2 = norms("bk_field_norms_noalloc", dom.brick(1), dom.brick(0), short)
    r2, want2 = norms("bk_field_norms", dom.brick(1), dom.brick(0), short)
    assert s2 == 0 and r2 == 0
    assert close(got2, want2), (got2, want2)
    assert got2 != got1


def test_noalloc_norms_report_an_out_of_range_brick_then_recover():
    """A listed brick past the storage is skipped (never read) and this call returns
    BK_ERR_BOUNDS; the error word is private to the call, so the next in-range call returns 0
    with the norms of bk_field_norms.  Device memory in use is the same before and after the
    calls: nothing was allocated."""
    import torch
    dom = GridDomain(32)
    arr = stencils.uniform(43, int(np.prod(dom.adims))).reshape(dom.adims)
    dom.set_field(0, arr)
    dom.upload()
    B.brickSweep(dom.brick(0), dom.brick(1), dom.dev_interior, stencils.make("star13", 4))
    B.synchronize()
    norms("bk_field_norms_noalloc", dom.brick(1), dom.brick(0), dom.dev_interior)  # first call on this device
    bad = B.BrickList(np.concatenate([dom.interior[:5], [dom.nbricks + 7], dom.interior[5:9]]).astype(np.uint32))
    status, _ = norms("bk_field_norms_noalloc", dom.brick(1), dom.brick(0), bad)
    assert status == _abi.BK_ERR_BOUNDS
    assert "out of range" in _abi.lib().bk_last_error().decode()
    s_ok, got = norms("bk_field_norms_noalloc", dom.brick(1), dom.brick(0), dom.dev_interior)
    r_ok, want = norms("bk_field_norms", dom.brick(1), dom.brick(0), dom.dev_interior)
    assert s_ok == 0 and r_ok == 0 and close(got, want), (got, want)
    B.synchronize()
    # bk_field_norms keeps a buffer made on its first call, and the list above is a device
    # buffer; from here on only no-alloc calls run, and free device memory must not move
    free1, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        s_again, _ = norms("bk_field_norms_noalloc", dom.brick(1), dom.brick(0), dom.dev_interior)
        assert s_again == 0
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free1


def test_noalloc_norms_reject_lists_beyond_the_static_maximum():
    dom = GridDomain(16)
    big = B.BrickList(np.zeros(MAX_BRICKS + 1, dtype=np.uint32))
    status, _ = norms("bk_field_norms_noalloc", dom.brick(0), dom.brick(1), big)
    assert status == _abi.BK_ERR_ARG
    msg = _abi.lib().bk_last_error().decode()
    assert str(MAX_BRICKS) in msg and "split" in msg
    # exactly the maximum is accepted
    full = B.BrickList(np.full(MAX_BRICKS, dom.interior[0], dtype=np.uint32))
    status, out = norms("bk_field_norms_noalloc", dom.brick(0), dom.brick(0), full)
    assert status == 0 and out[0] == 0.0 and out[1] == 0.0
