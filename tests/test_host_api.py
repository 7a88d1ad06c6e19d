"""CPU tests of the host side: the C ABI library loads and exports what the header
declares, host-only ABI calls behave, and the reference-named host API matches
the oracle."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from bricklib_gb300 import _abi, bricks as B, stencils
from bricklib_gb300.domain import GridDomain
from oracle import oracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for h in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if not h.endswith(".h"):
            continue
        src = open(os.path.join(ROOT, "include", h)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(bk_\w+)\s*\(", src, flags=re.M)
    return sorted(set(names))


def test_library_exports_every_declared_symbol():
    L = _abi.lib()
    names = declared_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    # every declared symbol has a ctypes signature in the binding
    assert not [n for n in names if n not in _abi.SIGNATURES], "binding lags the header"
    assert L.bk_abi_version() == 1


def test_stencil_families():
    lay = B.Layout()
    for name, fam in [("star7", 1), ("star13", 1), ("star25", 1), ("cube27", 2), ("cube125", 2), ("heat7", 1)]:
        r, f = B.stencil_family(stencils.make(name, 1), lay)
        assert f == fam, name
        assert r == stencils.make(name, 1).radius
    # a 19-point stencil has no dedicated family: generic
    taps = [t for t in stencils.cube_taps(1)[0] if sum(1 for a in t if a) <= 2]
    r, f = B.stencil_family(stencils.custom("d3pt19", taps, np.ones(len(taps))), lay)
    assert (r, f) == (1, 0)
    # a non-row-major fold routes everything to the generic family
    r, f = B.stencil_family(stencils.make("star7", 1), B.Layout((8, 8, 8), (1, 2, 2)))
    assert f == 0


def _kernel_for(name, lay=None, dtype=_abi.BK_F64, acc=_abi.BK_ACC_NATIVE, offset=0, base=1 << 20, odd_out=False):
    """bk_sweep_kernel on host-only field descriptors (the pointer is never dereferenced);
    `odd_out`: an output storage of step 2 x size + 1 with the field at offset 1."""
    lay = lay or B.Layout()
    size = lay.size
    fin = _abi.bk_field(C.c_void_p(base), 100, 2 * size, offset, dtype)
    fout = _abi.bk_field(C.c_void_p(base), 100, 2 * size, size if offset == 0 else 0, dtype)
    if odd_out:
        fout = _abi.bk_field(C.c_void_p(base + (1 << 24)), 100, 2 * size + 1, 1, dtype)
    out = C.c_char_p()
    _abi.call("bk_sweep_kernel", C.byref(fin), C.byref(fout), C.byref(B.to_c_stencil(stencils.make(name, 1))),
              C.byref(lay.to_c()), acc, C.byref(out))
    return out.value.decode()


def test_kernel_choice(monkeypatch):
    monkeypatch.delenv("BK_SWEEP_ONESHOT", raising=False)
    monkeypatch.delenv("BK_SWEEP_PIPELINED", raising=False)
    monkeypatch.delenv("BK_TMA_ROW", raising=False)
    for name in ("star7", "star13", "star25", "heat7"):
        assert _kernel_for(name) == "sweep_star_tma_kernel", name
        for dt in (_abi.BK_F32, _abi.BK_BF16):
            assert _kernel_for(name, dtype=dt) == "sweep_star_row_kernel", (name, dt)
            assert _kernel_for(name, dtype=dt, acc=_abi.BK_ACC_COMPENSATED) == "sweep_star_row_kernel", (name, dt)
    monkeypatch.setenv("BK_TMA_ROW", "0")
    assert _kernel_for("star7", dtype=_abi.BK_F32) == "sweep_star_tma_kernel"
    monkeypatch.delenv("BK_TMA_ROW")
    assert _kernel_for("star7", acc=_abi.BK_ACC_FLOATFLOAT) == "sweep_star_tma_kernel"
    assert _kernel_for("cube27") == "sweep2_kernel"
    assert _kernel_for("cube125", dtype=_abi.BK_F32) == "sweep2_kernel"
    assert _kernel_for("cube27", acc=_abi.BK_ACC_FLOATFLOAT) == "sweep_kernel"
    # the 125-point cube's coefficients are mirror-symmetric: float-float on pair sums
    assert _kernel_for("cube125", acc=_abi.BK_ACC_FLOATFLOAT) == "sweep2_kernel"
    assert _kernel_for("cond7") == "sweep_kernel"  # pointwise operations: one-shot kernel only
    assert _kernel_for("star7", lay=B.Layout((8, 8, 8), (1, 2, 2))) == "sweep_kernel"
    assert _kernel_for("star7", lay=B.Layout((4, 4, 4), (1, 4, 4))) == "sweep2_kernel"
    assert _kernel_for("star7", base=(1 << 20) + 8) == "sweep_kernel"  # not 16-byte aligned
    # output bricks off the two-element boundary: no kernel that stores output pairs
    assert _kernel_for("cube125", odd_out=True) == "sweep_kernel"
    assert _kernel_for("cube27", dtype=_abi.BK_F32, odd_out=True) == "sweep_kernel"
    assert _kernel_for("star7", dtype=_abi.BK_F32, odd_out=True) == "sweep_star_tma_kernel"
    assert _kernel_for("star7", odd_out=True) == "sweep_star_tma_kernel"
    monkeypatch.setenv("BK_SWEEP_PIPELINED", "1")
    assert _kernel_for("star7") == "sweep2_kernel"
    monkeypatch.setenv("BK_SWEEP_ONESHOT", "1")
    assert _kernel_for("star7") == "sweep_kernel"


def test_in_and_out_fields_that_alias_are_rejected():
    """A sweep never writes an element it reads: one storage seen with two steps, or two
    storages whose bytes overlap, is rejected before any launch (3-D and 4-D); the interleaved
    bIn / bOut of one storage (offsets a brick apart) and separate storages are accepted."""
    from bricklib_gb300 import bricks4 as B4
    lay = B.Layout()
    size, base = lay.size, 1 << 20
    cst = B.to_c_stencil(stencils.make("star7", 1))

    def kernel(fin, fout):
        out = C.c_char_p()
        return _abi.lib().bk_sweep_kernel(C.byref(fin), C.byref(fout), C.byref(cst), C.byref(lay.to_c()),
                                          _abi.BK_ACC_NATIVE, C.byref(out))

    f = _abi.bk_field
    ok_pairs = [
        (f(C.c_void_p(base), 100, 2 * size, 0, _abi.BK_F64), f(C.c_void_p(base), 100, 2 * size, size, _abi.BK_F64)),
        (f(C.c_void_p(base), 100, size, 0, _abi.BK_F64), f(C.c_void_p(base + 100 * size * 8), 100, size, 0, _abi.BK_F64)),
    ]
    bad_pairs = [
        # one storage, two steps: brick b of one field meets brick b' of the other
        (f(C.c_void_p(base), 100, 2 * size, 0, _abi.BK_F64), f(C.c_void_p(base), 100, 3 * size, size, _abi.BK_F64)),
        # two storages overlapping in memory
        (f(C.c_void_p(base), 100, size, 0, _abi.BK_F64), f(C.c_void_p(base + 50 * size * 8), 100, size, 0, _abi.BK_F64)),
        # one storage, offsets less than a brick apart
        (f(C.c_void_p(base), 100, 2 * size, 0, _abi.BK_F64), f(C.c_void_p(base), 100, 2 * size, 8, _abi.BK_F64)),
    ]
    for a, b in ok_pairs:
        assert kernel(a, b) == 0, _abi.lib().bk_last_error()
    for a, b in bad_pairs:
        assert kernel(a, b) == _abi.BK_ERR_ARG
        assert b"overlap" in _abi.lib().bk_last_error() or b"share storage" in _abi.lib().bk_last_error()
    # 4-D: the same rule (nlist 0, so nothing would launch even if the fields were accepted)
    st4 = B4.to_c_stencil4(B4.mpi9pt())
    lay4 = B4.Layout4().to_c()
    good4 = (f(C.c_void_p(base), 100, 512, 0, _abi.BK_F64), f(C.c_void_p(base), 100, 512, 256, _abi.BK_F64))
    bad4 = (f(C.c_void_p(base), 100, 512, 0, _abi.BK_F64), f(C.c_void_p(base), 100, 768, 256, _abi.BK_F64))
    for (a, b), want in ((good4, 0), (bad4, _abi.BK_ERR_ARG)):
        got = _abi.lib().bk_sweep4(None, 0, C.byref(a), C.byref(b), None, 0, C.byref(st4), C.byref(lay4), None)
        assert got == want, _abi.lib().bk_last_error()


def test_sweep4_list_length_is_checked_before_any_launch():
    """4-D sweeps walk their list with 32-bit positions: a list of 2^31 or more bricks is
    BK_ERR_ARG, reported before anything touches the device (the pointers here are never read)."""
    from bricklib_gb300 import bricks4 as B4
    f = _abi.bk_field
    base = 1 << 20
    st4 = B4.to_c_stencil4(B4.mpi9pt())
    lay4 = B4.Layout4().to_c()
    a, b = f(C.c_void_p(base), 100, 512, 0, _abi.BK_F64), f(C.c_void_p(base), 100, 512, 256, _abi.BK_F64)
    fake = C.c_void_p(base)
    got = _abi.lib().bk_sweep4(fake, 100, C.byref(a), C.byref(b), fake, 1 << 31, C.byref(st4), C.byref(lay4), None)
    assert got == _abi.BK_ERR_ARG and b"2^31" in _abi.lib().bk_last_error()


def test_stencil_errors_are_reported_not_raised_in_c():
    bad = stencils.custom("far", [(0, 0, 9)], [1.0])
    with pytest.raises(_abi.BkError) as e:
        B.stencil_family(bad, B.Layout())
    assert e.value.status == _abi.BK_ERR_ARG and "brick dim" in str(e.value)
    with pytest.raises(_abi.BkError) as e:
        B.stencil_family(stencils.custom("r5", [(0, 0, 5)], [1.0]), B.Layout((8, 8, 32), (1, 1, 32)))
    assert e.value.status == _abi.BK_ERR_UNSUPPORTED


def test_pipeline_depth_setting_is_checked():
    """bk_set_pipeline_depth takes 0 (the kernels' defaults) or 2..4 stages and keeps the value
    per host thread; anything else is BK_ERR_ARG and leaves the setting alone."""
    lib = _abi.lib()
    assert lib.bk_get_pipeline_depth() == 0
    for bad in (1, 5, -2):
        assert lib.bk_set_pipeline_depth(bad) == _abi.BK_ERR_ARG
    assert lib.bk_get_pipeline_depth() == 0
    assert lib.bk_set_pipeline_depth(3) == 0 and lib.bk_get_pipeline_depth() == 3
    assert lib.bk_set_pipeline_depth(0) == 0 and lib.bk_get_pipeline_depth() == 0


def test_periodic_plan_abi_matches_oracle():
    dom = GridDomain(16, device=False)
    plan = B.GhostPlan.__new__(B.GhostPlan)
    nb_c, gb_c = (C.c_long * 3)(*dom.nb), (C.c_long * 3)(*dom.gb)
    cnt = C.c_long()
    _abi.call("bk_periodic_plan", dom.grid.ctypes.data_as(C.c_void_p), nb_c, gb_c, None, 0, C.byref(cnt))
    pairs = np.empty((cnt.value, 2), dtype=np.uint32)
    _abi.call("bk_periodic_plan", dom.grid.ctypes.data_as(C.c_void_p), nb_c, gb_c,
              pairs.ctypes.data_as(C.c_void_p), cnt.value, C.byref(cnt))
    np.testing.assert_array_equal(pairs, oracle.periodic_plan(dom.grid, dom.nb, dom.gb))


@pytest.mark.parametrize("bdim,fold", [((8, 8, 8), (1, 4, 8)), ((8, 8, 8), (2, 4, 4)), ((4, 4, 4), (1, 4, 4))])
def test_copy_to_from_brick_matches_oracle(bdim, fold):
    lay = B.Layout(bdim, fold)
    dom = GridDomain(16, layout=lay, device=False)
    arr = stencils.uniform(3, int(np.prod(dom.adims))).reshape(dom.adims)
    dom.set_field(0, arr)
    odom = oracle.Domain(16, bdim=bdim, fold=fold)
    dat = odom.alloc()
    odom.to_bricks(arr, dat, 0)
    np.testing.assert_array_equal(dom.storage.host, dat)
    np.testing.assert_array_equal(dom.get_field(0), odom.from_bricks(dat, 0))


def test_bf16_rounding():
    x = np.array([1.0, 1.00390625, 1.01171875, -3.5, 1e-3], dtype=np.float32)
    back = B.bf16_to_f32(B.f32_to_bf16(x))
    assert back[0] == 1.0 and back[1] == 1.0  # ties to even
    assert back[2] == np.float32(1.015625)
    assert back[3] == -3.5
    assert abs(back[4] - 1e-3) / 1e-3 < 2 ** -8


def test_cpp_headers_match_reference_accessor(tmp_path):
    """include/brick.h + bricksetup.h compiled with g++: accessor offsets and init_grid
    equal the golden vectors made by the reference's own headers."""
    import shutil
    import subprocess
    if not shutil.which("g++"):
        pytest.skip("g++ not available")
    exe, out = tmp_path / "host_api_check", tmp_path / "out.bin"
    subprocess.check_call(["g++", "-O1", "-std=c++17", "-I", os.path.join(ROOT, "include"),
                           os.path.join(ROOT, "tests", "cpp", "host_api_check.cpp"), "-o", str(exe)])
    subprocess.check_call([str(exe), str(out)])
    raw = open(out, "rb").read()
    z = np.load(os.path.join(ROOT, "tests", "golden", "layouts.npz"))
    pos = 0
    for lid in range(7):
        want = z[f"offsets_{lid}"]
        got = np.frombuffer(raw, dtype=np.int64, count=len(want), offset=pos)
        pos += 8 * len(want)
        np.testing.assert_array_equal(got, want, err_msg=f"layout {lid}")
    g = np.load(os.path.join(ROOT, "tests", "golden", "init_grid.npz"))
    grid = np.frombuffer(raw, dtype=np.uint32, count=60, offset=pos)
    adj = np.frombuffer(raw, dtype=np.uint32, count=60 * 27, offset=pos + 240)
    np.testing.assert_array_equal(grid, g["grid"])
    np.testing.assert_array_equal(adj, g["adj"])


@pytest.mark.parametrize("nb", [(3, 4, 5), (1, 2, 3), (1, 1, 1)])
def test_periodic_adjacency_points_at_wrapped_interior_bricks(nb):
    """The batch's periodic adjacency (host side): every neighbour of an interior brick is the
    interior brick at the wrapped position, and entries between interior bricks are unchanged
    (one-brick-wide axes wrap onto the brick itself)."""
    from bricklib_gb300 import batch as BT
    g = tuple(x + 2 for x in nb)  # (k, j, i) bricks with one ghost brick per side
    grid, info = B.init_grid(list(reversed(g)))
    nb_c, gb_c = (C.c_long * 3)(*nb), (C.c_long * 3)(1, 1, 1)
    cnt = C.c_long()
    gr = np.ascontiguousarray(grid, dtype=np.uint32)
    _abi.call("bk_periodic_plan", gr.ctypes.data_as(C.c_void_p), nb_c, gb_c, None, 0, C.byref(cnt))
    pairs = np.empty((cnt.value, 2), dtype=np.uint32)
    _abi.call("bk_periodic_plan", gr.ctypes.data_as(C.c_void_p), nb_c, gb_c, pairs.ctypes.data_as(C.c_void_p),
              cnt.value, C.byref(cnt))
    wadj = BT.periodic_adjacency(info.adj, pairs)
    g3 = grid.reshape(g)
    for k in range(1, g[0] - 1):
        for j in range(1, g[1] - 1):
            for i in range(1, g[2] - 1):
                b = g3[k, j, i]
                for s in range(27):
                    dk, dj, di = s // 9 - 1, (s // 3) % 3 - 1, s % 3 - 1
                    wk = 1 + (k + dk - 1) % nb[0]
                    wj = 1 + (j + dj - 1) % nb[1]
                    wi = 1 + (i + di - 1) % nb[2]
                    assert wadj[b, s] == g3[wk, wj, wi], (b, s)
                    if 1 <= k + dk <= nb[0] and 1 <= j + dj <= nb[1] and 1 <= i + di <= nb[2]:
                        assert wadj[b, s] == info.adj[b, s]


def test_bench_instruction_counts_follow_the_symmetry_the_kernels_use():
    """bench.py's floating-point instructions per point (the numerator of roofline.compute
    pipe_frac) follow the coefficient symmetry the kernels exploit: FP64 mirror-symmetric cubes
    stream along i (37 with k <-> j symmetry, 43 without), FP32 / BF16 ones too (compensated:
    Dot2 W sums), a cube without the symmetry takes a multiply-add per tap."""
    import sys
    sys.path.insert(0, ROOT)
    import bench
    from tests.test_gpu_sweep import _mirror_symmetric_cube
    nat = _abi.BK_ACC_NATIVE
    assert bench.fp_instructions_per_point(stencils.make("cube125", 3), nat, _abi.BK_F64) == 37.0
    assert bench.fp_instructions_per_point(_mirror_symmetric_cube(2, 5), nat, _abi.BK_F64) == 43.0
    assert bench.fp_instructions_per_point(_mirror_symmetric_cube(1, 5, kj=True), nat, _abi.BK_F64) == 13.0
    assert bench.fp_instructions_per_point(stencils.make("cube125", 3), nat, _abi.BK_F32) == 37.0
    assert bench.fp_instructions_per_point(_mirror_symmetric_cube(2, 5), nat, _abi.BK_BF16) == 43.0
    assert bench.fp_instructions_per_point(_mirror_symmetric_cube(1, 5), nat, _abi.BK_F32) == 14.0
    assert bench.fp_instructions_per_point(stencils.make("cube125", 3), _abi.BK_ACC_COMPENSATED,
                                           _abi.BK_F32) == 15 + 3 * 52 + 22
    assert bench.fp_instructions_per_point(stencils.make("cube27", 3), nat, _abi.BK_F64) == 27.0
    assert bench.fp_instructions_per_point(stencils.make("star25", 3), nat, _abi.BK_F64) == 25.0
    assert bench.fp_instructions_per_point(stencils.make("cube125", 3), _abi.BK_ACC_FLOATFLOAT, _abi.BK_F64) == 125.0
