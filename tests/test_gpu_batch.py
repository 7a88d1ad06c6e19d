"""Batched form: many uneven periodic domains in one persistent launch per step."""
import numpy as np
import pytest

from bricklib_gb300 import _abi, batch as BT, bricks as B, stencils
from bricklib_gb300._abi import call
from bricklib_gb300.domain import GridDomain
from bricklib_gb300._abi import BK_ACC_COMPENSATED, BK_ACC_NATIVE, BK_F32, BK_F64
from oracle import oracle

pytestmark = pytest.mark.gpu


def small_workload(nd=8, multiple=8, hi=48):
    return BT.make_workload(ndom=nd, seed=9, lo=16, hi=hi, multiple=multiple)


def fields(b, which):
    out = []
    for ds in b.doms:
        host = B.movBrickStorage(ds.storage, to_device=False).host
        out.append(host.reshape(ds.nbricks, -1)[:, which * ds.lay.size:(which + 1) * ds.lay.size].copy())
    return out


def per_domain_steps(w, lay, dtype, steps, acc=BK_ACC_NATIVE):
    res = []
    for spec in w.domains:
        ds = BT.DomainStorage(spec, lay, dtype)
        BT.init_domain(ds)
        plan = B.GhostPlan(ds.pairs)
        lst = B.BrickList(ds.interior)
        B.timeSteps(ds.field(0), ds.field(1), lst, w.stencils[spec.stencil], steps, plan=plan, acc=acc,
                    use_graph=False)
        B.synchronize()
        host = B.movBrickStorage(ds.storage, to_device=False).host
        res.append(host.reshape(ds.nbricks, -1)[:, (steps % 2) * lay.size:((steps % 2) + 1) * lay.size].copy())
    return res


def test_batch_equals_per_domain_runs_and_oracle():
    w = small_workload()
    lay = B.Layout()
    steps = 6
    b = BT.Batch(w, lay, BK_F32)
    b.run(steps, use_graph=True)
    B.synchronize()
    assert b.parity == steps % 2
    got = fields(b, b.parity)
    want = per_domain_steps(w, lay, BK_F32, steps)
    ref64 = per_domain_steps(w, lay, BK_F64, steps)
    for d, spec in enumerate(w.domains):
        ds = b.doms[d]
        idx = ds.interior
        g, f32, f64 = got[d][idx], want[d][idx], ref64[d][idx]
        # same storage type, per-domain launch vs batch: FP32 arithmetic up to tap grouping
        assert np.abs(g - f32).max() <= 1e-6 * np.abs(f64).max(), d
        # the FP32 batch against the FP64 run of the same domain: the 1e-5 spec
        assert np.abs(g - f64).max() <= 1e-5 * np.abs(f64).max(), d
    # one domain against the CPU oracle (FP64 array path from the same initial values)
    spec = w.domains[0]
    ds = BT.DomainStorage(spec, lay, BK_F64)
    BT.init_domain(ds)
    host0 = B.movBrickStorage(ds.storage, to_device=False).host
    n = spec.n
    odom = oracle.Domain(n)
    a = odom.from_bricks(host0, 0)
    # from_bricks copies only the interior: refill the ghost zone periodically each step
    o = odom.ghost + odom.pad
    st = w.stencils[spec.stencil]
    bb = np.zeros_like(a)
    for _ in range(steps):
        oracle.array_periodic_fill(a, (o,) * 3, n, (8, 8, 8))
        oracle.array_sweep(a, bb, (o,) * 3, tuple(o + x for x in n), st.offsets(), st.coeff)
        a, bb = bb, a
    dat = odom.alloc()
    odom.to_bricks(a, dat, 0)
    orc = dat.reshape(odom.nbricks, odom.step)[:, :odom.bsize][ds.interior]
    assert np.abs(got[0][ds.interior] - orc).max() <= 1e-5 * np.abs(orc).max()
    b.close()


def test_batch_graph_and_plain_bitwise_equal_and_layouts_agree():
    w = small_workload(nd=6, multiple=32, hi=64)
    res = []
    for g in (True, False):
        b = BT.Batch(w, B.Layout(), BK_F32)
        b.run(4, use_graph=g)
        B.synchronize()
        res.append(fields(b, b.parity))
        b.close()
    for x, y in zip(*res):
        np.testing.assert_array_equal(x, y)
    # the point arithmetic does not depend on the brick layout: load the same arrays into
    # every layout (copyToBrick), run, and compare the interiors as arrays
    arrays = []
    for spec in w.domains:
        arrays.append(stencils.uniform(spec.seed, int(np.prod([x + 2 * 32 + 16 for x in spec.n]))))
    base = None
    for bdim, fold in BT.CANDIDATES:
        lay = B.Layout(bdim, fold)
        assert BT.layout_valid(w, lay)
        b = BT.Batch(w, lay, BK_F32, init=False)
        for ds, a in zip(b.doms, arrays):
            big = a.reshape([x + 2 * 32 + 16 for x in ds.spec.n])
            sub = big[tuple(slice(32 - b_, 32 - b_ + x + 2 * b_ + 16) for x, b_ in zip(ds.spec.n, bdim))]
            host = np.zeros(ds.nbricks * 2 * lay.size, np.float32)
            st = B.BrickStorage(ds.nbricks, 2 * lay.size, BK_F32, host=host)
            g = [x + 2 * b_ for x, b_ in zip(reversed(ds.spec.n), reversed(bdim))]
            B.copyToBrick(g, [8] * 3, [0] * 3, np.ascontiguousarray(sub), ds.grid, B.Brick(ds.info, st, 0, lay))
            ds.storage.device.upload(host)
        b.run(4)
        B.synchronize()
        arrs = []
        for ds, f in zip(b.doms, fields(b, b.parity)):
            dat = np.zeros(ds.nbricks * 2 * lay.size, np.float32)
            dat.reshape(ds.nbricks, -1)[:, :lay.size] = f
            st = B.BrickStorage(ds.nbricks, 2 * lay.size, BK_F32, host=dat)
            arr = np.zeros(tuple(x + 2 * b_ + 16 for x, b_ in zip(ds.spec.n, bdim)))
            B.copyFromBrick(list(reversed(ds.spec.n)), [8] * 3, list(reversed(bdim)), arr, ds.grid,
                            B.Brick(ds.info, st, 0, lay))
            arrs.append(arr[tuple(slice(8 + b_, 8 + b_ + x) for x, b_ in zip(ds.spec.n, bdim))])
        b.close()
        if base is None:
            base = arrs
        elif lay.offsets().tolist() == list(range(lay.size)) and tuple(bdim) == (8, 8, 8):
            # row-major 8x8x8 layouts run the same pipelined kernel: bit-identical
            for x, y in zip(base, arrs):
                np.testing.assert_array_equal(x, y)
        else:
            # other folds run the one-shot kernel, which orders cube taps differently, and
            # only 8x8x8 bricks have the pair-sum path of mirror-symmetric cubes
            for x, y in zip(base, arrs):
                assert np.abs(x - y).max() <= 1e-6 * np.abs(y).max()


def test_pipeline_depth_leaves_the_bits_unchanged():
    """The batch's pipeline-depth knob (the TMA-fed star kernels' stage count, one of the
    autotuner's launch-shape settings) changes no result: every depth gives the bits of the
    kernels' defaults, and so does the library-wide setting on a plain sweep."""
    w = small_workload(nd=6, multiple=16, hi=64)
    res = {}
    for stg in (0, 2, 3, 4):
        b = BT.Batch(w, B.Layout(), BK_F32)
        call("bk_batch_set_stages", b.h, stg)
        b.run(4, use_graph=True)
        B.synchronize()
        res[stg] = fields(b, b.parity)
        b.close()
    for stg in (2, 3, 4):
        for x, y in zip(res[0], res[stg]):
            np.testing.assert_array_equal(x.view(np.uint8), y.view(np.uint8), err_msg=f"stages {stg}")
    assert _abi.lib().bk_get_pipeline_depth() == 0  # the batch restored the caller's setting
    dom = GridDomain(64, dtype=BK_F32)
    dom.set_field(0, stencils.uniform(5, int(np.prod(dom.adims))).reshape(dom.adims))
    dom.upload()
    st = stencils.make("star13", 3)
    outs = []
    for stg in (0, 4):
        call("bk_set_pipeline_depth", stg)
        B.brickSweep(dom.brick(0), dom.brick(1), dom.dev_interior, st)
        B.synchronize()
        dom.download()
        outs.append(dom.get_field(1))
    call("bk_set_pipeline_depth", 0)
    np.testing.assert_array_equal(outs[0].view(np.uint8), outs[1].view(np.uint8))


def test_domain_alone_equals_domain_in_the_mix():
    w = small_workload(nd=5)
    b = BT.Batch(w, B.Layout(), BK_F32, BK_ACC_COMPENSATED)
    b.run(3)
    B.synchronize()
    mix = fields(b, b.parity)
    b.close()
    for d in (0, 3):
        alone = BT.Workload([w.domains[d]], w.stencils)
        b1 = BT.Batch(alone, B.Layout(), BK_F32, BK_ACC_COMPENSATED)
        b1.run(3)
        B.synchronize()
        np.testing.assert_array_equal(fields(b1, b1.parity)[0], mix[d])
        b1.close()


@pytest.mark.parametrize("lo,hi", [(16, 48), (8, 16)])
def test_periodic_adjacency_equals_ghost_fill(lo, hi):
    """The periodic boundary through the adjacency (no fill) and through ghost bricks refreshed
    before every step give the same interior, bit for bit (8-cell edges: a domain one brick
    wide, whose every neighbour is itself)."""
    w = BT.make_workload(ndom=6, seed=21, lo=lo, hi=hi, multiple=8)
    res = []
    for wrap in (True, False):
        b = BT.Batch(w, B.Layout(), BK_F32, wrap=wrap)
        b.run(5)
        B.synchronize()
        res.append([f[ds.interior] for f, ds in zip(fields(b, b.parity), b.doms)])
        b.close()
    for x, y in zip(*res):
        np.testing.assert_array_equal(x, y)


@pytest.mark.parametrize("wrap", [True, False])
def test_arena_batch_equals_per_domain_storages(wrap):
    """Domains as brick ranges of one arena (one brick set swept by the plain kernels, stars on
    the TMA-fed ones) and domains in storages of their own (the batch-mode kernels) give the
    same interiors bit for bit, with the boundary in the adjacency and with ghost fills."""
    w = small_workload(nd=8)
    res = []
    from bricklib_gb300 import _abi
    for arena in (True, False):
        b = BT.Batch(w, B.Layout(), BK_F32, wrap=wrap, arena=arena)
        assert _abi.lib().bk_batch_is_arena(b.h) == (1 if arena else 0)
        b.run(5)
        B.synchronize()
        assert B.error_flags() == 0
        res.append([f[ds.interior] for f, ds in zip(fields(b, b.parity), b.doms)])
        b.close()
    for x, y in zip(*res):
        np.testing.assert_array_equal(x, y)


def test_batch_rejects_bad_domains():
    from bricklib_gb300 import _abi
    import ctypes as C
    w = small_workload(nd=1)
    ds = BT.DomainStorage(w.domains[0], B.Layout(), BK_F32)
    d = ds.desc(5)  # stencil index out of range
    sts = (_abi.bk_stencil * 1)(B.to_c_stencil(w.stencils[0]))
    h = C.c_void_p()
    st = _abi.lib().bk_batch_create(C.byref(h), C.byref(d), 1, sts, 1, C.byref(B.Layout().to_c()), BK_F32, 0)
    assert st == _abi.BK_ERR_ARG
    assert b"malformed" in _abi.lib().bk_last_error()


def _oracle_steps(spec, st, steps, init_cells):
    """The oracle's periodic array steps (FP64) of one domain from its initial cells."""
    n = spec.n
    odom = oracle.Domain(n)
    o = odom.ghost + odom.pad
    a = np.zeros(odom.adims)
    a[o:o + n[0], o:o + n[1], o:o + n[2]] = init_cells
    bb = np.zeros_like(a)
    for _ in range(steps):
        oracle.array_periodic_fill(a, (o,) * 3, n, (8, 8, 8))
        oracle.array_sweep(a, bb, (o,) * 3, tuple(o + x for x in n), st.offsets(), st.coeff)
        a, bb = bb, a
    return a[o:o + n[0], o:o + n[1], o:o + n[2]]


@pytest.mark.parametrize("bdim,fold", [((16, 8, 8), (1, 4, 8)), ((8, 8, 32), (1, 1, 32)), ((8, 8, 32), (1, 4, 8))],
                         ids=["16x8x8", "8x8x32", "8x8x32f48"])
@pytest.mark.parametrize("arena", [True, False])
def test_partial_brick_domains_match_the_oracle(bdim, fold, arena):
    """Domains whose edges are not whole bricks (here multiples of 8 on 16- or 32-wide bricks):
    padded to whole bricks, periodic through the cell-level wrap fill.  Every domain's cells
    after 5 FP64 steps equal the oracle's periodic array steps at 1e-12 (mixed test), in arena
    and per-storage batches, with the segments as parallel branches and one after another."""
    w = BT.Workload([BT.DomainSpec((24, 40, 16), 0, 11), BT.DomainSpec((40, 24, 56), 1, 12),
                     BT.DomainSpec((56, 16, 24), 2, 13), BT.DomainSpec((32, 32, 40), 3, 14),
                     BT.DomainSpec((16, 16, 32), 0, 15)],
                    [stencils.make(s, 21) for s in BT.BATCH_SHAPES])
    lay = B.Layout(bdim, fold)
    assert BT.layout_valid(w, lay)
    steps = 5
    for conc in (1, 0):
        b = BT.Batch(w, lay, BK_F64, arena=arena)
        assert sum(ds.partial for ds in b.doms) >= 3
        init = [ds.cells(0).copy() for ds in b.doms]
        _abi_call("bk_batch_set_concurrent", b.h, conc)
        b.run(steps, use_graph=bool(conc))
        B.synchronize()
        assert B.error_flags() == 0
        for d, (spec, ds) in enumerate(zip(w.domains, b.doms)):
            got = ds.cells(b.parity)
            want = _oracle_steps(spec, w.stencils[spec.stencil], steps, init[d])
            diff = np.abs(got - want)
            ok = (diff < 1e-12) | (diff < (np.abs(got) + np.abs(want)) * 1e-12)
            assert ok.all(), (d, conc, float(diff.max()))
        b.close()


def test_partial_brick_fp32_batch_within_1e5_of_fp64():
    """The FP32 batch of partial-brick domains against the FP64 batch: normwise 1e-5 per domain."""
    w = BT.make_workload(ndom=12, seed=5, lo=16, hi=64, multiple=8)
    lay = B.Layout((16, 8, 8), (1, 4, 8))
    b32, b64 = BT.Batch(w, lay, BK_F32), BT.Batch(w, lay, BK_F64)
    b32.run(10)
    b64.run(10)
    B.synchronize()
    for d32, d64 in zip(b32.doms, b64.doms):
        a, r = d32.cells(b32.parity).astype(np.float64), d64.cells(b64.parity)
        assert np.abs(a - r).max() <= 1e-5 * np.abs(r).max()
    b32.close()
    b64.close()


def _abi_call(name, *args):
    from bricklib_gb300._abi import call
    call(name, *args)
