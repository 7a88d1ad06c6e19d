"""The CPU oracle against the golden vectors made by bricklib's own CPU brick
path (tests/golden/make_golden.py), plus relational checks of the parts the
reference has no single-node code for (periodic ghost fill)."""
import glob
import os

import numpy as np
import pytest

from oracle import oracle
from bricklib_gb300 import stencils

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def test_uniform_stream_matches_c():
    a = oracle.fill_uniform(1000, 77)
    b = stencils.uniform(77, 1000)
    np.testing.assert_array_equal(a, b)


def test_layout_offsets_match_reference_accessor():
    z = np.load(os.path.join(GOLD, "layouts.npz"))
    for lid in range(7):
        bdim, fold = tuple(z[f"bdim_{lid}"]), tuple(z[f"fold_{lid}"])
        want = z[f"offsets_{lid}"]
        got = np.array([oracle.brick_offset(bdim, fold, k, j, i)
                        for k in range(bdim[0]) for j in range(bdim[1]) for i in range(bdim[2])])
        np.testing.assert_array_equal(got, want, err_msg=f"layout {lid}")


def test_init_grid_matches_reference():
    z = np.load(os.path.join(GOLD, "init_grid.npz"))
    grid, adj = oracle.init_grid(*z["dims"])
    np.testing.assert_array_equal(grid, z["grid"])
    np.testing.assert_array_equal(adj, z["adj"])


LAYOUT_OF = {0: ((8, 8, 8), (1, 4, 8)), 4: ((4, 4, 4), (1, 4, 4))}


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLD, "sweep_*.npz"))),
                         ids=lambda p: os.path.basename(p)[6:-4])
def test_brick_sweep_matches_golden(path):
    z = np.load(path)
    n = int(z["n"])
    assert int(z["ref_match"]) == 1 and float(z["arr_maxdiff"]) == 0.0
    bdim, fold = LAYOUT_OF[int(z["layout"])]
    dom = oracle.Domain(n, bdim=bdim, fold=fold)
    inp = stencils.uniform(int(z["seed_in"]), int(np.prod(dom.adims))).reshape(dom.adims)
    assert inp.sum() == float(z["input_sum"])
    dat = dom.alloc()
    dom.to_bricks(inp, dat, 0)
    pre = int(z["pre_op"]) if "pre_op" in z else 0
    post = int(z["post_op"]) if "post_op" in z else 0
    oracle.brick_sweep(dom.adj, dat, dom.step, 0, dat, dom.step, dom.bsize, dom.interior,
                       bdim, fold, z["offsets"], z["coeff"], pre=pre, post=post)
    got = dom.interior_view(dom.from_bricks(dat, dom.bsize))
    # same taps, same order, separately rounded doubles: bit-identical
    np.testing.assert_array_equal(got, z["out"])
    # array oracle over the same interior
    out = np.zeros_like(inp)
    o = dom.ghost + dom.pad
    oracle.array_sweep(inp, out, (o, o, o), (o + n, o + n, o + n), z["offsets"], z["coeff"], pre=pre, post=post)
    np.testing.assert_array_equal(dom.interior_view(out), z["out"])
    bad, maxdiff, _ = dom.compare(out, dat, dom.bsize, 1e-12)
    assert bad == 0 and maxdiff == 0.0


def test_compare_catches_planted_error():
    dom = oracle.Domain(16)
    inp = stencils.uniform(5, int(np.prod(dom.adims))).reshape(dom.adims)
    dat = dom.alloc()
    dom.to_bricks(inp, dat, 0)
    dom.to_bricks(inp, dat, dom.bsize)
    o = dom.ghost + dom.pad
    inp2 = inp.copy()
    inp2[o + 3, o + 5, o + 7] += 1e-9
    bad, maxdiff, _ = dom.compare(inp2, dat, dom.bsize, 1e-12)
    assert bad == 1 and abs(maxdiff - 1e-9) < 1e-15


def test_periodic_plan_equals_array_periodic_fill():
    n = 16
    dom = oracle.Domain(n)
    o = dom.ghost + dom.pad
    arr = stencils.uniform(11, int(np.prod(dom.adims))).reshape(dom.adims)
    dat = dom.alloc()
    dom.to_bricks(arr, dat, 0)
    pairs = oracle.periodic_plan(dom.grid, dom.nb, dom.gb)
    assert len(pairs) == np.prod(dom.gdims) - np.prod(dom.nb)
    oracle.apply_plan(dat, dom.step, 0, dom.bsize, pairs)
    oracle.array_periodic_fill(arr, (o, o, o), (n, n, n), (8, 8, 8))
    # every brick (ghost ones included) now equals the periodically filled array
    g = n + 16
    back = np.zeros_like(arr)
    oracle.copy_brick(False, (g, g, g), (8, 8, 8), (0, 0, 0), back, dom.grid, dat, dom.step, 0,
                      dom.bdim, dom.fold)
    np.testing.assert_array_equal(back[8:8 + g, 8:8 + g, 8:8 + g], arr[8:8 + g, 8:8 + g, 8:8 + g])
