"""4-D bricks (weak/main-4d.cpp) on the host: layouts and init_grid<4> against the reference's
own accessor and init_grid (golden vectors), the copies, and the 4-D array oracle against the
reference's 4-D brick kernel."""
import os

import numpy as np
import pytest

from bricklib_gb300 import bricks4 as B4, stencils
from oracle import array4

GOLD = os.path.join(os.path.dirname(__file__), "golden")
FOLDS = {0: (1, 1, 2, 4), 1: (1, 1, 2, 2), 2: (1, 1, 1, 1)}


@pytest.mark.parametrize("fid", [0, 1, 2])
def test_layout4_matches_reference_accessor(fid):
    z = np.load(os.path.join(GOLD, "layouts4.npz"))
    np.testing.assert_array_equal(B4.Layout4(fold=FOLDS[fid]).offsets(), z[f"offsets_{fid}"])


def test_init_grid4_matches_reference():
    z = np.load(os.path.join(GOLD, "init_grid4.npz"))
    dl, dk, dj, di = (int(x) for x in z["dims"])
    grid, adj = B4.init_grid([di, dj, dk, dl])
    np.testing.assert_array_equal(grid, z["grid"])
    np.testing.assert_array_equal(adj.reshape(-1), z["adj"])


def test_copies_round_trip():
    lay = B4.Layout4()
    g = (3, 2, 4, 2)
    grid, _ = B4.init_grid(list(reversed(g)))
    arr = np.random.default_rng(1).random(tuple(x * 4 + 6 for x in g))
    store = np.zeros(len(grid) * 512)
    B4.copy_to_bricks(arr, grid, g, (3, 3, 3, 3), store, 512, 256, lay)
    back = np.zeros_like(arr)
    B4.copy_from_bricks(back, grid, g, (3, 3, 3, 3), store, 512, 256, lay)
    sl = tuple(slice(3, 3 + x * 4) for x in g)
    np.testing.assert_array_equal(back[sl], arr[sl])
    assert np.all(store.reshape(-1, 512)[:, :256] == 0)


@pytest.mark.parametrize("name", ["mpi9pt", "mpi9pt_fold1", "star9"])
def test_array_oracle4_matches_reference_brick_kernel(name):
    """The reference's 4-D accessor brick kernel equals its array kernel bit for bit; the
    numpy array oracle reproduces that output."""
    z = np.load(os.path.join(GOLD, f"sweep4_{name}.npz"))
    assert int(z["ref_match"]) == 1 and float(z["arr_maxdiff"]) == 0.0
    n = int(z["n"])
    S = n + 24
    arr = stencils.uniform(int(z["seed_in"]), S ** 4).reshape((S,) * 4)
    got = array4.array_sweep4(arr, [tuple(t) for t in z["offsets"]], z["coeff"], (12,) * 4, (n,) * 4)
    np.testing.assert_array_equal(got, z["out"])
