"""BrickDecomp layout producer (bk_decomp_*): equal to the oracle's restatement of
include/brick-mpi.h:178-464, plus the reference's own relational checks -- adjacency symmetry
(single/mpi.cpp:80-87) and grid consistency -- and the exchange as a periodic wrap."""
import glob
import os

import numpy as np
import pytest

from bricklib_gb300 import _abi, decomp as D
from oracle import decomp_oracle as O

CASES = [
    # dims (contiguous first), bdim, depth, numfield, elem bytes, page size, skin list
    ((32, 32, 32), (8, 8, 8), 8, 1, 8, 4096, D.SKIN3D_GOOD),
    ((32, 24, 40), (8, 8, 8), 8, 2, 8, 4096, D.SKIN3D_GOOD),
    ((32, 32, 32), (8, 8, 8), 8, 1, 4, 4096, D.SKIN3D_GOOD),      # 2 KB bricks: page padding
    ((48, 32, 32), (8, 8, 8), 16, 1, 2, 4096, D.SKIN3D_NORMAL),   # 1 KB bricks, 2-brick ghost
    ((32, 32, 32), (8, 8, 8), 8, 1, 8, 1, D.SKIN3D_GOOD),         # unpadded layout
    ((16, 16, 16), (4, 4, 4), 4, 1, 8, 4096, D.SKIN3D_GOOD),
    ((32, 32), (8, 8), 8, 1, 8, 4096, D.all_regions(2)),
    ((16, 16, 16, 16), (4, 4, 4, 4), 8, 1, 8, 4096, D.all_regions(4)),  # weak/main-4d.cpp shapes
]


GOLD = os.path.join(os.path.dirname(__file__), "golden")
REF_CASES = sorted(glob.glob(os.path.join(GOLD, "decomp_*.npz")))
REF_CASES = [p for p in REF_CASES if not p.endswith("skin_lists.npz")]


def test_skin_orders_are_the_references():
    """SKIN3D_GOOD / SKIN3D_NORMAL and the neighbour enumeration equal the reference's own
    (src/brick-mpi.cpp:9-112, dumped by the reference build)."""
    z = np.load(os.path.join(GOLD, "decomp_skin_lists.npz"))
    assert [int(x) for x in z["good"]] == D.SKIN3D_GOOD
    assert [int(x) for x in z["normal"]] == D.SKIN3D_NORMAL
    for dim in (2, 3, 4):
        assert [int(x) for x in z[f"neighbors{dim}"] if x] == D.all_regions(dim)


@pytest.mark.parametrize("path", REF_CASES, ids=lambda p: os.path.basename(p)[7:-4])
def test_layout_equals_the_references_own_brickdecomp(path):
    """bk_decomp_* against BrickDecomp::initialize of the reference itself (brick-mpi.h:322-464,
    compiled into the reference checker): every field bit for bit."""
    z = np.load(path)
    dt = {8: _abi.BK_F64, 4: _abi.BK_F32, 2: _abi.BK_BF16}[int(z["elem_bytes"])]
    d = D.BrickDecomp([int(x) for x in z["dims"]], int(z["depth"]), [int(x) for x in z["bdim"]], int(z["numfield"]),
                      dt, int(z["pagesize"]))
    d.initialize([int(x) for x in z["skinlist"]])
    assert d.nbricks == int(z["nbricks"])
    assert d.sep_pos == [int(x) for x in z["sep_pos"]]
    assert d.skin_size == [int(x) for x in z["skin_size"]]
    np.testing.assert_array_equal(d.grid, z["grid"])
    # the reference writes the rows of the bricks its grid holds; reserved and padding bricks'
    # rows are uninitialised there (recorded as 0) and all-zero here
    used = np.setdiff1d(np.arange(d.nbricks), z["unused"])
    np.testing.assert_array_equal(d.adj[used], z["adj"][used])
    assert not d.adj[z["unused"]].any()
    keys = ["neighbor", "skin_st", "skin_ed", "pos", "len", "first_pad", "last_pad"]
    for mine, ref in ((d.ghost, z["ghost"]), (d.skin, z["skin"])):
        assert [[int(r[k]) for k in keys] for r in mine] == ref.tolist()
    d.close()


def _dec(case):
    dims, bdim, depth, nf, eb, page, skin = case
    dt = {8: _abi.BK_F64, 4: _abi.BK_F32, 2: _abi.BK_BF16}[eb]
    d = D.BrickDecomp(dims, depth, bdim, nf, dt, page)
    d.initialize(skin)
    return d


@pytest.mark.parametrize("case", CASES, ids=lambda c: "x".join(map(str, c[0])) + f"-p{c[5]}-e{c[4]}-f{c[3]}")
def test_layout_equals_oracle(case):
    dims, bdim, depth, nf, eb, page, skin = case
    d = _dec(case)
    want = O.decompose(dims, bdim, depth, nf, eb, page, skin)
    assert d.nbricks == want["nbricks"]
    assert d.sep_pos == want["sep_pos"]
    assert d.skin_size == want["skin_size"]
    np.testing.assert_array_equal(d.grid, np.asarray(want["grid"], np.uint32))
    np.testing.assert_array_equal(d.adj, np.asarray(want["adj"], np.uint32))
    assert d.ghost == want["ghost"] and d.skin == want["skin"]


@pytest.mark.parametrize("case", CASES[:6], ids=lambda c: "x".join(map(str, c[0])) + f"-p{c[5]}-e{c[4]}")
def test_adjacency_symmetry_and_grid_consistency(case):
    d = _dec(case)
    n = d.dim
    w = 3 ** n
    t = d.t_dims
    pos = np.indices(tuple(reversed(t))).reshape(n, -1)[::-1]  # coordinates, dimension 0 first
    flat = sum(pos[q] * d.stride[q] for q in range(n))
    # every grid position holds a distinct brick, none of them the reserved bricks
    assert len(set(d.grid.tolist())) == d.grid.size and d.grid.min() >= 1
    for s in range(w):
        off = [(s // 3 ** q) % 3 - 1 for q in range(n)]
        c = [pos[q] + off[q] for q in range(n)]
        inside = np.all([(c[q] >= 0) & (c[q] < t[q]) for q in range(n)], axis=0)
        nbr = np.where(inside, d.grid[np.where(inside, flat + sum(off[q] * d.stride[q] for q in range(n)), 0)], 0)
        np.testing.assert_array_equal(d.adj[d.grid[flat], s], nbr)
    # the reference's check: adj[adj[l][id]][w-1-id] == l away from the grid's outer layer
    core = np.all([(pos[q] >= 1) & (pos[q] < t[q] - 1) for q in range(n)], axis=0)
    for l in d.grid[flat[core]]:
        assert all(d.adj[d.adj[l, s], w - 1 - s] == l for s in range(w))


@pytest.mark.parametrize("case", CASES, ids=lambda c: "x".join(map(str, c[0])) + f"-p{c[5]}-e{c[4]}-f{c[3]}")
def test_exchange_is_the_periodic_wrap(case):
    """Apply the exchange links on a host storage in which every brick holds its grid
    position: afterwards every ghost position holds its periodic image's position."""
    d = _dec(case)
    n = d.dim
    t, g = d.t_dims, [d.depth // b for b in d.bdim]
    inner = [x // b for x, b in zip(d.dims_el, d.bdim)]
    step = 4  # elements of 8 bytes per brick in this emulation
    store = np.full(d.nbricks * step, -1, np.int64)
    pos = np.indices(tuple(reversed(t))).reshape(n, -1)[::-1]
    flat = sum(pos[q] * d.stride[q] for q in range(n))
    interior = np.all([(pos[q] >= g[q]) & (pos[q] < g[q] + inner[q]) for q in range(n)], axis=0)
    for f, b in zip(flat[interior], d.grid[flat[interior]]):
        store[b * step:(b + 1) * step] = f
    base = 1 << 20  # a stand-in storage address; links are offsets from it
    links = d.exchange_links(base, step * 8)
    assert len(links) == d.nregions
    raw = store.view(np.uint8)
    for frm, to, nbytes in links.tolist():
        frm, to = frm - base, to - base
        raw[to:to + nbytes] = raw[frm:frm + nbytes].copy()
    wrapped = sum(((pos[q] - g[q]) % inner[q] + g[q]) * d.stride[q] for q in range(n))
    got = store.reshape(d.nbricks, step)[d.grid[flat], 0]
    np.testing.assert_array_equal(got, wrapped)


def test_bad_arguments_are_reported():
    with pytest.raises(_abi.BkError):
        D.BrickDecomp((30, 32, 32), 8).initialize(D.SKIN3D_GOOD)  # not whole bricks
    with pytest.raises(_abi.BkError):
        D.BrickDecomp((8, 32, 32), 8).initialize(D.SKIN3D_GOOD)  # narrower than two ghost depths
    with pytest.raises(_abi.BkError):
        D.BrickDecomp((32, 32, 32), 8).initialize([D.bitset([1, -1])])  # both sides of one dimension
