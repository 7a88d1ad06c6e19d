"""Generate the golden fixtures in this directory from bricklib's own CPU brick
path (oracle/_ref/libbrickref.so, compiled from the reference sources by
`make -C oracle ref`).  Run from the repository root:

    python tests/golden/make_golden.py

Fixtures written:
  layouts.npz       in-brick element offsets computed by the reference accessor
                    (include/brick.h:213-327) for seven brick-dims / vector-fold pairs
  init_grid.npz     grid and adjacency of init_grid<3> (include/bricksetup.h:73-90) on 5x4x3
  layouts4.npz      4-D in-brick offsets of Brick<Dim<4,4,4,4>, Dim<fold>> for the folds of
                    weak/main-4d.cpp:33-52: (2,4), (2,2), (1)
  init_grid4.npz    grid and adjacency of init_grid<4> on 5x4x3x2
  sweep4_<name>.npz one 4-D sweep on an 8^4 interior (ghost 8, padding 4, weak/main-4d.cpp):
                    mpi9pt (stencils/mpi9pt.py, alpha 0.2 / beta 0.1) with fold (2,4) and fold (1),
                    and a 9-point star with seeded coefficients; input uniform[-1,1) seed 1234
  decomp_<case>.npz the reference's BrickDecomp layouts (grid, adjacency, g_region records, skin
                    sizes) for the cases of DECOMP_CASES; decomp_skin_lists.npz its skin orders
                    and allneighbors order (`--decomp` writes only these)
  sweep_<shape>.npz one sweep on a 16^3 interior (sweep_cond7: the reference's cond kernel,
                    |sum coeff * max(x, 0)|, stencils/3axis.cpp:94-163) (+8 ghost, +8 padding) through
                    copyToBrick -> accessor brick kernel -> compareBrick -> copyFromBrick,
                    input uniform[-1,1) from splitmix64 seed 1234: the interior output,
                    the max |brick - array| difference and the reference's compareBrick verdict
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import oracle  # noqa: E402
from bricklib_gb300 import stencils  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))

LAYOUTS = {  # id: (bdim k,j,i ; fold k,j,i)
    0: ((8, 8, 8), (1, 4, 8)),
    1: ((8, 8, 8), (1, 1, 8)),
    2: ((8, 8, 8), (1, 2, 2)),
    3: ((8, 8, 8), (2, 4, 4)),
    4: ((4, 4, 4), (1, 4, 4)),
    5: ((16, 8, 8), (1, 4, 8)),
    6: ((8, 8, 32), (1, 4, 8)),
}

N = 16
SEED_IN = 1234
SEED_COEFF = 99


def main():
    oracle.build()
    R = oracle.ref()
    if R is None:
        raise SystemExit("reference checker not built (needs the reference tree)")

    lay = {}
    for lid, (bdim, fold) in LAYOUTS.items():
        out = np.zeros(int(np.prod(bdim)), dtype=np.int64)
        assert R.ref_layout_offsets(lid, out) == 0
        lay[f"offsets_{lid}"] = out
        lay[f"bdim_{lid}"] = np.asarray(bdim)
        lay[f"fold_{lid}"] = np.asarray(fold)
    np.savez(os.path.join(OUT, "layouts.npz"), **lay)

    gk, gj, gi = 3, 4, 5
    grid = np.zeros(gk * gj * gi, dtype=np.uint32)
    adj = np.zeros(gk * gj * gi * 27, dtype=np.uint32)
    R.ref_init_grid(gk, gj, gi, grid, adj)
    np.savez(os.path.join(OUT, "init_grid.npz"), grid=grid, adj=adj, dims=np.asarray([gk, gj, gi]))

    S = N + 32
    inp = stencils.uniform(SEED_IN, S * S * S)
    cases = [(name, 0) for name in stencils.PLAIN_SHAPES] + [("heat7", 0), ("lap7", 0), ("star7", 4)]
    for name, lid in cases:
        st = stencils.make(name, SEED_COEFF)
        offs = st.offsets().reshape(-1).astype(np.int32)
        ob = np.zeros(S * S * S)
        oa = np.zeros(S * S * S)
        ok = R.ref_sweep(lid, N, inp, st.npoints, offs, st.coeff, ob, oa)
        assert ok in (0, 1)
        ob = ob.reshape(S, S, S)[16:16 + N, 16:16 + N, 16:16 + N].copy()
        oa = oa.reshape(S, S, S)[16:16 + N, 16:16 + N, 16:16 + N].copy()
        tag = name if lid == 0 else f"{name}_layout{lid}"
        np.savez(os.path.join(OUT, f"sweep_{tag}.npz"), out=ob, arr_maxdiff=np.max(np.abs(ob - oa)),
                 ref_match=ok, n=N, seed_in=SEED_IN, seed_coeff=SEED_COEFF, layout=lid,
                 offsets=st.offsets(), coeff=st.coeff, input_sum=inp.sum())
        print(f"{tag:22s} compareBrick={ok} max|brick-array|={np.max(np.abs(ob - oa)):.3e}")

    # the cond kernel (3axis.cpp:94-163): coeff[0..6] as the reference indexes them
    coeff = stencils.uniform01(SEED_COEFF, 7)
    ob = np.zeros(S * S * S)
    oa = np.zeros(S * S * S)
    ok = R.ref_cond(N, inp, coeff, ob, oa)
    ob = ob.reshape(S, S, S)[16:16 + N, 16:16 + N, 16:16 + N].copy()
    oa = oa.reshape(S, S, S)[16:16 + N, 16:16 + N, 16:16 + N].copy()
    st = stencils.make("cond7", SEED_COEFF)
    np.savez(os.path.join(OUT, "sweep_cond7.npz"), out=ob, arr_maxdiff=np.max(np.abs(ob - oa)),
             ref_match=ok, n=N, seed_in=SEED_IN, seed_coeff=SEED_COEFF, layout=0,
             offsets=st.offsets(), coeff=st.coeff, input_sum=inp.sum(), pre_op=1, post_op=2)
    print(f"{'cond7':22s} compareBrick={ok} max|brick-array|={np.max(np.abs(ob - oa)):.3e}")

    # ---------------------------------------------------------------- 4-D
    lay4 = {}
    for fid, fold in ((0, (2, 4)), (1, (2, 2)), (2, (1,))):
        out = np.zeros(256, dtype=np.int64)
        assert R.ref_layout_offsets4(fid, out) == 0
        lay4[f"offsets_{fid}"] = out
        lay4[f"fold_{fid}"] = np.asarray(fold)
    np.savez(os.path.join(OUT, "layouts4.npz"), **lay4)
    dl, dk, dj, di = 2, 3, 4, 5
    grid = np.zeros(dl * dk * dj * di, dtype=np.uint32)
    adj = np.zeros(dl * dk * dj * di * 81, dtype=np.uint32)
    R.ref_init_grid4(dl, dk, dj, di, grid, adj)
    np.savez(os.path.join(OUT, "init_grid4.npz"), grid=grid, adj=adj, dims=np.asarray([dl, dk, dj, di]))
    n4 = 8
    S4 = n4 + 24
    inp4 = stencils.uniform(SEED_IN, S4 ** 4)
    taps9 = [(0, 0, 0, 0), (0, 0, 0, 1), (0, 0, 0, -1), (0, 0, 1, 0), (0, 0, -1, 0), (0, 1, 0, 0), (0, -1, 0, 0),
             (1, 0, 0, 0), (-1, 0, 0, 0)]  # mpi9pt.py order, (dl, dk, dj, di)
    cases4 = [("mpi9pt", 0, np.array([0.2] + [0.1] * 8)), ("mpi9pt_fold1", 2, np.array([0.2] + [0.1] * 8)),
              ("star9", 0, stencils.uniform01(SEED_COEFF, 9))]
    for name, fid, c9 in cases4:
        offs = np.asarray(taps9, dtype=np.int32).reshape(-1)
        ob = np.zeros(S4 ** 4)
        oa = np.zeros(S4 ** 4)
        ok = R.ref_sweep4(fid, n4, inp4, 9, offs, c9, ob, oa)
        sl = (slice(12, 12 + n4),) * 4
        ob = ob.reshape((S4,) * 4)[sl].copy()
        oa = oa.reshape((S4,) * 4)[sl].copy()
        np.savez(os.path.join(OUT, f"sweep4_{name}.npz"), out=ob, arr_maxdiff=np.max(np.abs(ob - oa)), ref_match=ok,
                 n=n4, seed_in=SEED_IN, fold=fid, offsets=np.asarray(taps9), coeff=c9)
        print(f"{'4d ' + name:22s} compareBrick={ok} max|brick-array|={np.max(np.abs(ob - oa)):.3e}")


# BrickDecomp cases: (name, bcase of ref_decomp, dims contiguous first, brick dims, depth,
# numfield, element bytes, page bytes, skin list); bcase 0 <3,8,8,8>, 1 <3,4,4,4>, 2 <2,8,8>,
# 3 <4,4,4,4,4>.  Skin lists: "good" / "normal" are the reference's skin3d_good / skin3d_normal,
# "all" its allneighbors order without the empty region.
DECOMP_CASES = [
    ("good_f1", 0, (32, 32, 32), (8, 8, 8), 8, 1, 8, 4096, "good"),
    ("good_f2_aniso", 0, (32, 24, 40), (8, 8, 8), 8, 2, 8, 4096, "good"),
    ("good_e4_padded", 0, (32, 32, 32), (8, 8, 8), 8, 1, 4, 4096, "good"),
    ("normal_e2_ghost2", 0, (48, 32, 32), (8, 8, 8), 16, 1, 2, 4096, "normal"),
    ("good_unpadded", 0, (32, 32, 32), (8, 8, 8), 8, 1, 8, 1, "good"),
    ("good_unpadded_f2", 0, (40, 32, 24), (8, 8, 8), 8, 2, 8, 1, "good"),
    ("good_b4", 1, (16, 16, 16), (4, 4, 4), 4, 1, 8, 4096, "good"),
    ("all2d", 2, (32, 32), (8, 8), 8, 1, 8, 4096, "all"),
    ("all4d", 3, (16, 16, 16, 16), (4, 4, 4, 4), 8, 1, 8, 4096, "all"),
]


def decomp_main():
    """decomp_<name>.npz: the reference's own BrickDecomp<dim, bdim>(dims, depth, numfield)
    .initialize(skin) (include/brick-mpi.h:298-464, oracle/ref_decomp.cpp): nbricks, sep_pos,
    the grid (position -> brick, dimension 0 fastest), the adjacency, the ghost and skin g_region
    records (7 int64 each) and the skin sizes; plus the skin lists it was given."""
    oracle.build()
    R = oracle.ref()
    if R is None:
        raise SystemExit("reference checker not built (needs the reference tree)")
    lists = {}
    for which, key in ((0, "good"), (1, "normal")):
        n = R.ref_skin_list(which, None)
        a = np.zeros(n, np.uint64)
        R.ref_skin_list(which, a.ctypes.data)
        lists[key] = a
    for dim in (2, 3, 4):
        n = R.ref_allneighbors(dim, None)
        a = np.zeros(n, np.uint64)
        R.ref_allneighbors(dim, a.ctypes.data)
        lists[f"neighbors{dim}"] = a
    np.savez(os.path.join(OUT, "decomp_skin_lists.npz"), **lists)
    for name, bcase, dims, bdim, depth, nf, eb, page, skin in DECOMP_CASES:
        dim = len(dims)
        sk = lists[skin] if skin != "all" else lists[f"neighbors{dim}"]
        sk = np.ascontiguousarray(sk[sk != 0] if skin == "all" else sk, np.uint64)
        dv = np.asarray(dims, np.uint32)
        info = np.zeros(6, np.int64)
        assert R.ref_decomp(bcase, dv, depth, nf, eb, page, sk, len(sk), info, None, None, None, None) == 0
        nb, gsize, nreg = int(info[0]), int(info[4]), int(info[5])
        grid = np.zeros(gsize, np.uint32)
        adj = np.zeros(nb * 3 ** dim, np.uint32)
        regions = np.zeros(2 * nreg * 7, np.int64)
        skin_size = np.zeros(len(sk), np.int64)
        assert R.ref_decomp(bcase, dv, depth, nf, eb, page, sk, len(sk), info, grid.ctypes.data, adj.ctypes.data,
                            regions.ctypes.data, skin_size.ctypes.data) == 0
        # initialize writes the adjacency rows of the bricks the grid holds (brick-mpi.h:460-463);
        # rows of reserved and page-padding bricks stay as allocated (uninitialised): recorded as 0
        adj = adj.reshape(nb, 3 ** dim)
        unused = np.setdiff1d(np.arange(nb), grid)
        adj[unused] = 0
        np.savez_compressed(os.path.join(OUT, f"decomp_{name}.npz"), dims=dv, bdim=np.asarray(bdim), depth=depth,
                            numfield=nf, elem_bytes=eb, pagesize=page, skinlist=sk, nbricks=nb,
                            sep_pos=info[1:4].copy(), grid=grid, adj=adj, unused=unused,
                            ghost=regions[:7 * nreg].reshape(nreg, 7), skin=regions[7 * nreg:].reshape(nreg, 7),
                            skin_size=skin_size)
        print(f"decomp {name:18s} nbricks={nb} sep_pos={info[1:4].tolist()} regions={nreg}")


if __name__ == "__main__":
    if "--decomp" not in sys.argv:
        main()
    decomp_main()
