"""Test infrastructure (the oracle): a plain-Python restatement of the reference's
BrickDecomp layout producer, include/brick-mpi.h:178-464 (with allneighbors of
src/brick-mpi.cpp:9-23), used to check bk_decomp_* on small decompositions.

Parity unpinned against the reference binary: the reference's BrickDecomp lives in a header
that needs MPI, which this machine does not have; the restatement follows the source and is
checked relationally by the tests (the reference's own adjacency-symmetry check of
single/mpi.cpp:80-87, grid consistency, and the exchange as a periodic wrap).
"""
from __future__ import annotations

from typing import Dict, List, Sequence


def _bit(p: int) -> int:  # bitset.h:22-26
    return 1 << (p if p >= 0 else 31 - p)


def _has(s: int, p: int) -> bool:
    return bool(s & _bit(p))


def _flip(s: int) -> int:  # bitset.h operator!
    mask = (1 << 32) - 1
    return ((s & mask) << 31) | (s >> 31)


def _neighbours(dim: int) -> List[int]:  # brick-mpi.cpp:9-23
    out: List[int] = []

    def rec(cur, idx):
        if idx > dim:
            out.append(cur)
            return
        rec(cur ^ _bit(idx), idx + 1)
        rec(cur, idx + 1)
        rec(cur ^ _bit(-idx), idx + 1)

    rec(0, 1)
    return out


def decompose(dims_el: Sequence[int], bdim: Sequence[int], depth: int, numfield: int, elem_bytes: int,
              pagesize: int, skinlist: Sequence[int]) -> Dict:
    dim = len(dims_el)
    dims = [x // b for x, b in zip(dims_el, bdim)]              # brick-mpi.h:298-310
    g = [depth // b for b in bdim]
    t_dims = [dims[d] + 2 * g[d] for d in range(dim)]           # brick-mpi.h:326-337
    stride = []
    size = 1
    for d in range(dim):
        stride.append(size)
        size *= t_dims[d]
    grid = [0] * size
    bsize = elem_bytes * numfield
    for b in bdim:
        bsize *= b
    factor = pagesize // bsize if bsize < pagesize else 1       # brick-mpi.h:344-352
    pos = [factor]

    def region_size(r):                                         # brick-mpi.h:252-260
        n = 1
        for d in range(dim):
            n *= g[d] if (_has(r, d + 1) or _has(r, -d - 1)) else dims[d] - 2 * g[d]
        return n

    def calc_pad(r):                                            # brick-mpi.h:364-370
        return factor - (region_size(r) + factor - 1) % factor - 1

    def _populate(region, ref, d):                              # brick-mpi.h:220-238
        if d == -1:
            grid[ref] = pos[0]
            pos[0] += 1
            return
        sec, st = 0, 0
        if _has(region, d + 1):
            sec, st = 1, dims[d]
        if _has(region, -d - 1):
            sec, st = -1, g[d]
        if sec != 0:
            for i in range(g[d]):
                _populate(region, ref + (st + i) * stride[d], d - 1)
        else:
            for i in range(2 * g[d], dims[d]):
                _populate(region, ref + i * stride[d], d - 1)

    def mypop(owner, region):                                   # brick-mpi.h:240-250, 356-362
        ref = 0
        for d in range(dim):
            if _has(owner, d + 1):
                ref += dims[d] * stride[d]
            if _has(owner, -d - 1):
                ref -= dims[d] * stride[d]
        _populate(region, ref, dim - 1)
        pos[0] = (pos[0] + factor - 1) // factor * factor

    ns = len(skinlist)
    pad_first = []
    last = 0
    for i in range(ns):                                         # brick-mpi.h:375-382
        nxt = skinlist[i + 1] if i < ns - 1 else 0
        pad_first.append(bin(last & skinlist[i]).count("1") < bin(skinlist[i] & nxt).count("1"))
        last = skinlist[i]
    st_pos = []
    mypop(0, 0)                                                 # brick-mpi.h:384-388
    st_pos.append(pos[0])
    sep = [pos[0], 0, 0]
    skin_size = []
    for i in range(ns):                                         # brick-mpi.h:390-400
        ppos = pos[0]
        if pad_first[i]:
            pos[0] += calc_pad(skinlist[i])
        if skinlist[i] != 0:
            mypop(0, skinlist[i])
        st_pos.append(pos[0])
        skin_size.append(pos[0] - ppos)
    sep[1] = pos[0]
    ghost, skin = [], []
    for n in _neighbours(dim):                                  # brick-mpi.h:402-450
        if n == 0:
            continue
        inv = _flip(n)
        gr = {"neighbor": n}
        sr = {"neighbor": inv}
        lst = -1
        for l in range(ns):
            if (inv & skinlist[l]) == inv:
                if lst < 0:
                    lst = l
                    gr["skin_st"] = sr["skin_st"] = l
                    gr["first_pad"] = sr["first_pad"] = calc_pad(skinlist[l]) if pad_first[l] else 0
                    gr["pos"] = pos[0]
                    sr["pos"] = st_pos[l]
                if pad_first[l]:
                    pos[0] += calc_pad(skinlist[l])
                mypop(n, skinlist[l])
            elif lst >= 0:
                lst = l
                gr["last_pad"] = sr["last_pad"] = 0 if pad_first[lst - 1] else calc_pad(skinlist[lst - 1])
                gr["skin_ed"] = lst
                gr["len"] = pos[0] - gr["pos"]
                ghost.append(dict(gr))
                sr["len"] = st_pos[lst] - sr["pos"]
                sr["skin_ed"] = lst
                skin.append(dict(sr))
                lst = -1
        if lst >= 0:
            lst = ns
            gr["last_pad"] = sr["last_pad"] = 0 if pad_first[lst - 1] else calc_pad(skinlist[lst - 1])
            gr["skin_ed"] = lst
            gr["len"] = pos[0] - gr["pos"]
            ghost.append(dict(gr))
            sr["len"] = st_pos[ns] - sr["pos"]
            sr["skin_ed"] = lst
            skin.append(dict(sr))
    sep[2] = pos[0]
    nb = pos[0]
    w = 3 ** dim
    adj = [[0] * w for _ in range(nb)]

    def _adj(ref, d, idx, out):                                 # brick-mpi.h:262-286
        cur = ref
        if cur >= 0:
            cur = (ref // stride[d]) % t_dims[d]
        idx *= 3
        for i in range(3):
            outside = i + cur < 1 or i + cur > t_dims[d] or ref < 0
            if d == 0:
                out[idx + i] = 0 if outside else grid[ref + i - 1]
            else:
                _adj(-1 if outside else ref + (i - 1) * stride[d], d - 1, idx + i, out)

    for i in range(size):                                       # brick-mpi.h:458-463
        _adj(i, dim - 1, 0, adj[grid[i]])
    return {"grid": grid, "adj": adj, "ghost": ghost, "skin": skin, "sep_pos": sep, "skin_size": skin_size,
            "nbricks": nb, "t_dims": t_dims, "stride": stride, "factor": factor}
