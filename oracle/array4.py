"""Test infrastructure (the oracle): the plain 4-D array stencil -- the array kernel of
weak/main-4d.cpp (its ST_CPU form of stencils/mpi9pt.py) on a runtime tap list -- and the
periodic wrap of a 4-D array.  Used by the tests to check bk_sweep4; pinned by the golden
vectors of the reference's 4-D brick path (tests/golden/sweep4_*.npz)."""
from __future__ import annotations

from typing import Sequence

import numpy as np


def array_sweep4(arr: np.ndarray, taps: Sequence, coeff: Sequence[float], org: Sequence[int],
                 n: Sequence[int]) -> np.ndarray:
    """out[x] = sum_t c_t * arr[org + x + tap_t] over x in [0, n), taps (dl, dk, dj, di), summed in
    tap order with separate multiply and add (the reference's array loop)."""
    out = None
    for (dl, dk, dj, di), c in zip(taps, coeff):
        term = c * arr[org[0] + dl:org[0] + dl + n[0], org[1] + dk:org[1] + dk + n[1],
                       org[2] + dj:org[2] + dj + n[2], org[3] + di:org[3] + di + n[3]]
        out = term if out is None else out + term
    return out


def periodic_fill4(arr: np.ndarray, org: Sequence[int], n: Sequence[int], ghost: int) -> None:
    """Ghost cells (ghost wide on each side of arr[org : org + n]) <- their periodic images."""
    for d in range(4):
        lo, hi = org[d], org[d] + n[d]
        src_hi = [slice(None)] * 4
        dst_lo = [slice(None)] * 4
        src_hi[d], dst_lo[d] = slice(hi - ghost, hi), slice(lo - ghost, lo)
        arr[tuple(dst_lo)] = arr[tuple(src_hi)]
        src_lo = [slice(None)] * 4
        dst_hi = [slice(None)] * 4
        src_lo[d], dst_hi[d] = slice(lo, lo + ghost), slice(hi, hi + ghost)
        arr[tuple(dst_hi)] = arr[tuple(src_lo)]
