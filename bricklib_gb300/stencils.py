"""Stencil shapes, seeded coefficients and seeded inputs.

A stencil is a list of taps ``(dk, dj, di)`` with one FP64 coefficient each;
``out(k, j, i) = sum_t c_t * in(k + dk_t, j + dj_t, i + di_t)``.  Tap order is
the order of the reference's stencil scripts, which is also the summation order
of the CPU brick path:

* ``star7``   stencils/7pt.py:19-25 (centre, i+1, i-1, j+1, j-1, k+1, k-1; 7 coefficients,
  one per tap, as ``coeff[0..6]`` in stencils/3axis.cpp:58-63)
* ``star13``  stencils/mpi13pt.py:18-31 (centre, then the ring at distance 1 and 2)
* ``star25``  stencils/mpi25pt.py:20-45 (rings 1..4)
* ``cube27``  the 27-point cube of stencils/3axis.cpp:165-247 with one coefficient per tap.
  The reference's hand loop reads (k+1, j+1, i) where (k, j+1, i) is meant
  (3axis.cpp:195,225); this module uses the full cube.
* ``cube125`` stencils/mpi125pt.py:12-164 (10 symmetry classes by sorted |offset|)
* ``heat7``   stencils/mpi7pt.py with MPI_ALPHA = 0.4, MPI_BETA = 0.1 (stencils/fake.h:11-12)

Seeded values use splitmix64, the same stream as the oracle's
``orc_fill_uniform``: value n of seed s is ``splitmix64(s + n) >> 11`` scaled to
[0, 1).
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import List, Sequence, Tuple

import numpy as np

Tap = Tuple[int, int, int]

_MASK = (1 << 64) - 1


def splitmix64(x: np.ndarray) -> np.ndarray:
    x = (x.astype(np.uint64) + np.uint64(0x9E3779B97F4A7C15))
    x = (x ^ (x >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    x = (x ^ (x >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return x ^ (x >> np.uint64(31))


def uniform01(seed: int, n: int, start: int = 0) -> np.ndarray:
    idx = (np.arange(start, start + n, dtype=np.uint64) + np.uint64(seed & _MASK))
    with np.errstate(over="ignore"):
        bits = splitmix64(idx) >> np.uint64(11)
    return bits.astype(np.float64) * (1.0 / 9007199254740992.0)


def uniform(seed: int, n: int, lo: float = -1.0, hi: float = 1.0) -> np.ndarray:
    return lo + (hi - lo) * uniform01(seed, n)


@dataclass
class Stencil:
    """A tap list with FP64 coefficients (the payload of ``bk_stencil``)."""
    name: str
    taps: List[Tap]
    coeff: np.ndarray
    classes: List[int] = field(default_factory=list)  # symmetry class of each tap
    pre_op: int = 0   # 0 none, 1 max(x, 0) on every input value
    post_op: int = 0  # 0 none, 2 |sum|

    @property
    def npoints(self) -> int:
        return len(self.taps)

    @property
    def radius(self) -> int:
        return max(max(abs(a) for a in t) for t in self.taps)

    @property
    def flops_per_point(self) -> int:
        return 2 * self.npoints

    def offsets(self) -> np.ndarray:
        return np.asarray(self.taps, dtype=np.int32).reshape(-1, 3)

    def is_star(self) -> bool:
        return all(sum(1 for a in t if a) <= 1 for t in self.taps)


def star_taps(r: int) -> Tuple[List[Tap], List[int]]:
    taps: List[Tap] = [(0, 0, 0)]
    cls = [0]
    for d in range(1, r + 1):
        taps += [(0, 0, d), (0, 0, -d), (0, d, 0), (0, -d, 0), (d, 0, 0), (-d, 0, 0)]
        cls += [d] * 6
    return taps, cls


def cube_taps(r: int) -> Tuple[List[Tap], List[int]]:
    taps: List[Tap] = []
    rng = range(-r, r + 1)
    for dk in rng:
        for dj in rng:
            for di in rng:
                taps.append((dk, dj, di))
    keys = sorted({tuple(sorted((abs(a) for a in t))) for t in taps})
    cls = [keys.index(tuple(sorted(abs(a) for a in t))) for t in taps]
    return taps, cls


def _normalise(c: np.ndarray) -> np.ndarray:
    return c / c.sum()


def make(name: str, seed: int = 0) -> Stencil:
    """Build one of the named shapes with seeded coefficients normalised to sum 1
    (``heat7`` and ``lap7`` have fixed coefficients)."""
    if name in ("star7", "star13", "star25"):
        r = {"star7": 1, "star13": 2, "star25": 4}[name]
        taps, cls = star_taps(r)
        if name == "star7":  # one coefficient per tap (3axis.cpp coeff[0..6])
            c = uniform01(seed, len(taps))
        else:  # one per ring, as the mpi*pt.py scripts
            ring = uniform01(seed, r + 1)
            c = ring[np.asarray(cls)]
        return Stencil(name, taps, _normalise(c), cls)
    if name == "cube27":
        taps, cls = cube_taps(1)
        return Stencil(name, taps, _normalise(uniform01(seed, len(taps))), list(range(27)))
    if name == "cube125":
        taps, cls = cube_taps(2)
        per_class = uniform01(seed, 10)
        return Stencil(name, taps, _normalise(per_class[np.asarray(cls)]), cls)
    if name == "heat7":  # explicit Jacobi heat step, dt*alpha/h^2 = 0.1
        taps, cls = star_taps(1)
        c = np.array([0.4] + [0.1] * 6)
        return Stencil(name, taps, c, cls)
    if name == "lap7":  # 7-point Laplacian, h = 1/128
        taps, cls = star_taps(1)
        inv_h2 = 128.0 * 128.0
        c = np.array([-6.0 * inv_h2] + [inv_h2] * 6)
        return Stencil(name, taps, c, cls)
    if name == "cond7":  # stencils/cond.py, 3axis.cpp:94-163: |sum c_t * max(x_t, 0)|, 3axis.cpp tap order
        taps = [(1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1), (0, 0, 0)]
        cidx = [5, 6, 3, 4, 1, 2, 0]  # coeff[5] * in(k+1) + coeff[6] * in(k-1) + ...
        c = uniform01(seed, 7)
        return Stencil(name, taps, c[np.asarray(cidx)], list(range(7)), pre_op=1, post_op=2)
    raise ValueError(f"unknown stencil {name!r}")


PLAIN_SHAPES = ("star7", "star13", "star25", "cube27", "cube125")


def custom(name: str, taps: Sequence[Tap], coeff: Sequence[float]) -> Stencil:
    taps = [tuple(int(a) for a in t) for t in taps]
    c = np.asarray(coeff, dtype=np.float64)
    if len(taps) != len(c) or not taps:
        raise ValueError("taps and coefficients must be non-empty and of equal length")
    return Stencil(name, taps, c, list(range(len(taps))))
