"""Grid declarations of the stencil language (st.grid.Grid): grid(i + 1, j, k) is a
reference to the grid at an offset; output(i, j, k).assign(expr) records the computation."""
from __future__ import annotations

from .expr import Expr, Index, IndexOff, as_expr


class Grid:
    def __init__(self, name: str, dims: int):
        self.name, self.dims = name, dims
        self.assigned = None  # (offsets, expression) once assigned

    def __call__(self, *idx):
        if len(idx) != self.dims:
            raise ValueError(f"grid {self.name} has {self.dims} dimensions")
        offs = []
        for a, x in enumerate(idx):
            if isinstance(x, Index):
                n, o = x.n, 0
            elif isinstance(x, IndexOff):
                n, o = x.n, x.off
            else:
                raise ValueError("grid indices must be an Index plus or minus a constant")
            if n != a:
                raise ValueError("grid indices must follow the axis order (i, j, k)")
            offs.append(o)
        return GridRef(self, tuple(offs))


class GridRef(Expr):
    def __init__(self, grid: Grid, offsets):
        self.grid, self.offsets = grid, offsets  # offsets in axis order (i, j, k, ...)

    def assign(self, rhs):
        self.grid.assigned = (self.offsets, as_expr(rhs))
        return self
