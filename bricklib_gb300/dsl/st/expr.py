"""Expression nodes of the stencil language: the names a stencil script imports from
st.expr (Index, ConstRef, If and arithmetic on them).  Nodes only record the expression;
bricklib_gb300.dsl.lower turns an assigned expression into taps and coefficients."""
from __future__ import annotations


def as_expr(x):
    if isinstance(x, Expr):
        return x
    if isinstance(x, (int, float)):
        return Lit(float(x))
    if isinstance(x, str):
        return ConstRef(x)
    raise TypeError(f"cannot use {x!r} in a stencil expression")


class Expr:
    def _bin(self, op, other, swap=False):
        a, b = (as_expr(other), self) if swap else (self, as_expr(other))
        return Op(op, a, b)

    def __add__(self, o): return self._bin("+", o)
    def __radd__(self, o): return self._bin("+", o, True)
    def __sub__(self, o): return self._bin("-", o)
    def __rsub__(self, o): return self._bin("-", o, True)
    def __mul__(self, o): return self._bin("*", o)
    def __rmul__(self, o): return self._bin("*", o, True)
    def __truediv__(self, o): return self._bin("/", o)
    def __rtruediv__(self, o): return self._bin("/", o, True)
    def __neg__(self): return Op("neg", self)
    def __pos__(self): return self
    def __lt__(self, o): return self._bin("<", o)
    def __le__(self, o): return self._bin("<=", o)
    def __gt__(self, o): return self._bin(">", o)
    def __ge__(self, o): return self._bin(">=", o)
    def __hash__(self): return id(self)


class Lit(Expr):
    def __init__(self, v: float):
        self.v = v


class ConstRef(Expr):
    """A named constant resolved at lowering time (a C macro such as MPI_B0, an array
    element such as coeff[3], or a numeric literal written as a string)."""

    def __init__(self, name: str):
        self.name = name


class Index(Expr):
    """Axis n of the iteration space (0 = the contiguous axis i, 1 = j, 2 = k)."""

    def __init__(self, n: int):
        self.n = n

    def __add__(self, o):
        if isinstance(o, int):
            return IndexOff(self.n, o)
        return Expr.__add__(self, o)

    def __radd__(self, o):
        return self.__add__(o)

    def __sub__(self, o):
        if isinstance(o, int):
            return IndexOff(self.n, -o)
        return Expr.__sub__(self, o)

    def __hash__(self):
        return id(self)


class IndexOff(Expr):
    """Index n shifted by a constant."""

    def __init__(self, n: int, off: int):
        self.n, self.off = n, off

    def __add__(self, o):
        if isinstance(o, int):
            return IndexOff(self.n, self.off + o)
        return Expr.__add__(self, o)

    def __sub__(self, o):
        if isinstance(o, int):
            return IndexOff(self.n, self.off - o)
        return Expr.__sub__(self, o)


class Op(Expr):
    def __init__(self, op: str, *args):
        self.op, self.args = op, args


class If(Expr):
    """If(cond, then, else)."""

    def __init__(self, cond, then, other):
        self.cond, self.then, self.other = as_expr(cond), as_expr(then), as_expr(other)


class Call(Expr):
    def __init__(self, name: str, args):
        self.name, self.args = name, [as_expr(a) for a in args]
