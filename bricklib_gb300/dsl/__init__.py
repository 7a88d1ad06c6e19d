"""Stencil-language front end: run a bricklib stencil script (the `.py` files the
reference's code generator reads, e.g. stencils/7pt.py, stencils/mpi13pt.py) and lower the
grid assigned in STENCIL to a tap list for bk_sweep.

    st = load_stencil("stencils/mpi13pt.py", constants_from_header("stencils/fake.h"))
    st = load_stencil("stencils/7pt.py", {"coeff": [c0, ..., c6]})

Scripts import `st.expr`, `st.grid` and `st.func`; this package provides those modules,
so a script runs unchanged (the reference resolves the same names in codegen/st).
Lowering accepts expressions linear in the input grid -- sums of constant-times-reference
terms, products by constants, negation, division by constants.  Taps keep the order in
which the script first mentions them (the reference's summation order); repeated taps
merge their coefficients.  The cond stencil's pattern -- max(x, 0) around every input
reference and If(s > 0, s, -s) around the sum (stencils/cond.py) -- lowers to the sweep's
pointwise pre / post operations; other non-linear scripts raise NotLinear.
"""
from __future__ import annotations

import importlib
import os
import re
import sys
from typing import Dict, List, Optional, Tuple

from .. import stencils

HERE = os.path.dirname(os.path.abspath(__file__))


class NotLinear(ValueError):
    pass


SYMBOLIC: Dict = {}  # constants table that keeps every named constant as a C++ expression


def _modules():
    """The st package of this front end, importable under the names scripts use."""
    mods = {}
    if HERE not in sys.path:
        sys.path.insert(0, HERE)
    for name in ("st", "st.expr", "st.grid", "st.func"):
        mods[name] = importlib.import_module(name)
    return mods


def constants_from_header(path: str) -> Dict[str, float]:
    """`#define NAME number` lines of a C header (e.g. stencils/fake.h MPI_ALPHA ...)."""
    out = {}
    pat = re.compile(r"^\s*#\s*define\s+(\w+)\s+([-+0-9.eE]+)\s*$")
    with open(path) as f:
        for line in f:
            m = pat.match(line)
            if m:
                try:
                    out[m.group(1)] = float(m.group(2))
                except ValueError:
                    pass
    return out


class SymCoef:
    """A coefficient linear in named constants -- {name: factor}, the empty name for the
    literal part -- for lowering a script to C++ source, where ConstRef("coeff[5]") or
    ConstRef("MPI_ALPHA") stay expressions of the caller's scope."""

    def __init__(self, terms: Dict[str, float]):
        self.t = {k: float(v) for k, v in terms.items() if v != 0.0}

    @staticmethod
    def of(x) -> "SymCoef":
        return x if isinstance(x, SymCoef) else SymCoef({"": float(x)})

    def literal(self) -> Optional[float]:
        return self.t.get("", 0.0) if set(self.t) <= {""} else None

    def __add__(self, o):
        o = SymCoef.of(o)
        t = dict(self.t)
        for k, v in o.t.items():
            t[k] = t.get(k, 0.0) + v
        return SymCoef(t)

    __radd__ = __add__

    def __neg__(self):
        return SymCoef({k: -v for k, v in self.t.items()})

    def __sub__(self, o):
        return self + (-SymCoef.of(o))

    def __rsub__(self, o):
        return SymCoef.of(o) - self

    def __mul__(self, o):
        o = SymCoef.of(o)
        a, b = self.literal(), o.literal()
        if a is None and b is None:
            raise NotLinear("product of two named constants: give one of them a value")
        if b is not None:
            return SymCoef({k: v * b for k, v in self.t.items()})
        return SymCoef({k: v * a for k, v in o.t.items()})

    __rmul__ = __mul__

    def __truediv__(self, o):
        b = SymCoef.of(o).literal()
        if b is None:
            raise NotLinear("division by a named constant")
        return SymCoef({k: v / b for k, v in self.t.items()})

    def __eq__(self, o):
        try:
            o = SymCoef.of(o)
        except (TypeError, ValueError):
            return NotImplemented
        return self.t == o.t

    def __ne__(self, o):
        r = self.__eq__(o)
        return r if r is NotImplemented else not r

    def __hash__(self):
        return hash(tuple(sorted(self.t.items())))

    def cpp(self) -> str:
        """The coefficient as a C++ expression (names as written in the script)."""
        if not self.t:
            return "0.0"
        parts = []
        for k in sorted(self.t, key=lambda x: (x == "", x)):
            v = self.t[k]
            if k == "":
                parts.append(repr(v))
            elif v == 1.0:
                parts.append(f"({k})")
            elif v == -1.0:
                parts.append(f"-({k})")
            else:
                parts.append(f"{v!r} * ({k})")
        return " + ".join(parts).replace("+ -", "- ")


def _const(name: str, consts: Dict):
    try:
        return float(name)
    except ValueError:
        pass
    if consts is SYMBOLIC:
        return SymCoef({name.strip(): 1.0})
    if name in consts:
        return float(consts[name])
    m = re.fullmatch(r"\s*(\w+)\s*\[\s*(\d+)\s*\]\s*", name)
    if m and m.group(1) in consts:
        return float(consts[m.group(1)][int(m.group(2))])
    raise KeyError(f"no value for constant {name!r}")


def _linear(e, consts, inp, order: List[Tuple[int, int, int]]):
    """(constant term, {tap: coefficient}) of an expression linear in grid `inp`."""
    ex = importlib.import_module("st.expr")
    gr = importlib.import_module("st.grid")
    if isinstance(e, ex.Lit):
        return e.v, {}
    if isinstance(e, ex.ConstRef):
        return _const(e.name, consts), {}
    if isinstance(e, gr.GridRef):
        if e.grid is not inp:
            raise NotLinear(f"reads grid {e.grid.name} besides the input")
        o = e.offsets
        tap = (o[2], o[1], o[0]) if len(o) == 3 else tuple(reversed(o))
        if tap not in order:
            order.append(tap)
        return 0.0, {tap: 1.0}
    if isinstance(e, ex.Op):
        if e.op == "neg":
            c, t = _linear(e.args[0], consts, inp, order)
            return -c, {k: -v for k, v in t.items()}
        a, b = e.args
        ca, ta = _linear(a, consts, inp, order)
        cb, tb = _linear(b, consts, inp, order)
        if e.op in ("+", "-"):
            s = 1.0 if e.op == "+" else -1.0
            t = dict(ta)
            for k, v in tb.items():
                t[k] = t.get(k, 0.0) + s * v
            return ca + s * cb, t
        if e.op == "*":
            if ta and tb:
                raise NotLinear("product of two grid references")
            if ta:
                return ca * cb, {k: v * cb for k, v in ta.items()}
            return ca * cb, {k: v * ca for k, v in tb.items()}
        if e.op == "/":
            if tb:
                raise NotLinear("division by a grid reference")
            return ca / cb, {k: v / cb for k, v in ta.items()}
        raise NotLinear(f"operator {e.op}")
    if isinstance(e, (ex.If, ex.Call)):
        raise NotLinear(f"{type(e).__name__} is not a linear stencil")
    raise NotLinear(f"unsupported node {type(e).__name__}")


def _is_zero(e, consts) -> bool:
    ex = importlib.import_module("st.expr")
    try:
        return (isinstance(e, ex.Lit) and e.v == 0.0) or (isinstance(e, ex.ConstRef) and _const(e.name, consts) == 0.0)
    except KeyError:
        return False


def _strip_ops(expr, consts):
    """Recognise the pointwise operations of the cond stencil (stencils/cond.py):
    If(s > 0, s, -s) around the sum (post |.|) and max(x, 0) around every input reference
    (pre max(., 0)).  Returns (expression without them, pre_op, post_op)."""
    ex = importlib.import_module("st.expr")
    gr = importlib.import_module("st.grid")
    post = 0
    if isinstance(expr, ex.If):
        c = expr.cond
        if (isinstance(c, ex.Op) and c.op == ">" and c.args[0] is expr.then and _is_zero(c.args[1], consts)
                and isinstance(expr.other, ex.Op) and expr.other.op == "neg" and expr.other.args[0] is expr.then):
            expr, post = expr.then, 2
        else:
            raise NotLinear("only If(s > 0, s, -s) (an absolute value) is supported")
    found = {"relu": 0, "plain": 0}

    def unwrap(e):
        if isinstance(e, ex.Call):
            if e.name == "max" and len(e.args) == 2 and isinstance(e.args[0], gr.GridRef) and _is_zero(e.args[1], consts):
                found["relu"] += 1
                return e.args[0]
            raise NotLinear(f"function {e.name} is not supported")
        if isinstance(e, gr.GridRef):
            found["plain"] += 1
            return e
        if isinstance(e, ex.Op):
            return ex.Op(e.op, *[unwrap(a) for a in e.args])
        return e

    expr = unwrap(expr)
    if found["relu"] and found["plain"]:
        raise NotLinear("max(x, 0) must wrap every input reference or none")
    return expr, (1 if found["relu"] else 0), post


def load_stencil(path: str, constants: Optional[Dict] = None, name: Optional[str] = None,
                 input_grid: Optional[str] = None) -> stencils.Stencil:
    """Run a stencil script and lower its (single) output grid to a Stencil."""
    low = lower_script(path, constants, input_grid)
    st = stencils.custom(name or os.path.splitext(os.path.basename(path))[0], low["taps"], low["coeff"])
    st.pre_op, st.post_op = low["pre_op"], low["post_op"]
    return st


def lower_script(path: str, constants: Optional[Dict] = None, input_grid: Optional[str] = None) -> Dict:
    """Run a stencil script and lower its output grid: {"taps": [(dk, dj, di), ...], "coeff":
    [...], "pre_op", "post_op", "input": name, "output": name}.  With constants=SYMBOLIC every
    named constant stays a SymCoef (a C++ expression of the caller's scope)."""
    _modules()
    ns: Dict = {"__name__": "__stencil__", "__file__": path}
    with open(path) as f:
        code = compile(f.read(), path, "exec")
    exec(code, ns)
    outs = ns.get("STENCIL")
    if not outs:
        raise ValueError(f"{path} defines no STENCIL")
    if len(outs) != 1:
        raise ValueError("one output grid per stencil is supported")
    out = outs[0]
    if out.assigned is None:
        raise ValueError(f"output grid {out.name} is never assigned")
    offs, expr = out.assigned
    if any(offs):
        raise ValueError("the output must be assigned at the centre (i, j, k)")
    gr = importlib.import_module("st.grid")
    grids = [v for v in ns.values() if isinstance(v, gr.Grid) and v is not out]
    if input_grid:
        grids = [g for g in grids if g.name == input_grid]
    if len(grids) != 1:
        raise ValueError("the script must declare exactly one input grid (or name it with input_grid)")
    consts = constants if constants is not None else {}
    expr, pre, post = _strip_ops(expr, consts)
    order: List[Tuple[int, int, int]] = []
    c0, taps = _linear(expr, consts, grids[0], order)
    if c0 != 0.0:
        raise NotLinear("affine term (a constant added to the stencil) is not supported")
    order = [t for t in order if taps.get(t, 0.0) != 0.0]
    return {"taps": order, "coeff": [taps[t] for t in order], "pre_op": pre, "post_op": post,
            "input": grids[0].name, "output": out.name}
