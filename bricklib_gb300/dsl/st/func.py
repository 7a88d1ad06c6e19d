"""Named functions of the stencil language (st.func.Func), e.g. Func("max", 2)."""
from __future__ import annotations

from .expr import Call


class Func:
    def __init__(self, name: str, nargs: int):
        self.name, self.nargs = name, nargs

    def __call__(self, *args):
        if len(args) != self.nargs:
            raise ValueError(f"{self.name} takes {self.nargs} arguments")
        return Call(self.name, args)
