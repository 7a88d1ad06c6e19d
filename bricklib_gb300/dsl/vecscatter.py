"""Source-to-source lowering of brick(...) stencil statements for the GB300 engine.

The reference's build runs its `vecscatter` code generator on every C++/CUDA source that
contains `brick("x.py", VEC, (dims), (fold), b);` statements (include/vecscatter.h:62,
codegen/vecscatter:145-186): each statement becomes generated code that computes brick b.
This tool takes the same sources and lowers each such statement in a host brick loop to the
GB300 engine instead:

    for (long tk = GB; tk < STRIDEB - GB; ++tk)             {  // lowered
      for (long tj = GB; tj < STRIDEB - GB; ++tj)             static bk_vs::Site bk_vs_site_0;
        for (long ti = GB; ti < STRIDEB - GB; ++ti) {   ->    bk_vs_site_0.begin();
          unsigned b = grid[tk][tj][ti];                      for (...) ... { unsigned b = ...;
          brick("7pt.py", VSVEC, (BDIM), (VFOLD), b);            bk_vs_site_0.visit(b); }
        }                                                     bk_vs_site_0.sweep(bIn, bOut, <taps>);
                                                            }

The loop nest around the statement still runs (serially) and records the bricks it visits; one
bk_sweep then computes all of them.  The stencil script is read at lowering time (relative
paths relative to the source file, as the reference resolves them) and becomes a BrickStencil
tap list whose coefficients are the script's constants as C++ expressions of the caller's
scope (ConstRef("coeff[5]") -> coeff[5]).  The input and output Bricks are the variables named
by the script's grids.  include/brick-vs.h holds bk_vs::Site, which also runs bricks that live
in host memory (device mirrors, copied in and out around the sweep).  A statement that is not
in a host brick loop (e.g. inside a __global__ kernel) is reported, not lowered: there the
kernel and its launch are replaced by one brickSweep call over the launched bricks.

    python -m bricklib_gb300.dsl.vecscatter SRC -o DST
    python -m bricklib_gb300.dsl.vecscatter --stencil-header 7pt.py mpi13pt.py -o stencils.h
"""
from __future__ import annotations

import argparse
import os
import re
import sys
from typing import Dict, List, Optional, Tuple

from . import SYMBOLIC, lower_script

class LoweringError(ValueError):
    pass


def _code_mask(src: str) -> List[bool]:
    """True for characters that are code (not comment, string or character literal)."""
    mask = [True] * len(src)
    i, n = 0, len(src)
    while i < n:
        c = src[i]
        if src.startswith("//", i):
            j = src.find("\n", i)
            j = n if j < 0 else j
            mask[i:j] = [False] * (j - i)
            i = j
        elif src.startswith("/*", i):
            j = src.find("*/", i + 2)
            j = n if j < 0 else j + 2
            mask[i:j] = [False] * (j - i)
            i = j
        elif c in "\"'":
            j = i + 1
            while j < n and src[j] != c:
                j += 2 if src[j] == "\\" else 1
            j = min(n, j + 1)
            mask[i:j] = [False] * (j - i)
            i = j
        else:
            i += 1
    return mask


def _match_forward(src, mask, i, op, cl) -> int:
    """Index of the bracket closing the one at i."""
    depth = 0
    for p in range(i, len(src)):
        if not mask[p]:
            continue
        if src[p] == op:
            depth += 1
        elif src[p] == cl:
            depth -= 1
            if depth == 0:
                return p
    raise LoweringError("unbalanced brackets")


def _match_back(src, mask, i, op, cl) -> int:
    """Index of the bracket opening the one closed at i."""
    depth = 0
    for p in range(i, -1, -1):
        if not mask[p]:
            continue
        if src[p] == cl:
            depth += 1
        elif src[p] == op:
            depth -= 1
            if depth == 0:
                return p
    raise LoweringError("unbalanced brackets")


def _prev_code(src, mask, i) -> int:
    """Index of the last code character before i that is not white space (-1 if none)."""
    p = i - 1
    while p >= 0 and (not mask[p] or src[p].isspace()):
        p -= 1
    return p


def _split_args(text: str) -> List[str]:
    out, depth, cur = [], 0, []
    for ch in text:
        if ch in "([{":
            depth += 1
        elif ch in ")]}":
            depth -= 1
        if ch == "," and depth == 0:
            out.append("".join(cur).strip())
            cur = []
        else:
            cur.append(ch)
    out.append("".join(cur).strip())
    return out


def find_brick_statements(src: str) -> List[Dict]:
    """Every `brick(file, vec, dims, fold, idx[, stride]);` statement: its span and arguments."""
    mask = _code_mask(src)
    found = []
    for m in re.finditer(r"\bbrick\s*\(", src):
        if not mask[m.start()]:
            continue
        # a statement, not the macro's definition or a member call
        p = _prev_code(src, mask, m.start())
        if p >= 0 and src[p] not in ";{}):":
            continue
        line_start = src.rfind("\n", 0, m.start()) + 1
        if src[line_start:m.start()].lstrip().startswith("#"):
            continue
        op = src.index("(", m.start())
        cl = _match_forward(src, mask, op, "(", ")")
        args = _split_args(src[op + 1:cl])
        if len(args) not in (5, 6):
            continue
        q = cl + 1
        while q < len(src) and src[q].isspace():
            q += 1
        if q >= len(src) or src[q] != ";":
            raise LoweringError(f"brick(...) at line {src.count(chr(10), 0, m.start()) + 1} is not a statement")
        script = args[0].strip()
        if not (script.startswith('"') and script.endswith('"')):
            raise LoweringError("the first argument of brick(...) must be a string literal (the stencil script)")
        found.append({"start": m.start(), "end": q + 1, "script": script[1:-1], "vec": args[1], "dims": args[2],
                      "fold": args[3], "bidx": args[4], "line": src.count("\n", 0, m.start()) + 1})
    return found


def _is_for_header(src: str, mask: List[bool], close: int) -> bool:
    """Whether the parenthesis closed at `close` is the header of a for statement."""
    kw = _prev_code(src, mask, _match_back(src, mask, close, "(", ")"))
    return kw >= 2 and src[kw - 2:kw + 1] == "for" and not (kw >= 3 and (src[kw - 3].isalnum() or src[kw - 3] == "_"))


def _enclosing_for_nest(src: str, mask: List[bool], st: int) -> Optional[Tuple[int, int]]:
    """(start, end) of the for-loop nest whose innermost body holds the statement at st: the
    outermost `for` of consecutive for headers (each the unbraced body of the previous one),
    through the closing brace of the innermost body.  A parallel-for line right before the
    nest (an `#pragma omp ...` line or the reference's _PARFOR macro) is part of it.  None
    when the statement is not in a for loop."""
    p = _prev_code(src, mask, st)
    if p < 0:
        return None
    body_close = None
    if src[p] == ")" and _is_for_header(src, mask, p):  # unbraced body: for (...) brick(...);
        hdr_end = p
    else:  # the innermost block holding the statement
        depth, q = 0, st - 1
        while q >= 0:
            if mask[q] and src[q] == "}":
                depth += 1
            elif mask[q] and src[q] == "{":
                if depth == 0:
                    break
                depth -= 1
            q -= 1
        if q < 0:
            return None
        body_close = _match_forward(src, mask, q, "{", "}")
        hdr_end = _prev_code(src, mask, q)
    outer = None
    while hdr_end >= 0 and src[hdr_end] == ")" and _is_for_header(src, mask, hdr_end):
        outer = _prev_code(src, mask, _match_back(src, mask, hdr_end, "(", ")")) - 2
        hdr_end = _prev_code(src, mask, outer)
    if outer is None:
        return None
    # a parallel-for line right before the nest
    line_start = src.rfind("\n", 0, outer) + 1
    prev_line_end = line_start - 1
    prev_line_start = src.rfind("\n", 0, max(prev_line_end, 0)) + 1
    prev_line = src[prev_line_start:max(prev_line_end, 0)].strip()
    start = line_start
    if prev_line.startswith("#pragma omp") or prev_line == "_PARFOR":
        start = prev_line_start
    return start, (body_close + 1 if body_close is not None else None)


def stencil_initializer(script_path: str) -> Tuple[str, Dict]:
    """The script lowered to a BrickStencil expression with coefficients as C++ expressions."""
    low = lower_script(script_path, SYMBOLIC)
    expr = "BrickStencil()" + "".join(f".add({t[0]}, {t[1]}, {t[2]}, {c.cpp()})"
                                      for t, c in zip(low["taps"], low["coeff"]))
    if low["pre_op"] or low["post_op"]:
        expr = f"bk_vs::with_ops({expr}, {low['pre_op']}, {low['post_op']})"
    return expr, low


def lower_source(src: str, path: str = "<source>", script_dir: Optional[str] = None) -> Tuple[str, List[Dict]]:
    """Lower every brick(...) statement in a host brick loop; returns the new source and a
    report per statement ({"line", "script", "lowered", "why"})."""
    script_dir = script_dir or os.path.dirname(os.path.abspath(path))
    stmts = find_brick_statements(src)
    mask = _code_mask(src)
    report = []
    edits = []
    for n, s in enumerate(stmts):
        nest = _enclosing_for_nest(src, mask, s["start"])
        if nest is None:
            report.append({"line": s["line"], "script": s["script"], "lowered": False,
                           "why": "not in a host brick loop (replace the kernel and its launch by brickSweep)"})
            continue
        start, end = nest
        if end is None:  # unbraced innermost body: the nest ends with the statement
            end = s["end"]
        script = s["script"] if os.path.isabs(s["script"]) else os.path.join(script_dir, s["script"])
        expr, low = stencil_initializer(script)
        site = f"bk_vs_site_{n}"
        body = src[start:s["start"]] + f"{site}.visit({s['bidx']});" + src[s["end"]:end]
        line_at_start = src.count("\n", 0, start) + 1
        first = body.split("\n", 1)
        if first[0].strip().startswith("#pragma omp") or first[0].strip() == "_PARFOR":
            body = first[1] if len(first) > 1 else ""  # the nest runs serially: it only records bricks
            line_at_start += 1
        line_after = src.count("\n", 0, end) + 1
        block = (f"{{  /* brick(\"{s['script']}\", {s['vec']}, {s['dims']}, {s['fold']}, {s['bidx']}) lowered to one "
                 f"GB300 sweep over the bricks this loop visits */\n"
                 f"static bk_vs::Site {site};\n{site}.begin();\n"
                 f"#line {line_at_start} \"{path}\"\n{body}\n"
                 f"{site}.sweep({low['input']}, {low['output']}, {expr});\n}}\n"
                 f"#line {line_after} \"{path}\"\n")
        edits.append((start, end, block))
        report.append({"line": s["line"], "script": s["script"], "lowered": True, "why": ""})
    out = src
    for start, end, block in sorted(edits, reverse=True):
        out = out[:start] + block + out[end:]
    if edits:
        out = f'#include "brick-vs.h"\n#line 1 "{path}"\n' + out
    return out, report


def stencil_header(scripts: List[str]) -> str:
    """A C++ header with one BK_STENCIL_<name> macro per script: the script's BrickStencil,
    its coefficients evaluated where the macro is used."""
    lines = ["// generated by bricklib_gb300.dsl.vecscatter --stencil-header", "#pragma once",
             '#include "brick-vs.h"', ""]
    for sc in scripts:
        expr, low = stencil_initializer(sc)
        name = re.sub(r"\W", "_", os.path.splitext(os.path.basename(sc))[0]).upper()
        lines.append(f"// {os.path.basename(sc)}: {len(low['taps'])} taps, {low['input']} -> {low['output']}")
        lines.append(f"#define BK_STENCIL_{name} ({expr})")
    return "\n".join(lines) + "\n"


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(prog="python -m bricklib_gb300.dsl.vecscatter", description=__doc__.split("\n")[0])
    ap.add_argument("inputs", nargs="+")
    ap.add_argument("-o", "--output", required=True)
    ap.add_argument("--stencil-header", action="store_true", help="inputs are stencil scripts: write a header")
    a = ap.parse_args(argv)
    if a.stencil_header:
        text = stencil_header(a.inputs)
    else:
        if len(a.inputs) != 1:
            ap.error("one source file per run")
        with open(a.inputs[0]) as f:
            src = f.read()
        text, report = lower_source(src, os.path.abspath(a.inputs[0]))
        for r in report:
            print(f"{a.inputs[0]}:{r['line']}: brick(\"{r['script']}\") "
                  + ("lowered" if r["lowered"] else f"NOT lowered: {r['why']}"), file=sys.stderr)
    with open(a.output, "w") as f:
        f.write(text)
    return 0


if __name__ == "__main__":
    sys.exit(main())
