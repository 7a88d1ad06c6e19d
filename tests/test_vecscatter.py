"""The brick(...) statement front end for C++ sources (bricklib_gb300.dsl.vecscatter): the
reference's `brick("x.py", VEC, (dims), (fold), b);` in a per-brick loop (include/vecscatter.h:62,
codegen/vecscatter:145-186) lowered to one sweep; the stencil script read at lowering time into a
BrickStencil with the script's constants as C++ expressions.  CPU tests: the lowering, a
compile of the lowered program, the header mode; the GPU run is tests/test_gpu_vecscatter.py."""
import os
import shutil
import subprocess

import pytest

from bricklib_gb300 import dsl
from bricklib_gb300.dsl import vecscatter as VS
from oracle import oracle

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
PROG = os.path.join(HERE, "cpp", "vs_bricks.cpp")
_TREE = oracle.reference_tree()


def test_program_loop_is_lowered_to_one_sweep():
    src = open(PROG).read()
    out, report = VS.lower_source(src, PROG)
    assert [r["lowered"] for r in report] == [True]
    assert out.startswith('#include "brick-vs.h"')
    assert "bk_vs_site_0.visit(b);" in out and "brick(" not in out.split("int main")[0].split("bk_vs_site_0")[1]
    # the parallel-for line of the nest is dropped: the loop only records bricks
    assert "#pragma omp parallel for collapse(2)" not in out
    want = "BrickStencil()" + "".join(f".add({dk}, {dj}, {di}, (coeff[{n}]))" for n, (dk, dj, di) in enumerate(
        [(0, 0, 0), (0, 0, 1), (0, 0, -1), (0, 1, 0), (0, -1, 0), (1, 0, 0), (-1, 0, 0)]))
    assert f"bk_vs_site_0.sweep(bIn, bOut, {want});" in out
    # diagnostics of the kept loop still point at the original lines
    line = src.split("\n").index("  for (long tk = GB; tk < STRIDEB - GB; ++tk)") + 1
    assert f'#line {line} "{PROG}"' in out


@pytest.mark.skipif(shutil.which("g++") is None, reason="no C++ compiler")
def test_lowered_program_compiles(tmp_path):
    out, _ = VS.lower_source(open(PROG).read(), PROG)
    p = tmp_path / "vs_lowered.cpp"
    p.write_text(out)
    cuda = "/usr/local/cuda/include"
    r = subprocess.run(["g++", "-std=c++17", "-fopenmp", "-fsyntax-only", "-I", os.path.join(ROOT, "include"), "-I",
                        cuda, str(p)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_statement_outside_a_loop_is_reported_not_lowered():
    src = ('__global__ void k(unsigned (*grid)[4][4], Brick3D bIn, Brick3D bOut) {\n'
           '  unsigned b = grid[blockIdx.z][blockIdx.y][blockIdx.x];\n'
           '  brick("vs_star7.py", VSVEC, (8, 8, 8), (4, 8), b);\n}\n')
    out, report = VS.lower_source(src, os.path.join(HERE, "cpp", "kernel.cu"))
    assert report == [{"line": 3, "script": "vs_star7.py", "lowered": False,
                       "why": "not in a host brick loop (replace the kernel and its launch by brickSweep)"}]
    assert out == src


def test_unbraced_loop_and_comments():
    src = ('void f() {\n  // brick("no.py", V, (8,8,8), (4,8), b); in a comment\n'
           '  for (unsigned b = 0; b < n; ++b)\n    brick("vs_star7.py", VSVEC, (8, 8, 8), (4, 8), b);\n  g();\n}\n')
    out, report = VS.lower_source(src, os.path.join(HERE, "cpp", "f.cpp"))
    assert [r["lowered"] for r in report] == [True]
    assert "bk_vs_site_0.visit(b);" in out and "g();" in out and 'brick("no.py"' in out


def test_stencil_header_and_symbolic_coefficients(tmp_path):
    h = VS.stencil_header([os.path.join(HERE, "cpp", "vs_star7.py")])
    assert "#define BK_STENCIL_VS_STAR7 (BrickStencil().add(0, 0, 0, (coeff[0]))" in h
    s = tmp_path / "half.py"
    s.write_text("from st.expr import Index, ConstRef\nfrom st.grid import Grid\ni,j,k=Index(0),Index(1),Index(2)\n"
                 "a=Grid('a',3)\nb=Grid('b',3)\nb(i,j,k).assign(0.5*ConstRef('ALPHA')*(a(i+1,j,k)+a(i-1,j,k))"
                 " - ConstRef('BETA')*a(i,j,k))\nSTENCIL=[b]\n")
    low = dsl.lower_script(str(s), dsl.SYMBOLIC)
    assert [c.cpp() for c in low["coeff"]] == ["0.5 * (ALPHA)", "0.5 * (ALPHA)", "-(BETA)"]
    assert (low["input"], low["output"]) == ("a", "b")
    s.write_text("from st.expr import Index, ConstRef\nfrom st.grid import Grid\ni,j,k=Index(0),Index(1),Index(2)\n"
                 "a=Grid('a',3)\nb=Grid('b',3)\nb(i,j,k).assign(ConstRef('A')*ConstRef('B')*a(i,j,k))\nSTENCIL=[b]\n")
    with pytest.raises(dsl.NotLinear):
        dsl.lower_script(str(s), dsl.SYMBOLIC)


@pytest.mark.skipif(_TREE is None, reason="the reference tree is not here")
def test_reference_3axis_cpp_brick_loops_are_lowered():
    """stencils/3axis.cpp:68-76 (7pt.py) and its cond.py loop: both brick(...) statements lower,
    with the cond stencil's pointwise operations."""
    path = os.path.join(_TREE, "stencils", "3axis.cpp")
    out, report = VS.lower_source(open(path).read(), path)
    assert [(r["script"], r["lowered"]) for r in report] == [("7pt.py", True), ("cond.py", True)]
    assert "bk_vs_site_0.sweep(bIn, bOut, BrickStencil().add(0, 0, 0, (coeff[0]))" in out
    assert "bk_vs_site_1.sweep(bIn, bOut, bk_vs::with_ops(BrickStencil()" in out and ", 1, 2));" in out
