"""Stencil-language front end: scripts lower to the tap lists the sweep takes."""
import os

import numpy as np
import pytest

from bricklib_gb300 import dsl, stencils
from oracle import oracle

HERE = os.path.dirname(os.path.abspath(__file__))
_TREE = oracle.reference_tree()  # $BRICKLIB_REF or the oracle recipe's default; None when absent
REF = os.path.join(_TREE, "stencils") if _TREE else ""


def test_loop_script_lowers_to_star13():
    st = dsl.load_stencil(os.path.join(HERE, "golden", "dsl", "star13_loops.py"), {"W0": 0.4, "W1": 0.07, "W2": 0.03})
    want = stencils.star_taps(2)[0]
    assert st.taps == want
    cls = stencils.star_taps(2)[1]
    np.testing.assert_array_equal(st.coeff, np.array([0.4, 0.07, 0.03])[cls])


def test_four_dimensional_script_lowers_to_the_4d_star():
    """A 4-D script lowers to (dl, dk, dj, di) taps: the tap set and weights of
    stencils/mpi9pt.py (bk_sweep4 takes the list as is)."""
    from bricklib_gb300 import bricks4
    st = dsl.load_stencil(os.path.join(HERE, "golden", "dsl", "star9_4d_loops.py"), {"A": 0.2, "B": 0.1})
    want = bricks4.mpi9pt()
    assert sorted(zip(st.taps, st.coeff)) == sorted(zip(want.taps, want.coeff))
    assert bricks4.to_c_stencil4(st).npoints == 9


def test_nonlinear_and_missing_constants_are_reported(tmp_path):
    p = tmp_path / "bad.py"
    p.write_text("from st.expr import Index\nfrom st.grid import Grid\ni,j,k=Index(0),Index(1),Index(2)\n"
                 "a=Grid('a',3)\nb=Grid('b',3)\nb(i,j,k).assign(a(i,j,k)*a(i+1,j,k))\nSTENCIL=[b]\n")
    with pytest.raises(dsl.NotLinear):
        dsl.load_stencil(str(p))
    q = tmp_path / "missing.py"
    q.write_text("from st.expr import Index, ConstRef\nfrom st.grid import Grid\ni,j,k=Index(0),Index(1),Index(2)\n"
                 "a=Grid('a',3)\nb=Grid('b',3)\nb(i,j,k).assign(ConstRef('Q')*a(i,j,k))\nSTENCIL=[b]\n")
    with pytest.raises(KeyError):
        dsl.load_stencil(str(q))


@pytest.mark.skipif(not os.path.isdir(REF), reason="the reference's stencil scripts are not here")
def test_reference_scripts_lower_to_the_plain_shapes():
    consts = dsl.constants_from_header(os.path.join(REF, "fake.h"))
    assert consts["MPI_ALPHA"] == 0.4 and consts["MPI_C9"] == 0.001
    coeff = list(np.linspace(0.1, 0.7, 7))
    st7 = dsl.load_stencil(os.path.join(REF, "7pt.py"), {"coeff": coeff})
    assert st7.taps == stencils.star_taps(1)[0]
    np.testing.assert_array_equal(st7.coeff, coeff)
    for script, shape, r in [("mpi7pt.py", "star", 1), ("mpi13pt.py", "star", 2), ("mpi25pt.py", "star", 4),
                             ("mpi125pt.py", "cube", 2)]:
        st = dsl.load_stencil(os.path.join(REF, script), consts)
        want = (stencils.star_taps(r) if shape == "star" else stencils.cube_taps(r))[0]
        assert sorted(st.taps) == sorted(want), script
        if shape == "star":
            assert st.taps == want, script  # same order: the summation order of the script
    heat = dsl.load_stencil(os.path.join(REF, "mpi7pt.py"), consts)
    np.testing.assert_allclose(heat.coeff, stencils.make("heat7").coeff)
    cond = dsl.load_stencil(os.path.join(REF, "cond.py"), {"coeff": coeff})
    want = stencils.make("cond7", 0)
    assert (cond.pre_op, cond.post_op) == (want.pre_op, want.post_op) == (1, 2)
    assert sorted(cond.taps) == sorted(want.taps)
