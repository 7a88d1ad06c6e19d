"""The C++ drop-in driver (tests/cpp/single_gb300.cpp): the reference's single-node
CUDA test rewritten against include/brick.h, bricksetup.h, brick-gb300.h and
brickcompare.h, checked at 1e-12 for five stencil shapes."""
import os
import subprocess

import pytest

from bricklib_gb300 import build as _b

pytestmark = pytest.mark.gpu


def test_cpp_single_node_driver():
    exe = _b.build_cpp_driver()
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "result match" in r.stdout
    for name in ("d3pt7", "d3pt13", "d3pt25", "d3pt27", "d3pt125", "decomp", "d4pt9"):
        assert f"{name} match" in r.stdout
