"""The C++ brick program tests/cpp/vs_bricks.cpp -- the reference's single-node CPU pattern with
a brick("vs_star7.py", ...) statement in its per-brick loop -- lowered by
bricklib_gb300.dsl.vecscatter, compiled against the library and run: its bricks in host memory
(twice) and in device memory, each pass checked by compareBrick against the array loop at 1e-12."""
import os
import subprocess

import pytest

from bricklib_gb300 import build

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def test_lowered_brick_program_matches_its_array_loop(tmp_path):
    exe = build.build_lowered_program(os.path.join(HERE, "cpp", "vs_bricks.cpp"), str(tmp_path / "vs_bricks"))
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and "result match" in r.stdout, r.stdout + r.stderr
