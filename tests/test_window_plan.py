"""The windowed band LU-SGS sweep's plan (meshcfd_gb300/csrc/mcfd_window_plan.h,
plain C++ shared with the library): executed on the host the way
k_lusgs_window executes it, it reproduces the natural-order forward
substitution bit for bit on structured, long-range-coupled and randomly
numbered grids, for clusters of 8 and 16 blocks, roomy and tight
shared-memory limits (shortened windows, plans refused), and schedules with
wide levels outside the windows; every recomputed row equals its owner's and
every row is owned once.  The device sweep's own bits are checked against
the other engines in tests/test_gpu_implicit.py."""

import shutil
import subprocess
from pathlib import Path

import pytest

HERE = Path(__file__).resolve().parent


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_window_plan_executes_to_the_forward_substitution(tmp_path):
    exe = tmp_path / "window_plan_check"
    subprocess.run(["g++", "-O2", "-ffp-contract=off", "-std=c++17", "-o", str(exe),
                    str(HERE / "window_plan_check.cpp")], check=True)
    for seed in (1, 2, 3):
        out = subprocess.run([str(exe), str(seed)], capture_output=True, text=True)
        assert out.returncode == 0, out.stdout + out.stderr
        assert "failures=0" in out.stdout
        planned = int(out.stdout.split("planned=")[1].split()[0])
        assert planned > 200, out.stdout  # most cases fit the limits and are checked
