"""Throughput probe of the integer-pipe division, square root and product
(tests/arith_throughput.cu, compiled here for sm_103a against the product
header): bit-identical to the FP64 unit along long dependency chains, and
its measured rates printed (run with -s to see them)."""

import subprocess
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu

HERE = Path(__file__).resolve().parent


def test_integer_pipe_arithmetic_throughput(tmp_path, cuda_device):
    from meshcfd_gb300.build import nvcc

    try:
        compiler = nvcc()
    except RuntimeError:
        pytest.skip("needs nvcc")
    exe = tmp_path / "arith_throughput"
    subprocess.run([compiler, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-o", str(exe),
                    str(HERE / "arith_throughput.cu")], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    print(out.stdout)
    assert out.returncode == 0, out.stdout + out.stderr
    rates = dict(line.split() for line in out.stdout.splitlines() if line and not line.startswith(("cuda", "mismatches")))
    rates = {k: float(v) for k, v in rates.items()}
    assert "mismatches=0" in out.stdout
    # the integer-pipe division is faster than the FP64 unit's on GB300
    assert rates["div_int"] > rates["div_fp64"]
