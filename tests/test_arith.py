"""The integer-pipe IEEE division, square root and product that the residual
kernels use in place of the FP64 unit's: bit-identical results on the host
(the header compiled as plain C++ against the host's IEEE arithmetic) and on
the GPU (through mcfd_ieee_div_sqrt / mcfd_ieee_mul against the FP64 unit's
`/`, `sqrt` and `*`)."""

import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

HERE = Path(__file__).resolve().parent


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_host_division_and_root_are_ieee(tmp_path):
    exe = tmp_path / "arith_check"
    subprocess.run(["g++", "-O2", "-ffp-contract=off", "-std=c++17", "-o", str(exe),
                    str(HERE / "arith_check.cpp")], check=True)
    for seed in (1, 2):
        out = subprocess.run([str(exe), "400000", str(seed)], capture_output=True, text=True)
        assert out.returncode == 0, out.stdout + out.stderr
        assert "mismatches=0" in out.stdout


def _operands(n, seed):
    """Random doubles over several exponent spans, with runs of zero / one
    significand bits and a few planted relations (a / a, nearly equal,
    divisor near 1), plus zeros, subnormals, extremes, infinities and NaN."""
    rng = np.random.default_rng(seed)

    def draw(span):
        mant = rng.integers(0, 1 << 52, size=n, dtype=np.uint64)
        kind = rng.integers(0, 8, size=n)
        mant = np.where(kind == 0, mant & np.uint64(0xffff000000000), mant)
        mant = np.where(kind == 1, mant | np.uint64(0x0000ffffffffff), mant)
        mant = np.where(kind == 2, np.uint64(0), mant)
        exp = np.clip(1023 + rng.integers(-span, span + 1, size=n), 0, 2047).astype(np.uint64)
        sign = rng.integers(0, 2, size=n).astype(np.uint64)
        return ((sign << np.uint64(63)) | (exp << np.uint64(52)) | mant).view(np.float64)

    spans = np.array([1, 30, 200, 700, 1100])
    a = np.concatenate([draw(s) for s in spans])
    b = np.concatenate([draw(s) for s in spans])
    m = len(a)
    idx = np.arange(m)
    b = np.where(idx % 16 == 3, -a, b)
    b = np.where(idx % 16 == 5, (a.view(np.uint64) ^ np.uint64(1)).view(np.float64), b)
    b = np.where(idx % 16 == 7, (np.uint64(0x3ff0000000000000) | (idx.astype(np.uint64) & np.uint64(3))).view(np.float64), b)
    specials = np.array([0.0, -0.0, 1.0, -1.0, 2.0, 0.5, 3.0, 1e-300, 1e300, 1.7976931348623157e308,
                         2.2250738585072014e-308, 5e-324, 2.225073858507201e-308, np.inf, -np.inf, np.nan,
                         0.1, 1.4, 0.4, 1e-10, 1e10])
    sa, sb = np.meshgrid(specials, specials)
    return np.concatenate([a, sa.ravel()]), np.concatenate([b, sb.ravel()])


def _same_bits(x, y):
    return (x.view(np.uint64) == y.view(np.uint64)) | (np.isnan(x) & np.isnan(y))


@pytest.mark.gpu
def test_gpu_division_and_root_match_the_fp64_unit(cuda_device):
    import torch
    from meshcfd_gb300 import _lib

    lib = _lib.native()
    stream = torch.cuda.current_stream().cuda_stream
    for seed in (0, 1, 2, 3):
        a_np, b_np = _operands(1 << 20, seed)
        a = torch.as_tensor(a_np, device=cuda_device)
        b = torch.as_tensor(b_np, device=cuda_device)
        q = torch.empty_like(a)
        r = torch.empty_like(a)
        assert lib.mcfd_ieee_div_sqrt(a.data_ptr(), b.data_ptr(), a.numel(), q.data_ptr(), r.data_ptr(), stream) == 0
        qn, rn = (a / b).cpu().numpy(), torch.sqrt(a).cpu().numpy()
        torch.cuda.synchronize()
        ok_q = _same_bits(q.cpu().numpy(), qn)
        ok_r = _same_bits(r.cpu().numpy(), rn)
        assert ok_q.all(), (a_np[~ok_q][:3], b_np[~ok_q][:3])
        assert ok_r.all(), a_np[~ok_r][:3]
        # and against numpy's (host IEEE) results, non-NaN entries
        with np.errstate(all="ignore"):
            assert _same_bits(qn, a_np / b_np).all()


@pytest.mark.gpu
def test_gpu_reciprocal_candidate_division_matches_the_fp64_unit(cuda_device):
    """The sweeps' division (reciprocal candidate, exact remainder test,
    integer-pipe fallback) on the random operands, and on quotients planted
    next to midpoints of two doubles, where a candidate is most often
    rejected."""
    import torch
    from meshcfd_gb300 import _lib

    lib = _lib.native()
    stream = torch.cuda.current_stream().cuda_stream
    rng = np.random.default_rng(11)
    b_mid = np.ldexp(1.0 + rng.random(1 << 18), rng.integers(-30, 30, 1 << 18))
    m = np.ldexp(1.0 + rng.random(1 << 18), rng.integers(-8, 8, 1 << 18))
    a_mid = b_mid * (m + np.ldexp(1.0, np.frexp(m)[1] - 54))  # a / b next to the midpoint above m
    for seed in (7, 8, None):
        a_np, b_np = _operands(1 << 20, seed) if seed is not None else (
            np.concatenate([a_mid, np.nextafter(a_mid, 0.0), np.nextafter(a_mid, np.inf)]), np.tile(b_mid, 3))
        a = torch.as_tensor(a_np, device=cuda_device)
        b = torch.as_tensor(b_np, device=cuda_device)
        q = torch.empty_like(a)
        assert lib.mcfd_ieee_div_fma(a.data_ptr(), b.data_ptr(), a.numel(), q.data_ptr(), stream) == 0
        ref = (a / b).cpu().numpy()
        torch.cuda.synchronize()
        ok = _same_bits(q.cpu().numpy(), ref)
        assert ok.all(), (a_np[~ok][:3], b_np[~ok][:3])
    assert lib.mcfd_ieee_div_fma(None, None, 4, None, stream) == 1


@pytest.mark.gpu
def test_gpu_product_matches_the_fp64_unit(cuda_device):
    import torch
    from meshcfd_gb300 import _lib

    lib = _lib.native()
    stream = torch.cuda.current_stream().cuda_stream
    for seed in (4, 5, 6):
        a_np, b_np = _operands(1 << 20, seed)
        a = torch.as_tensor(a_np, device=cuda_device)
        b = torch.as_tensor(b_np, device=cuda_device)
        p = torch.empty_like(a)
        assert lib.mcfd_ieee_mul(a.data_ptr(), b.data_ptr(), a.numel(), p.data_ptr(), stream) == 0
        ref = (a * b).cpu().numpy()
        torch.cuda.synchronize()
        ok = _same_bits(p.cpu().numpy(), ref)
        assert ok.all(), (a_np[~ok][:3], b_np[~ok][:3])
        with np.errstate(all="ignore"):
            assert _same_bits(ref, a_np * b_np).all()
    assert lib.mcfd_ieee_mul(None, None, 4, None, stream) == 1


@pytest.mark.gpu
def test_gpu_division_entry_point_arguments(cuda_device):
    import torch
    from meshcfd_gb300 import _lib

    lib = _lib.native()
    stream = torch.cuda.current_stream().cuda_stream
    a = torch.tensor([4.0, 9.0], dtype=torch.float64, device=cuda_device)
    r = torch.zeros_like(a)
    assert lib.mcfd_ieee_div_sqrt(a.data_ptr(), None, 2, None, r.data_ptr(), stream) == 0
    assert r.cpu().tolist() == [2.0, 3.0]
    assert lib.mcfd_ieee_div_sqrt(a.data_ptr(), None, 2, r.data_ptr(), None, stream) == 1  # quotient needs b
    assert lib.mcfd_ieee_div_sqrt(None, None, 2, None, r.data_ptr(), stream) == 1
    assert lib.mcfd_ieee_div_sqrt(a.data_ptr(), None, 0, None, None, stream) == 0
