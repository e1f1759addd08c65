"""The allocation-free sum-of-squares entry point against the allocating one.

mcfd_residual_sumsq_noalloc exists for callers that cannot allocate device
memory (for instance a convergence monitor running inside a host time loop
whose device memory belongs to another allocator): it keeps its scratch in a
fixed __device__ array instead of a geometry handle's arena.  It must give the
same sums as mcfd_residual_sumsq, call after call, and refuse sizes beyond its
stated maximum.  This file is collected last on purpose.
"""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _handle_for(n):
    from meshcfd_gb300.device import DeviceGeometry
    from meshcfd_gb300.geometry import build_geometry
    from meshcfd_gb300.meshes import vortex_case

    case, _ = vortex_case(n, split="half")
    return DeviceGeometry(build_geometry(case.mesh, case))


@pytest.mark.parametrize("n", (12, 160))
def test_noalloc_sumsq_matches_allocating_entry_point(cuda_device, n):
    import torch
    from meshcfd_gb300 import _lib

    lib = _lib.native()
    dg = _handle_for(n)
    stream = torch.cuda.current_stream().cuda_stream
    gen = torch.Generator(device=cuda_device).manual_seed(n)
    for call in range(2):  # two calls in a row share the scratch array
        R = torch.randn(dg.n_cells, 4, dtype=torch.float64, device=cuda_device, generator=gen) * (1.0 + call)
        expected = torch.empty(4, dtype=torch.float64, device=cuda_device)
        assert lib.mcfd_residual_sumsq(dg.handle, R.data_ptr(), expected.data_ptr(), stream) == 0
        got = torch.full((4,), float("nan"), dtype=torch.float64, device=cuda_device)
        launches = lib.mcfd_launch_count()
        assert lib.mcfd_residual_sumsq_noalloc(R.data_ptr(), dg.n_cells, got.data_ptr(), stream) == 0
        assert lib.mcfd_launch_count() - launches == 2  # its two kernels are counted like every other launch
        torch.cuda.synchronize()
        np.testing.assert_array_equal(got.cpu().numpy(), expected.cpu().numpy())
        np.testing.assert_allclose(got.cpu().numpy(), (R * R).sum(dim=0).cpu().numpy(), rtol=1e-12)


def test_noalloc_sumsq_rejects_sizes_beyond_its_maximum(cuda_device):
    import torch
    from meshcfd_gb300 import _lib

    lib = _lib.native()
    R = torch.ones(8, 4, dtype=torch.float64, device=cuda_device)
    out = torch.zeros(4, dtype=torch.float64, device=cuda_device)
    stream = torch.cuda.current_stream().cuda_stream
    rc = lib.mcfd_residual_sumsq_noalloc(R.data_ptr(), (1 << 30) + 1, out.data_ptr(), stream)
    assert rc == 5
    assert b"maximum" in lib.mcfd_error_string(rc)
    assert lib.mcfd_residual_sumsq_noalloc(R.data_ptr(), 0, out.data_ptr(), stream) == 1
    assert lib.mcfd_residual_sumsq_noalloc(None, 8, out.data_ptr(), stream) == 1
    torch.cuda.synchronize()
    assert torch.equal(out, torch.zeros_like(out))
