"""PyTorch custom ops over the C ABI.

Each op is a thin call into ``libmeshcfd_gb300.so`` on the current CUDA
stream; there is no CPU implementation (a CPU tensor is rejected).  The
geometry is referenced by its native handle (an integer), so the ops compose
with ``torch.compile``-free eager code and CUDA graph capture alike.
"""

from __future__ import annotations

import ctypes as C

import torch

from . import _lib

_NS = "meshcfd_gb300"


def _cfg(flux: int, recon: int, limiter: int, gamma: float, ax: float, ay: float, cfl: float = 0.5):
    cfg = _lib.Config()
    cfg.flux, cfg.reconstruction, cfg.limiter, cfg.mode = flux, recon, limiter, 0
    cfg.gamma, cfg.acceleration_x, cfg.acceleration_y, cfg.cfl = gamma, ax, ay, cfl
    return cfg


def _stream() -> int:
    return torch.cuda.current_stream().cuda_stream


def _require_cuda(*tensors):
    for t in tensors:
        if not t.is_cuda or t.dtype != torch.float64 or not t.is_contiguous():
            raise ValueError("meshcfd_gb300 ops take contiguous CUDA float64 tensors (no CPU path)")


@torch.library.custom_op(f"{_NS}::primitive", mutates_args=())
def primitive(U: torch.Tensor, geom: int, gamma: float) -> torch.Tensor:
    """conservative_to_primitive (euler.py:20-40) on the device."""
    _require_cuda(U)
    P = torch.empty_like(U)
    lib = _lib.native()
    lib.check(lib.mcfd_primitive(geom, C.byref(_cfg(0, 0, 0, gamma, 0.0, 0.0)), U.data_ptr(), P.data_ptr(), _stream()),
              "mcfd_primitive")
    return P


@primitive.register_fake
def _(U, geom, gamma):
    return torch.empty_like(U)


@torch.library.custom_op(f"{_NS}::residual", mutates_args=())
def residual(U: torch.Tensor, geom: int, flux: int, recon: int, limiter: int, gamma: float, ax: float,
             ay: float) -> torch.Tensor:
    """_residual (solver.py:2437-2718) on the device."""
    _require_cuda(U)
    R = torch.empty_like(U)
    lib = _lib.native()
    lib.check(lib.mcfd_residual(geom, C.byref(_cfg(flux, recon, limiter, gamma, ax, ay)), U.data_ptr(), R.data_ptr(),
                                _stream()), "mcfd_residual")
    return R


@residual.register_fake
def _(U, geom, flux, recon, limiter, gamma, ax, ay):
    return torch.empty_like(U)


@torch.library.custom_op(f"{_NS}::time_step", mutates_args=())
def time_step(P: torch.Tensor, geom: int, gamma: float, cfl: float, time_limit: float) -> torch.Tensor:
    """min(_stable_time_step, time_limit) (solver.py:4117-4129, 455-461) as a
    one-element device tensor."""
    _require_cuda(P)
    out = torch.empty(1, dtype=torch.float64, device=P.device)
    lib = _lib.native()
    lib.check(lib.mcfd_time_steps(geom, C.byref(_cfg(0, 0, 0, gamma, 0.0, 0.0, cfl)), P.data_ptr(), None,
                                  out.data_ptr(), float(time_limit), _stream()), "mcfd_time_steps")
    return out


@time_step.register_fake
def _(P, geom, gamma, cfl, time_limit):
    return P.new_empty(1)


@torch.library.custom_op(f"{_NS}::local_time_steps", mutates_args=())
def local_time_steps(P: torch.Tensor, geom: int, gamma: float, cfl: float) -> torch.Tensor:
    """_stable_time_steps (solver.py:4132-4343) as an (n_cells,) device tensor."""
    _require_cuda(P)
    out = torch.empty(P.shape[0], dtype=torch.float64, device=P.device)
    lib = _lib.native()
    lib.check(lib.mcfd_time_steps(geom, C.byref(_cfg(0, 0, 0, gamma, 0.0, 0.0, cfl)), P.data_ptr(), out.data_ptr(),
                                  None, float("inf"), _stream()), "mcfd_time_steps")
    return out


@local_time_steps.register_fake
def _(P, geom, gamma, cfl):
    return P.new_empty(P.shape[0])


@torch.library.custom_op(f"{_NS}::explicit_step_", mutates_args=("U",))
def explicit_step_(U: torch.Tensor, dt: torch.Tensor, geom: int, scheme: int, flux: int, recon: int, limiter: int,
                   gamma: float, ax: float, ay: float) -> None:
    """One explicit Euler / SSP-RK2 / SSP-RK3 / SSPRK(5,4) step in place
    (solver.py:532-806, 1128-1182)."""
    _require_cuda(U, dt)
    per_cell = int(dt.numel() == U.shape[0] and U.shape[0] != 1)
    lib = _lib.native()
    lib.check(lib.mcfd_explicit_step(geom, C.byref(_cfg(flux, recon, limiter, gamma, ax, ay)), scheme, U.data_ptr(),
                                     dt.data_ptr(), per_cell, _stream()), "mcfd_explicit_step")


@explicit_step_.register_fake
def _(U, dt, geom, scheme, flux, recon, limiter, gamma, ax, ay):
    return None
