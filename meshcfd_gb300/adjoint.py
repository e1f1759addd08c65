"""Discrete adjoint of a wall pressure force through SSP-RK3 time marching.

There is no counterpart in the reference (its solver is not differentiable).
The forward run is the reference's RK3 step (solver.py:566-567, 676-678,
754-756) with a fixed time step; the functional is the wall pressure force
J = sum over wall faces of p (n . d) L at the final state (`mcfd_wall_force`).
The adjoint walks the steps backwards with the transposed residual Jacobian
(`mcfd_vjp_at`, three products per step), replaying each segment of
``checkpoint_every`` steps from its stored state with the forward step, which
records every stage's state, primitive and face states
(`mcfd_explicit_step_record`), so the linearisation points are the forward
run's own, bit for bit.  For one step
U1 = U + dt R(U), U2 = 3/4 U + 1/4 (U1 + dt R(U1)), U' = 1/3 U + 2/3 (U2 + dt R(U2)):

    l2 = 2/3 (l' + dt R(U2)^T l'),   l1 = 1/4 (l2 + dt R(U1)^T l2),
    l  = 1/3 l' + 3/4 l2 + l1 + dt R(U)^T l1,

and the far-field-state gradient collects the same products' parameter parts.
"""

from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from .device import DeviceGeometry, _stream_ptr, make_config


class ResidualFunction(torch.autograd.Function):
    """R = residual(U) with the hand-written reverse mode as its backward."""

    @staticmethod
    def forward(ctx, U, geom: DeviceGeometry, cfg):
        ctx.save_for_backward(U)
        ctx.geom, ctx.cfg = geom, cfg
        return geom.residual(U.contiguous(), cfg)

    @staticmethod
    def backward(ctx, grad_R):
        (U,) = ctx.saved_tensors
        geom, cfg = ctx.geom, ctx.cfg
        out = torch.empty_like(U)
        geom.lib.check(geom.lib.mcfd_vjp(geom.handle, C.byref(cfg), U.data_ptr(), grad_R.contiguous().data_ptr(),
                                         out.data_ptr(), None, _stream_ptr()), "mcfd_vjp")
        return out, None, None


class WallForceAdjoint:
    """Forward RK3 with checkpoints and the reverse sweep for one geometry.

    ``dt``: one fixed time step, or a CUDA tensor of per-cell steps (a batch
    of cases, each with its own step).  With ``case_offsets`` (cell offsets
    of the cases of a batch) :meth:`functional_per_case` gives every case's
    wall force; the gradient of their sum restricted to a case's cells is
    that case's gradient, because the cases do not interact."""

    def __init__(self, geom: DeviceGeometry, settings, dt, direction=(1.0, 0.0), checkpoint_every: int = 20,
                 mode: str = "exact", case_offsets=None):
        self.geom = geom
        self.cfg = make_config(settings, mode)
        # the reverse sweep linearises at the forward step's own face states
        self.cfg_vjp = make_config(settings, "exact" if mode == "fma" else mode)
        dev = geom.device
        if isinstance(dt, torch.Tensor):
            if dt.shape != (geom.n_cells,) or dt.dtype != torch.float64 or not dt.is_cuda:
                raise ValueError("per-cell dt must be a CUDA float64 tensor of shape (n_cells,)")
            self.per_cell = True
            self.dt_dev = dt.contiguous()
            self.dt = self.dt_dev.view(-1, 1)
            self.far_dt = self.dt_dev[geom.far_owner].view(-1, 1)
        else:
            self.per_cell = False
            self.dt = float(dt)
            self.dt_dev = torch.full((1,), self.dt, dtype=torch.float64, device=dev)
            self.far_dt = self.dt
        self.dt_col = self.dt_dev.view(-1, 1)
        self.direction = direction
        self.k = int(checkpoint_every)
        self.case_offsets = None if case_offsets is None else np.asarray(case_offsets, dtype=np.int64)
        self.W = torch.empty(geom.n_cells, 4, dtype=torch.float64, device=dev)
        self.far = torch.zeros(max(geom.n_far_field, 1), 4, dtype=torch.float64, device=dev)
        self.far_acc = torch.zeros_like(self.far)
        self.checkpoints = []
        self.steps = 0

    # ---------------------------------------------------------------- forward
    def step(self, U):
        self.geom.explicit_step(U, self.cfg, 2, self.dt_dev)

    def functional_per_case(self, U) -> np.ndarray:
        """The wall force of every case (``case_offsets``) at state U."""
        g = self.geom
        P = g.primitive(U, self.cfg)
        w = g.wall_normal_length[:, 0] * self.direction[0] + g.wall_normal_length[:, 1] * self.direction[1]
        lengths = torch.as_tensor(np.diff(self.case_offsets), device=g.device)
        return torch.segment_reduce(P[:, 3] * w, "sum", lengths=lengths).cpu().numpy()

    def forward(self, U0: torch.Tensor, steps: int) -> torch.Tensor:
        U = U0.clone()
        self.checkpoints = [U0.clone()]
        for s in range(1, steps + 1):
            self.step(U)
            if s % self.k == 0 and s < steps:
                self.checkpoints.append(U.clone())
        self.steps = steps
        self.geom.check_status()
        return U

    def functional(self, U):
        J = (C.c_double * 1)()
        dJ = torch.empty_like(U)
        self.geom.lib.check(self.geom.lib.mcfd_wall_force(self.geom.handle, C.byref(self.cfg), U.data_ptr(),
                                                          float(self.direction[0]), float(self.direction[1]), J,
                                                          dJ.data_ptr(), _stream_ptr()), "mcfd_wall_force")
        return float(J[0]), dJ

    # --------------------------------------------------------------- reverse
    def _vjp(self, P, recon, lam, coef):
        """W = R'(U)^T lam at the state with primitive P and face states
        recon; the far-field-state gradient accumulates with weight coef dt
        (dt of each far face's owner cell)."""
        lib = self.geom.lib
        lib.check(lib.mcfd_vjp_at(self.geom.handle, C.byref(self.cfg_vjp), None, P.data_ptr(),
                                  recon.data_ptr() if recon is not None else None, lam.data_ptr(),
                                  self.W.data_ptr(), self.far.data_ptr(), _stream_ptr()), "mcfd_vjp_at")
        if self.geom.n_far_field:
            if self.per_cell:
                self.far_acc.addcmul_(self.far, self.far_dt, value=coef)
            else:
                self.far_acc.add_(self.far, alpha=coef * self.dt)
        return self.W

    def _plus_dt(self, x, w):
        """x + dt w as one kernel; a scalar dt is a 1x1 tensor, so that a
        batch (per-cell dt) and a single case round identically."""
        return torch.addcmul(x, w, self.dt_col)

    def _replay(self, U):
        """Advance U one step in place; returns, per stage, the primitive and
        face states the residual was evaluated at (the reverse sweep's
        linearisation points, written during the step)."""
        g, lib, n = self.geom, self.geom.lib, self.geom.n_cells
        dev = g.device
        Ps = [torch.empty(n, 4, dtype=torch.float64, device=dev) for _ in range(3)]
        recons = ([torch.empty(int(g.info.n_limiter), 4, dtype=torch.float64, device=dev) for _ in range(3)]
                  if self.cfg.reconstruction != 0 else [None] * 3)
        p_ptrs = (C.c_void_p * 3)(*[t.data_ptr() for t in Ps])
        r_ptrs = (C.c_void_p * 3)(*[t.data_ptr() if t is not None else None for t in recons])
        lib.check(lib.mcfd_explicit_step_record(g.handle, C.byref(self.cfg), 2, U.data_ptr(), self.dt_dev.data_ptr(),
                                                int(self.per_cell), p_ptrs, r_ptrs, 3, _stream_ptr()),
                  "mcfd_explicit_step_record")
        return Ps, recons

    def backward(self, lam_final: torch.Tensor) -> torch.Tensor:
        """Adjoint of the initial state; the far-field-state gradient per
        far-field face accumulates in ``self.far_acc``.  Each segment is
        replayed from its checkpoint with the forward step, keeping every
        step's stage states and their primitive and face states."""
        dt = self.dt
        lam = lam_final.clone()
        self.far_acc.zero_()
        for seg in range(len(self.checkpoints) - 1, -1, -1):
            start = seg * self.k
            end = min(start + self.k, self.steps)
            U = self.checkpoints[seg].clone()
            records = [self._replay(U) for _ in range(start, end)]
            for Ps, recons in reversed(records):
                w = self._vjp(Ps[2], recons[2], lam, 2.0 / 3.0)
                lam2 = self._plus_dt(lam, w).mul_(2.0 / 3.0)
                w = self._vjp(Ps[1], recons[1], lam2, 0.25)
                lam1 = self._plus_dt(lam2, w).mul_(0.25)
                w = self._vjp(Ps[0], recons[0], lam1, 1.0)
                new = self._plus_dt(lam1, w)
                new.add_(lam, alpha=1.0 / 3.0).add_(lam2, alpha=0.75)
                lam = new
            del records
        self.geom.check_status()
        return lam

    def gradient(self, U0: torch.Tensor, steps: int):
        """J, dJ/dU0 (device), far-field-state gradient per far face (host)."""
        UN = self.forward(U0, steps)
        J, dJ = self.functional(UN)
        lam0 = self.backward(dJ)
        return J, lam0, self.far_acc.cpu().numpy()


class WallForceFunction(torch.autograd.Function):
    """J(U0) = wall force after ``steps`` RK3 steps from U0, as a torch op whose
    backward is the checkpointed discrete adjoint."""

    @staticmethod
    def forward(ctx, U0, adjoint: WallForceAdjoint, steps: int):
        UN = adjoint.forward(U0.contiguous(), int(steps))
        J, dJ = adjoint.functional(UN)
        ctx.adjoint, ctx.dJ = adjoint, dJ
        return torch.tensor(J, dtype=torch.float64, device=U0.device)

    @staticmethod
    def backward(ctx, grad_J):
        lam0 = ctx.adjoint.backward(ctx.dJ)
        return grad_J * lam0, None, None


def conservative_jacobian_T(P: np.ndarray, lam: np.ndarray, gamma: float) -> np.ndarray:
    """Per cell, (dU/dP)^T lambda for U = primitive_to_conservative(P)
    (euler.py:8-17): the chain rule from an initial state given in
    primitive variables (rows of P) to those variables."""
    rho, u, v, p = P.T
    l0, l1, l2, l3 = lam.T
    out = np.column_stack((
        l0 + l1 * u + l2 * v + l3 * 0.5 * (u * u + v * v),
        l1 * rho + l3 * rho * u,
        l2 * rho + l3 * rho * v,
        l3 / (gamma - 1.0),
    ))
    return out
