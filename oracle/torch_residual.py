"""FP64 PyTorch-op restatement of the inviscid residual, for autograd checks.

Test infrastructure only (the product never imports it): the residual of
solver._residual (solver.py:2437-2718) written with index_select /
index_add_ / scatter_reduce so that torch autograd differentiates it — with
respect to the conservative state and to the far-field states — as an
independent cross-check of the hand-written reverse mode.  It follows the
same formulas as the C restatement (first order / MUSCL linear with the four
limiters of _kernels.py:10-67, Rusanov / HLLC / Roe of euler.py:80-262,
wall / symmetry, periodic, velocity-inlet, pressure-outlet and far-field
boundaries of solver.py:2502-2625, far-field states of solver.py:4350-4409,
body force of solver.py:2700-2712) but in its own operation order, so values
agree with the oracle to rounding (~1e-13), not bit for bit.
"""

from __future__ import annotations

import math

import numpy as np

import torch

FLUX = {"Rusanov": 0, "HLLC": 1, "Roe": 2}
LIMITER = {"Barth-Jespersen": 0, "Minmod": 1, "Van Leer": 2, "Venkatakrishnan": 3, "Venkatakrishnan K": 4}


def _t(a, dtype=torch.float64, shape=None):
    arr = np.asarray(a)
    if shape is not None:
        arr = arr.reshape(shape)
    return torch.as_tensor(np.ascontiguousarray(arr), dtype=dtype)


def primitive(U, gamma):
    rho = U[:, 0]
    vx = U[:, 1] / rho
    vy = U[:, 2] / rho
    p = (gamma - 1.0) * (U[:, 3] - 0.5 * rho * (vx * vx + vy * vy))
    return torch.stack((rho, vx, vy, p), 1)


def _state_and_flux(q, n, gamma):
    rho, vx, vy, p = q.unbind(1)
    un = vx * n[:, 0] + vy * n[:, 1]
    E = p / (gamma - 1.0) + 0.5 * rho * (vx * vx + vy * vy)
    U = torch.stack((rho, rho * vx, rho * vy, E), 1)
    F = torch.stack((rho * un, rho * vx * un + p * n[:, 0], rho * vy * un + p * n[:, 1], (E + p) * un), 1)
    return U, F, un


def rusanov(L, R, n, gamma):
    UL, FL, unl = _state_and_flux(L, n, gamma)
    UR, FR, unr = _state_and_flux(R, n, gamma)
    a = unl.abs() + torch.sqrt(gamma * L[:, 3] / L[:, 0])
    b = unr.abs() + torch.sqrt(gamma * R[:, 3] / R[:, 0])
    s = torch.where(a >= b, a, b)
    return 0.5 * (FL + FR - s[:, None] * (UR - UL))


def hllc(L, R, n, gamma):
    UL, FL, unl = _state_and_flux(L, n, gamma)
    UR, FR, unr = _state_and_flux(R, n, gamma)
    cl = torch.sqrt(gamma * L[:, 3] / L[:, 0])
    cr = torch.sqrt(gamma * R[:, 3] / R[:, 0])
    wl = torch.minimum(unl - cl, unr - cr)
    wr = torch.maximum(unl + cl, unr + cr)
    den = L[:, 0] * (wl - unl) - R[:, 0] * (wr - unr)
    den = torch.where(den.abs() > 1e-14, den, torch.copysign(torch.full_like(den, 1e-14), den))
    contact = (R[:, 3] - L[:, 3] + L[:, 0] * unl * (wl - unl) - R[:, 0] * unr * (wr - unr)) / den

    def star(q, U, un, wave):
        factor = q[:, 0] * (wave - un) / (wave - contact)
        vx = q[:, 1] + (contact - un) * n[:, 0]
        vy = q[:, 2] + (contact - un) * n[:, 1]
        e = factor * (U[:, 3] / q[:, 0] + (contact - un) * (contact + q[:, 3] / (q[:, 0] * (wave - un))))
        return torch.stack((factor, factor * vx, factor * vy, e), 1)

    fsl = FL + wl[:, None] * (star(L, UL, unl, wl) - UL)
    fsr = FR + wr[:, None] * (star(R, UR, unr, wr) - UR)
    out = torch.where((wr > 0.0)[:, None], fsr, FR)
    out = torch.where((contact >= 0.0)[:, None], fsl, out)
    return torch.where((wl >= 0.0)[:, None], FL, out)


def roe(L, R, n, gamma):
    UL, FL, unl = _state_and_flux(L, n, gamma)
    UR, FR, unr = _state_and_flux(R, n, gamma)
    nx, ny = n[:, 0], n[:, 1]
    rl, rr = torch.sqrt(L[:, 0]), torch.sqrt(R[:, 0])
    den = rl + rr
    vx = (rl * L[:, 1] + rr * R[:, 1]) / den
    vy = (rl * L[:, 2] + rr * R[:, 2]) / den
    # the reference's averaged "enthalpy" is p / rho + |u|^2 / 2 (euler.py:186-190)
    H = (rl * (L[:, 3] / L[:, 0] + 0.5 * (L[:, 1] ** 2 + L[:, 2] ** 2))
         + rr * (R[:, 3] / R[:, 0] + 0.5 * (R[:, 1] ** 2 + R[:, 2] ** 2))) / den
    un = vx * nx + vy * ny
    ut = -vx * ny + vy * nx
    c2 = (gamma - 1.0) * (H - 0.5 * (vx * vx + vy * vy))
    c = torch.sqrt(c2)
    ravg = rl * rr
    utl = -L[:, 1] * ny + L[:, 2] * nx
    utr = -R[:, 1] * ny + R[:, 2] * nx
    dr, dun, dut, dp = R[:, 0] - L[:, 0], unr - unl, utr - utl, R[:, 3] - L[:, 3]
    s = torch.stack(((dp - ravg * c * dun) / (2.0 * c2), dr - dp / c2, ravg * dut, (dp + ravg * c * dun) / (2.0 * c2)), 1)
    lam = torch.stack((un - c, un, un, un + c), 1)
    fix = (0.1 * c)[:, None]
    a = lam.abs()
    a = torch.where(a < fix, 0.5 * (a * a / fix + fix), a)
    w = a * s
    one, zero = torch.ones_like(un), torch.zeros_like(un)
    E = torch.stack((torch.stack((one, one, zero, one), 1),
                     torch.stack((un - c, un, zero, un + c), 1),
                     torch.stack((ut, ut, one, ut), 1),
                     torch.stack((H - un * c, 0.5 * (un * un + ut * ut), ut, H + un * c), 1)), 1)
    d = (E * w[:, None, :]).sum(2)
    diss = torch.stack((d[:, 0], d[:, 1] * nx - d[:, 2] * ny, d[:, 1] * ny + d[:, 2] * nx, d[:, 3]), 1)
    return 0.5 * (FL + FR - diss)


def numerical_flux(code, L, R, n, gamma):
    return (rusanov, hllc, roe)[code](L, R, n, gamma)


def far_field_states(inside, far, n, gamma):
    """Characteristic far-field ghost state (solver.py:4350-4409)."""
    ni = inside[:, 1] * n[:, 0] + inside[:, 2] * n[:, 1]
    nf = far[:, 1] * n[:, 0] + far[:, 2] * n[:, 1]
    ci = torch.sqrt(gamma * inside[:, 3] / inside[:, 0])
    cf = torch.sqrt(gamma * far[:, 3] / far[:, 0])
    out_inv = ni + 2.0 * ci / (gamma - 1.0)
    in_inv = nf - 2.0 * cf / (gamma - 1.0)
    vb = 0.5 * (out_inv + in_inv)
    cb = 0.25 * (gamma - 1.0) * (out_inv - in_inv)
    src = torch.where((vb < 0.0)[:, None], far, inside)
    entropy = src[:, 3] / src[:, 0] ** gamma
    rho = (cb * cb / (gamma * entropy)) ** (1.0 / (gamma - 1.0))
    p = entropy * rho ** gamma
    tx, ty = -n[:, 1], n[:, 0]
    vt = src[:, 1] * tx + src[:, 2] * ty
    sub = torch.stack((rho, vb * n[:, 0] + vt * tx, vb * n[:, 1] + vt * ty, p), 1)
    out = torch.where((ni >= ci)[:, None], inside, sub)
    return torch.where((ni <= -ci)[:, None], far, out)


class TorchResidual:
    """R(U, far_states) for one geometry and settings; differentiable."""

    def __init__(self, geometry, settings):
        g = geometry
        self.gamma = float(settings.gamma)
        self.flux = FLUX[settings.flux]
        self.muscl = settings.reconstruction == "MUSCL linear"
        if settings.reconstruction not in ("First order", "MUSCL linear"):
            raise NotImplementedError(settings.reconstruction)
        self.limiter = LIMITER[settings.limiter]
        self.venkat_k = float(getattr(settings, "venkatakrishnan_k", 5.0))
        self.ax, self.ay = float(settings.acceleration_x), float(settings.acceleration_y)
        i64 = torch.int64
        self.C = len(g.areas)
        self.areas = _t(g.areas)
        self.centers = _t(g.centers, shape=(-1, 2))
        self.face_centers = _t(g.face_centers, shape=(-1, 2))
        self.normals = _t(g.face_normals, shape=(-1, 2))
        self.lengths = _t(g.face_lengths)
        self.owners = _t(g.owners, i64)
        self.neighbours = _t(g.neighbours, i64)
        self.interior = _t(g.interior_faces, i64)
        self.int_own_off = _t(g.interior_owner_offsets, shape=(-1, 2))
        self.int_nb_off = _t(g.interior_neighbour_offsets, shape=(-1, 2))
        self.per_a = _t(g.periodic_faces_a, i64)
        self.per_b = _t(g.periodic_faces_b, i64)
        self.wall = _t(g.wall_faces, i64)
        self.wall_vel = _t(g.wall_velocities, shape=(-1, 2))
        self.vin = _t(g.velocity_inlet_faces, i64)
        self.vin_states = _t(g.velocity_inlet_states, shape=(-1, 4))
        self.pout = _t(g.pressure_outlet_faces, i64)
        self.pout_p = _t(g.pressure_outlet_pressures)
        self.far = _t(g.far_field_faces, i64)
        self.far_states = _t(g.far_field_states, shape=(-1, 4))
        self.gsrc = _t(g.gradient_sources, i64)
        self.gnb = _t(g.gradient_neighbours, i64)
        self.gcx = _t(g.gradient_coefficients_x)
        self.gcy = _t(g.gradient_coefficients_y)
        self.lcell = _t(g.limiter_cells, i64)
        self.ldx = _t(g.limiter_dx)
        self.ldy = _t(g.limiter_dy)

    # ------------------------------------------------------------ reconstruction
    def gradients_and_factors(self, P):
        d = P.index_select(0, self.gnb) - P.index_select(0, self.gsrc)
        gx = torch.zeros_like(P).index_add_(0, self.gsrc, self.gcx[:, None] * d)
        gy = torch.zeros_like(P).index_add_(0, self.gsrc, self.gcy[:, None] * d)
        nb = P.index_select(0, self.gnb)
        idx = self.gsrc[:, None].expand(-1, 4)
        lo = P.scatter_reduce(0, idx, nb, "amin", include_self=True)
        hi = P.scatter_reduce(0, idx, nb, "amax", include_self=True)
        c = self.lcell
        cv = P.index_select(0, c)
        inc = gx.index_select(0, c) * self.ldx[:, None] + gy.index_select(0, c) * self.ldy[:, None]
        if self.limiter == 4:  # Venkatakrishnan with K (extension): least face factor, no cap
            t = self.venkat_k * torch.sqrt(self.areas.index_select(0, c))
            e2 = ((t * t) * t)[:, None]
            d1 = torch.where(inc > 0.0, hi.index_select(0, c) - cv, lo.index_select(0, c) - cv)
            f = ((d1 * d1 + e2) + 2.0 * d1 * inc) / (((d1 * d1 + 2.0 * (inc * inc)) + d1 * inc) + e2)
            phi = torch.full_like(P, math.inf).scatter_reduce(0, c[:, None].expand(-1, 4), f, "amin",
                                                              include_self=True)
            return gx, gy, phi
        tol = 1e-14 * torch.clamp(cv.abs(), min=1.0)
        one = torch.ones_like(cv)
        up = (hi.index_select(0, c) - cv) / torch.where(inc > tol, inc, one)
        down = (lo.index_select(0, c) - cv) / torch.where(inc < -tol, inc, one)
        ratio = torch.where(inc > tol, up, torch.where(inc < -tol, down, one))
        ratio = torch.clamp(ratio, min=0.0)
        if self.limiter <= 1:
            f = torch.clamp(ratio, max=1.0)
        elif self.limiter == 2:
            f = torch.where(ratio > 0.0, torch.clamp(2.0 * ratio / (1.0 + ratio), max=1.0), torch.zeros_like(ratio))
        else:
            eps = 1e-12
            f = torch.clamp((ratio * ratio + 2.0 * ratio + eps) / (ratio * ratio + ratio + 2.0 + eps), max=1.0)
        phi = torch.ones_like(P).scatter_reduce(0, c[:, None].expand(-1, 4), f, "amin", include_self=True)
        return gx, gy, phi

    def _recon(self, P, grads, cells, off):
        q = P.index_select(0, cells)
        if grads is None:
            return q
        gx, gy, phi = grads
        inc = gx.index_select(0, cells) * off[:, 0:1] + gy.index_select(0, cells) * off[:, 1:2]
        return q + phi.index_select(0, cells) * inc

    def _boundary_offsets(self, faces):
        own = self.owners.index_select(0, faces)
        return own, self.face_centers.index_select(0, faces) - self.centers.index_select(0, own)

    # ------------------------------------------------------------------ residual
    def __call__(self, U, far_states=None):
        gamma = self.gamma
        far_states = self.far_states if far_states is None else far_states
        P = primitive(U, gamma)
        grads = self.gradients_and_factors(P) if (self.muscl and len(self.gsrc)) else None
        R = torch.zeros_like(U)
        if len(self.interior):
            f = self.interior
            o, nb = self.owners.index_select(0, f), self.neighbours.index_select(0, f)
            L = self._recon(P, grads, o, self.int_own_off)
            Rt = self._recon(P, grads, nb, self.int_nb_off)
            flux = numerical_flux(self.flux, L, Rt, self.normals.index_select(0, f), gamma)
            lf = self.lengths.index_select(0, f)[:, None]
            R = R.index_add(0, o, -(lf / self.areas.index_select(0, o)[:, None]) * flux)
            R = R.index_add(0, nb, (lf / self.areas.index_select(0, nb)[:, None]) * flux)
        if len(self.per_a):
            oa, offa = self._boundary_offsets(self.per_a)
            ob, offb = self._boundary_offsets(self.per_b)
            L = self._recon(P, grads, oa, offa)
            Rt = self._recon(P, grads, ob, offb)
            integ = numerical_flux(self.flux, L, Rt, self.normals.index_select(0, self.per_a), gamma) \
                * self.lengths.index_select(0, self.per_a)[:, None]
            R = R.index_add(0, oa, -integ / self.areas.index_select(0, oa)[:, None])
            R = R.index_add(0, ob, integ / self.areas.index_select(0, ob)[:, None])
        for kind, faces in (("wall", self.wall), ("vin", self.vin), ("pout", self.pout), ("far", self.far)):
            if not len(faces):
                continue
            own, off = self._boundary_offsets(faces)
            n = self.normals.index_select(0, faces)
            inside = self._recon(P, grads, own, off)
            if kind == "wall":
                wv = self.wall_vel.index_select(0, faces) if len(self.wall_vel) else torch.zeros_like(n)
                un = (inside[:, 1] - wv[:, 0]) * n[:, 0] + (inside[:, 2] - wv[:, 1]) * n[:, 1]
                ext = torch.stack((inside[:, 0], inside[:, 1] - 2.0 * un * n[:, 0],
                                   inside[:, 2] - 2.0 * un * n[:, 1], inside[:, 3]), 1)
            elif kind == "vin":
                ext = self.vin_states
            elif kind == "pout":
                ext = torch.cat((inside[:, :3], self.pout_p[:, None]), 1)
            else:
                ext = far_field_states(inside, far_states, n, gamma)
            fl = numerical_flux(self.flux, inside, ext, n, gamma)
            R = R.index_add(0, own, -(fl * self.lengths.index_select(0, faces)[:, None])
                            / self.areas.index_select(0, own)[:, None])
        if self.ax != 0.0 or self.ay != 0.0:
            rho = P[:, 0]
            body = torch.stack((torch.zeros_like(rho), rho * self.ax, rho * self.ay,
                                rho * (self.ax * P[:, 1] + self.ay * P[:, 2])), 1)
            R = R + body
        return R
