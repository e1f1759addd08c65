"""ORACLE — test infrastructure only.

Restatement of the reference's implicit Euler (src/meshcfd/core/solver.py:
1185-1567) on top of the C oracle's residual.  The linear algebra uses SciPy
(scipy.sparse, spsolve_triangular, gmres: the reference's own dependency,
pyproject.toml `scipy>=1.14`), called the way the reference calls it.
"""

from __future__ import annotations

import math
from dataclasses import replace

import numpy as np
from scipy.sparse import coo_matrix, eye, kron, tril, triu
from scipy.sparse.linalg import LinearOperator, gmres, spsolve_triangular

from .oracle import Oracle, OracleError


class ImplicitOracle:
    def __init__(self, geometry):
        self.g = geometry
        self.orc = Oracle(geometry)

    # solver.py:1185-1323 (LU-SGS branch)
    def preconditioner(self, primitive, settings, time_step):
        g = self.g
        C = len(primitive)
        diagonal = np.ones(C)
        rows = list(range(C))
        cols = list(range(C))
        entries = [1.0] * C
        sound = np.sqrt(settings.gamma * primitive[:, 3] / primitive[:, 0])
        dt = np.full(C, time_step, dtype=float) if np.ndim(time_step) == 0 else np.asarray(time_step, dtype=float)
        faces = np.asarray(g.interior_faces)
        if len(faces):
            o, n = g.owners[faces], g.neighbours[faces]
            nrm = g.face_normals[faces]
            radius = np.maximum(np.abs(np.sum(primitive[o, 1:3] * nrm, axis=1)) + sound[o],
                                np.abs(np.sum(primitive[n, 1:3] * nrm, axis=1)) + sound[n])
            coef = 0.5 * radius * g.face_lengths[faces]
            oc, nc = dt[o] * coef, dt[n] * coef
            np.add.at(diagonal, o, oc / g.areas[o])
            np.add.at(diagonal, n, nc / g.areas[n])
            rows += o.tolist(); cols += n.tolist(); entries += (-oc / g.areas[o]).tolist()
            rows += n.tolist(); cols += o.tolist(); entries += (-nc / g.areas[n]).tolist()
        fa, fb = np.asarray(g.periodic_faces_a), np.asarray(g.periodic_faces_b)
        if len(fa):
            oa, ob = g.owners[fa], g.owners[fb]
            radius = np.maximum(np.abs(np.sum(primitive[oa, 1:3] * g.face_normals[fa], axis=1)) + sound[oa],
                                np.abs(np.sum(primitive[ob, 1:3] * g.face_normals[fb], axis=1)) + sound[ob])
            coef = 0.5 * radius * g.face_lengths[fa]
            ca, cb = dt[oa] * coef, dt[ob] * coef
            np.add.at(diagonal, oa, ca / g.areas[oa])
            np.add.at(diagonal, ob, cb / g.areas[ob])
            rows += oa.tolist(); cols += ob.tolist(); entries += (-ca / g.areas[oa]).tolist()
            rows += ob.tolist(); cols += oa.tolist(); entries += (-cb / g.areas[ob]).tolist()
        bf = np.flatnonzero(np.asarray(g.neighbours) < 0)
        if len(bf):
            o = g.owners[bf]
            radius = np.abs(np.sum(primitive[o, 1:3] * g.face_normals[bf], axis=1)) + sound[o]
            np.add.at(diagonal, o, dt[o] * radius * g.face_lengths[bf] / g.areas[o])
        for i, v in enumerate(diagonal):
            entries[i] = v
        A = coo_matrix((entries, (rows, cols)), shape=(C, C)).tocsc()
        B = kron(A, eye(4, format="csc"), format="csc")
        D = np.maximum(np.repeat(A.diagonal(), 4), 1e-14)
        lower, upper = tril(B, format="csr"), triu(B, format="csr")

        def apply(v):
            y = spsolve_triangular(lower, v, lower=True)
            return spsolve_triangular(upper, D * y, lower=False)

        return LinearOperator((4 * C, 4 * C), matvec=apply, dtype=float)

    # solver.py:1532-1567
    def operator(self, state, rate, scale, time_step, settings1):
        shape = state.shape
        snorm = float(np.linalg.norm(state / scale))
        fd = math.sqrt(np.finfo(float).eps)

        def mv(v):
            d = v.reshape(shape)
            dn = float(np.linalg.norm(d))
            if dn == 0.0:
                return v.copy()
            eps = fd * max(1.0, snorm) / dn
            pr = self.orc.residual(state + eps * scale * d, settings1)
            jv = (pr - rate) / eps
            step = time_step if np.ndim(time_step) == 0 else np.asarray(time_step)[:, None]
            return (d - step * jv / scale).ravel()

        return LinearOperator((state.size, state.size), matvec=mv, dtype=float)

    @staticmethod
    def scales(state, primitive, gamma):
        """solver.py:1393-1413"""
        rho = max(float(np.max(primitive[:, 0])), 1e-12)
        speed = max(float(np.max(np.abs(primitive[:, 1:3]))),
                    float(np.max(np.sqrt(gamma * primitive[:, 3] / primitive[:, 0]))), 1e-12)
        s = np.maximum(np.max(np.abs(state), axis=0), 1e-12)
        s[0] = max(s[0], rho)
        s[1:3] = np.maximum(s[1:3], rho * speed)
        s[3] = max(s[3], rho * speed**2, float(np.max(primitive[:, 3])) / (gamma - 1.0))
        return s[None, :]

    # solver.py:1489-1529
    @staticmethod
    def solve_gmres(op, M, b, tol, max_iter, m):
        x = np.zeros_like(b)
        used = 0
        while used < max_iter:
            count = [0]
            restart = min(m, max_iter - used)
            x, info = gmres(op, b, x0=x, M=M, restart=restart, maxiter=1, rtol=tol, atol=0.0,
                            callback=lambda _r: count.__setitem__(0, count[0] + 1), callback_type="pr_norm")
            used += count[0]
            if info == 0:
                return x, used
            if info < 0:
                raise OracleError(f"Implicit Euler GMRES broke down (status {info}).")
            if count[0] == 0:
                break
        raise OracleError("Implicit Euler GMRES did not converge")

    # solver.py:1371-1486 (flow-only state)
    def solve_once(self, initial, time_step, settings):
        settings1 = replace(settings, reconstruction="First order")
        state = initial.copy()
        P = self.orc.primitive(state, settings.gamma)
        scale = self.scales(state, P, settings.gamma)
        step = time_step if np.ndim(time_step) == 0 else np.asarray(time_step)[:, None]

        def evaluate(c):
            rate = self.orc.residual(c, settings)
            return rate, c - initial - step * rate

        for _ in range(12):
            rate, eq = evaluate(state)
            seq = eq / scale
            en = float(np.max(np.abs(seq)))
            un = float(np.max(np.abs((state - initial) / scale)))
            if en <= 1e-9 * max(1.0, un):
                return state
            P = self.orc.primitive(state, settings.gamma)
            M = self.preconditioner(P, settings1, time_step)
            jr = self.orc.residual(state, settings1)
            op = self.operator(state, jr, scale, time_step, settings1)
            corr, _ = self.solve_gmres(op, M, -seq.ravel(), settings.gmres_tolerance, settings.gmres_max_iterations,
                                       settings.gmres_krylov_dimension)
            accepted = False
            damping = 1.0
            for _ in range(8):
                cand = state + damping * corr.reshape(state.shape) * scale
                try:
                    _, ceq = evaluate(cand)
                    cn = float(np.max(np.abs(ceq / scale)))
                except (OracleError, ValueError, FloatingPointError):
                    cn = math.inf
                if cn < en:
                    state = cand
                    accepted = True
                    break
                damping *= 0.5
            if not accepted:
                raise OracleError("Implicit Euler Newton iteration could not reduce its residual.")
        raise OracleError("Implicit Euler Newton iteration did not converge.")

    # solver.py:1337-1368
    def step(self, initial, time_step, settings, allow_time_step_reduction=True):
        attempted = float(time_step) if np.ndim(time_step) == 0 else np.asarray(time_step, dtype=float).copy()
        last = None
        for _ in range(12 if allow_time_step_reduction else 1):
            try:
                return self.solve_once(initial, attempted, settings), attempted
            except OracleError as error:
                last = error
                attempted *= 0.5
        raise OracleError(f"Implicit Euler could not converge: {last}")
