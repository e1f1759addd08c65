"""ORACLE — test infrastructure only; never part of the product path.

NumPy restatement of the reference's laminar viscous terms (no SST):
_dynamic_viscosity (solver.py:2721-2737), _viscous_inlet_states (2740-2785),
_viscous_gradients (3615-3714) with weighted_least_squares_gradients
(_kernels.py:163-205), _viscous_flux (3717-3747), _viscous_residual
(3750-4114) and the viscous part of _stable_time_steps (4245-4335).  Same
loop structure and expression order; np.dot of two 2-vectors and the 3x2 @ 2
products are NumPy's own (BLAS), as in the reference.
"""

from __future__ import annotations

import numpy as np


class OracleViscousError(ValueError):
    pass


def dynamic_viscosity(temperature, s):
    if s.viscosity_model == "Constant":
        return np.full_like(temperature, s.dynamic_viscosity, dtype=float)
    if s.viscosity_model == "Sutherland":
        tref = s.sutherland_reference_temperature
        mu = s.sutherland_reference_viscosity * (temperature / tref) ** 1.5
        mu *= (tref + s.sutherland_temperature) / (temperature + s.sutherland_temperature)
        if not np.isfinite(mu).all() or np.any(mu <= 0.0):
            raise OracleViscousError("Sutherland law produced an invalid viscosity.")
        return mu
    return np.zeros_like(temperature, dtype=float)


def _conductivity(mu, s):
    return mu * s.gamma * s.gas_constant / ((s.gamma - 1.0) * s.prandtl_number)


def far_field_states(inside, far, normals, gamma):
    """_far_field_boundary_states (solver.py:4350-4409), NumPy form."""
    ext = inside.copy()
    ni = np.sum(inside[:, 1:3] * normals, axis=1)
    nf = np.sum(far[:, 1:3] * normals, axis=1)
    ci = np.sqrt(gamma * inside[:, 3] / inside[:, 0])
    cf = np.sqrt(gamma * far[:, 3] / far[:, 0])
    inflow = ni <= -ci
    ext[inflow] = far[inflow]
    sub = ~inflow & (ni < ci)
    if np.any(sub):
        out_inv = ni[sub] + 2.0 * ci[sub] / (gamma - 1.0)
        in_inv = nf[sub] - 2.0 * cf[sub] / (gamma - 1.0)
        vb = 0.5 * (out_inv + in_inv)
        cb = 0.25 * (gamma - 1.0) * (out_inv - in_inv)
        src = np.where((vb < 0.0)[:, None], far[sub], inside[sub])
        entropy = src[:, 3] / src[:, 0] ** gamma
        rho = (cb * cb / (gamma * entropy)) ** (1.0 / (gamma - 1.0))
        p = entropy * rho ** gamma
        n = normals[sub]
        t = np.column_stack((-n[:, 1], n[:, 0]))
        vt = np.sum(src[:, 1:3] * t, axis=1)
        vel = vb[:, None] * n + vt[:, None] * t
        ext[sub] = np.column_stack((rho, vel, p))
    return ext


def inlet_states(P, g, s, orc):
    """Exterior states of the inlet-type faces from the cell values."""
    states = {int(f): st for f, st in zip(g.velocity_inlet_faces, g.velocity_inlet_states)}
    owners = np.asarray(g.owners)
    k = 0
    for boundary in getattr(g, "pressure_inlets", ()):
        ext = orc.boundary_states(k, P[owners[boundary.faces]], s.gamma, s.gas_constant)
        states.update({int(f): st for f, st in zip(boundary.faces, ext)})
        k += 1
    for boundary in getattr(g, "mass_flow_inlets", ()):
        ext = orc.boundary_states(k, P[owners[boundary.faces]], s.gamma, s.gas_constant)
        states.update({int(f): st for f, st in zip(boundary.faces, ext)})
        k += 1
    if len(g.far_field_faces):
        faces = np.asarray(g.far_field_faces)
        ext = far_field_states(P[owners[faces]], np.asarray(g.far_field_states).reshape(-1, 4),
                               np.asarray(g.face_normals).reshape(-1, 2)[faces], s.gamma)
        states.update({int(f): st for f, st in zip(faces, ext)})
    return states


def weighted_least_squares(n_cells, src, dx, dy, diff):
    m = diff.shape[1]
    xx, xy, yy = np.zeros(n_cells), np.zeros(n_cells), np.zeros(n_cells)
    bx, by = np.zeros((n_cells, m)), np.zeros((n_cells, m))
    for e in range(len(src)):
        c = src[e]
        w = 1.0 / max(dx[e] * dx[e] + dy[e] * dy[e], 1e-300)
        wx, wy = w * dx[e], w * dy[e]
        xx[c] += wx * dx[e]
        xy[c] += wx * dy[e]
        yy[c] += wy * dy[e]
        bx[c] += wx * diff[e]
        by[c] += wy * diff[e]
    grad = np.zeros((n_cells, m, 2))
    det = xx * yy - xy * xy
    ok = det > 1e-14 * np.maximum(xx * yy, 1e-300)
    inv = np.zeros(n_cells)
    inv[ok] = 1.0 / det[ok]
    for k in range(m):
        grad[ok, k, 0] = (bx[ok, k] * yy[ok] - by[ok, k] * xy[ok]) * inv[ok]
        grad[ok, k, 1] = (by[ok, k] * xx[ok] - bx[ok, k] * xy[ok]) * inv[ok]
    return grad


def _walls(g):
    return {int(f): b for b in getattr(g, "wall_thermal_boundaries", ()) for f in b.faces}


def _no_slip(mechanical):
    return mechanical in ("No-slip", "Prescribed velocity")


def viscous_gradients(P, g, s, orc):
    rho = P[:, 0]
    T = P[:, 3] / (rho * s.gas_constant)
    if not np.isfinite(T).all() or np.any(T <= 0.0):
        raise OracleViscousError("Viscous flow requires finite positive temperature.")
    cv = np.column_stack((P[:, 1:3], T))
    src = np.asarray(g.gradient_sources)
    nb = np.asarray(g.gradient_neighbours)
    diff = [cv[nb] - cv[src]]
    srcs, dxs, dys = [src], [np.asarray(g.gradient_dx)], [np.asarray(g.gradient_dy)]
    inlet = {f: np.array((st[1], st[2], st[3] / (st[0] * s.gas_constant)))
             for f, st in inlet_states(P, g, s, orc).items()}
    walls = _walls(g)
    owners = np.asarray(g.owners)
    normals_all = np.asarray(g.face_normals).reshape(-1, 2)
    fc = np.asarray(g.face_centers).reshape(-1, 2)
    centers = np.asarray(g.centers).reshape(-1, 2)
    b_src, b_dx, b_dy, b_diff = [], [], [], []
    for f in np.asarray(g.diffusive_boundary_faces):
        o = int(owners[f])
        n = normals_all[f]
        off = fc[f] - centers[o]
        kind = g.patch_kinds[int(g.patch_ids[f])]
        nd = float(np.dot(off, n))
        ghost_off = 2.0 * nd * n if kind in ("Wall", "Symmetry") else 2.0 * off
        ghost = cv[o].copy()
        if kind == "Wall":
            wall = walls[int(f)]
            if _no_slip(wall.mechanical_condition):
                ghost[:2] = 2.0 * np.asarray(g.wall_velocities).reshape(-1, 2)[f] - ghost[:2]
            else:
                ghost[:2] -= 2.0 * float(np.dot(ghost[:2], n)) * n
            if wall.condition == "Temperature":
                ghost[2] = 2.0 * wall.value - cv[o, 2]
            else:
                mu = float(dynamic_viscosity(T[o:o + 1], s)[0])
                k = _conductivity(mu, s)
                nd2 = float(np.dot(off, n))
                ghost[2] += 2.0 * nd2 * wall.value / k
        elif kind == "Symmetry":
            vel = cv[o, :2]
            ghost[:2] -= 2.0 * float(np.dot(vel, n)) * n
        elif int(f) in inlet:
            ghost = 2.0 * inlet[int(f)] - ghost
        b_src.append(o)
        b_dx.append(ghost_off[0])
        b_dy.append(ghost_off[1])
        b_diff.append(ghost - cv[o])
    if b_src:
        srcs.append(np.asarray(b_src, dtype=int))
        dxs.append(np.asarray(b_dx))
        dys.append(np.asarray(b_dy))
        diff = np.vstack((diff[0], np.asarray(b_diff)))
    else:
        diff = diff[0]
    src_all = np.concatenate(srcs)
    if not len(src_all):
        return np.zeros((len(P), 3, 2))
    return weighted_least_squares(len(P), src_all, np.concatenate(dxs), np.concatenate(dys), diff)


def viscous_flux(grad, vel, mu, k, normals):
    du_dx, du_dy = grad[:, 0, 0], grad[:, 0, 1]
    dv_dx, dv_dy = grad[:, 1, 0], grad[:, 1, 1]
    div = du_dx + dv_dy
    txx = mu * (2.0 * du_dx - (2.0 / 3.0) * div)
    tyy = mu * (2.0 * dv_dy - (2.0 / 3.0) * div)
    txy = mu * (du_dy + dv_dx)
    tx = txx * normals[:, 0] + txy * normals[:, 1]
    ty = txy * normals[:, 0] + tyy * normals[:, 1]
    q = k * np.sum(grad[:, 2, :] * normals, axis=1)
    return np.column_stack((np.zeros(len(normals)), tx, ty, vel[:, 0] * tx + vel[:, 1] * ty + q))


def viscous_residual(P, g, s, orc, divergence):
    """``divergence(flux)``: the reference's CSR product
    interior_divergence_operator @ flux (the oracle's own, from the C side)."""
    T = P[:, 3] / (P[:, 0] * s.gas_constant)
    cv = np.column_stack((P[:, 1:3], T))
    mu = dynamic_viscosity(T, s)
    kc = _conductivity(mu, s)
    grad = viscous_gradients(P, g, s, orc)
    R = np.zeros((len(P), 4))
    owners = np.asarray(g.owners)
    neighbours = np.asarray(g.neighbours)
    normals_all = np.asarray(g.face_normals).reshape(-1, 2)
    lengths = np.asarray(g.face_lengths)
    areas = np.asarray(g.areas)
    faces = np.asarray(g.interior_faces)
    if len(faces):
        o, n = owners[faces], neighbours[faces]
        flux = viscous_flux(0.5 * (grad[o] + grad[n]), 0.5 * (P[o, 1:3] + P[n, 1:3]), 0.5 * (mu[o] + mu[n]),
                            0.5 * (kc[o] + kc[n]), normals_all[faces])
        R -= divergence(flux)
    fa, fb = np.asarray(g.periodic_faces_a), np.asarray(g.periodic_faces_b)
    if len(fa):
        oa, ob = owners[fa], owners[fb]
        flux = viscous_flux(0.5 * (grad[oa] + grad[ob]), 0.5 * (P[oa, 1:3] + P[ob, 1:3]), 0.5 * (mu[oa] + mu[ob]),
                            0.5 * (kc[oa] + kc[ob]), normals_all[fa])
        integ = flux * lengths[fa, None]
        np.add.at(R, oa, integ / areas[oa, None])
        np.add.at(R, ob, -integ / areas[ob, None])
    walls = _walls(g)
    inlet = inlet_states(P, g, s, orc)
    fc = np.asarray(g.face_centers).reshape(-1, 2)
    centers = np.asarray(g.centers).reshape(-1, 2)
    wv = np.asarray(g.wall_velocities).reshape(-1, 2)
    for f in np.asarray(g.diffusive_boundary_faces):
        o = int(owners[f])
        n = normals_all[f]
        off = fc[f] - centers[o]
        nd = float(np.dot(off, n))
        if nd <= 1e-14:
            raise OracleViscousError("Boundary face has invalid cell-center distance.")
        kind = g.patch_kinds[int(g.patch_ids[f])]
        fg = grad[o].copy()
        bv = np.array((P[o, 1], P[o, 2], T[o]))
        if kind == "Wall":
            b = walls[int(f)]
            if _no_slip(b.mechanical_condition):
                w = wv[f]
                for comp in (0, 1):
                    dn = (w[comp] - bv[comp] - float(np.dot(fg[comp], off - nd * n))) / nd
                    fg[comp] += (dn - float(np.dot(fg[comp], n))) * n
                    bv[comp] = w[comp]
            else:
                tan_off = off - nd * n
                nvel = float(np.dot(bv[:2], n))
                bv[:2] += fg[:2] @ off
                bv[:2] -= float(np.dot(bv[:2], n)) * n
                gnv = n[0] * fg[0] + n[1] * fg[1]
                dn = -(nvel + float(np.dot(gnv, tan_off))) / nd
                desired = np.outer(dn * n, n)
                vg = fg[:2]
                vg += desired - (vg @ n)[:, None] * n
            if b.condition == "Temperature":
                dn = (b.value - bv[2] - float(np.dot(fg[2], off - nd * n))) / nd
                bv[2] = b.value
            else:
                dn = b.value / kc[o]
                bv[2] += float(np.dot(fg[2], off))
            fg[2] += (dn - float(np.dot(fg[2], n))) * n
        elif kind == "Symmetry":
            nvel = float(np.dot(bv[:2], n))
            dvel = -nvel / nd * n
            for comp in (0, 1):
                fg[comp] += (dvel[comp] - float(np.dot(fg[comp], n))) * n
            fg[2] -= float(np.dot(fg[2], n)) * n
            bv[:2] -= nvel * n
        else:
            st = inlet.get(int(f))
            if st is not None:
                bv = np.array((st[1], st[2], st[3] / (st[0] * s.gas_constant)))
                for comp in range(3):
                    dn = (bv[comp] - cv[o, comp] - float(np.dot(fg[comp], off - nd * n))) / nd
                    fg[comp] += (dn - float(np.dot(fg[comp], n))) * n
            else:
                fg -= np.outer(fg @ n, n)
                bv += fg @ off
        face_mu = float(dynamic_viscosity(np.array([bv[2]]), s)[0])
        face_k = _conductivity(face_mu, s)
        flux = viscous_flux(fg[None, :, :], bv[None, :2], np.array([face_mu]), np.array([face_k]), n[None, :])[0]
        if kind == "Wall" and walls[int(f)].condition == "Heat Flux":
            flux[3] = walls[int(f)].value
        R[o] += flux * lengths[f] / areas[o]
    return R


def diffusion_sum(P, g, s):
    """The viscous part of _stable_time_steps (solver.py:4250-4330); the
    caller adds 2 x this to the convective spectral sum."""
    T = P[:, 3] / (P[:, 0] * s.gas_constant)
    mu = dynamic_viscosity(T, s)
    eff = np.maximum((4.0 / 3.0) * mu / P[:, 0], mu / (P[:, 0] * min(s.prandtl_number, 0.9)))
    out = np.zeros(len(P))
    owners = np.asarray(g.owners)
    neighbours = np.asarray(g.neighbours)
    normals_all = np.asarray(g.face_normals).reshape(-1, 2)
    lengths = np.asarray(g.face_lengths)
    centers = np.asarray(g.centers).reshape(-1, 2)
    fc = np.asarray(g.face_centers).reshape(-1, 2)
    faces = np.asarray(g.interior_faces)
    if len(faces):
        o, n = owners[faces], neighbours[faces]
        dist = np.abs(np.sum((centers[n] - centers[o]) * normals_all[faces], axis=1))
        contrib = np.maximum(eff[o], eff[n]) * lengths[faces] / np.maximum(dist, 1e-14)
        np.add.at(out, o, contrib)
        np.add.at(out, n, contrib)
    fa, fb = np.asarray(g.periodic_faces_a), np.asarray(g.periodic_faces_b)
    if len(fa):
        oa, ob = owners[fa], owners[fb]
        dist = np.abs(np.sum((fc[fa] - centers[oa]) * normals_all[fa], axis=1)) + \
            np.abs(np.sum((fc[fb] - centers[ob]) * normals_all[fb], axis=1))
        contrib = np.maximum(eff[oa], eff[ob]) * lengths[fa] / np.maximum(dist, 1e-14)
        np.add.at(out, oa, contrib)
        np.add.at(out, ob, contrib)
    for f in np.asarray(g.diffusive_boundary_faces):
        o = owners[f]
        dist = abs(float(np.dot(fc[f] - centers[o], normals_all[f])))
        out[o] += eff[o] * lengths[f] / max(dist, 1e-14)
    return out
