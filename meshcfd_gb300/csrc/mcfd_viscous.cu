// Laminar viscous terms (no SST) of the residual and the time step.
//
// * k_visc_cells: T = p / (rho R), mu (constant or Sutherland,
//   solver.py:2721-2737), conductivity mu gamma R / ((gamma - 1) Pr), and the
//   time step's effective diffusivity (solver.py:4257-4260);
// * k_visc_gradients (per cell): weighted least-squares gradients of
//   (u, v, T) (_kernels.py:163-205) over the cell's gradient entries in the
//   reference's order, then its ghost entries on diffusive boundary faces
//   (_viscous_gradients, solver.py:3615-3714);
// * k_visc_faces: the averaged face flux on interior and periodic faces
//   (_viscous_flux, solver.py:3717-3747);
// * k_visc_boundary (per diffusive boundary face): the reference's boundary
//   corrections of the face gradient and values (solver.py:3939-4114);
// * k_visc_gather (per cell): derivative = 0 - D @ flux (D the SciPy CSR
//   divergence, ascending face order), then the periodic and boundary terms
//   in the reference's np.add.at / loop order;
// * k_visc_diffusion (per cell): the time step's diffusion sum
//   (solver.py:4261-4330).
// np.dot of two 2-vectors is the BLAS dot of the reference's platform,
// fma(a1, b1, a0 * b0); a k x 2 matrix times a 2-vector (k >= 2) is its gemv,
// fma(a0, b0, a1 * b1) per row: written out here, so constant-viscosity cases
// follow the reference's rounding.  Sutherland's (T / Tref)^1.5 is NumPy's
// array power there and CUDA pow here (last-place differences).
#include "mcfd_device.cuh"
#include "mcfd_internal.h"

namespace mcfd {
namespace {

constexpr int kBlock = 128;
inline int blocks_for(int n) { return (n + kBlock - 1) / kBlock; }

__device__ __forceinline__ void flag(DevStatus* st, int bits, int cell) {
  atomicOr(&st->code, bits);
  atomicMin(&st->first_cell, cell);
}

// BLAS dot of two 2-vectors / gemv row of the reference's platform
__device__ __forceinline__ double dot2(double a0, double a1, double b0, double b1) { return ::fma(a1, b1, a0 * b0); }
__device__ __forceinline__ double gemv_row(double a0, double a1, double b0, double b1) {
  return ::fma(a0, b0, a1 * b1);
}

struct Visc {
  int model;
  double mu0, suth_mu, suth_t, suth_s, gamma, R, pr;
};

// _dynamic_viscosity; *bad set when Sutherland's law gives an invalid value
__device__ __forceinline__ double viscosity(const Visc& v, double T, bool* bad) {
  if (v.model == MCFD_VISC_CONSTANT) return v.mu0;
  double mu = v.suth_mu * pow(div_rn(T, v.suth_t), 1.5);
  mu *= div_rn(v.suth_t + v.suth_s, T + v.suth_s);
  if (!isfinite(mu) || !(mu > 0.0)) *bad = true;
  return mu;
}
__device__ __forceinline__ double conductivity(const Visc& v, double mu) {
  return div_rn(mu * v.gamma * v.R, (v.gamma - 1.0) * v.pr);
}

// _viscous_flux for one face: components 1..3 (the mass component is zero)
__device__ __forceinline__ void viscous_flux(const double g[6], double u, double v, double mu, double k, double nx,
                                             double ny, double out[4]) {
  const double du_dx = g[0], du_dy = g[1], dv_dx = g[2], dv_dy = g[3];
  const double div = du_dx + dv_dy;
  const double txx = mu * (2.0 * du_dx - (2.0 / 3.0) * div);
  const double tyy = mu * (2.0 * dv_dy - (2.0 / 3.0) * div);
  const double txy = mu * (du_dy + dv_dx);
  const double tx = txx * nx + txy * ny;
  const double ty = txy * nx + tyy * ny;
  const double q = k * (g[4] * nx + g[5] * ny);
  out[0] = 0.0;
  out[1] = tx;
  out[2] = ty;
  out[3] = u * tx + v * ty + q;
}

__global__ void __launch_bounds__(kBlock) k_visc_cells(DevGeom g, const double* __restrict__ P, Visc vs,
                                                       double* __restrict__ cell) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= g.n_cells) return;
  const St4 p = ld4(P + 4 * (size_t)c);
  const double T = div_rn(p.d, p.a * vs.R);
  bool bad = false;
  const double mu = viscosity(vs, T, &bad);
  int bits = 0;
  if (!isfinite(T) || !(T > 0.0)) bits |= MCFD_S_VISC_TEMPERATURE;
  if (bad) bits |= MCFD_S_VISC_SUTHERLAND;
  if (bits) flag(g.status, bits, c);
  const double k = conductivity(vs, mu);
  const double prm = vs.pr < 0.9 ? vs.pr : 0.9;
  const double e1 = div_rn((4.0 / 3.0) * mu, p.a), e2 = div_rn(mu, p.a * prm);
  st4(cell + 4 * (size_t)c, St4{T, mu, k, e2 > e1 ? e2 : e1});
}

// exterior (u, v, T) of an inlet-type face from the cell values
__device__ __forceinline__ bool inlet_values(const DevGeom& g, const double* P, int j, int o, double2 n, double gamma,
                                             double R, double out[3], int* bits) {
  const int code = g.diff_inlet[j];
  const int src = code >> 28, idx = code & 0x0fffffff;
  St4 st;
  if (src == 1) st = ld4(g.ff_vin_state + 4 * (size_t)idx);
  else if (src == 2) st = ld4(g.bc_ext_dt + 4 * (size_t)idx);
  else if (src == 3) *bits |= far_field_state(ld4(P + 4 * (size_t)o), ld4(g.ff_far_state + 4 * (size_t)idx), n.x, n.y,
                                              gamma, &st);
  else return false;
  out[0] = st.b;
  out[1] = st.c;
  out[2] = div_rn(st.d, st.a * R);
  return true;
}

__global__ void __launch_bounds__(kBlock) k_visc_gradients(DevGeom g, const double* __restrict__ P, Visc vs,
                                                           const double* __restrict__ cell,
                                                           double* __restrict__ grad) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= g.n_cells) return;
  const St4 p = ld4(P + 4 * (size_t)c);
  const St4 cc = ld4(cell + 4 * (size_t)c);
  const double cv[3] = {p.b, p.c, cc.a};
  double xx = 0.0, xy = 0.0, yy = 0.0, bx[3] = {0.0, 0.0, 0.0}, by[3] = {0.0, 0.0, 0.0};
  auto add = [&](double dx, double dy, const double diff[3]) {
    const double r2 = dx * dx + dy * dy;
    const double w = div_rn(1.0, r2 > 1e-300 ? r2 : 1e-300);
    const double wx = w * dx, wy = w * dy;
    xx += wx * dx;
    xy += wx * dy;
    yy += wy * dy;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      bx[k] += wx * diff[k];
      by[k] += wy * diff[k];
    }
  };
  for (int e = g.grad_ptr[c], e1 = g.grad_ptr[c + 1]; e < e1; ++e) {
    const int nb = g.grad_nb[e];
    const St4 q = ld4(P + 4 * (size_t)nb);
    const double diff[3] = {q.b - cv[0], q.c - cv[1], cell[4 * (size_t)nb] - cv[2]};
    const double2 d = g.grad_d[e];
    add(d.x, d.y, diff);
  }
  int bits = 0;
  for (int i = g.vb_ptr[c], i1 = g.vb_ptr[c + 1]; i < i1; ++i) {
    const int j = g.vb_j[i];
    const double2 nn = g.diff_normal[j];
    const double nx = nn.x, ny = nn.y;
    double ghost[3] = {cv[0], cv[1], cv[2]};
    const int kind = g.diff_kind[j];
    if (kind == MCFD_DIFF_WALL_NO_SLIP || kind == MCFD_DIFF_WALL_SLIP) {
      if (kind == MCFD_DIFF_WALL_NO_SLIP) {
        const double2 wv = g.diff_wallv[j];
        ghost[0] = 2.0 * wv.x - ghost[0];
        ghost[1] = 2.0 * wv.y - ghost[1];
      } else {
        const double t = 2.0 * dot2(ghost[0], ghost[1], nx, ny);
        ghost[0] -= t * nx;
        ghost[1] -= t * ny;
      }
      if (g.diff_thermal[j] == 0) {
        ghost[2] = 2.0 * g.diff_value[j] - cv[2];
      } else {
        const double k = cc.c;  // conductivity of the cell's own temperature
        ghost[2] += div_rn(2.0 * g.diff_nd[j] * g.diff_value[j], k);
      }
    } else if (kind == MCFD_DIFF_SYMMETRY) {
      const double t = 2.0 * dot2(cv[0], cv[1], nx, ny);
      ghost[0] -= t * nx;
      ghost[1] -= t * ny;
    } else if (kind == MCFD_DIFF_INLET) {
      double iv[3];
      if (inlet_values(g, P, j, c, make_double2(nx, ny), vs.gamma, vs.R, iv, &bits)) {
        ghost[0] = 2.0 * iv[0] - ghost[0];
        ghost[1] = 2.0 * iv[1] - ghost[1];
        ghost[2] = 2.0 * iv[2] - ghost[2];
      }
    }
    const double diff[3] = {ghost[0] - cv[0], ghost[1] - cv[1], ghost[2] - cv[2]};
    const double2 go = g.diff_ghost[j];
    add(go.x, go.y, diff);
  }
  if (bits) flag(g.status, bits, c);
  double out[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  const double det = xx * yy - xy * xy;
  const double xxyy = xx * yy;
  if (det > 1e-14 * (xxyy > 1e-300 ? xxyy : 1e-300)) {
    const double inv = div_rn(1.0, det);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      out[2 * k] = (bx[k] * yy - by[k] * xy) * inv;
      out[2 * k + 1] = (by[k] * xx - bx[k] * xy) * inv;
    }
  }
  double* dst = grad + 6 * (size_t)c;
#pragma unroll
  for (int k = 0; k < 6; ++k) dst[k] = out[k];
}

__global__ void __launch_bounds__(kBlock) k_visc_faces(DevGeom g, const double* __restrict__ P,
                                                       const double* __restrict__ cell,
                                                       const double* __restrict__ grad, double* __restrict__ flux) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int n_faces = g.seg_begin[SEG_PERIODIC + 1];  // interior, then periodic pairs
  if (i >= n_faces) return;
  const int o = g.ff_lcell[i], nb = g.ff_rcell[i];
  const double2 n = g.ff_normal[i];
  const double* go = grad + 6 * (size_t)o;
  const double* gn = grad + 6 * (size_t)nb;
  double fg[6];
#pragma unroll
  for (int k = 0; k < 6; ++k) fg[k] = 0.5 * (go[k] + gn[k]);
  const St4 po = ld4(P + 4 * (size_t)o), pn = ld4(P + 4 * (size_t)nb);
  const St4 co = ld4(cell + 4 * (size_t)o), cn = ld4(cell + 4 * (size_t)nb);
  double out[4];
  viscous_flux(fg, 0.5 * (po.b + pn.b), 0.5 * (po.c + pn.c), 0.5 * (co.b + cn.b), 0.5 * (co.c + cn.c), n.x, n.y,
               out);
  st4(flux + 4 * (size_t)i, St4{out[0], out[1], out[2], out[3]});
}

__global__ void __launch_bounds__(kBlock) k_visc_boundary(DevGeom g, const double* __restrict__ P, Visc vs,
                                                          const double* __restrict__ cell,
                                                          const double* __restrict__ grad,
                                                          double* __restrict__ bflux) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= g.n_diffusive) return;
  const int o = g.diff_owner[j];
  const double2 nn = g.diff_normal[j];
  const double nx = nn.x, ny = nn.y;
  const double2 off = g.diff_offset[j];
  const double nd = g.diff_nd[j];
  int bits = 0;
  if (nd <= 1e-14) bits |= MCFD_S_VISC_DISTANCE;
  const St4 p = ld4(P + 4 * (size_t)o);
  const St4 cc = ld4(cell + 4 * (size_t)o);
  double fg[6];
#pragma unroll
  for (int k = 0; k < 6; ++k) fg[k] = grad[6 * (size_t)o + k];
  double bv[3] = {p.b, p.c, cc.a};
  const double cv[3] = {p.b, p.c, cc.a};
  const double tox = off.x - nd * nx, toy = off.y - nd * ny;  // offset - d n
  const int kind = g.diff_kind[j];
  if (kind == MCFD_DIFF_WALL_NO_SLIP || kind == MCFD_DIFF_WALL_SLIP) {
    if (kind == MCFD_DIFF_WALL_NO_SLIP) {
      const double2 wv = g.diff_wallv[j];
      const double w[2] = {wv.x, wv.y};
#pragma unroll
      for (int comp = 0; comp < 2; ++comp) {
        const double dn = div_rn(w[comp] - bv[comp] - dot2(fg[2 * comp], fg[2 * comp + 1], tox, toy), nd);
        const double t = dn - dot2(fg[2 * comp], fg[2 * comp + 1], nx, ny);
        fg[2 * comp] += t * nx;
        fg[2 * comp + 1] += t * ny;
        bv[comp] = w[comp];
      }
    } else {
      const double nvel = dot2(bv[0], bv[1], nx, ny);
      bv[0] += gemv_row(fg[0], fg[1], off.x, off.y);
      bv[1] += gemv_row(fg[2], fg[3], off.x, off.y);
      const double t = dot2(bv[0], bv[1], nx, ny);
      bv[0] -= t * nx;
      bv[1] -= t * ny;
      const double gnv0 = nx * fg[0] + ny * fg[2], gnv1 = nx * fg[1] + ny * fg[3];
      const double dn = div_rn(-(nvel + dot2(gnv0, gnv1, tox, toy)), nd);
      const double d0 = dn * nx, d1 = dn * ny;  // desired = outer(dn n, n)
      const double r0 = gemv_row(fg[0], fg[1], nx, ny), r1 = gemv_row(fg[2], fg[3], nx, ny);
      fg[0] += d0 * nx - r0 * nx;
      fg[1] += d0 * ny - r0 * ny;
      fg[2] += d1 * nx - r1 * nx;
      fg[3] += d1 * ny - r1 * ny;
    }
    double dn;
    if (g.diff_thermal[j] == 0) {
      dn = div_rn(g.diff_value[j] - bv[2] - dot2(fg[4], fg[5], tox, toy), nd);
      bv[2] = g.diff_value[j];
    } else {
      dn = div_rn(g.diff_value[j], cc.c);
      bv[2] += dot2(fg[4], fg[5], off.x, off.y);
    }
    const double t = dn - dot2(fg[4], fg[5], nx, ny);
    fg[4] += t * nx;
    fg[5] += t * ny;
  } else if (kind == MCFD_DIFF_SYMMETRY) {
    const double nvel = dot2(bv[0], bv[1], nx, ny);
    const double s = div_rn(-nvel, nd);
    const double dvel[2] = {s * nx, s * ny};
#pragma unroll
    for (int comp = 0; comp < 2; ++comp) {
      const double t = dvel[comp] - dot2(fg[2 * comp], fg[2 * comp + 1], nx, ny);
      fg[2 * comp] += t * nx;
      fg[2 * comp + 1] += t * ny;
    }
    const double t = dot2(fg[4], fg[5], nx, ny);
    fg[4] -= t * nx;
    fg[5] -= t * ny;
    bv[0] -= nvel * nx;
    bv[1] -= nvel * ny;
  } else {
    double iv[3];
    if (kind == MCFD_DIFF_INLET && inlet_values(g, P, j, o, make_double2(nx, ny), vs.gamma, vs.R, iv, &bits)) {
      bv[0] = iv[0];
      bv[1] = iv[1];
      bv[2] = iv[2];
#pragma unroll
      for (int comp = 0; comp < 3; ++comp) {
        const double dn = div_rn(bv[comp] - cv[comp] - dot2(fg[2 * comp], fg[2 * comp + 1], tox, toy), nd);
        const double t = dn - dot2(fg[2 * comp], fg[2 * comp + 1], nx, ny);
        fg[2 * comp] += t * nx;
        fg[2 * comp + 1] += t * ny;
      }
    } else {  // zero normal gradient: fg -= outer(fg @ n, n); bv += fg @ offset
#pragma unroll
      for (int comp = 0; comp < 3; ++comp) {
        const double r = gemv_row(fg[2 * comp], fg[2 * comp + 1], nx, ny);
        fg[2 * comp] -= r * nx;
        fg[2 * comp + 1] -= r * ny;
      }
#pragma unroll
      for (int comp = 0; comp < 3; ++comp) bv[comp] += gemv_row(fg[2 * comp], fg[2 * comp + 1], off.x, off.y);
    }
  }
  bool bad = false;
  const double mu = viscosity(vs, bv[2], &bad);
  if (bad) bits |= MCFD_S_VISC_SUTHERLAND;
  const double k = conductivity(vs, mu);
  double out[4];
  viscous_flux(fg, bv[0], bv[1], mu, k, nx, ny, out);
  if ((kind == MCFD_DIFF_WALL_NO_SLIP || kind == MCFD_DIFF_WALL_SLIP) && g.diff_thermal[j] == 1)
    out[3] = g.diff_value[j];
  if (bits) flag(g.status, bits, o);
  st4(bflux + 4 * (size_t)j, St4{out[0], out[1], out[2], out[3]});
}

__global__ void __launch_bounds__(kBlock) k_visc_gather(DevGeom g, const double* __restrict__ flux,
                                                        const double* __restrict__ bflux, double* __restrict__ r) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= g.n_cells) return;
  double s[4] = {0.0, 0.0, 0.0, 0.0};
  for (int j = g.gi_ptr[c], j1 = g.gi_ptr[c + 1]; j < j1; ++j) {
    const double a = g.gi_coef[j];
    const St4 F = ld4(flux + 4 * (size_t)g.gi_flux[j]);
    s[0] = s[0] + a * F.a;
    s[1] = s[1] + a * F.b;
    s[2] = s[2] + a * F.c;
    s[3] = s[3] + a * F.d;
  }
  double d[4] = {0.0 - (0.0 + s[0]), 0.0 - (0.0 + s[1]), 0.0 - (0.0 + s[2]), 0.0 - (0.0 + s[3])};
  const double area = g.area[c];
  for (int i = g.vg_ptr[c], i1 = g.vg_ptr[c + 1]; i < i1; ++i) {
    const int code = g.vg_code[i];
    const int kind = code >> 28, idx = code & 0x0fffffff;
    if (kind == 2) {  // diffusive boundary face: flux L / A
      const double len = g.diff_len[idx];
      const St4 F = ld4(bflux + 4 * (size_t)idx);
      d[0] = d[0] + div_rn(F.a * len, area);
      d[1] = d[1] + div_rn(F.b * len, area);
      d[2] = d[2] + div_rn(F.c * len, area);
      d[3] = d[3] + div_rn(F.d * len, area);
    } else {  // periodic pair idx: (flux L) / A on side a, -(flux L) / A on side b
      const int fi = g.seg_begin[SEG_PERIODIC] + idx;
      const double len = g.ff_len[fi];
      const St4 F = ld4(flux + 4 * (size_t)fi);
      double v[4] = {F.a * len, F.b * len, F.c * len, F.d * len};
      if (kind == 1) {
        v[0] = -v[0]; v[1] = -v[1]; v[2] = -v[2]; v[3] = -v[3];
      }
      d[0] = d[0] + div_rn(v[0], area);
      d[1] = d[1] + div_rn(v[1], area);
      d[2] = d[2] + div_rn(v[2], area);
      d[3] = d[3] + div_rn(v[3], area);
    }
  }
  st4(r + 4 * (size_t)c, St4{d[0], d[1], d[2], d[3]});
}

__global__ void __launch_bounds__(kBlock) k_visc_diffusion(DevGeom g, const double* __restrict__ cell,
                                                           double* __restrict__ diff) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= g.n_cells) return;
  const double ec = cell[4 * (size_t)c + 3];
  double sum = 0.0;
  for (int i = g.vd_ptr[c], i1 = g.vd_ptr[c + 1]; i < i1; ++i) {
    const int other = g.vd_other[i];
    double e = ec;
    if (other >= 0) {
      const double eo = cell[4 * (size_t)other + 3];
      e = eo > ec ? eo : ec;  // np.maximum
    }
    const double dist = g.vd_dist[i];
    sum += div_rn(e * g.vd_len[i], dist > 1e-14 ? dist : 1e-14);
  }
  diff[c] = sum;
}

Visc visc_of(const mcfd_config& cfg) {
  return Visc{cfg.viscosity_model, cfg.dynamic_viscosity, cfg.sutherland_reference_viscosity,
              cfg.sutherland_reference_temperature, cfg.sutherland_temperature, cfg.gamma, cfg.gas_constant,
              cfg.prandtl_number};
}

}  // namespace

cudaError_t launch_viscous_residual(const DevGeom& g, const mcfd_config& cfg, const double* P, const ViscousWork& w,
                                    cudaStream_t s) {
  const Visc vs = visc_of(cfg);
  const int C = g.n_cells, nf = g.seg_begin[SEG_PERIODIC + 1];
  count_launch(4 + (g.n_diffusive > 0));
  k_visc_cells<<<blocks_for(C), kBlock, 0, s>>>(g, P, vs, w.cell);
  k_visc_gradients<<<blocks_for(C), kBlock, 0, s>>>(g, P, vs, w.cell, w.grad);
  if (nf > 0) k_visc_faces<<<blocks_for(nf), kBlock, 0, s>>>(g, P, w.cell, w.grad, w.flux);
  if (g.n_diffusive > 0)
    k_visc_boundary<<<blocks_for(g.n_diffusive), kBlock, 0, s>>>(g, P, vs, w.cell, w.grad, w.bflux);
  k_visc_gather<<<blocks_for(C), kBlock, 0, s>>>(g, w.flux, w.bflux, w.r);
  return cudaGetLastError();
}

cudaError_t launch_viscous_diffusion(const DevGeom& g, const mcfd_config& cfg, const double* P,
                                     const ViscousWork& w, cudaStream_t s) {
  const Visc vs = visc_of(cfg);
  const int C = g.n_cells;
  count_launch(2);
  k_visc_cells<<<blocks_for(C), kBlock, 0, s>>>(g, P, vs, w.cell);
  k_visc_diffusion<<<blocks_for(C), kBlock, 0, s>>>(g, w.cell, w.diff);
  return cudaGetLastError();
}

}  // namespace mcfd
