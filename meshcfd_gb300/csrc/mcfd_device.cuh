// Device arithmetic of the residual path: primitive recovery, Euler fluxes,
// boundary ghost states, limiter.  Every function restates one reference
// routine and keeps its expression order, so that a translation unit built
// without FMA contraction (-fmad=false) reproduces the reference's IEEE
// results operation for operation.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/meshcfd_gb300.h"

namespace mcfd {

struct St4 {
  double a, b, c, d;
};

__device__ __forceinline__ St4 ld4(const double* p) {
  const double2* q = reinterpret_cast<const double2*>(p);
  double2 x = q[0], y = q[1];
  return St4{x.x, x.y, y.x, y.y};
}
__device__ __forceinline__ St4 ld4_nc(const double* p) {
  const double2* q = reinterpret_cast<const double2*>(p);
  double2 x = __ldg(q), y = __ldg(q + 1);
  return St4{x.x, x.y, y.x, y.y};
}
__device__ __forceinline__ void st4(double* p, const St4& s) {
  double2* q = reinterpret_cast<double2*>(p);
  q[0] = make_double2(s.a, s.b);
  q[1] = make_double2(s.c, s.d);
}

// Python / NumPy min/max semantics on non-NaN data, written as selects.
__device__ __forceinline__ double py_min(double a, double b) { return (b < a) ? b : a; }
__device__ __forceinline__ double py_max(double a, double b) { return (b > a) ? b : a; }

__device__ __forceinline__ bool finite4(const St4& s) {
  return isfinite(s.a) && isfinite(s.b) && isfinite(s.c) && isfinite(s.d);
}

// euler.conservative_to_primitive (euler.py:20-40), one row.
__device__ __forceinline__ St4 cons_to_prim(const St4& U, double gamma, bool* ok) {
  double rho = U.a;
  double ux = U.b / rho;
  double uy = U.c / rho;
  double p = (gamma - 1.0) * (U.d - (0.5 * (U.b * U.b + U.c * U.c)) / rho);
  St4 P{rho, ux, uy, p};
  *ok = finite4(P) && rho > 0.0 && p > 0.0;
  return P;
}

// euler.physical_flux (euler.py:43-57): flux and conservative state.
__device__ __forceinline__ void physical_flux(const St4& q, double nx, double ny, double gamma,
                                              double F[4], double U[4]) {
  double rho = q.a, ux = q.b, uy = q.c, p = q.d;
  double energy = p / (gamma - 1.0) + (0.5 * rho) * (ux * ux + uy * uy);
  double un = ux * nx + uy * ny;
  U[0] = rho;
  U[1] = rho * ux;
  U[2] = rho * uy;
  U[3] = energy;
  F[0] = rho * un;
  F[1] = (rho * ux) * un + p * nx;
  F[2] = (rho * uy) * un + p * ny;
  F[3] = (energy + p) * un;
}

__device__ __forceinline__ double sound_speed(double rho, double p, double gamma) {
  return sqrt((gamma * p) / rho);
}

// euler._rusanov_flux (euler.py:80-93).
__device__ __forceinline__ void rusanov_flux(const St4& L, const St4& R, double nx, double ny,
                                             double gamma, double out[4]) {
  double FL[4], UL[4], FR[4], UR[4];
  physical_flux(L, nx, ny, gamma, FL, UL);
  physical_flux(R, nx, ny, gamma, FR, UR);
  double unl = L.b * nx + L.c * ny;
  double unr = R.b * nx + R.c * ny;
  double sl = fabs(unl) + sound_speed(L.a, L.d, gamma);
  double sr = fabs(unr) + sound_speed(R.a, R.d, gamma);
  double s = (sl >= sr) ? sl : sr;  // np.maximum
#pragma unroll
  for (int k = 0; k < 4; ++k) out[k] = 0.5 * ((FL[k] + FR[k]) - s * (UR[k] - UL[k]));
}

// HLLC flux.  KERNEL_BRANCHES selects the branch structure of the fused
// compiled kernel (_kernels.py:127-159): S_L>=0 -> F_L, S_R<=0 -> F_R, then the
// contact sign.  Otherwise the NumPy selection of euler._hllc_flux
// (euler.py:155-163): S_L>=0 -> F_L, S*>=0 -> F*_L, S_R>0 -> F*_R, else F_R,
// followed by its finiteness check (euler.py:164-165).  Returns false when the
// NumPy form produced a non-finite value.
template <bool KERNEL_BRANCHES>
__device__ __forceinline__ bool hllc_flux(const St4& L, const St4& R, double nx, double ny,
                                          double gamma, double out[4]) {
  double FL[4], UL[4], FR[4], UR[4];
  physical_flux(L, nx, ny, gamma, FL, UL);
  physical_flux(R, nx, ny, gamma, FR, UR);
  double rl = L.a, pl = L.d, rr = R.a, pr = R.d;
  double unl = L.b * nx + L.c * ny;
  double unr = R.b * nx + R.c * ny;
  double cl = sound_speed(rl, pl, gamma);
  double cr = sound_speed(rr, pr, gamma);
  double wl = py_min(unl - cl, unr - cr);
  double wr = py_max(unl + cl, unr + cr);
  double den = rl * (wl - unl) - rr * (wr - unr);
  if (!(fabs(den) > 1e-14)) den = copysign(1e-14, den);
  double contact = ((pr - pl) + (rl * unl) * (wl - unl) - (rr * unr) * (wr - unr)) / den;

  int branch;  // 0: F_L, 1: F*_L, 2: F*_R, 3: F_R
  if (KERNEL_BRANCHES) {
    if (wl >= 0.0) branch = 0;
    else if (wr <= 0.0) branch = 3;
    else branch = (contact >= 0.0) ? 1 : 2;
  } else {
    if (wl >= 0.0) branch = 0;
    else if (contact >= 0.0) branch = 1;
    else if (wr > 0.0) branch = 2;
    else branch = 3;
  }
  if (branch == 0 || branch == 3) {
    const double* F = (branch == 0) ? FL : FR;
#pragma unroll
    for (int k = 0; k < 4; ++k) out[k] = F[k];
  } else {
    const bool left = (branch == 1);
    const St4& q = left ? L : R;
    const double* U = left ? UL : UR;
    const double* F = left ? FL : FR;
    double un = left ? unl : unr;
    double wave = left ? wl : wr;
    double rho = q.a, pressure = q.d;
    double factor = (rho * (wave - un)) / (wave - contact);
    double sux = q.b + (contact - un) * nx;
    double suy = q.c + (contact - un) * ny;
    double se = factor * (U[3] / rho + (contact - un) * (contact + pressure / (rho * (wave - un))));
    double star[4] = {factor, factor * sux, factor * suy, se};
#pragma unroll
    for (int k = 0; k < 4; ++k) out[k] = F[k] + wave * (star[k] - U[k]);
  }
  if (!KERNEL_BRANCHES) {
    return isfinite(out[0]) && isfinite(out[1]) && isfinite(out[2]) && isfinite(out[3]);
  }
  return true;
}

// euler._roe_flux (euler.py:169-262).  Returns a status bit (0 if fine).  The
// eigenvector contraction follows np.einsum's reduction order for four terms
// on the reference's platform: (t0 + t2) + (t1 + t3).
__device__ __forceinline__ int roe_flux(const St4& L, const St4& R, double nx, double ny,
                                        double gamma, double out[4]) {
  double FL[4], UL[4], FR[4], UR[4];
  physical_flux(L, nx, ny, gamma, FL, UL);
  physical_flux(R, nx, ny, gamma, FR, UR);
  double root_l = sqrt(L.a), root_r = sqrt(R.a);
  double den = root_l + root_r;
  double vx = (root_l * L.b + root_r * R.b) / den;
  double vy = (root_l * L.c + root_r * R.c) / den;
  double H = (root_l * (L.d / L.a + 0.5 * (L.b * L.b + L.c * L.c)) +
              root_r * (R.d / R.a + 0.5 * (R.b * R.b + R.c * R.c))) / den;
  double un = vx * nx + vy * ny;
  double ut = vx * -ny + vy * nx;
  double c2 = (gamma - 1.0) * (H - 0.5 * (vx * vx + vy * vy));
  if (!(c2 > 0.0) || !isfinite(c2)) {
    out[0] = out[1] = out[2] = out[3] = 0.0;
    return MCFD_S_ROE_SOUND;
  }
  double c = sqrt(c2);
  double ravg = root_l * root_r;
  double unl = L.b * nx + L.c * ny, unr = R.b * nx + R.c * ny;
  double utl = L.b * -ny + L.c * nx, utr = R.b * -ny + R.c * nx;
  double dr = R.a - L.a, dun = unr - unl, dut = utr - utl, dp = R.d - L.d;
  double am = (dp - (ravg * c) * dun) / (2.0 * c2);
  double ap = (dp + (ravg * c) * dun) / (2.0 * c2);
  double ac = dr - dp / c2;
  double as = ravg * dut;
  double lam[4] = {un - c, un, un, un + c};
  double fix = 0.1 * c;
  double w[4];
  double strength[4] = {am, ac, as, ap};
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    double a = fabs(lam[j]);
    if (a < fix) a = 0.5 * ((a * a) / fix + fix);
    w[j] = a * strength[j];
  }
  double e[4][4] = {{1.0, 1.0, 0.0, 1.0},
                    {un - c, un, 0.0, un + c},
                    {ut, ut, 1.0, ut},
                    {H - un * c, 0.5 * (un * un + ut * ut), ut, H + un * c}};
  double d[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    double t0 = e[i][0] * w[0], t1 = e[i][1] * w[1], t2 = e[i][2] * w[2], t3 = e[i][3] * w[3];
    d[i] = (t0 + t2) + (t1 + t3);
  }
  double diss[4] = {d[0], d[1] * nx - d[2] * ny, d[1] * ny + d[2] * nx, d[3]};
#pragma unroll
  for (int k = 0; k < 4; ++k) out[k] = 0.5 * ((FL[k] + FR[k]) - diss[k]);
  if (!(isfinite(out[0]) && isfinite(out[1]) && isfinite(out[2]) && isfinite(out[3])))
    return MCFD_S_ROE_NONFINITE;
  return 0;
}

// Far-field characteristic ghost state (solver.py:4350-4409), one face.
// Returns a status bit (0 if fine).
__device__ __forceinline__ int far_field_state(const St4& in, const St4& far, double nx,
                                               double ny, double gamma, St4* ext) {
  double un_i = in.b * nx + in.c * ny;
  double un_f = far.b * nx + far.c * ny;
  double c_i = sound_speed(in.a, in.d, gamma);
  double c_f = sound_speed(far.a, far.d, gamma);
  if (un_i <= -c_i) {
    *ext = far;
    return 0;
  }
  if (un_i >= c_i) {
    *ext = in;
    return 0;
  }
  double out_inv = un_i + (2.0 * c_i) / (gamma - 1.0);
  double in_inv = un_f - (2.0 * c_f) / (gamma - 1.0);
  double vb = 0.5 * (out_inv + in_inv);
  double cb = (0.25 * (gamma - 1.0)) * (out_inv - in_inv);
  if (!isfinite(cb) || cb <= 0.0) {
    *ext = in;
    return MCFD_S_FARFIELD_SOUND;
  }
  const St4& src = (vb < 0.0) ? far : in;
  double entropy = src.d / pow(src.a, gamma);
  double rho = pow((cb * cb) / (gamma * entropy), 1.0 / (gamma - 1.0));
  double p = entropy * pow(rho, gamma);
  double tx = -ny, ty = nx;
  double vt = src.b * tx + src.c * ty;
  St4 s{rho, vb * nx + vt * tx, vb * ny + vt * ty, p};
  *ext = s;
  if (!finite4(s) || !(rho > 0.0) || !(p > 0.0)) return MCFD_S_FARFIELD_STATE;
  return 0;
}

// One limiter entry (_kernels.py:40-65): the face factor for one variable.
template <int LIMITER>
__device__ __forceinline__ double limiter_face_factor(double value, double increment, double lo,
                                                      double hi) {
  double tolerance = 1e-14 * py_max(fabs(value), 1.0);
  double ratio = 1.0;
  if (increment > tolerance) ratio = (hi - value) / increment;
  else if (increment < -tolerance) ratio = (lo - value) / increment;
  ratio = (0.0 > ratio) ? 0.0 : ratio;
  double f;
  if (LIMITER <= 1) {
    f = py_min(ratio, 1.0);
  } else if (LIMITER == 2) {
    f = (ratio > 0.0) ? py_min(1.0, (2.0 * ratio) / (1.0 + ratio)) : 0.0;
  } else {
    const double eps = 1e-12;
    f = ((ratio * ratio + 2.0 * ratio) + eps) / (((ratio * ratio + ratio) + 2.0) + eps);
    f = py_min(f, 1.0);
  }
  return f;
}

}  // namespace mcfd
