// Device arithmetic of the residual path: primitive recovery, Euler fluxes,
// boundary ghost states, limiter.  Every function restates one reference
// routine and keeps its expression order, so that a translation unit built
// without FMA contraction (-fmad=false) reproduces the reference's IEEE
// results operation for operation.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/meshcfd_gb300.h"
#include "mcfd_arith.cuh"

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


// ---------------------------------------------------------------------------
// IEEE-754 comparisons evaluated on the integer pipe.  On GB300 the FP64 pipe
// issues ~1/38 the integer rate (measured), and compares / min / max /
// finiteness tests take FP64 issue slots like arithmetic does.  Sign and
// exponent masks go through ia::bits_and / ia::sign_xor so that they stay
// integer instructions.  Each helper
// below returns exactly the IEEE result for non-NaN operands (signed zeros
// compare equal); NaN never reaches a decision whose outcome matters (every
// path that can produce NaN also sets a status bit from a finiteness test).
namespace icmp {

__device__ __forceinline__ long long bits(double x) { return (long long)ia::bits(x); }

// Monotone key: x < y  <=>  key(x) < key(y); -0 and +0 both map to 0.
__device__ __forceinline__ long long key(double x) {
  long long b = bits(x);
  long long k = b ^ ((b >> 63) & 0x7fffffffffffffffLL);
  return k - (k >> 63);
}
__device__ __forceinline__ bool lt(double a, double b) { return key(a) < key(b); }
// both operands >= 0 (either zero may be signed)
__device__ __forceinline__ bool lt_nonneg(double a, double b) {
  return ia::bits_and(ia::bits(a), ~ia::kSign) < ia::bits_and(ia::bits(b), ~ia::kSign);
}
// a < c and a > c for a constant c > 0 (gt also for c = +0)
__device__ __forceinline__ bool lt_pos(double a, double c) { return bits(a) < bits(c); }
__device__ __forceinline__ bool gt_pos(double a, double c) { return bits(a) > bits(c); }
// -a > c for c >= +0  (a < -c)
__device__ __forceinline__ bool neg_gt_pos(double a, double c) {
  return (long long)ia::sign_xor(ia::bits(a), ia::kSign) > bits(c);
}
__device__ __forceinline__ bool abs_gt(double a, double c) {
  return ia::bits_and(ia::bits(a), ~ia::kSign) > (unsigned long long)bits(c);
}
__device__ __forceinline__ bool gt0(double a) { return bits(a) > 0; }
__device__ __forceinline__ bool le0(double a) { return bits(a) <= 0; }
__device__ __forceinline__ bool ge0(double a) {
  long long b = bits(a);
  return b >= 0 || b == (long long)0x8000000000000000ULL;
}
__device__ __forceinline__ bool finite(double a) {
  return ia::bits_and(ia::bits(a), 0x7ff0000000000000ull) != 0x7ff0000000000000ull;
}
// Python min(a, b) / max(a, b): the first argument unless the second is
// strictly smaller / larger.
__device__ __forceinline__ double py_min(double a, double b) { return lt(b, a) ? b : a; }
__device__ __forceinline__ double py_max(double a, double b) { return lt(a, b) ? b : a; }

}  // namespace icmp

using icmp::py_max;
using icmp::py_min;

__device__ __forceinline__ bool finite4(const St4& s) {
  return icmp::finite(s.a) && icmp::finite(s.b) && icmp::finite(s.c) && icmp::finite(s.d);
}

// euler.conservative_to_primitive (euler.py:20-40), one row.
__device__ __forceinline__ St4 cons_to_prim(const St4& U, double gamma, bool* ok) {
  double rho = U.a;
  const unsigned long long rx = recip_fixed(rho);  // the three quotients share the divisor
  double ux = div_rn_recip(U.b, rho, rx);
  double uy = div_rn_recip(U.c, rho, rx);
  double p = (gamma - 1.0) * (U.d - div_rn_recip(0.5 * (U.b * U.b + U.c * U.c), rho, rx));
  St4 P{rho, ux, uy, p};
  *ok = finite4(P) && icmp::gt0(rho) && icmp::gt0(p);
  return P;
}

// Products of the exact flux functions that a translation unit may evaluate
// on the integer pipe (mul_rn, the same IEEE result): MCFD_FLUX_INT_MUL is a
// mask of call sites -- 1 normal velocities, sound speeds and wave terms,
// 2 the physical flux, 4 the HLLC star state -- set by a stage-kernel unit
// before it includes this header; 0 (the FP64 unit) everywhere else.
#ifndef MCFD_FLUX_INT_MUL
#define MCFD_FLUX_INT_MUL 0
#endif
enum FluxMulSite { FMUL_WAVES = 1, FMUL_PHYSICAL = 2, FMUL_STAR = 4 };

template <int SITE>
__device__ __forceinline__ double fmul(double a, double b) {
  if constexpr ((MCFD_FLUX_INT_MUL & SITE) != 0) return mul_rn(a, b);
  else return a * b;
}

// euler.physical_flux (euler.py:43-57): flux and conservative state, with
// the normal velocity un = ux nx + uy ny given (the callers compute it too).
__device__ __forceinline__ void physical_flux_un(const St4& q, double un, double nx, double ny, double gamma,
                                                 double F[4], double U[4]) {
  constexpr int S = FMUL_PHYSICAL;
  double rho = q.a, ux = q.b, uy = q.c, p = q.d;
  double energy = div_rn(p, gamma - 1.0) + fmul<S>(fmul<S>(0.5, rho), fmul<S>(ux, ux) + fmul<S>(uy, uy));
  const double mx = fmul<S>(rho, ux), my = fmul<S>(rho, uy);
  U[0] = rho;
  U[1] = mx;
  U[2] = my;
  U[3] = energy;
  F[0] = fmul<S>(rho, un);
  F[1] = fmul<S>(mx, un) + fmul<S>(p, nx);
  F[2] = fmul<S>(my, un) + fmul<S>(p, ny);
  F[3] = fmul<S>(energy + p, un);
}

__device__ __forceinline__ void physical_flux(const St4& q, double nx, double ny, double gamma,
                                              double F[4], double U[4]) {
  physical_flux_un(q, q.b * nx + q.c * ny, nx, ny, gamma, F, U);
}

__device__ __forceinline__ double sound_speed(double rho, double p, double gamma) {
  return sqrt_rn(div_rn(fmul<FMUL_WAVES>(gamma, p), rho));
}

// euler._rusanov_flux (euler.py:80-93).
__device__ __forceinline__ void rusanov_flux(const St4& L, const St4& R, double nx, double ny,
                                             double gamma, double out[4]) {
  double FL[4], UL[4], FR[4], UR[4];
  physical_flux(L, nx, ny, gamma, FL, UL);
  physical_flux(R, nx, ny, gamma, FR, UR);
  double unl = L.b * nx + L.c * ny;
  double unr = R.b * nx + R.c * ny;
  double sl = abs_of(unl) + sound_speed(L.a, L.d, gamma);
  double sr = abs_of(unr) + sound_speed(R.a, R.d, gamma);
  double s = icmp::lt_nonneg(sl, sr) ? sr : sl;  // np.maximum
#pragma unroll
  for (int k = 0; k < 4; ++k) out[k] = 0.5 * ((FL[k] + FR[k]) - s * (UR[k] - UL[k]));
}

// HLLC flux.  KERNEL_BRANCHES selects the branch structure of the fused
// compiled kernel (_kernels.py:127-159): S_L>=0 -> F_L, S_R<=0 -> F_R, then the
// contact sign.  Otherwise the NumPy selection of euler._hllc_flux
// (euler.py:155-163): S_L>=0 -> F_L, S*>=0 -> F*_L, S_R>0 -> F*_R, else F_R,
// followed by its finiteness check (euler.py:164-165).  Returns false when the
// NumPy form produced a non-finite value.
//
// Every branch uses one side's physical flux and conservative state only, so
// the side is chosen first and its physical flux evaluated alone (the same
// expressions as for both sides, so the same values).
template <bool KERNEL_BRANCHES>
__device__ __forceinline__ bool hllc_flux(const St4& L, const St4& R, double nx, double ny,
                                          double gamma, double out[4]) {
  constexpr int W = FMUL_WAVES, T = FMUL_STAR;
  double rl = L.a, pl = L.d, rr = R.a, pr = R.d;
  double unl = fmul<W>(L.b, nx) + fmul<W>(L.c, ny);
  double unr = fmul<W>(R.b, nx) + fmul<W>(R.c, ny);
  double cl = sound_speed(rl, pl, gamma);
  double cr = sound_speed(rr, pr, gamma);
  double wl = py_min(unl - cl, unr - cr);
  double wr = py_max(unl + cl, unr + cr);
  const double dl = wl - unl, dr = wr - unr;
  double den = fmul<W>(rl, dl) - fmul<W>(rr, dr);
  if (!icmp::abs_gt(den, 1e-14)) den = with_sign_of(1e-14, den);
  double contact = div_rn((pr - pl) + fmul<W>(fmul<W>(rl, unl), dl) - fmul<W>(fmul<W>(rr, unr), dr), den);

  int branch;  // 0: F_L, 1: F*_L, 2: F*_R, 3: F_R
  if (KERNEL_BRANCHES) {
    if (icmp::ge0(wl)) branch = 0;
    else if (icmp::le0(wr)) branch = 3;
    else branch = icmp::ge0(contact) ? 1 : 2;
  } else {
    if (icmp::ge0(wl)) branch = 0;
    else if (icmp::ge0(contact)) branch = 1;
    else if (icmp::gt0(wr)) branch = 2;
    else branch = 3;
  }
  const bool left = branch <= 1;
  const St4 q = left ? L : R;
  const double un = left ? unl : unr;
  double F[4], U[4];
  physical_flux_un(q, un, nx, ny, gamma, F, U);
  if (branch == 0 || branch == 3) {
#pragma unroll
    for (int k = 0; k < 4; ++k) out[k] = F[k];
  } else {
    double wave = left ? wl : wr;
    double rho = q.a, pressure = q.d;
    const double m = fmul<T>(rho, wave - un), cu = contact - un;
    double factor = div_rn(m, wave - contact);
    double sux = q.b + fmul<T>(cu, nx);
    double suy = q.c + fmul<T>(cu, ny);
    double se = fmul<T>(factor, div_rn(U[3], rho) + fmul<T>(cu, contact + div_rn(pressure, m)));
    double star[4] = {factor, fmul<T>(factor, sux), fmul<T>(factor, suy), se};
#pragma unroll
    for (int k = 0; k < 4; ++k) out[k] = F[k] + fmul<T>(wave, star[k] - U[k]);
  }
  if (!KERNEL_BRANCHES) {
    return icmp::finite(out[0]) && icmp::finite(out[1]) && icmp::finite(out[2]) && icmp::finite(out[3]);
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
  double root_l = sqrt_rn(L.a), root_r = sqrt_rn(R.a);
  double den = root_l + root_r;
  double vx = div_rn(root_l * L.b + root_r * R.b, den);
  double vy = div_rn(root_l * L.c + root_r * R.c, den);
  double H = div_rn(root_l * (div_rn(L.d, L.a) + 0.5 * (L.b * L.b + L.c * L.c)) +
                    root_r * (div_rn(R.d, R.a) + 0.5 * (R.b * R.b + R.c * R.c)), den);
  double un = vx * nx + vy * ny;
  double ut = vx * -ny + vy * nx;
  double c2 = (gamma - 1.0) * (H - 0.5 * (vx * vx + vy * vy));
  if (!icmp::gt0(c2) || !icmp::finite(c2)) {
    out[0] = out[1] = out[2] = out[3] = 0.0;
    return MCFD_S_ROE_SOUND;
  }
  double c = sqrt_rn(c2);
  double ravg = root_l * root_r;
  double unl = L.b * nx + L.c * ny, unr = R.b * nx + R.c * ny;
  double utl = L.b * -ny + L.c * nx, utr = R.b * -ny + R.c * nx;
  double dr = R.a - L.a, dun = unr - unl, dut = utr - utl, dp = R.d - L.d;
  double am = div_rn(dp - (ravg * c) * dun, 2.0 * c2);
  double ap = div_rn(dp + (ravg * c) * dun, 2.0 * c2);
  double ac = dr - div_rn(dp, c2);
  double as = ravg * dut;
  double lam[4] = {un - c, un, un, un + c};
  double fix = 0.1 * c;
  double w[4];
  double strength[4] = {am, ac, as, ap};
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    double a = abs_of(lam[j]);
    if (icmp::lt_nonneg(a, fix)) a = 0.5 * (div_rn(a * a, fix) + fix);
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
  if (!(icmp::finite(out[0]) && icmp::finite(out[1]) && icmp::finite(out[2]) && icmp::finite(out[3])))
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
  if (!icmp::lt(-c_i, un_i)) {  // un_i <= -c_i
    *ext = far;
    return 0;
  }
  if (!icmp::lt(un_i, c_i)) {  // un_i >= c_i
    *ext = in;
    return 0;
  }
  double out_inv = un_i + div_rn(2.0 * c_i, gamma - 1.0);
  double in_inv = un_f - div_rn(2.0 * c_f, gamma - 1.0);
  double vb = 0.5 * (out_inv + in_inv);
  double cb = (0.25 * (gamma - 1.0)) * (out_inv - in_inv);
  if (!icmp::finite(cb) || icmp::le0(cb)) {
    *ext = in;
    return MCFD_S_FARFIELD_SOUND;
  }
  const St4& src = icmp::ge0(vb) ? in : far;
  double entropy = div_rn(src.d, pow(src.a, gamma));
  double rho = pow(div_rn(cb * cb, gamma * entropy), div_rn(1.0, gamma - 1.0));
  double p = entropy * pow(rho, gamma);
  double tx = -ny, ty = nx;
  double vt = src.b * tx + src.c * ty;
  St4 s{rho, vb * nx + vt * tx, vb * ny + vt * ty, p};
  *ext = s;
  if (!finite4(s) || !icmp::gt0(rho) || !icmp::gt0(p)) return MCFD_S_FARFIELD_STATE;
  return 0;
}

// One limiter entry (_kernels.py:40-65): the face factor for one variable.
// `tolerance` = 1e-14 * max(|value|, 1) is hoisted by the caller (it is the
// same for every entry of a cell and variable).
template <int LIMITER>
__device__ __forceinline__ double limiter_face_factor(double value, double increment, double lo,
                                                      double hi, double tolerance) {
  // One division on a selected numerator (no divergent branches); the same
  // operands as the reference's two branches, so the same quotient.
  const bool pos = icmp::gt_pos(increment, tolerance);
  const bool neg = icmp::neg_gt_pos(increment, tolerance);
  const double num = pos ? (hi - value) : (lo - value);
  const double q = div_rn(num, (pos || neg) ? increment : 1.0);
  double ratio = (pos || neg) ? q : 1.0;
  ratio = icmp::ge0(ratio) ? ratio : 0.0;  // max(ratio, 0.0)
  double f;
  if (LIMITER <= 1) {
    f = icmp::gt_pos(ratio, 1.0) ? 1.0 : ratio;  // min(ratio, 1.0)
  } else if (LIMITER == 2) {
    if (icmp::gt0(ratio)) {
      double q = div_rn(2.0 * ratio, 1.0 + ratio);
      f = icmp::lt_pos(q, 1.0) ? q : 1.0;  // min(1.0, q)
    } else {
      f = 0.0;
    }
  } else {
    const double eps = 1e-12;
    f = div_rn((ratio * ratio + 2.0 * ratio) + eps, ((ratio * ratio + ratio) + 2.0) + eps);
    f = icmp::gt_pos(f, 1.0) ? 1.0 : f;  // min(f, 1.0)
  }
  return f;
}

// Limiter factor of a cell from its smallest ratio.  Correctly rounded
// division is monotone in the divisor, so over the entries with a positive
// increment the reference's smallest ratio (hi - v) / inc is the one at the
// largest increment, and over negative increments (lo - v) / inc is smallest
// at the most negative one: both are the reference's own quotients.  Every
// limiter function is non-decreasing in the ratio (Venkatakrishnan's is
// capped at 1 where it would decrease), so the minimum over entries of g(r)
// is g(min r) — exact for Barth-Jespersen and Minmod, and for Van Leer and
// Venkatakrishnan equal up to a possible last-place tie between near-equal
// entries.  Three divisions per variable instead of two per entry.
template <int LIMITER>
__device__ __forceinline__ double limiter_factor_min_ratio(double value, double lo, double hi,
                                                          double pos_max, double neg_min,
                                                          bool has_pos, bool has_neg, bool flat) {
  double r = 1.0;  // the tolerance band's ratio (only used when flat)
  bool any = flat;
  const double rp = div_rn(hi - value, has_pos ? pos_max : 1.0);
  const double rn = div_rn(lo - value, has_neg ? neg_min : -1.0);
  if (has_pos) {
    double x = icmp::ge0(rp) ? rp : 0.0;
    r = (!any || icmp::lt(x, r)) ? x : r;
    any = true;
  }
  if (has_neg) {
    double x = icmp::ge0(rn) ? rn : 0.0;
    r = (!any || icmp::lt(x, r)) ? x : r;
    any = true;
  }
  if (!any) return 1.0;
  double f;
  if (LIMITER <= 1) {
    f = icmp::gt_pos(r, 1.0) ? 1.0 : r;
  } else if (LIMITER == 2) {
    const double q = div_rn(twice(r), 1.0 + r);
    f = icmp::gt0(r) ? (icmp::lt_pos(q, 1.0) ? q : 1.0) : 0.0;
  } else {
    const double eps = 1e-12;
    const double rr = r * r;
    f = div_rn((rr + twice(r)) + eps, ((rr + r) + 2.0) + eps);
    f = icmp::gt_pos(f, 1.0) ? 1.0 : f;
  }
  return f;
}

// Venkatakrishnan's limiter in its published form with the smoothing
// constant (V. Venkatakrishnan, "Convergence to steady state solutions of the
// Euler equations on unstructured grids with limiters", J. Comput. Phys. 118,
// 120-130, 1995), an extension beside the reference's form (which has no K):
// for a face increment d2 = grad . r and d1 = max - v (d2 > 0) or min - v
// (d2 <= 0),
//   f = (d1^2 + e2 + 2 d1 d2) / (d1^2 + 2 d2^2 + d1 d2 + e2),
//   e2 = (K sqrt(A))^3,
// and the cell factor is the minimum over its faces, not capped at 1 (f
// exceeds 1 slightly where d2 is small against d1, as in the paper).  f is a
// rational function of (d1, d2) with e2 > 0, so away from ties between faces
// and between extreme neighbours the factor is differentiable, which is what
// a gradient check against finite differences needs.  f = 1 at d2 = 0.
// Products and sums of the smooth form go through __dmul_rn / __dadd_rn,
// which are never contracted into FMA: every kernel (forward in each
// variant, tangent and reverse) evaluates the same bits, so the reverse
// sweep's minimising face is the forward's.
__device__ __forceinline__ double venkat_k_e2(double k, double area) {
  const double t = __dmul_rn(k, sqrt_rn(area));
  return __dmul_rn(__dmul_rn(t, t), t);
}

struct VenkatK {
  double f, N, D, d1;
};

__device__ __forceinline__ VenkatK venkat_k_face(double value, double increment, double lo, double hi, double e2) {
  VenkatK r;
  r.d1 = icmp::gt0(increment) ? __dadd_rn(hi, -value) : __dadd_rn(lo, -value);
  const double d1d1 = __dmul_rn(r.d1, r.d1), d12 = __dmul_rn(r.d1, increment);
  r.N = __dadd_rn(__dadd_rn(d1d1, e2), __dadd_rn(d12, d12));
  r.D = __dadd_rn(__dadd_rn(__dadd_rn(d1d1, __dmul_rn(2.0, __dmul_rn(increment, increment))), d12), e2);
  r.f = div_rn(r.N, r.D);
  return r;
}

// partial derivatives of f with respect to d1 and d2 (from N, D of the face)
__device__ __forceinline__ void venkat_k_slopes(const VenkatK& v, double increment, double* df_dd1, double* df_dd2) {
  const double inv = div_rn(1.0, v.D * v.D);
  *df_dd1 = ((2.0 * v.d1 + 2.0 * increment) * v.D - v.N * (2.0 * v.d1 + increment)) * inv;
  *df_dd2 = ((2.0 * v.d1) * v.D - v.N * (4.0 * increment + v.d1)) * inv;
}

__device__ __forceinline__ double limiter_tolerance(double value) {
  double m = abs_of(value);
  return 1e-14 * (icmp::lt_pos(m, 1.0) ? 1.0 : m);  // 1e-14 * max(|v|, 1.0)
}

// ---------------------------------------------------------------------------
// Fast variants (FMA contraction on, fewer FP64 divisions).  Same algorithms
// as above; rounding differs from the reference at the last-place level.

// Primitive recovery with one reciprocal instead of three divisions.
__device__ __forceinline__ St4 cons_to_prim_fast(const St4& U, double gamma, bool* ok) {
  double rho = U.a;
  double inv = div_rn(1.0, rho);
  double ux = U.b * inv;
  double uy = U.c * inv;
  double p = (gamma - 1.0) * (U.d - 0.5 * (U.b * U.b + U.c * U.c) * inv);
  St4 P{rho, ux, uy, p};
  *ok = finite4(P) && icmp::gt0(rho) && icmp::gt0(p);
  return P;
}

// physical_flux with the internal energy as p * (1/(gamma-1)).
__device__ __forceinline__ void physical_flux_fast_un(const St4& q, double un, double nx, double ny,
                                                      double inv_gm1, double F[4], double U[4]) {
  double rho = q.a, ux = q.b, uy = q.c, p = q.d;
  double energy = p * inv_gm1 + 0.5 * rho * (ux * ux + uy * uy);
  U[0] = rho;
  U[1] = rho * ux;
  U[2] = rho * uy;
  U[3] = energy;
  F[0] = rho * un;
  F[1] = U[1] * un + p * nx;
  F[2] = U[2] * un + p * ny;
  F[3] = (energy + p) * un;
}

__device__ __forceinline__ void physical_flux_fast(const St4& q, double nx, double ny, double inv_gm1,
                                                   double F[4], double U[4]) {
  physical_flux_fast_un(q, q.b * nx + q.c * ny, nx, ny, inv_gm1, F, U);
}

// HLLC with shared reciprocals: one division for both 1/rho, one for the
// contact speed, one for the star state (rho(S-un) and S-S* share it).
template <bool KERNEL_BRANCHES>
__device__ __forceinline__ bool hllc_flux_fast(const St4& L, const St4& R, double nx, double ny,
                                               double gamma, double inv_gm1, double out[4]) {
  double rl = L.a, pl = L.d, rr = R.a, pr = R.d;
  double t = div_rn(1.0, rl * rr);
  double irl = rr * t, irr = rl * t;
  double unl = L.b * nx + L.c * ny;
  double unr = R.b * nx + R.c * ny;
  double cl = sqrt_rn(gamma * pl * irl);
  double cr = sqrt_rn(gamma * pr * irr);
  double wl = py_min(unl - cl, unr - cr);
  double wr = py_max(unl + cl, unr + cr);
  double ml = rl * (wl - unl), mr = rr * (wr - unr);
  double den = ml - mr;
  if (!icmp::abs_gt(den, 1e-14)) den = with_sign_of(1e-14, den);
  double contact = div_rn((pr - pl) + unl * ml - unr * mr, den);
  int branch;
  if (KERNEL_BRANCHES) {
    if (icmp::ge0(wl)) branch = 0;
    else if (icmp::le0(wr)) branch = 3;
    else branch = icmp::ge0(contact) ? 1 : 2;
  } else {
    if (icmp::ge0(wl)) branch = 0;
    else if (icmp::ge0(contact)) branch = 1;
    else if (icmp::gt0(wr)) branch = 2;
    else branch = 3;
  }
  const bool left = branch <= 1;
  const St4 q = left ? L : R;
  const double un = left ? unl : unr;
  double F[4], U[4];
  physical_flux_fast_un(q, un, nx, ny, inv_gm1, F, U);
  if (branch == 0 || branch == 3) {
#pragma unroll
    for (int k = 0; k < 4; ++k) out[k] = F[k];
  } else {
    double wave = left ? wl : wr;
    double m = left ? ml : mr;          // rho (S - un)
    double irho = left ? irl : irr;
    double d = wave - contact;
    double s = div_rn(1.0, m * d);
    double factor = m * m * s;          // rho (S - un) / (S - S*)
    double p_over_m = q.d * d * s;      // p / (rho (S - un))
    double sux = q.b + (contact - un) * nx;
    double suy = q.c + (contact - un) * ny;
    double se = factor * (U[3] * irho + (contact - un) * (contact + p_over_m));
    double star[4] = {factor, factor * sux, factor * suy, se};
#pragma unroll
    for (int k = 0; k < 4; ++k) out[k] = F[k] + wave * (star[k] - U[k]);
  }
  if (!KERNEL_BRANCHES)
    return icmp::finite(out[0]) && icmp::finite(out[1]) && icmp::finite(out[2]) && icmp::finite(out[3]);
  return true;
}

__device__ __forceinline__ void rusanov_flux_fast(const St4& L, const St4& R, double nx, double ny, double gamma,
                                                  double inv_gm1, double out[4]) {
  double FL[4], UL[4], FR[4], UR[4];
  physical_flux_fast(L, nx, ny, inv_gm1, FL, UL);
  physical_flux_fast(R, nx, ny, inv_gm1, FR, UR);
  double t = div_rn(1.0, L.a * R.a);
  double unl = L.b * nx + L.c * ny;
  double unr = R.b * nx + R.c * ny;
  double sl = abs_of(unl) + sqrt_rn(gamma * L.d * (R.a * t));
  double sr = abs_of(unr) + sqrt_rn(gamma * R.d * (L.a * t));
  double s = icmp::lt_nonneg(sl, sr) ? sr : sl;
#pragma unroll
  for (int k = 0; k < 4; ++k) out[k] = 0.5 * ((FL[k] + FR[k]) - s * (UR[k] - UL[k]));
}

__device__ __forceinline__ int roe_flux_fast(const St4& L, const St4& R, double nx, double ny, double gamma,
                                             double inv_gm1, double out[4]) {
  double FL[4], UL[4], FR[4], UR[4];
  physical_flux_fast(L, nx, ny, inv_gm1, FL, UL);
  physical_flux_fast(R, nx, ny, inv_gm1, FR, UR);
  double root_l = sqrt_rn(L.a), root_r = sqrt_rn(R.a);
  double iden = div_rn(1.0, root_l + root_r);
  double vx = (root_l * L.b + root_r * R.b) * iden;
  double vy = (root_l * L.c + root_r * R.c) * iden;
  // The reference's averaged "enthalpy" is sqrt(rho)-weighted p/rho + |u|^2/2
  // (euler.py:181-185); with rho = root^2, root * p / rho = p / root.
  double H = (div_rn(L.d, root_l) + div_rn(R.d, root_r) + 0.5 * (root_l * (L.b * L.b + L.c * L.c) +
                                                  root_r * (R.b * R.b + R.c * R.c))) * iden;
  double un = vx * nx + vy * ny;
  double ut = vx * -ny + vy * nx;
  double c2 = (gamma - 1.0) * (H - 0.5 * (vx * vx + vy * vy));
  if (!icmp::gt0(c2) || !icmp::finite(c2)) {
    out[0] = out[1] = out[2] = out[3] = 0.0;
    return MCFD_S_ROE_SOUND;
  }
  double c = sqrt_rn(c2);
  double ic2 = div_rn(1.0, c2);
  double ravg = root_l * root_r;
  double unl = L.b * nx + L.c * ny, unr = R.b * nx + R.c * ny;
  double utl = L.b * -ny + L.c * nx, utr = R.b * -ny + R.c * nx;
  double dr = R.a - L.a, dun = unr - unl, dut = utr - utl, dp = R.d - L.d;
  double am = (dp - (ravg * c) * dun) * (0.5 * ic2);
  double ap = (dp + (ravg * c) * dun) * (0.5 * ic2);
  double ac = dr - dp * ic2;
  double as = ravg * dut;
  double lam[4] = {un - c, un, un, un + c};
  double fix = 0.1 * c, ifix = div_rn(10.0, c);
  double w[4];
  double strength[4] = {am, ac, as, ap};
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    double a = abs_of(lam[j]);
    if (icmp::lt_nonneg(a, fix)) a = 0.5 * (a * a * ifix + fix);
    w[j] = a * strength[j];
  }
  double d0 = w[0] + w[1] + w[3];
  double d1 = (un - c) * w[0] + un * w[1] + (un + c) * w[3];
  double d2 = ut * (w[0] + w[1] + w[3]) + w[2];
  double d3 = (H - un * c) * w[0] + 0.5 * (un * un + ut * ut) * w[1] + ut * w[2] + (H + un * c) * w[3];
  double diss[4] = {d0, d1 * nx - d2 * ny, d1 * ny + d2 * nx, d3};
#pragma unroll
  for (int k = 0; k < 4; ++k) out[k] = 0.5 * ((FL[k] + FR[k]) - diss[k]);
  if (!(icmp::finite(out[0]) && icmp::finite(out[1]) && icmp::finite(out[2]) && icmp::finite(out[3])))
    return MCFD_S_ROE_NONFINITE;
  return 0;
}

// Cell limiter factor from the extreme increments.  Every limiter function g
// of the reference is non-decreasing in the ratio r (Venkatakrishnan's
// (r^2+2r+e)/(r^2+r+2+e) on [0,2] and capped at 1 beyond), so the minimum of
// g(r_e) over the entries is g(min_e r_e), and min_e r_e is reached at the
// largest positive increment ((hi-v)/inc) or the largest negative one
// ((v-lo)/|inc|), or is 1 when an increment lies within the tolerance band.
// The two candidate ratios a/b are compared by cross-multiplication and the
// limiter function is evaluated as a rational function of (a, b): one
// division per variable instead of two per entry.
template <int LIMITER>
__device__ __forceinline__ double limiter_factor_fast(double hi_minus_v, double pos_max, double v_minus_lo,
                                                      double neg_max, bool has_pos, bool has_neg, bool flat) {
  double a, b;
  if (has_pos && has_neg) {
    bool pos_smaller = !icmp::lt_nonneg(v_minus_lo * pos_max, hi_minus_v * neg_max);
    a = pos_smaller ? hi_minus_v : v_minus_lo;
    b = pos_smaller ? pos_max : neg_max;
  } else if (has_pos) {
    a = hi_minus_v;
    b = pos_max;
  } else if (has_neg) {
    a = v_minus_lo;
    b = neg_max;
  } else {
    return flat ? (LIMITER == 3 ? div_rn(3.0 + 1e-12, 4.0 + 1e-12) : 1.0) : 1.0;
  }
  if (flat && !icmp::lt_nonneg(a, b)) {  // the tolerance band's ratio 1 is the smallest
    a = 1.0;
    b = 1.0;
  }
  if (LIMITER <= 1) {
    return icmp::lt_nonneg(a, b) ? div_rn(a, b) : 1.0;
  } else if (LIMITER == 2) {
    if (!icmp::gt0(a)) return 0.0;
    double q = div_rn(2.0 * a, a + b);
    return icmp::lt_pos(q, 1.0) ? q : 1.0;
  } else {
    const double eps = 1e-12;
    if (!icmp::lt_nonneg(a, 2.0 * b)) return 1.0;
    double bb = b * b;
    return div_rn(a * a + 2.0 * a * b + eps * bb, a * a + a * b + 2.0 * bb + eps * bb);
  }
}

}  // namespace mcfd
