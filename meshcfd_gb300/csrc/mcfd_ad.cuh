// Forward-mode derivatives of the residual's pointwise functions.
//
// Dual<N> carries a value and N tangent components; every function below is a
// template over the scalar type, so Dual<1> gives an exact Jacobian-vector
// product and Dual<8> the full 4x8 Jacobian of a face flux (for the reverse
// mode).  The formulas are the reference's (euler.py, solver.py:4350-4409);
// only values decide branches, so at a switch the derivative is that of the
// branch the value takes (a subgradient of min / max / the HLLC regions).
#pragma once

#include <cuda_runtime.h>

#include "mcfd_device.cuh"

namespace mcfd {
namespace ad {

template <int N>
struct Dual {
  double v;
  double d[N];
  __device__ __forceinline__ Dual() : v(0.0) {
#pragma unroll
    for (int k = 0; k < N; ++k) d[k] = 0.0;
  }
  __device__ __forceinline__ Dual(double x) : v(x) {  // NOLINT: constants promote
#pragma unroll
    for (int k = 0; k < N; ++k) d[k] = 0.0;
  }
};

template <int N>
__device__ __forceinline__ Dual<N> operator+(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r;
  r.v = a.v + b.v;
#pragma unroll
  for (int k = 0; k < N; ++k) r.d[k] = a.d[k] + b.d[k];
  return r;
}
template <int N>
__device__ __forceinline__ Dual<N> operator-(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r;
  r.v = a.v - b.v;
#pragma unroll
  for (int k = 0; k < N; ++k) r.d[k] = a.d[k] - b.d[k];
  return r;
}
template <int N>
__device__ __forceinline__ Dual<N> operator-(const Dual<N>& a) {
  Dual<N> r;
  r.v = -a.v;
#pragma unroll
  for (int k = 0; k < N; ++k) r.d[k] = -a.d[k];
  return r;
}
template <int N>
__device__ __forceinline__ Dual<N> operator*(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r;
  r.v = a.v * b.v;
#pragma unroll
  for (int k = 0; k < N; ++k) r.d[k] = a.d[k] * b.v + a.v * b.d[k];
  return r;
}
template <int N>
__device__ __forceinline__ Dual<N> operator/(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r;
  const double ib = div_rn(1.0, b.v);
  r.v = a.v * ib;
#pragma unroll
  for (int k = 0; k < N; ++k) r.d[k] = (a.d[k] - r.v * b.d[k]) * ib;
  return r;
}
template <int N>
__device__ __forceinline__ Dual<N> sqrt(const Dual<N>& a) {
  Dual<N> r;
  r.v = sqrt_rn(a.v);
  const double h = div_rn(0.5, r.v);
#pragma unroll
  for (int k = 0; k < N; ++k) r.d[k] = a.d[k] * h;
  return r;
}
template <int N>
__device__ __forceinline__ Dual<N> fabs(const Dual<N>& a) {
  return icmp::neg_gt_pos(a.v, 0.0) ? -a : a;  // a.v < 0
}
template <int N>
__device__ __forceinline__ Dual<N> pow(const Dual<N>& a, double e) {
  Dual<N> r;
  r.v = ::pow(a.v, e);
  const double g = e * ::pow(a.v, e - 1.0);
#pragma unroll
  for (int k = 0; k < N; ++k) r.d[k] = a.d[k] * g;
  return r;
}

__device__ __forceinline__ double val(double x) { return x; }
template <int N>
__device__ __forceinline__ double val(const Dual<N>& x) {
  return x.v;
}

template <typename T>
struct S4 {
  T a, b, c, d;
};

template <typename T>
__device__ __forceinline__ T tmin(const T& a, const T& b) {  // Python min(a, b)
  return icmp::lt(val(b), val(a)) ? b : a;
}
template <typename T>
__device__ __forceinline__ T tmax(const T& a, const T& b) {  // Python max(a, b)
  return icmp::lt(val(a), val(b)) ? b : a;
}

// euler.conservative_to_primitive
template <typename T>
__device__ __forceinline__ S4<T> prim(const S4<T>& U, double gamma) {
  T rho = U.a;
  T ux = U.b / rho;
  T uy = U.c / rho;
  T p = T(gamma - 1.0) * (U.d - T(0.5) * (U.b * U.b + U.c * U.c) / rho);
  return S4<T>{rho, ux, uy, p};
}

// euler.physical_flux
template <typename T>
__device__ __forceinline__ void physical(const S4<T>& q, double nx, double ny, double gamma, T F[4], T U[4]) {
  T energy = q.d / T(gamma - 1.0) + T(0.5) * q.a * (q.b * q.b + q.c * q.c);
  T un = q.b * T(nx) + q.c * T(ny);
  U[0] = q.a;
  U[1] = q.a * q.b;
  U[2] = q.a * q.c;
  U[3] = energy;
  F[0] = q.a * un;
  F[1] = U[1] * un + q.d * T(nx);
  F[2] = U[2] * un + q.d * T(ny);
  F[3] = (energy + q.d) * un;
}

template <typename T>
__device__ __forceinline__ T sound(const S4<T>& q, double gamma) {
  return sqrt(T(gamma) * q.d / q.a);
}

template <typename T>
__device__ __forceinline__ void rusanov(const S4<T>& L, const S4<T>& R, double nx, double ny, double gamma,
                                        T out[4]) {
  T FL[4], UL[4], FR[4], UR[4];
  physical(L, nx, ny, gamma, FL, UL);
  physical(R, nx, ny, gamma, FR, UR);
  T sl = fabs(L.b * T(nx) + L.c * T(ny)) + sound(L, gamma);
  T sr = fabs(R.b * T(nx) + R.c * T(ny)) + sound(R, gamma);
  T s = val(sl) >= val(sr) ? sl : sr;
#pragma unroll
  for (int k = 0; k < 4; ++k) out[k] = T(0.5) * ((FL[k] + FR[k]) - s * (UR[k] - UL[k]));
}

template <typename T, bool KERNEL_BRANCHES>
__device__ __forceinline__ void hllc(const S4<T>& L, const S4<T>& R, double nx, double ny, double gamma, T out[4]) {
  T FL[4], UL[4], FR[4], UR[4];
  physical(L, nx, ny, gamma, FL, UL);
  physical(R, nx, ny, gamma, FR, UR);
  T unl = L.b * T(nx) + L.c * T(ny), unr = R.b * T(nx) + R.c * T(ny);
  T cl = sound(L, gamma), cr = sound(R, gamma);
  T wl = tmin(unl - cl, unr - cr);
  T wr = tmax(unl + cl, unr + cr);
  T den = L.a * (wl - unl) - R.a * (wr - unr);
  if (!(::fabs(val(den)) > 1e-14)) den = T(::copysign(1e-14, val(den)));
  T contact = ((R.d - L.d) + L.a * unl * (wl - unl) - R.a * unr * (wr - unr)) / den;
  int branch;
  if (KERNEL_BRANCHES) {
    if (val(wl) >= 0.0) branch = 0;
    else if (val(wr) <= 0.0) branch = 3;
    else branch = val(contact) >= 0.0 ? 1 : 2;
  } else {
    if (val(wl) >= 0.0) branch = 0;
    else if (val(contact) >= 0.0) branch = 1;
    else if (val(wr) > 0.0) branch = 2;
    else branch = 3;
  }
  if (branch == 0 || branch == 3) {
#pragma unroll
    for (int k = 0; k < 4; ++k) out[k] = branch == 0 ? FL[k] : FR[k];
    return;
  }
  const bool left = branch == 1;
  const S4<T>& q = left ? L : R;
  const T* U = left ? UL : UR;
  const T* F = left ? FL : FR;
  T un = left ? unl : unr;
  T wave = left ? wl : wr;
  T factor = q.a * (wave - un) / (wave - contact);
  T sux = q.b + (contact - un) * T(nx);
  T suy = q.c + (contact - un) * T(ny);
  T se = factor * (U[3] / q.a + (contact - un) * (contact + q.d / (q.a * (wave - un))));
  T star[4] = {factor, factor * sux, factor * suy, se};
#pragma unroll
  for (int k = 0; k < 4; ++k) out[k] = F[k] + wave * (star[k] - U[k]);
}

template <typename T>
__device__ __forceinline__ void roe(const S4<T>& L, const S4<T>& R, double nx, double ny, double gamma, T out[4]) {
  T FL[4], UL[4], FR[4], UR[4];
  physical(L, nx, ny, gamma, FL, UL);
  physical(R, nx, ny, gamma, FR, UR);
  T rl = sqrt(L.a), rr = sqrt(R.a);
  T den = rl + rr;
  T vx = (rl * L.b + rr * R.b) / den;
  T vy = (rl * L.c + rr * R.c) / den;
  T H = (rl * (L.d / L.a + T(0.5) * (L.b * L.b + L.c * L.c)) + rr * (R.d / R.a + T(0.5) * (R.b * R.b + R.c * R.c))) / den;
  T un = vx * T(nx) + vy * T(ny);
  T ut = vx * T(-ny) + vy * T(nx);
  T c2 = T(gamma - 1.0) * (H - T(0.5) * (vx * vx + vy * vy));
  T c = sqrt(c2);
  T ravg = rl * rr;
  T unl = L.b * T(nx) + L.c * T(ny), unr = R.b * T(nx) + R.c * T(ny);
  T utl = L.b * T(-ny) + L.c * T(nx), utr = R.b * T(-ny) + R.c * T(nx);
  T dr = R.a - L.a, dun = unr - unl, dut = utr - utl, dp = R.d - L.d;
  T am = (dp - ravg * c * dun) / (T(2.0) * c2);
  T ap = (dp + ravg * c * dun) / (T(2.0) * c2);
  T ac = dr - dp / c2;
  T as = ravg * dut;
  T lam[4] = {un - c, un, un, un + c};
  T fix = T(0.1) * c;
  T strength[4] = {am, ac, as, ap};
  T w[4];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    T a = fabs(lam[j]);
    if (val(a) < val(fix)) a = T(0.5) * (a * a / fix + fix);
    w[j] = a * strength[j];
  }
  T d0 = w[0] + w[1] + w[3];
  T d1 = (un - c) * w[0] + un * w[1] + (un + c) * w[3];
  T d2 = ut * (w[0] + w[1] + w[3]) + w[2];
  T d3 = (H - un * c) * w[0] + T(0.5) * (un * un + ut * ut) * w[1] + ut * w[2] + (H + un * c) * w[3];
  T diss[4] = {d0, d1 * T(nx) - d2 * T(ny), d1 * T(ny) + d2 * T(nx), d3};
#pragma unroll
  for (int k = 0; k < 4; ++k) out[k] = T(0.5) * ((FL[k] + FR[k]) - diss[k]);
}

template <typename T>
__device__ __forceinline__ S4<T> far_field(const S4<T>& in, const S4<T>& far, double nx, double ny, double gamma) {
  T ui = in.b * T(nx) + in.c * T(ny);
  T uf = far.b * T(nx) + far.c * T(ny);
  T ci = sound(in, gamma), cf = sound(far, gamma);
  if (val(ui) <= -val(ci)) return far;
  if (val(ui) >= val(ci)) return in;
  T out_inv = ui + T(2.0) * ci / T(gamma - 1.0);
  T in_inv = uf - T(2.0) * cf / T(gamma - 1.0);
  T vb = T(0.5) * (out_inv + in_inv);
  T cb = T(0.25 * (gamma - 1.0)) * (out_inv - in_inv);
  const S4<T>& src = val(vb) < 0.0 ? far : in;
  T entropy = src.d / pow(src.a, gamma);
  T rho = pow(cb * cb / (T(gamma) * entropy), 1.0 / (gamma - 1.0));
  T p = entropy * pow(rho, gamma);
  T vt = src.b * T(-ny) + src.c * T(nx);
  return S4<T>{rho, vb * T(nx) + vt * T(-ny), vb * T(ny) + vt * T(nx), p};
}

template <typename T>
__device__ __forceinline__ void numerical_flux(int flux, bool kernel_hllc, const S4<T>& L, const S4<T>& R, double nx,
                                               double ny, double gamma, T out[4]) {
  if (flux == MCFD_FLUX_RUSANOV) rusanov(L, R, nx, ny, gamma, out);
  else if (flux == MCFD_FLUX_HLLC) {
    if (kernel_hllc) hllc<T, true>(L, R, nx, ny, gamma, out);
    else hllc<T, false>(L, R, nx, ny, gamma, out);
  } else roe(L, R, nx, ny, gamma, out);
}

}  // namespace ad
}  // namespace mcfd
