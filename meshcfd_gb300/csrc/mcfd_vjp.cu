// Reverse mode: U_bar = (dR/dU)^T lambda for the residual of mcfd_residual,
// and the wall pressure-force functional.  No counterpart in the reference
// (it has no derivatives beyond its finite-difference JVP).
//
// Kernels, none with atomics:
// * k_vjp_face (per flux face): the face adjoint F_bar = sum over the face's
//   cells of the divergence coefficient times lambda, then the face-state
//   adjoints Q_bar_L, Q_bar_R = (dF/dQ)^T F_bar from a 4x8 forward-mode
//   Jacobian of the flux (ghost states included; on far-field faces the
//   second four tangents are the far-field state, giving its gradient);
// * k_vjp_cell (per cell): reverse of the face states Q = P + phi (G . r),
//   of the limiter through its minimising entry and extreme neighbour, and of
//   the least-squares gradient; contributions to neighbours are written per
//   gradient entry;
// * k_vjp_collect (per cell): gathers the neighbours' entry contributions
//   through each entry's twin (b -> a for a -> b), then U_bar = (dP/dU)^T P_bar.
// Switches (HLLC region, limiter band, extreme neighbour, min over entries)
// follow the state's values: the result is the transpose of mcfd_jvp's
// Jacobian to rounding.  Compiled with FMA contraction and shared
// reciprocals: derivatives need accuracy, not the reference's rounding.
#include "mcfd_ad.cuh"
#include "mcfd_internal.h"
#include "mcfd_vjp.h"

namespace mcfd {
namespace {

constexpr int kBlock = 256;
inline int blocks_for(int n) { return (n + kBlock - 1) / kBlock; }

template <int N>
__device__ __forceinline__ ad::Dual<N> seed(double v, int k) {
  ad::Dual<N> x(v);
  if (k >= 0) x.d[k] = 1.0;
  return x;
}

// ------------------------------------------------ hand-written reverse mode
//
// Reverse sweeps of the Rusanov and HLLC fluxes (the same expressions, branch
// choices and Python min / max tie rules as mcfd_ad.cuh, so the result is
// the transpose of the forward-mode Jacobian to rounding) at a fraction of
// the cost of the 4x8 dual-number Jacobian.  qb accumulates.

// physical_flux (euler.py:43-57): adjoints of F and of U = (r, r u, r v, E)
__device__ __forceinline__ void physical_bar(const St4& q, double nx, double ny, double inv_gm1, const double Fb[4],
                                             const double Ub[4], double qb[4]) {
  const double r = q.a, u = q.b, v = q.c, p = q.d;
  const double un = u * nx + v * ny;
  const double E = p * inv_gm1 + 0.5 * r * (u * u + v * v);
  const double unb = Fb[0] * r + Fb[1] * (r * u) + Fb[2] * (r * v) + Fb[3] * (E + p);
  const double U1b = Fb[1] * un + Ub[1], U2b = Fb[2] * un + Ub[2], Eb = Fb[3] * un + Ub[3];
  qb[0] += Fb[0] * un + Ub[0] + U1b * u + U2b * v + Eb * (0.5 * (u * u + v * v));
  qb[1] += U1b * r + Eb * (r * u) + unb * nx;
  qb[2] += U2b * r + Eb * (r * v) + unb * ny;
  qb[3] += Fb[1] * nx + Fb[2] * ny + Fb[3] * un + Eb * inv_gm1;
}

// c = sqrt(gamma p / r): dc/dp = gamma / (2 r c), dc/dr = -c / (2 r)
struct Sound {
  double c, dp, dr, inv_r;
};
__device__ __forceinline__ Sound sound_d(const St4& q, double gamma) {
  const double inv_r = div_rn(1.0, q.a);
  const double c = sqrt_rn(gamma * q.d * inv_r);
  const double h = 0.5 * inv_r;
  return Sound{c, div_rn(gamma * h, c), -c * h, inv_r};
}

__device__ __forceinline__ void rusanov_bar(const St4& L, const St4& R, double nx, double ny, double gamma,
                                            double inv_gm1, const double Fb[4], double Lb[4], double Rb[4]) {
  const double unl = L.b * nx + L.c * ny, unr = R.b * nx + R.c * ny;
  const Sound sl_ = sound_d(L, gamma), sr_ = sound_d(R, gamma);
  const double sl = abs_of(unl) + sl_.c, sr = abs_of(unr) + sr_.c;
  const bool left = !icmp::lt_nonneg(sl, sr);  // sl >= sr
  const double s = left ? sl : sr;
  const double UL[4] = {L.a, L.a * L.b, L.a * L.c, L.d * inv_gm1 + 0.5 * L.a * (L.b * L.b + L.c * L.c)};
  const double UR[4] = {R.a, R.a * R.b, R.a * R.c, R.d * inv_gm1 + 0.5 * R.a * (R.b * R.b + R.c * R.c)};
  double FLb[4], ULb[4], URb[4], sb = 0.0;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    FLb[k] = 0.5 * Fb[k];
    sb -= 0.5 * Fb[k] * (UR[k] - UL[k]);
    URb[k] = -0.5 * s * Fb[k];
    ULb[k] = 0.5 * s * Fb[k];
  }
  physical_bar(L, nx, ny, inv_gm1, FLb, ULb, Lb);
  physical_bar(R, nx, ny, inv_gm1, FLb, URb, Rb);
  double* qb = left ? Lb : Rb;
  const Sound& sd = left ? sl_ : sr_;
  const double unb = icmp::neg_gt_pos(left ? unl : unr, 0.0) ? negate(sb) : sb;
  qb[0] += sb * sd.dr;
  qb[1] += unb * nx;
  qb[2] += unb * ny;
  qb[3] += sb * sd.dp;
}

template <bool KERNEL_BRANCHES>
__device__ __forceinline__ void hllc_bar(const St4& L, const St4& R, double nx, double ny, double gamma,
                                         double inv_gm1, const double Fb[4], double Lb[4], double Rb[4]) {
  const double unl = L.b * nx + L.c * ny, unr = R.b * nx + R.c * ny;
  const Sound sl_ = sound_d(L, gamma), sr_ = sound_d(R, gamma);
  const double cl = sl_.c, cr = sr_.c;
  const double a1 = unl - cl, b1 = unr - cr;
  const bool wl_right = icmp::lt(b1, a1);
  const double wl = wl_right ? b1 : a1;
  const double a2 = unl + cl, b2 = unr + cr;
  const bool wr_right = icmp::lt(a2, b2);
  const double wr = wr_right ? b2 : a2;
  double den = L.a * (wl - unl) - R.a * (wr - unr);
  const bool guarded = !icmp::abs_gt(den, 1e-14);
  if (guarded) den = with_sign_of(1e-14, den);
  const double inv_den = div_rn(1.0, den);
  const double contact = ((R.d - L.d) + L.a * unl * (wl - unl) - R.a * unr * (wr - unr)) * inv_den;
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
  // Branches 0 and 3 take one side's physical flux; the star branches add
  // the star state's terms.  physical_bar runs once for every lane (with a
  // zero state adjoint outside the star region), so a warp mixing
  // supersonic and subsonic faces does not issue it twice.
  const bool star = branch == 1 || branch == 2;
  const bool left = branch <= 1;
  const St4& q = left ? L : R;
  double* qb = left ? Lb : Rb;
  double Uqb[4] = {0.0, 0.0, 0.0, 0.0};
  double wb = 0.0, rb = 0.0, suxb = 0.0, suyb = 0.0, unb = 0.0, pb = 0.0, contactb = 0.0;
  if (star) {
    const double un = left ? unl : unr, w = left ? wl : wr;
    const double r = q.a, u = q.b, v = q.c, p = q.d;
    const double inv_r = left ? sl_.inv_r : sr_.inv_r;
    const double E = p * inv_gm1 + 0.5 * r * (u * u + v * v);
    const double Uq[4] = {r, r * u, r * v, E};
    const double wu = w - un;
    const double B = w - contact, inv_B = div_rn(1.0, B), A = r * wu, factor = A * inv_B;
    const double dc = contact - un;
    const double sux = u + dc * nx, suy = v + dc * ny;
    const double inv_Z = div_rn(inv_r, wu);  // 1 / (r (w - un))
    const double pz = p * inv_Z;
    const double Y = contact + pz, Er = E * inv_r, X = Er + dc * Y;
    const double star_state[4] = {factor, factor * sux, factor * suy, factor * X};
    // Reverse sweep.  Products that share a factor are grouped (Uq_bar =
    // -star_bar exactly; Z_bar and A_bar enter r, w and un only through their
    // sum; the contact's numerator and denominator adjoints through
    // numb * un + denb per side), which removes about a fifth of the FP64
    // operations of the term-by-term transpose; the results agree to rounding.
    double starb[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      wb += Fb[k] * (star_state[k] - Uq[k]);
      starb[k] = w * Fb[k];
      Uqb[k] = negate(starb[k]);
    }
    const double factorb = starb[0] + starb[1] * sux + starb[2] * suy + starb[3] * X;
    suxb = starb[1] * factor;
    suyb = starb[2] * factor;
    const double Xb = starb[3] * factor;
    const double Xr = Xb * inv_r;
    Uqb[3] += Xr;
    const double dcb = Xb * Y + suxb * nx + suyb * ny;
    const double Yb = Xb * dc;
    pb = Yb * inv_Z;
    const double Ab = factorb * inv_B;
    const double ZA = Ab - pb * pz;  // Z_bar + A_bar, Z_bar = -Yb pz / Z
    rb = ZA * wu - Xr * Er;
    unb = negate(dcb + ZA * r);
    wb += ZA * r - Ab * factor;  // + B_bar = -A_bar factor
    contactb = Yb + dcb + Ab * factor;
  }
  physical_bar(q, nx, ny, inv_gm1, Fb, Uqb, qb);
  if (!star) return;
  qb[0] += rb;
  qb[1] += suxb + unb * nx;
  qb[2] += suyb + unb * ny;
  qb[3] += pb;
  // contact = num / den: num_bar = contact_bar / den, den_bar = -num_bar contact
  const double numb = contactb * inv_den, denb = guarded ? 0.0 : negate(numb * contact);
  Rb[3] += numb;
  Lb[3] -= numb;
  const double dl = wl - unl, dr = wr - unr;
  const double tl = numb * unl + denb, tr = numb * unr + denb;
  Lb[0] += tl * dl;
  Rb[0] -= tr * dr;
  double unlb = L.a * (numb * dl - tl), unrb = R.a * (tr - numb * dr);
  double wlb = left ? wb : 0.0, wrb = left ? 0.0 : wb, clb = 0.0, crb = 0.0;
  wlb += L.a * tl;
  wrb -= R.a * tr;
  if (wl_right) {
    unrb += wlb;
    crb -= wlb;
  } else {
    unlb += wlb;
    clb -= wlb;
  }
  if (wr_right) {
    unrb += wrb;
    crb += wrb;
  } else {
    unlb += wrb;
    clb += wrb;
  }
  Lb[0] += clb * sl_.dr;
  Lb[3] += clb * sl_.dp;
  Rb[0] += crb * sr_.dr;
  Rb[3] += crb * sr_.dp;
  Lb[1] += unlb * nx;
  Lb[2] += unlb * ny;
  Rb[1] += unrb * nx;
  Rb[2] += unrb * ny;
}

// Resident 256-thread blocks per SM the face reverse is compiled for.
#ifndef MCFD_VJP_FACE_MIN_BLOCKS
#define MCFD_VJP_FACE_MIN_BLOCKS 1
#endif

// Face VJP by the hand-written reverse (Rusanov / HLLC on every segment but
// the far field, whose ghost state keeps the dual-number path).
template <int FLUX, int SEG, bool FO, bool KH>
__global__ void __launch_bounds__(kBlock, MCFD_VJP_FACE_MIN_BLOCKS) k_vjp_face_rev(DevGeom g, const double* __restrict__ P,
                                                         const double* __restrict__ recon,
                                                         const double* __restrict__ lambda, double gamma,
                                                         double inv_gm1, double* __restrict__ slot_bar) {
  const int begin = g.seg_begin[SEG];
  const int f = begin + blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= g.seg_begin[SEG + 1]) return;
  const double2 n = g.ff_normal[f];
  const double len = g.ff_len[f];
  const int lc = g.ff_lcell[f];
  const St4 la = ld4(lambda + 4 * (size_t)lc);
  const double wl = div_rn(-len, g.area[lc]);
  double fb[4] = {wl * la.a, wl * la.b, wl * la.c, wl * la.d};
  if (SEG == SEG_INTERIOR || SEG == SEG_PERIODIC) {
    const St4 lb = ld4(lambda + 4 * (size_t)g.ff_rcell[f]);
    const double wr = div_rn(len, g.area[g.ff_rcell[f]]);
    fb[0] += wr * lb.a; fb[1] += wr * lb.b; fb[2] += wr * lb.c; fb[3] += wr * lb.d;
  }
  const St4 L = FO ? ld4(P + 4 * (size_t)lc) : ld4(recon + 4 * (size_t)g.ff_lslot[f]);
  St4 R;
  double2 wv = make_double2(0.0, 0.0);
  if (SEG == SEG_INTERIOR || SEG == SEG_PERIODIC) {
    R = FO ? ld4(P + 4 * (size_t)g.ff_rcell[f]) : ld4(recon + 4 * (size_t)g.ff_rslot[f]);
  } else if (SEG == SEG_WALL) {
    wv = g.ff_wall_velocity[f - begin];
    const double un = (L.b - wv.x) * n.x + (L.c - wv.y) * n.y;
    R = St4{L.a, L.b - 2.0 * un * n.x, L.c - 2.0 * un * n.y, L.d};
  } else if (SEG == SEG_VIN) {
    R = ld4(g.ff_vin_state + 4 * (size_t)(f - begin));
  } else {
    R = St4{L.a, L.b, L.c, g.ff_pout_pressure[f - begin]};
  }
  double Lb[4] = {0.0, 0.0, 0.0, 0.0}, Rb[4] = {0.0, 0.0, 0.0, 0.0};
  if (FLUX == MCFD_FLUX_RUSANOV) rusanov_bar(L, R, n.x, n.y, gamma, inv_gm1, fb, Lb, Rb);
  else hllc_bar<(SEG == SEG_INTERIOR) && KH>(L, R, n.x, n.y, gamma, inv_gm1, fb, Lb, Rb);
  if (SEG == SEG_WALL) {  // R = mirror(L)
    const double unb = -2.0 * (Rb[1] * n.x + Rb[2] * n.y);
    Lb[0] += Rb[0];
    Lb[1] += Rb[1] + unb * n.x;
    Lb[2] += Rb[2] + unb * n.y;
    Lb[3] += Rb[3];
  } else if (SEG == SEG_POUT) {
    Lb[0] += Rb[0];
    Lb[1] += Rb[1];
    Lb[2] += Rb[2];
  }
  st4(slot_bar + 4 * (size_t)g.ff_lslot[f], St4{Lb[0], Lb[1], Lb[2], Lb[3]});
  if (SEG == SEG_INTERIOR || SEG == SEG_PERIODIC)
    st4(slot_bar + 4 * (size_t)g.ff_rslot[f], St4{Rb[0], Rb[1], Rb[2], Rb[3]});
}

template <int FLUX, int SEG, bool FO, bool KH>
__global__ void __launch_bounds__(kBlock) k_vjp_face(DevGeom g, const double* __restrict__ P,
                                                     const double* __restrict__ recon,
                                                     const double* __restrict__ lambda, double gamma,
                                                     double* __restrict__ slot_bar, double* __restrict__ far_bar) {
  using D8 = ad::Dual<8>;
  using S = ad::S4<D8>;
  const int begin = g.seg_begin[SEG];
  const int f = begin + blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= g.seg_begin[SEG + 1]) return;
  const double2 n = g.ff_normal[f];
  const double len = g.ff_len[f];
  const int lc = g.ff_lcell[f];
  // face adjoint (solver.py:2164-2165 coefficients, boundary -(F L)/A)
  const St4 la = ld4(lambda + 4 * (size_t)lc);
  const double wl = div_rn(-len, g.area[lc]);
  double fb[4] = {wl * la.a, wl * la.b, wl * la.c, wl * la.d};
  if (SEG == SEG_INTERIOR || SEG == SEG_PERIODIC) {
    const int rc = g.ff_rcell[f];
    const St4 lb = ld4(lambda + 4 * (size_t)rc);
    const double wr = div_rn(len, g.area[rc]);
    fb[0] += wr * lb.a; fb[1] += wr * lb.b; fb[2] += wr * lb.c; fb[3] += wr * lb.d;
  }
  const St4 qL = FO ? ld4(P + 4 * (size_t)lc) : ld4(recon + 4 * (size_t)g.ff_lslot[f]);
  S L{seed<8>(qL.a, 0), seed<8>(qL.b, 1), seed<8>(qL.c, 2), seed<8>(qL.d, 3)};
  S R;
  if (SEG == SEG_INTERIOR || SEG == SEG_PERIODIC) {
    const St4 qR = FO ? ld4(P + 4 * (size_t)g.ff_rcell[f]) : ld4(recon + 4 * (size_t)g.ff_rslot[f]);
    R = S{seed<8>(qR.a, 4), seed<8>(qR.b, 5), seed<8>(qR.c, 6), seed<8>(qR.d, 7)};
  } else if (SEG == SEG_WALL) {
    const double2 wv = g.ff_wall_velocity[f - begin];
    D8 un = (L.b - D8(wv.x)) * D8(n.x) + (L.c - D8(wv.y)) * D8(n.y);
    R = S{L.a, L.b - D8(2.0) * un * D8(n.x), L.c - D8(2.0) * un * D8(n.y), L.d};
  } else if (SEG == SEG_VIN) {
    const St4 x = ld4(g.ff_vin_state + 4 * (size_t)(f - begin));
    R = S{D8(x.a), D8(x.b), D8(x.c), D8(x.d)};
  } else if (SEG == SEG_POUT) {
    R = S{L.a, L.b, L.c, D8(g.ff_pout_pressure[f - begin])};
  } else {
    const St4 x = ld4(g.ff_far_state + 4 * (size_t)(f - begin));
    S far{seed<8>(x.a, 4), seed<8>(x.b, 5), seed<8>(x.c, 6), seed<8>(x.d, 7)};
    R = ad::far_field(L, far, n.x, n.y, gamma);
  }
  D8 F[4];
  ad::numerical_flux<D8>(FLUX, (SEG == SEG_INTERIOR) && KH, L, R, n.x, n.y, gamma, F);
  double bar[8];
#pragma unroll
  for (int t = 0; t < 8; ++t) bar[t] = fb[0] * F[0].d[t] + fb[1] * F[1].d[t] + fb[2] * F[2].d[t] + fb[3] * F[3].d[t];
  st4(slot_bar + 4 * (size_t)g.ff_lslot[f], St4{bar[0], bar[1], bar[2], bar[3]});
  if (SEG == SEG_INTERIOR || SEG == SEG_PERIODIC)
    st4(slot_bar + 4 * (size_t)g.ff_rslot[f], St4{bar[4], bar[5], bar[6], bar[7]});
  if (SEG == SEG_FAR && far_bar) st4(far_bar + 4 * (size_t)(f - begin), St4{bar[4], bar[5], bar[6], bar[7]});
}

template <int LIMITER>
__device__ __forceinline__ double limiter_slope(double r) {
  if (LIMITER <= 1) return icmp::lt(r, 1.0) ? 1.0 : 0.0;
  if (LIMITER == 2) {
    if (!icmp::gt0(r)) return 0.0;
    return icmp::lt(r, 1.0) ? div_rn(2.0, (1.0 + r) * (1.0 + r)) : 0.0;  // 2r / (1 + r) < 1 iff r < 1
  }
  const double eps = 1e-12;
  const double N = r * r + 2.0 * r + eps, D = r * r + r + 2.0 + eps;
  if (N > D) return 0.0;  // capped at 1
  const double inv_D = div_rn(1.0, D);
  return ((2.0 * r + 2.0) * D - N * (2.0 * r + 1.0)) * (inv_D * inv_D);
}

// The cell reverse of one variable (the cell kernel's loop body): the
// variable's gradient and extremes, limiter minimum and its first entry,
// then the reverse of the face states, of the limiter and of the gradient.
// One variable's state is live at a time (96 registers instead of 128 with
// spills for all four at once), and its increments are kept for the reverse
// instead of being recomputed.  NS > 0 compiles the cell for exactly NS
// limiter entries (the cell order makes the count warp-uniform, so a warp of
// triangles issues no FP64 work for a fourth entry); NS = 0 handles any
// count, keeping the first four increments.
// The cell reverse of one variable for the smooth Venkatakrishnan form: the
// forward's gradient, increments and face factors in the forward kernels'
// rounding (separately rounded products), the first face of least factor,
// then the reverse of the face states and of that face's factor through d1
// (the extreme neighbour, or the cell) and d2 (the gradient).
template <int NS>
__device__ __forceinline__ void vjp_cell_variable_vk(const DevGeom& g, const double* __restrict__ P,
                                                     const double* __restrict__ slot_bar, int v, double pv,
                                                     int e0, int e1, int s0, int s1, double& pb,
                                                     double* __restrict__ ent_bar, double e2) {
  double gx = 0.0, gy = 0.0, lo = pv, hi = pv;
  int lo_e = -1, hi_e = -1;
  for (int e = e0; e < e1; ++e) {
    const double q = P[4 * (size_t)g.grad_nb[e] + v];
    const double d = q - pv;
    gx = gx + mul_rn(g.grad_cx[e], d);
    gy = gy + mul_rn(g.grad_cy[e], d);
    if (icmp::lt(q, lo)) { lo = q; lo_e = e; }
    if (icmp::lt(hi, q)) { hi = q; hi_e = e; }
  }
  constexpr int kCache = NS > 0 ? NS : 4;
  double incs[kCache];
  double phi = 1.0, arg_inc = 0.0;
  int arg = -1;
  auto consider = [&](int s, double inc) {
    const double f = venkat_k_face(pv, inc, lo, hi, e2).f;
    if (arg < 0 || icmp::lt(f, phi)) {
      phi = f;
      arg = s;
      arg_inc = inc;
    }
  };
#pragma unroll
  for (int k = 0; k < kCache; ++k) {
    incs[k] = 0.0;
    if (NS > 0 || s0 + k < s1) {
      const double2 dd = g.lim_d[s0 + k];
      incs[k] = __dadd_rn(mul_rn(gx, dd.x), mul_rn(gy, dd.y));
      consider(s0 + k, incs[k]);
    }
  }
  if (NS == 0) {
    for (int s = s0 + kCache; s < s1; ++s) {
      const double2 dd = g.lim_d[s];
      consider(s, __dadd_rn(mul_rn(gx, dd.x), mul_rn(gy, dd.y)));
    }
  }
  // reverse of Q_s = P + phi (G . r_s)
  double phib = 0.0, gxb = 0.0, gyb = 0.0;
  auto face_reverse = [&](int s, double inc, const double2& dd) {
    const double qb = slot_bar[4 * (size_t)g.lim_slot[s] + v];
    phib += qb * inc;
    const double qphi = qb * phi;
    gxb += qphi * dd.x;
    gyb += qphi * dd.y;
  };
#pragma unroll
  for (int k = 0; k < kCache; ++k)
    if (NS > 0 || s0 + k < s1) face_reverse(s0 + k, incs[k], g.lim_d[s0 + k]);
  if (NS == 0) {
    for (int s = s0 + kCache; s < s1; ++s) {
      const double2 dd = g.lim_d[s];
      face_reverse(s, __dadd_rn(mul_rn(gx, dd.x), mul_rn(gy, dd.y)), dd);
    }
  }
  // reverse of phi = f(d1, d2) at the minimising face
  double extb = 0.0;
  int ext_e = -1;
  if (arg >= 0) {
    const VenkatK f = venkat_k_face(pv, arg_inc, lo, hi, e2);
    double a, b;
    venkat_k_slopes(f, arg_inc, &a, &b);
    const double d1b = a * phib, incb = b * phib;
    pb -= d1b;
    const int ee = icmp::gt0(arg_inc) ? hi_e : lo_e;
    if (ee < 0) pb += d1b;  // the extreme is the cell itself
    else { extb = d1b; ext_e = ee; }
    const double2 dd = g.lim_d[arg];
    gxb += incb * dd.x;
    gyb += incb * dd.y;
  }
  // reverse of G = sum_e coef_e (P_nb - P_c): neighbour share per entry
  for (int e = e0; e < e1; ++e) {
    const double w = g.grad_cx[e] * gxb + g.grad_cy[e] * gyb;
    pb -= w;
    ent_bar[4 * (size_t)e + v] = w + (ext_e == e ? extb : 0.0);
  }
}

template <int LIMITER, int NS>
__device__ __forceinline__ void vjp_cell_variable(const DevGeom& g, const double* __restrict__ P,
                                                  const double* __restrict__ slot_bar, int v, double pv,
                                                  int e0, int e1, int s0, int s1, double& pb,
                                                  double* __restrict__ ent_bar) {
  double gx = 0.0, gy = 0.0, lo = pv, hi = pv;
  int lo_e = -1, hi_e = -1;
  for (int e = e0; e < e1; ++e) {
    const double q = P[4 * (size_t)g.grad_nb[e] + v];
    const double d = q - pv;
    gx = gx + g.grad_cx[e] * d;
    gy = gy + g.grad_cy[e] * d;
    if (icmp::lt(q, lo)) { lo = q; lo_e = e; }
    if (icmp::lt(hi, q)) { hi = q; hi_e = e; }
  }
  // phi = min over entries of f(max(r, 0)) and its first entry, from the
  // three candidates (largest positive increment, most negative, first
  // entry in the tolerance band)
  const double tol = limiter_tolerance(pv);
  double pmax = 0.0, nmin = 0.0;
  int ps = -1, ns = -1, fs = -1;
  constexpr int kCache = NS > 0 ? NS : 4;
  double incs[kCache];
  auto classify = [&](int s, double inc) {
    if (icmp::gt_pos(inc, tol)) {
      if (ps < 0 || icmp::lt(pmax, inc)) { pmax = inc; ps = s; }
    } else if (icmp::neg_gt_pos(inc, tol)) {
      if (ns < 0 || icmp::lt(inc, nmin)) { nmin = inc; ns = s; }
    } else if (fs < 0) {
      fs = s;
    }
  };
#pragma unroll
  for (int k = 0; k < kCache; ++k) {
    incs[k] = 0.0;
    if (NS > 0 || s0 + k < s1) {
      const double2 dd = g.lim_d[s0 + k];
      incs[k] = mul_rn(gx, dd.x) + gy * dd.y;
      classify(s0 + k, incs[k]);
    }
  }
  if (NS == 0) {
    for (int s = s0 + kCache; s < s1; ++s) {
      const double2 dd = g.lim_d[s];
      classify(s, mul_rn(gx, dd.x) + gy * dd.y);
    }
  }
  double phi = 1.0;
  int arg = -1;
  {
    const int cand[3] = {ps, ns, fs};
    const double cinc[3] = {pmax, nmin, 0.0};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      if (cand[k] < 0) continue;
      const double f = limiter_face_factor<LIMITER>(pv, cinc[k], lo, hi, tol);
      if (icmp::lt_nonneg(f, phi) || (icmp::key(f) == icmp::key(phi) && arg >= 0 && cand[k] < arg)) {
        phi = f;
        arg = cand[k];
      }
    }
  }
  // reverse of Q_s = P + phi (G . r_s)
  double phib = 0.0, gxb = 0.0, gyb = 0.0;
  auto face_reverse = [&](int s, double inc, const double2& dd) {
    const double qb = slot_bar[4 * (size_t)g.lim_slot[s] + v];
    phib += qb * inc;
    const double qphi = mul_rn(qb, phi);
    gxb += qphi * dd.x;
    gyb += qphi * dd.y;
  };
#pragma unroll
  for (int k = 0; k < kCache; ++k)
    if (NS > 0 || s0 + k < s1) face_reverse(s0 + k, incs[k], g.lim_d[s0 + k]);
  if (NS == 0) {
    for (int s = s0 + kCache; s < s1; ++s) {
      const double2 dd = g.lim_d[s];
      face_reverse(s, mul_rn(gx, dd.x) + gy * dd.y, dd);
    }
  }
  // reverse of the limiter through its minimising entry
  double extb = 0.0;
  int ext_e = -1;
  if (arg >= 0) {
    const double2 dd = g.lim_d[arg];
    const int k = arg - s0;
    double inc = incs[0];
#pragma unroll
    for (int m = 1; m < kCache; ++m)
      if (k == m) inc = incs[m];
    if (NS == 0 && k >= kCache) inc = mul_rn(gx, dd.x) + gy * dd.y;
    const bool pos = icmp::gt_pos(inc, tol), neg = icmp::neg_gt_pos(inc, tol);
    if (pos || neg) {
      const double num = pos ? hi - pv : lo - pv;
      const double inv_inc = div_rn(1.0, inc);
      const double r = num * inv_inc;
      if (icmp::gt0(r)) {
        const double rb = limiter_slope<LIMITER>(r) * phib;
        const double numb = rb * inv_inc;
        const double incb = -numb * r;
        pb -= numb;
        const int ee = pos ? hi_e : lo_e;
        if (ee < 0) pb += numb;  // the extreme is the cell itself
        else { extb = numb; ext_e = ee; }
        gxb += incb * dd.x;
        gyb += incb * dd.y;
      }
    }
  }
  // reverse of G = sum_e coef_e (P_nb - P_c): neighbour share per entry
  for (int e = e0; e < e1; ++e) {
    const double w = mul_rn(g.grad_cx[e], gxb) + g.grad_cy[e] * gyb;
    pb -= w;
    ent_bar[4 * (size_t)e + v] = w + (ext_e == e ? extb : 0.0);
  }
}

// Resident 256-thread blocks per SM the cell reverse is compiled for.
#ifndef MCFD_VJP_CELL_MIN_BLOCKS
#define MCFD_VJP_CELL_MIN_BLOCKS 2
#endif

template <int LIMITER, bool FO>
__global__ void __launch_bounds__(kBlock, MCFD_VJP_CELL_MIN_BLOCKS) k_vjp_cell(DevGeom g, const double* __restrict__ P,
                                                     const double* __restrict__ lambda,
                                                     const double* __restrict__ slot_bar, double ax, double ay,
                                                     double* __restrict__ pbar, double* __restrict__ ent_bar,
                                                     double venkat_k) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= g.n_cells) return;
  const int c = g.cell_order[i];  // groups equal stencil sizes; outputs do not depend on the order
  const St4 p = ld4(P + 4 * (size_t)c);
  const double pv[4] = {p.a, p.b, p.c, p.d};
  const int e0 = g.grad_ptr[c], e1 = g.grad_ptr[c + 1];
  const int s0 = g.lim_ptr[c], s1 = g.lim_ptr[c + 1];
  double pb[4] = {0.0, 0.0, 0.0, 0.0};
  for (int s = s0; s < s1; ++s) {
    const St4 q = ld4(slot_bar + 4 * (size_t)g.lim_slot[s]);
    pb[0] += q.a; pb[1] += q.b; pb[2] += q.c; pb[3] += q.d;
  }
  if constexpr (!FO && LIMITER == MCFD_LIMITER_VENKATAKRISHNAN_K) {
    const double e2 = venkat_k_e2(venkat_k, g.area[c]);
    if (s1 - s0 == 3) {
#pragma unroll
      for (int v = 0; v < 4; ++v) vjp_cell_variable_vk<3>(g, P, slot_bar, v, pv[v], e0, e1, s0, s1, pb[v], ent_bar, e2);
    } else if (s1 - s0 == 4) {
#pragma unroll
      for (int v = 0; v < 4; ++v) vjp_cell_variable_vk<4>(g, P, slot_bar, v, pv[v], e0, e1, s0, s1, pb[v], ent_bar, e2);
    } else {
#pragma unroll
      for (int v = 0; v < 4; ++v) vjp_cell_variable_vk<0>(g, P, slot_bar, v, pv[v], e0, e1, s0, s1, pb[v], ent_bar, e2);
    }
  } else if (!FO) {
    if (s1 - s0 == 3) {
#pragma unroll
      for (int v = 0; v < 4; ++v) vjp_cell_variable<LIMITER, 3>(g, P, slot_bar, v, pv[v], e0, e1, s0, s1, pb[v], ent_bar);
    } else if (s1 - s0 == 4) {
#pragma unroll
      for (int v = 0; v < 4; ++v) vjp_cell_variable<LIMITER, 4>(g, P, slot_bar, v, pv[v], e0, e1, s0, s1, pb[v], ent_bar);
    } else {
#pragma unroll
      for (int v = 0; v < 4; ++v) vjp_cell_variable<LIMITER, 0>(g, P, slot_bar, v, pv[v], e0, e1, s0, s1, pb[v], ent_bar);
    }
  }
  if (ax != 0.0 || ay != 0.0) {  // body force (solver.py:2709-2715)
    const St4 l = ld4(lambda + 4 * (size_t)c);
    pb[0] += l.b * ax + l.c * ay + l.d * (ax * p.b + ay * p.c);
    pb[1] += l.d * p.a * ax;
    pb[2] += l.d * p.a * ay;
  }
  st4(pbar + 4 * (size_t)c, St4{pb[0], pb[1], pb[2], pb[3]});
}

template <bool FO>
__global__ void __launch_bounds__(kBlock) k_vjp_collect(DevGeom g, const double* __restrict__ P,
                                                        const double* __restrict__ pbar,
                                                        const double* __restrict__ ent_bar, double gamma,
                                                        double* __restrict__ ubar) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= g.n_cells) return;
  St4 pb = ld4(pbar + 4 * (size_t)c);
  if (!FO) {
    for (int e = g.grad_ptr[c]; e < g.grad_ptr[c + 1]; ++e) {
      const St4 x = ld4(ent_bar + 4 * (size_t)g.grad_twin[e]);
      pb.a += x.a; pb.b += x.b; pb.c += x.c; pb.d += x.d;
    }
  }
  // U_bar = (dP/dU)^T P_bar for P = (rho, m / rho, n / rho, (gamma - 1)(E - (m^2 + n^2) / (2 rho))):
  //   rho_bar = rho_b - (u u_b + v v_b) / rho + (gamma - 1) (u^2 + v^2) / 2 p_b
  //   m_bar = u_b / rho - (gamma - 1) u p_b,  n_bar = v_b / rho - (gamma - 1) v p_b
  //   E_bar = (gamma - 1) p_b
  const St4 q = ld4(P + 4 * (size_t)c);  // the primitive of U: rho, u, v, p
  const double inv = div_rn(1.0, q.a), vx = q.b, vy = q.c;
  const double gp = (gamma - 1.0) * pb.d;
  const double ub = pb.b * inv, vb = pb.c * inv;
  const St4 out{pb.a - (vx * ub + vy * vb) + 0.5 * gp * (vx * vx + vy * vy), ub - gp * vx, vb - gp * vy, gp};
  st4(ubar + 4 * (size_t)c, out);
}

// wall pressure force: per cell, its wall faces' p_c (n . dir) L, and the
// derivative of p_c with respect to U_c
__global__ void __launch_bounds__(kBlock) k_wall_force(DevGeom g, const double* __restrict__ U, double gamma,
                                                       double dx, double dy, double* __restrict__ cell_force,
                                                       double* __restrict__ dJdU) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= g.n_cells) return;
  double w = 0.0;
  for (int j = g.gb_ptr[c]; j < g.gb_ptr[c + 1]; ++j) {
    const int f = g.gb_flux[j];
    if (f < g.seg_begin[SEG_WALL] || f >= g.seg_begin[SEG_WALL + 1]) continue;
    const double2 n = g.ff_normal[f];
    w += (n.x * dx + n.y * dy) * g.ff_len[f];
  }
  const St4 u = ld4(U + 4 * (size_t)c);
  const double inv = div_rn(1.0, u.a), vx = u.b * inv, vy = u.c * inv;
  const double p = (gamma - 1.0) * (u.d - 0.5 * (u.b * u.b + u.c * u.c) * inv);
  cell_force[c] = p * w;
  if (dJdU) {
    const double gm = gamma - 1.0;
    st4(dJdU + 4 * (size_t)c, St4{w * gm * 0.5 * (vx * vx + vy * vy), -w * gm * vx, -w * gm * vy, w * gm});
  }
}

__global__ void k_sum_partial(int n, const double* __restrict__ x, double* __restrict__ partials) {
  __shared__ double sh[kBlock];
  double acc = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) acc += x[i];
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int w = kBlock / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) partials[blockIdx.x] = sh[0];
}

__global__ void k_sum_final(int blocks, const double* __restrict__ partials, double* out) {
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int b = 0; b < blocks; ++b) s += partials[b];
    out[0] = s;
  }
}

// The interior segment runs on s; the boundary segments (periodic, wall,
// inlet, outlet, far field: few faces, some of them in dual numbers and
// latency-bound) on w.side, forked from s after the slot adjoints are zeroed
// and joined back before the cell reverse.  Faces write disjoint slots.
template <int FLUX, bool FO, bool KH>
void face_segments(const DevGeom& g, const double* P, const double* recon, const double* lambda, double gamma,
                   double* slot_bar, double* far_bar, const VjpWork& w, cudaStream_t s) {
  const double inv_gm1 = 1.0 / (gamma - 1.0);  // correctly rounded, as div_rn on the device
  const int n_boundary = g.seg_begin[SEG_COUNT] - g.seg_begin[SEG_INTERIOR + 1];
  const bool fork = n_boundary > 0 && w.side;
  if (fork) {
    cudaEventRecord(w.fork, s);
    cudaStreamWaitEvent(w.side, w.fork, 0);
  }
#define MCFD_SEG(SEGV, STREAM)                                                                                  \
  {                                                                                                             \
    int n = g.seg_begin[SEGV + 1] - g.seg_begin[SEGV];                                                          \
    if (n > 0) {                                                                                                \
      count_launch();                                                                                           \
      if (FLUX != MCFD_FLUX_ROE && SEGV != SEG_FAR)                                                             \
        k_vjp_face_rev<(FLUX == MCFD_FLUX_ROE ? MCFD_FLUX_HLLC : FLUX), SEGV, FO, KH>                           \
            <<<seg_blocks(n), seg_threads(n), 0, STREAM>>>(g, P, recon, lambda, gamma, inv_gm1, slot_bar);      \
      else                                                                                                      \
        k_vjp_face<FLUX, SEGV, FO, KH><<<seg_blocks(n), seg_threads(n), 0, STREAM>>>(g, P, recon, lambda,       \
                                                                                     gamma, slot_bar, far_bar); \
    }                                                                                                           \
  }
  const cudaStream_t b = fork ? w.side : s;
  MCFD_SEG(SEG_FAR, b)
  MCFD_SEG(SEG_WALL, b)
  MCFD_SEG(SEG_PERIODIC, b)
  MCFD_SEG(SEG_VIN, b)
  MCFD_SEG(SEG_POUT, b)
  MCFD_SEG(SEG_INTERIOR, s)
#undef MCFD_SEG
  if (fork) {
    cudaEventRecord(w.join, w.side);
    cudaStreamWaitEvent(s, w.join, 0);
  }
}

}  // namespace

cudaError_t launch_vjp(const DevGeom& g, const mcfd_config& cfg, const double* U, const double* P_in,
                       const double* recon_in, const double* lambda, const VjpWork& w, double* ubar,
                       double* far_bar, cudaStream_t s) {
  const int C = g.n_cells;
  const bool fo = cfg.reconstruction == MCFD_RECON_FIRST_ORDER;
  if (!fo && !g.has_twins) return cudaErrorNotSupported;
  // face states as the forward step of the same mode computes them (the fast
  // kernel's limiter minimum equals the exact one; fma would not), unless
  // the caller recorded them during the forward step
  const double* P = P_in ? P_in : w.P;
  const double* recon = recon_in ? recon_in : w.recon;
  cudaError_t e = cudaSuccess;
  if (!P_in) e = exact::launch_primitive(g, cfg, U, w.P, s);
  if (e == cudaSuccess && !fo && !recon_in)
    e = cfg.mode == MCFD_MODE_FAST ? fast::launch_reconstruct(g, cfg, P, w.recon, s)
                                   : exact::launch_reconstruct(g, cfg, P, w.recon, s);
  if (e != cudaSuccess) return e;
  cudaMemsetAsync(w.slot_bar, 0, 4 * sizeof(double) * (size_t)g.n_slots, s);
  const bool kh = cfg.reconstruction != MCFD_RECON_MUSCL_PARABOLIC;
  switch (cfg.flux) {
    case MCFD_FLUX_RUSANOV:
      if (fo) face_segments<0, true, false>(g, P, recon, lambda, cfg.gamma, w.slot_bar, far_bar, w, s);
      else face_segments<0, false, false>(g, P, recon, lambda, cfg.gamma, w.slot_bar, far_bar, w, s);
      break;
    case MCFD_FLUX_HLLC:
      if (fo) face_segments<1, true, true>(g, P, recon, lambda, cfg.gamma, w.slot_bar, far_bar, w, s);
      else if (kh) face_segments<1, false, true>(g, P, recon, lambda, cfg.gamma, w.slot_bar, far_bar, w, s);
      else face_segments<1, false, false>(g, P, recon, lambda, cfg.gamma, w.slot_bar, far_bar, w, s);
      break;
    default:
      if (fo) face_segments<2, true, false>(g, P, recon, lambda, cfg.gamma, w.slot_bar, far_bar, w, s);
      else face_segments<2, false, false>(g, P, recon, lambda, cfg.gamma, w.slot_bar, far_bar, w, s);
      break;
  }
  count_launch(2);
  const double ax = cfg.acceleration_x, ay = cfg.acceleration_y;
  if (fo) {
    k_vjp_cell<0, true><<<blocks_for(C), kBlock, 0, s>>>(g, P, lambda, w.slot_bar, ax, ay, w.pbar, w.ent_bar, 0.0);
    k_vjp_collect<true><<<blocks_for(C), kBlock, 0, s>>>(g, P, w.pbar, w.ent_bar, cfg.gamma, ubar);
  } else {
    switch (cfg.limiter) {
      case 0: k_vjp_cell<0, false><<<blocks_for(C), kBlock, 0, s>>>(g, P, lambda, w.slot_bar, ax, ay, w.pbar, w.ent_bar, 0.0); break;
      case 1: k_vjp_cell<1, false><<<blocks_for(C), kBlock, 0, s>>>(g, P, lambda, w.slot_bar, ax, ay, w.pbar, w.ent_bar, 0.0); break;
      case 2: k_vjp_cell<2, false><<<blocks_for(C), kBlock, 0, s>>>(g, P, lambda, w.slot_bar, ax, ay, w.pbar, w.ent_bar, 0.0); break;
      case 3: k_vjp_cell<3, false><<<blocks_for(C), kBlock, 0, s>>>(g, P, lambda, w.slot_bar, ax, ay, w.pbar, w.ent_bar, 0.0); break;
      default:
        k_vjp_cell<MCFD_LIMITER_VENKATAKRISHNAN_K, false><<<blocks_for(C), kBlock, 0, s>>>(
            g, P, lambda, w.slot_bar, ax, ay, w.pbar, w.ent_bar, cfg.venkat_k);
        break;
    }
    k_vjp_collect<false><<<blocks_for(C), kBlock, 0, s>>>(g, P, w.pbar, w.ent_bar, cfg.gamma, ubar);
  }
  return cudaGetLastError();
}

cudaError_t launch_wall_force(const DevGeom& g, const mcfd_config& cfg, const double* U, double dx, double dy,
                              const VjpWork& w, double* J_dev, double* dJdU, cudaStream_t s) {
  const int C = g.n_cells;
  const int blocks = 152 * 4;
  count_launch(3);
  k_wall_force<<<blocks_for(C), kBlock, 0, s>>>(g, U, cfg.gamma, dx, dy, w.pbar, dJdU);
  k_sum_partial<<<blocks, kBlock, 0, s>>>(C, w.pbar, w.partials);
  k_sum_final<<<1, 32, 0, s>>>(blocks, w.partials, J_dev);
  return cudaGetLastError();
}

}  // namespace mcfd
