// Exact Jacobian-vector product of the residual (forward mode).
//
// dR = (dR/dU) dU for the residual of mcfd_residual (first order or MUSCL
// linear with the four limiters, all fluxes and boundary kinds), evaluated
// with Dual<1> numbers in the same kernel structure as the residual:
// tangent of the primitive recovery (per cell), of the reconstruction (per
// cell: LSQ gradient, limiter through its minimising entry and the extreme
// neighbours, face states), of the face fluxes (per flux face, ghost states
// included) and of the divergence gather (per cell, reference order).  It is
// the exact counterpart of the reference's finite-difference product
// (solver.py:1532-1567).  Values are recomputed in the exact operation order,
// so the switch decisions (limiter band, extreme neighbour, HLLC region,
// far-field regime) are those of the residual itself.
#include "mcfd_ad.cuh"
#include "mcfd_internal.h"
#include "mcfd_jvp.h"

namespace mcfd {
namespace {

using D1 = ad::Dual<1>;
constexpr int kBlock = 256;
inline int blocks_for(int n) { return (n + kBlock - 1) / kBlock; }

__device__ __forceinline__ D1 dual(double v, double d) {
  D1 x(v);
  x.d[0] = d;
  return x;
}

__device__ __forceinline__ ad::S4<D1> ld4d(const double* p, const double* dp, size_t i) {
  const St4 a = ld4(p + 4 * i), b = ld4(dp + 4 * i);
  return ad::S4<D1>{dual(a.a, b.a), dual(a.b, b.b), dual(a.c, b.c), dual(a.d, b.d)};
}

__global__ void k_prim_tangent(int C, const double* __restrict__ U, const double* __restrict__ dU, double gamma,
                               double* __restrict__ P, double* __restrict__ dP) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= C) return;
  // values in the reference's exact order; tangents from the dual form
  bool ok;
  const St4 p = cons_to_prim(ld4(U + 4 * (size_t)c), gamma, &ok);
  const ad::S4<D1> q = ad::prim(ld4d(U, dU, c), gamma);
  st4(P + 4 * (size_t)c, p);
  st4(dP + 4 * (size_t)c, St4{q.a.d[0], q.b.d[0], q.c.d[0], q.d.d[0]});
}

// derivative of the limiter function g at ratio r (0 where it is capped)
template <int LIMITER>
__device__ __forceinline__ double limiter_slope(double r) {
  if (LIMITER <= 1) return r < 1.0 ? 1.0 : 0.0;
  if (LIMITER == 2) {
    if (!(r > 0.0)) return 0.0;
    const double q = div_rn(2.0 * r, 1.0 + r);
    return q < 1.0 ? div_rn(2.0, (1.0 + r) * (1.0 + r)) : 0.0;
  }
  const double eps = 1e-12;
  const double N = r * r + 2.0 * r + eps, D = r * r + r + 2.0 + eps;
  if (div_rn(N, D) > 1.0) return 0.0;
  return div_rn((2.0 * r + 2.0) * D - N * (2.0 * r + 1.0), D * D);
}

template <int LIMITER>
__global__ void __launch_bounds__(kBlock) k_reconstruct_tangent(DevGeom g, const double* __restrict__ P,
                                                                const double* __restrict__ dP,
                                                                double* __restrict__ dQ, double venkat_k) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= g.n_cells) return;
  const St4 p = ld4(P + 4 * (size_t)c), tp = ld4(dP + 4 * (size_t)c);
  const double pv[4] = {p.a, p.b, p.c, p.d}, dpv[4] = {tp.a, tp.b, tp.c, tp.d};
  double gx[4] = {0, 0, 0, 0}, gy[4] = {0, 0, 0, 0}, dgx[4] = {0, 0, 0, 0}, dgy[4] = {0, 0, 0, 0};
  double lo[4], hi[4], dlo[4], dhi[4];
  for (int v = 0; v < 4; ++v) {
    lo[v] = hi[v] = pv[v];
    dlo[v] = dhi[v] = dpv[v];
  }
  for (int e = g.grad_ptr[c]; e < g.grad_ptr[c + 1]; ++e) {
    const int nb = g.grad_nb[e];
    const double cx = g.grad_cx[e], cy = g.grad_cy[e];
    const St4 q = ld4(P + 4 * (size_t)nb), tq = ld4(dP + 4 * (size_t)nb);
    const double qv[4] = {q.a, q.b, q.c, q.d}, dqv[4] = {tq.a, tq.b, tq.c, tq.d};
    for (int v = 0; v < 4; ++v) {
      const double d = qv[v] - pv[v];
      gx[v] = gx[v] + cx * d;
      gy[v] = gy[v] + cy * d;
      const double dd = dqv[v] - dpv[v];
      dgx[v] += cx * dd;
      dgy[v] += cy * dd;
      if (icmp::lt(qv[v], lo[v])) { lo[v] = qv[v]; dlo[v] = dqv[v]; }
      if (icmp::lt(hi[v], qv[v])) { hi[v] = qv[v]; dhi[v] = dqv[v]; }
    }
  }
  double phi[4] = {1.0, 1.0, 1.0, 1.0}, dphi[4] = {0.0, 0.0, 0.0, 0.0};
  const int s0 = g.lim_ptr[c], s1 = g.lim_ptr[c + 1];
  if constexpr (LIMITER == MCFD_LIMITER_VENKATAKRISHNAN_K) {
    // the smooth form: the minimising face's factor and its total derivative
    // through d1 (the extreme neighbour or the cell) and d2 (the gradient)
    const double e2 = venkat_k_e2(venkat_k, g.area[c]);
    for (int s = s0; s < s1; ++s) {
      const double2 dd = g.lim_d[s];
      for (int v = 0; v < 4; ++v) {
        const double inc = gx[v] * dd.x + gy[v] * dd.y;
        const double dinc = dgx[v] * dd.x + dgy[v] * dd.y;
        const VenkatK f = venkat_k_face(pv[v], inc, lo[v], hi[v], e2);
        if (s == s0 || icmp::lt(f.f, phi[v])) {
          phi[v] = f.f;
          double a, b;
          venkat_k_slopes(f, inc, &a, &b);
          const double dd1 = (icmp::gt0(inc) ? dhi[v] : dlo[v]) - dpv[v];
          dphi[v] = a * dd1 + b * dinc;
        }
      }
    }
  } else
  for (int s = s0; s < s1; ++s) {
    const double2 dd = g.lim_d[s];
    for (int v = 0; v < 4; ++v) {
      const double inc = gx[v] * dd.x + gy[v] * dd.y;
      const double dinc = dgx[v] * dd.x + dgy[v] * dd.y;
      const double tol = limiter_tolerance(pv[v]);
      const double f = limiter_face_factor<LIMITER>(pv[v], inc, lo[v], hi[v], tol);
      if (icmp::lt_nonneg(f, phi[v])) {
        phi[v] = f;
        double df = 0.0;
        const bool pos = icmp::gt_pos(inc, tol), neg = icmp::neg_gt_pos(inc, tol);
        if (pos || neg) {
          const double num = pos ? hi[v] - pv[v] : lo[v] - pv[v];
          const double dnum = pos ? dhi[v] - dpv[v] : dlo[v] - dpv[v];
          const double r = div_rn(num, inc);
          if (r > 0.0) df = div_rn(limiter_slope<LIMITER>(r) * (dnum - r * dinc), inc);
        }
        dphi[v] = df;
      }
    }
  }
  for (int s = s0; s < s1; ++s) {
    const double2 dd = g.lim_d[s];
    double out[4];
    for (int v = 0; v < 4; ++v) {
      const double inc = gx[v] * dd.x + gy[v] * dd.y;
      const double dinc = dgx[v] * dd.x + dgy[v] * dd.y;
      out[v] = dpv[v] + dphi[v] * inc + phi[v] * dinc;
    }
    st4(dQ + 4 * (size_t)g.lim_slot[s], St4{out[0], out[1], out[2], out[3]});
  }
}

template <int FLUX, int SEG, bool FO, bool KH>
__global__ void __launch_bounds__(kBlock) k_flux_tangent(DevGeom g, const double* __restrict__ P,
                                                         const double* __restrict__ dP,
                                                         const double* __restrict__ recon,
                                                         const double* __restrict__ drecon,
                                                         double* __restrict__ dflux, double gamma) {
  const int begin = g.seg_begin[SEG];
  const int f = begin + blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= g.seg_begin[SEG + 1]) return;
  const double2 n = g.ff_normal[f];
  using S = ad::S4<D1>;
  const S L = FO ? ld4d(P, dP, g.ff_lcell[f]) : ld4d(recon, drecon, g.ff_lslot[f]);
  S R;
  if (SEG == SEG_INTERIOR || SEG == SEG_PERIODIC) {
    R = FO ? ld4d(P, dP, g.ff_rcell[f]) : ld4d(recon, drecon, g.ff_rslot[f]);
  } else if (SEG == SEG_WALL) {
    const double2 wv = g.ff_wall_velocity[f - begin];
    D1 un = (L.b - D1(wv.x)) * D1(n.x) + (L.c - D1(wv.y)) * D1(n.y);
    R = S{L.a, L.b - D1(2.0) * un * D1(n.x), L.c - D1(2.0) * un * D1(n.y), L.d};
  } else if (SEG == SEG_VIN) {
    const St4 x = ld4(g.ff_vin_state + 4 * (size_t)(f - begin));
    R = S{D1(x.a), D1(x.b), D1(x.c), D1(x.d)};
  } else if (SEG == SEG_POUT) {
    R = S{L.a, L.b, L.c, D1(g.ff_pout_pressure[f - begin])};
  } else {
    const St4 x = ld4(g.ff_far_state + 4 * (size_t)(f - begin));
    R = ad::far_field(L, S{D1(x.a), D1(x.b), D1(x.c), D1(x.d)}, n.x, n.y, gamma);
  }
  D1 out[4];
  ad::numerical_flux<D1>(FLUX, (SEG == SEG_INTERIOR) && KH, L, R, n.x, n.y, gamma, out);
  st4(dflux + 4 * (size_t)f, St4{out[0].d[0], out[1].d[0], out[2].d[0], out[3].d[0]});
}

__global__ void __launch_bounds__(kBlock) k_gather_tangent(DevGeom g, const double* __restrict__ P,
                                                           const double* __restrict__ dP,
                                                           const double* __restrict__ dflux, double ax,
                                                           double ay, double* __restrict__ dR) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= g.n_cells) return;
  double r[4] = {0.0, 0.0, 0.0, 0.0};
  for (int j = g.gi_ptr[c]; j < g.gi_ptr[c + 1]; ++j) {
    const double a = g.gi_coef[j];
    const St4 F = ld4(dflux + 4 * (size_t)g.gi_flux[j]);
    r[0] += a * F.a; r[1] += a * F.b; r[2] += a * F.c; r[3] += a * F.d;
  }
  const int jb0 = g.gb_ptr[c], jb1 = g.gb_ptr[c + 1];
  if (jb0 < jb1) {
    const double ia = div_rn(1.0, g.area[c]);
    for (int j = jb0; j < jb1; ++j) {
      const double w = g.gb_len[j] * ia;
      const St4 F = ld4(dflux + 4 * (size_t)g.gb_flux[j]);
      r[0] += w * F.a; r[1] += w * F.b; r[2] += w * F.c; r[3] += w * F.d;
    }
  }
  if (ax != 0.0 || ay != 0.0) {
    const St4 p = ld4(P + 4 * (size_t)c), t = ld4(dP + 4 * (size_t)c);
    r[1] += t.a * ax;
    r[2] += t.a * ay;
    r[3] += t.a * (ax * p.b + ay * p.c) + p.a * (ax * t.b + ay * t.c);
  }
  st4(dR + 4 * (size_t)c, St4{r[0], r[1], r[2], r[3]});
}

template <int FLUX, bool FO, bool KH>
void flux_tangent_segments(const DevGeom& g, const double* P, const double* dP, const double* recon,
                           const double* drecon, double* dflux, double gamma, cudaStream_t s) {
#define MCFD_SEG(SEGV)                                                                                     \
  {                                                                                                        \
    int n = g.seg_begin[SEGV + 1] - g.seg_begin[SEGV];                                                     \
    if (n > 0) count_launch(), k_flux_tangent<FLUX, SEGV, FO, KH><<<seg_blocks(n), seg_threads(n), 0, s>>>( \
                   g, P, dP, recon, drecon, dflux, gamma);                                                 \
  }
  MCFD_SEG(SEG_INTERIOR)
  MCFD_SEG(SEG_PERIODIC)
  MCFD_SEG(SEG_WALL)
  MCFD_SEG(SEG_VIN)
  MCFD_SEG(SEG_POUT)
  MCFD_SEG(SEG_FAR)
#undef MCFD_SEG
}

}  // namespace

cudaError_t launch_jvp(const DevGeom& g, const mcfd_config& cfg, const double* U, const double* dU,
                       const JvpWork& w, double* dR, cudaStream_t s) {
  const int C = g.n_cells;
  count_launch();
  k_prim_tangent<<<blocks_for(C), kBlock, 0, s>>>(C, U, dU, cfg.gamma, w.P, w.dP);
  const bool fo = cfg.reconstruction == MCFD_RECON_FIRST_ORDER;
  if (!fo) {
    // face-state values from the exact residual kernels, tangents here
    cudaError_t e = exact::launch_reconstruct(g, cfg, w.P, w.recon, s);
    if (e != cudaSuccess) return e;
    count_launch();
    switch (cfg.limiter) {
      case 0: k_reconstruct_tangent<0><<<blocks_for(C), kBlock, 0, s>>>(g, w.P, w.dP, w.drecon, 0.0); break;
      case 1: k_reconstruct_tangent<1><<<blocks_for(C), kBlock, 0, s>>>(g, w.P, w.dP, w.drecon, 0.0); break;
      case 2: k_reconstruct_tangent<2><<<blocks_for(C), kBlock, 0, s>>>(g, w.P, w.dP, w.drecon, 0.0); break;
      case 3: k_reconstruct_tangent<3><<<blocks_for(C), kBlock, 0, s>>>(g, w.P, w.dP, w.drecon, 0.0); break;
      default:
        k_reconstruct_tangent<MCFD_LIMITER_VENKATAKRISHNAN_K><<<blocks_for(C), kBlock, 0, s>>>(g, w.P, w.dP, w.drecon,
                                                                                              cfg.venkat_k);
        break;
    }
  }
  const bool kh = cfg.reconstruction != MCFD_RECON_MUSCL_PARABOLIC;
  switch (cfg.flux) {
    case MCFD_FLUX_RUSANOV:
      if (fo) flux_tangent_segments<0, true, false>(g, w.P, w.dP, w.recon, w.drecon, w.dflux, cfg.gamma, s);
      else flux_tangent_segments<0, false, false>(g, w.P, w.dP, w.recon, w.drecon, w.dflux, cfg.gamma, s);
      break;
    case MCFD_FLUX_HLLC:
      if (fo) flux_tangent_segments<1, true, true>(g, w.P, w.dP, w.recon, w.drecon, w.dflux, cfg.gamma, s);
      else if (kh) flux_tangent_segments<1, false, true>(g, w.P, w.dP, w.recon, w.drecon, w.dflux, cfg.gamma, s);
      else flux_tangent_segments<1, false, false>(g, w.P, w.dP, w.recon, w.drecon, w.dflux, cfg.gamma, s);
      break;
    default:
      if (fo) flux_tangent_segments<2, true, false>(g, w.P, w.dP, w.recon, w.drecon, w.dflux, cfg.gamma, s);
      else flux_tangent_segments<2, false, false>(g, w.P, w.dP, w.recon, w.drecon, w.dflux, cfg.gamma, s);
      break;
  }
  count_launch();
  k_gather_tangent<<<blocks_for(C), kBlock, 0, s>>>(g, w.P, w.dP, w.dflux, cfg.acceleration_x, cfg.acceleration_y, dR);
  return cudaGetLastError();
}

}  // namespace mcfd

namespace mcfd {
namespace {

// the scales are read from the prepared operator's device copy, so a
// captured GMRES step uses the current ones
__global__ void k_scale_dir(int n4, const double* __restrict__ v, const double* __restrict__ scale,
                            double* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n4) out[i] = scale[i & 3] * v[i];
}

__global__ void k_exact_combine(int n4, const double* __restrict__ v, const double* __restrict__ dR,
                                const double* __restrict__ scale, const double* __restrict__ dt, int dt_per_cell,
                                double* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n4) return;
  const double d = dt_per_cell ? dt[i >> 2] : dt[0];
  out[i] = v[i] - div_rn(d * dR[i], scale[i & 3]);
}

}  // namespace

cudaError_t exact_operator(const DevGeom& g, const mcfd_config& cfg1, const ImplicitState& st, const JvpWork& w,
                           const double* v, double* out, cudaStream_t s) {
  const int n4 = 4 * g.n_cells;
  count_launch();
  k_scale_dir<<<blocks_for(n4), kBlock, 0, s>>>(n4, v, st.scale_dev, w.sv);
  cudaError_t e = launch_jvp(g, cfg1, st.state, w.sv, w, w.dR, s);
  if (e != cudaSuccess) return e;
  count_launch();
  k_exact_combine<<<blocks_for(n4), kBlock, 0, s>>>(n4, v, w.dR, st.scale_dev, st.dt, st.dt_per_cell, out);
  return cudaGetLastError();
}

}  // namespace mcfd
