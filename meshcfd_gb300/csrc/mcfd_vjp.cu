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
// Jacobian to rounding.
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
  const double wl = -len / g.area[lc];
  double fb[4] = {wl * la.a, wl * la.b, wl * la.c, wl * la.d};
  if (SEG == SEG_INTERIOR || SEG == SEG_PERIODIC) {
    const int rc = g.ff_rcell[f];
    const St4 lb = ld4(lambda + 4 * (size_t)rc);
    const double wr = len / g.area[rc];
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
  if (LIMITER <= 1) return r < 1.0 ? 1.0 : 0.0;
  if (LIMITER == 2) {
    if (!(r > 0.0)) return 0.0;
    const double q = 2.0 * r / (1.0 + r);
    return q < 1.0 ? 2.0 / ((1.0 + r) * (1.0 + r)) : 0.0;
  }
  const double eps = 1e-12;
  const double N = r * r + 2.0 * r + eps, D = r * r + r + 2.0 + eps;
  if (N / D > 1.0) return 0.0;
  return ((2.0 * r + 2.0) * D - N * (2.0 * r + 1.0)) / (D * D);
}

template <int LIMITER, bool FO>
__global__ void __launch_bounds__(kBlock) k_vjp_cell(DevGeom g, const double* __restrict__ P,
                                                     const double* __restrict__ lambda,
                                                     const double* __restrict__ slot_bar, double ax, double ay,
                                                     double* __restrict__ pbar, double* __restrict__ ent_bar) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= g.n_cells) return;
  const St4 p = ld4(P + 4 * (size_t)c);
  const double pv[4] = {p.a, p.b, p.c, p.d};
  const int e0 = g.grad_ptr[c], e1 = g.grad_ptr[c + 1];
  const int s0 = g.lim_ptr[c], s1 = g.lim_ptr[c + 1];
  double pb[4] = {0.0, 0.0, 0.0, 0.0};
  for (int s = s0; s < s1; ++s) {
    const St4 q = ld4(slot_bar + 4 * (size_t)g.lim_slot[s]);
    pb[0] += q.a; pb[1] += q.b; pb[2] += q.c; pb[3] += q.d;
  }
  if (!FO) {
    // forward values in the residual's exact order
    double gx[4] = {0, 0, 0, 0}, gy[4] = {0, 0, 0, 0}, lo[4], hi[4];
    int lo_e[4] = {-1, -1, -1, -1}, hi_e[4] = {-1, -1, -1, -1};
    for (int v = 0; v < 4; ++v) lo[v] = hi[v] = pv[v];
    for (int e = e0; e < e1; ++e) {
      const St4 q = ld4(P + 4 * (size_t)g.grad_nb[e]);
      const double qv[4] = {q.a, q.b, q.c, q.d};
      for (int v = 0; v < 4; ++v) {
        const double d = qv[v] - pv[v];
        gx[v] = gx[v] + g.grad_cx[e] * d;
        gy[v] = gy[v] + g.grad_cy[e] * d;
        if (icmp::lt(qv[v], lo[v])) { lo[v] = qv[v]; lo_e[v] = e; }
        if (icmp::lt(hi[v], qv[v])) { hi[v] = qv[v]; hi_e[v] = e; }
      }
    }
    double phi[4] = {1.0, 1.0, 1.0, 1.0};
    int arg[4] = {-1, -1, -1, -1};
    for (int s = s0; s < s1; ++s) {
      const double2 dd = g.lim_d[s];
      for (int v = 0; v < 4; ++v) {
        const double inc = gx[v] * dd.x + gy[v] * dd.y;
        const double f = limiter_face_factor<LIMITER>(pv[v], inc, lo[v], hi[v], limiter_tolerance(pv[v]));
        if (icmp::lt_nonneg(f, phi[v])) { phi[v] = f; arg[v] = s; }
      }
    }
    // reverse of Q_s = P + phi (G . r_s)
    double phib[4] = {0, 0, 0, 0}, gxb[4] = {0, 0, 0, 0}, gyb[4] = {0, 0, 0, 0};
    for (int s = s0; s < s1; ++s) {
      const double2 dd = g.lim_d[s];
      const St4 q = ld4(slot_bar + 4 * (size_t)g.lim_slot[s]);
      const double qb[4] = {q.a, q.b, q.c, q.d};
      for (int v = 0; v < 4; ++v) {
        phib[v] += qb[v] * (gx[v] * dd.x + gy[v] * dd.y);
        gxb[v] += qb[v] * phi[v] * dd.x;
        gyb[v] += qb[v] * phi[v] * dd.y;
      }
    }
    // reverse of the limiter through its minimising entry
    double extb[4] = {0, 0, 0, 0};
    int ext_e[4] = {-1, -1, -1, -1};
    for (int v = 0; v < 4; ++v) {
      if (arg[v] < 0) continue;
      const double2 dd = g.lim_d[arg[v]];
      const double inc = gx[v] * dd.x + gy[v] * dd.y;
      const double tol = limiter_tolerance(pv[v]);
      const bool pos = icmp::gt_pos(inc, tol), neg = icmp::neg_gt_pos(inc, tol);
      if (!(pos || neg)) continue;
      const double num = pos ? hi[v] - pv[v] : lo[v] - pv[v];
      const double r = num / inc;
      if (!(r > 0.0)) continue;
      const double rb = limiter_slope<LIMITER>(r) * phib[v];
      const double numb = rb / inc;
      const double incb = -rb * r / inc;
      pb[v] -= numb;
      const int ee = pos ? hi_e[v] : lo_e[v];
      if (ee < 0) pb[v] += numb;  // the extreme is the cell itself
      else { extb[v] = numb; ext_e[v] = ee; }
      gxb[v] += incb * dd.x;
      gyb[v] += incb * dd.y;
    }
    // reverse of G = sum_e coef_e (P_nb - P_c): neighbour share per entry
    for (int e = e0; e < e1; ++e) {
      double out[4];
      for (int v = 0; v < 4; ++v) {
        const double w = g.grad_cx[e] * gxb[v] + g.grad_cy[e] * gyb[v];
        pb[v] -= w;
        out[v] = w + (ext_e[v] == e ? extb[v] : 0.0);
      }
      st4(ent_bar + 4 * (size_t)e, St4{out[0], out[1], out[2], out[3]});
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
__global__ void __launch_bounds__(kBlock) k_vjp_collect(DevGeom g, const double* __restrict__ U,
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
  // U_bar = (dP/dU)^T P_bar
  using D4 = ad::Dual<4>;
  const St4 u = ld4(U + 4 * (size_t)c);
  const ad::S4<D4> q = ad::prim(ad::S4<D4>{seed<4>(u.a, 0), seed<4>(u.b, 1), seed<4>(u.c, 2), seed<4>(u.d, 3)}, gamma);
  double out[4];
  for (int k = 0; k < 4; ++k) out[k] = pb.a * q.a.d[k] + pb.b * q.b.d[k] + pb.c * q.c.d[k] + pb.d * q.d.d[k];
  st4(ubar + 4 * (size_t)c, St4{out[0], out[1], out[2], out[3]});
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
  const double inv = 1.0 / u.a, vx = u.b * inv, vy = u.c * inv;
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

template <int FLUX, bool FO, bool KH>
void face_segments(const DevGeom& g, const double* P, const double* recon, const double* lambda, double gamma,
                   double* slot_bar, double* far_bar, cudaStream_t s) {
#define MCFD_SEG(SEGV)                                                                                          \
  {                                                                                                             \
    int n = g.seg_begin[SEGV + 1] - g.seg_begin[SEGV];                                                          \
    if (n > 0) count_launch(), k_vjp_face<FLUX, SEGV, FO, KH><<<blocks_for(n), kBlock, 0, s>>>(                 \
                   g, P, recon, lambda, gamma, slot_bar, far_bar);                                              \
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

cudaError_t launch_vjp(const DevGeom& g, const mcfd_config& cfg, const double* U, const double* lambda,
                       const VjpWork& w, double* ubar, double* far_bar, cudaStream_t s) {
  const int C = g.n_cells;
  const bool fo = cfg.reconstruction == MCFD_RECON_FIRST_ORDER;
  if (!fo && !g.has_twins) return cudaErrorNotSupported;
  cudaError_t e = exact::launch_primitive(g, cfg, U, w.P, s);
  if (e == cudaSuccess && !fo) e = exact::launch_reconstruct(g, cfg, w.P, w.recon, s);
  if (e != cudaSuccess) return e;
  cudaMemsetAsync(w.slot_bar, 0, 4 * sizeof(double) * (size_t)g.n_slots, s);
  const bool kh = cfg.reconstruction != MCFD_RECON_MUSCL_PARABOLIC;
  switch (cfg.flux) {
    case MCFD_FLUX_RUSANOV:
      if (fo) face_segments<0, true, false>(g, w.P, w.recon, lambda, cfg.gamma, w.slot_bar, far_bar, s);
      else face_segments<0, false, false>(g, w.P, w.recon, lambda, cfg.gamma, w.slot_bar, far_bar, s);
      break;
    case MCFD_FLUX_HLLC:
      if (fo) face_segments<1, true, true>(g, w.P, w.recon, lambda, cfg.gamma, w.slot_bar, far_bar, s);
      else if (kh) face_segments<1, false, true>(g, w.P, w.recon, lambda, cfg.gamma, w.slot_bar, far_bar, s);
      else face_segments<1, false, false>(g, w.P, w.recon, lambda, cfg.gamma, w.slot_bar, far_bar, s);
      break;
    default:
      if (fo) face_segments<2, true, false>(g, w.P, w.recon, lambda, cfg.gamma, w.slot_bar, far_bar, s);
      else face_segments<2, false, false>(g, w.P, w.recon, lambda, cfg.gamma, w.slot_bar, far_bar, s);
      break;
  }
  count_launch(2);
  const double ax = cfg.acceleration_x, ay = cfg.acceleration_y;
  if (fo) {
    k_vjp_cell<0, true><<<blocks_for(C), kBlock, 0, s>>>(g, w.P, lambda, w.slot_bar, ax, ay, w.pbar, w.ent_bar);
    k_vjp_collect<true><<<blocks_for(C), kBlock, 0, s>>>(g, U, w.pbar, w.ent_bar, cfg.gamma, ubar);
  } else {
    switch (cfg.limiter) {
      case 0: k_vjp_cell<0, false><<<blocks_for(C), kBlock, 0, s>>>(g, w.P, lambda, w.slot_bar, ax, ay, w.pbar, w.ent_bar); break;
      case 1: k_vjp_cell<1, false><<<blocks_for(C), kBlock, 0, s>>>(g, w.P, lambda, w.slot_bar, ax, ay, w.pbar, w.ent_bar); break;
      case 2: k_vjp_cell<2, false><<<blocks_for(C), kBlock, 0, s>>>(g, w.P, lambda, w.slot_bar, ax, ay, w.pbar, w.ent_bar); break;
      default: k_vjp_cell<3, false><<<blocks_for(C), kBlock, 0, s>>>(g, w.P, lambda, w.slot_bar, ax, ay, w.pbar, w.ent_bar); break;
    }
    k_vjp_collect<false><<<blocks_for(C), kBlock, 0, s>>>(g, U, w.pbar, w.ent_bar, cfg.gamma, ubar);
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
