// Kernels of the FP64 residual / explicit-step path (sm_103a).
//
// This file is compiled three times (mcfd_kernels_{exact,fast,fma}.cu):
// * exact (MCFD_FAST 0, -fmad=false): every multiply and add rounds
//   separately and every expression keeps the reference's order, so each
//   kernel reproduces the reference bit for bit where the reference itself is
//   IEEE-deterministic (everything except pow() in the far-field state);
// * fast (MCFD_FAST 1, -fmad=false): exact arithmetic, but the limiter takes
//   the cell minimum through the smallest ratio (limiter_factor_min_ratio):
//   3 divisions per variable instead of 2 per limiter entry; bit-exact for
//   Barth-Jespersen / Minmod, last-place ties possible for Van Leer /
//   Venkatakrishnan;
// * fma (MCFD_FAST 2, FMA contraction): additionally shared reciprocals in
//   the fluxes and primitive recovery and a one-division rational limiter.
//   Rounding differs from the reference in the last places of every flux;
//   on fine meshes the residual's cancellation (sum of O(1) fluxes times
//   L/A ~ 1/h) amplifies that to ~1e-11 relative, so this variant is a
//   throughput option outside the 1e-12 parity bar.
// Compares, min/max and finiteness tests run on the integer pipe in both.
//
// Per explicit stage: reconstruct (per cell, MUSCL only) -> flux (per flux
// face, one launch per face segment) -> gather (per cell: divergence in the
// reference's accumulation order, boundary adds, body force, finiteness
// check, stage combination, primitive recovery of the new stage state).
// There are no atomics on the data path: the face->cell scatter of the
// reference is a deterministic CSR gather.
#ifndef MCFD_FAST
#error "define MCFD_FAST (0 or 1) and MCFD_VARIANT before including this file"
#endif

// Flux products on the integer pipe (mcfd_device.cuh): the HLLC star state in
// the exact-arithmetic variants (+1.8 % on the 1024^2 vortex step; adding a
// second site group lost), none in the fma variant (its products contract).
#if !defined(MCFD_FLUX_INT_MUL) && MCFD_FAST != 2
#define MCFD_FLUX_INT_MUL 4
#endif

#include <cooperative_groups.h>

#include <type_traits>

#include "mcfd_device.cuh"
#include "mcfd_internal.h"

namespace mcfd {
namespace MCFD_VARIANT {

namespace cg = cooperative_groups;

static constexpr int kBlock = 256;
static constexpr bool kFast = MCFD_FAST == 2;      // fast arithmetic (fluxes, primitive)
static constexpr bool kMinRatio = MCFD_FAST == 1;  // min-ratio limiter, exact arithmetic

// Products that the exact-arithmetic variants evaluate on the integer pipe
// (mul_rn, the same IEEE result) to take load off the FP64 pipe, which bounds
// these kernels.  MCFD_INT_MUL is a mask of the call sites that do so; the
// fma variant always keeps the native product so that it can contract into
// DFMA.
enum IntMulSite {
  MUL_GRADIENT = 1,   // reconstruction: gradient sums  c (q - p)
  MUL_INCREMENT = 2,  // reconstruction: face increments  grad . r
  MUL_OUTPUT = 4,     // reconstruction: limited face value  phi inc
  MUL_GATHER = 8,     // gather: divergence  a F and the stage combination
};
// Defaults measured on the 1024^2 vortex RK3 step (GB300): all sites for the
// exact variant (+7 %), gradient + output + gather for the fast variant
// (+8 %; its variable-at-a-time increments lose from the longer chains).
#ifndef MCFD_INT_MUL
#if MCFD_FAST == 0
#define MCFD_INT_MUL 15
#elif MCFD_FAST == 1
#define MCFD_INT_MUL 13
#else
#define MCFD_INT_MUL 0
#endif
#endif

template <int SITE>
__device__ __forceinline__ double kmul(double a, double b) {
  if constexpr (kFast || (MCFD_INT_MUL & SITE) == 0) return a * b;
  else return mul_rn(a, b);
}

__device__ __forceinline__ St4 to_prim(const St4& U, double gamma, bool* ok) {
  if constexpr (kFast) return cons_to_prim_fast(U, gamma, ok);
  else return cons_to_prim(U, gamma, ok);
}

__device__ __forceinline__ void flag_cell(DevStatus* st, int bits, int cell) {
  atomicOr(&st->code, bits);
  atomicMin(&st->first_cell, cell);
}
__device__ __forceinline__ void flag_face(DevStatus* st, int bits, int face) {
  atomicOr(&st->code, bits);
  atomicMin(&st->first_face, face);
}

// ---------------------------------------------------------------- primitive

__global__ void __launch_bounds__(kBlock) k_primitive(int n, const double* __restrict__ U,
                                                      double* __restrict__ P, double gamma,
                                                      DevStatus* st) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  bool ok;
  St4 p = to_prim(ld4(U + 4 * (size_t)c), gamma, &ok);
  if (!ok) flag_cell(st, MCFD_S_NONPHYSICAL_STATE, c);
  st4(P + 4 * (size_t)c, p);
}

// ----------------------------------------------------------- reconstruction
//
// _kernels.linear_gradients_and_factors (_kernels.py:240-273) and
// limited_gradient_factors (_kernels.py:10-67), as a per-cell gather: the
// gradient sums run over this cell's entries in the reference's global entry
// order (so the floating-point sums are identical), the local min/max and the
// limiter minimum are order-free.  The result is written per limiter entry
// ("slot") as the reconstructed face state P + phi * (grad . r), which is
// exactly the left/right state of the fused flux kernel (_kernels.py:90-98)
// and of _reconstruct (solver.py:2418-2434).
//
// The per-cell kernels visit cells through g.cell_order, which groups cells
// with the same stencil and face counts so that a warp's loops share one trip
// count (on mixed meshes a warp of triangles and quads otherwise runs every
// triangle lane idle through the fourth entry, which still costs FP64 issue
// slots).  Each cell's arithmetic and outputs do not depend on the order.

// Least-squares gradient sums of one cell over its entries in the
// reference's order (np.zeros, then += c (q - p) per entry) and the
// neighbour extremes.  The first entry's sum is 0.0 + t, which is t itself
// except that -0.0 becomes +0.0: plus_zero on the integer pipe gives those
// bits without an FP64 addition.
__device__ __forceinline__ void gradient_sums(const DevGeom& g, const double* __restrict__ P, int c,
                                              const double pv[4], double gx[4], double gy[4], double lo[4],
                                              double hi[4]) {
  auto visit = [&](int e, auto first) {
    const int nb = g.grad_nb[e];
    const double cx = g.grad_cx[e], cy = g.grad_cy[e];
    const St4 q = ld4(P + 4 * (size_t)nb);
    const double qv[4] = {q.a, q.b, q.c, q.d};
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const double d = qv[v] - pv[v];
      const double tx = kmul<MUL_GRADIENT>(cx, d), ty = kmul<MUL_GRADIENT>(cy, d);
      if constexpr (decltype(first)::value) {
        gx[v] = plus_zero(tx);
        gy[v] = plus_zero(ty);
      } else {
        gx[v] = gx[v] + tx;
        gy[v] = gy[v] + ty;
      }
      // density and pressure are positive (checked at primitive recovery), so
      // their order is the order of the raw bits; velocities need the key.
      const bool below = (v == 0 || v == 3) ? icmp::lt_pos(qv[v], lo[v]) : icmp::lt(qv[v], lo[v]);
      const bool above = (v == 0 || v == 3) ? icmp::gt_pos(qv[v], hi[v]) : icmp::lt(hi[v], qv[v]);
      if (below) lo[v] = qv[v];
      if (above) hi[v] = qv[v];
    }
  };
  int e = g.grad_ptr[c];
  const int e1 = g.grad_ptr[c + 1];
  if (e < e1) {
    visit(e++, std::true_type{});
  } else {
#pragma unroll
    for (int v = 0; v < 4; ++v) gx[v] = gy[v] = 0.0;
  }
  for (; e < e1; ++e) visit(e, std::false_type{});
}

// Resident 256-thread blocks per SM the generic kernel is compiled for.
#ifndef MCFD_RECON_GENERIC_MIN_BLOCKS
#define MCFD_RECON_GENERIC_MIN_BLOCKS 2
#endif

template <int LIMITER>
__global__ void __launch_bounds__(kBlock, MCFD_RECON_GENERIC_MIN_BLOCKS) k_reconstruct(DevGeom g, const double* __restrict__ P,
                                                                                       double* __restrict__ recon,
                                                                                       double venkat_k) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= g.n_cells) return;
  const int c = g.cell_order[i];
  const St4 p = ld4(P + 4 * (size_t)c);
  double gx[4], gy[4];
  double lo[4] = {p.a, p.b, p.c, p.d}, hi[4] = {p.a, p.b, p.c, p.d};
  const double pv[4] = {p.a, p.b, p.c, p.d};
  gradient_sums(g, P, c, pv, gx, gy, lo, hi);
  double phi[4] = {1.0, 1.0, 1.0, 1.0};
  const int s0 = g.lim_ptr[c], s1 = g.lim_ptr[c + 1];
  if constexpr (LIMITER == MCFD_LIMITER_VENKATAKRISHNAN_K) {
    // minimum over the faces of the smooth face function (no cap at 1)
    const double e2 = venkat_k_e2(venkat_k, g.area[c]);
    for (int s = s0; s < s1; ++s) {
      const double2 d = g.lim_d[s];
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        const double inc = kmul<MUL_INCREMENT>(gx[v], d.x) + kmul<MUL_INCREMENT>(gy[v], d.y);
        const double f = venkat_k_face(pv[v], inc, lo[v], hi[v], e2).f;
        if (s == s0 || icmp::lt(f, phi[v])) phi[v] = f;
      }
    }
  } else {
    double tol[4];
#pragma unroll
    for (int v = 0; v < 4; ++v) tol[v] = limiter_tolerance(pv[v]);
    for (int s = s0; s < s1; ++s) {
      const double2 d = g.lim_d[s];
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        double inc = kmul<MUL_INCREMENT>(gx[v], d.x) + kmul<MUL_INCREMENT>(gy[v], d.y);
        double f = limiter_face_factor<LIMITER>(pv[v], inc, lo[v], hi[v], tol[v]);
        if (icmp::lt_nonneg(f, phi[v])) phi[v] = f;
      }
    }
  }
  for (int s = s0; s < s1; ++s) {
    const double2 d = g.lim_d[s];
    double out[4];
#pragma unroll
    for (int v = 0; v < 4; ++v) out[v] = pv[v] + phi[v] * (kmul<MUL_INCREMENT>(gx[v], d.x) + kmul<MUL_INCREMENT>(gy[v], d.y));
    st4(recon + 4 * (size_t)g.lim_slot[s], St4{out[0], out[1], out[2], out[3]});
  }
}

// Reconstruction through the cell's smallest ratio (fast and fma variants):
// gradients as in the exact kernel, one pass over the limiter entries that
// keeps the largest positive and most negative increments, the factor from
// limiter_factor_min_ratio (fast) or limiter_factor_fast (fma), and the
// increments kept in registers for the face-state write.  NS > 0 compiles the
// cell for exactly NS limiter entries (triangles 3, quadrilaterals 4; the
// cell order makes the count warp-uniform); NS = 0 handles any count, caching
// the first four increments.
template <int LIMITER, int NS>
__device__ __forceinline__ void reconstruct_cell_fast(const DevGeom& g, const double* __restrict__ P,
                                                      double* __restrict__ recon, int c, const St4& p,
                                                      int s0, int s1) {
  const double pv[4] = {p.a, p.b, p.c, p.d};
  double gx[4], gy[4];
  double lo[4] = {p.a, p.b, p.c, p.d}, hi[4] = {p.a, p.b, p.c, p.d};
  gradient_sums(g, P, c, pv, gx, gy, lo, hi);
  double tol[4], pos[4], neg[4];
  bool has_pos[4], has_neg[4], flat[4];
#pragma unroll
  for (int v = 0; v < 4; ++v) {
    tol[v] = limiter_tolerance(pv[v]);
    pos[v] = 0.0;
    neg[v] = 0.0;
    has_pos[v] = has_neg[v] = flat[v] = false;
  }
  auto classify = [&](int v, double inc) {
    if (icmp::gt_pos(inc, tol[v])) {
      has_pos[v] = true;
      if (icmp::lt_nonneg(pos[v], inc)) pos[v] = inc;
    } else if (icmp::neg_gt_pos(inc, tol[v])) {
      has_neg[v] = true;
      const double m = negate(inc);
      if (icmp::lt_nonneg(neg[v], m)) neg[v] = m;
    } else {
      flat[v] = true;
    }
  };
  constexpr int kCache = NS > 0 ? NS : 4;
  double inc_cache[kCache][4];
#pragma unroll
  for (int k = 0; k < kCache; ++k) {
    if (NS > 0 || s0 + k < s1) {
      const double2 d = g.lim_d[s0 + k];
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        double inc = kmul<MUL_INCREMENT>(gx[v], d.x) + kmul<MUL_INCREMENT>(gy[v], d.y);
        inc_cache[k][v] = inc;
        classify(v, inc);
      }
    }
  }
  if (NS == 0) {
    for (int s = s0 + kCache; s < s1; ++s) {
      const double2 d = g.lim_d[s];
#pragma unroll
      for (int v = 0; v < 4; ++v) classify(v, kmul<MUL_INCREMENT>(gx[v], d.x) + kmul<MUL_INCREMENT>(gy[v], d.y));
    }
  }
  double phi[4];
#pragma unroll
  for (int v = 0; v < 4; ++v) {
    if constexpr (kMinRatio)
      phi[v] = limiter_factor_min_ratio<LIMITER>(pv[v], lo[v], hi[v], pos[v], negate(neg[v]), has_pos[v], has_neg[v], flat[v]);
    else
      phi[v] = limiter_factor_fast<LIMITER>(hi[v] - pv[v], pos[v], pv[v] - lo[v], neg[v], has_pos[v], has_neg[v], flat[v]);
  }
#pragma unroll
  for (int k = 0; k < kCache; ++k) {
    if (NS > 0 || s0 + k < s1) {
      St4 o{pv[0] + phi[0] * inc_cache[k][0], pv[1] + phi[1] * inc_cache[k][1],
            pv[2] + phi[2] * inc_cache[k][2], pv[3] + phi[3] * inc_cache[k][3]};
      st4(recon + 4 * (size_t)g.lim_slot[s0 + k], o);
    }
  }
  if (NS == 0) {
    for (int s = s0 + kCache; s < s1; ++s) {
      const double2 d = g.lim_d[s];
      double out[4];
#pragma unroll
      for (int v = 0; v < 4; ++v) out[v] = pv[v] + phi[v] * (kmul<MUL_INCREMENT>(gx[v], d.x) + kmul<MUL_INCREMENT>(gy[v], d.y));
      st4(recon + 4 * (size_t)g.lim_slot[s], St4{out[0], out[1], out[2], out[3]});
    }
  }
}

// The same cell for exactly NS limiter entries, one variable at a time: the
// variable's increments, limiter factor and face values are finished before
// the next variable starts, which keeps one variable's limiter state live
// instead of four (fewer registers than the all-variables form, so no FP64
// work is recomputed to relieve register pressure).  Face values are stored
// per variable.
template <int LIMITER, int NS>
__device__ __forceinline__ void reconstruct_cell_fast_by_variable(const DevGeom& g, const double* __restrict__ P,
                                                                  double* __restrict__ recon, int c,
                                                                  const St4& p, int s0) {
  const double pv[4] = {p.a, p.b, p.c, p.d};
  double gx[4], gy[4];
  double lo[4] = {p.a, p.b, p.c, p.d}, hi[4] = {p.a, p.b, p.c, p.d};
  gradient_sums(g, P, c, pv, gx, gy, lo, hi);
  double2 dk[NS];
  size_t out[NS];
#pragma unroll
  for (int k = 0; k < NS; ++k) {
    dk[k] = g.lim_d[s0 + k];
    out[k] = 4 * (size_t)g.lim_slot[s0 + k];
  }
#pragma unroll
  for (int v = 0; v < 4; ++v) {
    const double tol = limiter_tolerance(pv[v]);
    double pos = 0.0, neg = 0.0, inc[NS];
    bool has_pos = false, has_neg = false, flat = false;
#pragma unroll
    for (int k = 0; k < NS; ++k) {
      inc[k] = kmul<MUL_INCREMENT>(gx[v], dk[k].x) + kmul<MUL_INCREMENT>(gy[v], dk[k].y);
      if (icmp::gt_pos(inc[k], tol)) {
        has_pos = true;
        if (icmp::lt_nonneg(pos, inc[k])) pos = inc[k];
      } else if (icmp::neg_gt_pos(inc[k], tol)) {
        has_neg = true;
        const double m = negate(inc[k]);
        if (icmp::lt_nonneg(neg, m)) neg = m;
      } else {
        flat = true;
      }
    }
    double phi;
    if constexpr (kMinRatio)
      phi = limiter_factor_min_ratio<LIMITER>(pv[v], lo[v], hi[v], pos, negate(neg), has_pos, has_neg, flat);
    else
      phi = limiter_factor_fast<LIMITER>(hi[v] - pv[v], pos, pv[v] - lo[v], neg, has_pos, has_neg, flat);
#pragma unroll
    for (int k = 0; k < NS; ++k) recon[out[k] + v] = pv[v] + kmul<MUL_OUTPUT>(phi, inc[k]);
  }
}

// Register bound of the 3 / 4-entry kernel: MCFD_RECON_MAXNREG caps the
// registers a thread directly; otherwise the bound is MCFD_RECON_MIN_BLOCKS
// resident 256-thread blocks per SM.
#ifndef MCFD_RECON_MIN_BLOCKS
#define MCFD_RECON_MIN_BLOCKS 3
#endif
#ifdef MCFD_RECON_MAXNREG
#define MCFD_RECON_BOUND __maxnreg__(MCFD_RECON_MAXNREG)
#else
#define MCFD_RECON_BOUND __launch_bounds__(kBlock, MCFD_RECON_MIN_BLOCKS)
#endif

// Cells with 3 or 4 limiter entries (cell_order[0 .. n_lim34)); the kernel
// for any other count is separate, so that its register budget does not set
// this one's occupancy.
template <int LIMITER>
__global__ void MCFD_RECON_BOUND k_reconstruct_fast(DevGeom g, const double* __restrict__ P, double* __restrict__ recon) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= g.n_lim34) return;
  const int c = g.cell_order[i];
  const St4 p = ld4(P + 4 * (size_t)c);
  const int s0 = g.lim_ptr[c];
  if (g.lim_ptr[c + 1] - s0 == 3) reconstruct_cell_fast_by_variable<LIMITER, 3>(g, P, recon, c, p, s0);
  else reconstruct_cell_fast_by_variable<LIMITER, 4>(g, P, recon, c, p, s0);
}

// The same reconstruction with one thread per (cell, variable): the four
// variables of a cell are independent (gradient, extremes, limiter and face
// values of variable v read only variable v), so four adjacent threads take
// one cell's variables and run exactly the per-variable code above, with a
// quarter of its registers: more warps per SM to hide the latency of the
// integer-pipe divisions.  Cells with 3 or 4 limiter entries; results are
// those of k_reconstruct_fast.
template <int LIMITER, int NS>
__device__ __forceinline__ void reconstruct_variable_fast(const DevGeom& g, const double* __restrict__ P,
                                                          double* __restrict__ recon, int c, int v, double pv,
                                                          int s0) {
  double gx = 0.0, gy = 0.0, lo = pv, hi = pv;
  const bool positive = (v == 0 || v == 3);  // density and pressure: the raw bits order them
  auto visit = [&](int e, auto first) {  // the first sum is 0.0 + t: plus_zero (gradient_sums)
    const double q = P[4 * (size_t)g.grad_nb[e] + v];
    const double d = q - pv;
    const double tx = kmul<MUL_GRADIENT>(g.grad_cx[e], d), ty = kmul<MUL_GRADIENT>(g.grad_cy[e], d);
    if constexpr (decltype(first)::value) {
      gx = plus_zero(tx);
      gy = plus_zero(ty);
    } else {
      gx = gx + tx;
      gy = gy + ty;
    }
    const bool below = positive ? icmp::lt_pos(q, lo) : icmp::lt(q, lo);
    const bool above = positive ? icmp::gt_pos(q, hi) : icmp::lt(hi, q);
    if (below) lo = q;
    if (above) hi = q;
  };
  int e = g.grad_ptr[c];
  const int e1 = g.grad_ptr[c + 1];
  if (e < e1) visit(e++, std::true_type{});
  for (; e < e1; ++e) visit(e, std::false_type{});
  const double tol = limiter_tolerance(pv);
  double pos = 0.0, neg = 0.0, inc[NS];
  bool has_pos = false, has_neg = false, flat = false;
#pragma unroll
  for (int k = 0; k < NS; ++k) {
    const double2 dk = g.lim_d[s0 + k];
    inc[k] = kmul<MUL_INCREMENT>(gx, dk.x) + kmul<MUL_INCREMENT>(gy, dk.y);
    if (icmp::gt_pos(inc[k], tol)) {
      has_pos = true;
      if (icmp::lt_nonneg(pos, inc[k])) pos = inc[k];
    } else if (icmp::neg_gt_pos(inc[k], tol)) {
      has_neg = true;
      const double m = negate(inc[k]);
      if (icmp::lt_nonneg(neg, m)) neg = m;
    } else {
      flat = true;
    }
  }
  double phi;
  if constexpr (kMinRatio)
    phi = limiter_factor_min_ratio<LIMITER>(pv, lo, hi, pos, negate(neg), has_pos, has_neg, flat);
  else
    phi = limiter_factor_fast<LIMITER>(hi - pv, pos, pv - lo, neg, has_pos, has_neg, flat);
#pragma unroll
  for (int k = 0; k < NS; ++k) recon[4 * (size_t)g.lim_slot[s0 + k] + v] = pv + kmul<MUL_OUTPUT>(phi, inc[k]);
}

// 6 resident 256-thread blocks per SM (40 registers, a 4-byte spill) for the
// per-variable reconstruction: 0.394 against 0.406 ms per launch on the
// 1024^2 vortex (47 registers at 4 blocks); 5 blocks (46 registers) 0.410.
#ifndef MCFD_RECON_SPLIT_MIN_BLOCKS
#define MCFD_RECON_SPLIT_MIN_BLOCKS 6
#endif

template <int LIMITER>
__global__ void __launch_bounds__(kBlock, MCFD_RECON_SPLIT_MIN_BLOCKS) k_reconstruct_fast_split(
    DevGeom g, const double* __restrict__ P, double* __restrict__ recon) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = t >> 2, v = t & 3;
  if (i >= g.n_lim34) return;
  const int c = g.cell_order[i];
  const double pv = P[4 * (size_t)c + v];
  const int s0 = g.lim_ptr[c];
  if (g.lim_ptr[c + 1] - s0 == 3) reconstruct_variable_fast<LIMITER, 3>(g, P, recon, c, v, pv, s0);
  else reconstruct_variable_fast<LIMITER, 4>(g, P, recon, c, v, pv, s0);
}

template <int LIMITER>
__global__ void __launch_bounds__(kBlock) k_reconstruct_fast_any(DevGeom g, const double* __restrict__ P,
                                                                 double* __restrict__ recon) {
  const int i = g.n_lim34 + blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= g.n_cells) return;
  const int c = g.cell_order[i];
  const St4 p = ld4(P + 4 * (size_t)c);
  reconstruct_cell_fast<LIMITER, 0>(g, P, recon, c, p, g.lim_ptr[c], g.lim_ptr[c + 1]);
}

// -------------------------------------------------------------------- fluxes

template <int FLUX, bool KERNEL_HLLC>
__device__ __forceinline__ int numerical_flux(const St4& L, const St4& R, double nx, double ny,
                                              double gamma, double inv_gm1, double out[4]) {
  if (FLUX == MCFD_FLUX_RUSANOV) {
    if constexpr (kFast) rusanov_flux_fast(L, R, nx, ny, gamma, inv_gm1, out);
    else rusanov_flux(L, R, nx, ny, gamma, out);
    return 0;
  } else if (FLUX == MCFD_FLUX_HLLC) {
    bool ok;
    if constexpr (kFast) ok = hllc_flux_fast<KERNEL_HLLC>(L, R, nx, ny, gamma, inv_gm1, out);
    else ok = hllc_flux<KERNEL_HLLC>(L, R, nx, ny, gamma, out);
    return ok ? 0 : MCFD_S_HLLC_NONFINITE;
  } else {
    if constexpr (kFast) return roe_flux_fast(L, R, nx, ny, gamma, inv_gm1, out);
    else return roe_flux(L, R, nx, ny, gamma, out);
  }
}

// One flux face of segment SEG (face f of the flux-face list, `begin` the
// segment's first face).  FIRST_ORDER reads cell states directly (the
// reference's reconstruction is the identity there: zero gradients, unit
// factors).
template <int FLUX, int SEG, bool FIRST_ORDER, bool KERNEL_HLLC>
__device__ __forceinline__ void flux_face(const DevGeom& g, const double* P, const double* recon, double* flux,
                                          double gamma, double inv_gm1, int f, int begin) {
  const double2 n = g.ff_normal[f];
  const St4 L = FIRST_ORDER ? ld4(P + 4 * (size_t)g.ff_lcell[f]) : ld4(recon + 4 * (size_t)g.ff_lslot[f]);
  St4 R;
  int bits = 0;
  if (SEG == SEG_INTERIOR || SEG == SEG_PERIODIC) {
    R = FIRST_ORDER ? ld4(P + 4 * (size_t)g.ff_rcell[f]) : ld4(recon + 4 * (size_t)g.ff_rslot[f]);
  } else if (SEG == SEG_WALL) {
    // solver.py:2536-2543: mirror the velocity relative to the wall velocity.
    const double2 wv = g.ff_wall_velocity[f - begin];
    double un = (L.b - wv.x) * n.x + (L.c - wv.y) * n.y;
    R = St4{L.a, L.b - (2.0 * un) * n.x, L.c - (2.0 * un) * n.y, L.d};
  } else if (SEG == SEG_VIN) {
    R = ld4(g.ff_vin_state + 4 * (size_t)(f - begin));  // solver.py:2558
  } else if (SEG == SEG_POUT) {
    R = St4{L.a, L.b, L.c, g.ff_pout_pressure[f - begin]};  // solver.py:2581-2582
  } else if (SEG == SEG_FAR) {
    bits |= far_field_state(L, ld4(g.ff_far_state + 4 * (size_t)(f - begin)), n.x, n.y, gamma, &R);
  } else {
    R = ld4(g.bc_ext + 4 * (size_t)(f - begin));  // solver.py:2626-2698, states from k_bc_states
  }
  double out[4];
  bits |= numerical_flux<FLUX, (SEG == SEG_INTERIOR) && KERNEL_HLLC>(L, R, n.x, n.y, gamma, inv_gm1, out);
  if (bits) flag_face(g.status, bits, f);
  st4(flux + 4 * (size_t)f, St4{out[0], out[1], out[2], out[3]});
}

// One launch per segment keeps every warp on one code path.
template <int FLUX, int SEG, bool FIRST_ORDER, bool KERNEL_HLLC>
__global__ void __launch_bounds__(kBlock) k_flux(DevGeom g, const double* __restrict__ P,
                                                 const double* __restrict__ recon,
                                                 double* __restrict__ flux, double gamma,
                                                 double inv_gm1) {
  const int begin = g.seg_begin[SEG], end = g.seg_begin[SEG + 1];
  // grid-stride: the autotuner may give each thread several faces
  for (int f = begin + blockIdx.x * blockDim.x + threadIdx.x; f < end; f += gridDim.x * blockDim.x)
    flux_face<FLUX, SEG, FIRST_ORDER, KERNEL_HLLC>(g, P, recon, flux, gamma, inv_gm1, f, begin);
}

// --------------------------------------------------------------- time steps
//
// _stable_time_steps (solver.py:4132-4343), inviscid: per cell, the sum over
// its owner-side faces (face order) of (|u.n| + c) * L — with the exterior
// radius max'ed in on inlet / outlet / far-field faces — then over its
// neighbour-side interior faces; dt = CFL * A / sum; global = min.

// One cell's stable time step from its primitive p (flags status bits).
__device__ __forceinline__ double cell_time_step(const DevGeom& g, int c, const St4& p, double gamma, double cfl,
                                                 const double* __restrict__ diffusion, int* bits) {
  const double sound = sound_speed(p.a, p.d, gamma);
  double sum = 0.0;
  for (int e = g.dt_ptr[c], e1 = g.dt_ptr[c + 1]; e < e1; ++e) {
    const double2 n = g.dt_normal[e];
    const int info = g.dt_info[e];
    double radius = abs_of(p.b * n.x + p.c * n.y) + sound;
    const int kind = info >> 28;
    if (kind != DT_PLAIN) {
      const int idx = info & 0x0fffffff;
      St4 ext;
      if (kind == DT_VIN) ext = ld4(g.ff_vin_state + 4 * (size_t)idx);
      else if (kind == DT_POUT) ext = St4{p.a, p.b, p.c, g.ff_pout_pressure[idx]};
      else if (kind == DT_FAR) *bits |= far_field_state(p, ld4(g.ff_far_state + 4 * (size_t)idx), n.x, n.y, gamma, &ext);
      else ext = ld4(g.bc_ext_dt + 4 * (size_t)idx);  // solver.py:4153-4188, states from k_bc_states
      double er = abs_of(ext.b * n.x + ext.c * n.y) + sound_speed(ext.a, ext.d, gamma);
      radius = icmp::lt_nonneg(radius, er) ? er : radius;  // np.maximum
    }
    sum = sum + radius * g.dt_len[e];
  }
  if (diffusion) sum += 2.0 * diffusion[c];  // viscous terms (solver.py:4331)
  const double dt = div_rn(cfl * g.area[c], sum);
  if (!icmp::finite(dt) || !icmp::gt0(dt)) *bits |= MCFD_S_TIME_STEP;
  return dt;
}

// Block minimum of the positive time steps by warp shuffles, then one
// atomicMin on the bit pattern (positive doubles order like their bits).
// Every thread of the block calls it.
__device__ __forceinline__ void block_min_time_step(DevStatus* st, double dt, bool active) {
  long long m = (active && icmp::gt0(dt)) ? icmp::bits(dt) : 0x7ff0000000000000LL;
  for (int off = 16; off > 0; off >>= 1) {
    long long o = __shfl_down_sync(0xffffffffu, m, off);
    m = (o < m) ? o : m;
  }
  __shared__ long long warp_min[32];
  if ((threadIdx.x & 31) == 0) warp_min[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    long long b = warp_min[0];
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) b = (warp_min[w] < b) ? warp_min[w] : b;
    atomicMin(&st->dt_min_bits, (unsigned long long)b);
  }
}

__global__ void __launch_bounds__(kBlock) k_time_steps(DevGeom g, const double* __restrict__ P,
                                                       double gamma, double cfl,
                                                       double* __restrict__ dt_cells,
                                                       int want_min, const double* __restrict__ diffusion) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const bool active = i < g.n_cells;
  double dt = __longlong_as_double(0x7ff0000000000000LL);
  if (active) {
    const int c = g.cell_order[i];
    int bits = 0;
    dt = cell_time_step(g, c, ld4(P + 4 * (size_t)c), gamma, cfl, diffusion, &bits);
    if (bits) flag_cell(g.status, bits, c);
    if (dt_cells) dt_cells[c] = dt;
  }
  if (want_min) block_min_time_step(g.status, dt, active);
}

// ------------------------------------------------------------ gather + stage

__device__ __forceinline__ double stage_dt(const StageProgram& prog, int c) {
  return prog.dt_per_cell ? prog.dt[c] : prog.dt[0];
}

// Stage-combination shapes with their own code path (the generic loop over
// runtime term kinds lets the compiler predicate every kind's arithmetic into
// each evaluation, and predicated-off FP64 instructions still take FP64 issue
// slots):
//   SHAPE_EULER   u = x + dt r      terms {X 1.0 x, DTR 1.0} (1.0 * v == v)
//   SHAPE_X_XDTR  u = c0 x0 + c1 (x1 + dt r)   terms {X c0 x0, X_PLUS_DTR c1 x1}
// EXTRAS compiles the viscous residual and body-force adds in.
enum GatherShape { SHAPE_GENERIC = 0, SHAPE_EULER = 1, SHAPE_X_XDTR = 2 };

// Cell at visiting position i: divergence, boundary adds, extras, finiteness
// check, stage combination and primitive recovery of the new state.
template <int SHAPE, bool EXTRAS>
__device__ __forceinline__ void gather_cell(const DevGeom& g, const double* P, const double* flux, double gamma,
                                            double ax, double ay, const StageProgram& prog, int i,
                                            St4* q_out = nullptr) {
  const int c = g.cell_order[i];
  // interior divergence: SciPy CSR product, ascending face order
  // (solver.py:2160-2174, 2501); derivative starts from zero.
  // the first term's sum 0.0 + t is plus_zero(t) (integer pipe, same bits)
  double s[4] = {0.0, 0.0, 0.0, 0.0};
  int j = g.gi_ptr[c];
  const int j1 = g.gi_ptr[c + 1];
  if (j < j1) {
    const double a = g.gi_coef[j];
    const St4 F = ld4(flux + 4 * (size_t)g.gi_flux[j]);
    s[0] = plus_zero(kmul<MUL_GATHER>(a, F.a));
    s[1] = plus_zero(kmul<MUL_GATHER>(a, F.b));
    s[2] = plus_zero(kmul<MUL_GATHER>(a, F.c));
    s[3] = plus_zero(kmul<MUL_GATHER>(a, F.d));
    ++j;
  }
  for (; j < j1; ++j) {
    const double a = g.gi_coef[j];
    const St4 F = ld4(flux + 4 * (size_t)g.gi_flux[j]);
    s[0] = s[0] + kmul<MUL_GATHER>(a, F.a);
    s[1] = s[1] + kmul<MUL_GATHER>(a, F.b);
    s[2] = s[2] + kmul<MUL_GATHER>(a, F.c);
    s[3] = s[3] + kmul<MUL_GATHER>(a, F.d);
  }
  double r[4] = {plus_zero(s[0]), plus_zero(s[1]), plus_zero(s[2]), plus_zero(s[3])};  // 0.0 + s
  // boundary groups: np.add.at(derivative, owners, -(flux*L)/A) in BC order
  const int jb0 = g.gb_ptr[c], jb1 = g.gb_ptr[c + 1];
  if (jb0 < jb1) {
    const double area = g.area[c];
    for (int j = jb0; j < jb1; ++j) {
      const double len = g.gb_len[j];
      const St4 F = ld4(flux + 4 * (size_t)g.gb_flux[j]);
      r[0] = r[0] + div_rn(F.a * len, area);
      r[1] = r[1] + div_rn(F.b * len, area);
      r[2] = r[2] + div_rn(F.c * len, area);
      r[3] = r[3] + div_rn(F.d * len, area);
    }
  }
  if (EXTRAS) {
    if (prog.visc_r) {  // derivative += _viscous_residual(...) (solver.py:2699-2702)
      const St4 v = ld4(prog.visc_r + 4 * (size_t)c);
      r[0] = r[0] + v.a;
      r[1] = r[1] + v.b;
      r[2] = r[2] + v.c;
      r[3] = r[3] + v.d;
    }
    if (icmp::abs_gt(ax, 0.0) || icmp::abs_gt(ay, 0.0)) {  // ax != 0 or ay != 0 (solver.py:2709-2715)
      const St4 p = ld4(P + 4 * (size_t)c);
      r[1] = r[1] + p.a * ax;
      r[2] = r[2] + p.a * ay;
      r[3] = r[3] + p.a * (ax * p.b + ay * p.c);
    }
  }
  if (!(icmp::finite(r[0]) && icmp::finite(r[1]) && icmp::finite(r[2]) && icmp::finite(r[3])))
    flag_cell(g.status, MCFD_S_NONFINITE_RESIDUAL, c);
  if (prog.out_r) st4(prog.out_r + 4 * (size_t)c, St4{r[0], r[1], r[2], r[3]});
  if (!prog.out_u) return;
  const double dt = stage_dt(prog, c);
  double u[4];
  if (SHAPE == SHAPE_EULER) {
    const St4 x = ld4(prog.t[0].x + 4 * (size_t)c);
    u[0] = x.a + kmul<MUL_GATHER>(dt, r[0]);
    u[1] = x.b + kmul<MUL_GATHER>(dt, r[1]);
    u[2] = x.c + kmul<MUL_GATHER>(dt, r[2]);
    u[3] = x.d + kmul<MUL_GATHER>(dt, r[3]);
  } else if (SHAPE == SHAPE_X_XDTR) {
    const double c0 = prog.t[0].coef, c1 = prog.t[1].coef;
    const St4 x0 = ld4(prog.t[0].x + 4 * (size_t)c);
    const St4 x1 = ld4(prog.t[1].x + 4 * (size_t)c);
    u[0] = kmul<MUL_GATHER>(c0, x0.a) + kmul<MUL_GATHER>(c1, x1.a + kmul<MUL_GATHER>(dt, r[0]));
    u[1] = kmul<MUL_GATHER>(c0, x0.b) + kmul<MUL_GATHER>(c1, x1.b + kmul<MUL_GATHER>(dt, r[1]));
    u[2] = kmul<MUL_GATHER>(c0, x0.c) + kmul<MUL_GATHER>(c1, x1.c + kmul<MUL_GATHER>(dt, r[2]));
    u[3] = kmul<MUL_GATHER>(c0, x0.d) + kmul<MUL_GATHER>(c1, x1.d + kmul<MUL_GATHER>(dt, r[3]));
  } else {
  for (int t = 0; t < prog.n_terms; ++t) {
    const StageTerm term = prog.t[t];
    double v[4];
    if (term.kind == TERM_X) {
      const St4 x = ld4(term.x + 4 * (size_t)c);
      v[0] = term.coef * x.a; v[1] = term.coef * x.b; v[2] = term.coef * x.c; v[3] = term.coef * x.d;
    } else if (term.kind == TERM_X_PLUS_DTR) {
      const St4 x = ld4(term.x + 4 * (size_t)c);
      v[0] = term.coef * (x.a + dt * r[0]);
      v[1] = term.coef * (x.b + dt * r[1]);
      v[2] = term.coef * (x.c + dt * r[2]);
      v[3] = term.coef * (x.d + dt * r[3]);
    } else if (term.kind == TERM_DTR) {
      const double cdt = term.coef * dt;
      v[0] = cdt * r[0]; v[1] = cdt * r[1]; v[2] = cdt * r[2]; v[3] = cdt * r[3];
    } else {
      const double cdt = term.coef * dt;
      const St4 x = ld4(term.x + 4 * (size_t)c);
      v[0] = cdt * x.a; v[1] = cdt * x.b; v[2] = cdt * x.c; v[3] = cdt * x.d;
    }
    if (t == 0) {
      u[0] = v[0]; u[1] = v[1]; u[2] = v[2]; u[3] = v[3];
    } else {
      u[0] = u[0] + v[0]; u[1] = u[1] + v[1]; u[2] = u[2] + v[2]; u[3] = u[3] + v[3];
    }
  }
  }
  const St4 U = St4{u[0], u[1], u[2], u[3]};
  st4(prog.out_u + 4 * (size_t)c, U);
  if (prog.out_p) {
    bool ok;
    const St4 q = to_prim(U, gamma, &ok);
    if (!ok) flag_cell(g.status, MCFD_S_NONPHYSICAL_STATE, c);
    st4(prog.out_p + 4 * (size_t)c, q);
    if (q_out) *q_out = q;
  }
}

// Resident 256-thread blocks per SM of the gather (0: unbounded): 5 (48
// registers instead of 54) measured 0.159 against 0.161 ms per stage on the
// 1024^2 vortex; 6 spills.
#ifndef MCFD_GATHER_MIN_BLOCKS
#define MCFD_GATHER_MIN_BLOCKS 5
#endif
#if MCFD_GATHER_MIN_BLOCKS > 0
#define MCFD_GATHER_BOUND __launch_bounds__(kBlock, MCFD_GATHER_MIN_BLOCKS)
#else
#define MCFD_GATHER_BOUND __launch_bounds__(kBlock)
#endif

template <int SHAPE, bool EXTRAS>
__global__ void MCFD_GATHER_BOUND k_gather(DevGeom g, const double* __restrict__ P,
                                                   const double* __restrict__ flux, double gamma,
                                                   double ax, double ay, StageProgram prog) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < g.n_cells) gather_cell<SHAPE, EXTRAS>(g, P, flux, gamma, ax, ay, prog, i);
}

// The gather of a step's last stage that also computes the stable time steps
// of its new state from the primitive it has just recovered (cell_time_step,
// the same bits as k_time_steps on that primitive), which saves the
// time-step pass over the state of the next step.
// Resident 256-thread blocks per SM of the time-step gather: 4 (64
// registers, a 24-byte spill) measured 0.162 against 0.171 ms per stage on
// the 1024^2 vortex step (78 registers unbounded, 80 for 3 blocks); 0 leaves
// the kernel unbounded.
#ifndef MCFD_GATHER_DT_MIN_BLOCKS
#define MCFD_GATHER_DT_MIN_BLOCKS 4
#endif
#if MCFD_GATHER_DT_MIN_BLOCKS > 0
#define MCFD_GATHER_DT_BOUND __launch_bounds__(kBlock, MCFD_GATHER_DT_MIN_BLOCKS)
#else
#define MCFD_GATHER_DT_BOUND __launch_bounds__(kBlock)
#endif

template <int SHAPE, bool EXTRAS>
__global__ void MCFD_GATHER_DT_BOUND k_gather_dt(DevGeom g, const double* __restrict__ P,
                                                                              const double* __restrict__ flux,
                                                                              double gamma, double ax, double ay,
                                                                              StageProgram prog) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const bool active = i < g.n_cells;
  double dt = __longlong_as_double(0x7ff0000000000000LL);
  if (active) {
    St4 q;
    gather_cell<SHAPE, EXTRAS>(g, P, flux, gamma, ax, ay, prog, i, &q);
    const int c = g.cell_order[i];
    int bits = 0;
    dt = cell_time_step(g, c, q, gamma, prog.cfl, nullptr, &bits);
    if (bits) flag_cell(prog.next_dt_status, bits, c);
    if (prog.next_dt_cells) prog.next_dt_cells[c] = dt;
  }
  if (prog.next_dt_min) block_min_time_step(prog.next_dt_status, dt, active);
}

// ------------------------------------------------------ one launch per stage
//
// The three phases of an explicit stage — reconstruction, face fluxes,
// gather with the stage update — in one cooperative launch of one grid (as
// many resident blocks as the SMs hold), separated by grid barriers.  Each
// phase is a grid-stride loop over the items of its own kernel and runs the
// same per-item code (reconstruct_variable_fast / reconstruct_cell_fast,
// flux_face per segment, gather_cell), so the results are those of the
// three-launch stage bit for bit.  Built for the smallest-ratio variant with
// HLLC and MUSCL-linear reconstruction (one of the four capped limiters), inviscid,
// without pressure-inlet / mass-flow patches or a body force, and the Euler
// and x0 + (x1 + dt r) stage shapes; launch_stage_fused refuses the rest.
// No restrict qualifiers: the gather phase writes the primitive array that
// the first two phases read.
#ifndef MCFD_FUSED_MIN_BLOCKS
#define MCFD_FUSED_MIN_BLOCKS 3
#endif

template <int FLUX, int SEG>
__device__ __forceinline__ void flux_phase(const DevGeom& g, const double* P, const double* recon, double* flux,
                                           double gamma, double inv_gm1, int tid, int stride) {
  const int begin = g.seg_begin[SEG], end = g.seg_begin[SEG + 1];
  for (int f = begin + tid; f < end; f += stride)
    flux_face<FLUX, SEG, false, true>(g, P, recon, flux, gamma, inv_gm1, f, begin);
}

// Cells with other than 3 or 4 limiter entries (polygons): out of line, so
// that their larger register demand stays in this rarely taken call.
template <int LIMITER>
__device__ __noinline__ void reconstruct_cell_any(const DevGeom& g, const double* P, double* recon, int c) {
  reconstruct_cell_fast<LIMITER, 0>(g, P, recon, c, ld4(P + 4 * (size_t)c), g.lim_ptr[c], g.lim_ptr[c + 1]);
}

template <int LIMITER, int FLUX, int SHAPE>
__global__ void __launch_bounds__(kBlock, MCFD_FUSED_MIN_BLOCKS) k_stage_fused(DevGeom g, const double* P,
                                                                               double* recon, double* flux,
                                                                               double gamma, double inv_gm1,
                                                                               StageProgram prog) {
  cg::grid_group grid = cg::this_grid();
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int stride = gridDim.x * blockDim.x;  // a multiple of 4: t & 3 is the variable
  const int n4 = 4 * g.n_lim34;
  for (int t = tid; t < n4; t += stride) {
    const int c = g.cell_order[t >> 2], v = t & 3;
    const double pv = P[4 * (size_t)c + v];
    const int s0 = g.lim_ptr[c];
    if (g.lim_ptr[c + 1] - s0 == 3) reconstruct_variable_fast<LIMITER, 3>(g, P, recon, c, v, pv, s0);
    else reconstruct_variable_fast<LIMITER, 4>(g, P, recon, c, v, pv, s0);
  }
  for (int i = g.n_lim34 + tid; i < g.n_cells; i += stride) reconstruct_cell_any<LIMITER>(g, P, recon, g.cell_order[i]);
  grid.sync();
  flux_phase<FLUX, SEG_INTERIOR>(g, P, recon, flux, gamma, inv_gm1, tid, stride);
  flux_phase<FLUX, SEG_PERIODIC>(g, P, recon, flux, gamma, inv_gm1, tid, stride);
  flux_phase<FLUX, SEG_WALL>(g, P, recon, flux, gamma, inv_gm1, tid, stride);
  flux_phase<FLUX, SEG_VIN>(g, P, recon, flux, gamma, inv_gm1, tid, stride);
  flux_phase<FLUX, SEG_POUT>(g, P, recon, flux, gamma, inv_gm1, tid, stride);
  flux_phase<FLUX, SEG_FAR>(g, P, recon, flux, gamma, inv_gm1, tid, stride);
  grid.sync();
  for (int i = tid; i < g.n_cells; i += stride) gather_cell<SHAPE, false>(g, P, flux, gamma, 0.0, 0.0, prog, i);
}

__global__ void k_time_step_finalize(DevStatus* st, double* dt_min, double time_limit) {
  double stable = __longlong_as_double((long long)st->dt_min_bits);
  // min(stable, end_time - time) with Python's min semantics (solver.py:455-461)
  dt_min[0] = icmp::lt(time_limit, stable) ? time_limit : stable;
  st->dt_min_bits = 0x7ff0000000000000ULL;
}

// ------------------------------------------------------------------ launchers

static inline int blocks_for(int n) { return (n + kBlock - 1) / kBlock; }


cudaError_t launch_primitive(const DevGeom& g, const mcfd_config& cfg, const double* U, double* P,
                             cudaStream_t s) {
  if (g.n_cells > 0) count_launch(), k_primitive<<<blocks_for(g.n_cells), kBlock, 0, s>>>(g.n_cells, U, P, cfg.gamma, g.status);
  return cudaGetLastError();
}

cudaError_t launch_reconstruct(const DevGeom& g, const mcfd_config& cfg, const double* P,
                               double* recon, cudaStream_t s) {
  if (g.n_cells == 0) return cudaSuccess;
  const int t = g.tune_recon_threads ? g.tune_recon_threads : kBlock;
  const int b = (g.n_cells + t - 1) / t;
  if (cfg.limiter == MCFD_LIMITER_VENKATAKRISHNAN_K) {
    // the smooth form has no smallest-ratio shortcut: per-face evaluation in
    // every variant
    count_launch();
    k_reconstruct<MCFD_LIMITER_VENKATAKRISHNAN_K><<<b, t, 0, s>>>(g, P, recon, cfg.venkat_k);
    return cudaGetLastError();
  }
  if constexpr (kFast || kMinRatio) {
    if (g.n_lim34 > 0 && g.tune_recon_split) {
      const int bs = (int)((4LL * g.n_lim34 + t - 1) / t);
      count_launch();
      switch (cfg.limiter) {
        case 0: k_reconstruct_fast_split<0><<<bs, t, 0, s>>>(g, P, recon); break;
        case 1: k_reconstruct_fast_split<1><<<bs, t, 0, s>>>(g, P, recon); break;
        case 2: k_reconstruct_fast_split<2><<<bs, t, 0, s>>>(g, P, recon); break;
        default: k_reconstruct_fast_split<3><<<bs, t, 0, s>>>(g, P, recon); break;
      }
    } else if (g.n_lim34 > 0) {
      const int b34 = (g.n_lim34 + t - 1) / t;
      count_launch();
      switch (cfg.limiter) {
        case 0: k_reconstruct_fast<0><<<b34, t, 0, s>>>(g, P, recon); break;
        case 1: k_reconstruct_fast<1><<<b34, t, 0, s>>>(g, P, recon); break;
        case 2: k_reconstruct_fast<2><<<b34, t, 0, s>>>(g, P, recon); break;
        default: k_reconstruct_fast<3><<<b34, t, 0, s>>>(g, P, recon); break;
      }
    }
    if (g.n_cells > g.n_lim34) {
      const int ba = (g.n_cells - g.n_lim34 + kBlock - 1) / kBlock;
      count_launch();
      switch (cfg.limiter) {
        case 0: k_reconstruct_fast_any<0><<<ba, kBlock, 0, s>>>(g, P, recon); break;
        case 1: k_reconstruct_fast_any<1><<<ba, kBlock, 0, s>>>(g, P, recon); break;
        case 2: k_reconstruct_fast_any<2><<<ba, kBlock, 0, s>>>(g, P, recon); break;
        default: k_reconstruct_fast_any<3><<<ba, kBlock, 0, s>>>(g, P, recon); break;
      }
    }
  } else {
    count_launch();
    switch (cfg.limiter) {
      case 0: k_reconstruct<0><<<b, t, 0, s>>>(g, P, recon, 0.0); break;
      case 1: k_reconstruct<1><<<b, t, 0, s>>>(g, P, recon, 0.0); break;
      case 2: k_reconstruct<2><<<b, t, 0, s>>>(g, P, recon, 0.0); break;
      default: k_reconstruct<3><<<b, t, 0, s>>>(g, P, recon, 0.0); break;
    }
  }
  return cudaGetLastError();
}

// Boundary segments run on the side stream (when given) concurrently with
// the interior faces; every face writes only its own flux row.
template <int FLUX, bool FO, bool KH>
static void flux_segments(const DevGeom& g, const double* P, const double* recon, double* flux,
                          double gamma, cudaStream_t s, const SideStream* side) {
  const double inv_gm1 = 1.0 / (gamma - 1.0);
  const bool fork = side && side->stream && g.seg_begin[SEG_COUNT] > g.seg_begin[SEG_INTERIOR + 1];
  if (fork) {
    cudaEventRecord(side->fork, s);
    cudaStreamWaitEvent(side->stream, side->fork, 0);
  }
  const cudaStream_t b = fork ? side->stream : s;
#define MCFD_SEG(SEGV, STREAM)                                                      \
  {                                                                                 \
    int n = g.seg_begin[SEGV + 1] - g.seg_begin[SEGV];                              \
    if (n > 0) count_launch(), k_flux<FLUX, SEGV, FO, KH><<<flux_blocks(g, n), flux_threads(g, n), 0, STREAM>>>(g, P, recon, flux, gamma, inv_gm1); \
  }
  MCFD_SEG(SEG_PERIODIC, b)
  MCFD_SEG(SEG_WALL, b)
  MCFD_SEG(SEG_VIN, b)
  MCFD_SEG(SEG_POUT, b)
  MCFD_SEG(SEG_FAR, b)
  MCFD_SEG(SEG_BCX, b)
  MCFD_SEG(SEG_INTERIOR, s)
#undef MCFD_SEG
  if (fork) {
    cudaEventRecord(side->join, side->stream);
    cudaStreamWaitEvent(s, side->join, 0);
  }
}

cudaError_t launch_flux(const DevGeom& g, const mcfd_config& cfg, const double* P,
                        const double* recon, double* flux, cudaStream_t s, const SideStream* side) {
  const bool fo = cfg.reconstruction == MCFD_RECON_FIRST_ORDER;
  // The reference evaluates interior HLLC faces with its fused compiled kernel
  // when no curvature is present (solver.py:2479-2490); that kernel has its
  // own branch order.  Parabolic reconstruction uses the NumPy form.
  const bool kernel_hllc = cfg.reconstruction != MCFD_RECON_MUSCL_PARABOLIC;
  switch (cfg.flux) {
    case MCFD_FLUX_RUSANOV:
      if (fo) flux_segments<0, true, false>(g, P, recon, flux, cfg.gamma, s, side);
      else flux_segments<0, false, false>(g, P, recon, flux, cfg.gamma, s, side);
      break;
    case MCFD_FLUX_HLLC:
      if (fo) flux_segments<1, true, true>(g, P, recon, flux, cfg.gamma, s, side);
      else if (kernel_hllc) flux_segments<1, false, true>(g, P, recon, flux, cfg.gamma, s, side);
      else flux_segments<1, false, false>(g, P, recon, flux, cfg.gamma, s, side);
      break;
    default:
      if (fo) flux_segments<2, true, false>(g, P, recon, flux, cfg.gamma, s, side);
      else flux_segments<2, false, false>(g, P, recon, flux, cfg.gamma, s, side);
      break;
  }
  return cudaGetLastError();
}

cudaError_t launch_gather(const DevGeom& g, const mcfd_config& cfg, const double* P,
                          const double* flux, const StageProgram& prog, cudaStream_t s) {
  if (g.n_cells <= 0) return cudaSuccess;
  int shape = SHAPE_GENERIC;
  if (prog.out_u && prog.n_terms == 2 && prog.t[0].kind == TERM_X) {
    if (prog.t[1].kind == TERM_DTR && prog.t[0].coef == 1.0 && prog.t[1].coef == 1.0) shape = SHAPE_EULER;
    else if (prog.t[1].kind == TERM_X_PLUS_DTR) shape = SHAPE_X_XDTR;
  }
  const bool extras = prog.visc_r || cfg.acceleration_x != 0.0 || cfg.acceleration_y != 0.0;
  const int t = g.tune_gather_threads ? g.tune_gather_threads : kBlock;
  const int b = (g.n_cells + t - 1) / t;
  const double ax = cfg.acceleration_x, ay = cfg.acceleration_y;
  count_launch();
  if (prog.out_u && (prog.next_dt_cells || prog.next_dt_min) && !prog.visc_r) {
#define MCFD_GATHER_DT(SH, EX) k_gather_dt<SH, EX><<<b, t, 0, s>>>(g, P, flux, cfg.gamma, ax, ay, prog)
    if (extras) {
      if (shape == SHAPE_EULER) MCFD_GATHER_DT(SHAPE_EULER, true);
      else if (shape == SHAPE_X_XDTR) MCFD_GATHER_DT(SHAPE_X_XDTR, true);
      else MCFD_GATHER_DT(SHAPE_GENERIC, true);
    } else {
      if (shape == SHAPE_EULER) MCFD_GATHER_DT(SHAPE_EULER, false);
      else if (shape == SHAPE_X_XDTR) MCFD_GATHER_DT(SHAPE_X_XDTR, false);
      else MCFD_GATHER_DT(SHAPE_GENERIC, false);
    }
#undef MCFD_GATHER_DT
    return cudaGetLastError();
  }
#define MCFD_GATHER(SH, EX) k_gather<SH, EX><<<b, t, 0, s>>>(g, P, flux, cfg.gamma, ax, ay, prog)
  if (extras) {
    if (shape == SHAPE_EULER) MCFD_GATHER(SHAPE_EULER, true);
    else if (shape == SHAPE_X_XDTR) MCFD_GATHER(SHAPE_X_XDTR, true);
    else MCFD_GATHER(SHAPE_GENERIC, true);
  } else {
    if (shape == SHAPE_EULER) MCFD_GATHER(SHAPE_EULER, false);
    else if (shape == SHAPE_X_XDTR) MCFD_GATHER(SHAPE_X_XDTR, false);
    else MCFD_GATHER(SHAPE_GENERIC, false);
  }
#undef MCFD_GATHER
  return cudaGetLastError();
}

cudaError_t launch_time_steps(const DevGeom& g, const mcfd_config& cfg, const double* P,
                              double* dt_cells, double* dt_min, double time_limit,
                              cudaStream_t s) {
  if (g.n_cells > 0)
    count_launch(), k_time_steps<<<blocks_for(g.n_cells), kBlock, 0, s>>>(g, P, cfg.gamma, cfg.cfl, dt_cells,
                                                          dt_min != nullptr,
                                                          cfg.viscosity_model ? g.visc_diff : nullptr);
  if (dt_min) count_launch(), k_time_step_finalize<<<1, 1, 0, s>>>(g.status, dt_min, time_limit);
  return cudaGetLastError();
}


// Stage shape of a program (SHAPE_GENERIC when neither special shape fits).
static int stage_shape(const StageProgram& prog) {
  if (prog.out_u && prog.n_terms == 2 && prog.t[0].kind == TERM_X) {
    if (prog.t[1].kind == TERM_DTR && prog.t[0].coef == 1.0 && prog.t[1].coef == 1.0) return SHAPE_EULER;
    if (prog.t[1].kind == TERM_X_PLUS_DTR) return SHAPE_X_XDTR;
  }
  return SHAPE_GENERIC;
}

bool stage_fused_supported(const DevGeom& g, const mcfd_config& cfg, const StageProgram& prog) {
  if constexpr (!kMinRatio) return false;
  return cfg.flux == MCFD_FLUX_HLLC && cfg.reconstruction == MCFD_RECON_MUSCL_LINEAR && cfg.limiter >= 0 &&
         cfg.limiter <= 3 &&
         cfg.viscosity_model == MCFD_VISC_INVISCID && g.n_bc_patches == 0 && g.n_cells > 0 &&
         cfg.acceleration_x == 0.0 && cfg.acceleration_y == 0.0 && !prog.visc_r && prog.out_u &&
         !prog.next_dt_cells && !prog.next_dt_min && stage_shape(prog) != SHAPE_GENERIC;
}

template <int LIMITER, int FLUX, int SHAPE>
static cudaError_t launch_fused_as(const DevGeom& g, const mcfd_config& cfg, const double* P, double* recon,
                                   double* flux, const StageProgram& prog, cudaStream_t s, int* blocks_out) {
  auto kernel = k_stage_fused<LIMITER, FLUX, SHAPE>;
  int dev = 0, sms = 0, per_sm = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kBlock, 0);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) return cudaErrorCooperativeLaunchTooLarge;
  if (blocks_out) *blocks_out = per_sm;
  cudaLaunchConfig_t lc{};
  lc.gridDim = dim3(sms * per_sm);
  lc.blockDim = dim3(kBlock);
  lc.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  lc.attrs = attr;
  lc.numAttrs = 1;
  count_launch();
  return cudaLaunchKernelEx(&lc, kernel, g, P, recon, flux, cfg.gamma, 1.0 / (cfg.gamma - 1.0), prog);
}

template <int LIMITER, int FLUX>
static cudaError_t launch_fused_shape(const DevGeom& g, const mcfd_config& cfg, const double* P, double* recon,
                                      double* flux, const StageProgram& prog, cudaStream_t s, int* blocks) {
  if (stage_shape(prog) == SHAPE_EULER)
    return launch_fused_as<LIMITER, FLUX, SHAPE_EULER>(g, cfg, P, recon, flux, prog, s, blocks);
  return launch_fused_as<LIMITER, FLUX, SHAPE_X_XDTR>(g, cfg, P, recon, flux, prog, s, blocks);
}


cudaError_t launch_stage_fused(const DevGeom& g, const mcfd_config& cfg, const double* P, double* recon,
                               double* flux, const StageProgram& prog, cudaStream_t s, int* blocks_per_sm) {
  if (!stage_fused_supported(g, cfg, prog)) return cudaErrorNotSupported;
  if constexpr (kMinRatio) {
    switch (cfg.limiter) {
      case 0: return launch_fused_shape<0, MCFD_FLUX_HLLC>(g, cfg, P, recon, flux, prog, s, blocks_per_sm);
      case 1: return launch_fused_shape<1, MCFD_FLUX_HLLC>(g, cfg, P, recon, flux, prog, s, blocks_per_sm);
      case 2: return launch_fused_shape<2, MCFD_FLUX_HLLC>(g, cfg, P, recon, flux, prog, s, blocks_per_sm);
      default: return launch_fused_shape<3, MCFD_FLUX_HLLC>(g, cfg, P, recon, flux, prog, s, blocks_per_sm);
    }
  }
  return cudaErrorNotSupported;
}

}  // namespace MCFD_VARIANT
}  // namespace mcfd
