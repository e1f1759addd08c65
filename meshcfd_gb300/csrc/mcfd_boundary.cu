// Exterior states of pressure-inlet, mass-flow-inlet and mass-flow-outlet
// faces (solver.py:4412-4577), one block per boundary patch.
//
// * pressure inlet (_pressure_inlet_boundary_states): per face, the Mach
//   number by 64 bisection steps on the outgoing Riemann invariant, then the
//   isentropic static state from the total conditions;
// * mass-flow inlet (_mass_flow_inlet_boundary_states): one speed per patch by
//   80 bisection steps on the patch's integrated flow rate; every step the
//   block computes the face terms density * speed * projection * length in
//   parallel and one thread adds them in NumPy's pairwise order (np.sum);
//   density p / (R T) per face, velocity speed * direction on every face (the
//   reference builds a one-row velocity array there, which only works for
//   single-face patches, solver.py:4552-4554);
// * mass-flow outlet (_mass_flow_outlet_boundary_states): per face, the
//   normal velocity from the patch flow rate, tangential velocity kept.
// Checks set the reference's error bits and the lowest failing patch index.
// Python's scalar x**2 is libm pow and NumPy's array power its own SIMD code;
// both are reproduced only to the last place (x * x and CUDA pow here).
#include "mcfd_device.cuh"
#include "mcfd_internal.h"

namespace mcfd {
namespace {

constexpr int kBlock = 128;

__device__ __forceinline__ void flag_patch(DevStatus* st, int bits, int patch) {
  atomicOr(&st->code, bits);
  atomicMin(&st->first_patch, patch);
}

// NumPy's pairwise summation (np.add.reduce of a contiguous float64 array):
// fewer than 8 terms add in order, up to 128 terms use eight interleaved
// partial sums combined as ((r0+r1)+(r2+r3))+((r4+r5)+(r6+r7)) followed by
// the remainder, longer arrays split at n/2 rounded down to a multiple of 8.
__device__ double pairwise_sum(const double* a, int n) {
  if (n < 8) {
    double r = 0.0;
    for (int i = 0; i < n; ++i) r += a[i];
    return r;
  }
  if (n <= 128) {
    double r[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) r[j] = a[j];
    int i = 8;
    for (; i < n - (n % 8); i += 8)
#pragma unroll
      for (int j = 0; j < 8; ++j) r[j] += a[i + j];
    double res = ((r[0] + r[1]) + (r[2] + r[3])) + ((r[4] + r[5]) + (r[6] + r[7]));
    for (; i < n; ++i) res += a[i];
    return res;
  }
  int n2 = n / 2;
  n2 -= n2 % 8;
  return pairwise_sum(a, n2) + pairwise_sum(a + n2, n - n2);
}

__device__ __forceinline__ St4 interior_state(const DevGeom& g, const double* P, const double* recon, int f) {
  return recon ? ld4(recon + 4 * (size_t)g.ff_lslot[f]) : ld4(P + 4 * (size_t)g.ff_lcell[f]);
}

// outgoing invariant at Mach m: a0 / sqrt(1 + (gamma-1)/2 m^2) (dn m + 2/(gamma-1))
__device__ __forceinline__ double invariant_at(double m, double dn, double a0, double gamma) {
  const double ratio = 1.0 + 0.5 * (gamma - 1.0) * (m * m);
  const double sound = div_rn(a0, sqrt_rn(ratio));
  return sound * (dn * m + div_rn(2.0, gamma - 1.0));
}

__device__ void pressure_inlet(const DevGeom& g, const double* P, const double* recon, double gamma, double R,
                               int patch, double* ext) {
  const int base = g.seg_begin[SEG_BCX];
  const int j0 = g.bc_ptr[patch], j1 = g.bc_ptr[patch + 1];
  const double* v = g.bc_values + 4 * (size_t)patch;
  const double pt = v[0], tt = v[1], dx = v[2], dy = v[3];
  const double a0 = sqrt_rn(gamma * R * tt);
  for (int j = j0 + threadIdx.x; j < j1; j += blockDim.x) {
    const int f = base + j;
    const St4 q = interior_state(g, P, recon, f);
    const double2 n = g.ff_normal[f];
    const double dn = g.bc_dn[j];
    int bits = 0;
    if (dn >= -1e-12) bits |= MCFD_S_PIN_DIRECTION;
    const double c = sqrt_rn(div_rn(gamma * q.d, q.a));
    const double un = q.b * n.x + q.c * n.y;
    const double mach_in = div_rn(un, c);
    if (mach_in >= 1.0) bits |= MCFD_S_PIN_SUPERSONIC_OUT;
    if (mach_in <= -1.0) bits |= MCFD_S_PIN_SUPERSONIC_IN;
    const double outgoing = un + div_rn(2.0 * c, gamma - 1.0);
    if (!bits) {
      const double lo_v = invariant_at(0.0, dn, a0, gamma), hi_v = invariant_at(1.0, dn, a0, gamma);
      if (!(hi_v <= outgoing && outgoing <= lo_v)) bits |= MCFD_S_PIN_INCOMPATIBLE;
    }
    St4 out = q;
    if (!bits) {
      double low = 0.0, high = 1.0;
      for (int it = 0; it < 64; ++it) {
        const double mid = 0.5 * (low + high);
        if (invariant_at(mid, dn, a0, gamma) > outgoing) low = mid;
        else high = mid;
      }
      const double m = 0.5 * (low + high);
      const double t = div_rn(tt, 1.0 + 0.5 * (gamma - 1.0) * (m * m));
      const double p = pt * pow(div_rn(t, tt), div_rn(gamma, gamma - 1.0));
      const double rho = div_rn(p, R * t);
      const double speed = m * sqrt_rn(gamma * R * t);
      out = St4{rho, speed * dx, speed * dy, p};
      const bool finite = isfinite(out.a) && isfinite(out.b) && isfinite(out.c) && isfinite(out.d);
      if (!finite || !(rho > 0.0) || !(p > 0.0)) bits |= MCFD_S_PIN_STATE;
    }
    if (bits) flag_patch(g.status, bits, patch);
    st4(ext + 4 * (size_t)j, out);
  }
}

__device__ void mass_flow_inlet(const DevGeom& g, const double* P, const double* recon, double gamma, double R,
                                int patch, double* ext) {
  __shared__ int s_bad;
  __shared__ int s_below;
  const int base = g.seg_begin[SEG_BCX];
  const int j0 = g.bc_ptr[patch], j1 = g.bc_ptr[patch + 1], n = j1 - j0;
  const double* v = g.bc_values + 4 * (size_t)patch;
  const double mdot = v[0], tt = v[1], dx = v[2], dy = v[3];
  if (threadIdx.x == 0) s_bad = 0;
  __syncthreads();
  int bits = 0;
  for (int j = j0 + threadIdx.x; j < j1; j += blockDim.x) {
    const double proj = -g.bc_dn[j];
    if (proj <= 1e-12) bits |= MCFD_S_MFI_DIRECTION;
    const double p = interior_state(g, P, recon, base + j).d;
    if (p <= 0.0 || !isfinite(p)) bits |= MCFD_S_MFI_PRESSURE;
  }
  if (bits) {
    flag_patch(g.status, bits, patch);
    atomicOr(&s_bad, 1);
  }
  __syncthreads();
  const double cp = div_rn(gamma * R, gamma - 1.0);
  double speed = 0.0;
  if (!s_bad) {
    double* terms = g.bc_terms + j0;
    // flow_at(s) > or < the configured rate, decided by thread 0 for the block
    auto below = [&](double s) -> bool {
      const double rt = R * (tt - div_rn(s * s, 2.0 * cp));
      for (int j = j0 + threadIdx.x; j < j1; j += blockDim.x) {
        const St4 q = interior_state(g, P, recon, base + j);
        const double proj = -g.bc_dn[j];
        terms[j - j0] = div_rn(q.d, rt) * s * proj * g.ff_len[base + j];
      }
      __syncthreads();
      if (threadIdx.x == 0) s_below = (0.0 + pairwise_sum(terms, n)) < mdot;
      __syncthreads();
      const bool r = s_below != 0;
      __syncthreads();
      return r;
    };
    double low = 0.0, high = sqrt_rn(2.0 * cp * tt) * (1.0 - 1e-12);
    if (below(high)) {
      if (threadIdx.x == 0) flag_patch(g.status, MCFD_S_MFI_FLOW_RATE, patch);
    } else {
      for (int it = 0; it < 80; ++it) {
        const double mid = 0.5 * (low + high);
        if (below(mid)) low = mid;
        else high = mid;
      }
    }
    speed = 0.5 * (low + high);
  }
  const double rt = R * (tt - div_rn(speed * speed, 2.0 * cp));
  for (int j = j0 + threadIdx.x; j < j1; j += blockDim.x) {
    const St4 q = interior_state(g, P, recon, base + j);
    st4(ext + 4 * (size_t)j, St4{div_rn(q.d, rt), speed * dx, speed * dy, q.d});
  }
}

__device__ void mass_flow_outlet(const DevGeom& g, const double* P, const double* recon, int patch, double* ext) {
  const int base = g.seg_begin[SEG_BCX];
  const int j0 = g.bc_ptr[patch], j1 = g.bc_ptr[patch + 1];
  const double mdot = g.bc_values[4 * (size_t)patch], total_length = g.bc_values[4 * (size_t)patch + 1];
  for (int j = j0 + threadIdx.x; j < j1; j += blockDim.x) {
    const int f = base + j;
    const St4 q = interior_state(g, P, recon, f);
    if (q.a <= 0.0 || !isfinite(q.a)) flag_patch(g.status, MCFD_S_MFO_DENSITY, patch);
    const double2 n = g.ff_normal[f];
    const double vn = div_rn(mdot, total_length * q.a);
    const double tx = -n.y, ty = n.x;
    const double vt = q.b * tx + q.c * ty;
    st4(ext + 4 * (size_t)j, St4{q.a, vn * n.x + vt * tx, vn * n.y + vt * ty, q.d});
  }
}

__global__ void __launch_bounds__(kBlock) k_bc_states(DevGeom g, const double* __restrict__ P,
                                                      const double* __restrict__ recon, double gamma, double R,
                                                      double* __restrict__ ext) {
  const int patch = blockIdx.x;
  const int kind = g.bc_kind[patch];
  if (kind == MCFD_BC_PRESSURE_INLET) pressure_inlet(g, P, recon, gamma, R, patch, ext);
  else if (kind == MCFD_BC_MASS_FLOW_INLET) mass_flow_inlet(g, P, recon, gamma, R, patch, ext);
  else mass_flow_outlet(g, P, recon, patch, ext);
}

}  // namespace

cudaError_t launch_bc_states(const DevGeom& g, const mcfd_config& cfg, const double* P, const double* recon,
                             double* ext, cudaStream_t s) {
  if (g.n_bc_patches <= 0) return cudaSuccess;
  count_launch();
  k_bc_states<<<g.n_bc_patches, kBlock, 0, s>>>(g, P, recon, cfg.gamma, cfg.gas_constant, ext);
  return cudaGetLastError();
}

}  // namespace mcfd
