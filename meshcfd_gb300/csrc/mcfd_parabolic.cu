// MUSCL-parabolic reconstruction and the reference's reconstruction fields.
//
// _parabolic_reconstruction (solver.py:2322-2415), per cell (one thread):
//   * the stencil scale max(|dx|, |dy|) over the cell's two-ring entries;
//   * the weighted normal equations M (5x5) and right-hand sides B (5x4),
//     accumulated over the cell's entries in the reference's entry order
//     (np.add.at is sequential), weights 1 / max(|r/scale|^2, 1e-300);
//   * the rank gate np.linalg.matrix_rank(M) == 5: an LU with partial
//     pivoting gives the Frobenius condition number kappa_F = |M| |M^-1|;
//     below 1e12 the matrix is certainly of full rank (s_min / s_max >=
//     1 / kappa_F, far above the 5 eps threshold), otherwise one-sided
//     Jacobi singular values (Hestenes' method) and the rank rule decide;
//   * the solve by the same LU (row interchange to the first largest
//     |a_ik|, unit lower factor, right-looking); np.linalg.solve's LAPACK
//     gesv agrees to rounding (a few 1e-15 relative), not bit for bit;
//   * the limiter on the quadratic increment with two-ring extrema, or, for
//     cells that fail the gate, the linear gradient and limiter of
//     _limited_gradients (identical to the linear kernels, entry order kept).
// The face states are written per limiter slot as P + phi (G . r + the
// curvature term) in _reconstruct's order (solver.py:2418-2434).
//
// Compiled with -fmad=false: every product and sum rounds as the C oracle's
// restatement does, so the two agree bit for bit.
#include "mcfd_device.cuh"
#include "mcfd_internal.h"

namespace mcfd {
namespace {

constexpr int kBlock = 128;
constexpr double kEps = 2.220446049250313e-16;  // DBL_EPSILON

// Row interchange of rows k and p of a 5-column array with compile-time row
// indices only (the array stays in registers).
template <int K, int NC>
__device__ __forceinline__ void swap_rows(double (&A)[5][NC], int p) {
#pragma unroll
  for (int i = K + 1; i < 5; ++i) {
    if (p == i) {
#pragma unroll
      for (int j = 0; j < NC; ++j) {
        const double t = A[K][j];
        A[K][j] = A[i][j];
        A[i][j] = t;
      }
    }
  }
}

// Gaussian elimination with partial pivoting in place; false on a zero or
// non-finite pivot.
__device__ __forceinline__ bool lu5(double (&A)[5][5], int (&piv)[5]) {
  bool ok = true;
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    int p = k;
    double best = fabs(A[k][k]);
#pragma unroll
    for (int i = k + 1; i < 5; ++i) {
      const double a = fabs(A[i][k]);
      if (a > best) {
        best = a;
        p = i;
      }
    }
    piv[k] = p;
    if (!(best > 0.0) || !isfinite(best)) ok = false;
    if (!ok) return false;
    switch (k) {
      case 0: swap_rows<0, 5>(A, p); break;
      case 1: swap_rows<1, 5>(A, p); break;
      case 2: swap_rows<2, 5>(A, p); break;
      case 3: swap_rows<3, 5>(A, p); break;
      default: break;
    }
#pragma unroll
    for (int i = k + 1; i < 5; ++i) {
      const double l = div_rn(A[i][k], A[k][k]);
      A[i][k] = l;
#pragma unroll
      for (int j = k + 1; j < 5; ++j) A[i][j] = A[i][j] - l * A[k][j];
    }
  }
  return ok;
}

template <int M>
__device__ __forceinline__ void lu5_solve(const double (&LU)[5][5], const int (&piv)[5], double (&b)[5][M]) {
  swap_rows<0, M>(b, piv[0]);
  swap_rows<1, M>(b, piv[1]);
  swap_rows<2, M>(b, piv[2]);
  swap_rows<3, M>(b, piv[3]);
#pragma unroll
  for (int i = 1; i < 5; ++i)
#pragma unroll
    for (int j = 0; j < i; ++j)
#pragma unroll
      for (int v = 0; v < M; ++v) b[i][v] = b[i][v] - LU[i][j] * b[j][v];
#pragma unroll
  for (int i = 4; i >= 0; --i) {
#pragma unroll
    for (int j = i + 1; j < 5; ++j)
#pragma unroll
      for (int v = 0; v < M; ++v) b[i][v] = b[i][v] - LU[i][j] * b[j][v];
#pragma unroll
    for (int v = 0; v < M; ++v) b[i][v] = div_rn(b[i][v], LU[i][i]);
  }
}

// Singular values by one-sided Jacobi rotations; returns the rank by the
// rule of np.linalg.matrix_rank (s > max(s) * 5 * eps).
__device__ __noinline__ int jacobi_rank5(const double (&M)[5][5]) {
  double A[5][5];
#pragma unroll
  for (int i = 0; i < 5; ++i)
#pragma unroll
    for (int j = 0; j < 5; ++j) A[i][j] = M[i][j];
  for (int sweep = 0; sweep < 60; ++sweep) {
    bool rotated = false;
#pragma unroll
    for (int p = 0; p < 4; ++p)
#pragma unroll
      for (int q = p + 1; q < 5; ++q) {
        double alpha = 0.0, beta = 0.0, gam = 0.0;
#pragma unroll
        for (int i = 0; i < 5; ++i) {
          alpha += A[i][p] * A[i][p];
          beta += A[i][q] * A[i][q];
          gam += A[i][p] * A[i][q];
        }
        if (!(fabs(gam) > 1e-15 * sqrt_rn(alpha * beta))) continue;
        rotated = true;
        const double zeta = div_rn(beta - alpha, 2.0 * gam);
        const double t = fabs(zeta) > 1e150 ? div_rn(0.5, zeta)
                                            : div_rn(copysign(1.0, zeta), fabs(zeta) + sqrt_rn(1.0 + zeta * zeta));
        const double c = div_rn(1.0, sqrt_rn(1.0 + t * t)), sn = c * t;
#pragma unroll
        for (int i = 0; i < 5; ++i) {
          const double ap = A[i][p], aq = A[i][q];
          A[i][p] = c * ap - sn * aq;
          A[i][q] = sn * ap + c * aq;
        }
      }
    if (!rotated) break;
  }
  double sv[5], smax = 0.0;
#pragma unroll
  for (int j = 0; j < 5; ++j) {
    double n2 = 0.0;
#pragma unroll
    for (int i = 0; i < 5; ++i) n2 += A[i][j] * A[i][j];
    sv[j] = sqrt_rn(n2);
    if (sv[j] > smax) smax = sv[j];
  }
  int rank = 0;
#pragma unroll
  for (int j = 0; j < 5; ++j)
    if (sv[j] > smax * 5.0 * kEps) ++rank;
  return rank;
}

__device__ __forceinline__ bool full_rank5(const double (&M)[5][5], const double (&LU)[5][5], const int (&piv)[5],
                                           bool lu_ok) {
  if (lu_ok) {
    double X[5][5];
#pragma unroll
    for (int i = 0; i < 5; ++i)
#pragma unroll
      for (int j = 0; j < 5; ++j) X[i][j] = i == j ? 1.0 : 0.0;
    lu5_solve<5>(LU, piv, X);
    double na = 0.0, ni = 0.0;
#pragma unroll
    for (int i = 0; i < 5; ++i)
#pragma unroll
      for (int j = 0; j < 5; ++j) {
        na += M[i][j] * M[i][j];
        ni += X[i][j] * X[i][j];
      }
    const double kappa = sqrt_rn(na) * sqrt_rn(ni);
    if (isfinite(kappa) && kappa < 1e12) return true;
  }
  return jacobi_rank5(M) == 5;
}

// Linear gradient and limiter factors of one cell (_kernels.py:240-273 and
// 10-67), the same arithmetic as the exact linear kernel.
template <int LIMITER>
__device__ __forceinline__ void linear_cell(const DevGeom& g, const double* __restrict__ P, int c,
                                            const double (&pv)[4], double (&gx)[4], double (&gy)[4],
                                            double (&phi)[4]) {
  double lo[4], hi[4];
#pragma unroll
  for (int v = 0; v < 4; ++v) {
    gx[v] = gy[v] = 0.0;
    lo[v] = hi[v] = pv[v];
    phi[v] = 1.0;
  }
  const int e0 = g.grad_ptr[c], e1 = g.grad_ptr[c + 1];
  for (int e = e0; e < e1; ++e) {
    const St4 q = ld4(P + 4 * (size_t)g.grad_nb[e]);
    const double qv[4] = {q.a, q.b, q.c, q.d};
    const double cx = g.grad_cx[e], cy = g.grad_cy[e];
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const double d = qv[v] - pv[v];
      gx[v] = gx[v] + cx * d;
      gy[v] = gy[v] + cy * d;
      if (icmp::lt(qv[v], lo[v])) lo[v] = qv[v];
      if (icmp::lt(hi[v], qv[v])) hi[v] = qv[v];
    }
  }
  if (g.n_gradient == 0) return;  // _limited_gradients: zeros and ones (solver.py:2298-2302)
  const int s0 = g.lim_ptr[c], s1 = g.lim_ptr[c + 1];
  for (int s = s0; s < s1; ++s) {
    const double2 d = g.lim_d[s];
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const double inc = gx[v] * d.x + gy[v] * d.y;
      const double f = limiter_face_factor<LIMITER>(pv[v], inc, lo[v], hi[v], limiter_tolerance(pv[v]));
      if (icmp::lt_nonneg(f, phi[v])) phi[v] = f;
    }
  }
}

template <int LIMITER, bool PARABOLIC, bool FIELDS>
__global__ void __launch_bounds__(kBlock) k_reconstruct_full(DevGeom g, const double* __restrict__ P,
                                                             double* __restrict__ recon, double* __restrict__ grad_out,
                                                             double* __restrict__ curv_out,
                                                             double* __restrict__ fac_out) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= g.n_cells) return;
  const St4 p = ld4(P + 4 * (size_t)c);
  const double pv[4] = {p.a, p.b, p.c, p.d};
  double gx[4], gy[4], kxx[4] = {0, 0, 0, 0}, kxy[4] = {0, 0, 0, 0}, kyy[4] = {0, 0, 0, 0}, phi[4];
  bool full = false;
  if (PARABOLIC && g.n_parabolic > 0) {
    const int e0 = g.par_ptr[c], e1 = g.par_ptr[c + 1];
    double scale = 0.0;
    for (int e = e0; e < e1; ++e) {
      const double2 d = g.par_d[e];
      const double a = fabs(d.x), b = fabs(d.y);
      const double m = a >= b ? a : b;
      if (m > scale) scale = m;
    }
    if (!(scale >= 1e-300)) scale = 1e-300;
    double M[5][5], B[5][4], lo[4], hi[4];
#pragma unroll
    for (int i = 0; i < 5; ++i) {
#pragma unroll
      for (int j = 0; j < 5; ++j) M[i][j] = 0.0;
#pragma unroll
      for (int v = 0; v < 4; ++v) B[i][v] = 0.0;
    }
#pragma unroll
    for (int v = 0; v < 4; ++v) lo[v] = hi[v] = pv[v];
    for (int e = e0; e < e1; ++e) {
      const double2 d = g.par_d[e];
      const double nx = div_rn(d.x, scale), ny = div_rn(d.y, scale);
      const double dd[5] = {nx, ny, 0.5 * (nx * nx), nx * ny, 0.5 * (ny * ny)};
      const double r2 = nx * nx + ny * ny;
      const double w = div_rn(1.0, r2 >= 1e-300 ? r2 : 1e-300);
      const St4 q = ld4(P + 4 * (size_t)g.par_nb[e]);
      const double qv[4] = {q.a, q.b, q.c, q.d};
      double diff[4];
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        diff[v] = qv[v] - pv[v];
        if (icmp::lt(qv[v], lo[v])) lo[v] = qv[v];
        if (icmp::lt(hi[v], qv[v])) hi[v] = qv[v];
      }
#pragma unroll
      for (int i = 0; i < 5; ++i) {
        const double wi = w * dd[i];
#pragma unroll
        for (int j = 0; j < 5; ++j) M[i][j] += wi * dd[j];
#pragma unroll
        for (int v = 0; v < 4; ++v) B[i][v] += wi * diff[v];
      }
    }
    double LU[5][5];
#pragma unroll
    for (int i = 0; i < 5; ++i)
#pragma unroll
      for (int j = 0; j < 5; ++j) LU[i][j] = M[i][j];
    int piv[5] = {0, 1, 2, 3, 4};
    const bool ok = lu5(LU, piv);
    full = full_rank5(M, LU, piv, ok);
    if (full) {
      lu5_solve<4>(LU, piv, B);
      const double sc = scale, sc2 = scale * scale;
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        gx[v] = div_rn(B[0][v], sc);
        gy[v] = div_rn(B[1][v], sc);
        kxx[v] = div_rn(B[2][v], sc2);
        kxy[v] = div_rn(B[3][v], sc2);
        kyy[v] = div_rn(B[4][v], sc2);
        phi[v] = 1.0;
      }
      const int s0 = g.lim_ptr[c], s1 = g.lim_ptr[c + 1];
      for (int s = s0; s < s1; ++s) {
        const double2 d = g.lim_d[s];
#pragma unroll
        for (int v = 0; v < 4; ++v) {
          const double inc = gx[v] * d.x + gy[v] * d.y + 0.5 * kxx[v] * (d.x * d.x) + kxy[v] * (d.x * d.y) +
                             0.5 * kyy[v] * (d.y * d.y);
          const double f = limiter_face_factor<LIMITER>(pv[v], inc, lo[v], hi[v], limiter_tolerance(pv[v]));
          if (f < phi[v]) phi[v] = f;
        }
      }
    }
  }
  if (!full) linear_cell<LIMITER>(g, P, c, pv, gx, gy, phi);
  if (FIELDS) {
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      grad_out[8 * (size_t)c + 2 * v] = gx[v];
      grad_out[8 * (size_t)c + 2 * v + 1] = gy[v];
      fac_out[4 * (size_t)c + v] = phi[v];
      if (curv_out) {
        curv_out[12 * (size_t)c + 3 * v] = kxx[v];
        curv_out[12 * (size_t)c + 3 * v + 1] = kxy[v];
        curv_out[12 * (size_t)c + 3 * v + 2] = kyy[v];
      }
    }
    return;
  }
  const int s0 = g.lim_ptr[c], s1 = g.lim_ptr[c + 1];
  for (int s = s0; s < s1; ++s) {
    const double2 d = g.lim_d[s];
    double out[4];
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      double inc = gx[v] * d.x + gy[v] * d.y;
      if (PARABOLIC) inc += 0.5 * kxx[v] * (d.x * d.x) + kxy[v] * (d.x * d.y) + 0.5 * kyy[v] * (d.y * d.y);
      out[v] = pv[v] + phi[v] * inc;
    }
    st4(recon + 4 * (size_t)g.lim_slot[s], St4{out[0], out[1], out[2], out[3]});
  }
}

inline int blocks_for(int n) { return (n + kBlock - 1) / kBlock; }

template <bool PARABOLIC, bool FIELDS>
cudaError_t launch_full(const DevGeom& g, int limiter, const double* P, double* recon, double* grad, double* curv,
                        double* fac, cudaStream_t s) {
  if (g.n_cells == 0) return cudaSuccess;
  const int b = blocks_for(g.n_cells);
  count_launch();
  switch (limiter) {
    case 0: k_reconstruct_full<0, PARABOLIC, FIELDS><<<b, kBlock, 0, s>>>(g, P, recon, grad, curv, fac); break;
    case 1: k_reconstruct_full<1, PARABOLIC, FIELDS><<<b, kBlock, 0, s>>>(g, P, recon, grad, curv, fac); break;
    case 2: k_reconstruct_full<2, PARABOLIC, FIELDS><<<b, kBlock, 0, s>>>(g, P, recon, grad, curv, fac); break;
    default: k_reconstruct_full<3, PARABOLIC, FIELDS><<<b, kBlock, 0, s>>>(g, P, recon, grad, curv, fac); break;
  }
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_reconstruct_parabolic(const DevGeom& g, const mcfd_config& cfg, const double* P, double* recon,
                                         cudaStream_t s) {
  return launch_full<true, false>(g, cfg.limiter, P, recon, nullptr, nullptr, nullptr, s);
}

cudaError_t launch_reconstruction_fields(const DevGeom& g, const mcfd_config& cfg, const double* P, double* grad,
                                         double* curv, double* fac, cudaStream_t s) {
  if (cfg.reconstruction == MCFD_RECON_MUSCL_PARABOLIC)
    return launch_full<true, true>(g, cfg.limiter, P, nullptr, grad, curv, fac, s);
  return launch_full<false, true>(g, cfg.limiter, P, nullptr, grad, curv, fac, s);
}

}  // namespace mcfd
