/*
 * ORACLE — test infrastructure only; never part of the product path.
 *
 * A CPU restatement, in plain C, of the reference's residual / time-step hot
 * path (jesuspueblas/meshcfd, src/meshcfd/core).  It follows the reference's
 * own loop structure: the compiled kernels' global entry loops
 * (_kernels.py), the SciPy CSR divergence product, and the sequential
 * np.add.at scatters per boundary group, in the order _residual runs them.
 * It shares no code with the CUDA path.  Compile with -ffp-contract=off (no
 * FMA contraction; NumPy's elementwise ops round every product).
 *
 * Parity is pinned: tests/golden holds residuals, time steps and explicit
 * steps produced by the reference itself, and the CPU tests check this file
 * against them bit for bit.
 */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORC_NONPHYSICAL 0x01
#define ORC_NONFINITE_RESIDUAL 0x02
#define ORC_HLLC_NONFINITE 0x04
#define ORC_ROE_SOUND 0x08
#define ORC_ROE_NONFINITE 0x10
#define ORC_FARFIELD_SOUND 0x20
#define ORC_FARFIELD_STATE 0x40
#define ORC_TIME_STEP 0x80
#define ORC_PIN_DIRECTION 0x100
#define ORC_PIN_SUPERSONIC_OUT 0x200
#define ORC_PIN_SUPERSONIC_IN 0x400
#define ORC_PIN_INCOMPATIBLE 0x800
#define ORC_PIN_STATE 0x1000
#define ORC_MFI_DIRECTION 0x2000
#define ORC_MFI_PRESSURE 0x4000
#define ORC_MFI_FLOW_RATE 0x8000
#define ORC_MFO_DENSITY 0x10000
#define ORC_ARG 0x1000

typedef struct {
  int64_t n_cells, n_faces;
  const double *centers, *areas, *face_centers, *face_normals, *face_lengths, *wall_velocities;
  const int64_t *owners, *neighbours;
  int64_t n_interior;
  const int64_t* interior_faces;
  const double *interior_owner_offsets, *interior_neighbour_offsets;
  int64_t n_periodic;
  const int64_t *periodic_faces_a, *periodic_faces_b;
  int64_t n_wall;
  const int64_t* wall_faces;
  int64_t n_vin;
  const int64_t* vin_faces;
  const double* vin_states;
  int64_t n_pout;
  const int64_t* pout_faces;
  const double* pout_pressures;
  int64_t n_far;
  const int64_t* far_faces;
  const double* far_states;
  int64_t n_gradient;
  const int64_t *gradient_sources, *gradient_neighbours;
  const double *gradient_cx, *gradient_cy;
  int64_t n_limiter;
  const int64_t* limiter_cells;
  const double *limiter_dx, *limiter_dy;
  int64_t n_parabolic; /* two-ring stencil entries, source-major (solver.py:2241-2291) */
  const int64_t *parabolic_sources, *parabolic_neighbours;
  const double *parabolic_dx, *parabolic_dy;
  /* pressure-inlet (0), mass-flow-inlet (1), mass-flow-outlet (2) patches in
   * the reference's order; values per patch: (total p, total T, dir x, dir y)
   * / (mass flow, total T, dir x, dir y) / (mass flow, sum of lengths, 0, 0);
   * bc_dn: NumPy's normals @ direction per face */
  int64_t n_bc_patches;
  const int32_t* bc_kind;
  const double* bc_values;
  const int64_t *bc_offsets, *bc_faces;
  const double* bc_dn;
} orc_geom;

typedef struct {
  int32_t flux, reconstruction, limiter, pad;
  double gamma, acceleration_x, acceleration_y, cfl, gas_constant;
  double venkat_k; /* K of limiter code 4 */
} orc_settings;

/* ------------------------------------------------------------ euler.py */

/* euler.conservative_to_primitive (euler.py:20-40) */
int orc_conservative_to_primitive(int64_t n, const double* U, double gamma, double* P) {
  int bad = 0;
  for (int64_t i = 0; i < n; ++i) {
    const double* u = U + 4 * i;
    double rho = u[0];
    double vx = u[1] / rho, vy = u[2] / rho;
    double p = (gamma - 1.0) * (u[3] - 0.5 * (u[1] * u[1] + u[2] * u[2]) / rho);
    P[4 * i] = rho;
    P[4 * i + 1] = vx;
    P[4 * i + 2] = vy;
    P[4 * i + 3] = p;
    if (!isfinite(rho) || !isfinite(vx) || !isfinite(vy) || !isfinite(p) || rho <= 0.0 || p <= 0.0)
      bad = ORC_NONPHYSICAL;
  }
  return bad;
}

/* euler.primitive_to_conservative (euler.py:8-17) */
void orc_primitive_to_conservative(int64_t n, const double* P, double gamma, double* U) {
  for (int64_t i = 0; i < n; ++i) {
    const double* q = P + 4 * i;
    U[4 * i] = q[0];
    U[4 * i + 1] = q[0] * q[1];
    U[4 * i + 2] = q[0] * q[2];
    U[4 * i + 3] = q[3] / (gamma - 1.0) + 0.5 * q[0] * (q[1] * q[1] + q[2] * q[2]);
  }
}

/* euler.physical_flux (euler.py:43-57), one row */
static void physical_flux(const double* q, const double* n, double gamma, double* F, double* U) {
  double rho = q[0], vx = q[1], vy = q[2], p = q[3];
  U[0] = rho;
  U[1] = rho * vx;
  U[2] = rho * vy;
  U[3] = p / (gamma - 1.0) + 0.5 * rho * (vx * vx + vy * vy);
  double un = vx * n[0] + vy * n[1];
  F[0] = rho * un;
  F[1] = rho * vx * un + p * n[0];
  F[2] = rho * vy * un + p * n[1];
  F[3] = (U[3] + p) * un;
}

static double sound(const double* q, double gamma) { return sqrt(gamma * q[3] / q[0]); }

/* euler._rusanov_flux (euler.py:80-93) */
static int rusanov(const double* L, const double* R, const double* n, double gamma, double* out) {
  double FL[4], UL[4], FR[4], UR[4];
  physical_flux(L, n, gamma, FL, UL);
  physical_flux(R, n, gamma, FR, UR);
  double nl = L[1] * n[0] + L[2] * n[1], nr = R[1] * n[0] + R[2] * n[1];
  double a = fabs(nl) + sound(L, gamma), b = fabs(nr) + sound(R, gamma);
  double s = a >= b ? a : b;
  for (int k = 0; k < 4; ++k) out[k] = 0.5 * (FL[k] + FR[k] - s * (UR[k] - UL[k]));
  return 0;
}

/* star state of euler._hllc_flux (euler.py:122-148) */
static void hllc_star(const double* q, const double* U, double un, double wave, double contact,
                      const double* n, double* star) {
  double factor = q[0] * (wave - un) / (wave - contact);
  double vx = q[1] + (contact - un) * n[0];
  double vy = q[2] + (contact - un) * n[1];
  double energy = factor * (U[3] / q[0] + (contact - un) * (contact + q[3] / (q[0] * (wave - un))));
  star[0] = factor;
  star[1] = factor * vx;
  star[2] = factor * vy;
  star[3] = energy;
}

/* euler._hllc_flux (euler.py:96-166), vectorised form's selection */
static int hllc_numpy(const double* L, const double* R, const double* n, double gamma, double* out) {
  double FL[4], UL[4], FR[4], UR[4];
  physical_flux(L, n, gamma, FL, UL);
  physical_flux(R, n, gamma, FR, UR);
  double unl = L[1] * n[0] + L[2] * n[1], unr = R[1] * n[0] + R[2] * n[1];
  double cl = sound(L, gamma), cr = sound(R, gamma);
  double a = unl - cl, b = unr - cr;
  double wl = b < a ? b : a;
  a = unl + cl;
  b = unr + cr;
  double wr = b > a ? b : a;
  double den = L[0] * (wl - unl) - R[0] * (wr - unr);
  double safe = fabs(den) > 1e-14 ? den : copysign(1e-14, den);
  double contact = (R[3] - L[3] + L[0] * unl * (wl - unl) - R[0] * unr * (wr - unr)) / safe;
  double star[4];
  if (wl >= 0.0) {
    for (int k = 0; k < 4; ++k) out[k] = FL[k];
  } else if (contact >= 0.0) {
    hllc_star(L, UL, unl, wl, contact, n, star);
    for (int k = 0; k < 4; ++k) out[k] = FL[k] + wl * (star[k] - UL[k]);
  } else if (wr > 0.0) {
    hllc_star(R, UR, unr, wr, contact, n, star);
    for (int k = 0; k < 4; ++k) out[k] = FR[k] + wr * (star[k] - UR[k]);
  } else {
    for (int k = 0; k < 4; ++k) out[k] = FR[k];
  }
  for (int k = 0; k < 4; ++k)
    if (!isfinite(out[k])) return ORC_HLLC_NONFINITE;
  return 0;
}

/* euler._roe_flux (euler.py:169-262); np.einsum's four-term reduction on the
 * reference's platform adds (t0 + t2) + (t1 + t3). */
static int roe(const double* L, const double* R, const double* n, double gamma, double* out) {
  double FL[4], UL[4], FR[4], UR[4];
  physical_flux(L, n, gamma, FL, UL);
  physical_flux(R, n, gamma, FR, UR);
  double rl = sqrt(L[0]), rr = sqrt(R[0]);
  double den = rl + rr;
  double vx = (rl * L[1] + rr * R[1]) / den;
  double vy = (rl * L[2] + rr * R[2]) / den;
  double H = (rl * (L[3] / L[0] + 0.5 * (L[1] * L[1] + L[2] * L[2])) +
              rr * (R[3] / R[0] + 0.5 * (R[1] * R[1] + R[2] * R[2]))) / den;
  double un = vx * n[0] + vy * n[1];
  double ut = vx * -n[1] + vy * n[0];
  double c2 = (gamma - 1.0) * (H - 0.5 * (vx * vx + vy * vy));
  if (c2 <= 0.0 || !isfinite(c2)) return ORC_ROE_SOUND;
  double c = sqrt(c2), ravg = rl * rr;
  double unl = L[1] * n[0] + L[2] * n[1], unr = R[1] * n[0] + R[2] * n[1];
  double utl = L[1] * -n[1] + L[2] * n[0], utr = R[1] * -n[1] + R[2] * n[0];
  double dr = R[0] - L[0], dun = unr - unl, dut = utr - utl, dp = R[3] - L[3];
  double s[4];
  s[0] = (dp - ravg * c * dun) / (2.0 * c2);
  s[3] = (dp + ravg * c * dun) / (2.0 * c2);
  s[1] = dr - dp / c2;
  s[2] = ravg * dut;
  double lam[4] = {un - c, un, un, un + c};
  double fix = 0.1 * c, w[4];
  for (int j = 0; j < 4; ++j) {
    double a = fabs(lam[j]);
    if (a < fix) a = 0.5 * (a * a / fix + fix);
    w[j] = a * s[j];
  }
  double E[4][4] = {{1.0, 1.0, 0.0, 1.0},
                    {un - c, un, 0.0, un + c},
                    {ut, ut, 1.0, ut},
                    {H - un * c, 0.5 * (un * un + ut * ut), ut, H + un * c}};
  double d[4];
  for (int i = 0; i < 4; ++i) {
    double t0 = E[i][0] * w[0], t1 = E[i][1] * w[1], t2 = E[i][2] * w[2], t3 = E[i][3] * w[3];
    d[i] = (t0 + t2) + (t1 + t3);
  }
  double diss[4] = {d[0], d[1] * n[0] - d[2] * n[1], d[1] * n[1] + d[2] * n[0], d[3]};
  for (int k = 0; k < 4; ++k) {
    out[k] = 0.5 * (FL[k] + FR[k] - diss[k]);
    if (!isfinite(out[k])) return ORC_ROE_NONFINITE;
  }
  return 0;
}

/* euler.numerical_flux (euler.py:60-73) */
static int numerical_flux(int scheme, const double* L, const double* R, const double* n, double gamma,
                          double* out) {
  if (scheme == 0) return rusanov(L, R, n, gamma, out);
  if (scheme == 1) return hllc_numpy(L, R, n, gamma, out);
  return roe(L, R, n, gamma, out);
}

/* ------------------------------------------------------------ _kernels.py */

/* limited_gradient_factors (_kernels.py:10-67) */
/* code 4: Venkatakrishnan's limiter in its published form with the smoothing
 * constant K (J. Comput. Phys. 118, 120-130, 1995), an extension with no
 * counterpart in the reference: per face, d2 = grad . r, d1 = max - v
 * (d2 > 0) or min - v (d2 <= 0), e2 = (K sqrt(A))^3,
 * f = (d1^2 + e2 + 2 d1 d2) / (d1^2 + 2 d2^2 + d1 d2 + e2), and the cell
 * factor is the least f over its faces (no cap at 1). */
static double venkat_k_face(double v, double inc, double lo, double hi, double e2) {
  const double d1 = inc > 0.0 ? hi - v : lo - v;
  const double d1d1 = d1 * d1, d12 = d1 * inc;
  const double num = (d1d1 + e2) + (d12 + d12);
  const double den = ((d1d1 + 2.0 * (inc * inc)) + d12) + e2;
  return num / den;
}

static void limited_gradient_factors(int64_t C, const double* P, const double* grad, const orc_geom* g,
                                     int code, double venkat_k, double* factors) {
  double* lo = (double*)malloc(sizeof(double) * 4 * C);
  double* hi = (double*)malloc(sizeof(double) * 4 * C);
  memcpy(lo, P, sizeof(double) * 4 * C);
  memcpy(hi, P, sizeof(double) * 4 * C);
  for (int64_t i = 0; i < 4 * C; ++i) factors[i] = code == 4 ? INFINITY : 1.0;
  for (int64_t e = 0; e < g->n_gradient; ++e) {
    int64_t s = g->gradient_sources[e], nb = g->gradient_neighbours[e];
    for (int v = 0; v < 4; ++v) {
      double value = P[4 * nb + v];
      if (value < lo[4 * s + v]) lo[4 * s + v] = value;
      if (value > hi[4 * s + v]) hi[4 * s + v] = value;
    }
  }
  for (int64_t e = 0; e < g->n_limiter; ++e) {
    int64_t c = g->limiter_cells[e];
    double dx = g->limiter_dx[e], dy = g->limiter_dy[e];
    if (code == 4) {
      const double t = venkat_k * sqrt(g->areas[c]);
      const double e2 = (t * t) * t;
      for (int v = 0; v < 4; ++v) {
        const double cv = P[4 * c + v];
        const double inc = grad[8 * c + 2 * v] * dx + grad[8 * c + 2 * v + 1] * dy;
        const double f = venkat_k_face(cv, inc, lo[4 * c + v], hi[4 * c + v], e2);
        if (f < factors[4 * c + v]) factors[4 * c + v] = f;
      }
      continue;
    }
    for (int v = 0; v < 4; ++v) {
      double cv = P[4 * c + v];
      double inc = grad[8 * c + 2 * v] * dx + grad[8 * c + 2 * v + 1] * dy;
      double m = fabs(cv);
      double tol = 1e-14 * (1.0 > m ? 1.0 : m);
      double ratio = 1.0;
      if (inc > tol) ratio = (hi[4 * c + v] - cv) / inc;
      else if (inc < -tol) ratio = (lo[4 * c + v] - cv) / inc;
      ratio = 0.0 > ratio ? 0.0 : ratio;
      double f;
      if (code <= 1) f = 1.0 < ratio ? 1.0 : ratio;
      else if (code == 2) {
        if (ratio > 0.0) {
          double q = 2.0 * ratio / (1.0 + ratio);
          f = q < 1.0 ? q : 1.0;
        } else f = 0.0;
      } else {
        double eps = 1e-12;
        f = (ratio * ratio + 2.0 * ratio + eps) / (ratio * ratio + ratio + 2.0 + eps);
        f = 1.0 < f ? 1.0 : f;
      }
      if (f < factors[4 * c + v]) factors[4 * c + v] = f;
    }
  }
  free(lo);
  free(hi);
}

/* linear_gradients_and_factors (_kernels.py:240-273); grad is (C,4,2) */
void orc_linear_gradients_and_factors(const orc_geom* g, const double* P, int code, double venkat_k, double* grad,
                                      double* factors) {
  int64_t C = g->n_cells;
  memset(grad, 0, sizeof(double) * 8 * C);
  for (int64_t e = 0; e < g->n_gradient; ++e) {
    int64_t s = g->gradient_sources[e], nb = g->gradient_neighbours[e];
    double cx = g->gradient_cx[e], cy = g->gradient_cy[e];
    for (int v = 0; v < 4; ++v) {
      double d = P[4 * nb + v] - P[4 * s + v];
      grad[8 * s + 2 * v] += cx * d;
      grad[8 * s + 2 * v + 1] += cy * d;
    }
  }
  limited_gradient_factors(C, P, grad, g, code, venkat_k, factors);
}

/* reconstruct_hllc_flux (_kernels.py:71-160), one face */
static void kernel_hllc(const double* left, const double* right, const double* n, double gamma,
                        double* out) {
  double rl = left[0], vxl = left[1], vyl = left[2], pl = left[3];
  double rr = right[0], vxr = right[1], vyr = right[2], pr = right[3];
  double nx = n[0], ny = n[1];
  double unl = vxl * nx + vyl * ny, unr = vxr * nx + vyr * ny;
  double cl = sqrt(gamma * pl / rl), cr = sqrt(gamma * pr / rr);
  double a = unl - cl, b = unr - cr;
  double wl = b < a ? b : a;
  a = unl + cl;
  b = unr + cr;
  double wr = b > a ? b : a;
  double el = pl / (gamma - 1.0) + 0.5 * rl * (vxl * vxl + vyl * vyl);
  double er = pr / (gamma - 1.0) + 0.5 * rr * (vxr * vxr + vyr * vyr);
  double sl[4] = {rl, rl * vxl, rl * vyl, el}, sr[4] = {rr, rr * vxr, rr * vyr, er};
  double fl[4] = {rl * unl, rl * vxl * unl + pl * nx, rl * vyl * unl + pl * ny, (el + pl) * unl};
  double fr[4] = {rr * unr, rr * vxr * unr + pr * nx, rr * vyr * unr + pr * ny, (er + pr) * unr};
  double den = rl * (wl - unl) - rr * (wr - unr);
  if (fabs(den) <= 1e-14) den = copysign(1e-14, den);
  double contact = (pr - pl + rl * unl * (wl - unl) - rr * unr * (wr - unr)) / den;
  if (wl >= 0.0) {
    for (int k = 0; k < 4; ++k) out[k] = fl[k];
    return;
  }
  if (wr <= 0.0) {
    for (int k = 0; k < 4; ++k) out[k] = fr[k];
    return;
  }
  double rho, vx, vy, pressure, un, wave, energy;
  const double *state, *phys;
  if (contact >= 0.0) {
    rho = rl; vx = vxl; vy = vyl; pressure = pl; un = unl; wave = wl; energy = el; state = sl; phys = fl;
  } else {
    rho = rr; vx = vxr; vy = vyr; pressure = pr; un = unr; wave = wr; energy = er; state = sr; phys = fr;
  }
  double factor = rho * (wave - un) / (wave - contact);
  double svx = vx + (contact - un) * nx, svy = vy + (contact - un) * ny;
  double se = factor * (energy / rho + (contact - un) * (contact + pressure / (rho * (wave - un))));
  double star[4] = {factor, factor * svx, factor * svy, se};
  for (int k = 0; k < 4; ++k) out[k] = phys[k] + wave * (star[k] - state[k]);
}

/* ------------------------------------------------------------ solver.py */

/* _reconstruct (solver.py:2418-2434), one row; curv (C,4,3) or NULL */
static void reconstruct(const double* P, const double* grad, const double* fac, const double* curv, int64_t c,
                        double ox, double oy, double* out) {
  for (int v = 0; v < 4; ++v) {
    double inc = grad[8 * c + 2 * v] * ox + grad[8 * c + 2 * v + 1] * oy;
    if (curv) {
      const double* k = curv + 12 * c + 3 * v;
      inc += 0.5 * k[0] * (ox * ox) + k[1] * (ox * oy) + 0.5 * k[2] * (oy * oy);
    }
    out[v] = P[4 * c + v] + fac[4 * c + v] * inc;
  }
}

/* ---------------------------------------------- _parabolic_reconstruction */

/* Gaussian elimination with partial pivoting (row interchange to the first
 * largest |a_ik|, unit lower factor): the factorisation LAPACK's gesv uses
 * behind np.linalg.solve, in plain right-looking order.  Returns 0 on a zero
 * or non-finite pivot. */
static int lu5(double A[5][5], int piv[5]) {
  for (int k = 0; k < 5; ++k) {
    int p = k;
    double best = fabs(A[k][k]);
    for (int i = k + 1; i < 5; ++i)
      if (fabs(A[i][k]) > best) {
        best = fabs(A[i][k]);
        p = i;
      }
    piv[k] = p;
    if (!(best > 0.0) || !isfinite(best)) return 0;
    if (p != k)
      for (int j = 0; j < 5; ++j) {
        double t = A[k][j];
        A[k][j] = A[p][j];
        A[p][j] = t;
      }
    for (int i = k + 1; i < 5; ++i) {
      double l = A[i][k] / A[k][k];
      A[i][k] = l;
      for (int j = k + 1; j < 5; ++j) A[i][j] = A[i][j] - l * A[k][j];
    }
  }
  return 1;
}

/* b: [5][m] right-hand sides, overwritten with the solution. */
static void lu5_solve(double LU[5][5], const int piv[5], double* b, int m) {
  for (int k = 0; k < 5; ++k)
    if (piv[k] != k)
      for (int v = 0; v < m; ++v) {
        double t = b[k * m + v];
        b[k * m + v] = b[piv[k] * m + v];
        b[piv[k] * m + v] = t;
      }
  for (int i = 1; i < 5; ++i)
    for (int j = 0; j < i; ++j)
      for (int v = 0; v < m; ++v) b[i * m + v] = b[i * m + v] - LU[i][j] * b[j * m + v];
  for (int i = 4; i >= 0; --i) {
    for (int j = i + 1; j < 5; ++j)
      for (int v = 0; v < m; ++v) b[i * m + v] = b[i * m + v] - LU[i][j] * b[j * m + v];
    for (int v = 0; v < m; ++v) b[i * m + v] = b[i * m + v] / LU[i][i];
  }
}

/* Singular values by one-sided Jacobi rotations (Hestenes' method), then
 * the rank rule of np.linalg.matrix_rank: count of s > max(s) * 5 * eps. */
static int jacobi_rank5(const double M[5][5]) {
  double A[5][5];
  memcpy(A, M, sizeof(A));
  for (int sweep = 0; sweep < 60; ++sweep) {
    int rotated = 0;
    for (int p = 0; p < 4; ++p)
      for (int q = p + 1; q < 5; ++q) {
        double alpha = 0.0, beta = 0.0, gam = 0.0;
        for (int i = 0; i < 5; ++i) {
          alpha += A[i][p] * A[i][p];
          beta += A[i][q] * A[i][q];
          gam += A[i][p] * A[i][q];
        }
        if (!(fabs(gam) > 1e-15 * sqrt(alpha * beta))) continue;
        rotated = 1;
        double zeta = (beta - alpha) / (2.0 * gam);
        double t = fabs(zeta) > 1e150 ? 0.5 / zeta
                                      : copysign(1.0, zeta) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
        double c = 1.0 / sqrt(1.0 + t * t), sn = c * t;
        for (int i = 0; i < 5; ++i) {
          double ap = A[i][p], aq = A[i][q];
          A[i][p] = c * ap - sn * aq;
          A[i][q] = sn * ap + c * aq;
        }
      }
    if (!rotated) break;
  }
  double sv[5], smax = 0.0;
  for (int j = 0; j < 5; ++j) {
    double n2 = 0.0;
    for (int i = 0; i < 5; ++i) n2 += A[i][j] * A[i][j];
    sv[j] = sqrt(n2);
    if (sv[j] > smax) smax = sv[j];
  }
  int rank = 0;
  for (int j = 0; j < 5; ++j)
    if (sv[j] > smax * 5.0 * DBL_EPSILON) ++rank;
  return rank;
}

/* np.linalg.matrix_rank(M) == 5, decided without an SVD where the LU shows a
 * Frobenius condition number kappa_F = |M|_F |M^-1|_F below 1e12: then
 * s_min / s_max >= 1 / kappa_F is far above the 5 eps threshold.  Otherwise
 * (singular pivot, ill-conditioned) the Jacobi singular values decide. */
static int full_rank5(const double M[5][5], double LU[5][5], const int piv[5], int lu_ok) {
  if (lu_ok) {
    double X[25];
    for (int i = 0; i < 25; ++i) X[i] = (i % 6 == 0) ? 1.0 : 0.0;
    lu5_solve(LU, piv, X, 5);
    double na = 0.0, ni = 0.0;
    for (int i = 0; i < 5; ++i)
      for (int j = 0; j < 5; ++j) {
        na += M[i][j] * M[i][j];
        ni += X[5 * i + j] * X[5 * i + j];
      }
    double kappa = sqrt(na) * sqrt(ni);
    if (isfinite(kappa) && kappa < 1e12) return 1;
  }
  return jacobi_rank5(M) == 5;
}

/* _parabolic_reconstruction (solver.py:2322-2415): linear gradients and
 * factors (_limited_gradients), then for full-rank cells the weighted
 * least-squares quadratic fit over the two-ring stencil (np.add.at in entry
 * order, np.linalg.solve), and the limiter applied to the quadratic
 * increment with the two-ring local extrema. */
int orc_parabolic_reconstruction(const orc_geom* g, const double* P, int code, double* grad, double* curv,
                                 double* fac) {
  int64_t C = g->n_cells, NE = g->n_parabolic;
  if (g->n_gradient) orc_linear_gradients_and_factors(g, P, code, 0.0, grad, fac);
  else {
    memset(grad, 0, sizeof(double) * 8 * C);
    for (int64_t i = 0; i < 4 * C; ++i) fac[i] = 1.0;
  }
  memset(curv, 0, sizeof(double) * 12 * C);
  if (NE == 0) return 0;
  double* scales = (double*)calloc(C, sizeof(double));
  double* M = (double*)calloc(25 * C, sizeof(double));
  double* B = (double*)calloc(20 * C, sizeof(double));
  double* lo = (double*)malloc(sizeof(double) * 4 * C);
  double* hi = (double*)malloc(sizeof(double) * 4 * C);
  double* pf = (double*)malloc(sizeof(double) * 4 * C);
  unsigned char* full = (unsigned char*)calloc(C, 1);
  for (int64_t e = 0; e < NE; ++e) {
    int64_t s = g->parabolic_sources[e];
    double a = fabs(g->parabolic_dx[e]), b = fabs(g->parabolic_dy[e]);
    double m = a >= b ? a : b;
    if (m > scales[s]) scales[s] = m;
  }
  for (int64_t c = 0; c < C; ++c)
    if (!(scales[c] >= 1e-300)) scales[c] = 1e-300;
  for (int64_t e = 0; e < NE; ++e) {
    int64_t s = g->parabolic_sources[e], nb = g->parabolic_neighbours[e];
    double nx = g->parabolic_dx[e] / scales[s], ny = g->parabolic_dy[e] / scales[s];
    double d[5] = {nx, ny, 0.5 * (nx * nx), nx * ny, 0.5 * (ny * ny)};
    double r2 = nx * nx + ny * ny;
    double w = 1.0 / (r2 >= 1e-300 ? r2 : 1e-300);
    double diff[4];
    for (int v = 0; v < 4; ++v) diff[v] = P[4 * nb + v] - P[4 * s + v];
    for (int i = 0; i < 5; ++i) {
      double wi = w * d[i];
      for (int j = 0; j < 5; ++j) M[25 * s + 5 * i + j] += wi * d[j];
      for (int v = 0; v < 4; ++v) B[20 * s + 4 * i + v] += wi * diff[v];
    }
  }
  for (int64_t c = 0; c < C; ++c) {
    double A[5][5], LU[5][5];
    int piv[5];
    for (int i = 0; i < 5; ++i)
      for (int j = 0; j < 5; ++j) A[i][j] = LU[i][j] = M[25 * c + 5 * i + j];
    int ok = lu5(LU, piv);
    if (!full_rank5(A, LU, piv, ok)) continue;
    full[c] = 1;
    double x[20];
    memcpy(x, B + 20 * c, sizeof(x));
    lu5_solve(LU, piv, x, 4);
    double sc = scales[c], sc2 = sc * sc;
    for (int v = 0; v < 4; ++v) {
      grad[8 * c + 2 * v] = x[0 * 4 + v] / sc;
      grad[8 * c + 2 * v + 1] = x[1 * 4 + v] / sc;
      curv[12 * c + 3 * v] = x[2 * 4 + v] / sc2;
      curv[12 * c + 3 * v + 1] = x[3 * 4 + v] / sc2;
      curv[12 * c + 3 * v + 2] = x[4 * 4 + v] / sc2;
    }
  }
  memcpy(lo, P, sizeof(double) * 4 * C);
  memcpy(hi, P, sizeof(double) * 4 * C);
  for (int64_t e = 0; e < NE; ++e) {
    int64_t s = g->parabolic_sources[e], nb = g->parabolic_neighbours[e];
    for (int v = 0; v < 4; ++v) {
      double q = P[4 * nb + v];
      if (q < lo[4 * s + v]) lo[4 * s + v] = q;
      if (q > hi[4 * s + v]) hi[4 * s + v] = q;
    }
  }
  for (int64_t i = 0; i < 4 * C; ++i) pf[i] = 1.0;
  for (int64_t e = 0; e < g->n_limiter; ++e) {
    int64_t c = g->limiter_cells[e];
    double dx = g->limiter_dx[e], dy = g->limiter_dy[e];
    for (int v = 0; v < 4; ++v) {
      const double* k = curv + 12 * c + 3 * v;
      double inc = grad[8 * c + 2 * v] * dx + grad[8 * c + 2 * v + 1] * dy + 0.5 * k[0] * (dx * dx) +
                   k[1] * (dx * dy) + 0.5 * k[2] * (dy * dy);
      double cv = P[4 * c + v], m = fabs(cv);
      double tol = 1e-14 * (m > 1.0 ? m : 1.0);
      double ratio = 1.0;
      if (inc > tol) ratio = (hi[4 * c + v] - cv) / inc;
      else if (inc < -tol) ratio = (lo[4 * c + v] - cv) / inc;
      ratio = ratio >= 0.0 ? ratio : 0.0;
      double f;
      if (code <= 1) f = ratio < 1.0 ? ratio : 1.0;
      else if (code == 2) {
        if (ratio > 0.0) {
          double q = 2.0 * ratio / (1.0 + ratio);
          f = 1.0 < q ? 1.0 : q;
        } else f = 0.0;
      } else {
        double eps = 1e-12;
        f = (ratio * ratio + 2.0 * ratio + eps) / (ratio * ratio + ratio + 2.0 + eps);
        f = f < 1.0 ? f : 1.0;
      }
      if (f < pf[4 * c + v]) pf[4 * c + v] = f;
    }
  }
  for (int64_t c = 0; c < C; ++c)
    if (full[c])
      for (int v = 0; v < 4; ++v) fac[4 * c + v] = pf[4 * c + v];
  free(scales);
  free(M);
  free(B);
  free(lo);
  free(hi);
  free(pf);
  free(full);
  return 0;
}

/* _far_field_boundary_states (solver.py:4350-4409), one row */
static int far_field(const double* in, const double* far, const double* n, double gamma, double* ext) {
  double ni = in[1] * n[0] + in[2] * n[1], nf = far[1] * n[0] + far[2] * n[1];
  double ci = sound(in, gamma), cf = sound(far, gamma);
  memcpy(ext, in, 4 * sizeof(double));
  if (ni <= -ci) {
    memcpy(ext, far, 4 * sizeof(double));
    return 0;
  }
  if (ni >= ci) return 0;
  double out_inv = ni + 2.0 * ci / (gamma - 1.0);
  double in_inv = nf - 2.0 * cf / (gamma - 1.0);
  double vb = 0.5 * (out_inv + in_inv);
  double cb = 0.25 * (gamma - 1.0) * (out_inv - in_inv);
  if (!isfinite(cb) || cb <= 0.0) return ORC_FARFIELD_SOUND;
  const double* src = vb < 0.0 ? far : in;
  double entropy = src[3] / pow(src[0], gamma);
  double rho = pow(cb * cb / (gamma * entropy), 1.0 / (gamma - 1.0));
  double p = entropy * pow(rho, gamma);
  double tx = -n[1], ty = n[0];
  double vt = src[1] * tx + src[2] * ty;
  ext[0] = rho;
  ext[1] = vb * n[0] + vt * tx;
  ext[2] = vb * n[1] + vt * ty;
  ext[3] = p;
  if (!isfinite(ext[0]) || !isfinite(ext[1]) || !isfinite(ext[2]) || !isfinite(ext[3]) || rho <= 0.0 ||
      p <= 0.0)
    return ORC_FARFIELD_STATE;
  return 0;
}

/* The face fluxes of n rows of left / right primitive states and unit
 * normals: kind 0 Rusanov (euler.py:80-93), 1 HLLC (euler.py:96-166),
 * 2 Roe (euler.py:169-262), 3 the compiled kernel's HLLC
 * (_kernels.py:71-160); OR of the rows' status bits. */
int orc_face_fluxes(int kind, int64_t n, const double* L, const double* R, const double* normals, double gamma,
                    double* out) {
  int status = 0;
  for (int64_t i = 0; i < n; ++i) {
    const double *l = L + 4 * i, *r = R + 4 * i, *nrm = normals + 2 * i;
    double* o = out + 4 * i;
    if (kind == 0) status |= rusanov(l, r, nrm, gamma, o);
    else if (kind == 1) status |= hllc_numpy(l, r, nrm, gamma, o);
    else if (kind == 2) status |= roe(l, r, nrm, gamma, o);
    else kernel_hllc(l, r, nrm, gamma, o);
  }
  return status;
}

/* _far_field_boundary_states (solver.py:4350-4409) for n rows of interior
 * primitive states, far-field states and unit normals; OR of the rows'
 * status bits. */
int orc_far_field_states(int64_t n, const double* in, const double* far, const double* normals, double gamma,
                         double* ext) {
  int status = 0;
  for (int64_t i = 0; i < n; ++i) status |= far_field(in + 4 * i, far + 4 * i, normals + 2 * i, gamma, ext + 4 * i);
  return status;
}

/* NumPy's pairwise summation of a contiguous float64 array (np.sum). */
static double pairwise(const double* a, int64_t n) {
  if (n < 8) {
    double r = 0.0;
    for (int64_t i = 0; i < n; ++i) r += a[i];
    return r;
  }
  if (n <= 128) {
    double r[8];
    for (int j = 0; j < 8; ++j) r[j] = a[j];
    int64_t i = 8;
    for (; i < n - (n % 8); i += 8)
      for (int j = 0; j < 8; ++j) r[j] += a[i + j];
    double res = ((r[0] + r[1]) + (r[2] + r[3])) + ((r[4] + r[5]) + (r[6] + r[7]));
    for (; i < n; ++i) res += a[i];
    return res;
  }
  int64_t n2 = n / 2;
  n2 -= n2 % 8;
  return pairwise(a, n2) + pairwise(a + n2, n - n2);
}

/* invariant_at of _pressure_inlet_boundary_states; Python's float
 * candidate**2 is libm pow(candidate, 2.0) */
static double pin_invariant(double m, double dn, double a0, double gamma) {
  double ratio = 1.0 + 0.5 * (gamma - 1.0) * pow(m, 2.0);
  double sound = a0 / sqrt(ratio);
  return sound * (dn * m + 2.0 / (gamma - 1.0));
}

/* _pressure_inlet_boundary_states (solver.py:4412-4496), one patch of n faces;
 * in/ext [n][4], nrm [n][2] */
static int pressure_inlet_states(int64_t n, const double* in, const double* nrm, const double* dn, const double* v,
                                 double gamma, double R, double* ext) {
  for (int64_t i = 0; i < n; ++i)
    if (dn[i] >= -1e-12) return ORC_PIN_DIRECTION;
  double* c = (double*)malloc(sizeof(double) * (n + 1));
  double* un = (double*)malloc(sizeof(double) * (n + 1));
  double* mach = (double*)malloc(sizeof(double) * (n + 1));
  int st = 0;
  for (int64_t i = 0; i < n; ++i) {
    c[i] = sqrt(gamma * in[4 * i + 3] / in[4 * i]);
    un[i] = in[4 * i + 1] * nrm[2 * i] + in[4 * i + 2] * nrm[2 * i + 1];
    if (un[i] / c[i] >= 1.0) st = ORC_PIN_SUPERSONIC_OUT;
  }
  double a0 = sqrt(gamma * R * v[1]);
  for (int64_t i = 0; i < n && !st; ++i) {
    if (un[i] / c[i] <= -1.0) {
      st = ORC_PIN_SUPERSONIC_IN;
      break;
    }
    double outgoing = un[i] + 2.0 * c[i] / (gamma - 1.0);
    double lo_v = pin_invariant(0.0, dn[i], a0, gamma), hi_v = pin_invariant(1.0, dn[i], a0, gamma);
    if (!(hi_v <= outgoing && outgoing <= lo_v)) {
      st = ORC_PIN_INCOMPATIBLE;
      break;
    }
    double low = 0.0, high = 1.0;
    for (int it = 0; it < 64; ++it) {
      double mid = 0.5 * (low + high);
      if (pin_invariant(mid, dn[i], a0, gamma) > outgoing) low = mid;
      else high = mid;
    }
    mach[i] = 0.5 * (low + high);
  }
  for (int64_t i = 0; i < n && !st; ++i) {
    double t = v[1] / (1.0 + 0.5 * (gamma - 1.0) * (mach[i] * mach[i]));
    double p = v[0] * pow(t / v[1], gamma / (gamma - 1.0));
    double rho = p / (R * t);
    double speed = mach[i] * sqrt(gamma * R * t);
    double* e = ext + 4 * i;
    e[0] = rho;
    e[1] = speed * v[2];
    e[2] = speed * v[3];
    e[3] = p;
    if (!isfinite(e[0]) || !isfinite(e[1]) || !isfinite(e[2]) || !isfinite(e[3]) || rho <= 0.0 || p <= 0.0)
      st = ORC_PIN_STATE;
  }
  free(c);
  free(un);
  free(mach);
  return st;
}

/* _mass_flow_inlet_boundary_states (solver.py:4499-4554), one patch; the
 * velocity speed * direction on every face (the reference's one-row velocity
 * array works only for single-face patches) */
static int mass_flow_inlet_states(int64_t n, const double* in, const double* dn, const double* len,
                                  const double* v, double gamma, double R, double* ext) {
  for (int64_t i = 0; i < n; ++i)
    if (-dn[i] <= 1e-12) return ORC_MFI_DIRECTION;
  for (int64_t i = 0; i < n; ++i)
    if (in[4 * i + 3] <= 0.0 || !isfinite(in[4 * i + 3])) return ORC_MFI_PRESSURE;
  double cp = gamma * R / (gamma - 1.0);
  double* terms = (double*)malloc(sizeof(double) * (n + 1));
#define FLOW_AT(speed, out)                                                         \
  do {                                                                              \
    double t_ = v[1] - pow((speed), 2.0) / (2.0 * cp);                              \
    for (int64_t i = 0; i < n; ++i)                                                 \
      terms[i] = in[4 * i + 3] / (R * t_) * (speed) * (-dn[i]) * len[i];            \
    out = 0.0 + pairwise(terms, n);                                                 \
  } while (0)
  double low = 0.0, high = sqrt(2.0 * cp * v[1]) * (1.0 - 1e-12), flow;
  FLOW_AT(high, flow);
  if (flow < v[0]) {
    free(terms);
    return ORC_MFI_FLOW_RATE;
  }
  for (int it = 0; it < 80; ++it) {
    double mid = 0.5 * (low + high);
    FLOW_AT(mid, flow);
    if (flow < v[0]) low = mid;
    else high = mid;
  }
#undef FLOW_AT
  free(terms);
  double speed = 0.5 * (low + high);
  double t = v[1] - pow(speed, 2.0) / (2.0 * cp);
  for (int64_t i = 0; i < n; ++i) {
    ext[4 * i] = in[4 * i + 3] / (R * t);
    ext[4 * i + 1] = speed * v[2];
    ext[4 * i + 2] = speed * v[3];
    ext[4 * i + 3] = in[4 * i + 3];
  }
  return 0;
}

/* _mass_flow_outlet_boundary_states (solver.py:4557-4577), one patch */
static int mass_flow_outlet_states(int64_t n, const double* in, const double* nrm, const double* v, double* ext) {
  for (int64_t i = 0; i < n; ++i)
    if (in[4 * i] <= 0.0 || !isfinite(in[4 * i])) return ORC_MFO_DENSITY;
  for (int64_t i = 0; i < n; ++i) {
    double nx = nrm[2 * i], ny = nrm[2 * i + 1];
    double vn = v[0] / (v[1] * in[4 * i]);
    double vt = in[4 * i + 1] * -ny + in[4 * i + 2] * nx;
    ext[4 * i] = in[4 * i];
    ext[4 * i + 1] = vn * nx + vt * -ny;
    ext[4 * i + 2] = vn * ny + vt * nx;
    ext[4 * i + 3] = in[4 * i + 3];
  }
  return 0;
}

/* exterior states of one boundary patch k from interior states in [n][4] */
int bc_patch_states(const orc_geom* g, int64_t k, const double* in, double gamma, double R, double* ext) {
  int64_t b = g->bc_offsets[k], n = g->bc_offsets[k + 1] - b;
  double* nrm = (double*)malloc(sizeof(double) * 2 * (n + 1));
  double* len = (double*)malloc(sizeof(double) * (n + 1));
  for (int64_t i = 0; i < n; ++i) {
    int64_t f = g->bc_faces[b + i];
    nrm[2 * i] = g->face_normals[2 * f];
    nrm[2 * i + 1] = g->face_normals[2 * f + 1];
    len[i] = g->face_lengths[f];
  }
  const double* v = g->bc_values + 4 * k;
  int st;
  if (g->bc_kind[k] == 0) st = pressure_inlet_states(n, in, nrm, g->bc_dn + b, v, gamma, R, ext);
  else if (g->bc_kind[k] == 1) st = mass_flow_inlet_states(n, in, g->bc_dn + b, len, v, gamma, R, ext);
  else st = mass_flow_outlet_states(n, in, nrm, v, ext);
  free(nrm);
  free(len);
  return st;
}

/* exported for tests: the exterior states of boundary patch k */
int orc_bc_states(const orc_geom* g, int64_t k, const double* in, double gamma, double R, double* ext) {
  return bc_patch_states(g, k, in, gamma, R, ext);
}

/* SciPy CSR rows of interior_divergence_operator (solver.py:2160-2174):
 * for every cell, its interior-face columns in ascending order. */
typedef struct {
  int64_t* ptr;
  int64_t* col;
  double* val;
} orc_csr;

static void divergence_operator(const orc_geom* g, orc_csr* D) {
  int64_t C = g->n_cells, NI = g->n_interior;
  D->ptr = (int64_t*)calloc(C + 1, sizeof(int64_t));
  D->col = (int64_t*)malloc(sizeof(int64_t) * (2 * NI + 1));
  D->val = (double*)malloc(sizeof(double) * (2 * NI + 1));
  for (int64_t i = 0; i < NI; ++i) {
    int64_t f = g->interior_faces[i];
    D->ptr[g->owners[f] + 1]++;
    D->ptr[g->neighbours[f] + 1]++;
  }
  for (int64_t c = 0; c < C; ++c) D->ptr[c + 1] += D->ptr[c];
  int64_t* fill = (int64_t*)malloc(sizeof(int64_t) * (C + 1));
  memcpy(fill, D->ptr, sizeof(int64_t) * (C + 1));
  for (int64_t i = 0; i < NI; ++i) { /* columns arrive in ascending order */
    int64_t f = g->interior_faces[i], o = g->owners[f], nb = g->neighbours[f];
    double L = g->face_lengths[f];
    D->col[fill[o]] = i;
    D->val[fill[o]++] = -L / g->areas[o];
    D->col[fill[nb]] = i;
    D->val[fill[nb]++] = L / g->areas[nb];
  }
  free(fill);
}

typedef struct {
  int64_t n;
  const int64_t* faces;
} group_t;

/* _residual (solver.py:2437-2718), inviscid, no turbulence */
int orc_residual(const orc_geom* g, const orc_settings* s, const double* U, double* R) {
  int64_t C = g->n_cells, NI = g->n_interior;
  double gamma = s->gamma;
  int status = 0;
  double* P = (double*)malloc(sizeof(double) * 4 * C);
  double* grad = (double*)calloc(8 * C, sizeof(double));
  double* fac = (double*)malloc(sizeof(double) * 4 * C);
  double* curv = NULL;
  status |= orc_conservative_to_primitive(C, U, gamma, P);
  if (status) goto done;
  if (s->reconstruction == 2) {
    curv = (double*)calloc(12 * C, sizeof(double));
    orc_parabolic_reconstruction(g, P, s->limiter, grad, curv, fac);
  } else if (s->reconstruction == 1 && g->n_gradient) {
    orc_linear_gradients_and_factors(g, P, s->limiter, s->venkat_k, grad, fac);
  } else {
    for (int64_t i = 0; i < 4 * C; ++i) fac[i] = 1.0;
  }
  memset(R, 0, sizeof(double) * 4 * C);
  if (NI) {
    double* flux = (double*)malloc(sizeof(double) * 4 * NI);
    for (int64_t i = 0; i < NI; ++i) {
      int64_t f = g->interior_faces[i], o = g->owners[f], nb = g->neighbours[f];
      double L[4], Rt[4];
      const double* n = g->face_normals + 2 * f;
      const double* oo = g->interior_owner_offsets + 2 * i;
      const double* no = g->interior_neighbour_offsets + 2 * i;
      reconstruct(P, grad, fac, curv, o, oo[0], oo[1], L);
      reconstruct(P, grad, fac, curv, nb, no[0], no[1], Rt);
      if (s->flux == 1 && !curv) kernel_hllc(L, Rt, n, gamma, flux + 4 * i);
      else status |= numerical_flux(s->flux, L, Rt, n, gamma, flux + 4 * i);
    }
    orc_csr D;
    divergence_operator(g, &D);
    for (int64_t c = 0; c < C; ++c) {
      double acc[4] = {0.0, 0.0, 0.0, 0.0};
      for (int64_t j = D.ptr[c]; j < D.ptr[c + 1]; ++j)
        for (int v = 0; v < 4; ++v) acc[v] += D.val[j] * flux[4 * D.col[j] + v];
      for (int v = 0; v < 4; ++v) R[4 * c + v] += acc[v];
    }
    free(D.ptr);
    free(D.col);
    free(D.val);
    free(flux);
  }
  if (g->n_periodic) {
    int64_t NP = g->n_periodic;
    double* integ = (double*)malloc(sizeof(double) * 4 * NP);
    for (int64_t i = 0; i < NP; ++i) {
      int64_t fa = g->periodic_faces_a[i], fb = g->periodic_faces_b[i];
      int64_t oa = g->owners[fa], ob = g->owners[fb];
      double L[4], Rt[4], fl[4];
      reconstruct(P, grad, fac, curv, oa, g->face_centers[2 * fa] - g->centers[2 * oa],
                  g->face_centers[2 * fa + 1] - g->centers[2 * oa + 1], L);
      reconstruct(P, grad, fac, curv, ob, g->face_centers[2 * fb] - g->centers[2 * ob],
                  g->face_centers[2 * fb + 1] - g->centers[2 * ob + 1], Rt);
      status |= numerical_flux(s->flux, L, Rt, g->face_normals + 2 * fa, gamma, fl);
      for (int v = 0; v < 4; ++v) integ[4 * i + v] = fl[v] * g->face_lengths[fa];
    }
    for (int64_t i = 0; i < NP; ++i) {
      int64_t oa = g->owners[g->periodic_faces_a[i]];
      for (int v = 0; v < 4; ++v) R[4 * oa + v] += -integ[4 * i + v] / g->areas[oa];
    }
    for (int64_t i = 0; i < NP; ++i) {
      int64_t ob = g->owners[g->periodic_faces_b[i]];
      for (int v = 0; v < 4; ++v) R[4 * ob + v] += integ[4 * i + v] / g->areas[ob];
    }
    free(integ);
  }
  /* wall / symmetry, velocity inlet, pressure outlet, far field (solver.py:2529-2625) */
  group_t groups[4] = {{g->n_wall, g->wall_faces}, {g->n_vin, g->vin_faces},
                       {g->n_pout, g->pout_faces}, {g->n_far, g->far_faces}};
  for (int k = 0; k < 4; ++k) {
    int64_t n = groups[k].n;
    if (!n) continue;
    double* contrib = (double*)malloc(sizeof(double) * 4 * n);
    for (int64_t i = 0; i < n; ++i) {
      int64_t f = groups[k].faces[i], o = g->owners[f];
      const double* nrm = g->face_normals + 2 * f;
      double in[4], ext[4], fl[4];
      reconstruct(P, grad, fac, curv, o, g->face_centers[2 * f] - g->centers[2 * o],
                  g->face_centers[2 * f + 1] - g->centers[2 * o + 1], in);
      memcpy(ext, in, sizeof(ext));
      if (k == 0) {
        double wx = g->wall_velocities ? g->wall_velocities[2 * f] : 0.0;
        double wy = g->wall_velocities ? g->wall_velocities[2 * f + 1] : 0.0;
        double un = (in[1] - wx) * nrm[0] + (in[2] - wy) * nrm[1];
        ext[1] -= 2.0 * un * nrm[0];
        ext[2] -= 2.0 * un * nrm[1];
      } else if (k == 1) {
        memcpy(ext, g->vin_states + 4 * i, sizeof(ext));
      } else if (k == 2) {
        ext[3] = g->pout_pressures[i];
      } else {
        status |= far_field(in, g->far_states + 4 * i, nrm, gamma, ext);
      }
      status |= numerical_flux(s->flux, in, ext, nrm, gamma, fl);
      for (int v = 0; v < 4; ++v) contrib[4 * i + v] = -(fl[v] * g->face_lengths[f]) / g->areas[o];
    }
    for (int64_t i = 0; i < n; ++i) {
      int64_t o = g->owners[groups[k].faces[i]];
      for (int v = 0; v < 4; ++v) R[4 * o + v] += contrib[4 * i + v];
    }
    free(contrib);
  }
  /* pressure inlets, mass-flow inlets, mass-flow outlets (solver.py:2626-2698) */
  for (int64_t k = 0; k < g->n_bc_patches && !status; ++k) {
    int64_t b = g->bc_offsets[k], n = g->bc_offsets[k + 1] - b;
    double* in = (double*)malloc(sizeof(double) * 4 * (n + 1));
    double* ext = (double*)malloc(sizeof(double) * 4 * (n + 1));
    double* contrib = (double*)malloc(sizeof(double) * 4 * (n + 1));
    for (int64_t i = 0; i < n; ++i) {
      int64_t f = g->bc_faces[b + i], o = g->owners[f];
      reconstruct(P, grad, fac, curv, o, g->face_centers[2 * f] - g->centers[2 * o],
                  g->face_centers[2 * f + 1] - g->centers[2 * o + 1], in + 4 * i);
    }
    status |= bc_patch_states(g, k, in, gamma, s->gas_constant, ext);
    for (int64_t i = 0; i < n && !status; ++i) {
      int64_t f = g->bc_faces[b + i], o = g->owners[f];
      double fl[4];
      status |= numerical_flux(s->flux, in + 4 * i, ext + 4 * i, g->face_normals + 2 * f, gamma, fl);
      for (int v = 0; v < 4; ++v) contrib[4 * i + v] = -(fl[v] * g->face_lengths[f]) / g->areas[o];
    }
    for (int64_t i = 0; i < n && !status; ++i) {
      int64_t o = g->owners[g->bc_faces[b + i]];
      for (int v = 0; v < 4; ++v) R[4 * o + v] += contrib[4 * i + v];
    }
    free(in);
    free(ext);
    free(contrib);
  }
  if (s->acceleration_x != 0.0 || s->acceleration_y != 0.0) {
    for (int64_t c = 0; c < C; ++c) R[4 * c + 1] += P[4 * c] * s->acceleration_x;
    for (int64_t c = 0; c < C; ++c) R[4 * c + 2] += P[4 * c] * s->acceleration_y;
    for (int64_t c = 0; c < C; ++c)
      R[4 * c + 3] += P[4 * c] * (s->acceleration_x * P[4 * c + 1] + s->acceleration_y * P[4 * c + 2]);
  }
  for (int64_t i = 0; i < 4 * C; ++i)
    if (!isfinite(R[i])) {
      status |= ORC_NONFINITE_RESIDUAL;
      break;
    }
done:
  free(P);
  free(grad);
  free(fac);
  free(curv);
  return status;
}

/* _stable_time_steps (solver.py:4132-4343), inviscid */
int orc_stable_time_steps(const orc_geom* g, const orc_settings* s, const double* P, const double* diffusion,
                          double* dt) {
  int64_t C = g->n_cells, F = g->n_faces;
  double gamma = s->gamma;
  int status = 0;
  double* radius = (double*)malloc(sizeof(double) * (F + 1));
  double* cs = (double*)malloc(sizeof(double) * C);
  for (int64_t c = 0; c < C; ++c) cs[c] = sound(P + 4 * c, gamma);
  for (int64_t f = 0; f < F; ++f) {
    int64_t o = g->owners[f];
    radius[f] = fabs(P[4 * o + 1] * g->face_normals[2 * f] + P[4 * o + 2] * g->face_normals[2 * f + 1]) + cs[o];
  }
  /* exterior radius on inlet / outlet / far-field faces (solver.py:4190-4220) */
  for (int k = 0; k < 3; ++k) {
    int64_t n = k == 0 ? g->n_vin : (k == 1 ? g->n_pout : g->n_far);
    const int64_t* faces = k == 0 ? g->vin_faces : (k == 1 ? g->pout_faces : g->far_faces);
    for (int64_t i = 0; i < n; ++i) {
      int64_t f = faces[i], o = g->owners[f];
      const double* nrm = g->face_normals + 2 * f;
      double ext[4];
      memcpy(ext, P + 4 * o, sizeof(ext));
      if (k == 0) memcpy(ext, g->vin_states + 4 * i, sizeof(ext));
      else if (k == 1) ext[3] = g->pout_pressures[i];
      else status |= far_field(P + 4 * o, g->far_states + 4 * i, nrm, gamma, ext);
      double er = fabs(ext[1] * nrm[0] + ext[2] * nrm[1]) + sound(ext, gamma);
      radius[f] = radius[f] >= er ? radius[f] : er;
    }
  }
  /* pressure-inlet and mass-flow faces: states from the cell values */
  for (int64_t k = 0; k < g->n_bc_patches; ++k) {
    int64_t b = g->bc_offsets[k], n = g->bc_offsets[k + 1] - b;
    double* in = (double*)malloc(sizeof(double) * 4 * (n + 1));
    double* ext = (double*)malloc(sizeof(double) * 4 * (n + 1));
    for (int64_t i = 0; i < n; ++i) memcpy(in + 4 * i, P + 4 * g->owners[g->bc_faces[b + i]], 4 * sizeof(double));
    status |= bc_patch_states(g, k, in, gamma, s->gas_constant, ext);
    for (int64_t i = 0; i < n; ++i) {
      int64_t f = g->bc_faces[b + i];
      const double* nrm = g->face_normals + 2 * f;
      double er = fabs(ext[4 * i + 1] * nrm[0] + ext[4 * i + 2] * nrm[1]) + sound(ext + 4 * i, gamma);
      radius[f] = radius[f] >= er ? radius[f] : er;
    }
    free(in);
    free(ext);
  }
  double* sum = (double*)calloc(C, sizeof(double));
  for (int64_t f = 0; f < F; ++f) sum[g->owners[f]] += radius[f] * g->face_lengths[f];
  for (int64_t i = 0; i < g->n_interior; ++i) {
    int64_t f = g->interior_faces[i], nb = g->neighbours[f];
    double r = fabs(P[4 * nb + 1] * g->face_normals[2 * f] + P[4 * nb + 2] * g->face_normals[2 * f + 1]) + cs[nb];
    sum[nb] += r * g->face_lengths[f];
  }
  /* viscous terms: spectral_sum += 2 * diffusion_sum (solver.py:4331) */
  if (diffusion)
    for (int64_t c = 0; c < C; ++c) sum[c] += 2.0 * diffusion[c];
  for (int64_t c = 0; c < C; ++c) {
    dt[c] = s->cfl * g->areas[c] / sum[c];
    if (!isfinite(dt[c]) || dt[c] <= 0.0) status |= ORC_TIME_STEP;
  }
  free(radius);
  free(cs);
  free(sum);
  return status;
}

/* One explicit step (solver.py:532-806 and 1128-1182).  dt is a scalar
 * (dt_per_cell = 0) or [C] (local steady mode, _scale_cell_rate). */
int orc_explicit_step(const orc_geom* g, const orc_settings* s, int scheme, double* U, const double* dt,
                      int dt_per_cell) {
  int64_t C = g->n_cells, N = 4 * C;
  int st = 0;
  double* R = (double*)malloc(sizeof(double) * N);
  double* X[5];
  for (int k = 0; k < 5; ++k) X[k] = (double*)malloc(sizeof(double) * N);
  double* R3 = (double*)malloc(sizeof(double) * N);
  double* Pchk = (double*)malloc(sizeof(double) * N);
#define DT(i) (dt_per_cell ? dt[(i) / 4] : dt[0])
#define RES(src)                   \
  do {                             \
    st |= orc_residual(g, s, src, R); \
    if (st) goto out;              \
  } while (0)
  memcpy(X[0], U, sizeof(double) * N);
  if (scheme == 3) {
    static const double c1 = 0.391752226571890, a20 = 0.444370493651235, a21 = 0.555629506348765,
                        c2 = 0.368410593050371, a30 = 0.620101851488403, a32 = 0.379898148511597,
                        c3 = 0.251891774271694, a40 = 0.178079954393132, a43 = 0.821920045606868,
                        c4 = 0.544974750228521, a52 = 0.517231671970585, a53 = 0.096059710526147,
                        c5 = 0.063692468666290, a54 = 0.386708617503269, c6 = 0.226007483236906;
    RES(X[0]);
    for (int64_t i = 0; i < N; ++i) X[1][i] = X[0][i] + (c1 * DT(i)) * R[i];
    RES(X[1]);
    for (int64_t i = 0; i < N; ++i) X[2][i] = a20 * X[0][i] + a21 * X[1][i] + (c2 * DT(i)) * R[i];
    RES(X[2]);
    for (int64_t i = 0; i < N; ++i) X[3][i] = a30 * X[0][i] + a32 * X[2][i] + (c3 * DT(i)) * R[i];
    RES(X[3]);
    memcpy(R3, R, sizeof(double) * N);
    for (int64_t i = 0; i < N; ++i) X[4][i] = a40 * X[0][i] + a43 * X[3][i] + (c4 * DT(i)) * R[i];
    RES(X[4]);
    for (int64_t i = 0; i < N; ++i)
      U[i] = a52 * X[2][i] + a53 * X[3][i] + (c5 * DT(i)) * R3[i] + a54 * X[4][i] + (c6 * DT(i)) * R[i];
  } else {
    RES(X[0]);
    for (int64_t i = 0; i < N; ++i) X[1][i] = X[0][i] + DT(i) * R[i];
    if (scheme == 0) {
      memcpy(U, X[1], sizeof(double) * N);
    } else {
      st |= orc_conservative_to_primitive(C, X[1], s->gamma, Pchk);
      if (st) goto out;
      RES(X[1]);
      if (scheme == 1) {
        for (int64_t i = 0; i < N; ++i) U[i] = 0.5 * X[0][i] + 0.5 * (X[1][i] + DT(i) * R[i]);
      } else {
        for (int64_t i = 0; i < N; ++i) X[2][i] = 0.75 * X[0][i] + 0.25 * (X[1][i] + DT(i) * R[i]);
        st |= orc_conservative_to_primitive(C, X[2], s->gamma, Pchk);
        if (st) goto out;
        RES(X[2]);
        for (int64_t i = 0; i < N; ++i)
          U[i] = (1.0 / 3.0) * X[0][i] + (2.0 / 3.0) * (X[2][i] + DT(i) * R[i]);
      }
    }
  }
  st |= orc_conservative_to_primitive(C, U, s->gamma, Pchk);
out:
#undef DT
#undef RES
  free(R);
  for (int k = 0; k < 5; ++k) free(X[k]);
  free(R3);
  free(Pchk);
  return st;
}

/* ------------------------------------------------------- mesh geometry
 *
 * _build_geometry's cell and face loops (solver.py:1654-1696), so that the
 * CPU reference path builds its geometry without the product library.
 *
 * Cells: twice the signed area is Python's built-in sum() of the shoelace
 * cross products; for floats CPython >= 3.12 sums with Neumaier's
 * compensation (running sum t, compensation c, added once at the end when it
 * is non-zero and finite).  The centroid sums are plain left-to-right.
 *
 * Faces: np.linalg.norm of a 2-vector and np.dot of two 2-vectors are BLAS
 * dot products, which round as fma(a1, b1, a0 * b0) on the reference's
 * platform; the normal is (ey, -ex) / length, flipped when it points into the
 * owner.  Returns 4 and the offending id on a degenerate cell or face (the
 * reference's "Cell {id} has zero or invalid area." / "Face {id} has zero or
 * invalid length.").
 */
int orc_cell_geometry(int64_t n_cells, const int64_t* off, const int64_t* nodes, const double* pts,
                      double* centers, double* areas, int64_t* bad) {
  for (int64_t c = 0; c < n_cells; ++c) {
    const int64_t b = off[c], k = off[c + 1] - off[c];
    double total = 0.0, comp = 0.0;
    for (int64_t i = 0; i < k; ++i) {
      const double* p = pts + 2 * nodes[b + i];
      const double* q = pts + 2 * nodes[b + (i + 1) % k];
      const double x = p[0] * q[1] - q[0] * p[1];
      if (i == 0) {
        total = x;
        continue;
      }
      const double t = total + x;
      if (fabs(total) >= fabs(x))
        comp += (total - t) + x;
      else
        comp += (x - t) + total;
      total = t;
    }
    if (comp != 0.0 && isfinite(comp)) total += comp;
    if (!isfinite(total) || fabs(total) <= 1e-15) {
      *bad = c;
      return 4;
    }
    double xs = 0.0, ys = 0.0;
    for (int64_t i = 0; i < k; ++i) {
      const double* p = pts + 2 * nodes[b + i];
      const double* q = pts + 2 * nodes[b + (i + 1) % k];
      const double cross = p[0] * q[1] - q[0] * p[1];
      xs += (p[0] + q[0]) * cross;
      ys += (p[1] + q[1]) * cross;
    }
    centers[2 * c] = xs / (3.0 * total);
    centers[2 * c + 1] = ys / (3.0 * total);
    areas[c] = 0.5 * fabs(total);
  }
  return 0;
}

int orc_face_geometry(int64_t n_faces, const int64_t* face_nodes, const double* pts, const double* centers,
                      const int64_t* owners, double* face_centers, double* normals, double* lengths, int64_t* bad) {
  for (int64_t f = 0; f < n_faces; ++f) {
    const double* a = pts + 2 * face_nodes[2 * f];
    const double* b = pts + 2 * face_nodes[2 * f + 1];
    const double ex = b[0] - a[0], ey = b[1] - a[1];
    const double len = sqrt(fma(ey, ey, ex * ex));
    if (!isfinite(len) || len <= 1e-15) {
      *bad = f;
      return 4;
    }
    double nx = ey / len, ny = -ex / len;
    const double cx = 0.5 * (a[0] + b[0]), cy = 0.5 * (a[1] + b[1]);
    const double* o = centers + 2 * owners[f];
    if (fma(ny, cy - o[1], nx * (cx - o[0])) < 0.0) {
      nx = -nx;
      ny = -ny;
    }
    face_centers[2 * f] = cx;
    face_centers[2 * f + 1] = cy;
    normals[2 * f] = nx;
    normals[2 * f + 1] = ny;
    lengths[f] = len;
  }
  return 0;
}
