// Implicit Euler building blocks (solver.py:1185-1567) on the device:
//
// * the first-order scalar preconditioner matrix and its LU-SGS application
//   (_implicit_preconditioner, solver.py:1185-1323): diagonal
//   1 + sum dt_i rho_f L / (2 A_i) over interior and periodic faces +
//   dt_i rho L / A_i over boundary faces, off-diagonals -dt_i rho_f L/(2 A_i);
//   the forward solve (D+L) y = v and backward solve (D+U) x = D y run over
//   level sets of the natural-cell-order dependency graph, one cooperative
//   persistent kernel per sweep with a grid barrier between levels, so the
//   preconditioner is exactly the reference's (only independent rows run
//   concurrently);
// * the matrix-free operator v -> v - dt [R1(u + eps s v) - R1(u)] / (eps s)
//   (_matrix_free_implicit_operator, solver.py:1532-1567);
// * restarted GMRES(m) as the reference drives SciPy's gmres
//   (_solve_gmres, solver.py:1489-1529): left preconditioning, modified
//   Gram-Schmidt, Givens rotations, SciPy's inner/outer tolerance control.
// Vector reductions are deterministic two-level trees.
#include <cooperative_groups.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "mcfd_device.cuh"
#include "mcfd_implicit.h"

namespace cg = cooperative_groups;

namespace mcfd {
namespace {

constexpr int kBlock = 256;
constexpr int kRedBlocks = 152 * 4;

inline int blocks_for(long long n) { return (int)((n + kBlock - 1) / kBlock); }

// ------------------------------------------------------------ preconditioner

// coupling faces: 0.5 * max(|u_a.n_a| + c_a, |u_b.n_b| + c_b) * L
__global__ void k_coupling_coef(int n, const int* __restrict__ ca, const int* __restrict__ cb,
                                const double2* __restrict__ na, const double2* __restrict__ nb,
                                const double* __restrict__ len, const double* __restrict__ P,
                                double gamma, double* __restrict__ coef) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const St4 pa = ld4(P + 4 * (size_t)ca[k]);
  const St4 pb = ld4(P + 4 * (size_t)cb[k]);
  const double2 a = na[k], b = nb[k];
  double ra = fabs(pa.b * a.x + pa.c * a.y) + sound_speed(pa.a, pa.d, gamma);
  double rb = fabs(pb.b * b.x + pb.c * b.y) + sound_speed(pb.a, pb.d, gamma);
  double radius = icmp::lt_nonneg(ra, rb) ? rb : ra;  // np.maximum
  coef[k] = 0.5 * radius * len[k];
}

// boundary faces (every face without a neighbour, periodic ones included):
// dt_o * (|u_o.n| + c_o) * L / A_o
__global__ void k_boundary_term(int n, const int* __restrict__ owner, const double2* __restrict__ nrm,
                                const double* __restrict__ len, const double* __restrict__ P,
                                const double* __restrict__ area, const double* __restrict__ dt,
                                int dt_per_cell, double gamma, double* __restrict__ term) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const int o = owner[k];
  const St4 p = ld4(P + 4 * (size_t)o);
  const double2 m = nrm[k];
  double radius = fabs(p.b * m.x + p.c * m.y) + sound_speed(p.a, p.d, gamma);
  const double d = dt_per_cell ? dt[o] : dt[0];
  term[k] = div_rn(d * radius * len[k], area[o]);
}

// per cell: diagonal in the reference's np.add.at order and the row values
__global__ void k_lusgs_assemble(int C, const int* __restrict__ dptr, const int* __restrict__ dref,
                                 const double* __restrict__ coef, const double* __restrict__ bterm,
                                 const int* __restrict__ rptr, const int* __restrict__ rref,
                                 const int* __restrict__ rcol, const double* __restrict__ area,
                                 const double* __restrict__ dt, int dt_per_cell,
                                 double* __restrict__ diag, double* __restrict__ dclamp,
                                 double* __restrict__ rval) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= C) return;
  const double d = dt_per_cell ? dt[i] : dt[0];
  const double A = area[i];
  double s = 1.0;
  for (int e = dptr[i]; e < dptr[i + 1]; ++e) {
    const int r = dref[e];
    s = s + (r >= 0 ? div_rn(d * coef[r], A) : bterm[-r - 1]);
  }
  for (int e = rptr[i]; e < rptr[i + 1]; ++e) {
    const double v = div_rn(-(d * coef[rref[e]]), A);
    rval[e] = v;
    // a periodic pair whose two faces belong to one cell couples the cell to
    // itself: the reference's COO -> CSC conversion sums it into the diagonal
    if (rcol[e] == i) s = s + v;
  }
  diag[i] = s;
  dclamp[i] = icmp::lt_pos(s, 1e-14) ? 1e-14 : s;  // np.maximum(diagonal, 1e-14)
}

struct SweepArgs {
  int n_levels;
  const int* level_ptr;
  const int* level_cells;
  const int* row_ptr;   // this sweep's off-diagonal entries per cell
  const int* row_col;
  const int* row_val;   // index into rval
  const double* rval;
  const double* diag;
  const double* dclamp;  // backward sweep: right-hand side D * y
  const double* in;
  double* out;
  int backward;
};

// Level-scheduled triangular sweep: rows of one level are independent; the
// grid barrier orders the levels (cooperative launch: all blocks resident).
__global__ void __launch_bounds__(kBlock) k_lusgs_sweep(SweepArgs a) {
  cg::grid_group grid = cg::this_grid();
  const int stride = gridDim.x * blockDim.x;
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  for (int l = 0; l < a.n_levels; ++l) {
    const int b = a.level_ptr[l], e = a.level_ptr[l + 1];
    for (int t = b + tid; t < e; t += stride) {
      const int i = a.level_cells[t];
      St4 r = ld4(a.in + 4 * (size_t)i);
      double acc[4] = {r.a, r.b, r.c, r.d};
      if (a.backward) {
        const double dc = a.dclamp[i];
        for (int k = 0; k < 4; ++k) acc[k] = dc * acc[k];
      }
      for (int j = a.row_ptr[i]; j < a.row_ptr[i + 1]; ++j) {
        const double v = a.rval[a.row_val[j]];
        const St4 x = ld4(a.out + 4 * (size_t)a.row_col[j]);
        acc[0] = acc[0] - v * x.a;
        acc[1] = acc[1] - v * x.b;
        acc[2] = acc[2] - v * x.c;
        acc[3] = acc[3] - v * x.d;
      }
      const double dg = a.diag[i];
      st4(a.out + 4 * (size_t)i, St4{div_rn(acc[0], dg), div_rn(acc[1], dg), div_rn(acc[2], dg), div_rn(acc[3], dg)});
    }
    grid.sync();
  }
}

// ------------------------------------------------------------------ vectors

__global__ void __launch_bounds__(kBlock) k_dot_partial(long long n, const double* __restrict__ x,
                                                        const double* __restrict__ y,
                                                        double* __restrict__ partials) {
  __shared__ double sh[kBlock];
  double acc = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    acc += x[i] * y[i];
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int w = kBlock / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) partials[blockIdx.x] = sh[0];
}

__global__ void k_dot_final(int blocks, const double* __restrict__ partials, double* out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double s = 0.0;
    for (int b = 0; b < blocks; ++b) s += partials[b];
    out[0] = s;
  }
}

// y -= alpha[0] * x   (modified Gram-Schmidt update with a device scalar)
__global__ void k_axmy_dev(long long n, const double* __restrict__ alpha, const double* __restrict__ x,
                           double* __restrict__ y) {
  long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i < n) y[i] = y[i] - alpha[0] * x[i];
}

// Newton equation of the implicit step (solver.py:1415-1426):
// e = U - U0 - dt R ; b = -(e / s) ; max|e / s| ; max|(U - U0) / s|
__global__ void __launch_bounds__(kBlock) k_equation(int C, const double* __restrict__ U,
                                                     const double* __restrict__ U0,
                                                     const double* __restrict__ R,
                                                     const double* __restrict__ dt, int dt_per_cell,
                                                     ScaleVec s, double* __restrict__ b,
                                                     unsigned long long* __restrict__ maxima) {
  __shared__ unsigned long long m0[kBlock / 32], m1[kBlock / 32];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long e_abs = 0, u_abs = 0;
  if (i < 4 * C) {
    const double d = dt_per_cell ? dt[i >> 2] : dt[0];
    const double du = U[i] - U0[i];
    const double eq = du - d * R[i];
    const double se = div_rn(eq, s.v[i & 3]);
    if (b) b[i] = -se;
    e_abs = (unsigned long long)(icmp::bits(se) & 0x7fffffffffffffffLL);
    u_abs = (unsigned long long)(icmp::bits(div_rn(du, s.v[i & 3])) & 0x7fffffffffffffffLL);
  }
  for (int off = 16; off > 0; off >>= 1) {
    unsigned long long a = __shfl_down_sync(0xffffffffu, e_abs, off);
    unsigned long long c = __shfl_down_sync(0xffffffffu, u_abs, off);
    e_abs = a > e_abs ? a : e_abs;
    u_abs = c > u_abs ? c : u_abs;
  }
  if ((threadIdx.x & 31) == 0) {
    m0[threadIdx.x >> 5] = e_abs;
    m1[threadIdx.x >> 5] = u_abs;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long a = 0, c = 0;
    for (int w = 0; w < kBlock / 32; ++w) {
      a = m0[w] > a ? m0[w] : a;
      c = m1[w] > c ? m1[w] : c;
    }
    atomicMax(maxima, a);
    atomicMax(maxima + 1, c);
  }
}

// Scaling maxima (solver.py:1393-1413): max rho, max |u|,|v|, max sound speed,
// max p, and max |U_k| per column.  All values are |.| or positive, so their
// bit patterns order like the values and the maxima run on integers.
__global__ void __launch_bounds__(kBlock) k_scale_maxima(int C, const double* __restrict__ U,
                                                         const double* __restrict__ P, double gamma,
                                                         unsigned long long* __restrict__ maxima) {
  __shared__ unsigned long long sh[8][kBlock / 32];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long m[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  if (i < C) {
    const St4 p = ld4(P + 4 * (size_t)i);
    const St4 u = ld4(U + 4 * (size_t)i);
    const double vals[8] = {p.a, fabs(p.b), fabs(p.c), sound_speed(p.a, p.d, gamma), p.d,
                            fabs(u.a), fabs(u.b), fabs(u.c)};
    for (int k = 0; k < 8; ++k) m[k] = (unsigned long long)(icmp::bits(vals[k]) & 0x7fffffffffffffffLL);
    // column 3 of U goes in slot 7 after |U_2|: reuse by packing below
  }
  for (int k = 0; k < 8; ++k) {
    unsigned long long v = m[k];
    for (int off = 16; off > 0; off >>= 1) {
      unsigned long long o = __shfl_down_sync(0xffffffffu, v, off);
      v = o > v ? o : v;
    }
    if ((threadIdx.x & 31) == 0) sh[k][threadIdx.x >> 5] = v;
  }
  __syncthreads();
  if (threadIdx.x < 8) {
    unsigned long long v = 0;
    for (int w = 0; w < kBlock / 32; ++w) v = sh[threadIdx.x][w] > v ? sh[threadIdx.x][w] : v;
    atomicMax(maxima + threadIdx.x, v);
  }
}

__global__ void __launch_bounds__(kBlock) k_col3_max(int C, const double* __restrict__ U,
                                                     unsigned long long* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long v = 0;
  if (i < C) v = (unsigned long long)(icmp::bits(U[4 * (size_t)i + 3]) & 0x7fffffffffffffffLL);
  for (int off = 16; off > 0; off >>= 1) {
    unsigned long long o = __shfl_down_sync(0xffffffffu, v, off);
    v = o > v ? o : v;
  }
  if ((threadIdx.x & 31) == 0) atomicMax(out, v);
}

// sum over i of (U_i / s_k)^2
__global__ void __launch_bounds__(kBlock) k_scaled_sumsq_partial(long long n, const double* __restrict__ x,
                                                                 ScaleVec s, double* __restrict__ partials) {
  __shared__ double sh[kBlock];
  double acc = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const double q = div_rn(x[i], s.v[i & 3]);
    acc += q * q;
  }
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int w = kBlock / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) partials[blockIdx.x] = sh[0];
}

// out = U + (damping * dx) * s_k   (solver.py:1462-1464)
__global__ void k_candidate(int C, const double* __restrict__ U, const double* __restrict__ dx,
                            double damping, ScaleVec s, double* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < 4 * C) out[i] = U[i] + (damping * dx[i]) * s.v[i & 3];
}

__global__ void k_axpy(long long n, double a, const double* __restrict__ x, double* __restrict__ y) {
  long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i < n) y[i] = y[i] + a * x[i];
}

__global__ void k_scale(long long n, double a, double* __restrict__ x) {
  long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i < n) x[i] = x[i] * a;
}

// r = b - x
__global__ void k_sub(long long n, const double* __restrict__ b, const double* __restrict__ x,
                      double* __restrict__ r) {
  long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i < n) r[i] = b[i] - x[i];
}

// ------------------------------------------------------------- FD operator

// eps = sqrt(machine eps) * max(1, |u/s|) / |v|  (solver.py:1546-1561)
__global__ void k_fd_eps(const double* __restrict__ v_sumsq, double state_norm, double* eps_out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    const double dn = sqrt_rn(v_sumsq[0]);
    const double fd = 1.4901161193847656e-08;  // math.sqrt(np.finfo(float).eps)
    eps_out[0] = (dn == 0.0) ? 0.0 : div_rn(fd * (state_norm > 1.0 ? state_norm : 1.0), dn);
  }
}

// U_p = u + (eps * s_k) * v
__global__ void k_fd_perturb(int C, const double* __restrict__ u, const double* __restrict__ v,
                             const double* __restrict__ eps, ScaleVec s, double* __restrict__ up) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 4 * C) return;
  const double e = eps[0];
  up[i] = u[i] + (e * s.v[i & 3]) * v[i];
}

// out = v - dt * ((R_p - R) / eps) / s_k ; out = v when |v| = 0
__global__ void k_fd_combine(int C, const double* __restrict__ v, const double* __restrict__ rp,
                             const double* __restrict__ rate, const double* __restrict__ eps,
                             ScaleVec s, const double* __restrict__ dt, int dt_per_cell,
                             double* __restrict__ out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 4 * C) return;
  const double e = eps[0];
  if (e == 0.0) {
    out[i] = v[i];
    return;
  }
  const double d = dt_per_cell ? dt[i >> 2] : dt[0];
  const double jv = div_rn(rp[i] - rate[i], e);
  out[i] = v[i] - div_rn(d * jv, s.v[i & 3]);
}

}  // namespace

// ======================================================== host-side classes

cudaError_t implicit_dot(ImplicitState& st, long long n, const double* x, const double* y, double* out,
                         cudaStream_t s) {
  count_launch(2);
  k_dot_partial<<<kRedBlocks, kBlock, 0, s>>>(n, x, y, st.partials);
  k_dot_final<<<1, 32, 0, s>>>(kRedBlocks, st.partials, out);
  return cudaGetLastError();
}

cudaError_t implicit_build(ImplicitState& st, const ImplicitTopology& t) {
  const int C = t.n_cells;
  st.n_cells = C;
  // couplings: interior faces, then periodic pairs
  const int NC = (int)t.coupling_a.size();
  const int NB = (int)t.boundary_owner.size();
  st.n_coupling = NC;
  st.n_boundary = NB;
  // diagonal accumulation order per cell (solver.py:1229-1300): interior
  // owners, interior neighbours, periodic a, periodic b, boundary faces.
  std::vector<std::vector<int>> dlist(C);
  for (int k = 0; k < t.n_interior; ++k) dlist[t.coupling_a[k]].push_back(k);
  for (int k = 0; k < t.n_interior; ++k) dlist[t.coupling_b[k]].push_back(k);
  for (int k = t.n_interior; k < NC; ++k) dlist[t.coupling_a[k]].push_back(k);
  for (int k = t.n_interior; k < NC; ++k) dlist[t.coupling_b[k]].push_back(k);
  for (int b = 0; b < NB; ++b) dlist[t.boundary_owner[b]].push_back(-b - 1);
  // rows: entries (col, coupling) of the scalar matrix, split lower / upper
  std::vector<std::vector<std::pair<int, int>>> lower(C), upper(C);
  std::vector<int> rptr(C + 1, 0), rref;
  std::vector<std::vector<int>> rows(C);
  for (int k = 0; k < NC; ++k) {
    rows[t.coupling_a[k]].push_back(k);   // row a, column b
    rows[t.coupling_b[k]].push_back(~k);  // row b, column a
  }
  std::vector<int> dptr(C + 1, 0), dref, rcol;
  for (int i = 0; i < C; ++i) {
    dptr[i + 1] = dptr[i] + (int)dlist[i].size();
    dref.insert(dref.end(), dlist[i].begin(), dlist[i].end());
  }
  // row values are laid out per cell; rval index = position
  for (int i = 0; i < C; ++i) {
    rptr[i + 1] = rptr[i] + (int)rows[i].size();
    for (int code : rows[i]) {
      int k = code >= 0 ? code : ~code;
      int col = code >= 0 ? t.coupling_b[k] : t.coupling_a[k];
      rref.push_back(k);
      rcol.push_back(col);
      int slot = (int)rref.size() - 1;
      if (col < i) lower[i].push_back({col, slot});
      else if (col > i) upper[i].push_back({col, slot});
      // col == i (a periodic face paired with its own cell) lands on the
      // diagonal of kron(A, I4) in the reference; keep it in the lower part
      // so the diagonal solve still divides by the assembled diagonal
      else lower[i].push_back({col, slot});
    }
  }
  for (int i = 0; i < C; ++i) {
    std::sort(lower[i].begin(), lower[i].end());
    std::sort(upper[i].begin(), upper[i].end());
  }
  // level sets
  auto levels = [&](bool fwd, std::vector<int>& lptr, std::vector<int>& lcells) {
    std::vector<int> lev(C, 0);
    int nlev = 0;
    if (fwd) {
      for (int i = 0; i < C; ++i) {
        int m = 0;
        for (auto& e : lower[i])
          if (e.first < i) m = std::max(m, lev[e.first] + 1);
        lev[i] = m;
        nlev = std::max(nlev, m + 1);
      }
    } else {
      for (int i = C - 1; i >= 0; --i) {
        int m = 0;
        for (auto& e : upper[i]) m = std::max(m, lev[e.first] + 1);
        lev[i] = m;
        nlev = std::max(nlev, m + 1);
      }
    }
    lptr.assign(nlev + 1, 0);
    for (int i = 0; i < C; ++i) lptr[lev[i] + 1]++;
    for (int l = 0; l < nlev; ++l) lptr[l + 1] += lptr[l];
    lcells.resize(C);
    std::vector<int> fill(lptr.begin(), lptr.end() - 1);
    for (int i = 0; i < C; ++i) lcells[fill[lev[i]]++] = i;
    return nlev;
  };
  std::vector<int> flp, flc, blp, blc;
  st.n_levels_fwd = levels(true, flp, flc);
  st.n_levels_bwd = levels(false, blp, blc);
  auto csr = [&](std::vector<std::vector<std::pair<int, int>>>& rowsv, std::vector<int>& ptr,
                 std::vector<int>& col, std::vector<int>& val, bool drop_diag) {
    ptr.assign(C + 1, 0);
    for (int i = 0; i < C; ++i) {
      for (auto& e : rowsv[i]) {
        if (drop_diag && e.first == i) continue;
        col.push_back(e.first);
        val.push_back(e.second);
      }
      ptr[i + 1] = (int)col.size();
    }
  };
  std::vector<int> lptr, lcol, lval, uptr, ucol, uval;
  csr(lower, lptr, lcol, lval, true);
  csr(upper, uptr, ucol, uval, true);

  // device memory
  std::vector<std::pair<void**, size_t>> allocs;
  auto up = [&](const void* src, size_t bytes, void** dst) -> cudaError_t {
    cudaError_t e = cudaMalloc(dst, bytes ? bytes : 4);
    if (e != cudaSuccess) return e;
    st.owned.push_back(*dst);
    if (bytes) e = cudaMemcpy(*dst, src, bytes, cudaMemcpyHostToDevice);
    return e;
  };
  cudaError_t e = cudaSuccess;
#define UP(vec, field) \
  if (e == cudaSuccess) e = up(vec.data(), vec.size() * sizeof(vec[0]), (void**)&st.field)
  UP(t.coupling_a, ca);
  UP(t.coupling_b, cb);
  UP(t.coupling_na, na);
  UP(t.coupling_nb, nb);
  UP(t.coupling_len, clen);
  UP(t.boundary_owner, bowner);
  UP(t.boundary_normal, bnormal);
  UP(t.boundary_len, blen);
  UP(dptr, dptr);
  UP(dref, dref);
  UP(rptr, rptr);
  UP(rref, rref);
  UP(rcol, rcol);
  UP(flp, fwd_level_ptr);
  UP(flc, fwd_level_cells);
  UP(blp, bwd_level_ptr);
  UP(blc, bwd_level_cells);
  UP(lptr, lower_ptr);
  UP(lcol, lower_col);
  UP(lval, lower_val);
  UP(uptr, upper_ptr);
  UP(ucol, upper_col);
  UP(uval, upper_val);
#undef UP
  auto zeros = [&](size_t n, double** dst) {
    if (e == cudaSuccess) e = cudaMalloc((void**)dst, std::max<size_t>(n, 1) * sizeof(double));
    if (e == cudaSuccess) st.owned.push_back(*dst);
  };
  const size_t N4 = 4 * (size_t)C;
  zeros(NC, &st.coef);
  zeros(NB, &st.bterm);
  zeros(C, &st.diag);
  zeros(C, &st.dclamp);
  zeros(rref.size(), &st.rval);
  zeros(N4, &st.tmp);
  zeros(N4, &st.state);
  zeros(N4, &st.rate);
  zeros(N4, &st.up);
  zeros(N4, &st.rp);
  zeros(N4, &st.w);
  zeros(N4, &st.av);
  zeros(kRedBlocks, &st.partials);
  zeros(64, &st.scalars);
  if (e == cudaSuccess) {
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_lusgs_sweep, kBlock, 0);
    st.sweep_blocks = std::max(1, sms * std::min(per_sm, 2));
  }
  return e;
}

void implicit_free(ImplicitState& st) {
  for (void* p : st.owned) cudaFree(p);
  st.owned.clear();
  for (double* v : st.krylov) cudaFree(v);
  st.krylov.clear();
  if (st.hcol) cudaFree(st.hcol);
  st.hcol = nullptr;
  st.hcol_size = 0;
}

cudaError_t implicit_assemble(ImplicitState& st, const double* P, const double* area, const double* dt,
                              int dt_per_cell, double gamma, cudaStream_t s) {
  if (st.n_coupling > 0) {
    count_launch();
    k_coupling_coef<<<blocks_for(st.n_coupling), kBlock, 0, s>>>(st.n_coupling, st.ca, st.cb, st.na, st.nb,
                                                                 st.clen, P, gamma, st.coef);
  }
  if (st.n_boundary > 0) {
    count_launch();
    k_boundary_term<<<blocks_for(st.n_boundary), kBlock, 0, s>>>(st.n_boundary, st.bowner, st.bnormal, st.blen,
                                                                 P, area, dt, dt_per_cell, gamma, st.bterm);
  }
  count_launch();
  k_lusgs_assemble<<<blocks_for(st.n_cells), kBlock, 0, s>>>(st.n_cells, st.dptr, st.dref, st.coef, st.bterm,
                                                             st.rptr, st.rref, st.rcol, area, dt, dt_per_cell,
                                                             st.diag, st.dclamp, st.rval);
  return cudaGetLastError();
}

cudaError_t lusgs_apply(ImplicitState& st, const double* v, double* x, cudaStream_t s) {
  SweepArgs f{};
  f.n_levels = st.n_levels_fwd;
  f.level_ptr = st.fwd_level_ptr;
  f.level_cells = st.fwd_level_cells;
  f.row_ptr = st.lower_ptr;
  f.row_col = st.lower_col;
  f.row_val = st.lower_val;
  f.rval = st.rval;
  f.diag = st.diag;
  f.dclamp = st.dclamp;
  f.in = v;
  f.out = st.tmp;
  f.backward = 0;
  void* args_f[] = {&f};
  count_launch(2);
  cudaError_t e = cudaLaunchCooperativeKernel((const void*)k_lusgs_sweep, st.sweep_blocks, kBlock, args_f, 0, s);
  if (e != cudaSuccess) return e;
  SweepArgs b = f;
  b.n_levels = st.n_levels_bwd;
  b.level_ptr = st.bwd_level_ptr;
  b.level_cells = st.bwd_level_cells;
  b.row_ptr = st.upper_ptr;
  b.row_col = st.upper_col;
  b.row_val = st.upper_val;
  b.in = st.tmp;
  b.out = x;
  b.backward = 1;
  void* args_b[] = {&b};
  return cudaLaunchCooperativeKernel((const void*)k_lusgs_sweep, st.sweep_blocks, kBlock, args_b, 0, s);
}

cudaError_t fd_operator(ImplicitState& st, const ResidualFn& residual1, const double* v, double* out,
                        cudaStream_t s) {
  const int C = st.n_cells;
  const long long N = 4LL * C;
  const double* dt = st.dt;
  const int dt_per_cell = st.dt_per_cell;
  cudaError_t e = implicit_dot(st, N, v, v, st.scalars + 0, s);
  count_launch(3);
  k_fd_eps<<<1, 32, 0, s>>>(st.scalars + 0, st.state_norm, st.scalars + 1);
  k_fd_perturb<<<blocks_for(N), kBlock, 0, s>>>(C, st.state, v, st.scalars + 1, st.scale, st.up);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e == cudaSuccess) e = residual1(st.up, st.rp, s);
  k_fd_combine<<<blocks_for(N), kBlock, 0, s>>>(C, v, st.rp, st.rate, st.scalars + 1, st.scale, dt, dt_per_cell, out);
  if (e == cudaSuccess) e = cudaGetLastError();
  return e;
}

static double host_scalar(const double* d, cudaStream_t s, cudaError_t* e) {
  double h = 0.0;
  if (*e == cudaSuccess) *e = cudaMemcpyAsync(&h, d, sizeof(double), cudaMemcpyDeviceToHost, s);
  if (*e == cudaSuccess) *e = cudaStreamSynchronize(s);
  return h;
}

// LAPACK dlartg for finite, well-scaled inputs (Anderson's 2017 algorithm
// as in LAPACK 3.10+): c = |f| / d, r = sign(f) d, s = g / r.
static void lartg(double f, double g, double* c, double* sn, double* r) {
  if (g == 0.0) {
    *c = 1.0;
    *sn = 0.0;
    *r = f;
  } else if (f == 0.0) {
    *c = 0.0;
    *sn = g > 0.0 ? 1.0 : -1.0;
    *r = std::fabs(g);
  } else {
    double d = std::sqrt(f * f + g * g);
    *c = std::fabs(f) / d;
    *r = std::copysign(d, f);
    *sn = g / *r;
  }
}

int gmres_solve(ImplicitState& st, const MatvecFn& matvec, const double* b, double* x, double tol,
                int max_iter, int m, int* iterations, cudaStream_t s) {
  const long long N = 4LL * st.n_cells;
  cudaError_t e = cudaSuccess;
  auto grid = [&](long long n) { return blocks_for(n); };
  // Krylov basis (allocated once per size)
  if ((int)st.krylov.size() < m + 1) {
    for (int k = (int)st.krylov.size(); k < m + 1; ++k) {
      double* p = nullptr;
      e = cudaMalloc((void**)&p, N * sizeof(double));
      if (e != cudaSuccess) return GMRES_CUDA;
      st.krylov.push_back(p);
    }
  }
  double* w = st.w;
  double* av = st.av;
  if (st.hcol_size < m + 3) {
    if (st.hcol) cudaFree(st.hcol);
    st.hcol = nullptr;
    if (cudaMalloc((void**)&st.hcol, (m + 3) * sizeof(double)) != cudaSuccess) return GMRES_CUDA;
    st.hcol_size = m + 3;
  }
  const double eps = 2.220446049250313e-16;
  cudaMemsetAsync(x, 0, N * sizeof(double), s);
  int used = 0;
  *iterations = 0;
  bool x_nonzero = false;
  while (used < max_iter) {
    const int restart = std::min(m, max_iter - used);
    // ---- one SciPy gmres call with maxiter=1 (iterative.py, gmres)
    e = implicit_dot(st, N, b, b, st.scalars + 2, s);
    const double bnrm2 = std::sqrt(host_scalar(st.scalars + 2, s, &e));
    if (e != cudaSuccess) return GMRES_CUDA;
    if (bnrm2 == 0.0) {
      cudaMemcpyAsync(x, b, N * sizeof(double), cudaMemcpyDeviceToDevice, s);
      return GMRES_OK;
    }
    const double atol = tol * bnrm2;
    if (lusgs_apply(st, b, w, s) != cudaSuccess) return GMRES_CUDA;
    e = implicit_dot(st, N, w, w, st.scalars + 3, s);
    const double mb = std::sqrt(host_scalar(st.scalars + 3, s, &e));
    double ptol = mb * std::min(1.0, atol / bnrm2);
    double* r = st.krylov[0];
    if (x_nonzero) {
      if (matvec(x, av, s) != cudaSuccess) return GMRES_CUDA;
      count_launch();
      k_sub<<<grid(N), kBlock, 0, s>>>(N, b, av, r);
    } else {
      cudaMemcpyAsync(r, b, N * sizeof(double), cudaMemcpyDeviceToDevice, s);
    }
    e = implicit_dot(st, N, r, r, st.scalars + 4, s);
    if (std::sqrt(host_scalar(st.scalars + 4, s, &e)) < atol) return GMRES_OK;
    // v0 = psolve(r) / |psolve(r)|
    if (lusgs_apply(st, r, st.krylov[0], s) != cudaSuccess) return GMRES_CUDA;
    e = implicit_dot(st, N, st.krylov[0], st.krylov[0], st.scalars + 5, s);
    const double tmp0 = std::sqrt(host_scalar(st.scalars + 5, s, &e));
    count_launch();
    k_scale<<<grid(N), kBlock, 0, s>>>(N, 1.0 / tmp0, st.krylov[0]);
    std::vector<double> S(restart + 1, 0.0), gc(restart, 0.0), gs(restart, 0.0);
    std::vector<std::vector<double>> h(restart, std::vector<double>(restart + 1, 0.0));
    S[0] = tmp0;
    double presid = 0.0;
    bool breakdown = false;
    int col = 0;
    int inner = 0;
    double* hdev = st.hcol;  // h[col][0..col], then |w|^2 before and after at m+1, m+2
    for (col = 0; col < restart; ++col) {
      if (matvec(st.krylov[col], av, s) != cudaSuccess) return GMRES_CUDA;
      if (lusgs_apply(st, av, w, s) != cudaSuccess) return GMRES_CUDA;
      // modified Gram-Schmidt with device scalars (no host round trip)
      e = implicit_dot(st, N, w, w, hdev + m + 1, s);
      for (int k = 0; k <= col; ++k) {
        implicit_dot(st, N, st.krylov[k], w, hdev + k, s);
        count_launch();
        k_axmy_dev<<<grid(N), kBlock, 0, s>>>(N, hdev + k, st.krylov[k], w);
      }
      e = implicit_dot(st, N, w, w, hdev + m + 2, s);
      std::vector<double> hh(m + 3);
      if (e == cudaSuccess) e = cudaMemcpyAsync(hh.data(), hdev, (m + 3) * sizeof(double), cudaMemcpyDeviceToHost, s);
      if (e == cudaSuccess) e = cudaStreamSynchronize(s);
      if (e != cudaSuccess) return GMRES_CUDA;
      const double h0 = std::sqrt(hh[m + 1]), h1 = std::sqrt(hh[m + 2]);
      for (int k = 0; k <= col; ++k) h[col][k] = hh[k];
      h[col][col + 1] = h1;
      cudaMemcpyAsync(st.krylov[col + 1], w, N * sizeof(double), cudaMemcpyDeviceToDevice, s);
      if (h1 <= eps * h0) {
        h[col][col + 1] = 0.0;
        breakdown = true;
      } else {
        count_launch();
        k_scale<<<grid(N), kBlock, 0, s>>>(N, 1.0 / h1, st.krylov[col + 1]);
      }
      for (int k = 0; k < col; ++k) {
        const double c = gc[k], sn = gs[k];
        const double n0 = h[col][k], n1 = h[col][k + 1];
        h[col][k] = c * n0 + sn * n1;
        h[col][k + 1] = -sn * n0 + c * n1;
      }
      double c, sn, mag;
      lartg(h[col][col], h[col][col + 1], &c, &sn, &mag);
      gc[col] = c;
      gs[col] = sn;
      h[col][col] = mag;
      h[col][col + 1] = 0.0;
      const double t = -sn * S[col];
      S[col] = c * S[col];
      S[col + 1] = t;
      presid = std::fabs(t);
      ++inner;
      if (presid <= ptol || breakdown) break;
    }
    if (col == restart) col = restart - 1;
    // back substitution (upper triangular in h[k][k])
    if (h[col][col] == 0.0) S[col] = 0.0;
    std::vector<double> y(S.begin(), S.begin() + col + 1);
    for (int k = col; k > 0; --k) {
      if (y[k] != 0.0) {
        y[k] /= h[k][k];
        const double tk = y[k];
        for (int j = 0; j < k; ++j) y[j] -= tk * h[k][j];
      }
    }
    if (y[0] != 0.0) y[0] /= h[0][0];
    for (int k = 0; k <= col; ++k) {
      count_launch();
      k_axpy<<<grid(N), kBlock, 0, s>>>(N, y[k], st.krylov[k], x);
    }
    x_nonzero = true;
    if (matvec(x, av, s) != cudaSuccess) return GMRES_CUDA;
    count_launch();
    k_sub<<<grid(N), kBlock, 0, s>>>(N, b, av, st.tmp);
    e = implicit_dot(st, N, st.tmp, st.tmp, st.scalars + 6, s);
    const double rnorm = std::sqrt(host_scalar(st.scalars + 6, s, &e));
    if (e != cudaSuccess) return GMRES_CUDA;
    used += inner;
    *iterations = used;
    if (rnorm <= atol) return GMRES_OK;
    if (inner == 0) break;
  }
  return GMRES_NOT_CONVERGED;
}

cudaError_t implicit_equation(ImplicitState& st, const double* U, const double* U0, const double* R,
                              const double* dt, int dt_per_cell, ScaleVec scale, double* b_out,
                              double* norms_dev, cudaStream_t s) {
  const int C = st.n_cells;
  cudaError_t e = cudaMemsetAsync(norms_dev, 0, 2 * sizeof(double), s);
  count_launch();
  k_equation<<<blocks_for(4LL * C), kBlock, 0, s>>>(C, U, U0, R, dt, dt_per_cell, scale, b_out,
                                                    reinterpret_cast<unsigned long long*>(norms_dev));
  return e == cudaSuccess ? cudaGetLastError() : e;
}

cudaError_t implicit_maxima(ImplicitState& st, const double* U, const double* P, double gamma,
                            double* maxima_dev, cudaStream_t s) {
  const int C = st.n_cells;
  cudaError_t e = cudaMemsetAsync(maxima_dev, 0, 9 * sizeof(double), s);
  count_launch(2);
  k_scale_maxima<<<blocks_for(C), kBlock, 0, s>>>(C, U, P, gamma, reinterpret_cast<unsigned long long*>(maxima_dev));
  k_col3_max<<<blocks_for(C), kBlock, 0, s>>>(C, U, reinterpret_cast<unsigned long long*>(maxima_dev + 8));
  return e == cudaSuccess ? cudaGetLastError() : e;
}

cudaError_t implicit_scaled_sumsq(ImplicitState& st, const double* U, ScaleVec scale, double* out,
                                  cudaStream_t s) {
  count_launch(2);
  k_scaled_sumsq_partial<<<kRedBlocks, kBlock, 0, s>>>(4LL * st.n_cells, U, scale, st.partials);
  k_dot_final<<<1, 32, 0, s>>>(kRedBlocks, st.partials, out);
  return cudaGetLastError();
}

cudaError_t implicit_candidate(int C, const double* U, const double* dx, double damping, ScaleVec scale,
                               double* out, cudaStream_t s) {
  count_launch();
  k_candidate<<<blocks_for(4LL * C), kBlock, 0, s>>>(C, U, dx, damping, scale, out);
  return cudaGetLastError();
}

}  // namespace mcfd
