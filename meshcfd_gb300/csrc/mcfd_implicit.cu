// Implicit Euler building blocks (solver.py:1185-1567) on the device:
//
// * the first-order scalar preconditioner matrix and its LU-SGS application
//   (_implicit_preconditioner, solver.py:1185-1323): diagonal
//   1 + sum dt_i rho_f L / (2 A_i) over interior and periodic faces +
//   dt_i rho L / A_i over boundary faces, off-diagonals -dt_i rho_f L/(2 A_i);
//   the forward solve (D+L) y = v and backward solve (D+U) x = D y run over
//   level sets of the natural-cell-order dependency graph, so the
//   preconditioner is exactly the reference's (only independent rows run
//   concurrently): runs of narrow levels in one block that barriers between
//   levels and keeps the latest solutions in a shared-memory ring, wide
//   levels one grid launch each;
// * the matrix-free operator v -> v - dt [R1(u + eps s v) - R1(u)] / (eps s)
//   (_matrix_free_implicit_operator, solver.py:1532-1567);
// * restarted GMRES(m) as the reference drives SciPy's gmres
//   (_solve_gmres, solver.py:1489-1529): left preconditioning, modified
//   Gram-Schmidt, Givens rotations, SciPy's inner/outer tolerance control.
// Vector reductions are deterministic two-level trees.
#include <climits>
#include <cooperative_groups.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "mcfd_device.cuh"
#include "mcfd_implicit.h"
#include "mcfd_window_plan.h"

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

// ------------------------------------------------------------ LU-SGS sweeps
//
// Row at sweep position p, cell i: x_i = (r_i - sum_j a_ij x_j) / d_i over
// the off-diagonal entries in ascending column order, r = v (forward) or
// D y (backward, D the clamped diagonal); the products and differences round
// one at a time, the quotient is the correctly rounded one.

struct SweepDev {
  const int* level_ptr;
  const int* pos_cell;
  const int* ent_ptr;    // CSR of the rows (entries beyond the packed ones)
  const int* ent_cell;
  const int* ent_pos;
  const int* ent_val;
  const double* rval;
  const int* pk_cnt;
  const int* pk_pos;
  const int* pk_cell;
  const double* pk_val;
  const double* pk_diag;
  const double* pk_dc;
  const double2* pk_row;  // [C][4]: (diagonal, RN(1 / diagonal)), (recip_fixed bits, clamped diagonal), values
  const double* in;
  double* out;
  int backward;
};

constexpr int kWaveThreads = 512;
constexpr int kClusterThreads = 256;
constexpr int kRing = 4096;        // latest solved rows kept in shared memory (128 KiB)
constexpr int kWideLevel = 16384;  // wider levels get a grid launch each
constexpr int kPortableCluster = 8;  // the portable cluster size of the cluster sweep
constexpr int kDefaultEngine = kSweepDataflow;
constexpr size_t kRingBytes = kRing * 4 * sizeof(double);

// Everything of a row that does not depend on the solution: loaded for the
// next level before the block barrier, so a level's critical path is the
// reads of earlier solutions (shared memory) and the row's own arithmetic.
struct SweepRow {
  int i, n;
  St4 r;
  double dg;
  unsigned long long rx;  // recip_fixed(dg): the four quotients share the divisor's reciprocal
  double v[kSweepPack];
  int cp[kSweepPack], cc[kSweepPack];
};

// IM (integer products): the products of the row run on the integer pipe
// (mul_rn, the same IEEE result), which takes them off the FP64 pipe.
template <bool IM = false>
__device__ __forceinline__ void sweep_load(const SweepDev& a, int p, SweepRow& R) {
  R.i = a.pos_cell[p];
  R.n = a.pk_cnt[p];
#pragma unroll
  for (int k = 0; k < kSweepPack; ++k) {
    R.v[k] = a.pk_val[(size_t)p * kSweepPack + k];
    R.cp[k] = a.pk_pos[(size_t)p * kSweepPack + k];
    R.cc[k] = a.pk_cell[(size_t)p * kSweepPack + k];
  }
  R.dg = a.pk_diag[p];
  R.rx = recip_fixed(R.dg);
  const St4 r = ld4(a.in + 4 * (size_t)R.i);
  if (a.backward) {
    const double dc = a.pk_dc[p];
    if constexpr (IM) R.r = St4{mul_rn(dc, r.a), mul_rn(dc, r.b), mul_rn(dc, r.c), mul_rn(dc, r.d)};
    else R.r = St4{dc * r.a, dc * r.b, dc * r.c, dc * r.d};
  } else {
    R.r = r;
  }
}

template <bool IM = false>
__device__ __forceinline__ void sweep_sub(double acc[4], double v, const St4& x) {
  if constexpr (IM) {
    acc[0] = acc[0] - mul_rn(v, x.a);
    acc[1] = acc[1] - mul_rn(v, x.b);
    acc[2] = acc[2] - mul_rn(v, x.c);
    acc[3] = acc[3] - mul_rn(v, x.d);
  } else {
    acc[0] = acc[0] - v * x.a;
    acc[1] = acc[1] - v * x.b;
    acc[2] = acc[2] - v * x.c;
    acc[3] = acc[3] - v * x.d;
  }
}

// x_p = (r - sum_j a_j x_j) / d over the row's entries in ascending column
// order; earlier solutions from the ring when their position is at least
// ring_lo, else from global memory.  Writes the global solution and, when
// ring is given, the ring slot of position p.
template <bool IM = false>
__device__ __forceinline__ void sweep_solve(const SweepDev& a, const SweepRow& R, int p, const double* ring,
                                            int ring_lo, double* ring_out) {
  double acc[4] = {R.r.a, R.r.b, R.r.c, R.r.d};
#pragma unroll
  for (int k = 0; k < kSweepPack; ++k) {
    if (k < R.n) {
      St4 x;
      if (ring && R.cp[k] >= ring_lo) {
        const double* q = ring + 4 * (R.cp[k] & (kRing - 1));
        x = St4{q[0], q[1], q[2], q[3]};
      } else {
        x = ld4(a.out + 4 * (size_t)R.cc[k]);
      }
      sweep_sub<IM>(acc, R.v[k], x);
    }
  }
  if (R.n > kSweepPack) {  // the rest of a long row from the CSR
    for (int j = a.ent_ptr[p] + kSweepPack, j1 = a.ent_ptr[p + 1]; j < j1; ++j) {
      const int cp = a.ent_pos[j];
      St4 x;
      if (ring && cp >= ring_lo) {
        const double* q = ring + 4 * (cp & (kRing - 1));
        x = St4{q[0], q[1], q[2], q[3]};
      } else {
        x = ld4(a.out + 4 * (size_t)a.ent_cell[j]);
      }
      sweep_sub<IM>(acc, a.rval[a.ent_val[j]], x);
    }
  }
  const St4 res{div_rn_recip(acc[0], R.dg, R.rx), div_rn_recip(acc[1], R.dg, R.rx),
                div_rn_recip(acc[2], R.dg, R.rx), div_rn_recip(acc[3], R.dg, R.rx)};
  st4(a.out + 4 * (size_t)R.i, res);
  if (ring_out) {
    double* q = ring_out + 4 * (p & (kRing - 1));
    q[0] = res.a;
    q[1] = res.b;
    q[2] = res.c;
    q[3] = res.d;
  }
}

// Levels [l0, l1) in one block: rows of a level in parallel, a block barrier
// between levels, the next level's rows loaded before the barrier.  The
// solutions of the last kRing positions stay in shared memory (slot =
// position mod kRing); position p' is read from there when p' >= max(end of
// the current level - kRing, first position of the launch), which no row of
// the current level can overwrite.
__global__ void __launch_bounds__(kWaveThreads, 1) k_lusgs_wavefront(SweepDev a, int l0, int l1) {
  extern __shared__ double ring[];  // [kRing][4]
  const int base = a.level_ptr[l0];
  const int t = threadIdx.x;
  SweepRow R;
  int b = base, e = a.level_ptr[l0 + 1];
  bool have = b + t < e;
  if (have) sweep_load(a, b + t, R);
  for (int l = l0; l < l1; ++l) {
    const int lo = max(e - kRing, base);
    if (have) sweep_solve(a, R, b + t, ring, lo, ring);
    for (int p = b + t + (int)blockDim.x; p < e; p += blockDim.x) {  // levels wider than the block
      SweepRow W;
      sweep_load(a, p, W);
      sweep_solve(a, W, p, ring, lo, ring);
    }
    // the next level's rows, independent of this level's solutions
    if (l + 1 < l1) {
      b = e;
      e = a.level_ptr[l + 2];
      have = b + t < e;
      if (have) sweep_load(a, b + t, R);
    }
    __syncthreads();
  }
}

// The same sweep over a thread-block cluster of NC blocks (one per SM): the
// rows of a level are dealt out round robin (row b + rank + NC t in block
// `rank`), every block stores each solution it computes into the rings of
// all NC blocks (distributed shared memory), and a cluster barrier with
// release / acquire semantics separates the levels.  Reads of earlier
// solutions are local shared-memory loads, or, outside the ring, loads that
// bypass L1 (another block of the cluster may have written the line).  A
// level's FP64 work is split over NC SMs, which is what bounds the
// single-block sweep on narrow levels of a few hundred rows.
__device__ __forceinline__ St4 ld4_cg(const double* p) {
  const double2 a = __ldcg(reinterpret_cast<const double2*>(p));
  const double2 b = __ldcg(reinterpret_cast<const double2*>(p) + 1);
  return St4{a.x, a.y, b.x, b.y};
}

template <int NC>
__global__ void __launch_bounds__(kClusterThreads, 1) k_lusgs_cluster(SweepDev a, int l0, int l1) {
  extern __shared__ double ring[];  // [kRing][4], the same contents in every block of the cluster
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank();
  double* rings[NC];
#pragma unroll
  for (int r = 0; r < NC; ++r) rings[r] = cluster.map_shared_rank(ring, r);
  cluster.sync();  // every block is running before any remote store
  const int base = a.level_ptr[l0];
  const int stride = NC * (int)blockDim.x;
  const int first = rank + NC * (int)threadIdx.x;
  SweepRow R;
  int b = base, e = a.level_ptr[l0 + 1];
  bool have = b + first < e;
  if (have) sweep_load(a, b + first, R);
  auto solve = [&](const SweepRow& W, int p, int lo) {
    double acc[4] = {W.r.a, W.r.b, W.r.c, W.r.d};
#pragma unroll
    for (int k = 0; k < kSweepPack; ++k) {
      if (k < W.n) {
        St4 x;
        if (W.cp[k] >= lo) {
          const double* q = ring + 4 * (W.cp[k] & (kRing - 1));
          x = St4{q[0], q[1], q[2], q[3]};
        } else {
          x = ld4_cg(a.out + 4 * (size_t)W.cc[k]);
        }
        sweep_sub(acc, W.v[k], x);
      }
    }
    if (W.n > kSweepPack) {
      for (int j = a.ent_ptr[p] + kSweepPack, j1 = a.ent_ptr[p + 1]; j < j1; ++j) {
        const int cp = a.ent_pos[j];
        St4 x;
        if (cp >= lo) {
          const double* q = ring + 4 * (cp & (kRing - 1));
          x = St4{q[0], q[1], q[2], q[3]};
        } else {
          x = ld4_cg(a.out + 4 * (size_t)a.ent_cell[j]);
        }
        sweep_sub(acc, a.rval[a.ent_val[j]], x);
      }
    }
    const St4 res{div_rn_recip(acc[0], W.dg, W.rx), div_rn_recip(acc[1], W.dg, W.rx),
                  div_rn_recip(acc[2], W.dg, W.rx), div_rn_recip(acc[3], W.dg, W.rx)};
    st4(a.out + 4 * (size_t)W.i, res);
    const int slot = 4 * (p & (kRing - 1));
#pragma unroll
    for (int r = 0; r < NC; ++r) {
      double* q = rings[r] + slot;
      q[0] = res.a;
      q[1] = res.b;
      q[2] = res.c;
      q[3] = res.d;
    }
  };
  for (int l = l0; l < l1; ++l) {
    const int lo = max(e - kRing, base);
    if (have) solve(R, b + first, lo);
    for (int p = b + first + stride; p < e; p += stride) {
      SweepRow W;
      sweep_load(a, p, W);
      solve(W, p, lo);
    }
    if (l + 1 < l1) {
      b = e;
      e = a.level_ptr[l + 2];
      have = b + first < e;
      if (have) sweep_load(a, b + first, R);
    }
    cluster.sync();
  }
}

// The windowed band sweep (SweepWindows): block k of a thread-block
// cluster owns a band of consecutive cell ids.  Per window of levels it
// solves, level by level with a block barrier between levels, its own rows
// and the rows of other bands they depend on inside the window (the same
// arithmetic on the same inputs: the same bits as their owners'), reading
// the solutions from before the window ("externals") from global memory
// once, at the window's start, into shared-memory slots.  Only the rows a
// block owns go to global memory; a cluster barrier (release / acquire) at
// each window's start makes the previous window's rows visible to every
// block.  Everything else a window reads is staged into shared memory by
// asynchronous copies issued one window ahead: the window's row records
// (32 bytes: position, cell, slot, entry count, entry slots), its rows'
// values (64 bytes) and right-hand sides (32 bytes, times the clamped
// diagonal in the backward sweep), both copied per record by k_pack_window
// before each sweep, its externals (slot, cell) and level ranges, each
// contiguous per (window, block) in the plan.  So a level reads shared
// memory only.  Each row is solved by four lanes, one per component (warps
// 4 h + c hold component c of rows 32 h .. 32 h + 31), so a level's
// critical path holds a row's products and differences per entry once.  The
// arithmetic is sweep_solve's, component by component: the same bits.  No
// thread waits on a flag; every thread of every block passes the same
// barriers.
constexpr int kWinThreads = 256;                 // 8 warps: 64 rows of 4 components per pass
constexpr int kWinRowsPerPass = kWinThreads / 4;
constexpr int kWinMaxLevels = 32;                // levels per window at most
constexpr int kWinMaxSlots = 2048;               // shared-memory solution slots of 4 doubles (64 KiB)
constexpr int kWinMaxRows = 560;                 // row records per (window, block)
constexpr int kWinMaxExt = 512;                  // externals per (window, block)
constexpr int kWinRecBytes = 32, kWinRowBytes = 64, kWinRhsBytes = 32;
constexpr int kWinStageBytes = kWinMaxRows * (kWinRecBytes + kWinRowBytes + kWinRhsBytes) + kWinMaxExt * 8;
constexpr int kWinSmemBytes = kWinMaxSlots * 32 + 2 * kWinStageBytes;
static_assert(kWinSmemBytes + 2 * (kWinMaxLevels + 1) * 4 <= 227 * 1024, "the windowed sweep's shared memory");

struct WinDev {
  const int *l0, *l1, *gbase, *grp, *eslot;
  const int4* stage;    // [window * nc + block]: first record, records, first external, externals
  const int4* rec;      // [2 per record]
  const double2* row;   // [4 per record]
  const double* rhs;    // [4 per record]
  const int2* ext;      // (slot, cell) per external
};

__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"((unsigned)__cvta_generic_to_shared(dst)), "l"(src)
               : "memory");
}
__device__ __forceinline__ void cp_async8(void* dst, const void* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"((unsigned)__cvta_generic_to_shared(dst)), "l"(src)
               : "memory");
}
__device__ __forceinline__ void cp_async4(void* dst, const void* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"((unsigned)__cvta_generic_to_shared(dst)), "l"(src)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// One window's staging for this block: row records, values, right-hand
// sides, externals (buffer at st) and level ranges (gr).
struct WinStage {
  int nl, g0;  // levels; index of the first level range in w.grp
  int4 info;   // first record, records, first external, externals
};

__device__ __forceinline__ void win_stage_info(const WinDev& w, int win, int rank, int nc, WinStage& S) {
  const int nl = w.l1[win] - w.l0[win];
  S.nl = nl;
  S.g0 = w.gbase[win] + rank * (nl + 1);
  S.info = w.stage[win * nc + rank];
}

__device__ __forceinline__ void win_stage_copy(const WinDev& w, const WinStage& S, unsigned char* st, int* gr) {
  const int t = (int)threadIdx.x;
  const int r0 = S.info.x, nr = S.info.y, e0 = S.info.z, ne = S.info.w;
  for (int c = t; c < 2 * nr; c += kWinThreads)
    cp_async16(st + 16 * c, reinterpret_cast<const unsigned char*>(w.rec + 2 * (size_t)r0) + 16 * c);
  unsigned char* row = st + kWinMaxRows * kWinRecBytes;
  for (int c = t; c < 4 * nr; c += kWinThreads)
    cp_async16(row + 16 * c, reinterpret_cast<const unsigned char*>(w.row + 4 * (size_t)r0) + 16 * c);
  unsigned char* rhs = row + kWinMaxRows * kWinRowBytes;
  for (int c = t; c < 2 * nr; c += kWinThreads)
    cp_async16(rhs + 16 * c, reinterpret_cast<const unsigned char*>(w.rhs + 4 * (size_t)r0) + 16 * c);
  unsigned char* ext = rhs + kWinMaxRows * kWinRhsBytes;
  for (int c = t; c < ne; c += kWinThreads) cp_async8(ext + 8 * c, w.ext + e0 + c);
  if (t <= S.nl) cp_async4(gr + t, w.grp + S.g0 + t);
}

__device__ __forceinline__ void win_solve(const SweepDev& a, const WinDev& w, double* sl, const unsigned char* st,
                                          int r, int comp) {
  const int4* rec = reinterpret_cast<const int4*>(st);
  const double2* row = reinterpret_cast<const double2*>(st + kWinMaxRows * kWinRecBytes);
  const double* rhs = reinterpret_cast<const double*>(st + kWinMaxRows * (kWinRecBytes + kWinRowBytes));
  const int4 A = rec[2 * r], B = rec[2 * r + 1];
  const double2 d0 = row[4 * r], d2 = row[4 * r + 2], d3 = row[4 * r + 3];
  const double rx_bits = row[4 * r + 1].x;
  const int n = A.z >> 16, slot = A.z & 0xffff;
  double acc = rhs[4 * r + comp];
  const int es[kSweepPack] = {B.x, B.y, B.z, B.w};
  const double v[kSweepPack] = {d2.x, d2.y, d3.x, d3.y};
#pragma unroll
  for (int k = 0; k < kSweepPack; ++k)
    if (k < n) acc = acc - v[k] * sl[4 * es[k] + comp];
  if (n > kSweepPack) {  // the rest of a long row: values from the CSR, slots from the plan
    const int p = A.x >= 0 ? A.x : ~A.x;
    const int j0 = a.ent_ptr[p];
    for (int k = kSweepPack; k < n; ++k) acc = acc - a.rval[a.ent_val[j0 + k]] * sl[4 * w.eslot[A.w + k] + comp];
  }
  // the quotient from the row's reciprocal: the same bits as div_rn in
  // fewer dependent steps (div_rn_fma), the level's critical path
  const double res = div_rn_fma(acc, d0.x, d0.y, (unsigned long long)__double_as_longlong(rx_bits));
  sl[4 * slot + comp] = res;
  if (A.x >= 0) a.out[4 * (size_t)A.y + comp] = res;
}

template <int NC>
__global__ void __launch_bounds__(kWinThreads, 1) k_lusgs_window(SweepDev a, WinDev w, int w0, int w1) {
  extern __shared__ __align__(16) unsigned char smem[];
  double* sl = reinterpret_cast<double*>(smem);  // [kWinMaxSlots][4]
  unsigned char* stg = smem + kWinMaxSlots * 32;  // two staging buffers
  __shared__ int grp[2][kWinMaxLevels + 1];      // level ranges (record indices) of the staged windows
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank();
  const int comp = ((int)threadIdx.x >> 5) & 3;
  const int rl = (((int)threadIdx.x >> 7) << 5) | ((int)threadIdx.x & 31);  // row of the pass
  WinStage cur, nxt;
  win_stage_info(w, w0, rank, NC, cur);
  win_stage_copy(w, cur, stg, grp[0]);
  cp_async_commit();
  if (w0 + 1 < w1) win_stage_info(w, w0 + 1, rank, NC, nxt);
  for (int win = w0; win < w1; ++win) {
    const int buf = (win - w0) & 1;
    const unsigned char* st = stg + buf * kWinStageBytes;
    cp_async_wait<0>();  // this window's copies have landed
    cluster.sync();      // every thread's copies are visible; the rows solved before this window are in global memory
    const int2* ext = reinterpret_cast<const int2*>(st + kWinMaxRows * (kWinRecBytes + kWinRowBytes + kWinRhsBytes));
    for (int x = rl; x < cur.info.w; x += kWinRowsPerPass) {
      const int2 e = ext[x];
      sl[4 * e.x + comp] = __ldcg(a.out + 4 * (size_t)e.y + comp);
    }
    // the next window's staging, into the buffer the previous window read
    // (every thread passed that window's last barrier), in flight while this
    // window is solved
    WinStage after;
    if (win + 1 < w1) {
      win_stage_copy(w, nxt, stg + (buf ^ 1) * kWinStageBytes, grp[buf ^ 1]);
      cp_async_commit();
      if (win + 2 < w1) win_stage_info(w, win + 2, rank, NC, after);
    }
    __syncthreads();
    const int r0 = cur.info.x;
    for (int m = 0; m < cur.nl; ++m) {
      for (int r = grp[buf][m] - r0 + rl, r1 = grp[buf][m + 1] - r0; r < r1; r += kWinRowsPerPass)
        win_solve(a, w, sl, st, r, comp);
      __syncthreads();
    }
    cur = nxt;
    nxt = after;
  }
}

// Before a windowed sweep: each window record's 64-byte row (its
// position's, as the last assembly left it) and its right-hand side, times
// the clamped diagonal in the backward sweep (sweep_load's r).
__global__ void k_pack_window(int n, const int4* __restrict__ rec, const double2* __restrict__ pk_row,
                              const double* __restrict__ in, int backward, double2* __restrict__ row,
                              double* __restrict__ rhs) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  const int4 A = rec[2 * (size_t)r];
  const int p = A.x >= 0 ? A.x : ~A.x;
  double2 q[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    q[k] = pk_row[4 * (size_t)p + k];
    row[4 * (size_t)r + k] = q[k];
  }
  const St4 v = ld4(in + 4 * (size_t)A.y);
  const double dc = q[1].y;
  st4(rhs + 4 * (size_t)r, backward ? St4{dc * v.a, dc * v.b, dc * v.c, dc * v.d} : v);
}

// The same sweep in one block without a barrier per level: the rows are cut
// into chunks of at most 32 (by default) consecutive positions inside one
// level, chunk k
// goes to warp k mod kFlowWarps, and each warp works through its chunks in
// order.  A row waits only for the rows it reads: every solved row writes its
// solution into a shared-memory ring of kFlowRing positions and then the
// position into the slot's tag; a reader spins (bounded) until the tag of
// each earlier position it needs equals that position.  A warp starts a
// chunk only when every position more than kFlowAhead before its first row
// is solved (each warp publishes the first position of its current chunk),
// which (i) keeps a ring slot from being overwritten while a reader may still
// need it (a position is read from the ring only within 2048 positions, and
// the writer of that slot's next position waits for the reader's chunk) and
// (ii) makes every older position readable from global memory.  So narrow
// levels no longer wait for the whole previous level, and chunks of
// consecutive levels are in flight at once.  The oldest unfinished chunk can
// always proceed (its rows depend on earlier levels only, all solved), so
// the waits end; each one is bounded anyway, after which the block flags
// MCFD_S_SWEEP_TIMEOUT and every warp stops.  The arithmetic of each row is
// sweep_solve's, so the results equal the other schedules' bit for bit.
constexpr int kFlowRing = 4096;  // positions
constexpr int kFlowAhead = 2016;  // positions below start - kFlowAhead are solved when a chunk starts
constexpr int kFlowRingWindow = kFlowRing - kFlowAhead - 32;  // ring reads within this distance
constexpr long long kFlowSpinLimit = 1LL << 22;
constexpr int kFlowChunk = 32;  // default rows per chunk
constexpr size_t kFlowSmemBytes = kFlowRing * (4 * sizeof(double) + sizeof(int));
static_assert(kFlowRing >= 2 * kFlowAhead + 32, "ring reads must fall inside the guaranteed window");

template <int NT, bool IM>
__global__ void __launch_bounds__(NT, 1) k_lusgs_dataflow(SweepDev a, const int2* __restrict__ chunks, int k0, int k1,
                                                          DevStatus* status) {
  constexpr int kFlowWarps = NT / 32;
  extern __shared__ double flow_smem[];
  double* ring = flow_smem;                                      // [kFlowRing][4]
  volatile int* tag = reinterpret_cast<volatile int*>(ring + 4 * kFlowRing);  // [kFlowRing]
  __shared__ int prog[kFlowWarps];  // first position of each warp's current chunk (INT_MAX: none left)
  __shared__ int abort_flag;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int i = threadIdx.x; i < kFlowRing; i += blockDim.x) tag[i] = -1;
  if (lane == 0) prog[warp] = k0 + warp < k1 ? chunks[k0 + warp].x : INT_MAX;
  if (threadIdx.x == 0) abort_flag = 0;
  __syncthreads();
  volatile int* vprog = prog;
  volatile int* vabort = &abort_flag;
  const int base = chunks[k0].x;  // positions below were solved by earlier launches
  for (int k = k0 + warp; k < k1; k += kFlowWarps) {
    const int2 ch = chunks[k];
    const int start = ch.x;
    const bool have = lane < ch.y;
    const int p = start + lane;
    SweepRow R;
    if (have) sweep_load<IM>(a, p, R);
    // throttle: every position below start - kFlowAhead solved
    if (start - kFlowAhead > base) {  // warp-uniform loop: every exit is decided by the whole warp
      long long spins = 0;
      while (true) {
        const int v = lane < kFlowWarps ? vprog[lane] : INT_MAX;
        if (__reduce_min_sync(0xffffffffu, v) >= start - kFlowAhead) break;
        if (__any_sync(0xffffffffu, ++spins > kFlowSpinLimit || *vabort)) {
          if (lane == 0) *vabort = 1;
          break;
        }
      }
    }
    if (__any_sync(0xffffffffu, *vabort)) break;
    const int ring_lo = max(start - kFlowRingWindow, base);
    bool ok = true;
    if (have) {
      // wait for the tags of the ring-resident positions this row reads
      auto wait_tag = [&](int cp) {
        if (cp < ring_lo) return;
        long long spins = 0;
        while (tag[cp & (kFlowRing - 1)] != cp) {
          if (++spins > kFlowSpinLimit || *vabort) {
            ok = false;
            return;
          }
        }
      };
#pragma unroll
      for (int q = 0; q < kSweepPack; ++q)
        if (q < R.n && ok) wait_tag(R.cp[q]);
      if (R.n > kSweepPack)
        for (int j = a.ent_ptr[p] + kSweepPack, j1 = a.ent_ptr[p + 1]; j < j1 && ok; ++j) wait_tag(a.ent_pos[j]);
    }
    if (__any_sync(0xffffffffu, !ok)) {
      if (lane == 0) *vabort = 1;
      break;
    }
    __threadfence_block();  // the solutions behind the tags seen above
    if (have) {
      sweep_solve<IM>(a, R, p, ring, ring_lo, ring);
      __threadfence_block();
      tag[p & (kFlowRing - 1)] = p;
    }
    __syncwarp();
    if (lane == 0) {
      __threadfence_block();
      vprog[warp] = k + kFlowWarps < k1 ? chunks[k + kFlowWarps].x : INT_MAX;
    }
  }
  __syncthreads();
  if (threadIdx.x == 0 && abort_flag) {
    atomicOr(&status->code, MCFD_S_SWEEP_TIMEOUT);
  }
}

// The same per-row-wait sweep with one lane per (row, component): a chunk of
// at most 8 rows takes a warp, lane 4 r + v solving component v of the
// chunk's row r.  The FP64 work of a level is the same number of warp
// instructions as with one lane per row, but it is spread over four times as
// many warps (all four SM sub-partitions take part on narrow levels), and a
// row's dependent chain is its own component's products and differences
// only, so the time from a row's last input to its solution is about a
// quarter.  The ring, tags, throttle and bounds are k_lusgs_dataflow's; a
// row's tag is written once all four of its components are stored.  The
// component arithmetic is sweep_solve's, so the bits are the same.
template <int NT>
__global__ void __launch_bounds__(NT, 1) k_lusgs_dataflow_comp(SweepDev a, const int2* __restrict__ chunks, int k0,
                                                               int k1, DevStatus* status) {
  constexpr int kFlowWarps = NT / 32;
  extern __shared__ double flow_smem[];
  double* ring = flow_smem;                                                   // [kFlowRing][4]
  volatile int* tag = reinterpret_cast<volatile int*>(ring + 4 * kFlowRing);  // [kFlowRing]
  __shared__ int prog[kFlowWarps];
  __shared__ int abort_flag;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int rl = lane >> 2, v = lane & 3;  // row of the chunk, component
  for (int i = threadIdx.x; i < kFlowRing; i += blockDim.x) tag[i] = -1;
  if (lane == 0) prog[warp] = k0 + warp < k1 ? chunks[k0 + warp].x : INT_MAX;
  if (threadIdx.x == 0) abort_flag = 0;
  __syncthreads();
  volatile int* vprog = prog;
  volatile int* vabort = &abort_flag;
  const int base = chunks[k0].x;
  for (int k = k0 + warp; k < k1; k += kFlowWarps) {
    const int2 ch = chunks[k];
    const int start = ch.x;
    const bool have = rl < ch.y;
    const int p = start + rl;
    // the row's data (independent of the solutions)
    int i = 0, n = 0;
    double r = 0.0, dg = 1.0, vk[kSweepPack];
    int cp[kSweepPack], cc[kSweepPack];
    unsigned long long rx = 0;
    if (have) {
      i = a.pos_cell[p];
      n = a.pk_cnt[p];
#pragma unroll
      for (int q = 0; q < kSweepPack; ++q) {
        vk[q] = a.pk_val[(size_t)p * kSweepPack + q];
        cp[q] = a.pk_pos[(size_t)p * kSweepPack + q];
        cc[q] = a.pk_cell[(size_t)p * kSweepPack + q];
      }
      dg = a.pk_diag[p];
      rx = recip_fixed(dg);
      const double in = a.in[4 * (size_t)i + v];
      r = a.backward ? a.pk_dc[p] * in : in;
    }
    if (start - kFlowAhead > base) {  // warp-uniform loop, as in k_lusgs_dataflow
      long long spins = 0;
      while (true) {
        const int pv = lane < kFlowWarps ? vprog[lane] : INT_MAX;
        if (__reduce_min_sync(0xffffffffu, pv) >= start - kFlowAhead) break;
        if (__any_sync(0xffffffffu, ++spins > kFlowSpinLimit || *vabort)) {
          if (lane == 0) *vabort = 1;
          break;
        }
      }
    }
    if (__any_sync(0xffffffffu, *vabort)) break;
    const int ring_lo = max(start - kFlowRingWindow, base);
    bool ok = true;
    if (have) {
      auto wait_tag = [&](int dep) {
        if (dep < ring_lo) return;
        long long spins = 0;
        while (tag[dep & (kFlowRing - 1)] != dep) {
          if (++spins > kFlowSpinLimit || *vabort) {
            ok = false;
            return;
          }
        }
      };
#pragma unroll
      for (int q = 0; q < kSweepPack; ++q)
        if (q < n && ok) wait_tag(cp[q]);
      if (n > kSweepPack)
        for (int j = a.ent_ptr[p] + kSweepPack, j1 = a.ent_ptr[p + 1]; j < j1 && ok; ++j) wait_tag(a.ent_pos[j]);
    }
    if (__any_sync(0xffffffffu, !ok)) {
      if (lane == 0) *vabort = 1;
      break;
    }
    __threadfence_block();
    if (have) {
      double acc = r;
#pragma unroll
      for (int q = 0; q < kSweepPack; ++q) {
        if (q < n) {
          const double x = cp[q] >= ring_lo ? ring[4 * (cp[q] & (kFlowRing - 1)) + v] : a.out[4 * (size_t)cc[q] + v];
          acc = acc - vk[q] * x;
        }
      }
      if (n > kSweepPack) {
        for (int j = a.ent_ptr[p] + kSweepPack, j1 = a.ent_ptr[p + 1]; j < j1; ++j) {
          const int dep = a.ent_pos[j];
          const double x = dep >= ring_lo ? ring[4 * (dep & (kFlowRing - 1)) + v] : a.out[4 * (size_t)a.ent_cell[j] + v];
          acc = acc - a.rval[a.ent_val[j]] * x;
        }
      }
      const double res = div_rn_recip(acc, dg, rx);
      a.out[4 * (size_t)i + v] = res;
      ring[4 * (p & (kFlowRing - 1)) + v] = res;
    }
    __threadfence_block();  // each lane's component before the row's tag
    __syncwarp();
    __threadfence_block();
    if (have && v == 0) tag[p & (kFlowRing - 1)] = p;
    __syncwarp();
    if (lane == 0) {
      __threadfence_block();
      vprog[warp] = k + kFlowWarps < k1 ? chunks[k + kFlowWarps].x : INT_MAX;
    }
  }
  __syncthreads();
  if (threadIdx.x == 0 && abort_flag) atomicOr(&status->code, MCFD_S_SWEEP_TIMEOUT);
}

// One wide level over the whole grid (earlier levels finished in earlier
// launches on the same stream).
__global__ void __launch_bounds__(kBlock) k_lusgs_level(SweepDev a, int b, int e) {
  const int p = b + blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= e) return;
  SweepRow R;
  sweep_load(a, p, R);
  sweep_solve(a, R, p, nullptr, 0, nullptr);
}

// Values of the packed rows after an assembly: the entries' matrix values,
// the diagonal and the clamped diagonal in sweep order.
__global__ void k_pack_rows(int C, const int* __restrict__ pos_cell, const int* __restrict__ ent_ptr,
                            const int* __restrict__ ent_val, const double* __restrict__ rval,
                            const double* __restrict__ diag, const double* __restrict__ dclamp,
                            double* __restrict__ pk_val, double* __restrict__ pk_diag, double* __restrict__ pk_dc,
                            double2* __restrict__ pk_row) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= C) return;
  const int i = pos_cell[p];
  const int j0 = ent_ptr[p], n = ent_ptr[p + 1] - j0;
  double v[kSweepPack];
#pragma unroll
  for (int k = 0; k < kSweepPack; ++k) {
    v[k] = k < n ? rval[ent_val[j0 + k]] : 0.0;
    pk_val[(size_t)p * kSweepPack + k] = v[k];
  }
  const double d = diag[i], dc = dclamp[i];
  pk_diag[p] = d;
  pk_dc[p] = dc;
  // one 64-byte row for the windowed sweep, with the divisor's reciprocals
  // for its quotients (div_rn_fma)
  const unsigned long long X = recip_fixed(d);
  static_assert(kSweepPack == 4, "the windowed sweep's row holds four values");
  pk_row[4 * (size_t)p] = make_double2(d, div_rn_recip(1.0, d, X));
  pk_row[4 * (size_t)p + 1] = make_double2(__longlong_as_double((long long)X), dc);
  pk_row[4 * (size_t)p + 2] = make_double2(v[0], v[1]);
  pk_row[4 * (size_t)p + 3] = make_double2(v[2], v[3]);
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

// r = b - x
__global__ void k_sub(long long n, const double* __restrict__ b, const double* __restrict__ x,
                      double* __restrict__ r) {
  long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i < n) r[i] = b[i] - x[i];
}

// ------------------------------------------------------------- FD operator

// eps = sqrt(machine eps) * max(1, |u/s|) / |v|  (solver.py:1546-1561);
// |u/s| = sqrt of the prepared sum of squares
__global__ void k_fd_eps(const double* __restrict__ v_sumsq, const double* __restrict__ state_sumsq,
                         double* eps_out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    const double dn = sqrt_rn(v_sumsq[0]);
    const double state_norm = sqrt_rn(state_sumsq[0]);
    const double fd = 1.4901161193847656e-08;  // math.sqrt(np.finfo(float).eps)
    eps_out[0] = (dn == 0.0) ? 0.0 : div_rn(fd * (state_norm > 1.0 ? state_norm : 1.0), dn);
  }
}

// U_p = u + (eps * s_k) * v
__global__ void k_fd_perturb(int C, const double* __restrict__ u, const double* __restrict__ v,
                             const double* __restrict__ eps, const double* __restrict__ scale,
                             double* __restrict__ up) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 4 * C) return;
  const double e = eps[0];
  up[i] = u[i] + (e * scale[i & 3]) * v[i];
}

// out = v - dt * ((R_p - R) / eps) / s_k ; out = v when |v| = 0
__global__ void k_fd_combine(int C, const double* __restrict__ v, const double* __restrict__ rp,
                             const double* __restrict__ rate, const double* __restrict__ eps,
                             const double* __restrict__ scale, const double* __restrict__ dt, int dt_per_cell,
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
  out[i] = v[i] - div_rn(d * jv, scale[i & 3]);
}

__global__ void k_set_scale(ScaleVec s, double* __restrict__ out) {
  if (threadIdx.x < 4) out[threadIdx.x] = s.v[threadIdx.x];
}

// ------------------------------------------------------- GMRES on the device

// Deterministic grid dot product inside a cooperative kernel: block partials
// (grid-stride sums, shared-memory tree) into one of two buffers, a grid
// barrier, then every block adds the partials in the same fixed order (32
// strided lane sums and a shuffle tree).  Alternating buffers make one
// barrier per product enough: a block reads buffer k only before it reaches
// the barrier of product k + 1.
__device__ double grid_dot(cg::grid_group& grid, const double* __restrict__ x, const double* __restrict__ y,
                           long long n, double* __restrict__ partials, int& buf, double* sh) {
  double acc = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    acc += x[i] * y[i];
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int w = kBlock / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  double* part = partials + (size_t)buf * gridDim.x;
  if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
  buf ^= 1;
  grid.sync();
  if (threadIdx.x < 32) {
    double t = 0.0;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += 32) t += part[b];
    for (int off = 16; off > 0; off >>= 1) t += __shfl_down_sync(0xffffffffu, t, off);
    if (threadIdx.x == 0) sh[kBlock] = t;
  }
  __syncthreads();
  const double total = sh[kBlock];
  __syncthreads();
  return total;
}

// Modified Gram-Schmidt of w against basis vectors 0..col (col from the
// cycle state): hcol[k] = <v_k, w> then w -= hcol[k] v_k, in order;
// hcol[m + 1] = |w|^2 before, hcol[m + 2] = |w|^2 after.  Each thread
// updates the entries its grid-stride dot products read, so only the
// reductions need the grid barrier.
struct MgsArgs {
  const double* basis;
  long long n;
  double* w;
  const GmresCycle* cycle;
  double* hcol;
  int m;
  double* partials;  // [2][gridDim.x]
};

__global__ void __launch_bounds__(kBlock) k_mgs(MgsArgs a) {
  cg::grid_group grid = cg::this_grid();
  __shared__ double sh[kBlock + 1];
  int buf = 0;
  const int col = a.cycle->col;
  const double before = grid_dot(grid, a.w, a.w, a.n, a.partials, buf, sh);
  if (blockIdx.x == 0 && threadIdx.x == 0) a.hcol[a.m + 1] = before;
  for (int k = 0; k <= col; ++k) {
    const double* v = a.basis + (size_t)k * a.n;
    const double h = grid_dot(grid, v, a.w, a.n, a.partials, buf, sh);
    if (blockIdx.x == 0 && threadIdx.x == 0) a.hcol[k] = h;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < a.n; i += (long long)gridDim.x * blockDim.x)
      a.w[i] = a.w[i] - h * v[i];
  }
  const double after = grid_dot(grid, a.w, a.w, a.n, a.partials, buf, sh);
  if (blockIdx.x == 0 && threadIdx.x == 0) a.hcol[a.m + 2] = after;
}

// LAPACK dlartg for finite, well-scaled inputs (Anderson's 2017 algorithm
// as in LAPACK 3.10+): c = |f| / d, r = sign(f) d, s = g / r.
__device__ void lartg_dev(double f, double g, double* c, double* sn, double* r) {
  if (g == 0.0) {
    *c = 1.0;
    *sn = 0.0;
    *r = f;
  } else if (f == 0.0) {
    *c = 0.0;
    *sn = g > 0.0 ? 1.0 : -1.0;
    *r = fabs(g);
  } else {
    const double d = sqrt(f * f + g * g);
    *c = fabs(f) / d;
    *r = copysign(d, f);
    *sn = g / *r;
  }
}

// SciPy's inner-loop bookkeeping for column col (iterative.py, gmres):
// Hessenberg column from the Gram-Schmidt products, breakdown test
// h1 <= eps h0, the previous rotations applied, a new rotation, the
// residual estimate |S[col + 1]|, and the stop decision; sets the while
// condition of the captured inner loop when ``handle`` is given.
__global__ void k_givens(GmresCycle* cyc, const double* __restrict__ hcol, double* __restrict__ hess,
                         double* __restrict__ givens, int m, cudaGraphConditionalHandle handle, int use_handle) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const int col = cyc->col;
  double* H = hess + (size_t)col * (m + 1);
  double* gc = givens;
  double* gs = givens + m;
  double* S = givens + 2 * m;
  const double eps = 2.220446049250313e-16;
  const double h0 = sqrt(hcol[m + 1]), h1 = sqrt(hcol[m + 2]);
  for (int k = 0; k <= col; ++k) H[k] = hcol[k];
  H[col + 1] = h1;
  int breakdown = 0;
  double inv = 1.0;
  if (h1 <= eps * h0) {
    H[col + 1] = 0.0;
    breakdown = 1;
  } else {
    inv = 1.0 / h1;
  }
  for (int k = 0; k < col; ++k) {
    const double c = gc[k], sn = gs[k];
    const double n0 = H[k], n1 = H[k + 1];
    H[k] = c * n0 + sn * n1;
    H[k + 1] = -sn * n0 + c * n1;
  }
  double c, sn, mag;
  lartg_dev(H[col], H[col + 1], &c, &sn, &mag);
  gc[col] = c;
  gs[col] = sn;
  H[col] = mag;
  H[col + 1] = 0.0;
  const double t = -sn * S[col];
  S[col] = c * S[col];
  S[col + 1] = t;
  const double presid = fabs(t);
  cyc->presid = presid;
  cyc->inv_h1 = inv;
  cyc->breakdown = breakdown;
  cyc->last = col;
  cyc->inner = cyc->inner + 1;
  cyc->col = col + 1;
  const int done = (presid <= cyc->ptol) || breakdown || (col + 1 >= cyc->restart);
  cyc->done = done;
  if (use_handle) cudaGraphSetConditional(handle, done ? 0u : 1u);
}

// vcur = basis[col]
__global__ void k_take_column(const double* __restrict__ basis, long long n, const GmresCycle* cyc,
                              double* __restrict__ vcur) {
  const double* v = basis + (size_t)cyc->col * n;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    vcur[i] = v[i];
}

// basis[last + 1] = w * inv_h1 (w unscaled at breakdown)
__global__ void k_next_basis(double* __restrict__ basis, long long n, const GmresCycle* cyc,
                             const double* __restrict__ w) {
  double* v = basis + (size_t)(cyc->last + 1) * n;
  const int scale = !cyc->breakdown;
  const double inv = cyc->inv_h1;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    v[i] = scale ? w[i] * inv : w[i];
}

// start of a restart cycle: S = (|z|, 0, ...), basis[0] = z / |z|, cycle
// counters reset; |z|^2 given on the device
__global__ void k_cycle_start(GmresCycle* cyc, double* __restrict__ givens, int m, const double* __restrict__ zsq,
                              int restart, double ptol, double* __restrict__ inv_out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const double z = sqrt(zsq[0]);
  double* S = givens + 2 * m;
  for (int k = 0; k <= m; ++k) S[k] = 0.0;
  S[0] = z;
  inv_out[0] = 1.0 / z;
  cyc->col = 0;
  cyc->last = -1;
  cyc->restart = restart;
  cyc->inner = 0;
  cyc->breakdown = 0;
  cyc->done = 0;
  cyc->ptol = ptol;
  cyc->presid = 0.0;
  cyc->inv_h1 = 1.0;
}

// x = x * alpha[0]
__global__ void k_scale_dev(long long n, const double* __restrict__ alpha, double* __restrict__ x) {
  long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i < n) x[i] = x[i] * alpha[0];
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

// Launches of one sweep: runs of consecutive levels at most `wide` rows wide
// in one wavefront launch, each wider level alone in a grid launch.
static void sweep_schedule(SweepPlan& pl, int wide) {
  const std::vector<int>& lp = pl.host_level_ptr;
  const int nlev = (int)lp.size() - 1;
  pl.schedule.clear();
  int l = 0;
  while (l < nlev) {
    if (lp[l + 1] - lp[l] > wide) {
      pl.schedule.push_back({0, l, l + 1});
      ++l;
      continue;
    }
    int l1 = l;
    while (l1 < nlev && lp[l1 + 1] - lp[l1] <= wide) ++l1;
    pl.schedule.push_back({1, l, l1});
    l = l1;
  }
}

static void free_windows(SweepWindows& W);
static cudaError_t plan_windows(SweepPlan& pl, int C, int nc);

cudaError_t implicit_set_wide_level(ImplicitState& st, int wide, int engine) {
  st.wide_level = wide > 0 ? wide : kWideLevel;
  st.engine = engine > 0 ? engine : st.default_engine;
  // the per-component sweep takes chunks of at most 8 rows
  cudaError_t e = cudaSuccess;
  if (st.engine == kSweepDataflowComponents && st.chunk_rows > 8) e = implicit_set_chunk(st, 8);
  sweep_schedule(st.fwd, st.wide_level);
  sweep_schedule(st.bwd, st.wide_level);
  free_windows(st.fwd.win);
  free_windows(st.bwd.win);
  if (st.engine == kSweepWindow8 || st.engine == kSweepWindow16) {
    const int nc = st.engine == kSweepWindow16 ? 16 : 8;
    if (e == cudaSuccess) e = plan_windows(st.fwd, st.n_cells, nc);
    if (e == cudaSuccess) e = plan_windows(st.bwd, st.n_cells, nc);
  }
  st.inner_key = -1;  // the captured loop holds the old launches
  return e;
}

// The dataflow sweep's chunks: runs of at most `rows` consecutive positions
// inside one level (rows <= 32, one warp).
static cudaError_t sweep_chunks(SweepPlan& pl, int rows) {
  const std::vector<int>& lp = pl.host_level_ptr;
  std::vector<int2> ch;
  pl.host_chunk_ptr.assign(lp.size(), 0);
  for (size_t l = 0; l + 1 < lp.size(); ++l) {
    pl.host_chunk_ptr[l] = (int)ch.size();
    for (int p = lp[l]; p < lp[l + 1]; p += rows) ch.push_back(make_int2(p, std::min(rows, lp[l + 1] - p)));
  }
  pl.host_chunk_ptr.back() = (int)ch.size();
  return ch.empty() ? cudaSuccess : cudaMemcpy(pl.chunks, ch.data(), ch.size() * sizeof(int2), cudaMemcpyHostToDevice);
}

cudaError_t implicit_set_chunk(ImplicitState& st, int rows) {
  int r = rows > 0 ? rows : kFlowChunk;
  if (st.engine == kSweepDataflowComponents && r > 8) r = 8;  // a warp holds 8 rows of 4 components
  st.chunk_rows = r;
  cudaError_t e = sweep_chunks(st.fwd, r);
  if (e == cudaSuccess) e = sweep_chunks(st.bwd, r);
  st.inner_key = -1;  // the captured loop holds the old chunk ranges
  return e;
}

// Plans the windowed band sweep of pl's current schedule for a cluster of nc
// blocks (SweepWindows).  Each single-block run of the schedule is cut into
// windows of at most kWinMaxLevels levels, fewer where a block's rows, the
// rows they depend on inside the window and the rows read from before it
// would not fit the shared-memory slots or staging buffers; ok stays false
// when one level alone does not fit (the sweep then takes the per-row-wait
// engine).
static void free_windows(SweepWindows& W) {
  for (void* q : W.owned) cudaFree(q);
  W = SweepWindows{};
}

static cudaError_t plan_windows(SweepPlan& pl, int C, int nc) {
  free_windows(pl.win);
  SweepWindows& W = pl.win;
  std::vector<int> runs;
  for (const SweepPlan::Launch& l : pl.schedule) runs.insert(runs.end(), {l.wavefront, l.l0, l.l1});
  WindowPlanHost H;
  const WindowLimits lim{kWinMaxLevels, kWinMaxSlots, kWinMaxRows, kWinMaxExt};
  if (!plan_windows_host(pl.host_level_ptr, pl.host_pos_cell, pl.host_ent_ptr, pl.host_ent_pos, runs, C, nc, lim, H))
    return cudaSuccess;  // no plan: the sweep takes the per-row-wait engine
  W.nc = H.nc;
  W.band_rows = H.band_rows;
  W.n_records = H.n_records;
  W.run_w0 = H.run_w0;
  cudaError_t e = cudaSuccess;
  auto put = [&](const std::vector<int>& v, int** dst) {
    if (e != cudaSuccess) return;
    e = cudaMalloc((void**)dst, std::max<size_t>(v.size(), 4) * sizeof(int));
    if (e != cudaSuccess) return;
    W.owned.push_back(*dst);
    if (!v.empty()) e = cudaMemcpy(*dst, v.data(), v.size() * sizeof(int), cudaMemcpyHostToDevice);
  };
  put(H.l0, &W.l0);
  put(H.l1, &W.l1);
  put(H.gbase, &W.gbase);
  put(H.grp, &W.grp);
  put(H.stage, &W.stage);
  put(H.rec, &W.rec);
  put(H.eslot, &W.eslot);
  put(H.ext, &W.ext);
  for (double** dst : {&W.row, &W.rhs}) {
    if (e != cudaSuccess) break;
    const size_t per = dst == &W.row ? 8 : 4;  // doubles per record
    e = cudaMalloc((void**)dst, std::max<size_t>((size_t)W.n_records * per, 4) * sizeof(double));
    if (e == cudaSuccess) W.owned.push_back(*dst);
  }
  W.ok = e == cudaSuccess;
  return e;
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
  // level sets of the natural-order dependency graph: forward over the
  // lower entries (col < i), backward over the upper ones (col > i)
  auto levels = [&](bool fwd, std::vector<int>& lev) {
    lev.assign(C, 0);
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
    return nlev;
  };
  // sweep order: cells by level (stable in cell id); entries of each row in
  // ascending column order with the column's own sweep position
  struct HostPlan {
    std::vector<int> level_ptr, pos_cell, ent_ptr, ent_cell, ent_pos, ent_val;
  };
  auto plan = [&](bool fwd, HostPlan& hp) {
    std::vector<int> lev;
    const int nlev = levels(fwd, lev);
    hp.level_ptr.assign(nlev + 1, 0);
    for (int i = 0; i < C; ++i) hp.level_ptr[lev[i] + 1]++;
    for (int l = 0; l < nlev; ++l) hp.level_ptr[l + 1] += hp.level_ptr[l];
    hp.pos_cell.resize(C);
    std::vector<int> fill(hp.level_ptr.begin(), hp.level_ptr.end() - 1), pos_of(C);
    for (int i = 0; i < C; ++i) {
      pos_of[i] = fill[lev[i]]++;
      hp.pos_cell[pos_of[i]] = i;
    }
    hp.ent_ptr.assign(C + 1, 0);
    for (int p = 0; p < C; ++p) {
      const int i = hp.pos_cell[p];
      for (auto& e : (fwd ? lower : upper)[i]) {
        if (e.first == i) continue;  // a self-coupled periodic pair: on the diagonal
        hp.ent_cell.push_back(e.first);
        hp.ent_pos.push_back(pos_of[e.first]);
        hp.ent_val.push_back(e.second);
      }
      hp.ent_ptr[p + 1] = (int)hp.ent_cell.size();
    }
    return nlev;
  };
  HostPlan hf, hb;
  st.n_levels_fwd = plan(true, hf);
  st.n_levels_bwd = plan(false, hb);
  // packed topology: the first kSweepPack entries of every row
  struct Packed {
    std::vector<int> cnt, pos, cell;
  };
  auto pack = [&](const HostPlan& hp, Packed& pk) {
    pk.cnt.resize(C);
    pk.pos.assign((size_t)C * kSweepPack, 0);
    pk.cell.assign((size_t)C * kSweepPack, 0);
    for (int p = 0; p < C; ++p) {
      const int j0 = hp.ent_ptr[p], n = hp.ent_ptr[p + 1] - j0;
      pk.cnt[p] = n;
      for (int k = 0; k < kSweepPack && k < n; ++k) {
        pk.pos[(size_t)p * kSweepPack + k] = hp.ent_pos[j0 + k];
        pk.cell[(size_t)p * kSweepPack + k] = hp.ent_cell[j0 + k];
      }
    }
  };
  Packed pf, pb;
  pack(hf, pf);
  pack(hb, pb);

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
  UP(hf.level_ptr, fwd.level_ptr);
  UP(hf.pos_cell, fwd.pos_cell);
  UP(hf.ent_ptr, fwd.ent_ptr);
  UP(hf.ent_cell, fwd.ent_cell);
  UP(hf.ent_pos, fwd.ent_pos);
  UP(hf.ent_val, fwd.ent_val);
  UP(hb.level_ptr, bwd.level_ptr);
  UP(hb.pos_cell, bwd.pos_cell);
  UP(hb.ent_ptr, bwd.ent_ptr);
  UP(hb.ent_cell, bwd.ent_cell);
  UP(hb.ent_pos, bwd.ent_pos);
  UP(hb.ent_val, bwd.ent_val);
  UP(pf.cnt, fwd.pk_cnt);
  UP(pf.pos, fwd.pk_pos);
  UP(pf.cell, fwd.pk_cell);
  UP(pb.cnt, bwd.pk_cnt);
  UP(pb.pos, bwd.pk_pos);
  UP(pb.cell, bwd.pk_cell);
#undef UP
  for (int f = 0; f < 2; ++f) {
    SweepPlan& pl = f == 0 ? st.fwd : st.bwd;
    const HostPlan& hp = f == 0 ? hf : hb;
    pl.host_pos_cell = hp.pos_cell;
    pl.host_ent_ptr = hp.ent_ptr;
    pl.host_ent_pos = hp.ent_pos;
  }
  st.fwd.n_levels = st.n_levels_fwd;
  st.bwd.n_levels = st.n_levels_bwd;
  st.fwd.host_level_ptr = hf.level_ptr;
  st.bwd.host_level_ptr = hb.level_ptr;
  for (SweepPlan* pl : {&st.fwd, &st.bwd}) {  // room for chunks of one row
    if (e == cudaSuccess) e = cudaMalloc((void**)&pl->chunks, (size_t)std::max(C, 1) * sizeof(int2));
    if (e == cudaSuccess) st.owned.push_back(pl->chunks);
    if (e == cudaSuccess) e = sweep_chunks(*pl, kDefaultEngine == kSweepDataflowComponents ? 8 : kFlowChunk);
  }
  st.wide_level = kWideLevel;
  sweep_schedule(st.fwd, st.wide_level);
  sweep_schedule(st.bwd, st.wide_level);
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
  zeros(N4, &st.vcur);
  for (SweepPlan* pl : {&st.fwd, &st.bwd}) {
    zeros((size_t)C * kSweepPack, &pl->pk_val);
    zeros(C, &pl->pk_diag);
    zeros(C, &pl->pk_dc);
    zeros(8 * (size_t)C, (double**)&pl->pk_row);
  }
  zeros(kRedBlocks, &st.partials);
  zeros(64, &st.scalars);
  zeros(4, &st.scale_dev);
  zeros(C, &st.dt_buf);
  if (e == cudaSuccess) e = cudaMalloc((void**)&st.cycle, sizeof(GmresCycle));
  if (e == cudaSuccess) st.owned.push_back(st.cycle);
  if (e == cudaSuccess) e = cudaMallocHost((void**)&st.cycle_host, sizeof(GmresCycle));
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_lusgs_wavefront, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                 (int)kRingBytes);
  // Measured on the 512 x 256 bump (767 levels of at most 256 rows), one
  // LU-SGS application takes 3.20 ms in one block with per-row waits, 4.46 /
  // 4.82 ms in a cluster of 8 / 16 sharing every solution, and 1.82 / 1.25 ms
  // in the windowed band sweep on a cluster of 8 / 16, the default where the
  // device runs it (set after the cluster checks below).
  st.engine = kDefaultEngine;
  st.chunk_rows = kDefaultEngine == kSweepDataflowComponents ? 8 : kFlowChunk;
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_lusgs_dataflow<512, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                 (int)kFlowSmemBytes);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_lusgs_dataflow<1024, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                 (int)kFlowSmemBytes);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_lusgs_dataflow<256, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                 (int)kFlowSmemBytes);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_lusgs_dataflow<512, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                 (int)kFlowSmemBytes);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_lusgs_dataflow_comp<512>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                 (int)kFlowSmemBytes);
  st.cluster8_ok = false;
  if (e == cudaSuccess &&
      cudaFuncSetAttribute(k_lusgs_cluster<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kRingBytes) ==
          cudaSuccess) {
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(kPortableCluster);
    cfg.blockDim = dim3(kClusterThreads);
    cfg.dynamicSmemBytes = kRingBytes;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = kPortableCluster;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int clusters = 0;
    st.cluster8_ok = cudaOccupancyMaxActiveClusters(&clusters, k_lusgs_cluster<8>, &cfg) == cudaSuccess && clusters > 0;
  }
  st.cluster16_ok =
      cudaFuncSetAttribute(k_lusgs_cluster<16>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kRingBytes) ==
          cudaSuccess &&
      cudaFuncSetAttribute(k_lusgs_cluster<16>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess;
  // the windowed band sweeps: whether a cluster of 8 / 16 such blocks fits the device
  auto window_fits = [](auto kernel, int nc) {
    const int smem = kWinSmemBytes;
    if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess)
      return false;
    if (nc > kPortableCluster &&
        cudaFuncSetAttribute(kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess)
      return false;
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(nc);
    cfg.blockDim = dim3(kWinThreads);
    cfg.dynamicSmemBytes = smem;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = nc;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int clusters = 0;
    return cudaOccupancyMaxActiveClusters(&clusters, kernel, &cfg) == cudaSuccess && clusters > 0;
  };
  st.window8_ok = e == cudaSuccess && window_fits(k_lusgs_window<8>, 8);
  st.window16_ok = e == cudaSuccess && window_fits(k_lusgs_window<16>, 16);
  cudaGetLastError();
  st.default_engine = st.window16_ok ? kSweepWindow16 : (st.window8_ok ? kSweepWindow8 : kDefaultEngine);
  if (e == cudaSuccess) e = implicit_set_wide_level(st, 0, 0);
  if (e == cudaSuccess) {
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_mgs, kBlock, 0);
    st.mgs_blocks = std::max(1, sms * std::min(per_sm, 2));
    zeros(2 * (size_t)st.mgs_blocks, &st.mgs_partials);
  }
  st.dt = st.dt_buf;
  return e;
}

static void free_gmres_basis(ImplicitState& st) {
  if (st.inner_exec) cudaGraphExecDestroy(st.inner_exec);
  if (st.inner_graph) cudaGraphDestroy(st.inner_graph);
  st.inner_exec = nullptr;
  st.inner_graph = nullptr;
  st.inner_key = -1;
  for (double** p : {&st.basis, &st.hess, &st.givens, &st.hcol}) {
    if (*p) cudaFree(*p);
    *p = nullptr;
  }
  st.basis_m = 0;
}

void implicit_free(ImplicitState& st) {
  free_gmres_basis(st);
  if (st.cap_stream) cudaStreamDestroy(st.cap_stream);
  st.cap_stream = nullptr;
  for (void* p : st.owned) cudaFree(p);
  st.owned.clear();
  free_windows(st.fwd.win);
  free_windows(st.bwd.win);
  if (st.cycle_host) cudaFreeHost(st.cycle_host);
  st.cycle_host = nullptr;
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
  for (SweepPlan* pl : {&st.fwd, &st.bwd}) {
    count_launch();
    k_pack_rows<<<blocks_for(st.n_cells), kBlock, 0, s>>>(st.n_cells, pl->pos_cell, pl->ent_ptr, pl->ent_val,
                                                          st.rval, st.diag, st.dclamp, pl->pk_val, pl->pk_diag,
                                                          pl->pk_dc, pl->pk_row);
  }
  return cudaGetLastError();
}

static cudaError_t sweep(const SweepPlan& pl, const ImplicitState& st, const double* in, double* out, int backward,
                         cudaStream_t s) {
  SweepDev a{pl.level_ptr, pl.pos_cell, pl.ent_ptr, pl.ent_cell, pl.ent_pos, pl.ent_val, st.rval,
             pl.pk_cnt, pl.pk_pos, pl.pk_cell, pl.pk_val, pl.pk_diag, pl.pk_dc, pl.pk_row,
             in, out, backward};
  const bool window = st.engine == kSweepWindow8 || st.engine == kSweepWindow16;
  if (window && pl.win.ok && pl.win.n_records > 0) {
    count_launch();
    k_pack_window<<<blocks_for(pl.win.n_records), kBlock, 0, s>>>(
        pl.win.n_records, reinterpret_cast<const int4*>(pl.win.rec), pl.pk_row, in, backward,
        reinterpret_cast<double2*>(pl.win.row), pl.win.rhs);
  }
  for (size_t si = 0; si < pl.schedule.size(); ++si) {
    const SweepPlan::Launch& l = pl.schedule[si];
    count_launch();
    // the windowed sweep falls back to the default where it has no plan
    if (l.wavefront && (st.engine == kSweepDataflow || (window && !pl.win.ok))) {
      const int k0 = pl.host_chunk_ptr[l.l0], k1 = pl.host_chunk_ptr[l.l1];
      k_lusgs_dataflow<512, false><<<1, 512, kFlowSmemBytes, s>>>(a, pl.chunks, k0, k1, st.status);
    } else if (l.wavefront && st.engine == kSweepDataflowWide) {
      const int k0 = pl.host_chunk_ptr[l.l0], k1 = pl.host_chunk_ptr[l.l1];
      k_lusgs_dataflow<1024, false><<<1, 1024, kFlowSmemBytes, s>>>(a, pl.chunks, k0, k1, st.status);
    } else if (l.wavefront && st.engine == kSweepDataflowIntMul) {
      const int k0 = pl.host_chunk_ptr[l.l0], k1 = pl.host_chunk_ptr[l.l1];
      k_lusgs_dataflow<512, true><<<1, 512, kFlowSmemBytes, s>>>(a, pl.chunks, k0, k1, st.status);
    } else if (l.wavefront && st.engine == kSweepDataflowComponents) {
      const int k0 = pl.host_chunk_ptr[l.l0], k1 = pl.host_chunk_ptr[l.l1];
      k_lusgs_dataflow_comp<512><<<1, 512, kFlowSmemBytes, s>>>(a, pl.chunks, k0, k1, st.status);
    } else if (l.wavefront && st.engine == kSweepDataflowNarrow) {
      const int k0 = pl.host_chunk_ptr[l.l0], k1 = pl.host_chunk_ptr[l.l1];
      k_lusgs_dataflow<256, false><<<1, 256, kFlowSmemBytes, s>>>(a, pl.chunks, k0, k1, st.status);
    } else if (l.wavefront && (st.engine == kSweepCluster8 || st.engine == kSweepCluster16)) {
      cudaLaunchConfig_t cfg{};
      cfg.gridDim = dim3(st.engine);
      cfg.blockDim = dim3(kClusterThreads);
      cfg.dynamicSmemBytes = kRingBytes;
      cfg.stream = s;
      cudaLaunchAttribute attr[1];
      attr[0].id = cudaLaunchAttributeClusterDimension;
      attr[0].val.clusterDim.x = st.engine;
      attr[0].val.clusterDim.y = 1;
      attr[0].val.clusterDim.z = 1;
      cfg.attrs = attr;
      cfg.numAttrs = 1;
      const cudaError_t e = st.engine == 16 ? cudaLaunchKernelEx(&cfg, k_lusgs_cluster<16>, a, l.l0, l.l1)
                                             : cudaLaunchKernelEx(&cfg, k_lusgs_cluster<8>, a, l.l0, l.l1);
      if (e != cudaSuccess) return e;
    } else if (l.wavefront && window) {
      const SweepWindows& W = pl.win;
      const WinDev wd{W.l0,
                      W.l1,
                      W.gbase,
                      W.grp,
                      W.eslot,
                      reinterpret_cast<const int4*>(W.stage),
                      reinterpret_cast<const int4*>(W.rec),
                      reinterpret_cast<const double2*>(W.row),
                      W.rhs,
                      reinterpret_cast<const int2*>(W.ext)};
      const int w0 = W.run_w0[si], w1 = W.run_w0[si + 1];
      cudaLaunchConfig_t cfg{};
      cfg.gridDim = dim3(W.nc);
      cfg.blockDim = dim3(kWinThreads);
      cfg.dynamicSmemBytes = kWinSmemBytes;
      cfg.stream = s;
      cudaLaunchAttribute attr[1];
      attr[0].id = cudaLaunchAttributeClusterDimension;
      attr[0].val.clusterDim.x = W.nc;
      attr[0].val.clusterDim.y = 1;
      attr[0].val.clusterDim.z = 1;
      cfg.attrs = attr;
      cfg.numAttrs = 1;
      const cudaError_t e = W.nc == 16 ? cudaLaunchKernelEx(&cfg, k_lusgs_window<16>, a, wd, w0, w1)
                                       : cudaLaunchKernelEx(&cfg, k_lusgs_window<8>, a, wd, w0, w1);
      if (e != cudaSuccess) return e;
    } else if (l.wavefront) {
      k_lusgs_wavefront<<<1, kWaveThreads, kRingBytes, s>>>(a, l.l0, l.l1);
    } else {
      const int b = pl.host_level_ptr[l.l0], e = pl.host_level_ptr[l.l0 + 1];
      k_lusgs_level<<<blocks_for(e - b), kBlock, 0, s>>>(a, b, e);
    }
  }
  return cudaGetLastError();
}

cudaError_t lusgs_apply(ImplicitState& st, const double* v, double* x, cudaStream_t s) {
  cudaError_t e = sweep(st.fwd, st, v, st.tmp, 0, s);  // (D + L) y = v
  if (e == cudaSuccess) e = sweep(st.bwd, st, st.tmp, x, 1, s);  // (D + U) x = D y
  return e;
}

cudaError_t implicit_set_operator(ImplicitState& st, ScaleVec scale, const double* dt, int dt_per_cell,
                                  cudaStream_t s) {
  st.scale = scale;
  st.dt_per_cell = dt_per_cell;
  count_launch();
  k_set_scale<<<1, 32, 0, s>>>(scale, st.scale_dev);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(st.dt_buf, dt, (dt_per_cell ? (size_t)st.n_cells : 1) * sizeof(double),
                        cudaMemcpyDeviceToDevice, s);
  st.dt = st.dt_buf;
  return e;
}

cudaError_t fd_operator(ImplicitState& st, const ResidualFn& residual1, const double* v, double* out,
                        cudaStream_t s) {
  const int C = st.n_cells;
  const long long N = 4LL * C;
  cudaError_t e = implicit_dot(st, N, v, v, st.scalars + 0, s);
  count_launch(3);
  k_fd_eps<<<1, 32, 0, s>>>(st.scalars + 0, st.scalars + 8, st.scalars + 1);
  k_fd_perturb<<<blocks_for(N), kBlock, 0, s>>>(C, st.state, v, st.scalars + 1, st.scale_dev, st.up);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e == cudaSuccess) e = residual1(st.up, st.rp, s);
  k_fd_combine<<<blocks_for(N), kBlock, 0, s>>>(C, v, st.rp, st.rate, st.scalars + 1, st.scale_dev, st.dt,
                                                st.dt_per_cell, out);
  if (e == cudaSuccess) e = cudaGetLastError();
  return e;
}

static double host_scalar(const double* d, cudaStream_t s, cudaError_t* e) {
  double h = 0.0;
  if (*e == cudaSuccess) *e = cudaMemcpyAsync(&h, d, sizeof(double), cudaMemcpyDeviceToHost, s);
  if (*e == cudaSuccess) *e = cudaStreamSynchronize(s);
  return h;
}

// Krylov basis, Hessenberg columns and rotations for restart length m.
static cudaError_t ensure_gmres_basis(ImplicitState& st, int m) {
  if (st.basis_m >= m) return cudaSuccess;
  free_gmres_basis(st);
  const size_t N = 4 * (size_t)st.n_cells;
  cudaError_t e = cudaMalloc((void**)&st.basis, (size_t)(m + 1) * N * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc((void**)&st.hess, (size_t)m * (m + 1) * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc((void**)&st.givens, (size_t)(3 * m + 2) * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc((void**)&st.hcol, (size_t)(m + 3) * sizeof(double));
  if (e == cudaSuccess) st.basis_m = m;
  return e;
}

// One Arnoldi step of SciPy's inner loop, all on the device: basis[col] ->
// matvec -> preconditioner -> Gram-Schmidt -> Givens -> basis[col + 1].
static cudaError_t arnoldi_step(ImplicitState& st, const MatvecFn& matvec, int m, cudaGraphConditionalHandle handle,
                                int use_handle, cudaStream_t s) {
  const long long N = 4LL * st.n_cells;
  const int grid = (int)std::min<long long>(blocks_for(N), 152LL * 8);
  count_launch();
  k_take_column<<<grid, kBlock, 0, s>>>(st.basis, N, st.cycle, st.vcur);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = matvec(st.vcur, st.av, s);
  if (e == cudaSuccess) e = lusgs_apply(st, st.av, st.w, s);
  if (e == cudaSuccess) {
    MgsArgs a{st.basis, N, st.w, st.cycle, st.hcol, m, st.mgs_partials};
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(st.mgs_blocks);
    cfg.blockDim = dim3(kBlock);
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    count_launch();
    e = cudaLaunchKernelEx(&cfg, k_mgs, a);
  }
  if (e == cudaSuccess) {
    count_launch(2);
    k_givens<<<1, 32, 0, s>>>(st.cycle, st.hcol, st.hess, st.givens, m, handle, use_handle);
    k_next_basis<<<grid, kBlock, 0, s>>>(st.basis, N, st.cycle, st.w);
    e = cudaGetLastError();
  }
  return e;
}

// The inner loop as a graph: a while node whose body is one Arnoldi step;
// the Givens kernel clears the condition when the cycle is done.  Built once
// per (restart length, operator) and replayed for every cycle.  Returns false
// (and the caller steps from the host) when the runtime refuses any part.
static bool ensure_inner_graph(ImplicitState& st, const MatvecFn& matvec, int key, int m) {
  if (st.graph_failed) return false;
  if (st.inner_exec && st.inner_key == key) return true;
  if (st.inner_exec) cudaGraphExecDestroy(st.inner_exec);
  if (st.inner_graph) cudaGraphDestroy(st.inner_graph);
  st.inner_exec = nullptr;
  st.inner_graph = nullptr;
  if (!st.cap_stream && cudaStreamCreateWithFlags(&st.cap_stream, cudaStreamNonBlocking) != cudaSuccess) {
    st.graph_failed = true;
    return false;
  }
  cudaGraph_t graph = nullptr;
  cudaGraphConditionalHandle handle{};
  bool ok = cudaGraphCreate(&graph, 0) == cudaSuccess &&
            cudaGraphConditionalHandleCreate(&handle, graph, 1, cudaGraphCondAssignDefault) == cudaSuccess;
  cudaGraphNodeParams params{};
  cudaGraphNode_t node;
  if (ok) {
    params.type = cudaGraphNodeTypeConditional;
    params.conditional.handle = handle;
    params.conditional.type = cudaGraphCondTypeWhile;
    params.conditional.size = 1;
    ok = cudaGraphAddNode(&node, graph, nullptr, nullptr, 0, &params) == cudaSuccess;
  }
  if (ok) {
    cudaGraph_t body = params.conditional.phGraph_out[0];
    ok = cudaStreamBeginCaptureToGraph(st.cap_stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal) ==
         cudaSuccess;
    if (ok) {
      const long long before = launch_count();
      const bool step_ok = arnoldi_step(st, matvec, m, handle, 1, st.cap_stream) == cudaSuccess;
      count_launch(-(int)(launch_count() - before));  // captured, not launched
      cudaGraph_t captured = nullptr;
      ok = cudaStreamEndCapture(st.cap_stream, &captured) == cudaSuccess && step_ok;
      size_t nodes = 0;
      if (ok) ok = cudaGraphGetNodes(body, nullptr, &nodes) == cudaSuccess;
      st.inner_nodes = (int)nodes;
    }
  }
  if (ok) ok = cudaGraphInstantiate(&st.inner_exec, graph, 0) == cudaSuccess;
  if (!ok) {
    cudaGetLastError();  // clear a refused call's error
    if (st.inner_exec) cudaGraphExecDestroy(st.inner_exec);
    st.inner_exec = nullptr;
    if (graph) cudaGraphDestroy(graph);
    st.graph_failed = true;
    return false;
  }
  st.inner_graph = graph;
  st.inner_key = key;
  return true;
}

int gmres_solve(ImplicitState& st, const MatvecFn& matvec, int matvec_key, const double* b, double* x, double tol,
                int max_iter, int m, int* iterations, cudaStream_t s) {
  const long long N = 4LL * st.n_cells;
  cudaError_t e = cudaSuccess;
  auto grid = [&](long long n) { return blocks_for(n); };
  if (ensure_gmres_basis(st, m) != cudaSuccess) return GMRES_CUDA;
  const bool graph = matvec_key >= 0 && ensure_inner_graph(st, matvec, matvec_key * 4096 + m, m);
  double* w = st.w;
  double* av = st.av;
  cudaMemsetAsync(x, 0, N * sizeof(double), s);
  int used = 0;
  *iterations = 0;
  bool x_nonzero = false;
  std::vector<double> H, S;
  GmresCycle& cyc = *st.cycle_host;
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
    double* r = st.basis;
    if (x_nonzero) {
      if (matvec(x, av, s) != cudaSuccess) return GMRES_CUDA;
      count_launch();
      k_sub<<<grid(N), kBlock, 0, s>>>(N, b, av, r);
    } else {
      cudaMemcpyAsync(r, b, N * sizeof(double), cudaMemcpyDeviceToDevice, s);
    }
    e = implicit_dot(st, N, r, r, st.scalars + 4, s);
    if (std::sqrt(host_scalar(st.scalars + 4, s, &e)) < atol) return GMRES_OK;
    // v0 = psolve(r) / |psolve(r)|, S = (|psolve(r)|, 0, ...)
    if (lusgs_apply(st, r, w, s) != cudaSuccess) return GMRES_CUDA;
    cudaMemcpyAsync(st.basis, w, N * sizeof(double), cudaMemcpyDeviceToDevice, s);
    e = implicit_dot(st, N, st.basis, st.basis, st.scalars + 5, s);
    count_launch(2);
    k_cycle_start<<<1, 32, 0, s>>>(st.cycle, st.givens, m, st.scalars + 5, restart, ptol, st.scalars + 6);
    k_scale_dev<<<grid(N), kBlock, 0, s>>>(N, st.scalars + 6, st.basis);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) return GMRES_CUDA;
    // ---- the inner loop: graph replay, or one step at a time from the host
    if (graph) {
      e = cudaGraphLaunch(st.inner_exec, s);
      if (e == cudaSuccess) e = cudaMemcpyAsync(st.cycle_host, st.cycle, sizeof(GmresCycle), cudaMemcpyDeviceToHost, s);
      if (e == cudaSuccess) e = cudaStreamSynchronize(s);
      if (e != cudaSuccess) return GMRES_CUDA;
      count_launch(cyc.inner * st.inner_nodes);
    } else {
      do {
        if (arnoldi_step(st, matvec, m, cudaGraphConditionalHandle{}, 0, s) != cudaSuccess) return GMRES_CUDA;
        e = cudaMemcpyAsync(st.cycle_host, st.cycle, sizeof(GmresCycle), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return GMRES_CUDA;
      } while (!cyc.done);
    }
    const int col = cyc.last;
    const int inner = cyc.inner;
    // back substitution (upper triangular in h[k][k]) on the host
    H.resize((size_t)(col + 1) * (m + 1));
    S.resize(3 * (size_t)m + 2);
    e = cudaMemcpy(H.data(), st.hess, H.size() * sizeof(double), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(S.data(), st.givens, S.size() * sizeof(double), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return GMRES_CUDA;
    auto h = [&](int c, int k) { return H[(size_t)c * (m + 1) + k]; };
    std::vector<double> y(S.begin() + 2 * m, S.begin() + 2 * m + col + 1);
    if (h(col, col) == 0.0) y[col] = 0.0;
    for (int k = col; k > 0; --k) {
      if (y[k] != 0.0) {
        y[k] /= h(k, k);
        const double tk = y[k];
        for (int j = 0; j < k; ++j) y[j] -= tk * h(k, j);
      }
    }
    if (y[0] != 0.0) y[0] /= h(0, 0);
    for (int k = 0; k <= col; ++k) {
      count_launch();
      k_axpy<<<grid(N), kBlock, 0, s>>>(N, y[k], st.basis + (size_t)k * N, x);
    }
    x_nonzero = true;
    if (matvec(x, av, s) != cudaSuccess) return GMRES_CUDA;
    count_launch();
    k_sub<<<grid(N), kBlock, 0, s>>>(N, b, av, st.tmp);
    e = implicit_dot(st, N, st.tmp, st.tmp, st.scalars + 7, s);
    const double rnorm = std::sqrt(host_scalar(st.scalars + 7, s, &e));
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
