// Internal types of the implicit-Euler building blocks (mcfd_implicit.cu).
#pragma once

#include <cuda_runtime.h>

#include <functional>
#include <vector>

#include "mcfd_internal.h"

namespace mcfd {

struct ScaleVec {
  double v[4];
};

// Mesh topology of the scalar preconditioner matrix, gathered on the host at
// geometry creation.  Couplings: interior faces (owner a, neighbour b; both
// normals the face normal), then periodic pairs (owner of face a, owner of
// face b; each side with its own face's normal, length of face a).  Boundary
// faces: every face without a neighbour, in face order (periodic faces
// included, as the reference does, solver.py:1287-1300).
struct ImplicitTopology {
  int n_cells = 0;
  int n_interior = 0;
  std::vector<int> coupling_a, coupling_b;
  std::vector<double2> coupling_na, coupling_nb;
  std::vector<double> coupling_len;
  std::vector<int> boundary_owner;
  std::vector<double2> boundary_normal;
  std::vector<double> boundary_len;
};

// One triangular sweep of LU-SGS, laid out in sweep order: rows sorted by
// their level in the dependency graph of the reference's natural cell order
// (positions), each row's off-diagonal entries in ascending column order.
// The schedule is a list of launches over consecutive levels: runs of narrow
// levels in one single-block wavefront launch, each wide level in a grid
// launch of its own.
constexpr int kSweepPack = 4;

// How a run of narrow levels is swept: one block with a barrier per level,
// one block of 256, 512 or 1024 threads with per-row waits (no barrier per
// level),
// or a thread-block cluster of 8 / 16 blocks with a cluster barrier per
// level.
enum SweepEngine {
  kSweepBlock = 1,
  kSweepDataflow = 2,      // 512 threads
  kSweepDataflowWide = 3,  // 1024 threads
  kSweepDataflowNarrow = 4,  // 256 threads
  kSweepDataflowIntMul = 5,  // 512 threads, the row's products on the integer pipe
  kSweepDataflowComponents = 6,  // 512 threads, one lane per (row, component), chunks of 8 rows
  kSweepWindow8 = 7,   // cluster of 8 blocks owning bands of cells, windows of levels (SweepWindows)
  kSweepCluster8 = 8,
  kSweepWindow16 = 9,  // the same with 16 blocks
  kSweepCluster16 = 16
};

// The windowed band sweep of one plan for a cluster of nc blocks.  Block k
// owns the cells [k * band_rows, (k + 1) * band_rows).  The levels of each
// single-block run are cut into windows of consecutive levels; in a window,
// block k solves its own rows and every row of another band they depend on
// inside the window (recomputed, the same bits), reading the rows solved
// before the window ("externals") from global memory once, at the window's
// start, into shared-memory slots.  All of a (window, block)'s data is
// contiguous, so that it can be staged into shared memory in a few copies:
//   windows w: levels [l0[w], l1[w]); stage[w * nc + k] = (first record,
//     records, first external, externals) of block k;
//   level ranges: grp[gbase[w] + k * (nl + 1) + m], m = 0..nl, record
//     indices, nl = l1 - l0;
//   row record r: rec[8 r ..] = position (~position for a row of another
//     band, which is not stored to global memory), cell, slot | entries << 16,
//     the start of its entries' slots in eslot (entry order of the row), and
//     its first kSweepPack entry slots;
//   row[r] (64 bytes, refreshed after each assembly) and rhs[r] (32 bytes,
//     refreshed before each sweep): the record's position's values and its
//     right-hand side;
//   ext[e] = (slot, cell) of an external.
struct SweepWindows {
  int nc = 0, band_rows = 0, n_records = 0;
  bool ok = false;  // planned for the current schedule
  int *l0 = nullptr, *l1 = nullptr, *gbase = nullptr, *grp = nullptr, *stage = nullptr, *rec = nullptr,
      *eslot = nullptr, *ext = nullptr;
  double *row = nullptr, *rhs = nullptr;
  std::vector<int> run_w0;  // first window of each schedule entry (one more entry: the end)
  std::vector<void*> owned;
};

struct SweepPlan {
  int n_levels = 0;
  int* level_ptr = nullptr;  // [n_levels + 1] positions
  int* pos_cell = nullptr;   // [C] cell at each position
  int* ent_ptr = nullptr;    // [C + 1] entries per position
  int* ent_cell = nullptr;   // column cell of the entry
  int* ent_pos = nullptr;    // column position of the entry (sweep order)
  int* ent_val = nullptr;    // index into the row values
  // rows packed in sweep order with a fixed stride of kSweepPack entries
  // (longer rows continue in the CSR above): column position and cell
  // (topology, built once) and the matrix values, diagonal and clamped
  // diagonal (refreshed by every assembly)
  int* pk_cnt = nullptr;     // [C] entries of the row
  int* pk_pos = nullptr;     // [C][kSweepPack]
  int* pk_cell = nullptr;    // [C][kSweepPack]
  double* pk_val = nullptr;  // [C][kSweepPack]
  double* pk_diag = nullptr; // [C]
  double* pk_dc = nullptr;   // [C]
  double2* pk_row = nullptr; // [C][4] the windowed sweep's row: diagonal, RN(1 / diagonal), recip_fixed(diagonal), clamped diagonal, values
  std::vector<int> host_level_ptr;
  // host copies of the topology for planning the windowed sweep
  std::vector<int> host_pos_cell, host_ent_ptr, host_ent_pos;
  SweepWindows win;
  // chunks of at most 32 consecutive positions inside one level (start,
  // rows), for the dataflow sweep; chunk_ptr[l] = first chunk of level l
  int2* chunks = nullptr;
  std::vector<int> host_chunk_ptr;
  struct Launch {
    int wavefront;  // 1: single-block run of levels [l0, l1); 0: grid launch of level l0
    int l0, l1;
  };
  std::vector<Launch> schedule;
};

// Device-resident state of one GMRES restart cycle (SciPy's inner loop):
// the Hessenberg columns, Givens rotations and the residual estimate, so
// that an Arnoldi step needs no host round trip.
struct GmresCycle {
  int col;        // column of the next Arnoldi step
  int last;       // last column processed
  int restart;    // inner iterations allowed in this cycle
  int inner;      // inner iterations done
  int breakdown;
  int done;       // presid <= ptol, breakdown, or restart reached
  double ptol;
  double presid;
  double inv_h1;  // scale of the next basis vector (1 / h1, or 1 at breakdown)
};

struct ImplicitState {
  int n_cells = 0, n_coupling = 0, n_boundary = 0;
  int n_levels_fwd = 0, n_levels_bwd = 0;
  // topology (device)
  int *ca = nullptr, *cb = nullptr, *bowner = nullptr;
  double2 *na = nullptr, *nb = nullptr, *bnormal = nullptr;
  double *clen = nullptr, *blen = nullptr;
  int *dptr = nullptr, *dref = nullptr, *rptr = nullptr, *rref = nullptr, *rcol = nullptr;
  SweepPlan fwd, bwd;
  int wide_level = 0;  // levels wider than this get a grid launch each
  int engine = 0;      // how a run of narrow levels is swept (SweepEngine)
  int default_engine = kSweepDataflow;  // the fastest engine the device runs
  int chunk_rows = 32;  // rows per chunk of the per-row-wait sweeps
  bool cluster8_ok = false, cluster16_ok = false, window8_ok = false, window16_ok = false;
  DevStatus* status = nullptr;  // the geometry's status word (sweep time-outs)
  // values and vectors (device)
  double *coef = nullptr, *bterm = nullptr, *diag = nullptr, *dclamp = nullptr, *rval = nullptr;
  double *tmp = nullptr, *state = nullptr, *rate = nullptr, *up = nullptr, *rp = nullptr;
  double *w = nullptr, *av = nullptr, *vcur = nullptr, *partials = nullptr, *scalars = nullptr;
  // prepared operator: scales, |state / scale|^2 and the time steps live on
  // the device, so a captured GMRES step reads the current values
  ScaleVec scale{{1.0, 1.0, 1.0, 1.0}};
  double* scale_dev = nullptr;  // [4]
  double* dt_buf = nullptr;     // [C] copy of the prepared time steps
  const double* dt = nullptr;   // = dt_buf
  int dt_per_cell = 0;
  bool prepared = false;
  // Krylov basis ((m + 1) x 4C, one allocation) and the cycle state
  double* basis = nullptr;
  int basis_m = 0;
  GmresCycle* cycle = nullptr;      // device
  GmresCycle* cycle_host = nullptr;  // pinned mirror
  double* hess = nullptr;            // device [m][m + 1] Hessenberg columns
  double* givens = nullptr;          // device [3 m + 2]: c, s, S
  double* hcol = nullptr;            // device [m + 3]: dots, |w|^2 before / after
  double* mgs_partials = nullptr;    // device [2][mgs_blocks]
  int mgs_blocks = 0;
  cudaStream_t cap_stream = nullptr;  // stream the inner loop is captured on
  int inner_nodes = 0;                // nodes of one captured Arnoldi step
  // the inner loop as a graph with a device-evaluated while condition
  cudaGraphExec_t inner_exec = nullptr;
  cudaGraph_t inner_graph = nullptr;
  int inner_key = -1;  // (m, operator) the graph was built for
  bool graph_failed = false;
  std::vector<void*> owned;
};

enum GmresResult { GMRES_OK = 0, GMRES_NOT_CONVERGED = 1, GMRES_BREAKDOWN = 2, GMRES_CUDA = 3 };

using ResidualFn = std::function<cudaError_t(const double* U, double* R, cudaStream_t s)>;
using MatvecFn = std::function<cudaError_t(const double* v, double* out, cudaStream_t s)>;

cudaError_t implicit_build(ImplicitState& st, const ImplicitTopology& t);
void implicit_free(ImplicitState& st);
cudaError_t implicit_assemble(ImplicitState& st, const double* P, const double* area, const double* dt,
                              int dt_per_cell, double gamma, cudaStream_t s);
// operator set-up of mcfd_implicit_prepare: scales, |state / scale|^2 and a
// copy of the time steps into the state's device buffers
cudaError_t implicit_set_operator(ImplicitState& st, ScaleVec scale, const double* dt, int dt_per_cell,
                                  cudaStream_t s);
cudaError_t lusgs_apply(ImplicitState& st, const double* v, double* x, cudaStream_t s);
cudaError_t implicit_set_wide_level(ImplicitState& st, int wide, int engine);
cudaError_t implicit_set_chunk(ImplicitState& st, int rows);
cudaError_t fd_operator(ImplicitState& st, const ResidualFn& residual1, const double* v, double* out,
                        cudaStream_t s);
// matvec_key: distinguishes operators for the captured inner loop (a graph is
// rebuilt when it changes); count: kernels launched per captured step
int gmres_solve(ImplicitState& st, const MatvecFn& matvec, int matvec_key, const double* b, double* x, double tol,
                int max_iter, int m, int* iterations, cudaStream_t s);
// scaled norms and reductions of the Newton iteration
cudaError_t implicit_dot(ImplicitState& st, long long n, const double* x, const double* y, double* out,
                         cudaStream_t s);
cudaError_t implicit_equation(ImplicitState& st, const double* U, const double* U0, const double* R,
                              const double* dt, int dt_per_cell, ScaleVec scale, double* b_out,
                              double* norms_dev, cudaStream_t s);
cudaError_t implicit_maxima(ImplicitState& st, const double* U, const double* P, double gamma,
                            double* maxima_dev, cudaStream_t s);
cudaError_t implicit_scaled_sumsq(ImplicitState& st, const double* U, ScaleVec scale, double* out,
                                  cudaStream_t s);
cudaError_t implicit_candidate(int C, const double* U, const double* dx, double damping, ScaleVec scale,
                               double* out, cudaStream_t s);

}  // namespace mcfd
