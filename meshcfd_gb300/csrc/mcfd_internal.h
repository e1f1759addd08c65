// Internal structures shared by the API (host packing) and kernel translation
// units.  Not part of the public ABI.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/meshcfd_gb300.h"

namespace mcfd {

// Flux-face segments, in the order the reference accumulates boundary groups
// in _residual (solver.py:2502-2704): interior faces first (their sum is the
// CSR divergence product, solver.py:2501), then periodic pairs, walls and
// symmetry planes, velocity inlets, pressure outlets, far field.
// SEG_BCX: pressure-inlet and mass-flow faces, whose exterior states come from
// the per-patch boundary kernel (mcfd_boundary.cu) before the flux launch.
enum Segment { SEG_INTERIOR = 0, SEG_PERIODIC, SEG_WALL, SEG_VIN, SEG_POUT, SEG_FAR, SEG_BCX, SEG_COUNT };

// Kinds of dt entries (exterior state used for the boundary spectral radius,
// solver.py:4190-4220).
enum DtKind { DT_PLAIN = 0, DT_VIN = 1, DT_POUT = 2, DT_FAR = 3, DT_BCX = 4 };

struct DevStatus {
  int code;
  int first_cell;
  int first_face;
  int first_patch;
  unsigned long long dt_min_bits;  // atomicMin target for the global time step
};

// Everything a kernel needs, by value.  Index arrays are int32 (sizes are
// checked against 2^31 at creation).
struct DevGeom {
  int n_cells, n_faces, n_flux, n_slots, n_gradient;
  int seg_begin[SEG_COUNT + 1];
  const double* area;  // [C]
  // cells grouped by (gradient, limiter, gather, time-step) entry counts,
  // stable in cell id: the visiting order of the per-cell stage kernels
  const int* cell_order;  // [C]
  int n_lim34;            // cells cell_order[0 .. n_lim34) have 3 or 4 limiter entries
  // least-squares gradient entries grouped by source cell, reference order
  const int* grad_ptr;
  const int* grad_nb;
  const double* grad_cx;
  const double* grad_cy;
  const int* grad_twin;  // CSR position of the paired entry (b -> a for a -> b), or -1
  int has_twins;
  // limiter entries grouped by cell: slot id (reference entry index) + offset
  const int* lim_ptr;
  const int* lim_slot;
  const double2* lim_d;
  // MUSCL-parabolic two-ring stencil grouped by source, reference order
  int n_parabolic;
  const int* par_ptr;
  const int* par_nb;
  const double2* par_d;
  // flux faces
  const int* ff_lslot;  // recon slot of the interior-side state
  const int* ff_rslot;  // recon slot of the other side (interior/periodic), else -1
  const int* ff_lcell;  // cell of the left state
  const int* ff_rcell;  // cell of the right state (interior/periodic), else -1
  const double2* ff_normal;
  const double* ff_len;             // face length (periodic pairs: face a's)
  const double2* ff_wall_velocity;  // indexed by flux face - seg_begin[SEG_WALL]
  const double* ff_vin_state;       // [n_vin][4]
  const double* ff_pout_pressure;   // [n_pout]
  const double* ff_far_state;       // [n_far][4]
  // pressure-inlet / mass-flow patches over the SEG_BCX faces
  int n_bc_patches;
  const int* bc_ptr;       // [patches + 1], positions within SEG_BCX
  const int* bc_kind;      // [patches]
  const double* bc_values; // [patches][4]
  const double* bc_dn;     // [n_bcx] direction . normal
  double* bc_ext;          // [n_bcx][4] exterior states of the residual (written per evaluation)
  double* bc_ext_dt;       // [n_bcx][4] exterior states of the time step (from cell values)
  double* bc_terms;        // [n_bcx] mass-flow inlet scratch
  // cell gather: interior faces in ascending face order with the reference's
  // CSR divergence coefficient, then boundary contributions in BC order with a
  // signed face length.
  const int* gi_ptr;
  const int* gi_flux;
  const double* gi_coef;
  const int* gb_ptr;
  const int* gb_flux;
  const double* gb_len;
  // time-step entries: owner side of every face in face order, then the
  // neighbour side of interior faces.
  const int* dt_ptr;
  const double2* dt_normal;
  const double* dt_len;
  const int* dt_info;  // kind << 28 | index into the BC arrays
  DevStatus* status;
  // laminar viscous terms (n_diffusive = 0 when the geometry carries none)
  int has_viscous;            // the descriptor gave the viscous tables
  int n_diffusive;
  const double2* grad_d;      // [n_gradient] raw offsets, grouped like grad_nb
  const int* vb_ptr;          // [C + 1] diffusive faces per owner cell (positions j), diffusive order
  const int* vb_j;
  int viscous_ok;             // every diffusive wall face has thermal data
  const int* diff_owner;      // [n_diffusive] owner cell
  const double2* diff_normal;
  const double* diff_len;
  const int* diff_kind;       // MCFD_DIFF_*
  const int* diff_thermal;
  const double* diff_value;
  const int* diff_inlet;      // source << 28 | index
  const double* diff_nd;
  const double2* diff_ghost;
  const double2* diff_offset;
  const double2* diff_wallv;
  // viscous gather: periodic a (+), periodic b (-), diffusive faces, per cell in reference order
  const int* vg_ptr;
  const int* vg_code;         // kind << 28 | index: 0 periodic a (index k), 1 periodic b, 2 diffusive face j
  // time-step diffusion entries per cell: owner / neighbour side of interior faces, periodic, diffusive
  const int* vd_ptr;
  const int* vd_other;        // other cell, or -1 on diffusive boundary faces
  const double* vd_len;
  const double* vd_dist;      // raw distance (the kernel takes max(d, 1e-14))
  const double* visc_diff;    // [C] diffusion sum of the last viscous time step (workspace)
  // launch shapes chosen by mcfd_autotune (0: the defaults)
  int tune_recon_threads, tune_flux_threads, tune_flux_faces, tune_gather_threads;
  int tune_recon_split;  // fast variant: one thread per (cell, variable) for cells with 3 / 4 entries
};

// One term of an explicit stage combination, evaluated left to right.
enum TermKind { TERM_X = 0, TERM_X_PLUS_DTR = 1, TERM_DTR = 2, TERM_DTR_SAVED = 3 };
struct StageTerm {
  int kind;
  double coef;
  const double* x;  // state (TERM_X, TERM_X_PLUS_DTR) or saved residual
};
struct StageProgram {
  int n_terms;
  StageTerm t[5];
  const double* dt;  // device scalar or [C]
  int dt_per_cell;
  double* out_u;     // may be null (residual only)
  double* out_p;     // primitive of out_u, may be null
  double* out_r;     // residual store, may be null
  const double* visc_r;  // laminar viscous residual added before the body force, may be null
  // the stable time steps of the new state (out_u), computed by the gather
  // from its primitive: per cell into next_dt_cells (may be null) and, when
  // next_dt_min, their minimum into next_dt_status (as k_time_steps).  The
  // time-step bits go to next_dt_status as well: they belong to the step
  // that uses these time steps, not to the one that computed them.
  double* next_dt_cells;
  int next_dt_min;
  double cfl;
  DevStatus* next_dt_status;
};

struct Workspace {
  double* P;      // [C][4]
  double* recon;  // [slots][4]
  double* flux;   // [n_flux][4]
  double* stage[4];
  double* saved_r;
  double* partials;  // [blocks][4]
  int partial_blocks;
};

// A second stream with fork / join events: the boundary face segments run on
// it concurrently with the interior faces (disjoint outputs).
struct SideStream {
  cudaStream_t stream = nullptr;
  cudaEvent_t fork = nullptr, join = nullptr;
};

// kernels (mcfd_kernels_impl.cuh), one set per variant: mcfd::exact (reference
// operation order), mcfd::fast (smallest-ratio limiter), mcfd::fma (fewer
// divisions everywhere, FMA).
#define MCFD_DECLARE_LAUNCHERS(NS)                                                              \
  namespace NS {                                                                               \
  cudaError_t launch_primitive(const DevGeom& g, const mcfd_config& cfg, const double* U,      \
                               double* P, cudaStream_t s);                                     \
  cudaError_t launch_reconstruct(const DevGeom& g, const mcfd_config& cfg, const double* P,    \
                                 double* recon, cudaStream_t s);                               \
  cudaError_t launch_flux(const DevGeom& g, const mcfd_config& cfg, const double* P,           \
                          const double* recon, double* flux, cudaStream_t s,                   \
                          const SideStream* side);                                             \
  cudaError_t launch_gather(const DevGeom& g, const mcfd_config& cfg, const double* P,         \
                            const double* flux, const StageProgram& prog, cudaStream_t s);     \
  cudaError_t launch_time_steps(const DevGeom& g, const mcfd_config& cfg, const double* P,     \
                                double* dt_cells, double* dt_min, double time_limit,           \
                                cudaStream_t s);                                               \
  bool stage_fused_supported(const DevGeom& g, const mcfd_config& cfg, const StageProgram& prog); \
  cudaError_t launch_stage_fused(const DevGeom& g, const mcfd_config& cfg, const double* P,    \
                                 double* recon, double* flux, const StageProgram& prog,        \
                                 cudaStream_t s, int* blocks_per_sm);                          \
  }
MCFD_DECLARE_LAUNCHERS(exact)
MCFD_DECLARE_LAUNCHERS(fast)
MCFD_DECLARE_LAUNCHERS(fma)
#undef MCFD_DECLARE_LAUNCHERS

// Launch shape of a face segment: 256-thread blocks when the segment fills
// the 152 SMs, otherwise warp-multiple blocks spread over all SMs (a boundary
// segment of a few thousand faces would sit on a handful of SMs).
inline int seg_threads(int n) {
  if (n >= 152 * 256) return 256;
  int t = (n + 151) / 152;
  t = ((t + 31) / 32) * 32;
  return t < 32 ? 32 : (t > 256 ? 256 : t);
}
inline int seg_blocks(int n) { return (n + seg_threads(n) - 1) / seg_threads(n); }
// flux launch shape with the autotuned threads / faces per thread, if any
inline int flux_threads(const DevGeom& g, int n) {
  return g.tune_flux_threads && n >= 152 * g.tune_flux_threads ? g.tune_flux_threads : seg_threads(n);
}
inline int flux_blocks(const DevGeom& g, int n) {
  const int t = flux_threads(g, n);
  const int per_block = t * (g.tune_flux_threads && n >= 152 * g.tune_flux_threads && g.tune_flux_faces > 1
                                 ? g.tune_flux_faces : 1);
  return (n + per_block - 1) / per_block;
}

// variant-independent (mcfd_kernels_common.cu)
long long launch_count();
void count_launch(int n = 1);
cudaError_t launch_case_time_steps(int n_cells, int n_cases, const int* offsets, double* dt_case,
                                   double* dt_cells, cudaStream_t s);
// MUSCL parabolic and the reference's reconstruction fields (mcfd_parabolic.cu;
// exact arithmetic in every mode)
cudaError_t launch_reconstruct_parabolic(const DevGeom& g, const mcfd_config& cfg, const double* P, double* recon,
                                         cudaStream_t s);
cudaError_t launch_reconstruction_fields(const DevGeom& g, const mcfd_config& cfg, const double* P, double* grad,
                                         double* curv, double* fac, cudaStream_t s);
// laminar viscous terms (mcfd_viscous.cu): residual of the primitive state P
// into work.r (needs the cell-value boundary states in g.bc_ext_dt), and the
// time step's diffusion sum into diff
struct ViscousWork {
  double* cell = nullptr;   // [C][4] T, mu, conductivity, effective diffusivity
  double* grad = nullptr;   // [C][6] (du, dv, dT) x (x, y)
  double* flux = nullptr;   // [n_interior + n_periodic][4]
  double* bflux = nullptr;  // [n_diffusive][4]
  double* r = nullptr;      // [C][4]
  double* diff = nullptr;   // [C]
};
cudaError_t launch_viscous_residual(const DevGeom& g, const mcfd_config& cfg, const double* P, const ViscousWork& w,
                                    cudaStream_t s);
cudaError_t launch_viscous_diffusion(const DevGeom& g, const mcfd_config& cfg, const double* P,
                                     const ViscousWork& w, cudaStream_t s);
// pressure-inlet and mass-flow exterior states (mcfd_boundary.cu; exact
// arithmetic): from the face states of the residual (recon per slot, or P for
// first order when recon is null) into ext
cudaError_t launch_bc_states(const DevGeom& g, const mcfd_config& cfg, const double* P, const double* recon,
                             double* ext, cudaStream_t s);
// reduction kernels of the sum of squares.  kSumsqBlocks is the grid of the
// partial kernel for every entry point that reduces a residual (the handle's
// mcfd_residual_sumsq and the allocation-free variant): the grid fixes the
// summation order, so both give the same bits only while they share it.
constexpr int kSumsqBlocks = 152 * 4;
constexpr int kSumsqThreads = 256;
__global__ void k_sumsq_partial(int n, const double* __restrict__ R, double* __restrict__ partials);
__global__ void k_sumsq_final(int blocks, const double* __restrict__ partials, double* sums);
cudaError_t finalize_time_step(DevStatus* st, double* dt_min, double time_limit, cudaStream_t s);
cudaError_t launch_sumsq(const DevGeom& g, const double* R, double* partials, int blocks,
                         double* sums, cudaStream_t s);

}  // namespace mcfd
