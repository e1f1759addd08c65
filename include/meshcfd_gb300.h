/*
 * meshcfd_gb300 — C ABI of the GB300 (sm_103a) residual / time-step path.
 *
 * Every entry point takes plain pointers and sizes.  Device arrays are
 * caller-owned CUDA device pointers; host arrays are ordinary host memory.
 * Streams are passed as `void*` holding a `cudaStream_t` (NULL = legacy
 * default stream).  Functions return 0 on success or an MCFD_E_* code; none of
 * them traps or aborts.  Errors the numerics detect on the device (the
 * reference's ValueError/SolverError cases) are accumulated in a per-geometry
 * status word and returned by mcfd_status_fetch().
 *
 * State layout: conservative U and primitive P are (n_cells, 4) row-major
 * float64 arrays — (rho, rho*u, rho*v, E) and (rho, u, v, p) — in the
 * reference cell order (src/meshcfd/core/solver.py:2437-2442 takes and
 * returns exactly this shape).  Cell, face and entry ids are never renumbered
 * on output.
 *
 * The reference is a Python package whose hot path is the set of module
 * functions cited below; a Python caller binds these entry points with
 * ctypes (meshcfd_gb300/_lib.py holds one binding per entry point).
 */
#ifndef MESHCFD_GB300_H
#define MESHCFD_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MCFD_ABI_VERSION 6

/* ---- return codes (host-side failures) ---- */
#define MCFD_OK 0
#define MCFD_E_ARG 1         /* invalid argument (null pointer, bad size or code) */
#define MCFD_E_CUDA 2        /* a CUDA runtime call failed */
#define MCFD_E_UNSUPPORTED 3 /* option outside what the GPU path implements */
#define MCFD_E_GEOMETRY 4    /* geometry description inconsistent */
#define MCFD_E_TOO_LARGE 5   /* size beyond the fixed scratch of the allocation-free entry point */
#define MCFD_E_NOT_CONVERGED 6 /* GMRES reached its iteration limit (solver.py:1526-1529) */
#define MCFD_E_BREAKDOWN 7     /* GMRES broke down (solver.py:1522-1523) */

/* ---- device status bits (numerical failures; reference messages) ---- */
#define MCFD_S_NONPHYSICAL_STATE 0x01  /* euler.py:34-39 non-finite or non-positive rho/p */
#define MCFD_S_NONFINITE_RESIDUAL 0x02 /* solver.py:2716-2717 */
#define MCFD_S_HLLC_NONFINITE 0x04     /* euler.py:164-165 */
#define MCFD_S_ROE_SOUND 0x08          /* euler.py:191-192 */
#define MCFD_S_ROE_NONFINITE 0x10      /* euler.py:260-261 */
#define MCFD_S_FARFIELD_SOUND 0x20     /* solver.py:4382-4383 */
#define MCFD_S_FARFIELD_STATE 0x40     /* solver.py:4402-4407 */
#define MCFD_S_TIME_STEP 0x80          /* solver.py:4341-4342 */
/* pressure-inlet and mass-flow boundaries (messages name the patch given
 * by mcfd_status.first_patch) */
#define MCFD_S_PIN_DIRECTION 0x100        /* solver.py:4424-4428 */
#define MCFD_S_PIN_SUPERSONIC_OUT 0x200   /* solver.py:4433-4437 */
#define MCFD_S_PIN_SUPERSONIC_IN 0x400    /* solver.py:4445-4449 */
#define MCFD_S_PIN_INCOMPATIBLE 0x800     /* solver.py:4465-4469 */
#define MCFD_S_PIN_STATE 0x1000           /* solver.py:4491-4494 */
#define MCFD_S_MFI_DIRECTION 0x2000       /* solver.py:4508-4512 */
#define MCFD_S_MFI_PRESSURE 0x4000        /* solver.py:4513-4516 */
#define MCFD_S_MFI_FLOW_RATE 0x8000       /* solver.py:4536-4540 */
#define MCFD_S_MFO_DENSITY 0x10000        /* solver.py:4563-4566 */
/* laminar viscous terms */
#define MCFD_S_VISC_TEMPERATURE 0x20000   /* solver.py:3620-3621 */
#define MCFD_S_VISC_SUTHERLAND 0x40000    /* solver.py:2734-2735 */
#define MCFD_S_VISC_DISTANCE 0x80000      /* solver.py:3944-3945 */
/* No counterpart in the reference: an LU-SGS sweep of the implicit path waited
 * past its bound for a row it depends on and stopped (its output is invalid). */
#define MCFD_S_SWEEP_TIMEOUT 0x100000

typedef struct mcfd_status {
  int32_t code;       /* OR of MCFD_S_* bits since the last fetch */
  int32_t first_cell; /* lowest cell id that set a state/residual/time-step bit, or -1 */
  int32_t first_face; /* lowest flux-face index that set a flux bit, or -1 */
  int32_t first_patch; /* lowest boundary-patch index (mcfd_geom_desc.bc_*) that set a boundary bit, or -1 */
} mcfd_status;

/* ---- scheme codes ---- */
#define MCFD_FLUX_RUSANOV 0 /* euler.py:80-93 */
#define MCFD_FLUX_HLLC 1    /* euler.py:96-166, _kernels.py:71-160 */
#define MCFD_FLUX_ROE 2     /* euler.py:169-262 */
#define MCFD_RECON_FIRST_ORDER 0
#define MCFD_RECON_MUSCL_LINEAR 1
#define MCFD_RECON_MUSCL_PARABOLIC 2
/* limiter codes are the reference's own (solver.py:2303-2308) */
#define MCFD_LIMITER_BARTH_JESPERSEN 0
#define MCFD_LIMITER_MINMOD 1
#define MCFD_LIMITER_VAN_LEER 2
#define MCFD_LIMITER_VENKATAKRISHNAN 3
/* Venkatakrishnan's limiter in its published form with the smoothing constant
 * K (mcfd_config.venkat_k): per face (d1^2 + e2 + 2 d1 d2) / (d1^2 + 2 d2^2 +
 * d1 d2 + e2), e2 = (K sqrt(A))^3, minimum over faces, no cap.  No
 * counterpart in the reference (its Venkatakrishnan form has no K); MUSCL
 * linear only. */
#define MCFD_LIMITER_VENKATAKRISHNAN_K 4
/* kernel variants */
#define MCFD_MODE_EXACT 0 /* reference operation order, no FMA: bit-exact */
#define MCFD_MODE_FAST 1  /* exact arithmetic, limiter minimum via the smallest ratio */
#define MCFD_MODE_FMA 2   /* + shared reciprocals and FMA: ~1e-11 on fine meshes */
/* time integration (model.py:28-34) */
#define MCFD_TIME_EULER 0
#define MCFD_TIME_RK2 1
#define MCFD_TIME_RK3 2
#define MCFD_TIME_RK4 3 /* SSPRK(5,4), solver.py:1128-1182 */

typedef struct mcfd_config {
  int32_t flux;           /* MCFD_FLUX_* */
  int32_t reconstruction; /* MCFD_RECON_* */
  int32_t limiter;        /* MCFD_LIMITER_* */
  int32_t mode;           /* MCFD_MODE_*: kernel variant */
  double gamma;           /* ratio of specific heats (NumericalSettings.gamma) */
  double acceleration_x;  /* body force (solver.py:2709-2715) */
  double acceleration_y;
  double cfl;             /* used by mcfd_time_steps */
  double gas_constant;    /* NumericalSettings.gas_constant: pressure-inlet / mass-flow / viscous terms */
  int32_t viscosity_model; /* MCFD_VISC_* */
  int32_t reserved_i;
  double dynamic_viscosity;                /* Constant model */
  double sutherland_reference_viscosity;   /* Sutherland model (solver.py:2721-2737) */
  double sutherland_reference_temperature;
  double sutherland_temperature;
  double prandtl_number;
  double venkat_k;        /* K of MCFD_LIMITER_VENKATAKRISHNAN_K (> 0) */
  double reserved;
} mcfd_config;

/* viscosity models (model.py:24) */
#define MCFD_VISC_INVISCID 0
#define MCFD_VISC_CONSTANT 1
#define MCFD_VISC_SUTHERLAND 2
/* kinds of diffusive boundary faces (viscous terms, solver.py:3650-3690, 3947-4030) */
#define MCFD_DIFF_WALL_NO_SLIP 0
#define MCFD_DIFF_WALL_SLIP 1
#define MCFD_DIFF_SYMMETRY 2
#define MCFD_DIFF_INLET 3      /* exterior state given: velocity / pressure / mass-flow inlet, far field */
#define MCFD_DIFF_OTHER 4      /* zero normal gradient (outlets) */
#define MCFD_DIFF_WALL_UNKNOWN 5 /* wall without thermal data: the viscous path refuses it */

/* boundary patch kinds (solver.py:81-103) */
#define MCFD_BC_PRESSURE_INLET 0
#define MCFD_BC_MASS_FLOW_INLET 1
#define MCFD_BC_MASS_FLOW_OUTLET 2

/*
 * Geometry description: the arrays of the reference `_Geometry`
 * (solver.py:123-177) that the inviscid residual and the time step read.
 * Index arrays are int64 as NumPy produces them; all arrays are host memory
 * and are copied by mcfd_geom_create (the caller may free them afterwards).
 * Counts of zero allow NULL pointers.
 */
typedef struct mcfd_geom_desc {
  int64_t n_cells;
  int64_t n_faces;
  const double* areas;           /* [n_cells] */
  const double* face_normals;    /* [n_faces][2] */
  const double* face_lengths;    /* [n_faces] */
  const int64_t* owners;         /* [n_faces] */
  const int64_t* neighbours;     /* [n_faces], -1 on boundary faces */
  int64_t n_interior;
  const int64_t* interior_faces; /* [n_interior] ascending face ids */
  int64_t n_periodic;
  const int64_t* periodic_faces_a; /* [n_periodic] */
  const int64_t* periodic_faces_b; /* [n_periodic] */
  int64_t n_wall;                  /* wall + symmetry faces, reference order */
  const int64_t* wall_faces;
  const double* wall_velocities;   /* [n_faces][2] (may be NULL: zero) */
  int64_t n_velocity_inlet;
  const int64_t* velocity_inlet_faces;
  const double* velocity_inlet_states; /* [n][4] primitive */
  int64_t n_pressure_outlet;
  const int64_t* pressure_outlet_faces;
  const double* pressure_outlet_pressures; /* [n] */
  int64_t n_far_field;
  const int64_t* far_field_faces;
  const double* far_field_states; /* [n][4] primitive */
  int64_t n_gradient;             /* least-squares entries, reference order */
  const int64_t* gradient_sources;
  const int64_t* gradient_neighbours;
  const double* gradient_coefficients_x;
  const double* gradient_coefficients_y;
  int64_t n_limiter;              /* must equal n_faces + n_interior */
  const int64_t* limiter_cells;
  const double* limiter_dx;
  const double* limiter_dy;
  /* two-ring stencil of MUSCL parabolic (_parabolic_stencil,
   * solver.py:2241-2291), entries grouped by source in the reference's
   * order; n_parabolic = 0 when the geometry was built without it (the
   * reference then reconstructs linearly, solver.py:2327-2329). */
  int64_t n_parabolic;
  const int64_t* parabolic_sources;
  const int64_t* parabolic_neighbours;
  const double* parabolic_dx;
  const double* parabolic_dy;
  /* pressure-inlet, mass-flow-inlet and mass-flow-outlet patches
   * (_Geometry.pressure_inlets / mass_flow_inlets / mass_flow_outlets), in
   * the reference's order: all pressure inlets, then the mass-flow inlets,
   * then the mass-flow outlets. */
  int64_t n_bc_patches;
  const int32_t* bc_kind;      /* [n] MCFD_BC_* */
  const double* bc_values;     /* [n][4]: pressure inlet: total pressure, total temperature, direction x, y;
                                  mass-flow inlet: mass flow, total temperature, direction x, y;
                                  mass-flow outlet: mass flow, float(np.sum(face lengths)), 0, 0 */
  const int64_t* bc_offsets;   /* [n + 1] into bc_faces */
  const int64_t* bc_faces;     /* boundary face ids, patch by patch */
  const double* bc_direction_normal; /* [len(bc_faces)] normals @ direction as the reference computes it
                                        (inlets; 0 for outlets) */
  /* laminar viscous terms (needed only with a viscosity model) */
  const double* gradient_dx;        /* [n_gradient] raw offsets of the gradient entries */
  const double* gradient_dy;
  int64_t n_diffusive;              /* non-periodic boundary faces, ascending (diffusive_boundary_faces) */
  const int64_t* diffusive_faces;
  const int32_t* diffusive_kind;    /* MCFD_DIFF_* */
  const int32_t* diffusive_thermal; /* walls: 0 fixed temperature, 1 heat flux */
  const double* diffusive_value;    /* walls: temperature or heat flux */
  const int32_t* diffusive_inlet;   /* inlets: source << 28 | index: 1 velocity inlet, 2 pressure-inlet /
                                       mass-flow patch face (bc_faces position), 3 far field */
  const double* diffusive_normal_distance; /* float(np.dot(face_center - cell_center, normal)) */
  const double* diffusive_ghost_offset;    /* [n][2] 2 d n (walls, symmetry) or 2 (face_center - center) */
  const double* diffusive_offset;          /* [n][2] face_center - cell_center */
  const double* interior_distance; /* [n_interior] |(c_neighbour - c_owner) . n| (time-step diffusion) */
  const double* periodic_distance; /* [n_periodic] |(f_a - c_a) . n_a| + |(f_b - c_b) . n_b| */
} mcfd_geom_desc;

typedef struct mcfd_geom mcfd_geom; /* opaque device geometry + workspace */

typedef struct mcfd_geom_info {
  int64_t n_cells, n_faces, n_interior, n_periodic, n_boundary_flux;
  int64_t n_flux_faces;     /* interior + periodic + wall + inlet/outlet/far faces */
  int64_t n_gradient, n_limiter;
  int64_t device_bytes;     /* device memory held by the handle */
} mcfd_geom_info;

/* Library version (MCFD_ABI_VERSION). */
int mcfd_abi_version(void);
/* Short description of a return code. */
const char* mcfd_error_string(int code);

/*
 * Build the device geometry (CSR gathers in reference accumulation order,
 * face segments, workspace) on the current CUDA device.  Replaces the
 * reference's per-call use of `_Geometry` arrays inside `_residual`
 * (solver.py:2437-2718) and `_stable_time_steps` (solver.py:4132-4343).
 */
int mcfd_geom_create(const mcfd_geom_desc* desc, mcfd_geom** out);
int mcfd_geom_destroy(mcfd_geom* geom);
int mcfd_geom_get_info(const mcfd_geom* geom, mcfd_geom_info* info);

/*
 * P = conservative_to_primitive(U) with the positivity check
 * (euler.py:20-40; solver.py:1620-1629).  U, P: device [n_cells][4].
 */
int mcfd_primitive(mcfd_geom* geom, const mcfd_config* cfg, const double* U, double* P,
                   void* stream);

/*
 * R = _residual(U, geometry, settings) (solver.py:2437-2718) for inviscid
 * flow: reconstruction (first order / MUSCL linear with the four limiters),
 * Rusanov/HLLC/Roe fluxes on interior, periodic, wall/symmetry,
 * velocity-inlet, pressure-outlet and far-field faces, body force and the
 * finiteness check.  U, R: device [n_cells][4].  R may be NULL (the status
 * word is still updated).
 */
int mcfd_residual(mcfd_geom* geom, const mcfd_config* cfg, const double* U, double* R,
                  void* stream);

/*
 * Local stable time steps (solver.py:4132-4343, inviscid part) from the
 * primitive state P.  dt_cells (device [n_cells], may be NULL) receives
 * CFL*A_i/Sigma_i; dt_min (device scalar, may be NULL) receives
 * min(min_i dt_i, time_limit) — pass time_limit = end_time - time for the
 * reference's global adaptive step (solver.py:455-461), or +inf.
 */
int mcfd_time_steps(mcfd_geom* geom, const mcfd_config* cfg, const double* P,
                    double* dt_cells, double* dt_min, double time_limit, void* stream);

/*
 * One explicit step in place: U <- step(U).  `scheme` is MCFD_TIME_*
 * (explicit Euler solver.py:532-565, SSP-RK2 566-674, SSP-RK3 675-806,
 * SSPRK(5,4) 1128-1182).  dt: device pointer to one float64 (global step)
 * or to [n_cells] (dt_per_cell = 1, local steady mode, _scale_cell_rate
 * solver.py:1119-1125).  Every stage is fused: reconstruction, face flux,
 * cell gather + stage combination + primitive recovery of the new stage.
 * After the call the handle's primitive buffer holds P(U_new).
 */
int mcfd_explicit_step(mcfd_geom* geom, const mcfd_config* cfg, int32_t scheme, double* U,
                       const double* dt, int32_t dt_per_cell, void* stream);
/* mcfd_explicit_step followed by mcfd_time_steps on the new state: the time
 * steps of the next step (per cell into next_dt_cells and / or their minimum
 * with time_limit into next_dt_min; either or both may be NULL, neither may
 * alias dt or U)
 * — computed by the last stage from the primitive it recovers, where they
 * depend on the cell state alone (inviscid, no pressure-inlet or mass-flow
 * patches), else by the time-step pass; the same values either way.
 * primitive_current = 1 skips the primitive recovery at the start of the
 * step: the caller asserts that the handle's primitive buffer holds the
 * primitive of U, as the previous explicit step on this handle left it.
 * The reference computes the stable step at the top of each loop iteration
 * (solver.py:437-461); this is the same sequence with the step boundary
 * moved.  The status bits of these time steps (MCFD_S_TIME_STEP and the
 * boundary-state bits of the time-step pass) go to a second status word,
 * read by mcfd_status_fetch_next, so that a caller raises them with the step
 * that uses the time steps, as the reference does; the bits of the stages,
 * the new state's primitive recovery included (solver.py:808-810), stay in
 * the word mcfd_status_fetch reads.  start_residual (NULL or [n_cells][4]):
 * the first stage also stores the residual of U that it computes, the
 * reference's `derivative` (solver.py:466-468) on which its progress report
 * takes the per-component RMS (solver.py:943-950).  No counterpart in the
 * reference. */
int mcfd_explicit_step_next(mcfd_geom* geom, const mcfd_config* cfg, int32_t scheme, double* U,
                            const double* dt, int32_t dt_per_cell, int32_t primitive_current,
                            double* next_dt_cells, double* next_dt_min, double time_limit,
                            double* start_residual, void* stream);

/* The reconstruction fields of the reference for primitive P [n_cells][4]:
 * MUSCL linear -> _limited_gradients (solver.py:2294-2319): gradients
 * [n_cells][4][2] and factors [n_cells][4]; MUSCL parabolic ->
 * _parabolic_reconstruction (solver.py:2322-2415): also curvature
 * [n_cells][4][3] (xx, xy, yy; may be NULL).  Device arrays; exact
 * arithmetic whatever cfg->mode. */
int mcfd_reconstruction(mcfd_geom* geom, const mcfd_config* cfg, const double* P, double* gradients,
                        double* curvature, double* factors, void* stream);

/* Device pointer to the handle's primitive buffer [n_cells][4] (valid after
 * mcfd_primitive / mcfd_residual / mcfd_explicit_step on the same handle). */
const double* mcfd_geom_primitive(const mcfd_geom* geom);
/* Device pointer to intermediate stage state k (0..3) [n_cells][4] of the
 * last mcfd_explicit_step on the handle: for RK2 k = 0 is U1; for RK3 k = 0, 1
 * are U1, U2; for SSPRK(5,4) k = 0..3 are U1..U4.  Valid until the next call
 * on the handle; NULL for k out of range.  Used to replay a step's stages in
 * reverse (no counterpart in the reference). */
const double* mcfd_geom_stage_state(const mcfd_geom* geom, int32_t k);
/* Choose the launch shapes of the stage kernels for this geometry and
 * settings by timing candidates on the state U (device [n_cells][4]):
 * reconstruction and gather threads per block in {64, 128, 256}, flux
 * threads in {64, 128, 256} x faces per thread in {1, 2, 4}.  The choice
 * stays with the handle; chosen (host [5]) receives reconstruction threads,
 * flux threads, flux faces per thread, gather threads (0: default) and
 * whether the fast variant's reconstruction runs one thread per (cell,
 * variable) (1) or per cell (0).
 * Synchronises the stream.  No counterpart in the reference. */
int mcfd_autotune(mcfd_geom* geom, const mcfd_config* cfg, const double* U, int32_t* chosen, void* stream);
/* Set the launch shapes directly (host [5], the layout mcfd_autotune fills;
 * 0 = default), e.g. to replay a tuning saved from an earlier run.  Results
 * do not depend on them.  No counterpart in the reference. */
int mcfd_set_launch_shapes(mcfd_geom* geom, const int32_t* shapes);
/* on = 1: run each explicit stage (mcfd_explicit_step, _record) as one
 * cooperative launch of one resident grid — reconstruction, face fluxes and
 * gather separated by grid barriers — where the settings allow it (fast
 * mode, HLLC, MUSCL linear with a capped limiter, inviscid, no pressure-inlet or
 * mass-flow patches, no body force); other settings keep the launch per
 * kernel.  Results are identical either way.  on = 0 (the default) restores
 * the launch per kernel.  No counterpart in the reference. */
int mcfd_set_fused_stage(mcfd_geom* geom, int32_t on);
/* Resident 256-thread blocks per SM of the last one-launch stage (0 before
 * any).  No counterpart in the reference. */
int mcfd_fused_stage_blocks(const mcfd_geom* geom);
/* mcfd_explicit_step that also copies, for every stage k, the primitive state
 * it evaluates the residual at into stage_P[k] ([n_cells][4]) and, for MUSCL,
 * its face states into stage_recon[k] ([n_limiter][4], may be NULL): the
 * linearisation points a reverse sweep needs (mcfd_vjp_at).  n_stages >= the
 * scheme's stage count (1, 2, 3, 5).  No counterpart in the reference. */
int mcfd_explicit_step_record(mcfd_geom* geom, const mcfd_config* cfg, int32_t scheme, double* U,
                              const double* dt, int32_t dt_per_cell, double* const* stage_P,
                              double* const* stage_recon, int32_t n_stages, void* stream);

/*
 * Sum over cells of R[i][k]^2 for k = 0..3 into the device array sums[4]
 * (deterministic two-level tree).  The reference's per-component RMS
 * residual is sqrt(sums[k] / n_cells) (solver.py:944-950).
 */
int mcfd_residual_sumsq(mcfd_geom* geom, const double* R, double* sums, void* stream);

/*
 * Wait for `stream`, then return and clear the accumulated device status.
 */
int mcfd_status_fetch(mcfd_geom* geom, void* stream, mcfd_status* out);
/* The same for the status word of the look-ahead time steps that
 * mcfd_explicit_step_next computes. */
int mcfd_status_fetch_next(mcfd_geom* geom, void* stream, mcfd_status* out);

/* ---- implicit Euler (solver.py:1185-1567) ---- */

/*
 * Prepare the linearised implicit operator at state U (device [n_cells][4]):
 * the first-order scalar preconditioner (_implicit_preconditioner,
 * solver.py:1185-1300, assembled from P(U) and the time step), the
 * first-order residual R1(U) (jacobian_rate, solver.py:1445) with cfg's flux,
 * and |U / scales| (solver.py:1543).  dt: device scalar or [n_cells]
 * (dt_per_cell), copied on the stream.  scales: host [4], the per-variable
 * scaling of the Newton iteration.
 */
int mcfd_implicit_prepare(mcfd_geom* geom, const mcfd_config* cfg, const double* U, const double* dt,
                          int32_t dt_per_cell, const double* scales, void* stream);
/* out = v - dt [R1(U + eps s v) - R1(U)] / (eps s), eps = sqrt(eps_mach)
 * max(1,|U/s|) / |v| (_matrix_free_implicit_operator, solver.py:1532-1567).
 * v, out: device [4 n_cells]. */
int mcfd_implicit_matvec(mcfd_geom* geom, const double* v, double* out, void* stream);
/* Select the Jacobian of the GMRES operator: 0 = the reference's finite
 * difference (default), 1 = the exact Jacobian (mcfd_jvp of R1). */
int mcfd_implicit_set_jacobian(mcfd_geom* geom, int32_t exact);
/* Exact Jacobian-vector product of the residual: dR = (dR/dU)(U) dU, for the
 * same settings as mcfd_residual (forward mode; limiter and flux switches
 * differentiated on the branch the state takes).  No counterpart in the
 * reference, which only forms finite differences (solver.py:1532-1567).
 * U, dU, dR: device [n_cells][4]. */
int mcfd_jvp(mcfd_geom* geom, const mcfd_config* cfg, const double* U, const double* dU, double* dR,
             void* stream);
/* Reverse-mode product of the residual: U_bar = (dR/dU)(U)^T lambda, the
 * transpose of mcfd_jvp's Jacobian (same switches).  far_bar (device
 * [n_far_field][4], may be NULL) receives lambda^T dR/d(far-field state) per
 * far-field face.  No counterpart in the reference.  U, lambda, U_bar: device
 * [n_cells][4]. */
int mcfd_vjp(mcfd_geom* geom, const mcfd_config* cfg, const double* U, const double* lambda, double* U_bar,
             double* far_bar, void* stream);
/* mcfd_vjp at a state whose primitive P and (MUSCL) face states recon the
 * caller already has (from mcfd_explicit_step_record).  U may be NULL: the
 * product needs only P and recon. */
int mcfd_vjp_at(mcfd_geom* geom, const mcfd_config* cfg, const double* U, const double* P, const double* recon,
                const double* lambda, double* U_bar, double* far_bar, void* stream);
/* Pressure force on the wall faces along (dir_x, dir_y): J = sum over wall
 * faces of p(owner) (n . dir) L, with n pointing out of the fluid cell; dJdU
 * (device [n_cells][4], may be NULL) receives dJ/dU.  J: host scalar. */
int mcfd_wall_force(mcfd_geom* geom, const mcfd_config* cfg, const double* U, double dir_x, double dir_y,
                    double* J, double* dJdU, void* stream);
/* x = (D+U)^-1 D (D+L)^-1 v with the prepared scalar matrix applied to each
 * of the four variables (LU-SGS, solver.py:1302-1323, the two
 * spsolve_triangular calls): level-scheduled sweeps over the dependency
 * graph of the natural cell order, so the result is the sequential
 * triangular solves' (rows summed in ascending column order). */
int mcfd_lusgs_apply(mcfd_geom* geom, const double* v, double* x, void* stream);
/* Launch schedule of the LU-SGS sweeps: runs of levels at most wide_level
 * rows wide go to one launch, wider levels get a grid launch each.  engine
 * chooses how such a run is swept: 1 one block with a barrier per level;
 * 2, 3, 4: one block of 512, 1024 or 256 threads whose rows wait only for
 * the rows they read (no barrier per level, chunks of consecutive levels in
 * flight together); 5: as 2 with the rows' products on the integer pipe
 * (the same IEEE products); 6: as 2 with one thread per (row, component),
 * chunks of at most 8 rows; 8 or 16 a
 * thread-block cluster of that many blocks sharing their latest solutions in
 * distributed shared memory, a cluster barrier per level; 7 or 9 a cluster
 * of 8 or 16 blocks, each owning a band of consecutive cell ids, sweeping
 * windows of up to 32 levels with a block barrier per level and a cluster
 * barrier per window (each block recomputes the rows of other bands its own
 * rows depend on inside the window; a plan that does not fit shared memory
 * takes engine 2).  0 restores the defaults (wide_level 16384, engine 9
 * where the device runs clusters of 16, else 7, else 2); 7, 8, 9 or 16
 * returns MCFD_E_UNSUPPORTED where the device cannot run that cluster size.
 * Results do not depend on it.  No counterpart in the reference. */
int mcfd_implicit_set_sweep(mcfd_geom* geom, int32_t wide_level, int32_t engine);
/* Rows per chunk of the per-row-wait sweeps (engines 2-6): 1..32 (at most 8
 * for engine 6), 0 restores the default (32; 8 for engine 6).  A chunk is a run of consecutive rows of one level taken
 * by one warp.  Results do not depend on it.  No counterpart in the
 * reference. */
int mcfd_implicit_set_chunk(mcfd_geom* geom, int32_t rows);
/* Solve operator(x) = b with restarted GMRES(krylov_dim) preconditioned by
 * LU-SGS, as _solve_gmres drives SciPy's gmres (solver.py:1489-1529; left
 * preconditioning, modified Gram-Schmidt, Givens rotations).  b, x: device
 * [4 n_cells].  Returns MCFD_OK, MCFD_E_NOT_CONVERGED or MCFD_E_BREAKDOWN.
 * The Arnoldi steps of a restart cycle run without a host round trip: the
 * cycle is a CUDA graph whose loop condition the device sets. */
int mcfd_gmres(mcfd_geom* geom, const double* b, double* x, double tol, int32_t max_iter,
               int32_t krylov_dim, int32_t* iterations, void* stream);
/* Newton equation e = U - U0 - dt R (solver.py:1415-1418): writes
 * b = -(e / scales) when b is non-NULL and returns norms[0] = max|e / s|,
 * norms[1] = max|(U - U0) / s| (host [2]). */
int mcfd_implicit_equation(mcfd_geom* geom, const double* U, const double* U0, const double* R,
                           const double* dt, int32_t dt_per_cell, const double* scales, double* b,
                           double* norms, void* stream);
/* Maxima for the variable scaling (solver.py:1393-1413), host [9]:
 * max rho, max|u|, max|v|, max c, max p, max|U_0|, max|U_1|, max|U_2|, max|U_3|. */
int mcfd_implicit_scale_maxima(mcfd_geom* geom, const mcfd_config* cfg, const double* U,
                               double* maxima, void* stream);
/* out = U + (damping * dx) * scales (line-search candidate, solver.py:1462-1464). */
int mcfd_implicit_candidate(mcfd_geom* geom, const double* U, const double* dx, double damping,
                            const double* scales, double* out, void* stream);

/* ---- measurement ---- */

/* kernel classes for mcfd_profile_read */
#define MCFD_PROF_PRIMITIVE 0
#define MCFD_PROF_RECONSTRUCT 1
#define MCFD_PROF_FLUX 2
#define MCFD_PROF_GATHER 3
#define MCFD_PROF_TIME_STEP 4
#define MCFD_PROF_OTHER 5
#define MCFD_PROF_COUNT 6

/*
 * When enabled, every kernel launch group of this handle is bracketed by CUDA
 * events recorded on its launching stream.  mcfd_profile_read waits for the
 * last event, writes per-class total milliseconds and launch-group counts
 * (arrays of MCFD_PROF_COUNT), and clears the record.
 */
int mcfd_profile_enable(mcfd_geom* geom, int32_t enable);
int mcfd_profile_read(mcfd_geom* geom, double* total_ms, int64_t* groups);

/*
 * Batched cases (no counterpart in the reference, which solves one case per
 * call): the geometry holds independent cases back to back, cells of case k
 * in [case_offsets[k], case_offsets[k+1]) (device int32 [n_cases + 1]).
 * Writes each case's global stable time step (min over its cells,
 * solver.py:4117-4129) to dt_case (device [n_cases]) and broadcasts it to
 * dt_cells (device [n_cells]) for mcfd_explicit_step with dt_per_cell = 1.
 */
int mcfd_batch_time_steps(mcfd_geom* geom, const mcfd_config* cfg, const double* P,
                          const int32_t* case_offsets, int32_t n_cases, double* dt_case,
                          double* dt_cells, void* stream);

/* Number of kernels this library has launched in the process so far. */
int64_t mcfd_launch_count(void);

/*
 * Allocation-free sum of squares: sums[k] = sum over i < n_cells of
 * R[i][k]^2 (k = 0..3), the same reduction and summation order as
 * mcfd_residual_sumsq, but with no geometry handle and no device allocation.
 * No counterpart in the reference (it exists for callers that cannot call
 * cudaMalloc, such as a monitor inside a host time loop whose device memory is
 * owned by another allocator).  Its scratch is a fixed 19,456-byte __device__
 * array shared by all calls: overlapping calls race.  The first call on each
 * device looks up that array's address (call it once before any stream
 * capture); the address stays cached for the process, so do not call it
 * again on a device after cudaDeviceReset.  n_cells above 2^30 returns
 * MCFD_E_TOO_LARGE.  The status reads the thread's CUDA error state without
 * clearing it, so an earlier call's pending error is reported as MCFD_E_CUDA.
 */
int mcfd_residual_sumsq_noalloc(const double* R, int64_t n_cells, double* sums, void* stream);

/*
 * Element-wise IEEE binary64 division and square root exactly as the
 * residual kernels evaluate them (integer-pipe routines, round to nearest
 * even; bit-identical to the FP64 unit): quotient[i] = a[i] / b[i] and
 * root[i] = sqrt(a[i]) for i < n.  Device arrays; either output may be NULL
 * (b is read only for the quotient).  No reference counterpart: it exposes
 * the arithmetic the residual path is built on, for verification.
 */
int mcfd_ieee_div_sqrt(const double* a, const double* b, int64_t n, double* quotient, double* root,
                       void* stream);
/* Element-wise IEEE binary64 product on the integer pipe, as the
 * exact-arithmetic kernels evaluate part of their products:
 * product[i] = a[i] * b[i], bit-identical to the FP64 unit.  Device arrays of
 * n doubles.  No reference counterpart (verification). */
int mcfd_ieee_mul(const double* a, const double* b, int64_t n, double* product, void* stream);
/* Element-wise IEEE binary64 division as the LU-SGS sweeps evaluate it:
 * quotient[i] = a[i] / b[i] from the divisor's correctly rounded reciprocal
 * (a Markstein-corrected candidate accepted by an exact remainder test, the
 * integer-pipe division otherwise), bit-identical to the FP64 unit.  Device
 * arrays of n doubles.  No reference counterpart (verification). */
int mcfd_ieee_div_fma(const double* a, const double* b, int64_t n, double* quotient, void* stream);

/* ---- host helpers (no GPU needed) ---- */

/*
 * Cell centroids and areas by the shoelace formula in the reference's
 * operation order (solver.py:1655-1676).  Returns MCFD_E_GEOMETRY and sets
 * *bad_cell for a zero/invalid area ("Cell {id} has zero or invalid area.").
 */
int mcfd_host_cell_geometry(int64_t n_cells, const int64_t* cell_offsets,
                            const int64_t* cell_nodes, const double* points, double* centers,
                            double* areas, int64_t* bad_cell);

/*
 * Face centres, unit normals pointing out of the owner, and lengths
 * (solver.py:1678-1695).  The length is sqrt(fma(ey, ey, ex*ex)) and the
 * orientation test fma(n_y, d_y, n_x*d_x) — the FMA-based BLAS dot the
 * reference's np.linalg.norm / np.dot resolve to on FMA hardware.
 */
int mcfd_host_face_geometry(int64_t n_faces, const int64_t* face_nodes, const double* points,
                            const double* centers, const int64_t* owners, double* face_centers,
                            double* normals, double* lengths, int64_t* bad_face);

/*
 * The two-ring stencil of the MUSCL-parabolic reconstruction
 * (_parabolic_stencil, solver.py:2241-2291): per cell, a breadth-first search
 * of depth two over the gradient entries (sources, neighbours, dx, dy in the
 * reference's entry order), each (cell, offset) pair once with offsets keyed
 * by Python's round(offset / domain_scale, 10), pairs with a non-zero offset
 * kept in visiting order.  Host code (several threads).  Writes at most
 * `capacity` entries and the count to *out_count; MCFD_E_ARG when the count
 * exceeds capacity (*out_count then holds the count needed).
 */
int mcfd_host_parabolic_stencil(int64_t n_cells, int64_t n_entries, const int64_t* sources,
                                const int64_t* neighbours, const double* dx, const double* dy,
                                double domain_scale, int64_t capacity, int64_t* out_sources,
                                int64_t* out_neighbours, double* out_dx, double* out_dy,
                                int64_t* out_count);

/*
 * The geometry build's numeric loops on the device (device pointers, int64
 * indices; the same arrays as the host build bit for bit): cell centroids
 * and areas (mcfd_host_cell_geometry's sums, solver.py:1655-1676); face
 * centres, outward unit normals and lengths (mcfd_host_face_geometry,
 * solver.py:1678-1695); the least-squares gradient offsets, coefficients
 * (solver.py:2004-2078) of an entry list whose first n_interior_entries
 * entries are the interior faces' (owner, neighbour) pairs and the rest the
 * periodic pairs' (periodic_shifts [pairs][2]), with cell_entry_ptr /
 * cell_entry_order the entries of each cell in entry order and scratch
 * [2 n_entries + 3 n_cells] doubles; and the limiter-entry offsets (face
 * centre minus cell centre, solver.py:2098-2105).  bad_cell / bad_face:
 * device uint64 holding UINT64 / INT64 max on entry, left at the smallest
 * invalid cell (zero / non-finite area) or face (zero / non-finite length).
 * No counterpart as such in the reference (its loops run in Python).
 */
int mcfd_device_cell_geometry(int64_t n_cells, const int64_t* cell_offsets, const int64_t* cell_nodes,
                              const double* points, double* centers, double* areas, uint64_t* bad_cell,
                              void* stream);
int mcfd_device_face_geometry(int64_t n_faces, const int64_t* face_nodes, const double* points,
                              const double* centers, const int64_t* owners, double* face_centers, double* normals,
                              double* lengths, uint64_t* bad_face, void* stream);
int mcfd_device_gradient_coefficients(int64_t n_cells, int64_t n_entries, int64_t n_interior_entries,
                                      const int64_t* sources, const int64_t* neighbours, const double* centers,
                                      const double* periodic_shifts, const int64_t* cell_entry_ptr,
                                      const int64_t* cell_entry_order, double* dx, double* dy, double* cx,
                                      double* cy, double* scratch, void* stream);
int mcfd_device_limiter_offsets(int64_t n_slots, const int64_t* slot_faces, const int64_t* slot_cells,
                                const double* face_centers, const double* centers, double* dx, double* dy,
                                void* stream);

#ifdef __cplusplus
}
#endif

#endif /* MESHCFD_GB300_H */
