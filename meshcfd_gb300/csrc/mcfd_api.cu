// C ABI of the residual / explicit-step path: geometry packing (host), device
// workspace, and the orchestration of kernels per entry point.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <vector>

#include "mcfd_implicit.h"
#include "mcfd_jvp.h"
#include "mcfd_vjp.h"
#include "mcfd_internal.h"

using namespace mcfd;

struct ProfRecord {
  int cls;
  cudaEvent_t start, stop;
};

struct mcfd_geom {
  DevGeom g;
  bool profiling = false;
  std::vector<ProfRecord> records;
  std::vector<cudaEvent_t> event_pool;
  Workspace ws;
  void* arena = nullptr;       // one device allocation for geometry + workspace
  size_t arena_bytes = 0;
  DevStatus* status = nullptr;  // inside the arena
  DevStatus* status_next = nullptr;  // the look-ahead time steps' word (mcfd_explicit_step_next), inside the arena
  DevStatus* host_status = nullptr;  // pinned
  mcfd_geom_info info{};
  ImplicitTopology topo;       // host copy for the implicit path (built lazily)
  ImplicitState imp;
  bool imp_built = false;
  mcfd_config imp_cfg{};       // first-order settings of the prepared operator
  int imp_exact_jacobian = 0;  // GMRES operator: 0 finite differences (reference), 1 exact JVP
  JvpWork jvp;                 // tangent workspace (allocated on first use)
  VjpWork vjp;                 // adjoint workspace (allocated on first use)
  SideStream side;             // boundary face segments of the forward flux
  std::vector<void*> jvp_owned;
  ViscousWork visc;            // laminar viscous workspace (allocated on first use)
  // mcfd_explicit_step_record: per-stage copies of the primitive and face states
  double* const* rec_P = nullptr;
  double* const* rec_recon = nullptr;
  int rec_n = 0, rec_k = 0;
  // explicit stages as one cooperative launch where the settings allow it
  bool fused_stage = false;
  int fused_blocks = 0;  // resident blocks per SM of the last fused launch
};

namespace {

constexpr int64_t kMaxIndex = (int64_t)1 << 30;

struct Arena {
  std::vector<std::pair<size_t, size_t>> pieces;  // offset, bytes
  size_t size = 0;
  size_t take(size_t bytes) {
    size_t off = (size + 255) & ~(size_t)255;
    size = off + (bytes ? bytes : 1);
    return off;
  }
};

// Stable counting sort of entries by key; returns CSR pointers and the order.
void group_by(const std::vector<int>& key, int n_keys, std::vector<int>& ptr, std::vector<int>& order) {
  ptr.assign(n_keys + 1, 0);
  for (int k : key) ptr[k + 1]++;
  for (int i = 0; i < n_keys; ++i) ptr[i + 1] += ptr[i];
  order.resize(key.size());
  std::vector<int> fill(ptr.begin(), ptr.end() - 1);
  for (size_t e = 0; e < key.size(); ++e) order[fill[key[e]]++] = (int)e;
}

bool in_range(int64_t v, int64_t n) { return v >= 0 && v < n; }

}  // namespace


// ---- helpers (C++ linkage)
static int check_cfg(const mcfd_config* cfg) {
  if (!cfg) return MCFD_E_ARG;
  if (cfg->flux < 0 || cfg->flux > 2) return MCFD_E_ARG;
  if (cfg->limiter < 0 || cfg->limiter > MCFD_LIMITER_VENKATAKRISHNAN_K) return MCFD_E_ARG;
  if (cfg->limiter == MCFD_LIMITER_VENKATAKRISHNAN_K &&
      (!(cfg->venkat_k > 0.0) || !std::isfinite(cfg->venkat_k)))
    return MCFD_E_ARG;
  if (cfg->reconstruction < 0 || cfg->reconstruction > 2) return MCFD_E_ARG;
  if (!(cfg->gamma > 1.0)) return MCFD_E_ARG;
  if (cfg->mode < MCFD_MODE_EXACT || cfg->mode > MCFD_MODE_FMA) return MCFD_E_ARG;
  // the smooth Venkatakrishnan form is built for MUSCL linear only
  if (cfg->limiter == MCFD_LIMITER_VENKATAKRISHNAN_K && cfg->reconstruction == MCFD_RECON_MUSCL_PARABOLIC)
    return MCFD_E_UNSUPPORTED;
  if (cfg->viscosity_model < MCFD_VISC_INVISCID || cfg->viscosity_model > MCFD_VISC_SUTHERLAND) return MCFD_E_ARG;
  if (cfg->viscosity_model != MCFD_VISC_INVISCID && (!(cfg->gas_constant > 0.0) || !(cfg->prandtl_number > 0.0)))
    return MCFD_E_ARG;
  return MCFD_OK;
}

static int rc(cudaError_t e) { return e == cudaSuccess ? MCFD_OK : MCFD_E_CUDA; }

static cudaEvent_t take_event(mcfd_geom* h) {
  if (!h->event_pool.empty()) {
    cudaEvent_t e = h->event_pool.back();
    h->event_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

// Runs `launch` (returning cudaError_t), bracketed by events when profiling.
template <typename F>
static cudaError_t timed(mcfd_geom* h, int cls, cudaStream_t s, F&& launch) {
  if (!h->profiling) return launch();
  ProfRecord r{cls, take_event(h), take_event(h)};
  cudaEventRecord(r.start, s);
  cudaError_t e = launch();
  cudaEventRecord(r.stop, s);
  h->records.push_back(r);
  return e;
}

// Kernel variant dispatch on cfg.mode.
#define MCFD_DISPATCH(cfg, call) \
  ((cfg).mode == MCFD_MODE_FAST ? fast::call : (cfg).mode == MCFD_MODE_FMA ? fma::call : exact::call)

// One residual evaluation of the state whose primitive is in ws.P, followed
// by the gather with the given stage program.
// The laminar viscous workspace, allocated on the first viscous call; refuses
// geometries without the viscous tables (or with walls lacking thermal data).
static int ensure_viscous(mcfd_geom* h, const mcfd_config* cfg) {
  if (cfg->viscosity_model == MCFD_VISC_INVISCID) return MCFD_OK;
  if (!h->g.viscous_ok) return MCFD_E_UNSUPPORTED;
  if (h->visc.cell) return MCFD_OK;
  const size_t C = h->g.n_cells, NF = h->g.seg_begin[SEG_PERIODIC + 1], ND = h->g.n_diffusive;
  double** fields[] = {&h->visc.cell, &h->visc.grad, &h->visc.flux, &h->visc.bflux, &h->visc.r, &h->visc.diff};
  const size_t sizes[] = {4 * C, 6 * C, 4 * (NF > 0 ? NF : 1), 4 * (ND > 0 ? ND : 1), 4 * C, C};
  for (int k = 0; k < 6; ++k) {
    if (cudaMalloc((void**)fields[k], sizes[k] * sizeof(double)) != cudaSuccess) return MCFD_E_CUDA;
    h->jvp_owned.push_back(*fields[k]);
  }
  h->g.visc_diff = h->visc.diff;
  return MCFD_OK;
}

static cudaError_t stage(mcfd_geom* h, const mcfd_config& cfg, const StageProgram& prog_in,
                         cudaStream_t s) {
  StageProgram prog = prog_in;
  cudaError_t e = cudaSuccess;
  // mcfd_explicit_step_record: the face states go straight into the caller's
  // record buffer (the primitive is copied below)
  const bool record = h->rec_P && h->rec_k < h->rec_n;
  double* recon_out = h->ws.recon;
  if (record && h->rec_recon && h->rec_recon[h->rec_k] && cfg.reconstruction != MCFD_RECON_FIRST_ORDER)
    recon_out = h->rec_recon[h->rec_k];
  if (h->fused_stage && MCFD_DISPATCH(cfg, stage_fused_supported(h->g, cfg, prog))) {
    if (record) {
      const int k = h->rec_k++;
      e = cudaMemcpyAsync(h->rec_P[k], h->ws.P, 4 * sizeof(double) * (size_t)h->g.n_cells, cudaMemcpyDeviceToDevice,
                          s);
    }
    if (e == cudaSuccess)
      e = timed(h, MCFD_PROF_OTHER, s, [&] {
        return MCFD_DISPATCH(cfg, launch_stage_fused(h->g, cfg, h->ws.P, recon_out, h->ws.flux, prog, s,
                                                     &h->fused_blocks));
      });
    return e;
  }
  if (cfg.reconstruction == MCFD_RECON_MUSCL_LINEAR)
    e = timed(h, MCFD_PROF_RECONSTRUCT, s, [&] { return MCFD_DISPATCH(cfg, launch_reconstruct(h->g, cfg, h->ws.P, recon_out, s)); });
  else if (cfg.reconstruction == MCFD_RECON_MUSCL_PARABOLIC)
    e = timed(h, MCFD_PROF_RECONSTRUCT, s, [&] { return launch_reconstruct_parabolic(h->g, cfg, h->ws.P, recon_out, s); });
  if (e == cudaSuccess && h->g.n_bc_patches > 0) {
    const double* recon = cfg.reconstruction == MCFD_RECON_FIRST_ORDER ? nullptr : recon_out;
    e = timed(h, MCFD_PROF_FLUX, s, [&] { return launch_bc_states(h->g, cfg, h->ws.P, recon, h->g.bc_ext, s); });
  }
  if (e == cudaSuccess && cfg.viscosity_model != MCFD_VISC_INVISCID) {  // solver.py:2699-2702
    if (h->g.n_bc_patches > 0) e = launch_bc_states(h->g, cfg, h->ws.P, nullptr, h->g.bc_ext_dt, s);
    if (e == cudaSuccess)
      e = timed(h, MCFD_PROF_OTHER, s, [&] { return launch_viscous_residual(h->g, cfg, h->ws.P, h->visc, s); });
    prog.visc_r = h->visc.r;
  }
  if (e == cudaSuccess && record) {
    const int k = h->rec_k++;
    e = cudaMemcpyAsync(h->rec_P[k], h->ws.P, 4 * sizeof(double) * (size_t)h->g.n_cells, cudaMemcpyDeviceToDevice, s);
  }
  if (e == cudaSuccess)
    e = timed(h, MCFD_PROF_FLUX, s, [&] { return MCFD_DISPATCH(cfg, launch_flux(h->g, cfg, h->ws.P, recon_out, h->ws.flux, s, &h->side)); });
  if (e == cudaSuccess)
    e = timed(h, MCFD_PROF_GATHER, s, [&] { return MCFD_DISPATCH(cfg, launch_gather(h->g, cfg, h->ws.P, h->ws.flux, prog, s)); });
  return e;
}

static StageTerm term(int kind, double coef, const double* x) {
  StageTerm t;
  t.kind = kind;
  t.coef = coef;
  t.x = x;
  return t;
}

extern "C" {

int mcfd_abi_version(void) { return MCFD_ABI_VERSION; }

const char* mcfd_error_string(int code) {
  switch (code) {
    case MCFD_OK: return "ok";
    case MCFD_E_ARG: return "invalid argument";
    case MCFD_E_CUDA: return "CUDA runtime error";
    case MCFD_E_UNSUPPORTED: return "option not supported by the GPU path";
    case MCFD_E_GEOMETRY: return "inconsistent geometry description";
    case MCFD_E_TOO_LARGE: return "size exceeds the maximum of the allocation-free entry point";
    case MCFD_E_NOT_CONVERGED: return "GMRES did not converge";
    case MCFD_E_BREAKDOWN: return "GMRES broke down";
    default: return "unknown error";
  }
}

int mcfd_geom_create(const mcfd_geom_desc* d, mcfd_geom** out) {
  if (!d || !out) return MCFD_E_ARG;
  *out = nullptr;
  const int64_t C = d->n_cells, F = d->n_faces, NI = d->n_interior, NP = d->n_periodic;
  const int64_t NW = d->n_wall, NV = d->n_velocity_inlet, NO = d->n_pressure_outlet,
                NF = d->n_far_field, NG = d->n_gradient, NL = d->n_limiter;
  if (C <= 0 || F < 0 || C > kMaxIndex || F > kMaxIndex || NG > kMaxIndex) return MCFD_E_ARG;
  if (NL != F + NI) return MCFD_E_GEOMETRY;
  if (!d->areas || !d->owners || !d->neighbours || (F && (!d->face_normals || !d->face_lengths)))
    return MCFD_E_ARG;
  // ---- validate indices (so no kernel can index out of bounds)
  for (int64_t f = 0; f < F; ++f) {
    if (!in_range(d->owners[f], C)) return MCFD_E_GEOMETRY;
    if (d->neighbours[f] >= C) return MCFD_E_GEOMETRY;
  }
  for (int64_t i = 0; i < NI; ++i) {
    int64_t f = d->interior_faces[i];
    if (!in_range(f, F) || d->neighbours[f] < 0) return MCFD_E_GEOMETRY;
    if (i > 0 && f <= d->interior_faces[i - 1]) return MCFD_E_GEOMETRY;
  }
  auto check_faces = [&](const int64_t* faces, int64_t n) {
    for (int64_t i = 0; i < n; ++i)
      if (!in_range(faces[i], F) || d->neighbours[faces[i]] >= 0) return false;
    return true;
  };
  if (!check_faces(d->periodic_faces_a, NP) || !check_faces(d->periodic_faces_b, NP) ||
      !check_faces(d->wall_faces, NW) || !check_faces(d->velocity_inlet_faces, NV) ||
      !check_faces(d->pressure_outlet_faces, NO) || !check_faces(d->far_field_faces, NF))
    return MCFD_E_GEOMETRY;
  for (int64_t e = 0; e < NG; ++e)
    if (!in_range(d->gradient_sources[e], C) || !in_range(d->gradient_neighbours[e], C))
      return MCFD_E_GEOMETRY;
  for (int64_t s = 0; s < NL; ++s)
    if (!in_range(d->limiter_cells[s], C)) return MCFD_E_GEOMETRY;
  const int64_t NE = d->n_parabolic;
  if (NE < 0 || NE > kMaxIndex) return MCFD_E_ARG;
  if (NE && (!d->parabolic_sources || !d->parabolic_neighbours || !d->parabolic_dx || !d->parabolic_dy))
    return MCFD_E_ARG;
  for (int64_t e = 0; e < NE; ++e)
    if (!in_range(d->parabolic_sources[e], C) || !in_range(d->parabolic_neighbours[e], C)) return MCFD_E_GEOMETRY;
  const int64_t NBP = d->n_bc_patches;
  if (NBP < 0 || NBP > kMaxIndex) return MCFD_E_ARG;
  if (NBP && (!d->bc_kind || !d->bc_values || !d->bc_offsets || !d->bc_direction_normal)) return MCFD_E_ARG;
  const int64_t NB = NBP ? d->bc_offsets[NBP] : 0;
  const int64_t ND = d->n_diffusive;
  if (ND < 0 || ND > kMaxIndex) return MCFD_E_ARG;
  if (ND && (!d->diffusive_faces || !d->diffusive_kind || !d->diffusive_thermal || !d->diffusive_value ||
             !d->diffusive_inlet || !d->diffusive_normal_distance || !d->diffusive_ghost_offset ||
             !d->diffusive_offset))
    return MCFD_E_ARG;
  if (NBP) {
    if (d->bc_offsets[0] != 0) return MCFD_E_GEOMETRY;
    for (int64_t k = 0; k < NBP; ++k) {
      if (d->bc_offsets[k + 1] < d->bc_offsets[k]) return MCFD_E_GEOMETRY;
      if (d->bc_kind[k] < MCFD_BC_PRESSURE_INLET || d->bc_kind[k] > MCFD_BC_MASS_FLOW_OUTLET) return MCFD_E_ARG;
    }
    if (NB > kMaxIndex || (NB && !d->bc_faces)) return MCFD_E_ARG;
    if (!check_faces(d->bc_faces, NB)) return MCFD_E_GEOMETRY;
  }
  if (ND && !check_faces(d->diffusive_faces, ND)) return MCFD_E_GEOMETRY;
  for (int64_t j = 0; j < ND; ++j) {
    const int src = d->diffusive_inlet[j] >> 28, idx = d->diffusive_inlet[j] & 0x0fffffff;
    const int64_t limit = src == 1 ? NV : src == 2 ? NB : src == 3 ? NF : 1;
    if (src < 0 || src > 3 || idx >= limit || d->diffusive_kind[j] < 0 || d->diffusive_kind[j] > 5)
      return MCFD_E_GEOMETRY;
  }
  for (int64_t c = 0; c < C; ++c)
    if (!(d->areas[c] > 0.0)) return MCFD_E_GEOMETRY;

  // ---- flux faces
  const int64_t n_flux = NI + NP + NW + NV + NO + NF + NB;
  if (n_flux > kMaxIndex) return MCFD_E_ARG;
  int seg_begin[SEG_COUNT + 1];
  seg_begin[SEG_INTERIOR] = 0;
  seg_begin[SEG_PERIODIC] = (int)NI;
  seg_begin[SEG_WALL] = (int)(NI + NP);
  seg_begin[SEG_VIN] = (int)(NI + NP + NW);
  seg_begin[SEG_POUT] = (int)(NI + NP + NW + NV);
  seg_begin[SEG_FAR] = (int)(NI + NP + NW + NV + NO);
  seg_begin[SEG_BCX] = (int)(NI + NP + NW + NV + NO + NF);
  seg_begin[SEG_COUNT] = (int)n_flux;
  std::vector<int> lslot(n_flux), rslot(n_flux, -1), lcell(n_flux), rcell(n_flux, -1);
  std::vector<double> normal(2 * n_flux), flen(n_flux), wallv(2 * NW, 0.0), vin(4 * NV), pout(NO), far(4 * NF);
  auto set_face = [&](int64_t k, int64_t f) {
    lslot[k] = (int)f;
    lcell[k] = (int)d->owners[f];
    flen[k] = d->face_lengths[f];
    normal[2 * k] = d->face_normals[2 * f];
    normal[2 * k + 1] = d->face_normals[2 * f + 1];
  };
  for (int64_t i = 0; i < NI; ++i) {
    int64_t f = d->interior_faces[i];
    set_face(i, f);
    rslot[i] = (int)(F + i);
    rcell[i] = (int)d->neighbours[f];
  }
  for (int64_t i = 0; i < NP; ++i) {
    int64_t k = seg_begin[SEG_PERIODIC] + i;
    set_face(k, d->periodic_faces_a[i]);
    rslot[k] = (int)d->periodic_faces_b[i];
    rcell[k] = (int)d->owners[d->periodic_faces_b[i]];
  }
  for (int64_t i = 0; i < NW; ++i) {
    int64_t f = d->wall_faces[i];
    set_face(seg_begin[SEG_WALL] + i, f);
    if (d->wall_velocities) {
      wallv[2 * i] = d->wall_velocities[2 * f];
      wallv[2 * i + 1] = d->wall_velocities[2 * f + 1];
    }
  }
  for (int64_t i = 0; i < NV; ++i) {
    set_face(seg_begin[SEG_VIN] + i, d->velocity_inlet_faces[i]);
    for (int k = 0; k < 4; ++k) vin[4 * i + k] = d->velocity_inlet_states[4 * i + k];
  }
  for (int64_t i = 0; i < NO; ++i) {
    set_face(seg_begin[SEG_POUT] + i, d->pressure_outlet_faces[i]);
    pout[i] = d->pressure_outlet_pressures[i];
  }
  for (int64_t i = 0; i < NF; ++i) {
    set_face(seg_begin[SEG_FAR] + i, d->far_field_faces[i]);
    for (int k = 0; k < 4; ++k) far[4 * i + k] = d->far_field_states[4 * i + k];
  }
  std::vector<int> bc_ptr(NBP + 1, 0), bc_kind(NBP);
  std::vector<double> bc_values(4 * NBP), bc_dn(NB);
  for (int64_t k = 0; k < NBP; ++k) {
    bc_ptr[k + 1] = (int)d->bc_offsets[k + 1];
    bc_kind[k] = d->bc_kind[k];
    for (int j = 0; j < 4; ++j) bc_values[4 * k + j] = d->bc_values[4 * k + j];
  }
  for (int64_t i = 0; i < NB; ++i) {
    set_face(seg_begin[SEG_BCX] + i, d->bc_faces[i]);
    bc_dn[i] = d->bc_direction_normal[i];
  }

  // ---- cell gather, interior part: the SciPy CSR divergence operator
  // (solver.py:2160-2174) with data (-L)/A_owner and L/A_neighbour, summed per
  // row in ascending face (column) order.
  std::vector<int> key, gi_ptr, order;
  std::vector<int> gi_flux;
  std::vector<double> gi_coef;
  {
    key.resize(2 * NI);
    std::vector<double> coef(2 * NI);
    std::vector<int> col(2 * NI);
    for (int64_t i = 0; i < NI; ++i) {
      int64_t f = d->interior_faces[i];
      int64_t o = d->owners[f], n = d->neighbours[f];
      double L = d->face_lengths[f];
      key[2 * i] = (int)o;
      coef[2 * i] = -L / d->areas[o];
      col[2 * i] = (int)i;
      key[2 * i + 1] = (int)n;
      coef[2 * i + 1] = L / d->areas[n];
      col[2 * i + 1] = (int)i;
    }
    group_by(key, (int)C, gi_ptr, order);
    gi_flux.resize(order.size());
    gi_coef.resize(order.size());
    for (size_t j = 0; j < order.size(); ++j) {
      gi_flux[j] = col[order[j]];
      gi_coef[j] = coef[order[j]];
    }
  }
  // ---- cell gather, boundary part in the reference's group order
  // (solver.py:2502-2704): periodic owners_a (-), periodic owners_b (+),
  // walls, velocity inlets, pressure outlets, far field; within a group in
  // face-list order (np.add.at is sequential).
  std::vector<int> gb_ptr, gb_flux;
  std::vector<double> gb_len;
  {
    std::vector<int> bkey, bflux;
    std::vector<double> blen;
    for (int64_t i = 0; i < NP; ++i) {
      int64_t fa = d->periodic_faces_a[i];
      bkey.push_back((int)d->owners[fa]);
      bflux.push_back(seg_begin[SEG_PERIODIC] + (int)i);
      blen.push_back(-d->face_lengths[fa]);
    }
    for (int64_t i = 0; i < NP; ++i) {
      int64_t fa = d->periodic_faces_a[i], fb = d->periodic_faces_b[i];
      bkey.push_back((int)d->owners[fb]);
      bflux.push_back(seg_begin[SEG_PERIODIC] + (int)i);
      blen.push_back(d->face_lengths[fa]);
    }
    for (int seg = SEG_WALL; seg < SEG_COUNT; ++seg) {
      for (int k = seg_begin[seg]; k < seg_begin[seg + 1]; ++k) {
        int64_t f = lslot[k];
        bkey.push_back((int)d->owners[f]);
        bflux.push_back(k);
        blen.push_back(-d->face_lengths[f]);
      }
    }
    group_by(bkey, (int)C, gb_ptr, order);
    gb_flux.resize(order.size());
    gb_len.resize(order.size());
    for (size_t j = 0; j < order.size(); ++j) {
      gb_flux[j] = bflux[order[j]];
      gb_len[j] = blen[order[j]];
    }
  }
  std::vector<int> order_grad;
  // ---- gradient entries grouped by source, reference order kept
  std::vector<int> grad_ptr, grad_nb(NG), grad_twin(NG, -1);
  std::vector<double> grad_cx(NG), grad_cy(NG);
  bool twins_ok = (NG % 2) == 0;
  {
    key.resize(NG);
    for (int64_t e = 0; e < NG; ++e) key[e] = (int)d->gradient_sources[e];
    group_by(key, (int)C, grad_ptr, order);
    order_grad = order;
    std::vector<int> pos(NG);
    for (int64_t j = 0; j < NG; ++j) {
      int e = order[j];
      pos[e] = (int)j;
      grad_nb[j] = (int)d->gradient_neighbours[e];
      grad_cx[j] = d->gradient_coefficients_x[e];
      grad_cy[j] = d->gradient_coefficients_y[e];
    }
    // the reference appends entries in pairs (a -> b, b -> a) per face
    // (solver.py:2004-2021): the twin of entry e is e ^ 1
    for (int64_t e = 0; twins_ok && e < NG; ++e) {
      const int64_t t = e ^ 1;
      if (d->gradient_sources[e] != d->gradient_neighbours[t] || d->gradient_neighbours[e] != d->gradient_sources[t])
        twins_ok = false;
      else
        grad_twin[pos[e]] = pos[t];
    }
    if (!twins_ok) std::fill(grad_twin.begin(), grad_twin.end(), -1);
  }
  // ---- limiter entries grouped by cell
  std::vector<int> lim_ptr, lim_slot(NL);
  std::vector<double> lim_d(2 * NL);
  {
    key.resize(NL);
    for (int64_t s = 0; s < NL; ++s) key[s] = (int)d->limiter_cells[s];
    group_by(key, (int)C, lim_ptr, order);
    for (int64_t j = 0; j < NL; ++j) {
      int s = order[j];
      lim_slot[j] = s;
      lim_d[2 * j] = d->limiter_dx[s];
      lim_d[2 * j + 1] = d->limiter_dy[s];
    }
  }
  // ---- two-ring stencil entries grouped by source, reference order kept
  std::vector<int> par_ptr, par_nb(NE);
  std::vector<double> par_d(2 * NE);
  {
    key.resize(NE);
    for (int64_t e = 0; e < NE; ++e) key[e] = (int)d->parabolic_sources[e];
    group_by(key, (int)C, par_ptr, order);
    for (int64_t j = 0; j < NE; ++j) {
      int e = order[j];
      par_nb[j] = (int)d->parabolic_neighbours[e];
      par_d[2 * j] = d->parabolic_dx[e];
      par_d[2 * j + 1] = d->parabolic_dy[e];
    }
  }
  // ---- laminar viscous tables (solver.py:3615-4114, 4250-4335)
  const bool has_viscous = (d->gradient_dx && d->gradient_dy) || NG == 0;
  std::vector<double> grad_d(has_viscous ? 2 * NG : 0);
  if (has_viscous)
    for (int64_t j = 0; j < NG; ++j) {
      const int e = order_grad[j];
      grad_d[2 * j] = d->gradient_dx[e];
      grad_d[2 * j + 1] = d->gradient_dy[e];
    }
  std::vector<int> vb_ptr, vb_j(ND), diff_owner(ND), diff_kind(ND), diff_thermal(ND), diff_inlet(ND);
  std::vector<double> diff_normal(2 * ND), diff_len(ND), diff_value(ND), diff_nd(ND), diff_ghost(2 * ND),
      diff_offset(2 * ND), diff_wallv(2 * ND, 0.0);
  bool viscous_ok = has_viscous;
  {
    key.resize(ND);
    for (int64_t j = 0; j < ND; ++j) {
      const int64_t f = d->diffusive_faces[j];
      key[j] = (int)d->owners[f];
      diff_owner[j] = (int)d->owners[f];
      diff_normal[2 * j] = d->face_normals[2 * f];
      diff_normal[2 * j + 1] = d->face_normals[2 * f + 1];
      diff_len[j] = d->face_lengths[f];
      diff_kind[j] = d->diffusive_kind[j];
      diff_thermal[j] = d->diffusive_thermal[j];
      diff_inlet[j] = d->diffusive_inlet[j];
      diff_value[j] = d->diffusive_value[j];
      diff_nd[j] = d->diffusive_normal_distance[j];
      for (int k = 0; k < 2; ++k) {
        diff_ghost[2 * j + k] = d->diffusive_ghost_offset[2 * j + k];
        diff_offset[2 * j + k] = d->diffusive_offset[2 * j + k];
        if (d->wall_velocities) diff_wallv[2 * j + k] = d->wall_velocities[2 * f + k];
      }
      if (diff_kind[j] == MCFD_DIFF_WALL_UNKNOWN) viscous_ok = false;
    }
    group_by(key, (int)C, vb_ptr, order);
    for (int64_t i = 0; i < ND; ++i) vb_j[i] = order[i];
  }
  // viscous gather: periodic side a (pair order), side b, then diffusive faces
  std::vector<int> vg_ptr, vg_code;
  {
    std::vector<int> code;
    key.clear();
    for (int64_t k = 0; k < NP; ++k) key.push_back((int)d->owners[d->periodic_faces_a[k]]), code.push_back((int)k);
    for (int64_t k = 0; k < NP; ++k)
      key.push_back((int)d->owners[d->periodic_faces_b[k]]), code.push_back((1 << 28) | (int)k);
    for (int64_t j = 0; j < ND; ++j) key.push_back(diff_owner[j]), code.push_back((2 << 28) | (int)j);
    group_by(key, (int)C, vg_ptr, order);
    vg_code.resize(order.size());
    for (size_t i = 0; i < order.size(); ++i) vg_code[i] = code[order[i]];
  }
  // time-step diffusion: interior owners, interior neighbours, periodic a, b, diffusive faces
  std::vector<int> vd_ptr, vd_other;
  std::vector<double> vd_len, vd_dist;
  if (has_viscous && (NI == 0 || d->interior_distance) && (NP == 0 || d->periodic_distance)) {
    std::vector<int> other;
    std::vector<double> len, dist;
    key.clear();
    for (int side = 0; side < 2; ++side)
      for (int64_t i = 0; i < NI; ++i) {
        const int64_t f = d->interior_faces[i];
        key.push_back((int)(side ? d->neighbours[f] : d->owners[f]));
        other.push_back((int)(side ? d->owners[f] : d->neighbours[f]));
        len.push_back(d->face_lengths[f]);
        dist.push_back(d->interior_distance[i]);
      }
    for (int side = 0; side < 2; ++side)
      for (int64_t k = 0; k < NP; ++k) {
        const int64_t fa = d->periodic_faces_a[k], fb = d->periodic_faces_b[k];
        key.push_back((int)(side ? d->owners[fb] : d->owners[fa]));
        other.push_back((int)(side ? d->owners[fa] : d->owners[fb]));
        len.push_back(d->face_lengths[fa]);
        dist.push_back(d->periodic_distance[k]);
      }
    for (int64_t j = 0; j < ND; ++j) {
      key.push_back(diff_owner[j]);
      other.push_back(-1);
      len.push_back(diff_len[j]);
      dist.push_back(std::fabs(diff_nd[j]));
    }
    group_by(key, (int)C, vd_ptr, order);
    vd_other.resize(order.size());
    vd_len.resize(order.size());
    vd_dist.resize(order.size());
    for (size_t i = 0; i < order.size(); ++i) {
      vd_other[i] = other[order[i]];
      vd_len[i] = len[order[i]];
      vd_dist[i] = dist[order[i]];
    }
  } else {
    viscous_ok = false;
    vd_ptr.assign(C + 1, 0);
  }
  // ---- time-step entries (solver.py:4206-4226)
  std::vector<int> dt_ptr, dt_info;
  std::vector<double> dt_n, dt_len;
  {
    std::vector<int> face_info(F, 0);
    for (int64_t i = 0; i < NV; ++i) face_info[d->velocity_inlet_faces[i]] = (DT_VIN << 28) | (int)i;
    for (int64_t i = 0; i < NO; ++i) face_info[d->pressure_outlet_faces[i]] = (DT_POUT << 28) | (int)i;
    for (int64_t i = 0; i < NF; ++i) face_info[d->far_field_faces[i]] = (DT_FAR << 28) | (int)i;
    for (int64_t i = 0; i < NB; ++i) face_info[d->bc_faces[i]] = (DT_BCX << 28) | (int)i;
    std::vector<int> dface;
    std::vector<int> dinfo;
    key.clear();
    for (int64_t f = 0; f < F; ++f) {
      key.push_back((int)d->owners[f]);
      dface.push_back((int)f);
      dinfo.push_back(face_info[f]);
    }
    for (int64_t i = 0; i < NI; ++i) {
      int64_t f = d->interior_faces[i];
      key.push_back((int)d->neighbours[f]);
      dface.push_back((int)f);
      dinfo.push_back(0);
    }
    group_by(key, (int)C, dt_ptr, order);
    dt_info.resize(order.size());
    dt_n.resize(2 * order.size());
    dt_len.resize(order.size());
    for (size_t j = 0; j < order.size(); ++j) {
      int f = dface[order[j]];
      dt_info[j] = dinfo[order[j]];
      dt_n[2 * j] = d->face_normals[2 * f];
      dt_n[2 * j + 1] = d->face_normals[2 * f + 1];
      dt_len[j] = d->face_lengths[f];
    }
  }

  // ---- visiting order of the per-cell stage kernels: cells grouped by their
  // entry counts (stable), so that each warp's loops share one trip count;
  // cells with 3 or 4 limiter entries first (the fast reconstruction has a
  // kernel compiled for exactly those, and one for the rest)
  std::vector<int> cell_order(C);
  int n_lim34 = 0;
  {
    auto count = [](const std::vector<int>& ptr, size_t c) { return ptr.empty() ? 0 : ptr[c + 1] - ptr[c]; };
    std::vector<long long> ckey(C);
    for (size_t c = 0; c < C; ++c) {
      const long long k0 = count(grad_ptr, c), k1 = count(lim_ptr, c), k2 = count(gi_ptr, c),
                      k3 = count(gb_ptr, c), k4 = count(dt_ptr, c);
      auto clamp = [](long long v) { return v < 0 ? 0 : (v > 4095 ? 4095 : v); };
      const long long other = (k1 == 3 || k1 == 4) ? 0 : 1;
      n_lim34 += other ? 0 : 1;
      ckey[c] = ((((other * 4096 + clamp(k0)) * 4096 + clamp(k1)) * 4096 + clamp(k2)) * 4096 + clamp(k3)) * 64 +
                (k4 > 63 ? 63 : k4);
    }
    for (size_t c = 0; c < C; ++c) cell_order[c] = (int)c;
    std::stable_sort(cell_order.begin(), cell_order.end(), [&](int a, int b) { return ckey[a] < ckey[b]; });
  }

  // ---- arena layout
  Arena A;
  auto bytes_i = [](size_t n) { return n * sizeof(int); };
  auto bytes_d = [](size_t n) { return n * sizeof(double); };
  const int partial_blocks = kSumsqBlocks;
  size_t o_area = A.take(bytes_d(C)), o_cell_order = A.take(bytes_i(C));
  size_t o_grad_ptr = A.take(bytes_i(C + 1)), o_grad_nb = A.take(bytes_i(NG)),
         o_grad_cx = A.take(bytes_d(NG)), o_grad_cy = A.take(bytes_d(NG)), o_grad_twin = A.take(bytes_i(NG));
  size_t o_lim_ptr = A.take(bytes_i(C + 1)), o_lim_slot = A.take(bytes_i(NL)),
         o_lim_d = A.take(bytes_d(2 * NL));
  size_t o_par_ptr = A.take(bytes_i(C + 1)), o_par_nb = A.take(bytes_i(NE)), o_par_d = A.take(bytes_d(2 * NE));
  size_t o_bc_ptr = A.take(bytes_i(NBP + 1)), o_bc_kind = A.take(bytes_i(NBP)), o_bc_values = A.take(bytes_d(4 * NBP)),
         o_bc_dn = A.take(bytes_d(NB));
  size_t o_grad_d = A.take(bytes_d(grad_d.size())), o_vb_ptr = A.take(bytes_i(vb_ptr.size())),
         o_vb_j = A.take(bytes_i(ND)), o_diff_owner = A.take(bytes_i(ND)), o_diff_normal = A.take(bytes_d(2 * ND)),
         o_diff_len = A.take(bytes_d(ND)), o_diff_kind = A.take(bytes_i(ND)), o_diff_thermal = A.take(bytes_i(ND)),
         o_diff_value = A.take(bytes_d(ND)), o_diff_inlet = A.take(bytes_i(ND)), o_diff_nd = A.take(bytes_d(ND)),
         o_diff_ghost = A.take(bytes_d(2 * ND)), o_diff_offset = A.take(bytes_d(2 * ND)),
         o_diff_wallv = A.take(bytes_d(2 * ND)), o_vg_ptr = A.take(bytes_i(vg_ptr.size())),
         o_vg_code = A.take(bytes_i(vg_code.size())), o_vd_ptr = A.take(bytes_i(vd_ptr.size())),
         o_vd_other = A.take(bytes_i(vd_other.size())), o_vd_len = A.take(bytes_d(vd_len.size())),
         o_vd_dist = A.take(bytes_d(vd_dist.size()));
  size_t o_lslot = A.take(bytes_i(n_flux)), o_rslot = A.take(bytes_i(n_flux)),
         o_lcell = A.take(bytes_i(n_flux)), o_rcell = A.take(bytes_i(n_flux)),
         o_normal = A.take(bytes_d(2 * n_flux)), o_flen = A.take(bytes_d(n_flux)), o_wallv = A.take(bytes_d(2 * NW)),
         o_vin = A.take(bytes_d(4 * NV)), o_pout = A.take(bytes_d(NO)), o_far = A.take(bytes_d(4 * NF));
  size_t o_gi_ptr = A.take(bytes_i(C + 1)), o_gi_flux = A.take(bytes_i(gi_flux.size())),
         o_gi_coef = A.take(bytes_d(gi_coef.size()));
  size_t o_gb_ptr = A.take(bytes_i(C + 1)), o_gb_flux = A.take(bytes_i(gb_flux.size())),
         o_gb_len = A.take(bytes_d(gb_len.size()));
  size_t o_dt_ptr = A.take(bytes_i(C + 1)), o_dt_n = A.take(bytes_d(dt_n.size())),
         o_dt_len = A.take(bytes_d(dt_len.size())), o_dt_info = A.take(bytes_i(dt_info.size()));
  size_t o_status = A.take(sizeof(DevStatus)), o_status_next = A.take(sizeof(DevStatus));
  size_t o_P = A.take(bytes_d(4 * C)), o_recon = A.take(bytes_d(4 * NL)),
         o_flux = A.take(bytes_d(4 * n_flux));
  size_t o_stage[4];
  for (int k = 0; k < 4; ++k) o_stage[k] = A.take(bytes_d(4 * C));
  size_t o_saved = A.take(bytes_d(4 * C));
  size_t o_partials = A.take(bytes_d(4 * partial_blocks));
  size_t o_bc_ext = A.take(bytes_d(4 * NB)), o_bc_ext_dt = A.take(bytes_d(4 * NB)), o_bc_terms = A.take(bytes_d(NB));

  mcfd_geom* h = new mcfd_geom();
  cudaError_t err = cudaMalloc(&h->arena, A.size);
  if (err != cudaSuccess) {
    delete h;
    return MCFD_E_CUDA;
  }
  h->arena_bytes = A.size;
  char* base = static_cast<char*>(h->arena);
  std::vector<char> host(A.size, 0);
  auto put = [&](size_t off, const void* src, size_t bytes) {
    if (bytes) std::memcpy(host.data() + off, src, bytes);
  };
  put(o_area, d->areas, bytes_d(C));
  put(o_cell_order, cell_order.data(), bytes_i(C));
  put(o_grad_ptr, grad_ptr.data(), bytes_i(C + 1));
  put(o_grad_nb, grad_nb.data(), bytes_i(NG));
  put(o_grad_cx, grad_cx.data(), bytes_d(NG));
  put(o_grad_cy, grad_cy.data(), bytes_d(NG));
  put(o_grad_twin, grad_twin.data(), bytes_i(NG));
  put(o_lim_ptr, lim_ptr.data(), bytes_i(C + 1));
  put(o_lim_slot, lim_slot.data(), bytes_i(NL));
  put(o_lim_d, lim_d.data(), bytes_d(2 * NL));
  put(o_par_ptr, par_ptr.data(), bytes_i(C + 1));
  put(o_par_nb, par_nb.data(), bytes_i(NE));
  put(o_par_d, par_d.data(), bytes_d(2 * NE));
  put(o_bc_ptr, bc_ptr.data(), bytes_i(NBP + 1));
  put(o_bc_kind, bc_kind.data(), bytes_i(NBP));
  put(o_bc_values, bc_values.data(), bytes_d(4 * NBP));
  put(o_bc_dn, bc_dn.data(), bytes_d(NB));
  put(o_grad_d, grad_d.data(), bytes_d(grad_d.size()));
  put(o_vb_ptr, vb_ptr.data(), bytes_i(vb_ptr.size()));
  put(o_vb_j, vb_j.data(), bytes_i(ND));
  put(o_diff_owner, diff_owner.data(), bytes_i(ND));
  put(o_diff_normal, diff_normal.data(), bytes_d(2 * ND));
  put(o_diff_len, diff_len.data(), bytes_d(ND));
  put(o_diff_kind, diff_kind.data(), bytes_i(ND));
  put(o_diff_thermal, diff_thermal.data(), bytes_i(ND));
  put(o_diff_value, diff_value.data(), bytes_d(ND));
  put(o_diff_inlet, diff_inlet.data(), bytes_i(ND));
  put(o_diff_nd, diff_nd.data(), bytes_d(ND));
  put(o_diff_ghost, diff_ghost.data(), bytes_d(2 * ND));
  put(o_diff_offset, diff_offset.data(), bytes_d(2 * ND));
  put(o_diff_wallv, diff_wallv.data(), bytes_d(2 * ND));
  put(o_vg_ptr, vg_ptr.data(), bytes_i(vg_ptr.size()));
  put(o_vg_code, vg_code.data(), bytes_i(vg_code.size()));
  put(o_vd_ptr, vd_ptr.data(), bytes_i(vd_ptr.size()));
  put(o_vd_other, vd_other.data(), bytes_i(vd_other.size()));
  put(o_vd_len, vd_len.data(), bytes_d(vd_len.size()));
  put(o_vd_dist, vd_dist.data(), bytes_d(vd_dist.size()));
  put(o_lslot, lslot.data(), bytes_i(n_flux));
  put(o_rslot, rslot.data(), bytes_i(n_flux));
  put(o_lcell, lcell.data(), bytes_i(n_flux));
  put(o_rcell, rcell.data(), bytes_i(n_flux));
  put(o_normal, normal.data(), bytes_d(2 * n_flux));
  put(o_flen, flen.data(), bytes_d(n_flux));
  put(o_wallv, wallv.data(), bytes_d(2 * NW));
  put(o_vin, vin.data(), bytes_d(4 * NV));
  put(o_pout, pout.data(), bytes_d(NO));
  put(o_far, far.data(), bytes_d(4 * NF));
  put(o_gi_ptr, gi_ptr.data(), bytes_i(C + 1));
  put(o_gi_flux, gi_flux.data(), bytes_i(gi_flux.size()));
  put(o_gi_coef, gi_coef.data(), bytes_d(gi_coef.size()));
  put(o_gb_ptr, gb_ptr.data(), bytes_i(C + 1));
  put(o_gb_flux, gb_flux.data(), bytes_i(gb_flux.size()));
  put(o_gb_len, gb_len.data(), bytes_d(gb_len.size()));
  put(o_dt_ptr, dt_ptr.data(), bytes_i(C + 1));
  put(o_dt_n, dt_n.data(), bytes_d(dt_n.size()));
  put(o_dt_len, dt_len.data(), bytes_d(dt_len.size()));
  put(o_dt_info, dt_info.data(), bytes_i(dt_info.size()));
  DevStatus st0{0, std::numeric_limits<int>::max(), std::numeric_limits<int>::max(), std::numeric_limits<int>::max(),
                0x7ff0000000000000ULL};
  put(o_status, &st0, sizeof(st0));
  put(o_status_next, &st0, sizeof(st0));
  // geometry part only (workspace stays uninitialised)
  err = cudaMemcpy(base, host.data(), o_P, cudaMemcpyHostToDevice);
  if (err == cudaSuccess) err = cudaMallocHost(&h->host_status, sizeof(DevStatus));
  if (err == cudaSuccess) err = cudaStreamCreateWithFlags(&h->side.stream, cudaStreamNonBlocking);
  if (err == cudaSuccess) err = cudaEventCreateWithFlags(&h->side.fork, cudaEventDisableTiming);
  if (err == cudaSuccess) err = cudaEventCreateWithFlags(&h->side.join, cudaEventDisableTiming);
  if (err != cudaSuccess) {
    if (h->side.stream) cudaStreamDestroy(h->side.stream);
    if (h->side.fork) cudaEventDestroy(h->side.fork);
    if (h->host_status) cudaFreeHost(h->host_status);
    cudaFree(h->arena);
    delete h;
    return MCFD_E_CUDA;
  }
  DevGeom& g = h->g;
  g.n_cells = (int)C;
  g.n_faces = (int)F;
  g.n_flux = (int)n_flux;
  g.n_slots = (int)NL;
  g.n_gradient = (int)NG;
  for (int k = 0; k <= SEG_COUNT; ++k) g.seg_begin[k] = seg_begin[k];
#define AT(T, off) reinterpret_cast<T>(base + (off))
  g.area = AT(const double*, o_area);
  g.cell_order = AT(const int*, o_cell_order);
  g.n_lim34 = n_lim34;
  g.grad_ptr = AT(const int*, o_grad_ptr);
  g.grad_nb = AT(const int*, o_grad_nb);
  g.grad_cx = AT(const double*, o_grad_cx);
  g.grad_cy = AT(const double*, o_grad_cy);
  g.grad_twin = AT(const int*, o_grad_twin);
  g.has_twins = twins_ok ? 1 : 0;
  g.lim_ptr = AT(const int*, o_lim_ptr);
  g.lim_slot = AT(const int*, o_lim_slot);
  g.lim_d = AT(const double2*, o_lim_d);
  g.n_parabolic = (int)NE;
  g.par_ptr = AT(const int*, o_par_ptr);
  g.par_nb = AT(const int*, o_par_nb);
  g.par_d = AT(const double2*, o_par_d);
  g.n_bc_patches = (int)NBP;
  g.bc_ptr = AT(const int*, o_bc_ptr);
  g.bc_kind = AT(const int*, o_bc_kind);
  g.bc_values = AT(const double*, o_bc_values);
  g.bc_dn = AT(const double*, o_bc_dn);
  g.bc_ext = AT(double*, o_bc_ext);
  g.bc_ext_dt = AT(double*, o_bc_ext_dt);
  g.bc_terms = AT(double*, o_bc_terms);
  g.has_viscous = has_viscous ? 1 : 0;
  g.viscous_ok = viscous_ok ? 1 : 0;
  g.n_diffusive = (int)ND;
  g.grad_d = AT(const double2*, o_grad_d);
  g.vb_ptr = AT(const int*, o_vb_ptr);
  g.vb_j = AT(const int*, o_vb_j);
  g.diff_owner = AT(const int*, o_diff_owner);
  g.diff_normal = AT(const double2*, o_diff_normal);
  g.diff_len = AT(const double*, o_diff_len);
  g.diff_kind = AT(const int*, o_diff_kind);
  g.diff_thermal = AT(const int*, o_diff_thermal);
  g.diff_value = AT(const double*, o_diff_value);
  g.diff_inlet = AT(const int*, o_diff_inlet);
  g.diff_nd = AT(const double*, o_diff_nd);
  g.diff_ghost = AT(const double2*, o_diff_ghost);
  g.diff_offset = AT(const double2*, o_diff_offset);
  g.diff_wallv = AT(const double2*, o_diff_wallv);
  g.vg_ptr = AT(const int*, o_vg_ptr);
  g.vg_code = AT(const int*, o_vg_code);
  g.vd_ptr = AT(const int*, o_vd_ptr);
  g.vd_other = AT(const int*, o_vd_other);
  g.vd_len = AT(const double*, o_vd_len);
  g.vd_dist = AT(const double*, o_vd_dist);
  g.ff_lslot = AT(const int*, o_lslot);
  g.ff_rslot = AT(const int*, o_rslot);
  g.ff_lcell = AT(const int*, o_lcell);
  g.ff_rcell = AT(const int*, o_rcell);
  g.ff_normal = AT(const double2*, o_normal);
  g.ff_len = AT(const double*, o_flen);
  g.ff_wall_velocity = AT(const double2*, o_wallv);
  g.ff_vin_state = AT(const double*, o_vin);
  g.ff_pout_pressure = AT(const double*, o_pout);
  g.ff_far_state = AT(const double*, o_far);
  g.gi_ptr = AT(const int*, o_gi_ptr);
  g.gi_flux = AT(const int*, o_gi_flux);
  g.gi_coef = AT(const double*, o_gi_coef);
  g.gb_ptr = AT(const int*, o_gb_ptr);
  g.gb_flux = AT(const int*, o_gb_flux);
  g.gb_len = AT(const double*, o_gb_len);
  g.dt_ptr = AT(const int*, o_dt_ptr);
  g.dt_normal = AT(const double2*, o_dt_n);
  g.dt_len = AT(const double*, o_dt_len);
  g.dt_info = AT(const int*, o_dt_info);
  g.status = AT(DevStatus*, o_status);
  h->status = g.status;
  h->status_next = AT(DevStatus*, o_status_next);
  Workspace& w = h->ws;
  w.P = AT(double*, o_P);
  w.recon = AT(double*, o_recon);
  w.flux = AT(double*, o_flux);
  for (int k = 0; k < 4; ++k) w.stage[k] = AT(double*, o_stage[k]);
  w.saved_r = AT(double*, o_saved);
  w.partials = AT(double*, o_partials);
  w.partial_blocks = partial_blocks;
#undef AT
  mcfd_geom_info& info = h->info;
  info.n_cells = C;
  info.n_faces = F;
  info.n_interior = NI;
  info.n_periodic = NP;
  info.n_boundary_flux = NW + NV + NO + NF + NB;
  info.n_flux_faces = n_flux;
  info.n_gradient = NG;
  info.n_limiter = NL;
  info.device_bytes = (int64_t)A.size;
  // topology of the implicit preconditioner (solver.py:1185-1300)
  {
    ImplicitTopology& t = h->topo;
    t.n_cells = (int)C;
    t.n_interior = (int)NI;
    for (int64_t i = 0; i < NI; ++i) {
      int64_t f = d->interior_faces[i];
      double2 n = make_double2(d->face_normals[2 * f], d->face_normals[2 * f + 1]);
      t.coupling_a.push_back((int)d->owners[f]);
      t.coupling_b.push_back((int)d->neighbours[f]);
      t.coupling_na.push_back(n);
      t.coupling_nb.push_back(n);
      t.coupling_len.push_back(d->face_lengths[f]);
    }
    for (int64_t i = 0; i < NP; ++i) {
      int64_t fa = d->periodic_faces_a[i], fb = d->periodic_faces_b[i];
      t.coupling_a.push_back((int)d->owners[fa]);
      t.coupling_b.push_back((int)d->owners[fb]);
      t.coupling_na.push_back(make_double2(d->face_normals[2 * fa], d->face_normals[2 * fa + 1]));
      t.coupling_nb.push_back(make_double2(d->face_normals[2 * fb], d->face_normals[2 * fb + 1]));
      t.coupling_len.push_back(d->face_lengths[fa]);
    }
    for (int64_t f = 0; f < F; ++f) {
      if (d->neighbours[f] >= 0) continue;
      t.boundary_owner.push_back((int)d->owners[f]);
      t.boundary_normal.push_back(make_double2(d->face_normals[2 * f], d->face_normals[2 * f + 1]));
      t.boundary_len.push_back(d->face_lengths[f]);
    }
  }
  *out = h;
  return MCFD_OK;
}

int mcfd_geom_destroy(mcfd_geom* h) {
  if (!h) return MCFD_OK;
  for (ProfRecord& r : h->records) {
    cudaEventDestroy(r.start);
    cudaEventDestroy(r.stop);
  }
  for (cudaEvent_t e : h->event_pool) cudaEventDestroy(e);
  if (h->imp_built) implicit_free(h->imp);
  for (void* p : h->jvp_owned) cudaFree(p);
  if (h->side.stream) cudaStreamDestroy(h->side.stream);
  if (h->side.fork) cudaEventDestroy(h->side.fork);
  if (h->side.join) cudaEventDestroy(h->side.join);
  if (h->vjp.side) cudaStreamDestroy(h->vjp.side);
  if (h->vjp.fork) cudaEventDestroy(h->vjp.fork);
  if (h->vjp.join) cudaEventDestroy(h->vjp.join);
  cudaError_t e1 = cudaFree(h->arena);
  cudaError_t e2 = cudaFreeHost(h->host_status);
  delete h;
  return (e1 == cudaSuccess && e2 == cudaSuccess) ? MCFD_OK : MCFD_E_CUDA;
}

int mcfd_geom_get_info(const mcfd_geom* h, mcfd_geom_info* info) {
  if (!h || !info) return MCFD_E_ARG;
  *info = h->info;
  return MCFD_OK;
}

const double* mcfd_geom_primitive(const mcfd_geom* h) { return h ? h->ws.P : nullptr; }

int mcfd_reconstruction(mcfd_geom* h, const mcfd_config* cfg, const double* P, double* gradients,
                        double* curvature, double* factors, void* stream) {
  if (!h || !P || !gradients || !factors) return MCFD_E_ARG;
  int c = check_cfg(cfg);
  if (c) return c;
  if (cfg->reconstruction == MCFD_RECON_FIRST_ORDER) return MCFD_E_ARG;
  if (cfg->limiter == MCFD_LIMITER_VENKATAKRISHNAN_K) return MCFD_E_UNSUPPORTED;  // the reference's fields only
  cudaStream_t s = (cudaStream_t)stream;
  return rc(timed(h, MCFD_PROF_RECONSTRUCT, s,
                  [&] { return launch_reconstruction_fields(h->g, *cfg, P, gradients, curvature, factors, s); }));
}

int mcfd_explicit_step_record(mcfd_geom* h, const mcfd_config* cfg, int32_t scheme, double* U, const double* dt,
                              int32_t dt_per_cell, double* const* stage_P, double* const* stage_recon,
                              int32_t n_stages, void* stream) {
  static const int kStages[4] = {1, 2, 3, 5};
  if (!h || !stage_P || scheme < MCFD_TIME_EULER || scheme > MCFD_TIME_RK4 || n_stages < kStages[scheme])
    return MCFD_E_ARG;
  for (int k = 0; k < kStages[scheme]; ++k)
    if (!stage_P[k]) return MCFD_E_ARG;
  h->rec_P = stage_P;
  h->rec_recon = stage_recon;
  h->rec_n = n_stages;
  h->rec_k = 0;
  const int r = mcfd_explicit_step(h, cfg, scheme, U, dt, dt_per_cell, stream);
  h->rec_P = nullptr;
  h->rec_recon = nullptr;
  h->rec_n = h->rec_k = 0;
  return r;
}

int mcfd_autotune(mcfd_geom* h, const mcfd_config* cfg, const double* U, int32_t* chosen, void* stream) {
  if (!h || !U || !chosen) return MCFD_E_ARG;
  int c = check_cfg(cfg);
  if (c) return c;
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e = MCFD_DISPATCH(*cfg, launch_primitive(h->g, *cfg, U, h->ws.P, s));
  if (e != cudaSuccess) return MCFD_E_CUDA;
  cudaEvent_t a = take_event(h), b = take_event(h);
  // mean time of 3 launches after one warm-up
  auto time_ms = [&](auto&& launch) -> float {
    launch();
    cudaEventRecord(a, s);
    for (int r = 0; r < 3; ++r) launch();
    cudaEventRecord(b, s);
    cudaEventSynchronize(b);
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, a, b);
    return ms / 3.0f;
  };
  static const int kThreads[3] = {64, 128, 256};
  static const int kFaces[3] = {1, 2, 4};
  DevGeom& g = h->g;
  const bool muscl = cfg->reconstruction == MCFD_RECON_MUSCL_LINEAR;
  auto recon = [&] {
    if (cfg->reconstruction == MCFD_RECON_MUSCL_PARABOLIC)
      launch_reconstruct_parabolic(g, *cfg, h->ws.P, h->ws.recon, s);
    else if (muscl)
      MCFD_DISPATCH(*cfg, launch_reconstruct(g, *cfg, h->ws.P, h->ws.recon, s));
  };
  int best_recon = 0, best_flux_t = 0, best_flux_f = 1, best_gather = 0, best_split = 0;
  if (muscl) {
    // the fast variant's reconstruction also has a kernel with one thread per
    // (cell, variable); both give the same bits
    const int splits = cfg->mode == MCFD_MODE_FAST && cfg->limiter != MCFD_LIMITER_VENKATAKRISHNAN_K ? 2 : 1;
    float best = 1e30f;
    for (int sp = 0; sp < splits; ++sp)
      for (int t : kThreads) {
        g.tune_recon_threads = t;
        g.tune_recon_split = sp;
        const float ms = time_ms(recon);
        if (ms < best) best = ms, best_recon = t, best_split = sp;
      }
    g.tune_recon_threads = best_recon;
    g.tune_recon_split = best_split;
  }
  recon();
  {
    float best = 1e30f;
    for (int t : kThreads)
      for (int f : kFaces) {
        g.tune_flux_threads = t;
        g.tune_flux_faces = f;
        const float ms = time_ms([&] { MCFD_DISPATCH(*cfg, launch_flux(g, *cfg, h->ws.P, h->ws.recon, h->ws.flux, s, nullptr)); });
        if (ms < best) best = ms, best_flux_t = t, best_flux_f = f;
      }
    g.tune_flux_threads = best_flux_t;
    g.tune_flux_faces = best_flux_f;
  }
  {
    StageProgram prog{};
    prog.out_r = h->ws.saved_r;
    float best = 1e30f;
    for (int t : kThreads) {
      g.tune_gather_threads = t;
      const float ms = time_ms([&] { MCFD_DISPATCH(*cfg, launch_gather(g, *cfg, h->ws.P, h->ws.flux, prog, s)); });
      if (ms < best) best = ms, best_gather = t;
    }
    g.tune_gather_threads = best_gather;
  }
  h->event_pool.push_back(a);
  h->event_pool.push_back(b);
  chosen[0] = best_recon;
  chosen[1] = best_flux_t;
  chosen[2] = best_flux_f;
  chosen[3] = best_gather;
  chosen[4] = best_split;
  return rc(cudaGetLastError());
}

int mcfd_set_launch_shapes(mcfd_geom* h, const int32_t* shapes) {
  if (!h || !shapes) return MCFD_E_ARG;
  static const int allowed[] = {0, 32, 64, 96, 128, 192, 256};
  auto ok_threads = [&](int t) {
    for (int a : allowed)
      if (t == a) return true;
    return false;
  };
  if (!ok_threads(shapes[0]) || !ok_threads(shapes[1]) || !ok_threads(shapes[3]) || shapes[2] < 0 ||
      shapes[2] > 64 || shapes[4] < 0 || shapes[4] > 1)
    return MCFD_E_ARG;
  h->g.tune_recon_threads = shapes[0];
  h->g.tune_flux_threads = shapes[1];
  h->g.tune_flux_faces = shapes[2];
  h->g.tune_gather_threads = shapes[3];
  h->g.tune_recon_split = shapes[4];
  return MCFD_OK;
}

int mcfd_set_fused_stage(mcfd_geom* h, int32_t on) {
  if (!h || on < 0 || on > 1) return MCFD_E_ARG;
  h->fused_stage = on != 0;
  return MCFD_OK;
}

int mcfd_fused_stage_blocks(const mcfd_geom* h) { return h ? h->fused_blocks : 0; }

const double* mcfd_geom_stage_state(const mcfd_geom* h, int32_t k) {
  return (h && k >= 0 && k < 4) ? h->ws.stage[k] : nullptr;
}



int mcfd_primitive(mcfd_geom* h, const mcfd_config* cfg, const double* U, double* P, void* stream) {
  if (!h || !U || !P) return MCFD_E_ARG;
  int c = check_cfg(cfg);
  if (c) return c;
  cudaStream_t s = (cudaStream_t)stream;
  return rc(timed(h, MCFD_PROF_PRIMITIVE, s, [&] { return MCFD_DISPATCH(*cfg, launch_primitive(h->g, *cfg, U, P, s)); }));
}


int mcfd_residual(mcfd_geom* h, const mcfd_config* cfg, const double* U, double* R, void* stream) {
  if (!h || !U) return MCFD_E_ARG;
  int c = check_cfg(cfg);
  if (c) return c;
  if ((c = ensure_viscous(h, cfg))) return c;
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e = timed(h, MCFD_PROF_PRIMITIVE, s, [&] { return MCFD_DISPATCH(*cfg, launch_primitive(h->g, *cfg, U, h->ws.P, s)); });
  StageProgram prog{};
  prog.out_r = R;
  if (e == cudaSuccess) e = stage(h, *cfg, prog, s);
  return rc(e);
}

// The stable time steps of P with their status bits and minimum in *st.
static int time_steps_into(mcfd_geom* h, DevStatus* st, const mcfd_config* cfg, const double* P, double* dt_cells,
                           double* dt_min, double time_limit, cudaStream_t s) {
  DevGeom g = h->g;
  g.status = st;
  return rc(timed(h, MCFD_PROF_TIME_STEP, s,
                  [&] {
                    cudaError_t r = cudaSuccess;
                    if (g.n_bc_patches > 0) r = launch_bc_states(g, *cfg, P, nullptr, g.bc_ext_dt, s);
                    if (r == cudaSuccess && cfg->viscosity_model != MCFD_VISC_INVISCID)
                      r = launch_viscous_diffusion(g, *cfg, P, h->visc, s);
                    if (r == cudaSuccess)
                      r = MCFD_DISPATCH(*cfg, launch_time_steps(g, *cfg, P, dt_cells, dt_min, time_limit, s));
                    return r;
                  }));
}

int mcfd_time_steps(mcfd_geom* h, const mcfd_config* cfg, const double* P, double* dt_cells,
                    double* dt_min, double time_limit, void* stream) {
  if (!h || !P) return MCFD_E_ARG;
  int c = check_cfg(cfg);
  if (c) return c;
  if ((c = ensure_viscous(h, cfg))) return c;
  if (!(cfg->cfl > 0.0)) return MCFD_E_ARG;
  return time_steps_into(h, h->status, cfg, P, dt_cells, dt_min, time_limit, (cudaStream_t)stream);
}


// One explicit step (solver.py:532-806, 1128-1182).  primitive_current: the
// handle's primitive buffer already holds the primitive of U (as the final
// stage of the previous step left it), so the step starts without
// recomputing it.  next: the last stage also writes the stable time steps of
// the new state (NextDt), where the settings allow; the caller completes
// them otherwise.  start_residual (may be null): the first stage also stores
// the residual of U it computes (the reference's `derivative`,
// solver.py:466-468, which its progress report uses).
struct NextDt {
  double* cells = nullptr;
  int min = 0;
  double cfl = 0.0;
  DevStatus* status = nullptr;
};

static cudaError_t explicit_step_impl(mcfd_geom* h, const mcfd_config* cfg, int32_t scheme, double* U,
                                      const double* dt, int32_t dt_per_cell, bool primitive_current,
                                      const NextDt& next, double* start_residual, cudaStream_t s) {
  Workspace& w = h->ws;
  cudaError_t e = cudaSuccess;
  if (!primitive_current)
    e = timed(h, MCFD_PROF_PRIMITIVE, s, [&] { return MCFD_DISPATCH(*cfg, launch_primitive(h->g, *cfg, U, w.P, s)); });
  auto run = [&](std::initializer_list<StageTerm> terms, double* out, double* save_r) {
    if (e != cudaSuccess) return;
    StageProgram p{};
    p.n_terms = 0;
    for (const StageTerm& t : terms) p.t[p.n_terms++] = t;
    p.dt = dt;
    p.dt_per_cell = dt_per_cell;
    p.out_u = out;
    p.out_p = w.P;
    p.out_r = save_r;
    if (out == U) {  // the last stage
      p.next_dt_cells = next.cells;
      p.next_dt_min = next.min;
      p.cfl = next.cfl;
      p.next_dt_status = next.status;
    }
    e = stage(h, *cfg, p, s);
  };
  double *X1 = w.stage[0], *X2 = w.stage[1], *X3 = w.stage[2], *X4 = w.stage[3];
  switch (scheme) {
    case MCFD_TIME_EULER:  // solver.py:532-533
      run({term(TERM_X, 1.0, U), term(TERM_DTR, 1.0, nullptr)}, U, start_residual);
      break;
    case MCFD_TIME_RK2:  // solver.py:566-627
      run({term(TERM_X, 1.0, U), term(TERM_DTR, 1.0, nullptr)}, X1, start_residual);
      run({term(TERM_X, 0.5, U), term(TERM_X_PLUS_DTR, 0.5, X1)}, U, nullptr);
      break;
    case MCFD_TIME_RK3:  // solver.py:566-567, 676-678, 754-756
      run({term(TERM_X, 1.0, U), term(TERM_DTR, 1.0, nullptr)}, X1, start_residual);
      run({term(TERM_X, 0.75, U), term(TERM_X_PLUS_DTR, 0.25, X1)}, X2, nullptr);
      run({term(TERM_X, 1.0 / 3.0, U), term(TERM_X_PLUS_DTR, 2.0 / 3.0, X2)}, U, nullptr);
      break;
    default:  // SSPRK(5,4), solver.py:1128-1182
      run({term(TERM_X, 1.0, U), term(TERM_DTR, 0.391752226571890, nullptr)}, X1, start_residual);
      run({term(TERM_X, 0.444370493651235, U), term(TERM_X, 0.555629506348765, X1),
           term(TERM_DTR, 0.368410593050371, nullptr)}, X2, nullptr);
      run({term(TERM_X, 0.620101851488403, U), term(TERM_X, 0.379898148511597, X2),
           term(TERM_DTR, 0.251891774271694, nullptr)}, X3, nullptr);
      run({term(TERM_X, 0.178079954393132, U), term(TERM_X, 0.821920045606868, X3),
           term(TERM_DTR, 0.544974750228521, nullptr)}, X4, w.saved_r);
      run({term(TERM_X, 0.517231671970585, X2), term(TERM_X, 0.096059710526147, X3),
           term(TERM_DTR_SAVED, 0.063692468666290, w.saved_r), term(TERM_X, 0.386708617503269, X4),
           term(TERM_DTR, 0.226007483236906, nullptr)}, U, nullptr);
      break;
  }
  return e;
}

int mcfd_explicit_step(mcfd_geom* h, const mcfd_config* cfg, int32_t scheme, double* U,
                       const double* dt, int32_t dt_per_cell, void* stream) {
  if (!h || !U || !dt) return MCFD_E_ARG;
  int c = check_cfg(cfg);
  if (c) return c;
  if ((c = ensure_viscous(h, cfg))) return c;
  if (scheme < MCFD_TIME_EULER || scheme > MCFD_TIME_RK4) return MCFD_E_ARG;
  return rc(explicit_step_impl(h, cfg, scheme, U, dt, dt_per_cell, false, NextDt{}, nullptr, (cudaStream_t)stream));
}

int mcfd_explicit_step_next(mcfd_geom* h, const mcfd_config* cfg, int32_t scheme, double* U, const double* dt,
                            int32_t dt_per_cell, int32_t primitive_current, double* next_dt_cells,
                            double* next_dt_min, double time_limit, double* start_residual, void* stream) {
  if (!h || !U || !dt) return MCFD_E_ARG;
  // the stages read dt and U to the end
  if ((next_dt_cells && (next_dt_cells == dt || next_dt_cells == U)) ||
      (next_dt_min && (next_dt_min == dt || next_dt_min == U)) ||
      (start_residual && (start_residual == U || start_residual == dt)))
    return MCFD_E_ARG;
  int c = check_cfg(cfg);
  if (c) return c;
  if ((c = ensure_viscous(h, cfg))) return c;
  if (scheme < MCFD_TIME_EULER || scheme > MCFD_TIME_RK4) return MCFD_E_ARG;
  if ((next_dt_cells || next_dt_min) && !(cfg->cfl > 0.0)) return MCFD_E_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  // the last stage computes the time steps where they depend on the cell
  // state alone (inviscid, no pressure-inlet / mass-flow patches, whose
  // exterior states come from a pass of their own)
  const bool want = next_dt_cells || next_dt_min;
  const bool fused = cfg->viscosity_model == MCFD_VISC_INVISCID && h->g.n_bc_patches == 0;
  NextDt next;
  if (want && fused) {
    next.cells = next_dt_cells;
    next.min = next_dt_min != nullptr;
    next.cfl = cfg->cfl;
    next.status = h->status_next;
  }
  cudaError_t e =
      explicit_step_impl(h, cfg, scheme, U, dt, dt_per_cell, primitive_current != 0, next, start_residual, s);
  if (e != cudaSuccess) return MCFD_E_CUDA;
  if (!want) return MCFD_OK;
  if (!fused) return time_steps_into(h, h->status_next, cfg, h->ws.P, next_dt_cells, next_dt_min, time_limit, s);
  if (next_dt_min)
    e = timed(h, MCFD_PROF_TIME_STEP, s, [&] {
      count_launch();
      return finalize_time_step(h->status_next, next_dt_min, time_limit, s);
    });
  return rc(e);
}

int mcfd_residual_sumsq(mcfd_geom* h, const double* R, double* sums, void* stream) {
  if (!h || !R || !sums) return MCFD_E_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  return rc(timed(h, MCFD_PROF_OTHER, s,
                  [&] { return launch_sumsq(h->g, R, h->ws.partials, h->ws.partial_blocks, sums, s); }));
}

// Reads and clears one status word (keeping its time-step minimum).
static int fetch_status(mcfd_geom* h, DevStatus* dev, void* stream, mcfd_status* out) {
  if (!h || !out) return MCFD_E_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e = cudaMemcpyAsync(h->host_status, dev, sizeof(DevStatus), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return MCFD_E_CUDA;
  DevStatus st = *h->host_status;
  out->code = st.code;
  out->first_cell = st.first_cell == std::numeric_limits<int>::max() ? -1 : st.first_cell;
  out->first_face = st.first_face == std::numeric_limits<int>::max() ? -1 : st.first_face;
  out->first_patch = st.first_patch == std::numeric_limits<int>::max() ? -1 : st.first_patch;
  if (st.code) {
    DevStatus clear{0, std::numeric_limits<int>::max(), std::numeric_limits<int>::max(),
                    std::numeric_limits<int>::max(), st.dt_min_bits};
    *h->host_status = clear;
    e = cudaMemcpyAsync(dev, h->host_status, sizeof(DevStatus), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return MCFD_E_CUDA;
  }
  return MCFD_OK;
}

int mcfd_status_fetch(mcfd_geom* h, void* stream, mcfd_status* out) {
  return fetch_status(h, h ? h->status : nullptr, stream, out);
}

int mcfd_status_fetch_next(mcfd_geom* h, void* stream, mcfd_status* out) {
  return fetch_status(h, h ? h->status_next : nullptr, stream, out);
}


// ------------------------------------------------------------- implicit Euler

static int ensure_implicit(mcfd_geom* h) {
  if (h->imp_built) return MCFD_OK;
  if (implicit_build(h->imp, h->topo) != cudaSuccess) {
    implicit_free(h->imp);
    return MCFD_E_CUDA;
  }
  h->imp.status = h->status;
  h->imp_built = true;
  return MCFD_OK;
}

static ScaleVec scale_of(const double* scales) {
  ScaleVec v;
  for (int k = 0; k < 4; ++k) v.v[k] = scales[k];
  return v;
}

// first-order residual of the prepared operator
static cudaError_t residual_first_order(mcfd_geom* h, const double* U, double* R, cudaStream_t s) {
  const mcfd_config& c = h->imp_cfg;
  cudaError_t e = timed(h, MCFD_PROF_PRIMITIVE, s, [&] { return MCFD_DISPATCH(c, launch_primitive(h->g, c, U, h->ws.P, s)); });
  StageProgram prog{};
  prog.out_r = R;
  if (e == cudaSuccess) e = stage(h, c, prog, s);
  return e;
}

int mcfd_implicit_prepare(mcfd_geom* h, const mcfd_config* cfg, const double* U, const double* dt,
                          int32_t dt_per_cell, const double* scales, void* stream) {
  if (!h || !U || !dt || !scales) return MCFD_E_ARG;
  int c = check_cfg(cfg);
  if (c) return c;
  if ((c = ensure_viscous(h, cfg))) return c;
  if ((c = ensure_implicit(h))) return c;
  cudaStream_t s = (cudaStream_t)stream;
  ImplicitState& st = h->imp;
  mcfd_config first = *cfg;
  first.reconstruction = MCFD_RECON_FIRST_ORDER;  // replace(settings, reconstruction="First order")
  // the captured GMRES step holds this configuration's kernels: rebuild it
  // when the configuration or the time-step layout changes
  if (std::memcmp(&first, &h->imp_cfg, sizeof(first)) != 0 || st.dt_per_cell != (dt_per_cell != 0))
    st.inner_key = -1;
  h->imp_cfg = first;
  cudaError_t e = implicit_set_operator(st, scale_of(scales), dt, dt_per_cell != 0, s);
  const size_t bytes = 4 * (size_t)h->g.n_cells * sizeof(double);
  if (e == cudaSuccess) e = cudaMemcpyAsync(st.state, U, bytes, cudaMemcpyDeviceToDevice, s);
  // preconditioner from the state's primitive variables
  if (e == cudaSuccess)
    e = timed(h, MCFD_PROF_PRIMITIVE, s, [&] { return MCFD_DISPATCH(*cfg, launch_primitive(h->g, *cfg, U, h->ws.P, s)); });
  if (e == cudaSuccess)
    e = timed(h, MCFD_PROF_OTHER, s, [&] { return implicit_assemble(st, h->ws.P, h->g.area, st.dt, st.dt_per_cell, cfg->gamma, s); });
  // jacobian_rate = R1(state)
  if (e == cudaSuccess) e = residual_first_order(h, U, st.rate, s);
  // |state / scale|^2, read by the operator on the device
  if (e == cudaSuccess) e = implicit_scaled_sumsq(st, U, st.scale, st.scalars + 8, s);
  st.prepared = e == cudaSuccess;
  return rc(e);
}

static int ensure_jvp(mcfd_geom* h) {
  if (h->jvp.P) return MCFD_OK;
  const size_t c4 = 4 * (size_t)h->g.n_cells * sizeof(double);
  const size_t s4 = 4 * (size_t)h->g.n_slots * sizeof(double);
  const size_t f4 = 4 * (size_t)std::max(h->g.n_flux, 1) * sizeof(double);
  double** fields[] = {&h->jvp.P, &h->jvp.dP, &h->jvp.recon, &h->jvp.drecon, &h->jvp.dflux, &h->jvp.sv, &h->jvp.dR};
  const size_t sizes[] = {c4, c4, s4, s4, f4, c4, c4};
  for (int k = 0; k < 7; ++k) {
    if (cudaMalloc((void**)fields[k], sizes[k]) != cudaSuccess) return MCFD_E_CUDA;
    h->jvp_owned.push_back(*fields[k]);
  }
  return MCFD_OK;
}

static MatvecFn implicit_operator(mcfd_geom* h) {
  if (h->imp_exact_jacobian)
    return [h](const double* v, double* out, cudaStream_t ss) {
      return timed(h, MCFD_PROF_OTHER, ss, [&] { return exact_operator(h->g, h->imp_cfg, h->imp, h->jvp, v, out, ss); });
    };
  return [h](const double* v, double* out, cudaStream_t ss) {
    ResidualFn r1 = [h](const double* U, double* R, cudaStream_t s2) { return residual_first_order(h, U, R, s2); };
    return fd_operator(h->imp, r1, v, out, ss);
  };
}

int mcfd_implicit_matvec(mcfd_geom* h, const double* v, double* out, void* stream) {
  if (!h || !v || !out || !h->imp_built || !h->imp.prepared) return MCFD_E_ARG;
  return rc(implicit_operator(h)(v, out, (cudaStream_t)stream));
}

int mcfd_implicit_set_jacobian(mcfd_geom* h, int32_t exact) {
  if (!h) return MCFD_E_ARG;
  if (exact) {
    int c = ensure_jvp(h);
    if (c) return c;
  }
  h->imp_exact_jacobian = exact != 0;
  return MCFD_OK;
}

static int ensure_vjp(mcfd_geom* h) {
  if (h->vjp.P) return MCFD_OK;
  const size_t c4 = 4 * (size_t)h->g.n_cells * sizeof(double);
  const size_t s4 = 4 * (size_t)std::max(h->g.n_slots, 1) * sizeof(double);
  const size_t e4 = 4 * (size_t)std::max(h->g.n_gradient, 1) * sizeof(double);
  double** fields[] = {&h->vjp.P, &h->vjp.recon, &h->vjp.slot_bar, &h->vjp.pbar, &h->vjp.ent_bar, &h->vjp.partials};
  const size_t sizes[] = {c4, s4, s4, c4, e4, 616 * sizeof(double)};  // 608 block sums + the total
  for (int k = 0; k < 6; ++k) {
    if (cudaMalloc((void**)fields[k], sizes[k]) != cudaSuccess) return MCFD_E_CUDA;
    h->jvp_owned.push_back(*fields[k]);
  }
  if (cudaStreamCreateWithFlags(&h->vjp.side, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&h->vjp.fork, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&h->vjp.join, cudaEventDisableTiming) != cudaSuccess)
    return MCFD_E_CUDA;
  return MCFD_OK;
}

int mcfd_vjp(mcfd_geom* h, const mcfd_config* cfg, const double* U, const double* lambda, double* U_bar,
             double* far_bar, void* stream) {
  if (!h || !U || !lambda || !U_bar) return MCFD_E_ARG;
  int c = check_cfg(cfg);
  if (c) return c;
  if (cfg->reconstruction == MCFD_RECON_MUSCL_PARABOLIC || h->g.n_bc_patches > 0 ||
      cfg->viscosity_model != MCFD_VISC_INVISCID)
    return MCFD_E_UNSUPPORTED;
  if (cfg->reconstruction != MCFD_RECON_FIRST_ORDER && !h->g.has_twins) return MCFD_E_UNSUPPORTED;
  if ((c = ensure_vjp(h))) return c;
  cudaStream_t s = (cudaStream_t)stream;
  return rc(timed(h, MCFD_PROF_OTHER, s,
                  [&] { return launch_vjp(h->g, *cfg, U, nullptr, nullptr, lambda, h->vjp, U_bar, far_bar, s); }));
}

int mcfd_vjp_at(mcfd_geom* h, const mcfd_config* cfg, const double* U, const double* P, const double* recon,
                const double* lambda, double* U_bar, double* far_bar, void* stream) {
  if (!h || !P || !lambda || !U_bar) return MCFD_E_ARG;  // U is not needed once P is given
  int c = check_cfg(cfg);
  if (c) return c;
  if (cfg->reconstruction == MCFD_RECON_MUSCL_PARABOLIC || h->g.n_bc_patches > 0 ||
      cfg->viscosity_model != MCFD_VISC_INVISCID)
    return MCFD_E_UNSUPPORTED;
  if (cfg->reconstruction != MCFD_RECON_FIRST_ORDER && (!h->g.has_twins || !recon)) return MCFD_E_UNSUPPORTED;
  if ((c = ensure_vjp(h))) return c;
  cudaStream_t s = (cudaStream_t)stream;
  return rc(timed(h, MCFD_PROF_OTHER, s,
                  [&] { return launch_vjp(h->g, *cfg, U, P, recon, lambda, h->vjp, U_bar, far_bar, s); }));
}

int mcfd_wall_force(mcfd_geom* h, const mcfd_config* cfg, const double* U, double dir_x, double dir_y, double* J,
                    double* dJdU, void* stream) {
  if (!h || !U || !J) return MCFD_E_ARG;
  int c = check_cfg(cfg);
  if (c) return c;
  if ((c = ensure_vjp(h))) return c;
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e = launch_wall_force(h->g, *cfg, U, dir_x, dir_y, h->vjp, h->vjp.partials + 608, dJdU, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(J, h->vjp.partials + 608, sizeof(double), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  return rc(e);
}

int mcfd_jvp(mcfd_geom* h, const mcfd_config* cfg, const double* U, const double* dU, double* dR, void* stream) {
  if (!h || !U || !dU || !dR) return MCFD_E_ARG;
  int c = check_cfg(cfg);
  if (c) return c;
  if (cfg->reconstruction == MCFD_RECON_MUSCL_PARABOLIC || h->g.n_bc_patches > 0 ||
      cfg->viscosity_model != MCFD_VISC_INVISCID)
    return MCFD_E_UNSUPPORTED;
  if ((c = ensure_jvp(h))) return c;
  cudaStream_t s = (cudaStream_t)stream;
  return rc(timed(h, MCFD_PROF_OTHER, s, [&] { return launch_jvp(h->g, *cfg, U, dU, h->jvp, dR, s); }));
}

int mcfd_implicit_set_chunk(mcfd_geom* h, int32_t rows) {
  if (!h || rows < 0 || rows > 32) return MCFD_E_ARG;
  int c = ensure_implicit(h);
  if (c) return c;
  return rc(implicit_set_chunk(h->imp, rows));
}

int mcfd_lusgs_apply(mcfd_geom* h, const double* v, double* x, void* stream) {
  if (!h || !v || !x || !h->imp_built || !h->imp.prepared) return MCFD_E_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  return rc(timed(h, MCFD_PROF_OTHER, s, [&] { return lusgs_apply(h->imp, v, x, s); }));
}

int mcfd_implicit_set_sweep(mcfd_geom* h, int32_t wide_level, int32_t engine) {
  if (!h || wide_level < 0 || (engine < 0 || (engine > 9 && engine != 16)))
    return MCFD_E_ARG;
  int c = ensure_implicit(h);
  if (c) return c;
  if ((engine == 8 && !h->imp.cluster8_ok) || (engine == 16 && !h->imp.cluster16_ok) ||
      (engine == 7 && !h->imp.window8_ok) || (engine == 9 && !h->imp.window16_ok))
    return MCFD_E_UNSUPPORTED;
  return implicit_set_wide_level(h->imp, wide_level, engine) == cudaSuccess ? MCFD_OK : MCFD_E_CUDA;
}

int mcfd_gmres(mcfd_geom* h, const double* b, double* x, double tol, int32_t max_iter, int32_t krylov_dim,
               int32_t* iterations, void* stream) {
  if (!h || !b || !x || !h->imp_built || !h->imp.prepared || max_iter <= 0 || krylov_dim <= 0) return MCFD_E_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  MatvecFn mv = implicit_operator(h);
  int it = 0;
  // the inner loop runs as a captured graph unless events are being recorded
  // for profiling (a captured loop body holds kernels only)
  const int key = h->profiling ? -1 : (h->imp_exact_jacobian ? 1 : 0);
  int r = gmres_solve(h->imp, mv, key, b, x, tol, max_iter, krylov_dim, &it, s);
  if (iterations) *iterations = it;
  switch (r) {
    case GMRES_OK: return MCFD_OK;
    case GMRES_NOT_CONVERGED: return MCFD_E_NOT_CONVERGED;
    case GMRES_BREAKDOWN: return MCFD_E_BREAKDOWN;
    default: return MCFD_E_CUDA;
  }
}

int mcfd_implicit_equation(mcfd_geom* h, const double* U, const double* U0, const double* R, const double* dt,
                           int32_t dt_per_cell, const double* scales, double* b, double* norms, void* stream) {
  if (!h || !U || !U0 || !R || !dt || !scales || !norms) return MCFD_E_ARG;
  int c = ensure_implicit(h);
  if (c) return c;
  cudaStream_t s = (cudaStream_t)stream;
  ImplicitState& st = h->imp;
  cudaError_t e = implicit_equation(st, U, U0, R, dt, dt_per_cell, scale_of(scales), b, st.scalars + 10, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(norms, st.scalars + 10, 2 * sizeof(double), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  return rc(e);
}

int mcfd_implicit_scale_maxima(mcfd_geom* h, const mcfd_config* cfg, const double* U, double* maxima,
                               void* stream) {
  if (!h || !U || !maxima) return MCFD_E_ARG;
  int c = check_cfg(cfg);
  if (c) return c;
  if ((c = ensure_implicit(h))) return c;
  cudaStream_t s = (cudaStream_t)stream;
  ImplicitState& st = h->imp;
  cudaError_t e = MCFD_DISPATCH(*cfg, launch_primitive(h->g, *cfg, U, h->ws.P, s));
  if (e == cudaSuccess) e = implicit_maxima(st, U, h->ws.P, cfg->gamma, st.scalars + 16, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(maxima, st.scalars + 16, 9 * sizeof(double), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  return rc(e);
}

int mcfd_implicit_candidate(mcfd_geom* h, const double* U, const double* dx, double damping, const double* scales,
                            double* out, void* stream) {
  if (!h || !U || !dx || !scales || !out) return MCFD_E_ARG;
  return rc(implicit_candidate(h->g.n_cells, U, dx, damping, scale_of(scales), out, (cudaStream_t)stream));
}

int mcfd_profile_enable(mcfd_geom* h, int32_t enable) {
  if (!h) return MCFD_E_ARG;
  h->profiling = enable != 0;
  return MCFD_OK;
}

int mcfd_profile_read(mcfd_geom* h, double* total_ms, int64_t* groups) {
  if (!h || !total_ms || !groups) return MCFD_E_ARG;
  for (int k = 0; k < MCFD_PROF_COUNT; ++k) {
    total_ms[k] = 0.0;
    groups[k] = 0;
  }
  cudaError_t err = cudaSuccess;
  if (!h->records.empty()) err = cudaEventSynchronize(h->records.back().stop);
  for (ProfRecord& r : h->records) {
    float ms = 0.0f;
    if (err == cudaSuccess) err = cudaEventElapsedTime(&ms, r.start, r.stop);
    total_ms[r.cls] += ms;
    groups[r.cls] += 1;
    h->event_pool.push_back(r.start);
    h->event_pool.push_back(r.stop);
  }
  h->records.clear();
  return rc(err);
}

int64_t mcfd_launch_count(void) { return (int64_t)launch_count(); }

int mcfd_batch_time_steps(mcfd_geom* h, const mcfd_config* cfg, const double* P, const int32_t* case_offsets,
                          int32_t n_cases, double* dt_case, double* dt_cells, void* stream) {
  if (!h || !P || !case_offsets || n_cases <= 0 || !dt_case || !dt_cells) return MCFD_E_ARG;
  int c = check_cfg(cfg);
  if (c) return c;
  if ((c = ensure_viscous(h, cfg))) return c;
  if (!(cfg->cfl > 0.0)) return MCFD_E_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e = timed(h, MCFD_PROF_TIME_STEP, s, [&] {
    cudaError_t r = cudaSuccess;
    if (h->g.n_bc_patches > 0) r = launch_bc_states(h->g, *cfg, P, nullptr, h->g.bc_ext_dt, s);
    if (r == cudaSuccess && cfg->viscosity_model != MCFD_VISC_INVISCID)
      r = launch_viscous_diffusion(h->g, *cfg, P, h->visc, s);
    if (r == cudaSuccess) r = MCFD_DISPATCH(*cfg, launch_time_steps(h->g, *cfg, P, dt_cells, nullptr, 0.0, s));
    if (r == cudaSuccess) r = launch_case_time_steps(h->g.n_cells, n_cases, case_offsets, dt_case, dt_cells, s);
    return r;
  });
  return rc(e);
}

// ------------------------------------------------------------- host helpers

int mcfd_host_cell_geometry(int64_t n_cells, const int64_t* off, const int64_t* nodes,
                            const double* pts, double* centers, double* areas, int64_t* bad_cell) {
  if (!off || !nodes || !pts || !centers || !areas) return MCFD_E_ARG;
  for (int64_t c = 0; c < n_cells; ++c) {
    const int64_t b = off[c], e = off[c + 1], k = e - b;
    // twice_area = sum(x0*y1 - x1*y0) over consecutive vertex pairs.  The
    // reference uses Python's built-in sum(), which for floats (CPython >= 3.12)
    // is Neumaier's compensated summation (Z. angew. Math. Mech. 54, 1974):
    // running sum t, compensation c, c added once at the end when non-zero.
    double twice = 0.0, comp = 0.0;
    for (int64_t i = 0; i < k; ++i) {
      const double* p0 = pts + 2 * nodes[b + i];
      const double* p1 = pts + 2 * nodes[b + (i + 1) % k];
      double x = p0[0] * p1[1] - p1[0] * p0[1];
      if (i == 0) {
        twice = x;  // 0 + x: the int start value folds exactly
        continue;
      }
      double t = twice + x;
      if (std::fabs(twice) >= std::fabs(x)) comp += (twice - t) + x;
      else comp += (x - t) + twice;
      twice = t;
    }
    if (comp != 0.0 && std::isfinite(comp)) twice += comp;
    if (!std::isfinite(twice) || std::fabs(twice) <= 1e-15) {
      if (bad_cell) *bad_cell = c;
      return MCFD_E_GEOMETRY;
    }
    double xs = 0.0, ys = 0.0;
    for (int64_t i = 0; i < k; ++i) {
      const double* p0 = pts + 2 * nodes[b + i];
      const double* p1 = pts + 2 * nodes[b + (i + 1) % k];
      double cross = p0[0] * p1[1] - p1[0] * p0[1];
      xs += (p0[0] + p1[0]) * cross;
      ys += (p0[1] + p1[1]) * cross;
    }
    centers[2 * c] = xs / (3.0 * twice);
    centers[2 * c + 1] = ys / (3.0 * twice);
    areas[c] = 0.5 * std::fabs(twice);
  }
  return MCFD_OK;
}

int mcfd_host_face_geometry(int64_t n_faces, const int64_t* face_nodes, const double* pts,
                            const double* centers, const int64_t* owners, double* face_centers,
                            double* normals, double* lengths, int64_t* bad_face) {
  if (!face_nodes || !pts || !centers || !owners || !face_centers || !normals || !lengths)
    return MCFD_E_ARG;
  for (int64_t f = 0; f < n_faces; ++f) {
    const double* a = pts + 2 * face_nodes[2 * f];
    const double* b = pts + 2 * face_nodes[2 * f + 1];
    double ex = b[0] - a[0], ey = b[1] - a[1];
    double length = std::sqrt(std::fma(ey, ey, ex * ex));
    if (!std::isfinite(length) || length <= 1e-15) {
      if (bad_face) *bad_face = f;
      return MCFD_E_GEOMETRY;
    }
    double nx = ey / length, ny = -ex / length;
    double cx = 0.5 * (a[0] + b[0]), cy = 0.5 * (a[1] + b[1]);
    const double* o = centers + 2 * owners[f];
    double dx = cx - o[0], dy = cy - o[1];
    if (std::fma(ny, dy, nx * dx) < 0.0) {
      nx = -nx;
      ny = -ny;
    }
    face_centers[2 * f] = cx;
    face_centers[2 * f + 1] = cy;
    normals[2 * f] = nx;
    normals[2 * f + 1] = ny;
    lengths[f] = length;
  }
  return MCFD_OK;
}

}  // extern "C"
