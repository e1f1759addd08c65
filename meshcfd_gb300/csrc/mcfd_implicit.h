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

struct ImplicitState {
  int n_cells = 0, n_coupling = 0, n_boundary = 0;
  int n_levels_fwd = 0, n_levels_bwd = 0, sweep_blocks = 1;
  // topology (device)
  int *ca = nullptr, *cb = nullptr, *bowner = nullptr;
  double2 *na = nullptr, *nb = nullptr, *bnormal = nullptr;
  double *clen = nullptr, *blen = nullptr;
  int *dptr = nullptr, *dref = nullptr, *rptr = nullptr, *rref = nullptr, *rcol = nullptr;
  int *fwd_level_ptr = nullptr, *fwd_level_cells = nullptr, *bwd_level_ptr = nullptr, *bwd_level_cells = nullptr;
  int *lower_ptr = nullptr, *lower_col = nullptr, *lower_val = nullptr;
  int *upper_ptr = nullptr, *upper_col = nullptr, *upper_val = nullptr;
  // values and vectors (device)
  double *coef = nullptr, *bterm = nullptr, *diag = nullptr, *dclamp = nullptr, *rval = nullptr;
  double *tmp = nullptr, *state = nullptr, *rate = nullptr, *up = nullptr, *rp = nullptr;
  double *w = nullptr, *av = nullptr, *partials = nullptr, *scalars = nullptr;
  // prepared operator
  ScaleVec scale{{1.0, 1.0, 1.0, 1.0}};
  double state_norm = 0.0;
  const double* dt = nullptr;
  int dt_per_cell = 0;
  bool prepared = false;
  // Krylov basis and Hessenberg column scratch, grown on demand
  std::vector<double*> krylov;
  double* hcol = nullptr;
  int hcol_size = 0;
  std::vector<void*> owned;
};

enum GmresResult { GMRES_OK = 0, GMRES_NOT_CONVERGED = 1, GMRES_BREAKDOWN = 2, GMRES_CUDA = 3 };

using ResidualFn = std::function<cudaError_t(const double* U, double* R, cudaStream_t s)>;
using MatvecFn = std::function<cudaError_t(const double* v, double* out, cudaStream_t s)>;

cudaError_t implicit_build(ImplicitState& st, const ImplicitTopology& t);
void implicit_free(ImplicitState& st);
cudaError_t implicit_assemble(ImplicitState& st, const double* P, const double* area, const double* dt,
                              int dt_per_cell, double gamma, cudaStream_t s);
cudaError_t lusgs_apply(ImplicitState& st, const double* v, double* x, cudaStream_t s);
cudaError_t fd_operator(ImplicitState& st, const ResidualFn& residual1, const double* v, double* out,
                        cudaStream_t s);
int gmres_solve(ImplicitState& st, const MatvecFn& matvec, const double* b, double* x, double tol,
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
