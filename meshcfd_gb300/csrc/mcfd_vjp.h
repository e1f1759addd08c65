// Internal interface of the reverse-mode residual product (mcfd_vjp.cu).
#pragma once

#include "mcfd_internal.h"

namespace mcfd {

struct VjpWork {
  double* P = nullptr;         // primitive values [C][4]
  double* recon = nullptr;     // face-state values [slots][4]
  double* slot_bar = nullptr;  // face-state adjoints [slots][4]
  double* pbar = nullptr;      // primitive adjoints [C][4] (also per-cell scratch)
  double* ent_bar = nullptr;   // per gradient entry: share for the neighbour [E][4]
  double* partials = nullptr;  // reduction scratch [608 block sums + 8]
  // the boundary face segments run on a second stream, concurrently with
  // the interior faces (each face writes only its own two face-state slots)
  cudaStream_t side = nullptr;
  cudaEvent_t fork = nullptr, join = nullptr;
};

// P_in / recon_in: primitive and face states of U when the caller has them
// (null: computed here)
cudaError_t launch_vjp(const DevGeom& g, const mcfd_config& cfg, const double* U, const double* P_in,
                       const double* recon_in, const double* lambda,
                       const VjpWork& w, double* ubar, double* far_bar, cudaStream_t s);
cudaError_t launch_wall_force(const DevGeom& g, const mcfd_config& cfg, const double* U, double dx, double dy,
                              const VjpWork& w, double* J_dev, double* dJdU, cudaStream_t s);

}  // namespace mcfd
