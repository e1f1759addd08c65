// Internal interface of the exact Jacobian-vector product (mcfd_jvp.cu).
#pragma once

#include "mcfd_implicit.h"
#include "mcfd_internal.h"

namespace mcfd {

struct JvpWork {
  double* P = nullptr;       // primitive values [C][4]
  double* dP = nullptr;      // primitive tangents [C][4]
  double* recon = nullptr;   // face-state values [slots][4]
  double* drecon = nullptr;  // face-state tangents [slots][4]
  double* dflux = nullptr;   // flux tangents [n_flux][4]
  double* sv = nullptr;      // scaled direction [C][4] (implicit operator)
  double* dR = nullptr;      // residual tangent [C][4] (implicit operator)
};

cudaError_t launch_jvp(const DevGeom& g, const mcfd_config& cfg, const double* U, const double* dU,
                       const JvpWork& w, double* dR, cudaStream_t s);
// out = v - dt * (J (s v)) / s with J the exact Jacobian of R1 at the
// prepared state (the exact counterpart of the finite-difference operator)
cudaError_t exact_operator(const DevGeom& g, const mcfd_config& cfg1, const ImplicitState& st, const JvpWork& w,
                           const double* v, double* out, cudaStream_t s);

}  // namespace mcfd
