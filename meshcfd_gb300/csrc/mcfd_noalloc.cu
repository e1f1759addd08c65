// Allocation-free variant of the residual sum-of-squares reduction.
//
// Who needs it: code that cannot call cudaMalloc — for example a convergence
// monitor invoked from inside a host application's time loop whose device
// memory is owned by another allocator (it must not grow its own pool), or a
// caller that must not trigger the implicit device synchronisation an
// allocation can cause in the middle of a step.  Such a caller has no
// mcfd_geom handle (creating one allocates), so this entry point takes the
// residual array and its length directly.
//
// Scratch: the per-block partial sums live in a file-scope __device__ array
// of fixed size (kSumsqBlocks x 4 float64 = 19,456 bytes), present on every
// GPU that loads the library until the process exits.  Host code cannot use
// the symbol itself as a device address; the address is obtained once per
// device with cudaGetSymbolAddress, with that device current, on the first
// call made on that device (so that first call should come before any stream
// capture).  The address is then cached for the life of the process: after a
// cudaDeviceReset (or any other reset of the device's primary context) the
// cached address is stale, so do not call this entry point again on that
// device after a reset.  Every call shares the array: calls that overlap on
// the GPU (different streams, or another thread) race on it.  Each block
// overwrites its own four partials and the final kernel reads only those, so
// nothing needs clearing between calls.  The returned status reads the
// thread's CUDA error state after the launches (cudaPeekAtLastError, which
// does not clear it), so an error left by an earlier call in the same thread
// is reported as MCFD_E_CUDA too.
#include <mutex>

#include "mcfd_internal.h"

namespace {

// The grid of mcfd_residual_sumsq (kSumsqBlocks), so both entry points sum in
// the same order.
constexpr int64_t kMaxCells = (int64_t)1 << 30;
constexpr int kMaxDevices = 64;

__device__ __align__(256) double g_sumsq_scratch[mcfd::kSumsqBlocks * 4];

std::mutex g_setup_mutex;
double* g_scratch_address[kMaxDevices] = {};

}  // namespace

extern "C" int mcfd_residual_sumsq_noalloc(const double* R, int64_t n_cells, double* sums,
                                           void* stream) {
  if (!R || !sums || n_cells <= 0) return MCFD_E_ARG;
  if (n_cells > kMaxCells) return MCFD_E_TOO_LARGE;
  int device = -1;
  if (cudaGetDevice(&device) != cudaSuccess) return MCFD_E_CUDA;
  if (device < 0 || device >= kMaxDevices) return MCFD_E_ARG;
  double* scratch = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_address[device]) {
      void* address = nullptr;
      if (cudaGetSymbolAddress(&address, g_sumsq_scratch) != cudaSuccess || !address) return MCFD_E_CUDA;
      g_scratch_address[device] = static_cast<double*>(address);
    }
    scratch = g_scratch_address[device];
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  mcfd::count_launch(2);
  mcfd::k_sumsq_partial<<<mcfd::kSumsqBlocks, mcfd::kSumsqThreads, 0, s>>>(static_cast<int>(n_cells), R, scratch);
  if (cudaPeekAtLastError() != cudaSuccess) return MCFD_E_CUDA;
  mcfd::k_sumsq_final<<<1, 32, 0, s>>>(mcfd::kSumsqBlocks, scratch, sums);
  return cudaPeekAtLastError() == cudaSuccess ? MCFD_OK : MCFD_E_CUDA;
}
