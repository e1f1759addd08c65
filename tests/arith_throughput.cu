// Throughput of binary64 division, square root and product on this GPU: the
// FP64 unit against the integer-pipe routines of mcfd_arith.cuh, alone and
// interleaved (8 independent dependency chains per thread, 608 x 256
// threads, the second of two timed launches).  Each integer-pipe chain is
// also replayed with the FP64 unit's operation and compared bit for bit.
//
// Prints one line per case: "<case> <G ops/s>" and, last,
// "mismatches=<n>".  Exit status 0 when no result differs.
#include <cstdio>

#include "../meshcfd_gb300/csrc/mcfd_arith.cuh"

namespace {

constexpr int kBlocks = 152 * 4, kThreads = 256, kChains = 8;

enum Op { DIV = 0, SQRT = 1, MUL = 2, ADD = 3 };

// emulated chains: k < n_emu use the integer-pipe routine, the rest the FP64 unit
template <int OP>
__global__ void k_chain(double* out, int iters, int n_emu, double c) {
  double x[kChains];
#pragma unroll
  for (int k = 0; k < kChains; ++k) x[k] = 1.0 + threadIdx.x * 1e-3 + 0.1 * k;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < kChains; ++k) {
      const bool emu = k < n_emu;
      if (OP == DIV) x[k] = (emu ? mcfd::div_rn(c, x[k]) : c / x[k]) + 0.75;
      else if (OP == SQRT) x[k] = (emu ? mcfd::sqrt_rn(x[k]) : sqrt(x[k])) + 0.75;
      else if (OP == MUL) x[k] = emu ? mcfd::mul_rn(x[k], c) : x[k] * c;
      else x[k] = x[k] * c + 1e-3;
    }
  }
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < kChains; ++k) s += x[k];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// one chain through the integer routine and the same chain through the FP64
// unit (separately rounded operations, no contraction): the values must agree
// bit for bit at every step
template <int OP>
__global__ void k_compare(int iters, double c, unsigned long long* bad) {
  double x = 1.0 + threadIdx.x * 1e-3 + blockIdx.x * 1e-6, y = x;
  for (int i = 0; i < iters; ++i) {
    if (OP == DIV) { x = mcfd::div_rn(c, x) + 0.75; y = c / y + 0.75; }
    else if (OP == SQRT) { x = mcfd::sqrt_rn(x) + 0.75; y = sqrt(y) + 0.75; }
    else { x = __dadd_rn(mcfd::mul_rn(x, c), 0.125); y = __dadd_rn(__dmul_rn(y, c), 0.125); }
    if (__double_as_longlong(x) != __double_as_longlong(y)) {
      atomicAdd(bad, 1ull);
      return;
    }
  }
}

template <int OP>
double rate(double* out, int iters, int n_emu, double c, int ops_per_step) {
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  float ms = 0.0f;
  for (int rep = 0; rep < 2; ++rep) {
    cudaEventRecord(a);
    k_chain<OP><<<kBlocks, kThreads>>>(out, iters, n_emu, c);
    cudaEventRecord(b);
    cudaEventSynchronize(b);
    cudaEventElapsedTime(&ms, a, b);
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return (double)ops_per_step * kChains * iters * kBlocks * kThreads / (ms * 1e-3) * 1e-9;
}

}  // namespace

int main() {
  double* out = nullptr;
  unsigned long long* bad = nullptr;
  if (cudaMalloc(&out, kBlocks * kThreads * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&bad, sizeof(unsigned long long)) != cudaSuccess) {
    printf("allocation failed\n");
    return 2;
  }
  cudaMemset(bad, 0, sizeof(unsigned long long));
  k_compare<DIV><<<kBlocks, kThreads>>>(256, 1.5, bad);
  k_compare<SQRT><<<kBlocks, kThreads>>>(256, 0.0, bad);
  k_compare<MUL><<<kBlocks, kThreads>>>(256, 0.999999, bad);
  unsigned long long mismatches = 0;
  cudaMemcpy(&mismatches, bad, sizeof(mismatches), cudaMemcpyDeviceToHost);

  printf("fp64_fma_chain %.1f\n", rate<ADD>(out, 4096, 0, 0.999999, 1));
  printf("div_fp64 %.1f\n", rate<DIV>(out, 512, 0, 1.5, 1));
  printf("div_int %.1f\n", rate<DIV>(out, 512, kChains, 1.5, 1));
  printf("div_half_half %.1f\n", rate<DIV>(out, 512, kChains / 2, 1.5, 1));
  printf("sqrt_fp64 %.1f\n", rate<SQRT>(out, 512, 0, 0.0, 1));
  printf("sqrt_int %.1f\n", rate<SQRT>(out, 512, kChains, 0.0, 1));
  printf("mul_fp64 %.1f\n", rate<MUL>(out, 2048, 0, 0.9999999, 1));
  printf("mul_int %.1f\n", rate<MUL>(out, 2048, kChains, 0.9999999, 1));
  printf("mul_half_half %.1f\n", rate<MUL>(out, 2048, kChains / 2, 0.9999999, 1));
  const cudaError_t err = cudaDeviceSynchronize();
  printf("cuda %s\n", cudaGetErrorString(err));
  printf("mismatches=%llu\n", mismatches);
  cudaFree(out);
  cudaFree(bad);
  return (err == cudaSuccess && mismatches == 0) ? 0 : 1;
}
