// Variant-independent kernels: the residual sum of squares, the launch
// counter and the element-wise division / square root / product entry points.  Compiled
// with -fmad=false (plain additions in a fixed tree).
#include "mcfd_device.cuh"
#include "mcfd_internal.h"

namespace mcfd {

static constexpr int kBlock = 256;

// ------------------------------------------------------------- sum of squares

// Per thread a grid-stride sum, per warp a shuffle tree, per block the warps'
// sums added in warp order by one thread: a fixed order for a fixed grid
// (kSumsqBlocks x kSumsqThreads), so every call gives the same bits.
__global__ void __launch_bounds__(kSumsqThreads) k_sumsq_partial(int n, const double* __restrict__ R,
                                                                 double* __restrict__ partials) {
  __shared__ double warp_sum[kSumsqThreads / 32][4];
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
    const St4 r = ld4(R + 4 * (size_t)c);
    acc[0] += r.a * r.a; acc[1] += r.b * r.b; acc[2] += r.c * r.c; acc[3] += r.d * r.d;
  }
#pragma unroll
  for (int k = 0; k < 4; ++k)
    for (int off = 16; off > 0; off >>= 1) acc[k] += __shfl_down_sync(0xffffffffu, acc[k], off);
  if ((threadIdx.x & 31) == 0)
    for (int k = 0; k < 4; ++k) warp_sum[threadIdx.x >> 5][k] = acc[k];
  __syncthreads();
  if (threadIdx.x < 4) {
    double s = warp_sum[0][threadIdx.x];
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) s += warp_sum[w][threadIdx.x];
    partials[4 * blockIdx.x + threadIdx.x] = s;
  }
}

__global__ void k_sumsq_final(int blocks, const double* __restrict__ partials, double* sums) {
  if (threadIdx.x < 4) {
    double s = 0.0;
    for (int b = 0; b < blocks; ++b) s += partials[4 * b + threadIdx.x];
    sums[threadIdx.x] = s;
  }
}

// ------------------------------------------------------------ batched cases

// Per-case minimum of positive per-cell time steps (one block per case; the
// doubles' bit patterns order like the values), written to dt_case.
__global__ void __launch_bounds__(kBlock) k_case_min(const int* __restrict__ offsets,
                                                     const double* __restrict__ dt_cells,
                                                     double* __restrict__ dt_case) {
  const int k = blockIdx.x;
  const int b = offsets[k], e = offsets[k + 1];
  long long m = 0x7ff0000000000000LL;
  for (int c = b + threadIdx.x; c < e; c += blockDim.x) {
    const long long v = __double_as_longlong(dt_cells[c]);
    m = v < m ? v : m;
  }
  for (int off = 16; off > 0; off >>= 1) {
    const long long o = __shfl_down_sync(0xffffffffu, m, off);
    m = o < m ? o : m;
  }
  __shared__ long long wmin[kBlock / 32];
  if ((threadIdx.x & 31) == 0) wmin[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    long long r = wmin[0];
    for (int w = 1; w < kBlock / 32; ++w) r = wmin[w] < r ? wmin[w] : r;
    dt_case[k] = __longlong_as_double(r);
  }
}

// dt_cells[c] = dt_case[case of c] (binary search in the offset table)
__global__ void k_case_broadcast(int n_cells, int n_cases, const int* __restrict__ offsets,
                                 const double* __restrict__ dt_case, double* __restrict__ dt_cells) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n_cells) return;
  int lo = 0, hi = n_cases;  // offsets[lo] <= c < offsets[hi]
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (offsets[mid] <= c) lo = mid;
    else hi = mid;
  }
  dt_cells[c] = dt_case[lo];
}

cudaError_t launch_case_time_steps(int n_cells, int n_cases, const int* offsets, double* dt_case,
                                   double* dt_cells, cudaStream_t s) {
  count_launch(2);
  k_case_min<<<n_cases, kBlock, 0, s>>>(offsets, dt_cells, dt_case);
  k_case_broadcast<<<(n_cells + kBlock - 1) / kBlock, kBlock, 0, s>>>(n_cells, n_cases, offsets, dt_case, dt_cells);
  return cudaGetLastError();
}

// Kernels launched by this library (host-side counter, for measurement).
static long long g_launches = 0;
long long launch_count() { return __atomic_load_n(&g_launches, __ATOMIC_RELAXED); }
void count_launch(int n) { __atomic_fetch_add(&g_launches, (long long)n, __ATOMIC_RELAXED); }

cudaError_t launch_sumsq(const DevGeom& g, const double* R, double* partials, int blocks,
                         double* sums, cudaStream_t s) {
  count_launch(2);
  k_sumsq_partial<<<blocks, kSumsqThreads, 0, s>>>(g.n_cells, R, partials);
  k_sumsq_final<<<1, 32, 0, s>>>(blocks, partials, sums);
  return cudaGetLastError();
}

// ------------------------------------------------- division and square root

__global__ void __launch_bounds__(kBlock) k_ieee_div_sqrt(long long n, const double* __restrict__ a,
                                                          const double* __restrict__ b,
                                                          double* __restrict__ quotient,
                                                          double* __restrict__ root) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const double x = a[i];
    if (quotient) quotient[i] = div_rn(x, b[i]);
    if (root) root[i] = sqrt_rn(x);
  }
}

__global__ void __launch_bounds__(kBlock) k_ieee_div_fma(long long n, const double* __restrict__ a,
                                                         const double* __restrict__ b, double* __restrict__ quotient) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const double d = b[i];
    const unsigned long long X = recip_fixed(d);
    quotient[i] = div_rn_fma(a[i], d, div_rn_recip(1.0, d, X), X);
  }
}

__global__ void __launch_bounds__(kBlock) k_ieee_mul(long long n, const double* __restrict__ a,
                                                     const double* __restrict__ b, double* __restrict__ product) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    product[i] = mul_rn(a[i], b[i]);
}

// The global time step from the block minima (min with the end-time limit,
// Python's min semantics, solver.py:455-461); resets the minimum.
__global__ void k_finalize_time_step(DevStatus* st, double* dt_min, double time_limit) {
  const double stable = __longlong_as_double((long long)st->dt_min_bits);
  dt_min[0] = icmp::lt(time_limit, stable) ? time_limit : stable;
  st->dt_min_bits = 0x7ff0000000000000ULL;
}

cudaError_t finalize_time_step(DevStatus* st, double* dt_min, double time_limit, cudaStream_t s) {
  k_finalize_time_step<<<1, 1, 0, s>>>(st, dt_min, time_limit);
  return cudaGetLastError();
}

}  // namespace mcfd

extern "C" int mcfd_ieee_mul(const double* a, const double* b, int64_t n, double* product, void* stream) {
  if (n < 0 || (n > 0 && (!a || !b || !product))) return MCFD_E_ARG;
  if (n == 0) return MCFD_OK;
  const long long blocks = (n + mcfd::kBlock - 1) / mcfd::kBlock;
  mcfd::count_launch(1);
  mcfd::k_ieee_mul<<<(int)(blocks < 152 * 16 ? blocks : 152 * 16), mcfd::kBlock, 0,
                     static_cast<cudaStream_t>(stream)>>>(n, a, b, product);
  return cudaGetLastError() == cudaSuccess ? MCFD_OK : MCFD_E_CUDA;
}

extern "C" int mcfd_ieee_div_fma(const double* a, const double* b, int64_t n, double* quotient, void* stream) {
  if (n < 0 || (n > 0 && (!a || !b || !quotient))) return MCFD_E_ARG;
  if (n == 0) return MCFD_OK;
  const long long blocks = (n + mcfd::kBlock - 1) / mcfd::kBlock;
  mcfd::count_launch(1);
  mcfd::k_ieee_div_fma<<<(int)(blocks < 152 * 16 ? blocks : 152 * 16), mcfd::kBlock, 0,
                         static_cast<cudaStream_t>(stream)>>>(n, a, b, quotient);
  return cudaGetLastError() == cudaSuccess ? MCFD_OK : MCFD_E_CUDA;
}

extern "C" int mcfd_ieee_div_sqrt(const double* a, const double* b, int64_t n, double* quotient,
                                  double* root, void* stream) {
  if (n < 0 || (n > 0 && !a) || (quotient && !b)) return MCFD_E_ARG;
  if (n == 0 || (!quotient && !root)) return MCFD_OK;
  const long long blocks = (n + mcfd::kBlock - 1) / mcfd::kBlock;
  mcfd::count_launch(1);
  mcfd::k_ieee_div_sqrt<<<(int)(blocks < 152 * 16 ? blocks : 152 * 16), mcfd::kBlock, 0,
                          static_cast<cudaStream_t>(stream)>>>(n, a, b, quotient, root);
  return cudaGetLastError() == cudaSuccess ? MCFD_OK : MCFD_E_CUDA;
}
