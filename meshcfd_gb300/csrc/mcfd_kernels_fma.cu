// FMA variant: fast limiter, shared reciprocals, FMA contraction on.
#define MCFD_FAST 2
#define MCFD_VARIANT fma
#include "mcfd_kernels_impl.cuh"
