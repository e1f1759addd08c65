// Fast variant: exact arithmetic, limiter minimum through the smallest ratio.
#define MCFD_FAST 1
#define MCFD_VARIANT fast
#include "mcfd_kernels_impl.cuh"
