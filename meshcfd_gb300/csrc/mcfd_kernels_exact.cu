// Exact variant: reference operation order, no FMA contraction (-fmad=false).
#define MCFD_FAST 0
#define MCFD_VARIANT exact
#include "mcfd_kernels_impl.cuh"
