// kernels_dd_8.cu -- substep kernel variants, double-float state, 8 fields (entropy).
#include "kernels.cuh"
PCGB_DEFINE_KERNELS(kernel_dd_8, pcgb::dd, 8)
