// kernels_dd_7.cu -- substep kernel variants, double-float state, 7 fields.
#include "kernels.cuh"
PCGB_DEFINE_KERNELS(kernel_dd_7, pcgb::dd, 7)
