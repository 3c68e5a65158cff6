// kernels_upw_dd_8.cu -- substep kernels with the upwind corrections, double-float state, 8 fields
// (a translation unit of its own so that the two compile in parallel).
#include "kernels.cuh"
PCGB_DEFINE_UPW_KERNELS(kernel_dd_8_upw, pcgb::dd, 8)
