// kernels_upw_dd.cu -- substep kernels with the upwind corrections, double-float state, 7 and 8 fields.
#include "kernels.cuh"
PCGB_DEFINE_UPW_KERNELS(kernel_dd_7_upw, pcgb::dd, 7)
PCGB_DEFINE_UPW_KERNELS(kernel_dd_8_upw, pcgb::dd, 8)
