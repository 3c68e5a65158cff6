// kernels_upw_dd_7.cu -- substep kernels with the upwind corrections, double-float state, 7 fields.
#include "kernels.cuh"
PCGB_DEFINE_UPW_KERNELS(kernel_dd_7_upw, pcgb::dd, 7)
