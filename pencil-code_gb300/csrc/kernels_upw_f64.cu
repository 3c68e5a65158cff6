// kernels_upw_f64.cu -- substep kernels with the upwind corrections, double state, 7 and 8 fields.
#include "kernels.cuh"
PCGB_DEFINE_UPW_KERNELS(kernel_f64_7_upw, double, 7)
PCGB_DEFINE_UPW_KERNELS(kernel_f64_8_upw, double, 8)
