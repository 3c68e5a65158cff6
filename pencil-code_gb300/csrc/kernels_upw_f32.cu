// kernels_upw_f32.cu -- substep kernels with the upwind corrections, float state, 7 and 8 fields.
#include "kernels.cuh"
PCGB_DEFINE_UPW_KERNELS(kernel_f32_7_upw, float, 7)
PCGB_DEFINE_UPW_KERNELS(kernel_f32_8_upw, float, 8)
