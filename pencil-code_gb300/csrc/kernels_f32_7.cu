// kernels_f32_7.cu -- substep kernel variants, float state, 7 fields.
#include "kernels.cuh"
PCGB_DEFINE_KERNELS(kernel_f32_7, float, 7)
