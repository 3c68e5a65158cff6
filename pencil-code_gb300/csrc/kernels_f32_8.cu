// kernels_f32_8.cu -- substep kernel variants, float state, 8 fields.
#include "kernels.cuh"
PCGB_DEFINE_KERNELS(kernel_f32_8, float, 8)
