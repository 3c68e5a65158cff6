// kernels_f64_8.cu -- substep kernel variants, double state, 8 fields.
#include "kernels.cuh"
PCGB_DEFINE_KERNELS(kernel_f64_8, double, 8)
