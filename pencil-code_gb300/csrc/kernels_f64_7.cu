// kernels_f64_7.cu -- substep kernel variants, double state, 7 fields.
#include "kernels.cuh"
PCGB_DEFINE_KERNELS(kernel_f64_7, double, 7)
