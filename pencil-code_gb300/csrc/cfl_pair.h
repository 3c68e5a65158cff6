// cfl_pair.h -- the CFL pass of the FP32 packed-pair layout (cfl_pair.cu).
#pragma once
#include <cuda_runtime.h>

#include "pcgb_box.h"

namespace pcgb {

// Blocks of one pass over an nx x ny x nz box: the size of `partial` in doubles.
size_t cfl_pair_blocks(int nx, int ny, int nz);

// dt1 = max over cells of the CFL inverse timestep of the box's current f, then
// dt = 1/dt1 into the box state (unless its dt is fixed); `done` is a zeroed
// counter the pass leaves zeroed.
cudaError_t launch_cfl_pair(const PcgbBoxDev* dbox, int nf, int nx, int ny, int nz, double* partial,
                            unsigned int* done, cudaStream_t s);

}  // namespace pcgb
