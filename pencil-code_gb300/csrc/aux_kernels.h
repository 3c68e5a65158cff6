// aux_kernels.h -- launchers for the layout-conversion and ghost kernels.
#pragma once
#include <cuda_runtime.h>

namespace pcgb {
// Element codes passed as `tbytes` to the row and init kernels: 4 float,
// 8 double, kElemDD double-float (an 8-byte hi/lo pair of floats, dd.cuh),
// kElemDDPair two double-float fields packed as one 16-byte dd2 (lanes as in
// the FP32 pair layout).  launch_ghost_fill takes the element size in bytes.
constexpr int kElemDD = 16;
constexpr int kElemDDPair = 32;
cudaError_t launch_ghost_fill(int tbytes, void* f, int nx, int ny, int nz, int px, int my, int mz, int xoff, int nf,
                              cudaStream_t s);
// pairs = 1: packed field-pair layout (P0=(ux,ax) P1=(uy,ay) P2=(uz,az) P3=(lnrho,ss)), px/xoff in pair units
// Host rows of REAL type (hbytes 8: double, 4: float) <-> the device layout.
cudaError_t launch_load_rows(int tbytes, int hbytes, void* f, const void* stage, long long r0, long long nr, int mx,
                             int my, int mz, int px, int xoff, int nf, int pairs, cudaStream_t s);
// permask: bit d set when axis d is periodic (a ghost of a non-periodic axis gets no carry)
cudaError_t launch_store_rows(int tbytes, int hbytes, void* stage, const void* f, const void* carry, long long r0,
                              long long nr, int nx, int ny, int nz, int px, int my, int mz, int xoff, int nf, int pairs,
                              int permask, cudaStream_t s);
}  // namespace pcgb
namespace pcgb {
cudaError_t launch_init_field(int tbytes, void* f, int kind, int comp, double ampl, double a, double b, double c,
                              double k, unsigned long long seed, int nx, int ny, int nz, int px, int my, int xoff,
                              double x0, double y0, double z0, double dx, double dy, double dz, double ox,
                              double oy, double oz, int estride, cudaStream_t s);
}  // namespace pcgb
