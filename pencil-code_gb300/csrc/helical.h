// helical.h -- random helical forcing (iforce='helical') added to uu after a time step.
#pragma once
#include <cuda_runtime.h>

#include "pcgb_box.h"

namespace pcgb {

// One time step's forcing, fconst_coefs_hel (forcing.f90:1763-1880):
// wavevector, phase, the two polarisation coefficient vectors and
// force/ffnorm (the device multiplies by sqrt(dt) of the step).
struct HelRec {
  double kk[3], phase, coef1[3], coef2[3], fact0;
};

constexpr int kHelRing = 64;   // records kept on the device, indexed by step % kHelRing

// Size of a step's tables: coef1[3], coef2[3], 2 spare, fx[nx], fy[ny], fz[nz] as
// (re, im) doubles, followed by the same values rounded to float (for FP32 states).
__host__ __device__ inline long long hel_tab_doubles(int nx, int ny, int nz) { return 8 + 2LL * (nx + ny + nz); }
__host__ __device__ inline size_t hel_tab_bytes(int nx, int ny, int nz) {
  return (size_t)hel_tab_doubles(nx, ny, nz) * (sizeof(double) + sizeof(float));
}

// Draw the record of the next step from the ran0 stream `state` (two draws for
// phase and wavevector, one for the polarisation angle, as the reference draws them).
void helical_record(double cs0, double relhel, double force, const double* kxyz, int nk, double kav, int* state,
                    HelRec* rec);

// Element layout of the box's f array.
enum HelLayout { HEL_F32 = 0, HEL_F64 = 1, HEL_DD = 2, HEL_F32_PAIR = 3, HEL_DD_PAIR = 4 };

struct HelGeom {
  int nx, ny, nz, px, my, xoff;
  long long ps, fs;   // plane and slice strides in elements
  double x0, y0, z0, dx, dy, dz, k1;
  double ox, oy, oz;  // grid point i of an axis is x0 + (i + o) dx: o = 1/2 periodic, 0 otherwise
  int iax;            // first slice of aa (field-major layouts)
  int magnetic;       // 1: the force goes into aa (lmagnetic_forcing), 0: into uu
};

// Tables of the completed step (record ring[(nsub/3 - 1) % kHelRing], dt_last
// of `state`) into `tab`, then the forced field += Re[(coef1 + i coef2) fx fy fz]
// on every interior cell and its periodic ghost images.
cudaError_t launch_helical(int layout, void* f, const HelRec* ring, const PcgbBoxState* state, double* tab,
                           const HelGeom& g, cudaStream_t s);

// The tables of the step in progress (ring[(nsub/3) % kHelRing], its dt) before
// its last substep, whose update adds the force itself (PcgbBoxDev::hel_tab).
cudaError_t launch_helical_tables_pre(const HelRec* ring, const PcgbBoxState* state, double* tab, const HelGeom& g,
                                      cudaStream_t s);

}  // namespace pcgb
