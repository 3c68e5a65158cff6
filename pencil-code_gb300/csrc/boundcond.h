// boundcond.h -- non-periodic boundary conditions of the ghost zones and the
// grid of a box (boundcond.f90 bcx/bcy/bcz, grid.f90:123-151).
#pragma once
#include <cuda_runtime.h>

#include "pcgb300.h"

namespace pcgb {

// Number of fields of a parameter block (f-array order: uu, lnrho, [ss], aa).
inline int params_nf(const pcgb_params& p) { return p.lentropy ? 8 : 7; }

// A direction is periodic when every code of its fields is PCGB_BC_PER.
inline bool axis_periodic(const pcgb_params& p, int dir) {
  for (int k = 0; k < params_nf(p); ++k)
    if (p.bc[dir][k][0] != PCGB_BC_PER || p.bc[dir][k][1] != PCGB_BC_PER) return false;
  return true;
}

// grid.f90:123-151: dx = L/n on a periodic axis (cell centres, x_i = x0 + (i + 1/2) dx),
// L/(n - 1) otherwise (points on both boundaries, x_i = x0 + i dx), i = 0 .. n-1 interior.
inline double axis_spacing(const pcgb_params& p, int dir) {
  const int n = dir == 0 ? p.nx : dir == 1 ? p.ny : p.nz;
  return p.Lxyz[dir] / (axis_periodic(p, dir) ? n : n - 1);
}
inline double axis_offset(const pcgb_params& p, int dir) { return axis_periodic(p, dir) ? 0.5 : 0.0; }
inline double axis_position(const pcgb_params& p, int dir, int i) {
  return p.xyz0[dir] + ((double)i + axis_offset(p, dir)) * axis_spacing(p, dir);
}

// The ghost zones of the non-periodic directions of f, in the order of pde's
// boundconds_x, _y, _z (equ.f90): one launch per non-periodic direction.  The
// periodic directions' ghosts are the images the substep kernel writes.
// layout: the HelLayout code of the box's elements (helical.h).  carry: the FP32
// compensation carry (df at a step boundary) or null; where 'a' sets a boundary
// value to 0, its carry is set to 0 too.
cudaError_t launch_boundconds(int layout, void* f, void* carry, const pcgb_params& p, int nx, int ny, int nz, int px,
                              int my, int mz, int xoff, long long ps, long long fs, int nf, cudaStream_t s);

}  // namespace pcgb
