// helical_force.cuh -- the force of one step of random helical forcing at a grid
// point, Re[(coef1_c + i coef2_c) (fx fy) fz] (forcing.f90:2195-2230, fxyz_coefs_hel
// :1882-1930), from the step's tables (helical.cu: coef1[3], coef2[3], 2 spare, then
// fx[nx], fy[ny], fz[nz] as (re, im) pairs, fx carrying force/ffnorm sqrt(dt)).
// Shared by the apply kernel and the fused last-substep update, so both add the
// same values: arithmetic in R without contraction.
#pragma once

namespace pcgb {

__device__ __forceinline__ float rmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double rmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float radd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double radd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float rsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double rsub(double a, double b) { return __dsub_rn(a, b); }

// fx(i) fy(j); T: the table's element type (double, or its float copy)
template <typename R, typename T>
__device__ __forceinline__ void helical_fxy(const T* tab, int nx, int i, int j, R& pr, R& pi) {
  const T* fx = tab + 8;
  const T* fy = fx + 2 * nx;
  const R xr = (R)fx[2 * i], xi = (R)fx[2 * i + 1];
  const R yr = (R)fy[2 * j], yi = (R)fy[2 * j + 1];
  pr = rsub(rmul(xr, yr), rmul(xi, yi));
  pi = radd(rmul(xr, yi), rmul(xi, yr));
}

// the three force components at plane k from fx fy = (pr, pi)
template <typename R, typename T>
__device__ __forceinline__ void helical_fz(const T* tab, int nx, int ny, int k, R pr, R pi, R out[3]) {
  const T* fz = tab + 8 + 2 * nx + 2 * ny;
  const R zr = (R)fz[2 * k], zi = (R)fz[2 * k + 1];
  const R qr = rsub(rmul(pr, zr), rmul(pi, zi)), qi = radd(rmul(pr, zi), rmul(pi, zr));   // (fx fy) fz
#pragma unroll
  for (int c = 0; c < 3; ++c) out[c] = rsub(rmul((R)tab[c], qr), rmul((R)tab[3 + c], qi));
}

template <typename R, typename T>
__device__ __forceinline__ void helical_force_at(const T* tab, int nx, int ny, int i, int j, int k, R out[3]) {
  R pr, pi;
  helical_fxy(tab, nx, i, j, pr, pi);
  helical_fz(tab, nx, ny, k, pr, pi, out);
}

}  // namespace pcgb
