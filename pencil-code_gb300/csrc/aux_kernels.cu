// aux_kernels.cu -- layout conversion and ghost kernels used around the substep kernel.
//
// Host layout: the reference f-array f(mx,my,mz,nf), Fortran order, REAL=double,
// mx = nx+6 (no padding).  Device layout: rows of px elements with interior
// x = 0 at element xoff (ghosts at xoff-3 .. xoff-1 and xoff+nx .. xoff+nx+2),
// so row r of the host array (r = m + my*(n + mz*k)) starts at element
// px*r + xoff - 3 of the device array.
#include <cuda_runtime.h>
#include <stdint.h>
#include "aux_kernels.h"
#include "dd.cuh"

namespace pcgb {

__device__ __forceinline__ int wrap(int i, int n) {  // ghosted index -> interior image, 0-based interior
  int v = i - 3;
  if (v < 0) v += n;
  else if (v >= n) v -= n;
  return v;
}

// Periodic ghost fill (boundcond.f90:2387-2531 bc_per_x/y/z): every ghost cell
// takes the value of its interior image.  Reads interior cells only.
template <typename T>
__global__ void ghost_fill_kernel(T* __restrict__ f, int nx, int ny, int nz, int px, int my, int mz, int xoff,
                                  int nf) {
  const int mx = nx + 6;
  const long long total = (long long)mx * my * mz * nf;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total;
       q += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(q % mx);
    long long r = q / mx;
    const int j = (int)(r % my);
    r /= my;
    const int k = (int)(r % mz);
    const int fld = (int)(r / mz);
    const bool ghost = (i < 3) | (i >= nx + 3) | (j < 3) | (j >= ny + 3) | (k < 3) | (k >= nz + 3);
    if (!ghost) continue;
    const long long fo = (long long)fld * px * my * mz;
    const long long src = fo + (long long)(wrap(k, nz) + 3) * px * my + (long long)(wrap(j, ny) + 3) * px + xoff + wrap(i, nx);
    const long long dst = fo + (long long)k * px * my + (long long)j * px + xoff - 3 + i;
    f[dst] = f[src];
  }
}

// Device element of host-layout row `row` (r = m + my*(n + mz*field)), x index i
// (0..mx-1): field-major layout (pairs == 0) or packed pairs (pairs == 1, see
// cell_pair.cuh: P0=(ux,ax) P1=(uy,ay) P2=(uz,az) P3=(lnrho,ss)), in units of T.
__device__ __forceinline__ long long dev_index(long long row, int i, int my, int mz, int px, int xoff, int nf,
                                               int pairs) {
  if (!pairs) return row * px + xoff - 3 + i;
  const long long jk = row % ((long long)my * mz);
  const int fld = (int)(row / ((long long)my * mz));
  int pair, lane;
  if (fld < 3) { pair = fld; lane = 0; }
  else if (fld == 3) { pair = 3; lane = 0; }
  else if (nf == 8 && fld == 4) { pair = 3; lane = 1; }
  else { pair = fld - (nf - 3); lane = 1; }
  return 2 * (((long long)pair * my * mz + jk) * px + xoff - 3 + i) + lane;
}

// Rows [r0, r0+nr) of the host layout (REAL H: double, or float for the
// single-precision build) -> device layout (T).
template <typename T, typename H>
__global__ void load_rows_kernel(T* __restrict__ f, const H* __restrict__ stage, long long r0, long long nr, int mx,
                                 int my, int mz, int px, int xoff, int nf, int pairs) {
  const long long total = nr * mx;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total;
       q += (long long)gridDim.x * blockDim.x) {
    const long long r = q / mx;
    const int i = (int)(q - r * mx);
    f[dev_index(r0 + r, i, my, mz, px, xoff, nf, pairs)] = T((double)stage[q]);
  }
}

// Device layout (T) -> host-layout rows (REAL H).  With a carry array (FP32
// compensated mode), the value returned is f + carry of the interior image,
// summed in double and rounded once to H.
template <typename T, typename H>
__global__ void store_rows_kernel(H* __restrict__ stage, const T* __restrict__ f, const T* __restrict__ carry,
                                  long long r0, long long nr, int nx, int ny, int nz, int px, int my, int mz,
                                  int xoff, int nf, int pairs, int permask) {
  const int mx = nx + 6;
  const long long total = nr * mx;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total;
       q += (long long)gridDim.x * blockDim.x) {
    const long long r = q / mx;
    const int i = (int)(q - r * mx);
    const long long row = r0 + r;
    double v = (double)f[dev_index(row, i, my, mz, px, xoff, nf, pairs)];
    if (carry) {   // carry of the interior image of this (possibly ghost) cell
      const int j = (int)(row % my);
      long long rr = row / my;
      const int k = (int)(rr % mz);
      const long long fld = rr / mz;
      // a ghost of a non-periodic axis (bit clear in permask) holds its boundary value alone
      const bool bghost = (!(permask & 1) && (i < 3 || i >= nx + 3)) || (!(permask & 2) && (j < 3 || j >= ny + 3)) ||
                          (!(permask & 4) && (k < 3 || k >= nz + 3));
      const long long crow = (long long)(wrap(j, ny) + 3) + (long long)my * ((wrap(k, nz) + 3) + (long long)mz * fld);
      if (!bghost) v += (double)carry[dev_index(crow, wrap(i, nx) + 3, my, mz, px, xoff, nf, pairs)];
    }
    stage[q] = (H)v;
  }
}

// Double-float pair layout: device element e of 16 bytes holds (hi_a, hi_b,
// lo_a, lo_b); dev_index's pair index 2e + lane selects the field.
template <typename H>
__global__ void load_rows_ddpair_kernel(float* __restrict__ f, const H* __restrict__ stage, long long r0,
                                        long long nr, int mx, int my, int mz, int px, int xoff, int nf) {
  const long long total = nr * mx;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total;
       q += (long long)gridDim.x * blockDim.x) {
    const long long r = q / mx;
    const int i = (int)(q - r * mx);
    const long long pi = dev_index(r0 + r, i, my, mz, px, xoff, nf, 1);
    const long long e = pi >> 1, lane = pi & 1;
    const dd v((double)stage[q]);
    f[4 * e + lane] = v.hi;
    f[4 * e + 2 + lane] = v.lo;
  }
}

template <typename H>
__global__ void store_rows_ddpair_kernel(H* __restrict__ stage, const float* __restrict__ f, long long r0,
                                         long long nr, int nx, int my, int mz, int px, int xoff, int nf) {
  const int mx = nx + 6;
  const long long total = nr * mx;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total;
       q += (long long)gridDim.x * blockDim.x) {
    const long long r = q / mx;
    const int i = (int)(q - r * mx);
    const long long pi = dev_index(r0 + r, i, my, mz, px, xoff, nf, 1);
    const long long e = pi >> 1, lane = pi & 1;
    stage[q] = (H)((double)f[4 * e + lane] + (double)f[4 * e + 2 + lane]);
  }
}

static int grid_for(long long n, int threads) {
  long long g = (n + threads - 1) / threads;
  if (g > 65535LL * 16) g = 65535LL * 16;
  if (g < 1) g = 1;
  return (int)g;
}

cudaError_t launch_ghost_fill(int tbytes, void* f, int nx, int ny, int nz, int px, int my, int mz, int xoff, int nf,
                              cudaStream_t s) {
  const long long n = (long long)(nx + 6) * my * mz * nf;
  const int th = 256, g = grid_for(n, th);
  if (tbytes == 4)
    ghost_fill_kernel<float><<<g, th, 0, s>>>((float*)f, nx, ny, nz, px, my, mz, xoff, nf);
  else if (tbytes == 16)
    ghost_fill_kernel<float4><<<g, th, 0, s>>>((float4*)f, nx, ny, nz, px, my, mz, xoff, nf);
  else
    ghost_fill_kernel<double><<<g, th, 0, s>>>((double*)f, nx, ny, nz, px, my, mz, xoff, nf);
  return cudaGetLastError();
}

template <typename H>
static void load_rows(int tbytes, void* f, const H* stage, long long r0, long long nr, int mx, int my, int mz, int px,
                      int xoff, int nf, int pairs, cudaStream_t s) {
  const int th = 256, g = grid_for(nr * mx, th);
  if (tbytes == 4)
    load_rows_kernel<float, H><<<g, th, 0, s>>>((float*)f, stage, r0, nr, mx, my, mz, px, xoff, nf, pairs);
  else if (tbytes == kElemDD)
    load_rows_kernel<dd, H><<<g, th, 0, s>>>((dd*)f, stage, r0, nr, mx, my, mz, px, xoff, nf, pairs);
  else if (tbytes == kElemDDPair)
    load_rows_ddpair_kernel<H><<<g, th, 0, s>>>((float*)f, stage, r0, nr, mx, my, mz, px, xoff, nf);
  else
    load_rows_kernel<double, H><<<g, th, 0, s>>>((double*)f, stage, r0, nr, mx, my, mz, px, xoff, nf, pairs);
}

cudaError_t launch_load_rows(int tbytes, int hbytes, void* f, const void* stage, long long r0, long long nr, int mx,
                             int my, int mz, int px, int xoff, int nf, int pairs, cudaStream_t s) {
  if (hbytes == 4) load_rows(tbytes, f, (const float*)stage, r0, nr, mx, my, mz, px, xoff, nf, pairs, s);
  else load_rows(tbytes, f, (const double*)stage, r0, nr, mx, my, mz, px, xoff, nf, pairs, s);
  return cudaGetLastError();
}

template <typename H>
static void store_rows(int tbytes, H* stage, const void* f, const void* carry, long long r0, long long nr, int nx,
                       int ny, int nz, int px, int my, int mz, int xoff, int nf, int pairs, int permask,
                       cudaStream_t s) {
  const int th = 256, g = grid_for(nr * (nx + 6), th);
  if (tbytes == 4)
    store_rows_kernel<float, H><<<g, th, 0, s>>>(stage, (const float*)f, (const float*)carry, r0, nr, nx, ny, nz, px,
                                                 my, mz, xoff, nf, pairs, permask);
  else if (tbytes == kElemDD)
    store_rows_kernel<dd, H><<<g, th, 0, s>>>(stage, (const dd*)f, nullptr, r0, nr, nx, ny, nz, px, my, mz, xoff, nf,
                                              pairs, permask);
  else if (tbytes == kElemDDPair)
    store_rows_ddpair_kernel<H><<<g, th, 0, s>>>(stage, (const float*)f, r0, nr, nx, my, mz, px, xoff, nf);
  else
    store_rows_kernel<double, H><<<g, th, 0, s>>>(stage, (const double*)f, (const double*)carry, r0, nr, nx, ny, nz,
                                                  px, my, mz, xoff, nf, pairs, permask);
}

cudaError_t launch_store_rows(int tbytes, int hbytes, void* stage, const void* f, const void* carry, long long r0,
                              long long nr, int nx, int ny, int nz, int px, int my, int mz, int xoff, int nf, int pairs,
                              int permask, cudaStream_t s) {
  if (hbytes == 4)
    store_rows(tbytes, (float*)stage, f, carry, r0, nr, nx, ny, nz, px, my, mz, xoff, nf, pairs, permask, s);
  else
    store_rows(tbytes, (double*)stage, f, carry, r0, nr, nx, ny, nz, px, my, mz, xoff, nf, pairs, permask, s);
  return cudaGetLastError();
}

}  // namespace pcgb

namespace pcgb {

// splitmix64 (Steele, Lea & Flood 2014), used as a counter-based generator.
__device__ __forceinline__ unsigned long long splitmix64(unsigned long long x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

// Seeded initial conditions written on the device into one field's interior:
// kind 0: set to zero; 1: add ampl * N(0,1) (Box-Muller on two counter-based
// uniforms); 2: add the ABC flow component fld (hydro.f90:2214-2220) with
// amplitudes a,b,c and wavenumber k on the cell-centred grid.
// Value access of init_field_kernel: element e of a T array with a stride
// (field-major, or one lane of the FP32 pair layout), or one field of the
// double-float pair layout (hi at float 4e, lo at float 4e + 2 of a lane base).
template <typename T>
struct ElemRef {
  T* f;
  int stride;
  __device__ __forceinline__ double get(long long e) const { return (double)f[stride * e]; }
  __device__ __forceinline__ void set(long long e, double v) const { f[stride * e] = (T)v; }
};
struct DDPairRef {
  float* f;
  __device__ __forceinline__ double get(long long e) const { return (double)f[4 * e] + (double)f[4 * e + 2]; }
  __device__ __forceinline__ void set(long long e, double v) const {
    const dd d(v);
    f[4 * e] = d.hi;
    f[4 * e + 2] = d.lo;
  }
};

template <class REF>
__global__ void init_field_kernel(REF f, int kind, int comp, double ampl, double a, double b, double c, double k,
                                  unsigned long long seed, int nx, int ny, int nz, int px, int my, int xoff, double x0,
                                  double y0, double z0, double dx, double dy, double dz, double ox, double oy,
                                  double oz) {
  const long long total = (long long)nx * ny * nz;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total;
       q += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(q % nx);
    const long long r = q / nx;
    const int j = (int)(r % ny);
    const int kk = (int)(r / ny);
    const long long idx = (long long)(kk + 3) * px * my + (long long)(j + 3) * px + xoff + i;
    if (kind == 0) {
      f.set(idx, 0.0);
    } else if (kind == 1) {
      const unsigned long long h1 = splitmix64(seed * 0x100000001B3ull + 2ull * (unsigned long long)q);
      const unsigned long long h2 = splitmix64(h1 ^ 0xD1B54A32D192ED03ull);
      const double u1 = ((double)(h1 >> 11) + 1.0) * (1.0 / 9007199254740993.0);   // (0,1]
      const double u2 = (double)(h2 >> 11) * (1.0 / 9007199254740992.0);            // [0,1)
      const double g = sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
      f.set(idx, f.get(idx) + ampl * g);
    } else {
      // grid point i of an axis: x0 + (i + o) dx, o = 1/2 on a periodic axis, 0 otherwise
      const double x = x0 + ((double)i + ox) * dx, y = y0 + ((double)j + oy) * dy, z = z0 + ((double)kk + oz) * dz;
      double v;
      if (comp == 0) v = a * sin(k * z) + c * cos(k * y);
      else if (comp == 1) v = b * sin(k * x) + a * cos(k * z);
      else v = c * sin(k * y) + b * cos(k * x);
      f.set(idx, f.get(idx) + ampl * v);
    }
  }
}

cudaError_t launch_init_field(int tbytes, void* f, int kind, int comp, double ampl, double a, double b, double c,
                              double k, unsigned long long seed, int nx, int ny, int nz, int px, int my, int xoff,
                              double x0, double y0, double z0, double dx, double dy, double dz, double ox, double oy,
                              double oz, int estride,
                              cudaStream_t s) {
  const int th = 256, g = grid_for((long long)nx * ny * nz, th);
  if (tbytes == 4)
    init_field_kernel<<<g, th, 0, s>>>(ElemRef<float>{(float*)f, estride}, kind, comp, ampl, a, b, c, k, seed, nx, ny,
                                       nz, px, my, xoff, x0, y0, z0, dx, dy, dz, ox, oy, oz);
  else if (tbytes == kElemDD)
    init_field_kernel<<<g, th, 0, s>>>(ElemRef<dd>{(dd*)f, estride}, kind, comp, ampl, a, b, c, k, seed, nx, ny, nz,
                                       px, my, xoff, x0, y0, z0, dx, dy, dz, ox, oy, oz);
  else if (tbytes == kElemDDPair)
    init_field_kernel<<<g, th, 0, s>>>(DDPairRef{(float*)f}, kind, comp, ampl, a, b, c, k, seed, nx, ny, nz, px, my,
                                       xoff, x0, y0, z0, dx, dy, dz, ox, oy, oz);
  else
    init_field_kernel<<<g, th, 0, s>>>(ElemRef<double>{(double*)f, estride}, kind, comp, ampl, a, b, c, k, seed, nx,
                                       ny, nz, px, my, xoff, x0, y0, z0, dx, dy, dz, ox, oy, oz);
  return cudaGetLastError();
}

}  // namespace pcgb
