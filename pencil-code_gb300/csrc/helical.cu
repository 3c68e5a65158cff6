// helical.cu -- random helical forcing, iforce='helical' (forcing.f90:1307
// addforce, :2066-2474 forcing_hel, :1763-1880 fconst_coefs_hel, :1882-1930
// fxyz_coefs_hel), default options: no shear, no k-vector scaling, the new
// polarisation vectors, fda = 1, unit profiles, slope_ff = 0, cs0eff = cs0.
//
// After every time step the force, a single helical Fourier mode of the
// wavevector list, is added to uu (to aa with lmagnetic_forcing) as an Euler
// step (constant over the step):
//   uu_j += Re[(coef1_j + i coef2_j) fx(x) fy(y) fz(z)],
//   fx = exp(i(kx k1 x + phase)) force/ffnorm sqrt(dt), fy = exp(i ky k1 y),
//   fz = exp(i kz k1 z).
// The host draws each step's wavevector, phase and polarisation angle; a
// one-block kernel builds the 1-D factor tables of the completed step on the
// device (dt is the device's), and a second kernel applies them to every
// interior cell and its periodic ghost images.  For a box in the FP32 pair
// layout running the upwinding kernel variant the tables are built before the
// step's last substep and that substep's update adds the force (helical_force.cuh).
#include <cmath>
#include <type_traits>

#include "dd.cuh"
#include "helical.h"
#include "helical_force.cuh"
#include "mhd_common.cuh"

namespace pcgb {

// ran0 (general.f90:867-889): Lewis-Goodman-Miller minimal standard
// generator with the reference's XOR mask.
static double ran0(int* state) {
  const int ia = 16807, im = 2147483647, iq = 127773, ir = 2836, mask = 123459876;
  *state = *state ^ mask;
  const int k = *state / iq;
  *state = ia * (*state - k * iq) - ir * k;
  if (*state < 0) *state = *state + im;
  const double r = (1.0 / (double)im) * (double)(*state);
  *state = *state ^ mask;
  return r;
}

void helical_record(double cs0, double relhel, double force, const double* kxyz, int nk, double kav, int* state,
                    HelRec* rec) {
  const double pi = 3.14159265358979323846264338327950;
  const double fran1 = ran0(state), fran2 = ran0(state);
  const double phase = pi * (2.0 * fran1 - 1.0);
  const int ik = (int)((double)nk * (0.9999 * fran2) + 1.0);   // 1-based, forcing.f90:1798
  const double kx = kxyz[ik - 1], ky = kxyz[nk + ik - 1], kz = kxyz[2 * nk + ik - 1];
  const double k2 = (kx * kx + ky * ky) + kz * kz;
  const double k = std::sqrt(k2);
  double ex = 1.0, ey = 0.0, ez = 0.0;
  if (ky == 0.0 && kz == 0.0) { ex = 0.0; ey = 1.0; }
  // unit vectors perpendicular to k: e1 = k x e, e2 = k x e1 (forcing.f90:1858-1866)
  double e1[3] = {ky * ez - kz * ey, kz * ex - kx * ez, kx * ey - ky * ex};
  double nrm = (e1[0] * e1[0] + e1[1] * e1[1]) + e1[2] * e1[2];
  for (double& v : e1) v = v / std::sqrt(nrm);
  double e2[3] = {ky * e1[2] - kz * e1[1], kz * e1[0] - kx * e1[2], kx * e1[1] - ky * e1[0]};
  nrm = (e2[0] * e2[0] + e2[1] * e2[1]) + e2[2] * e2[2];
  for (double& v : e2) v = v / std::sqrt(nrm);
  const double phi = ran0(state) * 2.0 * pi;
  ex = std::cos(phi) * e1[0] + std::sin(phi) * e2[0];
  ey = std::cos(phi) * e1[1] + std::sin(phi) * e2[1];
  ez = std::cos(phi) * e1[2] + std::sin(phi) * e2[2];
  const double kde = (kx * ex + ky * ey) + kz * ez;
  const double kex = ky * ez - kz * ey, key = kz * ex - kx * ez, kez = kx * ey - ky * ex;
  const double kkex = ky * kez - kz * key, kkey = kz * kex - kx * kez, kkez = kx * key - ky * kex;
  const double ffnorm = std::sqrt(1.0 + relhel * relhel) * k * std::sqrt(k2 - kde * kde) / std::sqrt(kav * (cs0 * cs0 * cs0));
  rec->kk[0] = kx; rec->kk[1] = ky; rec->kk[2] = kz;
  rec->phase = phase;
  rec->coef1[0] = k * kex; rec->coef1[1] = k * key; rec->coef1[2] = k * kez;
  rec->coef2[0] = relhel * kkex; rec->coef2[1] = relhel * kkey; rec->coef2[2] = relhel * kkez;
  rec->fact0 = force / ffnorm;
}

// tab: coef1[3], coef2[3], 2 spare, then fx, fy, fz as (re, im) pairs.
// pre = 0: after the step (the step just completed, its dt_last); pre = 1: before
// its last substep (the step in progress, its dt, for the fused update).
__global__ void helical_tables_kernel(const HelRec* ring, const PcgbBoxState* S, double* tab, HelGeom g, int pre) {
  const unsigned long long step = pre ? S->nsub / 3ull : S->nsub / 3ull - 1ull;
  const HelRec r = ring[step % (unsigned long long)kHelRing];
  const double fact = __dmul_rn(r.fact0, sqrt(pre ? S->dt : S->dt_last));
  if (threadIdx.x < 3) {
    tab[threadIdx.x] = r.coef1[threadIdx.x];
    tab[3 + threadIdx.x] = r.coef2[threadIdx.x];
  }
  double* fx = tab + 8;   // fx [2 nx], then fy [2 ny] and fz [2 nz], consecutive
  // the same tables rounded to float, after the double ones (for FP32 states)
  float* tabf = reinterpret_cast<float*>(tab + hel_tab_doubles(g.nx, g.ny, g.nz));
  if (threadIdx.x < 3) {
    tabf[threadIdx.x] = (float)r.coef1[threadIdx.x];
    tabf[3 + threadIdx.x] = (float)r.coef2[threadIdx.x];
  }
  for (int i = threadIdx.x; i < g.nx + g.ny + g.nz; i += blockDim.x) {
    double re, im;
    if (i < g.nx) {
      const double x = __dadd_rn(g.x0, __dmul_rn((double)i + g.ox, g.dx));
      const double a = __dadd_rn(__dmul_rn(__dmul_rn(r.kk[0], g.k1), x), r.phase);
      re = __dmul_rn(cos(a), fact);
      im = __dmul_rn(sin(a), fact);
    } else if (i < g.nx + g.ny) {
      const int j = i - g.nx;
      const double y = __dadd_rn(g.y0, __dmul_rn((double)j + g.oy, g.dy));
      const double a = __dmul_rn(__dmul_rn(r.kk[1], g.k1), y);
      re = cos(a);
      im = sin(a);
    } else {
      const int k = i - g.nx - g.ny;
      const double z = __dadd_rn(g.z0, __dmul_rn((double)k + g.oz, g.dz));
      const double a = __dmul_rn(__dmul_rn(r.kk[2], g.k1), z);
      re = cos(a);
      im = sin(a);
    }
    fx[2 * i] = re;   // fx, fy, fz are consecutive
    fx[2 * i + 1] = im;
    tabf[8 + 2 * i] = (float)re;
    tabf[8 + 2 * i + 1] = (float)im;
  }
}


// The interior cell (x, y, z) and its periodic ghost images, as element offsets.
struct CellImages {
  Images ix, iy, iz;
  long long ps, px, xoff;
  __device__ __forceinline__ CellImages(int i, int j, int k, const HelGeom& g)
      : ix(i, g.nx), iy(j, g.ny), iz(k, g.nz), ps(g.ps), px(g.px), xoff(g.xoff) {}
  __device__ __forceinline__ long long at(int a, int b, int e) const {
    return (long long)(iz.v[a] + 3) * ps + (long long)(iy.v[b] + 3) * px + xoff + ix.v[e];
  }
  // store w at every image (the interior cell included)
  template <typename E>
  __device__ __forceinline__ void store(E* p, const E& w) const {
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
      for (int b = 0; b < 2; ++b)
#pragma unroll
        for (int e = 0; e < 2; ++e)
          if (a < iz.n && b < iy.n && e < ix.n) p[at(a, b, e)] = w;
  }
};

// Element access of one layout: the element type E, the slice of component c
// of uu (target 0) or aa (target 1), and the element with v added to the
// target value.  Pair layouts move whole elements; only the target lane changes.
template <int LAYOUT, typename R>
struct HelElem;
template <typename R>
struct HelElem<HEL_F32, R> {
  using E = float;
  static __device__ __forceinline__ E* slice(void* f, const HelGeom& g, int target, int c) {
    return static_cast<E*>(f) + (long long)(target ? g.iax + c : c) * g.fs;
  }
  static __device__ __forceinline__ E add(E e, int, R v) { return radd(e, (float)v); }
};
template <typename R>
struct HelElem<HEL_F64, R> {
  using E = double;
  static __device__ __forceinline__ E* slice(void* f, const HelGeom& g, int target, int c) {
    return static_cast<E*>(f) + (long long)(target ? g.iax + c : c) * g.fs;
  }
  static __device__ __forceinline__ E add(E e, int, R v) { return radd(e, (double)v); }
};
template <typename R>
struct HelElem<HEL_DD, R> {
  using E = float2;   // (hi, lo)
  static __device__ __forceinline__ E* slice(void* f, const HelGeom& g, int target, int c) {
    return static_cast<E*>(f) + (long long)(target ? g.iax + c : c) * g.fs;
  }
  static __device__ __forceinline__ E add(E e, int, R v) {
    const dd w(__dadd_rn((double)e.x + (double)e.y, (double)v));
    return make_float2(w.hi, w.lo);
  }
};
template <typename R>
struct HelElem<HEL_F32_PAIR, R> {
  using E = float2;   // pair (u_c, A_c)
  static __device__ __forceinline__ E* slice(void* f, const HelGeom& g, int, int c) {
    return static_cast<E*>(f) + (long long)c * g.fs;
  }
  static __device__ __forceinline__ E add(E e, int target, R v) {
    if (target) e.y = radd(e.y, (float)v);
    else e.x = radd(e.x, (float)v);
    return e;
  }
};
template <typename R>
struct HelElem<HEL_DD_PAIR, R> {
  using E = float4;   // dd2: (hi.x, hi.y, lo.x, lo.y)
  static __device__ __forceinline__ E* slice(void* f, const HelGeom& g, int, int c) {
    return static_cast<E*>(f) + (long long)c * g.fs;
  }
  static __device__ __forceinline__ E add(E e, int target, R v) {
    if (target) {
      const dd w(__dadd_rn((double)e.y + (double)e.w, (double)v));
      e.y = w.hi; e.w = w.lo;
    } else {
      const dd w(__dadd_rn((double)e.x + (double)e.z, (double)v));
      e.x = w.hi; e.z = w.lo;
    }
    return e;
  }
};

// forcing_hel with lmagnetic_forcing (forcing.f90:318-345, :2289-2311): the
// force goes into aa; uu receives forcing_rhs2 = Re[i coef3 fxyz] with coef3 =
// crosshel k (k x (k x e)) (:1968, :2276-2281), zero for the default crosshel = 0,
// so it is not applied.
// One thread per interior (x, y) and a run of kHelZ planes: x from
// blockIdx.x/threadIdx.x, y = blockIdx.y, planes from blockIdx.z; fx fy is
// formed once per thread.  The forced components of kHelB planes are loaded
// before any is stored (the stores could alias the loads as far as the
// compiler knows), which keeps 3 kHelB loads in flight per thread.  Each value
// is stored at the interior cell and at its periodic ghost images (copies of
// the interior value after a substep).
constexpr int kHelZ = 16, kHelB = 4;

template <int LAYOUT, typename R>
__global__ void helical_apply_kernel(void* f, const double* tab, HelGeom g) {
  using A = HelElem<LAYOUT, R>;
  using E = typename A::E;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y;
  if (i >= g.nx) return;
  const int k0 = blockIdx.z * kHelZ, k1 = min(k0 + kHelZ, g.nz);
  const int target = g.magnetic ? 1 : 0;
  R pr, pi;
  // FP32 layouts read the float copy of the tables (the same values (R)double gives)
  using TT = typename std::conditional<sizeof(R) == 4, float, double>::type;
  const TT* tt = (sizeof(R) == 4) ? reinterpret_cast<const TT*>(tab + hel_tab_doubles(g.nx, g.ny, g.nz))
                                  : reinterpret_cast<const TT*>(tab);
  helical_fxy(tt, g.nx, i, j, pr, pi);   // fx fy
  E* sl[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) sl[c] = A::slice(f, g, target, c);
  for (int kb = k0; kb < k1; kb += kHelB) {
    E e[kHelB][3];
#pragma unroll
    for (int u = 0; u < kHelB; ++u) {
      if (kb + u < k1) {
        const long long cell = (long long)(kb + u + 3) * g.ps + (long long)(j + 3) * g.px + g.xoff + i;
#pragma unroll
        for (int c = 0; c < 3; ++c) e[u][c] = sl[c][cell];
      }
    }
#pragma unroll
    for (int u = 0; u < kHelB; ++u) {
      if (kb + u < k1) {
        const int k = kb + u;
        R fh[3];
        helical_fz(tt, g.nx, g.ny, k, pr, pi, fh);
        const CellImages ci(i, j, k, g);
#pragma unroll
        for (int c = 0; c < 3; ++c) ci.store(sl[c], A::add(e[u][c], target, fh[c]));
      }
    }
  }
}

cudaError_t launch_helical(int layout, void* f, const HelRec* ring, const PcgbBoxState* state, double* tab,
                           const HelGeom& g, cudaStream_t s) {
  if (g.ny > 65535 || g.nz > 65535) return cudaErrorInvalidValue;   // grid y/z limits
  helical_tables_kernel<<<1, 256, 0, s>>>(ring, state, tab, g, 0);
  const dim3 grid((unsigned)((g.nx + 127) / 128), (unsigned)g.ny, (unsigned)((g.nz + kHelZ - 1) / kHelZ));
  switch (layout) {
    case HEL_F32: helical_apply_kernel<HEL_F32, float><<<grid, 128, 0, s>>>(f, tab, g); break;
    case HEL_F64: helical_apply_kernel<HEL_F64, double><<<grid, 128, 0, s>>>(f, tab, g); break;
    case HEL_DD: helical_apply_kernel<HEL_DD, double><<<grid, 128, 0, s>>>(f, tab, g); break;
    case HEL_F32_PAIR: helical_apply_kernel<HEL_F32_PAIR, float><<<grid, 128, 0, s>>>(f, tab, g); break;
    default: helical_apply_kernel<HEL_DD_PAIR, double><<<grid, 128, 0, s>>>(f, tab, g); break;
  }
  return cudaGetLastError();
}

cudaError_t launch_helical_tables_pre(const HelRec* ring, const PcgbBoxState* state, double* tab, const HelGeom& g,
                                      cudaStream_t s) {
  helical_tables_kernel<<<1, 256, 0, s>>>(ring, state, tab, g, 1);
  return cudaGetLastError();
}

}  // namespace pcgb
