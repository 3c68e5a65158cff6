// mhd_common.cuh -- pieces shared by the substep kernel's cell policies.
#pragma once

#include <math.h>
#include "pcgb_box.h"
#include "pcgb_ptx.cuh"
#include "dd.cuh"

namespace pcgb {

enum { MODE_SUBSTEP = 0, MODE_CFL = 1 };

// df of plane z+1 is loaded into registers during plane z; the lines of plane
// z+kDfPrefetch are requested into L2 so that load finds them there (5 planes
// ahead measured best on 1024^3: +7 % against no L2 prefetch, 2 ahead +5 %).
constexpr int kDfPrefetch = 5;

struct LaunchArgs {
  const PcgbBoxDev* boxes;    // [nboxes], sorted by tile0
  int nboxes;
  int total_tiles;            // sum of boxes[b].tiles
  unsigned int* work_counter; // non-null: persistent CTAs pull tiles from this counter
  int mode;                   // MODE_SUBSTEP or MODE_CFL
  unsigned int wait_limit;    // bounded mbarrier wait (iterations)
  int inject_wait_failure;    // test hook: also wait on a barrier nothing arrives on
};

// Williamson (1980) low-storage RK3, timestep.f90:43-44.
__device__ __forceinline__ double rk_alpha(int s) { return s == 0 ? 0.0 : (s == 1 ? -5.0 / 9.0 : -153.0 / 128.0); }
__device__ __forceinline__ double rk_beta(int s) { return s == 0 ? 1.0 / 3.0 : (s == 1 ? 15.0 / 16.0 : 8.0 / 15.0); }

__device__ __forceinline__ float texp(float v) { return expf(v); }
__device__ __forceinline__ double texp(double v) { return exp(v); }
__device__ __forceinline__ float tsqrt(float v) { return sqrtf(v); }
__device__ __forceinline__ double tsqrt(double v) { return sqrt(v); }
__device__ __forceinline__ float tabs(float v) { return fabsf(v); }
__device__ __forceinline__ double tabs(double v) { return fabs(v); }

// Stencil factors and grid constants in the arithmetic type.
template <typename T>
struct Fac {
  T fx, fy, fz;        // (1/60)*dx_1 ...            deriv.f90:127
  T sx, sy, sz;        // dx_1**2 ...                deriv.f90:502
  T mxy, myz, mxz;     // (1/720)*dx_1*dy_1 ...      deriv.f90:1392,1408,1424
  T dx1, dy1, dz1, dxyz2;
};

// Physics constants of one box in type T.
template <typename T>
struct Phys {
  T nu, eta, chi_cp, mu0, mu01, cs20, gamma_m1, gamma1, lnrho0, cv1, lnTT0, two_nu, eta_mu0, gamma_chi;
  T bx, by, bz, fact, fact2, abc_a, abc_b, abc_c, ampl_fc, cdt1, cdtv1;
  T maxdiffus;   // max(diffus_nu, diffus_eta, diffus_chi): constant in space for this physics
};

template <typename T>
__device__ __forceinline__ void make_fac(Fac<T>& F, const PcgbBoxDev& B) {
  F.dx1 = T(B.dx_1); F.dy1 = T(B.dy_1); F.dz1 = T(B.dz_1); F.dxyz2 = T(B.dxyz_2);
  F.fx = T((1.0 / 60.0) * B.dx_1); F.fy = T((1.0 / 60.0) * B.dy_1); F.fz = T((1.0 / 60.0) * B.dz_1);
  F.sx = T(B.dx_1 * B.dx_1); F.sy = T(B.dy_1 * B.dy_1); F.sz = T(B.dz_1 * B.dz_1);
  F.mxy = T(((1.0 / 720.0) * B.dx_1) * B.dy_1);
  F.myz = T(((1.0 / 720.0) * B.dy_1) * B.dz_1);
  F.mxz = T(((1.0 / 720.0) * B.dz_1) * B.dx_1);
}

template <typename T>
__device__ __forceinline__ void make_phys(Phys<T>& P, const PcgbBoxDev& B) {
  P.nu = T(B.nu); P.eta = T(B.eta); P.chi_cp = T(B.chi * B.cpp); P.mu0 = T(B.mu0); P.mu01 = T(B.mu01);
  P.cs20 = T(B.cs20); P.gamma_m1 = T(B.gamma_m1); P.gamma1 = T(B.gamma1); P.lnrho0 = T(B.lnrho0);
  P.cv1 = T(B.cv1); P.lnTT0 = T(B.lnTT0); P.two_nu = T(2.0 * B.nu); P.eta_mu0 = T(B.eta * B.mu0);
  P.gamma_chi = T(B.gamma * B.chi);
  P.bx = T(B.b_ext[0]); P.by = T(B.b_ext[1]); P.bz = T(B.b_ext[2]);
  P.fact = T(B.fact); P.fact2 = T(B.fact2); P.abc_a = T(B.abc_a); P.abc_b = T(B.abc_b); P.abc_c = T(B.abc_c);
  P.ampl_fc = T(B.ampl_fcont_uu); P.cdt1 = T(1.0 / B.cdt); P.cdtv1 = T(1.0 / B.cdtv);
  // viscosity.f90:2436, magnetic.f90:6541, entropy.f90:4905
  double mdiff = B.nu * B.dxyz_2;
  if (B.eta * B.dxyz_2 > mdiff) mdiff = B.eta * B.dxyz_2;
  if (B.lentropy && (B.gamma * B.chi) * B.dxyz_2 > mdiff) mdiff = (B.gamma * B.chi) * B.dxyz_2;
  P.maxdiffus = T(mdiff);
}

// Per-thread FP64 reduction accumulators (FP64 and double-float cells).
struct Acc {
  double v[PCGB_NSLOT];
  __device__ __forceinline__ void reset() {
#pragma unroll
    for (int i = 0; i < PCGB_NSLOT; ++i) v[i] = 0.0;
  }
  __device__ __forceinline__ double get(int q) const { return v[q]; }
};

// Per-thread diagnostic accumulators of the FP32 cells as double-float sums on the
// FP32 pipes: each addend's rounding error is caught exactly (TwoSum) and summed in
// lo, so a column's sum keeps about 48 bits; the maxima are exact in FP32.  (FP64
// arithmetic per cell -- an exp and about forty adds, multiplies and conversions --
// would run at GB300's FP64 rate, 1/64 of FP32's, and took longer than the RHS.)
struct AccF {
  float hi[PCGB_NSLOT], lo[PCGB_NSLOT];
  __device__ __forceinline__ void reset() {
#pragma unroll
    for (int i = 0; i < PCGB_NSLOT; ++i) hi[i] = lo[i] = 0.f;
  }
  __device__ __forceinline__ void add(int q, float x) {
    const float s = __fadd_rn(hi[q], x), bp = __fsub_rn(s, hi[q]);
    const float e = __fadd_rn(__fsub_rn(hi[q], __fsub_rn(s, bp)), __fsub_rn(x, bp));
    hi[q] = s;
    lo[q] = __fadd_rn(lo[q], e);
  }
  __device__ __forceinline__ void add2(int q, float xh, float xl) {   // a double-float addend
    add(q, xh);
    lo[q] = __fadd_rn(lo[q], xl);
  }
  __device__ __forceinline__ void max(int q, float x) { hi[q] = fmaxf(hi[q], x); }
  __device__ __forceinline__ double get(int q) const { return (double)hi[q] + (double)lo[q]; }
};

// One FP32 cell's diagnostic terms, for cells that add them only when their lane is live.
struct DiagF {
  float u2, b2, ekin, rho, divb2, j2, abh, abl;
  __device__ __forceinline__ void add_to(AccF& a) const {
    a.add(PCGB_S_U2SUM, u2);
    a.max(PCGB_S_U2MAX, u2);
    a.add(PCGB_S_B2SUM, b2);
    a.max(PCGB_S_B2MAX, b2);
    a.add(PCGB_S_EKINSUM, ekin);
    a.add(PCGB_S_RHOSUM, rho);
    a.add(PCGB_S_DIVB2SUM, divb2);
    a.add(PCGB_S_J2SUM, j2);
    a.add2(PCGB_S_ABSUM, abh, abl);
  }
};

// Accumulator type of a cell policy: AccF for FP32 arithmetic, Acc otherwise.
template <typename T>
struct AccOf { using type = Acc; };
template <>
struct AccOf<float> { using type = AccF; };

__device__ __forceinline__ bool slot_is_max(int s) {
  return s == PCGB_S_DT1MAX || s == PCGB_S_U2MAX || s == PCGB_S_B2MAX;
}

__device__ __forceinline__ double red_op(int q, double a, double b) {
  return slot_is_max(q) ? ((b > a || b != b) ? b : a) : a + b;
}

// CFL inverse timestep of one cell, set_dt1_max (equ.f90:1872-1905), with
// maxadvec/maxdiffus as assembled by hydro.f90:3500, magnetic.f90:5180,
// noentropy.f90:316 / entropy.f90:3640.
template <typename T>
__device__ __forceinline__ T cfl_dt1(const Phys<T>& P, const Fac<T>& F, const T u[3], const T bb[3], T rho1, T cs2) {
  T advec_uu = (tabs(u[0]) * F.dx1 + tabs(u[1]) * F.dy1) + tabs(u[2]) * F.dz1;
  // NaN-propagating max(0, advec_uu): a non-finite state must reach the dt
  // check (the reference stops on notanumber(p%advec_uu), hydro.f90:3510)
  T maxadvec = (advec_uu > T(0) || advec_uu != advec_uu) ? advec_uu : T(0);
  T t0 = bb[0] * F.dx1, t1 = bb[1] * F.dy1, t2 = bb[2] * F.dz1;
  T advec_va2 = (((t0 * t0 + t1 * t1) + t2 * t2) * P.mu01) * rho1;
  T advec_cs2 = cs2 * F.dxyz2;
  maxadvec = maxadvec + tsqrt((T(0) + advec_va2) + advec_cs2);
  T a = maxadvec * P.cdt1, d = P.maxdiffus * P.cdtv1;
  return tsqrt(a * a + d * d);
}

// Everything a cell needs to know about the current substep.
template <typename T>
struct StepFlags {
  int s;            // substep 0..2
  T alpha, dtb;     // alpha_s, dt*beta_s
  T cinv;           // 1/(dt*beta_{s+1}*alpha_{s+1}) for the compensated carry
  bool comp, read_df, write_df, want_cfl, want_diag;
};

// Periodic images of an interior index: the index itself and, near a face,
// its copy in the ghost zone on the opposite side (boundcond.f90:2387-2531).
// With n >= 6 cells on the axis an index has at most one ghost image (the
// runtime rejects smaller grids).
struct Images {
  int v[2];
  int n;
  __device__ __forceinline__ Images(int i, int nn) {
    v[0] = i; n = 1;
    if (i < 3) v[n++] = i + nn;
    else if (i >= nn - 3) v[n++] = i - nn;
  }
};

// Diagnostic accumulation (FP64) of one cell.
__device__ __forceinline__ void acc_diag(Acc& acc, double u2, double b2, double lnrho, double divb, double j2, double ab) {
  const double rho = exp(lnrho);
  acc.v[PCGB_S_U2SUM] += u2;
  acc.v[PCGB_S_U2MAX] = fmax(acc.v[PCGB_S_U2MAX], u2);
  acc.v[PCGB_S_B2SUM] += b2;
  acc.v[PCGB_S_B2MAX] = fmax(acc.v[PCGB_S_B2MAX], b2);
  acc.v[PCGB_S_EKINSUM] += 0.5 * rho * u2;
  acc.v[PCGB_S_RHOSUM] += rho;
  acc.v[PCGB_S_DIVB2SUM] += divb * divb;
  acc.v[PCGB_S_J2SUM] += j2;
  acc.v[PCGB_S_ABSUM] += ab;
}

}  // namespace pcgb
