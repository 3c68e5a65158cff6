// dd.cuh -- double-float arithmetic for FP64-class accuracy on the FP32 pipes.
//
// GB300 executes FP64 at 1/64 of its FP32 rate (1.2 vs ~70 TFLOP/s measured),
// which makes the native FP64 substep FP64-pipe bound.  A double-float value
// x = hi + lo keeps two FP32 numbers with |lo| <= ulp(hi)/2, i.e. a 48-bit
// significand (relative representation error <= 2^-49 against FP64's 2^-53),
// and computes on the FP32 pipes with error-free transformations:
//   TwoSum   -- Knuth, TAOCP vol. 2, sec. 4.2.2 (6 operations, any order of magnitudes)
//   Fast2Sum -- Dekker (1971), requires |a| >= |b| or a == 0 (3 operations)
//   TwoProd  -- product and its exact error with one FMA
// and the pair algorithms analysed in Joldes, Muller, Popescu, "Tight and
// rigorous error bounds for basic building blocks of double-word arithmetic",
// ACM TOMS 44(2), 2017: pair addition (below), DWTimesDW with FMA (Alg. 12,
// relative error <= 5u^2) and DWTimesFP (Alg. 9, <= 2u^2), u = 2^-24.  exp
// and sqrt go through native FP64 (one or two calls per cell).
#pragma once

#include <math.h>

namespace pcgb {

struct __align__(8) dd {
  float hi, lo;
  dd() = default;
  __host__ __device__ constexpr dd(float h, float l) : hi(h), lo(l) {}
  __host__ __device__ constexpr dd(int v) : hi((float)v), lo(0.f) {}   // |v| < 2^24: exact
  __host__ __device__ dd(double v) : hi((float)v), lo((float)(v - (double)(float)v)) {}
  __host__ __device__ explicit operator double() const { return (double)hi + (double)lo; }
};

template <typename T>
struct is_dd { static constexpr bool value = false; };
template <>
struct is_dd<dd> { static constexpr bool value = true; };

// s + e == a + b exactly (round-to-nearest; the _rn intrinsics keep the
// compiler from contracting or reordering)
__device__ __forceinline__ void dd_two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

__device__ __forceinline__ void dd_fast_two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  e = __fsub_rn(b, __fsub_rn(s, a));
}

// Pair addition: exact TwoSum of the high parts, low parts added in FP32,
// one Fast2Sum (Dekker's addition; the "sloppy" form of Joldes et al.).  Its
// relative error is not bounded when x ~ -y, but the low parts then cancel
// to within u|x|, so the absolute error stays near u^2 |x|: the 100-step
// parity against the FP64 oracle is the same as with AccurateDWPlusDW
// (Alg. 6, two TwoSums and two Fast2Sums), at 11 instead of 20 operations.
__device__ __forceinline__ dd operator+(dd x, dd y) {
  float sh, sl;
  dd_two_sum(x.hi, y.hi, sh, sl);
  const float w = __fadd_rn(sl, __fadd_rn(x.lo, y.lo));
  dd z;
  dd_fast_two_sum(sh, w, z.hi, z.lo);
  return z;
}

__device__ __forceinline__ dd operator-(dd x) { return dd(-x.hi, -x.lo); }
__device__ __forceinline__ dd operator-(dd x, dd y) { return x + dd(-y.hi, -y.lo); }

__device__ __forceinline__ dd operator*(dd x, dd y) {   // DWTimesDW with FMA
  const float ch = __fmul_rn(x.hi, y.hi);
  const float cl1 = __fmaf_rn(x.hi, y.hi, -ch);
  const float tl0 = __fmul_rn(x.lo, y.lo);
  const float tl1 = __fmaf_rn(x.hi, y.lo, tl0);
  const float cl2 = __fmaf_rn(x.lo, y.hi, tl1);
  const float cl3 = __fadd_rn(cl1, cl2);
  dd z;
  dd_fast_two_sum(ch, cl3, z.hi, z.lo);
  return z;
}

// x * c for a float c (integer stencil weights)
__device__ __forceinline__ dd dd_scale(dd x, float c) {   // DWTimesFP
  const float ch = __fmul_rn(x.hi, c);
  const float cl1 = __fmaf_rn(x.hi, c, -ch);
  const float cl3 = __fmaf_rn(x.lo, c, cl1);
  dd z;
  dd_fast_two_sum(ch, cl3, z.hi, z.lo);
  return z;
}

__device__ __forceinline__ bool operator>(dd a, dd b) { return a.hi > b.hi || (a.hi == b.hi && a.lo > b.lo); }
__device__ __forceinline__ bool operator!=(dd a, dd b) { return a.hi != b.hi || a.lo != b.lo; }

__device__ __forceinline__ dd texp(dd v) { return dd(exp((double)v)); }
__device__ __forceinline__ dd tsqrt(dd v) { return dd(sqrt((double)v)); }
__device__ __forceinline__ dd tabs(dd v) { return v.hi < 0.f ? -v : v; }

// Weight times value: the FP32/FP64 paths multiply by T(c); double-float
// values use the cheaper product with an exact FP32 weight.
template <typename T>
__device__ __forceinline__ T wmul(int c, T x) { return T(c) * x; }
template <>
__device__ __forceinline__ dd wmul<dd>(int c, dd x) { return dd_scale(x, (float)c); }

}  // namespace pcgb
