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

// Two double-float values in one 16-byte element, hi = (a.hi, b.hi) and
// lo = (a.lo, b.lo): the algorithms above run on both at once with packed
// f32x2 instructions (FADD2/FMUL2/FFMA2), lane by lane the same operations,
// so each lane's result equals the scalar dd result bit for bit.
struct __align__(16) dd2 {
  float2 hi, lo;
};

__device__ __forceinline__ float2 f2neg(float2 a) { return make_float2(-a.x, -a.y); }

__device__ __forceinline__ void dd2_two_sum(float2 a, float2 b, float2& s, float2& e) {
  s = __fadd2_rn(a, b);
  const float2 bb = __fadd2_rn(s, f2neg(a));
  e = __fadd2_rn(__fadd2_rn(a, f2neg(__fadd2_rn(s, f2neg(bb)))), __fadd2_rn(b, f2neg(bb)));
}

__device__ __forceinline__ void dd2_fast_two_sum(float2 a, float2 b, float2& s, float2& e) {
  s = __fadd2_rn(a, b);
  e = __fadd2_rn(b, f2neg(__fadd2_rn(s, f2neg(a))));
}

__device__ __forceinline__ dd2 operator+(dd2 x, dd2 y) {
  float2 sh, sl;
  dd2_two_sum(x.hi, y.hi, sh, sl);
  const float2 w = __fadd2_rn(sl, __fadd2_rn(x.lo, y.lo));
  dd2 z;
  dd2_fast_two_sum(sh, w, z.hi, z.lo);
  return z;
}

__device__ __forceinline__ dd2 operator-(dd2 x) { return dd2{f2neg(x.hi), f2neg(x.lo)}; }
__device__ __forceinline__ dd2 operator-(dd2 x, dd2 y) { return x + dd2{f2neg(y.hi), f2neg(y.lo)}; }

__device__ __forceinline__ dd2 operator*(dd2 x, dd2 y) {
  const float2 ch = __fmul2_rn(x.hi, y.hi);
  const float2 cl1 = __ffma2_rn(x.hi, y.hi, f2neg(ch));
  const float2 tl0 = __fmul2_rn(x.lo, y.lo);
  const float2 tl1 = __ffma2_rn(x.hi, y.lo, tl0);
  const float2 cl2 = __ffma2_rn(x.lo, y.hi, tl1);
  const float2 cl3 = __fadd2_rn(cl1, cl2);
  dd2 z;
  dd2_fast_two_sum(ch, cl3, z.hi, z.lo);
  return z;
}

__device__ __forceinline__ dd2 dd2_scale(dd2 x, float c) {
  const float2 cc = make_float2(c, c);
  const float2 ch = __fmul2_rn(x.hi, cc);
  const float2 cl1 = __ffma2_rn(x.hi, cc, f2neg(ch));
  const float2 cl3 = __ffma2_rn(x.lo, cc, cl1);
  dd2 z;
  dd2_fast_two_sum(ch, cl3, z.hi, z.lo);
  return z;
}

__device__ __forceinline__ dd2 dd2_splat(dd v) { return dd2{make_float2(v.hi, v.hi), make_float2(v.lo, v.lo)}; }
__device__ __forceinline__ dd dd2_lane0(dd2 x) { return dd(x.hi.x, x.lo.x); }
__device__ __forceinline__ dd dd2_lane1(dd2 x) { return dd(x.hi.y, x.lo.y); }
__device__ __forceinline__ dd2 dd2_pack(dd a, dd b) { return dd2{make_float2(a.hi, b.hi), make_float2(a.lo, b.lo)}; }

// Weight times value: the FP32/FP64 paths multiply by T(c); double-float
// values use the cheaper product with an exact FP32 weight.
template <typename T>
__device__ __forceinline__ T wmul(int c, T x) { return T(c) * x; }
template <>
__device__ __forceinline__ dd wmul<dd>(int c, dd x) { return dd_scale(x, (float)c); }

}  // namespace pcgb
