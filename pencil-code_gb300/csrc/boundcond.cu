// boundcond.cu -- symmetric and antisymmetric boundary conditions of the
// ghost zones, bc_sym_x / bc_sym_y / bc_sym_z (boundcond.f90:2637-2677,
// 3483-3530, 3842-3900) for the codes 's' (sgn +1), 'a' (sgn -1, boundary value
// set to 0) and 'a2' (sgn -1 relative to the boundary value):
//   lower side: f(n1-i) = sgn f(n1+i)       or  2 f(n1) + sgn f(n1+i)   (a2)
//   upper side: f(n2+i) = sgn f(n2-i)       or  2 f(n2) + sgn f(n2-i)   (a2, x and y)
//                                           or  f(n2) + (f(n2) + sgn f(n2-i))   (a2, z)
// for i = 1..3, over whole ghost planes (the other directions' ghosts included),
// one thread per line of cells normal to the boundary.  FP32 layouts compute in
// float, FP64 in double, the double-float layouts in double rounded back to
// the pair (a copy or a sign change is exact).
#include "boundcond.h"
#include "dd.cuh"
#include "helical.h"

namespace pcgb {

namespace {

// lane access of one element type; R is the arithmetic type
template <int L>
struct BcElem;
template <>
struct BcElem<HEL_F32> {
  using E = float; using R = float; static constexpr int NL = 1;
  static __device__ __forceinline__ R get(const E& e, int) { return e; }
  static __device__ __forceinline__ void set(E& e, int, R v) { e = v; }
};
template <>
struct BcElem<HEL_F64> {
  using E = double; using R = double; static constexpr int NL = 1;
  static __device__ __forceinline__ R get(const E& e, int) { return e; }
  static __device__ __forceinline__ void set(E& e, int, R v) { e = v; }
};
template <>
struct BcElem<HEL_DD> {
  using E = float2; using R = double; static constexpr int NL = 1;   // (hi, lo)
  static __device__ __forceinline__ R get(const E& e, int) { return (double)e.x + (double)e.y; }
  static __device__ __forceinline__ void set(E& e, int, R v) { const dd w(v); e = make_float2(w.hi, w.lo); }
};
template <>
struct BcElem<HEL_F32_PAIR> {
  using E = float2; using R = float; static constexpr int NL = 2;
  static __device__ __forceinline__ R get(const E& e, int l) { return l ? e.y : e.x; }
  static __device__ __forceinline__ void set(E& e, int l, R v) { if (l) e.y = v; else e.x = v; }
};
template <>
struct BcElem<HEL_DD_PAIR> {
  using E = float4; using R = double; static constexpr int NL = 2;   // (hi.x, hi.y, lo.x, lo.y)
  static __device__ __forceinline__ R get(const E& e, int l) {
    return l ? (double)e.y + (double)e.w : (double)e.x + (double)e.z;
  }
  static __device__ __forceinline__ void set(E& e, int l, R v) {
    const dd w(v);
    if (l) { e.y = w.hi; e.w = w.lo; } else { e.x = w.hi; e.z = w.lo; }
  }
};

__device__ __forceinline__ float badd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double badd(double a, double b) { return __dadd_rn(a, b); }

// codes of slice s, lane l, side d
struct BcCodes {
  int code[8][2][2];
};

struct BcGeom {
  int nx, ny, nz, px, my, mz, xoff;
  long long ps, fs;
};

template <int L>
__global__ void boundcond_kernel(void* f, void* carry, BcCodes c, BcGeom g, int dir, long long npos) {
  using A = BcElem<L>;
  using E = typename A::E;
  using R = typename A::R;
  const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (q >= npos) return;
  const int slice = (int)(blockIdx.y >> 1), side = (int)(blockIdx.y & 1u);
  const int mx = g.nx + 6;
  long long base, st;
  int n;
  if (dir == 0) {          // a row: y in [0, my), z in [0, mz)
    const int y = (int)(q % g.my), z = (int)(q / g.my);
    base = (long long)z * g.ps + (long long)y * g.px + g.xoff;
    st = 1; n = g.nx;
  } else if (dir == 1) {   // a column in y: x over the ghosted row, z in [0, mz)
    const int xi = (int)(q % mx), z = (int)(q / mx);
    base = (long long)z * g.ps + 3LL * g.px + (g.xoff - 3 + xi);
    st = g.px; n = g.ny;
  } else {                 // a column in z: x over the ghosted row, y in [0, my)
    const int xi = (int)(q % mx), y = (int)(q / mx);
    base = 3LL * g.ps + (long long)y * g.px + (g.xoff - 3 + xi);
    st = g.ps; n = g.nz;
  }
  E* p = static_cast<E*>(f) + (long long)slice * g.fs + base;   // interior index 0 of the line
  const long long b0 = side ? (long long)(n - 1) * st : 0;       // boundary point n1 or n2
  const long long in = side ? -st : st;                          // toward the interior
  const E e0 = p[b0];
  E ev[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) ev[i] = p[b0 + (i + 1) * in];
  E gh[3] = {e0, e0, e0};
  E eb = e0;
  bool zero_b = false;
#pragma unroll
  for (int l = 0; l < A::NL; ++l) {
    const int code = c.code[slice][l][side];
    const R v0 = A::get(e0, l);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      const R vi = A::get(ev[i], l);
      R gv;
      if (code == PCGB_BC_ASYM2) {
        if (dir == 2 && side) gv = badd(v0, badd(v0, -vi));   // bc_sym_z top, :3886
        else gv = badd(R(2) * v0, -vi);                        // 2 f(n1) + sgn f(n1+i)
      } else if (code == PCGB_BC_ASYM) {
        gv = -vi;
      } else {
        gv = vi;   // 's' (and the unused pad lane)
      }
      A::set(gh[i], l, gv);
    }
    if (code == PCGB_BC_ASYM) {   // set bdry value=0 (indep of initcond)
      A::set(eb, l, R(0));
      zero_b = true;
    }
  }
#pragma unroll
  for (int i = 0; i < 3; ++i) p[b0 - (i + 1) * in] = gh[i];
  if (zero_b) {
    p[b0] = eb;
    if (carry) {   // FP32 compensated state at a step boundary: the value is f + carry, both 0
      E* cp = static_cast<E*>(carry) + (long long)slice * g.fs + base + b0;
      E ce = *cp;
#pragma unroll
      for (int l = 0; l < A::NL; ++l)
        if (c.code[slice][l][side] == PCGB_BC_ASYM) A::set(ce, l, R(0));
      *cp = ce;
    }
  }
}

}  // namespace

cudaError_t launch_boundconds(int layout, void* f, void* carry, const pcgb_params& p, int nx, int ny, int nz, int px,
                              int my, int mz, int xoff, long long ps, long long fs, int nf, cudaStream_t s) {
  const bool pairs = (layout == HEL_F32_PAIR || layout == HEL_DD_PAIR);
  const int nslice = pairs ? 4 : nf;
  const int iax = nf - 3;
  BcGeom g{nx, ny, nz, px, my, mz, xoff, ps, fs};
  const int mx = nx + 6;
  for (int dir = 0; dir < 3; ++dir) {
    if (axis_periodic(p, dir)) continue;
    BcCodes c = {};
    for (int sl = 0; sl < nslice; ++sl)
      for (int l = 0; l < 2; ++l) {
        // field of slice sl, lane l: field-major slice = field; pairs (ux,ax) (uy,ay) (uz,az) (lnrho,ss|pad)
        int fld = -1;
        if (!pairs) fld = (l == 0) ? sl : -1;
        else if (sl < 3) fld = (l == 0) ? sl : iax + sl;
        else fld = (l == 0) ? 3 : (nf == 8 ? 4 : -1);
        for (int d = 0; d < 2; ++d) c.code[sl][l][d] = (fld >= 0) ? p.bc[dir][fld][d] : PCGB_BC_SYM;
      }
    const long long npos = dir == 0 ? (long long)my * mz : dir == 1 ? (long long)mx * mz : (long long)mx * my;
    const dim3 grid((unsigned)((npos + 255) / 256), (unsigned)(2 * nslice));
    switch (layout) {
      case HEL_F32: boundcond_kernel<HEL_F32><<<grid, 256, 0, s>>>(f, carry, c, g, dir, npos); break;
      case HEL_F64: boundcond_kernel<HEL_F64><<<grid, 256, 0, s>>>(f, carry, c, g, dir, npos); break;
      case HEL_DD: boundcond_kernel<HEL_DD><<<grid, 256, 0, s>>>(f, carry, c, g, dir, npos); break;
      case HEL_F32_PAIR: boundcond_kernel<HEL_F32_PAIR><<<grid, 256, 0, s>>>(f, carry, c, g, dir, npos); break;
      default: boundcond_kernel<HEL_DD_PAIR><<<grid, 256, 0, s>>>(f, carry, c, g, dir, npos); break;
    }
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

}  // namespace pcgb
