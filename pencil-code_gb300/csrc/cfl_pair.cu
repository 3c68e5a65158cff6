// cfl_pair.cu -- the CFL pass of the FP32 packed-pair layout as a light kernel
// of its own: set_dt1_max (equ.f90:1872-1905) over the current f and set_dt
// (sub.f90:4247) on the device, as the substep kernel's MODE_CFL does it, for
// the timestep taken from the current state (dt = 0 in run.in).
//
// The fused substep kernel stages every field plane by plane for the RHS; the
// CFL condition needs only u, lnrho, [ss] and B = curl A, so its pass through
// that pipeline is latency bound at one CTA per SM.  Here one thread owns an
// (x, y) column of a z-chunk: the z-derivatives of A_x and A_y come from
// 7-plane register windows, the x- and y-derivatives of A from neighbouring
// elements read through L1 (ghost zones are the periodic images kept by the
// substep kernel); each thread requests its column kPF planes ahead into L2,
// so the loads of a plane meet L2 rather than HBM latency.  The derivative
// arithmetic is PairCell::St::der's on the A lanes, so the per-cell values,
// and the maximum, are the fused pass's.
#include "cell_pair.cuh"
#include "cfl_pair.h"

namespace pcgb {

namespace {

constexpr int kTX = 32, kTY = 8, kZC = 64;   // block (x, y) and z-chunk
constexpr int kThreads = kTX * kTY;
constexpr int kPF = 4;   // the column's lines are requested into L2 this many planes ahead

// der_main (deriv.f90:127-129) on single values, in PairCell::St::der's order
__device__ __forceinline__ float der1(float m3, float m2, float m1, float p1, float p2, float p3, float fac) {
  const float a = __fsub_rn(p1, m1), b = __fsub_rn(p2, m2), c = __fsub_rn(p3, m3);
  const float t = __fadd_rn(__fmaf_rn(-9.f, b, __fmul_rn(45.f, a)), c);
  return __fmul_rn(fac, t);
}

__device__ __forceinline__ float nanmax(float a, float b) { return (b > a || b != b) ? b : a; }

template <int NF>
__global__ void __launch_bounds__(kThreads, 4) cfl_pair_kernel(const PcgbBoxDev* __restrict__ Bp, double* partial,
                                                             unsigned int* done) {
  const PcgbBoxDev& B = *Bp;
  PcgbBoxState* const S = B.state;
  const unsigned long long nsub = __ldcg(&S->nsub);
  const float2* const f = static_cast<const float2*>(B.f[nsub & 1ull]);
  Fac<float> F;
  make_fac(F, B);
  Phys<float> P;
  make_phys(P, B);
  const bool iso = B.isothermal != 0;
  constexpr bool ENTROPY = (NF == 8);

  const int x = blockIdx.x * kTX + threadIdx.x, y = blockIdx.y * kTY + threadIdx.y;
  const int z0 = blockIdx.z * kZC, z1 = min(z0 + kZC, B.nz);
  float dt1max = 0.f;
  if (x < B.nx && y < B.ny) {
    const long long fs = B.fs, ps = B.ps, px = B.px;
    // element (x, y) of pair 0 on array plane 0; array plane of interior z is z + 3
    const float2* const col = f + (long long)(y + 3) * px + B.xoff + x;
    const float2* const col1 = col + fs;
    // windows of A_x (pair 0, lane y) and A_y (pair 1, lane y): w[k] is array plane z + k
    float ax[7], ay[7];
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      ax[k] = __ldg(&col[(long long)(z0 + k) * ps].y);
      ay[k] = __ldg(&col1[(long long)(z0 + k) * ps].y);
    }
    for (int z = z0; z < z1; ++z) {
      if (z + 3 + kPF < B.mz) {   // every pair of this column, kPF planes ahead
#pragma unroll
        for (int p = 0; p < 4; ++p) prefetch_l2(col + p * fs + (long long)(z + 3 + kPF) * ps);
      }
      ax[6] = __ldg(&col[(long long)(z + 6) * ps].y);
      ay[6] = __ldg(&col1[(long long)(z + 6) * ps].y);
      const float2* const q = col + (long long)(z + 3) * ps;   // this cell, pair 0
      const float2 c0 = __ldg(q), c1 = __ldg(q + fs), c2 = __ldg(q + 2 * fs), c3 = __ldg(q + 3 * fs);
      const float2* const q1 = q + fs;
      const float2* const q2 = q + 2 * fs;
      // x-derivatives: A_y (pair 1), A_z (pair 2); y-derivatives: A_x (pair 0), A_z (pair 2)
      const float ay_x = der1(__ldg(&q1[-3].y), __ldg(&q1[-2].y), __ldg(&q1[-1].y), __ldg(&q1[1].y),
                              __ldg(&q1[2].y), __ldg(&q1[3].y), F.fx);
      const float az_x = der1(__ldg(&q2[-3].y), __ldg(&q2[-2].y), __ldg(&q2[-1].y), __ldg(&q2[1].y),
                              __ldg(&q2[2].y), __ldg(&q2[3].y), F.fx);
      const float ax_y = der1(__ldg(&q[-3 * px].y), __ldg(&q[-2 * px].y), __ldg(&q[-px].y), __ldg(&q[px].y),
                              __ldg(&q[2 * px].y), __ldg(&q[3 * px].y), F.fy);
      const float az_y = der1(__ldg(&q2[-3 * px].y), __ldg(&q2[-2 * px].y), __ldg(&q2[-px].y), __ldg(&q2[px].y),
                              __ldg(&q2[2 * px].y), __ldg(&q2[3 * px].y), F.fy);
      const float ax_z = der1(ax[0], ax[1], ax[2], ax[4], ax[5], ax[6], F.fz);
      const float ay_z = der1(ay[0], ay[1], ay[2], ay[4], ay[5], ay[6], F.fz);
      const float uu[3] = {c0.x, c1.x, c2.x};
      const float bb[3] = {az_y - ay_z, ax_z - az_x, ay_x - ax_y};   // curl A (PairCell::Tile::cfl)
      const float d = cell_cfl_only<float, NF>(P, F, uu, c3.x, ENTROPY ? c3.y : 0.f, bb, iso);
      dt1max = (d > dt1max || d != d) ? d : dt1max;
#pragma unroll
      for (int k = 0; k < 6; ++k) {
        ax[k] = ax[k + 1];
        ay[k] = ay[k + 1];
      }
    }
  }

  // block maximum (NaN-propagating), then the last block reduces the blocks
  __shared__ float wmax[kThreads / 32];
  __shared__ int last;
  const int tid = threadIdx.y * kTX + threadIdx.x;
  float v = dt1max;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = nanmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  if ((tid & 31) == 0) wmax[tid >> 5] = v;
  __syncthreads();
  const unsigned int nblk = gridDim.x * gridDim.y * gridDim.z;
  const unsigned int blk = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
  if (tid == 0) {
    float m = wmax[0];
    for (int w = 1; w < kThreads / 32; ++w) m = nanmax(m, wmax[w]);
    partial[blk] = (double)m;
    __threadfence();
    last = (atomicAdd(done, 1u) == nblk - 1u) ? 1 : 0;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  double r = 0.0;
  for (unsigned int i = tid; i < nblk; i += kThreads) r = red_op(PCGB_S_DT1MAX, r, __ldcg(&partial[i]));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) r = red_op(PCGB_S_DT1MAX, r, __shfl_xor_sync(0xffffffffu, r, o));
  __shared__ double wr[kThreads / 32];
  if ((tid & 31) == 0) wr[tid >> 5] = r;
  __syncthreads();
  if (tid == 0) {
    double m = wr[0];
    for (int w = 1; w < kThreads / 32; ++w) m = red_op(PCGB_S_DT1MAX, m, wr[w]);
    const double dtn = 1.0 / m;   // set_dt, sub.f90:4247
    if (!(dtn > 0.0) || !isfinite(dtn)) atomicOr(&S->err, PCGB_ERR_DT | PCGB_ERR_NONFINITE);
    if (B.dt_mode != PCGB_DT_FIXED) {
      S->dt = dtn;
      S->dt_next = dtn;
    }
    *done = 0u;
    __threadfence();
  }
}

}  // namespace

size_t cfl_pair_blocks(int nx, int ny, int nz) {
  return (size_t)((nx + kTX - 1) / kTX) * (size_t)((ny + kTY - 1) / kTY) * (size_t)((nz + kZC - 1) / kZC);
}

cudaError_t launch_cfl_pair(const PcgbBoxDev* dbox, int nf, int nx, int ny, int nz, double* partial,
                            unsigned int* done, cudaStream_t s) {
  const dim3 grid((unsigned)((nx + kTX - 1) / kTX), (unsigned)((ny + kTY - 1) / kTY),
                  (unsigned)((nz + kZC - 1) / kZC));
  if (grid.y > 65535u || grid.z > 65535u) return cudaErrorInvalidValue;
  const dim3 block(kTX, kTY);
  if (nf == 8) cfl_pair_kernel<8><<<grid, block, 0, s>>>(dbox, partial, done);
  else cfl_pair_kernel<7><<<grid, block, 0, s>>>(dbox, partial, done);
  return cudaGetLastError();
}

}  // namespace pcgb
