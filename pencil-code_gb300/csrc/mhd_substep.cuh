// mhd_substep.cuh -- the fused RK substep kernel (sm_103a).
//
// One launch advances every box of a batch by one 2N-RK3 substep
// (timestep.f90:77-202): it evaluates the compressible-MHD right-hand side of
// pde() (equ.f90:1386 rhs_cpu: hydro duu_dt, density dlnrho_dt, energy
// denergy_dt, magnetic daa_dt) with the 6th-order der/der2/bidiagonal derij
// stencils (deriv.f90:89,472,1367), then applies df = alpha*df + RHS and
// f_out = f_in + dt*beta*df, writing f_out's periodic ghost cells in the
// same pass (boundcond.f90:2387-2531).
//
// Work decomposition: a tile is TX x TY columns of one box swept over zd
// z-planes.  All NF fields of one ghosted plane (TX+8) x (TY+6) are staged
// into a ring of RING shared-memory slots by one 4-D TMA load per plane,
// tracked by one mbarrier per slot; the output plane z reads planes z-3..z+3.
//
// Reductions (CFL inverse timestep and the diagnostics) are accumulated in
// FP64, written per tile, and reduced in fixed tile order by the last CTA of
// each box, which also advances the box's step bookkeeping (substep index,
// time, dt) in device memory.  A time loop is therefore a sequence of
// identical launches.
#pragma once

#include <math.h>
#include "pcgb_box.h"
#include "pcgb_ptx.cuh"

namespace pcgb {

enum { MODE_SUBSTEP = 0, MODE_CFL = 1 };

struct LaunchArgs {
  const PcgbBoxDev* boxes;    // [nboxes], sorted by tile0
  int nboxes;
  int total_tiles;            // sum of boxes[b].tiles
  unsigned int* work_counter; // non-null: persistent CTAs pull tiles from this counter
  int mode;                   // MODE_SUBSTEP or MODE_CFL
  unsigned int wait_limit;    // bounded mbarrier wait (iterations)
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

template <typename T, int NF, int TX, int TY, int RING>
struct TileCfg {
  static constexpr int NT = TX * TY;
  static constexpr int NWARP = (NT + 31) / 32;
  static constexpr int BW = TX + 8;   // TMA box width: x0-4 .. x0+TX+4
  static constexpr int BH = TY + 6;   // TMA box rows:  y0-3 .. y0+TY+3
  static constexpr int FO = BW * BH;  // field stride inside a slot
  static constexpr int PLANE_BYTES = NF * FO * (int)sizeof(T);
  static constexpr int SLOT_BYTES = (PLANE_BYTES + 127) / 128 * 128;
  static constexpr int RED_OFF = RING * SLOT_BYTES + RING * 8;
  static constexpr int SMEM_BYTES = RED_OFF + NWARP * PCGB_NSLOT * 8 + 64;
};

// Stencil coefficients and grid factors in the arithmetic type.
template <typename T>
struct Fac {
  T fx, fy, fz;        // (1/60)*dx_1 ...            deriv.f90:127
  T sx, sy, sz;        // dx_1**2 ...                deriv.f90:502
  T mxy, myz, mxz;     // (1/720)*dx_1*dy_1 ...      deriv.f90:1392,1408,1424
  T dx1, dy1, dz1, dxyz2;
};

template <typename T, int NF, int TX, int TY, int RING>
struct Stencil {
  using C = TileCfg<T, NF, TX, TY, RING>;
  const T* pl[7];   // planes z-3..z+3, each at (field 0, row ty+3, col tx+4)
  Fac<T> F;

  __device__ __forceinline__ T v(int dz, int k, int dy, int dx) const {
    return pl[dz + 3][k * C::FO + dy * C::BW + dx];
  }
  // der_main, deriv.f90:127-129 (x), :140-142 (y), :158-160 (z)
  __device__ __forceinline__ T der(int k, int j) const {
    if (j == 0)
      return F.fx * ((T(45) * (v(0, k, 0, 1) - v(0, k, 0, -1)) - T(9) * (v(0, k, 0, 2) - v(0, k, 0, -2))) +
                      (v(0, k, 0, 3) - v(0, k, 0, -3)));
    if (j == 1)
      return F.fy * ((T(45) * (v(0, k, 1, 0) - v(0, k, -1, 0)) - T(9) * (v(0, k, 2, 0) - v(0, k, -2, 0))) +
                      (v(0, k, 3, 0) - v(0, k, -3, 0)));
    return F.fz * ((T(45) * (v(1, k, 0, 0) - v(-1, k, 0, 0)) - T(9) * (v(2, k, 0, 0) - v(-2, k, 0, 0))) +
                    (v(3, k, 0, 0) - v(-3, k, 0, 0)));
  }
  // der2_main 'standard', deriv.f90:39-41, :502-506
  __device__ __forceinline__ T der2(int k, int j) const {
    const T c0 = T(-490.0 / 180.0), c1 = T(270.0 / 180.0), c2 = T(-27.0 / 180.0), c3 = T(2.0 / 180.0);
    const T f0 = v(0, k, 0, 0);
    if (j == 0)
      return F.sx * (((c0 * f0 + c1 * (v(0, k, 0, 1) + v(0, k, 0, -1))) + c2 * (v(0, k, 0, 2) + v(0, k, 0, -2))) +
                      c3 * (v(0, k, 0, 3) + v(0, k, 0, -3)));
    if (j == 1)
      return F.sy * (((c0 * f0 + c1 * (v(0, k, 1, 0) + v(0, k, -1, 0))) + c2 * (v(0, k, 2, 0) + v(0, k, -2, 0))) +
                      c3 * (v(0, k, 3, 0) + v(0, k, -3, 0)));
    return F.sz * (((c0 * f0 + c1 * (v(1, k, 0, 0) + v(-1, k, 0, 0))) + c2 * (v(2, k, 0, 0) + v(-2, k, 0, 0))) +
                    c3 * (v(3, k, 0, 0) + v(-3, k, 0, 0)));
  }
  // derij_main bidiagonal, deriv.f90:1387-1447; (a,b) with a<b: 0=x,1=y,2=z
  __device__ __forceinline__ T derij(int k, int a, int b) const {
    T t[3];
#pragma unroll
    for (int d = 1; d <= 3; ++d) {
      if (a == 0 && b == 1)       // f(l+d,m+d) - f(l-d,m+d) + f(l-d,m-d) - f(l+d,m-d)
        t[d - 1] = ((v(0, k, d, d) - v(0, k, d, -d)) + v(0, k, -d, -d)) - v(0, k, -d, d);
      else if (a == 1 && b == 2)  // f(m+d,n+d) - f(m+d,n-d) + f(m-d,n-d) - f(m-d,n+d)
        t[d - 1] = ((v(d, k, d, 0) - v(-d, k, d, 0)) + v(-d, k, -d, 0)) - v(d, k, -d, 0);
      else                        // f(l+d,n+d) - f(l-d,n+d) + f(l-d,n-d) - f(l+d,n-d)
        t[d - 1] = ((v(d, k, 0, d) - v(d, k, 0, -d)) + v(-d, k, 0, -d)) - v(-d, k, 0, d);
    }
    const T fac = (a == 0 && b == 1) ? F.mxy : ((a == 1 && b == 2) ? F.myz : F.mxz);
    return fac * ((T(270) * t[0] - T(27) * t[1]) + T(2) * t[2]);
  }
};

// Per-thread FP64 reduction accumulators.
struct Acc {
  double v[PCGB_NSLOT];
  __device__ __forceinline__ void reset() {
#pragma unroll
    for (int i = 0; i < PCGB_NSLOT; ++i) v[i] = 0.0;
  }
};

__device__ __forceinline__ bool slot_is_max(int s) {
  return s == PCGB_S_DT1MAX || s == PCGB_S_U2MAX || s == PCGB_S_B2MAX;
}

// Physics constants of one box in type T.
template <typename T>
struct Phys {
  T nu, eta, chi_cp, mu0, mu01, cs20, gamma_m1, gamma1, lnrho0, cv1, lnTT0, two_nu, eta_mu0, gamma_chi;
  T bx, by, bz, fact, fact2, abc_a, abc_b, abc_c, ampl_fc, cdt1, cdtv1;
};

// Diagonal-free CFL inverse timestep of one cell, set_dt1_max (equ.f90:1872-1905)
// with maxadvec/maxdiffus as assembled by hydro.f90:3500, magnetic.f90:5180,
// noentropy.f90:316 / entropy.f90:3640, viscosity.f90:2436, magnetic.f90:6541,
// entropy.f90:4905.
template <typename T>
__device__ __forceinline__ T cfl_dt1(const Phys<T>& P, const Fac<T>& F, const T u[3], const T bb[3], T rho1, T cs2,
                                     T maxdiffus) {
  T advec_uu = (tabs(u[0]) * F.dx1 + tabs(u[1]) * F.dy1) + tabs(u[2]) * F.dz1;
  T maxadvec = advec_uu > T(0) ? advec_uu : T(0);
  T t0 = bb[0] * F.dx1, t1 = bb[1] * F.dy1, t2 = bb[2] * F.dz1;
  T advec_va2 = (((t0 * t0 + t1 * t1) + t2 * t2) * P.mu01) * rho1;
  T advec_cs2 = cs2 * F.dxyz2;
  maxadvec = maxadvec + tsqrt((T(0) + advec_va2) + advec_cs2);
  T a = maxadvec * P.cdt1, d = maxdiffus * P.cdtv1;
  return tsqrt(a * a + d * d);
}

template <typename T, int NF, int TX, int TY, int RING, int MINB>
__global__ void __launch_bounds__(TX* TY, MINB) mhd_substep_kernel(LaunchArgs args) {
  using C = TileCfg<T, NF, TX, TY, RING>;
  constexpr int IUX = 0, ILNRHO = 3, ISS = 4, IAX = NF - 3;
  constexpr bool ENTROPY = (NF == 8);
  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + RING * C::SLOT_BYTES);
  double* red = reinterpret_cast<double*>(smem + C::RED_OFF);
  int* sh = reinterpret_cast<int*>(smem + C::RED_OFF + C::NWARP * PCGB_NSLOT * 8);

  const int tid = threadIdx.x;
  const int tx = tid % TX, ty = tid / TX;
  const int lane = tid & 31, warp = tid >> 5;

  if (tid == 0) {
    for (int r = 0; r < RING; ++r) mbar_init(&full[r], 1);
    fence_mbar_init();
  }
  __syncthreads();

  unsigned long long gplane = 0;   // planes loaded by this CTA so far (ring phase tracking)
  int iter = 0;
  int failed = 0;

  while (true) {
    int w;
    if (args.work_counter) {
      if (tid == 0) sh[0] = (int)atomicAdd(args.work_counter, 1u);
      __syncthreads();
      w = sh[0];
      __syncthreads();
    } else {
      w = (iter == 0) ? (int)blockIdx.x : args.total_tiles;
    }
    ++iter;
    if (w >= args.total_tiles) break;

    // locate the box of work item w
    int b = 0;
    while (b + 1 < args.nboxes && args.boxes[b + 1].tile0 <= w) ++b;
    const PcgbBoxDev& B = args.boxes[b];
    PcgbBoxState* S = B.state;
    // box fields held in registers (stores through fout/dfp must not force reloads)
    const int bnx = B.nx, bny = B.ny, bnz = B.nz, bpx = B.px, bmy = B.my, bmz = B.mz, bxoff = B.xoff;
    const long long bps = B.ps, bfs = B.fs;
    const int blforcing = B.lforcing, biso = B.isothermal, bvh = B.lviscosity_heat, boh = B.lohmic_heat;

    const int lt = w - B.tile0;
    const int tix = lt % B.ntx, tiy = (lt / B.ntx) % B.nty, tiz = lt / (B.ntx * B.nty);
    const int x0 = tix * TX, y0 = tiy * TY, z0 = tiz * B.zd;
    const int z1 = min(z0 + B.zd, bnz);
    const int nplanes = (z1 - z0) + 6;

    const unsigned long long nsub = __ldcg(&S->nsub);
    const int s = (int)(nsub % 3ull);
    const int inb = (int)(nsub & 1ull);
    const CUtensorMap* tmap = &B.tmap[inb];
    T* __restrict__ fout = reinterpret_cast<T*>(B.f[inb ^ 1]);
    T* __restrict__ dfp = reinterpret_cast<T*>(B.df);
    const double dt = __ldcg(&S->dt);
    const bool mode_cfl = (args.mode == MODE_CFL);
    const unsigned long long step = nsub / 3ull + __ldcg(&S->step0);
    const bool want_diag = !mode_cfl && s == 0 &&
                           ((B.diag_every > 0 && (step % (unsigned long long)B.diag_every) == 0ull) ||
                            __ldcg(&S->diag_request) != 0);
    const bool want_cfl = mode_cfl || (s == 0 && B.dt_mode == PCGB_DT_LAGGED);
    const bool need_red = want_cfl || want_diag;

    // producer: prologue
    if (tid == 0) {
      prefetch_tensormap(tmap);
      const int npro = nplanes < RING ? nplanes : RING;
      for (int j = 0; j < npro; ++j) {
        const unsigned long long G = gplane + (unsigned long long)j;
        const int slot = (int)(G % RING);
        fence_proxy_async_smem();
        mbar_arrive_expect_tx(&full[slot], C::PLANE_BYTES);
        tma_load_4d(smem + slot * C::SLOT_BYTES, tmap, &full[slot], B.xoff + x0 - 4, y0, z0 + j, 0);
      }
    }

    // per-box constants in T
    Fac<T> F;
    F.dx1 = T(B.dx_1); F.dy1 = T(B.dy_1); F.dz1 = T(B.dz_1); F.dxyz2 = T(B.dxyz_2);
    F.fx = T((1.0 / 60.0) * B.dx_1); F.fy = T((1.0 / 60.0) * B.dy_1); F.fz = T((1.0 / 60.0) * B.dz_1);
    F.sx = T(B.dx_1 * B.dx_1); F.sy = T(B.dy_1 * B.dy_1); F.sz = T(B.dz_1 * B.dz_1);
    F.mxy = T(((1.0 / 720.0) * B.dx_1) * B.dy_1);
    F.myz = T(((1.0 / 720.0) * B.dy_1) * B.dz_1);
    F.mxz = T(((1.0 / 720.0) * B.dz_1) * B.dx_1);
    Phys<T> P;
    P.nu = T(B.nu); P.eta = T(B.eta); P.chi_cp = T(B.chi * B.cpp); P.mu0 = T(B.mu0); P.mu01 = T(B.mu01);
    P.cs20 = T(B.cs20); P.gamma_m1 = T(B.gamma_m1); P.gamma1 = T(B.gamma1); P.lnrho0 = T(B.lnrho0);
    P.cv1 = T(B.cv1); P.lnTT0 = T(B.lnTT0); P.two_nu = T(2.0 * B.nu); P.eta_mu0 = T(B.eta * B.mu0);
    P.gamma_chi = T(B.gamma * B.chi);
    P.bx = T(B.b_ext[0]); P.by = T(B.b_ext[1]); P.bz = T(B.b_ext[2]);
    P.fact = T(B.fact); P.fact2 = T(B.fact2); P.abc_a = T(B.abc_a); P.abc_b = T(B.abc_b); P.abc_c = T(B.abc_c);
    P.ampl_fc = T(B.ampl_fcont_uu); P.cdt1 = T(1.0 / B.cdt); P.cdtv1 = T(1.0 / B.cdtv);
    // maxdiffus: max(diffus_nu, diffus_eta, diffus_chi), all constant in space here
    double mdiff = B.nu * B.dxyz_2;
    if (B.eta * B.dxyz_2 > mdiff) mdiff = B.eta * B.dxyz_2;
    if (B.lentropy && (B.gamma * B.chi) * B.dxyz_2 > mdiff) mdiff = (B.gamma * B.chi) * B.dxyz_2;
    const T maxdiffus = T(mdiff);

    const T alpha = T(rk_alpha(s));
    const T dtb = T(dt * rk_beta(s));
    // compensated mode: df_stored = df + e / (dt*beta_{s+1}*alpha_{s+1})
    const T cinv = (B.comp && s < 2) ? T(1.0 / (dt * rk_beta(s + 1) * rk_alpha(s + 1))) : T(0);
    const bool comp = (B.comp != 0);
    const bool read_df = (s > 0) || comp;
    const bool write_df = (s < 2) || comp;

    const int x = x0 + tx, y = y0 + ty;
    const bool active = (x < bnx) && (y < bny);
    const T* sinx = reinterpret_cast<const T*>(B.forc);
    const T* cosx = sinx + bpx;
    const T* siny = cosx + bpx;
    const T* cosy = siny + bmy;
    const T* sinz = cosy + bmy;
    const T* cosz = sinz + bmz;

    // forcing factors that depend on x or y only, read once per tile
    T fsx = T(0), fcx = T(0), fsy = T(0), fcy = T(0);
    if (blforcing && active) {
      fsx = sinx[x + 3]; fcx = cosx[x + 3]; fsy = siny[y + 3]; fcy = cosy[y + 3];
    }
    // df of the first plane, prefetched; later planes are prefetched one plane ahead
    T dfnext[NF];
#pragma unroll
    for (int k = 0; k < NF; ++k) dfnext[k] = T(0);
    if (read_df && active && !mode_cfl) {
      const long long c0 = (long long)(z0 + 3) * bps + (long long)(y + 3) * bpx + bxoff + x;
#pragma unroll
      for (int k = 0; k < NF; ++k) dfnext[k] = dfp[k * bfs + c0];
    }

    Acc acc;
    acc.reset();
    T dt1max = T(0);

    for (int z = z0; z < z1; ++z) {
      const int j = z - z0;
      // wait for planes j..j+6 (only the newest is new after the first plane)
      const int jw0 = (j == 0) ? 0 : j + 6;
      int lfail = 0;
      for (int jw = jw0; jw <= j + 6; ++jw) {
        const unsigned long long G = gplane + (unsigned long long)jw;
        if (!mbar_wait_bounded(&full[G % RING], (uint32_t)((G / RING) & 1ull), args.wait_limit)) lfail = 1;
      }
      if (__syncthreads_or(lfail)) {
        failed = 1;
        // drain: wait (bounded) for every plane still in flight before leaving
        if (tid == 0) {
          const int hi = (j + RING < nplanes) ? j + RING : nplanes;
          for (int jw = j; jw < hi; ++jw) {
            const unsigned long long G = gplane + (unsigned long long)jw;
            mbar_wait_bounded(&full[G % RING], (uint32_t)((G / RING) & 1ull), args.wait_limit);
          }
        }
        break;
      }

      if (active && !mode_cfl) {
        Stencil<T, NF, TX, TY, RING> st;
        st.F = F;
#pragma unroll
        for (int d = 0; d < 7; ++d) {
          const unsigned long long G = gplane + (unsigned long long)(j + d);
          st.pl[d] = reinterpret_cast<const T*>(smem + (G % RING) * C::SLOT_BYTES) + (ty + 3) * C::BW + (tx + 4);
        }
        const long long cidx = (long long)(z + 3) * bps + (long long)(y + 3) * bpx + bxoff + x;
        T dfo[NF];
#pragma unroll
        for (int k = 0; k < NF; ++k) dfo[k] = dfnext[k];
        if (read_df && z + 1 < z1) {
#pragma unroll
          for (int k = 0; k < NF; ++k) dfnext[k] = dfp[k * bfs + cidx + bps];
        }

        // ---- hydro pencils (hydro.f90:3564-3990, sub.f90) ----
        T uu[3], uij[3][3];
#pragma unroll
        for (int i = 0; i < 3; ++i) {
          uu[i] = st.v(0, IUX + i, 0, 0);
#pragma unroll
          for (int jj = 0; jj < 3; ++jj) uij[i][jj] = st.der(IUX + i, jj);
        }
        const T u2 = (uu[0] * uu[0] + uu[1] * uu[1]) + uu[2] * uu[2];
        const T divu = (uij[0][0] + uij[1][1]) + uij[2][2];
        T sij[3][3];
#pragma unroll
        for (int jj = 0; jj < 3; ++jj) {
          sij[jj][jj] = uij[jj][jj] - T(1.0 / 3.0) * divu;
#pragma unroll
          for (int i = jj + 1; i < 3; ++i) {
            sij[i][jj] = T(0.5) * (uij[i][jj] + uij[jj][i]);
            sij[jj][i] = sij[i][jj];
          }
        }
        T ugu[3];
#pragma unroll
        for (int jj = 0; jj < 3; ++jj) ugu[jj] = (uu[0] * uij[jj][0] + uu[1] * uij[jj][1]) + uu[2] * uij[jj][2];
        T del2u[3], graddivu[3];
#pragma unroll
        for (int i = 0; i < 3; ++i) {
          T f0 = st.der2(IUX + i, 0), f1 = st.der2(IUX + i, 1), f2 = st.der2(IUX + i, 2);
          del2u[i] = (f0 + f1) + f2;
          // graddiv_i = sum_j d_i d_j u_j ; diagonal term from der2 (sub.f90:2646-2656)
          T g0 = (i == 0) ? f0 : st.derij(IUX + 0, 0 < i ? 0 : i, 0 < i ? i : 0);
          T g1 = (i == 1) ? f1 : st.derij(IUX + 1, 1 < i ? 1 : i, 1 < i ? i : 1);
          T g2 = (i == 2) ? f2 : st.derij(IUX + 2, 2 < i ? 2 : i, 2 < i ? i : 2);
          graddivu[i] = (g0 + g1) + g2;
        }
        // ---- density pencils (density.f90:2747-2800) ----
        const T lnrho = st.v(0, ILNRHO, 0, 0);
        const T rho1 = texp(-lnrho);
        T glnrho[3];
#pragma unroll
        for (int jj = 0; jj < 3; ++jj) glnrho[jj] = st.der(ILNRHO, jj);
        const T uglnrho = (uu[0] * glnrho[0] + uu[1] * glnrho[1]) + uu[2] * glnrho[2];
        T sglnrho[3];
#pragma unroll
        for (int i = 0; i < 3; ++i) sglnrho[i] = (sij[i][0] * glnrho[0] + sij[i][1] * glnrho[1]) + sij[i][2] * glnrho[2];
        // ---- EOS (eos_idealgas.f90:842-887) ----
        T cs2, ss = T(0), TT1 = T(0), gss[3] = {T(0), T(0), T(0)}, glnTT[3] = {T(0), T(0), T(0)}, del2lnTT = T(0);
        if (ENTROPY) {
          ss = st.v(0, ISS, 0, 0);
#pragma unroll
          for (int jj = 0; jj < 3; ++jj) gss[jj] = st.der(ISS, jj);
          const T del2lnrho = (st.der2(ILNRHO, 0) + st.der2(ILNRHO, 1)) + st.der2(ILNRHO, 2);
          const T del2ss = (st.der2(ISS, 0) + st.der2(ISS, 1)) + st.der2(ISS, 2);
          cs2 = P.cs20 * texp(P.cv1 * ss + P.gamma_m1 * (lnrho - P.lnrho0));
          const T lnTT = (P.lnTT0 + P.cv1 * ss) + P.gamma_m1 * (lnrho - P.lnrho0);
          TT1 = texp(-lnTT);
#pragma unroll
          for (int jj = 0; jj < 3; ++jj) glnTT[jj] = P.gamma_m1 * glnrho[jj] + P.cv1 * gss[jj];
          del2lnTT = P.gamma_m1 * del2lnrho + P.cv1 * del2ss;
        } else if (biso) {
          cs2 = P.cs20;
        } else {
          cs2 = P.cs20 * texp(P.gamma_m1 * (lnrho - P.lnrho0));
        }
        // ---- magnetic pencils (magnetic.f90:4310-4900, gij_etc sub.f90:2945) ----
        T aij[3][3];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
          for (int jj = 0; jj < 3; ++jj) aij[i][jj] = st.der(IAX + i, jj);
        T bb[3];
        bb[0] = aij[2][1] - aij[1][2];
        bb[1] = aij[0][2] - aij[2][0];
        bb[2] = aij[1][0] - aij[0][1];
        // d2A[j][k][i] = A_i,jk.  J = curl(b_ij) uses the six off-diagonal b_ij,
        // which need the mixed derivatives A_1,xy A_2,xy A_1,xz A_3,xz A_2,yz A_3,yz;
        // the other three (A_3,xy A_2,xz A_1,yz) enter only the diagonal b_ii,
        // i.e. div B, and are evaluated on diagnostic substeps only.
        T d2A[3][3][3];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
          for (int jj = 0; jj < 3; ++jj) d2A[jj][jj][i] = st.der2(IAX + i, jj);
        d2A[0][1][0] = st.derij(IAX + 0, 0, 1); d2A[1][0][0] = d2A[0][1][0];
        d2A[0][1][1] = st.derij(IAX + 1, 0, 1); d2A[1][0][1] = d2A[0][1][1];
        d2A[0][2][0] = st.derij(IAX + 0, 0, 2); d2A[2][0][0] = d2A[0][2][0];
        d2A[0][2][2] = st.derij(IAX + 2, 0, 2); d2A[2][0][2] = d2A[0][2][2];
        d2A[1][2][1] = st.derij(IAX + 1, 1, 2); d2A[2][1][1] = d2A[1][2][1];
        d2A[1][2][2] = st.derij(IAX + 2, 1, 2); d2A[2][1][2] = d2A[1][2][2];
        // off-diagonal b_ij = eps_ikl A_l,kj (sub.f90:3017-3019)
        T bij[3][3];
        bij[0][1] = d2A[1][1][2] - d2A[2][1][1];
        bij[0][2] = d2A[1][2][2] - d2A[2][2][1];
        bij[1][0] = d2A[2][0][0] - d2A[0][0][2];
        bij[1][2] = d2A[2][2][0] - d2A[0][2][2];
        bij[2][0] = d2A[0][0][1] - d2A[1][0][0];
        bij[2][1] = d2A[0][1][1] - d2A[1][1][0];
        bij[0][0] = bij[1][1] = bij[2][2] = T(0);
        if (want_diag) {
          const T a3xy = st.derij(IAX + 2, 0, 1), a2xz = st.derij(IAX + 1, 0, 2), a1yz = st.derij(IAX + 0, 1, 2);
          bij[0][0] = a3xy - a2xz;
          bij[1][1] = a1yz - a3xy;
          bij[2][2] = a2xz - a1yz;
        }
        T del2a[3];
#pragma unroll
        for (int i = 0; i < 3; ++i) del2a[i] = (d2A[0][0][i] + d2A[1][1][i]) + d2A[2][2][i];
        bb[0] = bb[0] + P.bx; bb[1] = bb[1] + P.by; bb[2] = bb[2] + P.bz;
        T jj3[3];
        jj3[0] = P.mu01 * (bij[2][1] - bij[1][2]);
        jj3[1] = P.mu01 * (bij[0][2] - bij[2][0]);
        jj3[2] = P.mu01 * (bij[1][0] - bij[0][1]);
        const T b2 = (bb[0] * bb[0] + bb[1] * bb[1]) + bb[2] * bb[2];
        const T j2 = (jj3[0] * jj3[0] + jj3[1] * jj3[1]) + jj3[2] * jj3[2];
        T jxbr[3], uxb[3];
        jxbr[0] = rho1 * (jj3[1] * bb[2] - jj3[2] * bb[1]);
        jxbr[1] = rho1 * (jj3[2] * bb[0] - jj3[0] * bb[2]);
        jxbr[2] = rho1 * (jj3[0] * bb[1] - jj3[1] * bb[0]);
        uxb[0] = uu[1] * bb[2] - uu[2] * bb[1];
        uxb[1] = uu[2] * bb[0] - uu[0] * bb[2];
        uxb[2] = uu[0] * bb[1] - uu[1] * bb[0];

        // ---- right-hand sides in module order (equ.f90:1268-1274) ----
        T dfn[NF];
        // duu_dt (hydro.f90:4421): -u.grad u, viscous force, continuous forcing
        T dfu[3];
#pragma unroll
        for (int jj = 0; jj < 3; ++jj) dfu[jj] = alpha * dfo[IUX + jj] - ugu[jj];
#pragma unroll
        for (int jj = 0; jj < 3; ++jj)
          dfu[jj] = dfu[jj] + P.nu * ((del2u[jj] + T(2) * sglnrho[jj]) + T(1.0 / 3.0) * graddivu[jj]);
        if (blforcing) {
          const T fc0 = P.fact * (P.abc_c * sinz[z + 3] + (P.fact2 * P.abc_b) * fcy);
          const T fc1 = P.fact * (P.abc_a * fsx + (P.fact2 * P.abc_c) * cosz[z + 3]);
          const T fc2 = P.fact * (P.abc_b * fsy + (P.fact2 * P.abc_a) * fcx);
          dfu[0] = dfu[0] + P.ampl_fc * fc0;
          dfu[1] = dfu[1] + P.ampl_fc * fc1;
          dfu[2] = dfu[2] + P.ampl_fc * fc2;
        }
        // dlnrho_dt (density.f90:2929-2930, :3059)
        dfn[ILNRHO] = alpha * dfo[ILNRHO] + (-divu - uglnrho);
        // denergy_dt: pressure force (+ entropy equation)
        if (!ENTROPY) {
#pragma unroll
          for (int jj = 0; jj < 3; ++jj) dfu[jj] = dfu[jj] + (-(cs2 * glnrho[jj]));
        } else {
#pragma unroll
          for (int jj = 0; jj < 3; ++jj) dfu[jj] = dfu[jj] + (-((cs2 * (glnrho[jj] + glnTT[jj])) * P.gamma1));
          const T ugss = (uu[0] * gss[0] + uu[1] * gss[1]) + uu[2] * gss[2];
          T dfs = alpha * dfo[ISS] - ugss;
          if (bvh) {
            T sij2 = sij[0][0] * sij[0][0];
            sij2 = sij2 + sij[1][1] * sij[1][1];
            sij2 = sij2 + T(2) * (sij[1][0] * sij[1][0]);
            sij2 = sij2 + sij[2][2] * sij[2][2];
            sij2 = sij2 + T(2) * (sij[2][0] * sij[2][0]);
            sij2 = sij2 + T(2) * (sij[2][1] * sij[2][1]);
            dfs = dfs + TT1 * (P.two_nu * sij2);
          }
          const T gs0 = glnrho[0] + glnTT[0], gs1 = glnrho[1] + glnTT[1], gs2 = glnrho[2] + glnTT[2];
          const T g2 = (gs0 * glnTT[0] + gs1 * glnTT[1]) + gs2 * glnTT[2];
          dfs = dfs + P.chi_cp * (del2lnTT + g2);
          if (boh) dfs = dfs + ((P.eta_mu0 * j2) * rho1) * TT1;
          dfn[ISS] = dfs;
        }
        // daa_dt (magnetic.f90:5531, :5589, :6247, :6524)
#pragma unroll
        for (int jj = 0; jj < 3; ++jj) dfu[jj] = dfu[jj] + jxbr[jj];
#pragma unroll
        for (int jj = 0; jj < 3; ++jj) dfn[IAX + jj] = alpha * dfo[IAX + jj] + (uxb[jj] + P.eta * del2a[jj]);
#pragma unroll
        for (int jj = 0; jj < 3; ++jj) dfn[IUX + jj] = dfu[jj];

        // ---- 2N update (timestep.f90:160) and periodic ghost images ----
        T fnew[NF], dsto[NF];
#pragma unroll
        for (int k = 0; k < NF; ++k) {
          const T fc = st.v(0, k, 0, 0);
          if (!comp) {
            fnew[k] = fc + dtb * dfn[k];
            dsto[k] = dfn[k];
          } else {
            // TwoSum of fc + y, y carrying the previous step's compensation on substep 1
            const T y = (s == 0) ? (dtb * dfn[k] + dfo[k]) : dtb * dfn[k];
            const T t = fc + y;
            const T bp = t - fc;
            const T e = (fc - (t - bp)) + (y - bp);
            fnew[k] = t;
            dsto[k] = (s < 2) ? (dfn[k] + e * cinv) : e;
          }
        }
        if (write_df) {
#pragma unroll
          for (int k = 0; k < NF; ++k) dfp[k * bfs + cidx] = dsto[k];
        }
#pragma unroll
        for (int k = 0; k < NF; ++k) fout[k * bfs + cidx] = fnew[k];
        const bool edge = (x < 3) | (x >= bnx - 3) | (y < 3) | (y >= bny - 3) | (z < 3) | (z >= bnz - 3);
        if (edge) {
          int xs[2], ys[2], zs[2], nxs = 0, nys = 0, nzs = 0;
          xs[nxs++] = x; if (x < 3) xs[nxs++] = x + bnx; else if (x >= bnx - 3) xs[nxs++] = x - bnx;
          ys[nys++] = y; if (y < 3) ys[nys++] = y + bny; else if (y >= bny - 3) ys[nys++] = y - bny;
          zs[nzs++] = z; if (z < 3) zs[nzs++] = z + bnz; else if (z >= bnz - 3) zs[nzs++] = z - bnz;
          for (int a = 0; a < nzs; ++a)
            for (int c = 0; c < nys; ++c)
              for (int e = 0; e < nxs; ++e) {
                if (a == 0 && c == 0 && e == 0) continue;
                const long long gi = (long long)(zs[a] + 3) * bps + (long long)(ys[c] + 3) * bpx + bxoff + xs[e];
#pragma unroll
                for (int k = 0; k < NF; ++k) fout[k * bfs + gi] = fnew[k];
              }
        }

        if (want_cfl) {
          const T d = cfl_dt1(P, F, uu, bb, rho1, cs2, maxdiffus);
          dt1max = (d > dt1max || d != d) ? d : dt1max;
        }
        if (want_diag) {
          const double du2 = (double)u2, db2 = (double)b2;
          const double divb = (double)((bij[0][0] + bij[1][1]) + bij[2][2]);
          const double aa0 = (double)st.v(0, IAX, 0, 0), aa1 = (double)st.v(0, IAX + 1, 0, 0),
                       aa2 = (double)st.v(0, IAX + 2, 0, 0);
          const double rho = exp((double)lnrho);
          acc.v[PCGB_S_U2SUM] += du2;
          acc.v[PCGB_S_U2MAX] = fmax(acc.v[PCGB_S_U2MAX], du2);
          acc.v[PCGB_S_B2SUM] += db2;
          acc.v[PCGB_S_B2MAX] = fmax(acc.v[PCGB_S_B2MAX], db2);
          acc.v[PCGB_S_EKINSUM] += 0.5 * rho * du2;
          acc.v[PCGB_S_RHOSUM] += rho;
          acc.v[PCGB_S_DIVB2SUM] += divb * divb;
          acc.v[PCGB_S_J2SUM] += (double)j2;
          acc.v[PCGB_S_ABSUM] += (aa0 * (double)bb[0] + aa1 * (double)bb[1]) + aa2 * (double)bb[2];
        }
      } else if (active && mode_cfl) {
        // CFL-only pass (PCGB_DT_CURRENT and the first step of PCGB_DT_LAGGED)
        Stencil<T, NF, TX, TY, RING> st;
        st.F = F;
#pragma unroll
        for (int d = 0; d < 7; ++d) {
          const unsigned long long G = gplane + (unsigned long long)(j + d);
          st.pl[d] = reinterpret_cast<const T*>(smem + (G % RING) * C::SLOT_BYTES) + (ty + 3) * C::BW + (tx + 4);
        }
        T uu[3] = {st.v(0, 0, 0, 0), st.v(0, 1, 0, 0), st.v(0, 2, 0, 0)};
        const T lnrho = st.v(0, ILNRHO, 0, 0);
        const T rho1 = texp(-lnrho);
        T cs2;
        if (ENTROPY) {
          cs2 = P.cs20 * texp(P.cv1 * st.v(0, ISS, 0, 0) + P.gamma_m1 * (lnrho - P.lnrho0));
        } else if (biso) {
          cs2 = P.cs20;
        } else {
          cs2 = P.cs20 * texp(P.gamma_m1 * (lnrho - P.lnrho0));
        }
        T bb[3];
        bb[0] = (st.der(IAX + 2, 1) - st.der(IAX + 1, 2)) + P.bx;
        bb[1] = (st.der(IAX + 0, 2) - st.der(IAX + 2, 0)) + P.by;
        bb[2] = (st.der(IAX + 1, 0) - st.der(IAX + 0, 1)) + P.bz;
        const T d = cfl_dt1(P, F, uu, bb, rho1, cs2, maxdiffus);
        dt1max = (d > dt1max || d != d) ? d : dt1max;
      }

      __syncthreads();   // every thread is done with plane j
      if (tid == 0 && j + RING < nplanes) {
        const unsigned long long G = gplane + (unsigned long long)(j + RING);
        const int slot = (int)(G % RING);
        fence_proxy_async_smem();
        mbar_arrive_expect_tx(&full[slot], C::PLANE_BYTES);
        tma_load_4d(smem + slot * C::SLOT_BYTES, tmap, &full[slot], bxoff + x0 - 4, y0, z0 + j + RING, 0);
      }
    }
    gplane += (unsigned long long)nplanes;
    if (failed) {
      if (tid == 0) atomicOr(&S->err, PCGB_ERR_TIMEOUT);
      break;
    }

    // ---- per-tile reduction (fixed order: lanes, then warps) ----
    if (need_red) {
      acc.v[PCGB_S_DT1MAX] = (double)dt1max;
#pragma unroll
      for (int q = 0; q < PCGB_NSLOT; ++q) {
        double vq = acc.v[q];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
          const double other = __shfl_xor_sync(0xffffffffu, vq, o);
          vq = slot_is_max(q) ? ((other > vq || other != other) ? other : vq) : vq + other;
        }
        if (lane == 0) red[warp * PCGB_NSLOT + q] = vq;
      }
      __syncthreads();
      if (tid < PCGB_NSLOT) {
        double r = red[tid];
        for (int wq = 1; wq < C::NWARP; ++wq) {
          const double o = red[wq * PCGB_NSLOT + tid];
          r = slot_is_max(tid) ? ((o > r || o != o) ? o : r) : r + o;
        }
        B.partial[(long long)lt * PCGB_NSLOT + tid] = r;
      }
    }

    // ---- last CTA of the box: reduce tiles in order, advance bookkeeping ----
    __threadfence();
    __syncthreads();
    if (tid == 0) {
      const unsigned int prev = atomicAdd(&S->done, 1u);
      sh[1] = (prev == (unsigned int)(B.tiles - 1)) ? 1 : 0;
    }
    __syncthreads();
    if (sh[1]) {
      __threadfence();
      if (need_red) {
        // each thread reduces a fixed strided subset in tile order, then a fixed-order combine
        double part[PCGB_NSLOT];
#pragma unroll
        for (int q = 0; q < PCGB_NSLOT; ++q) part[q] = 0.0;
        for (int t = tid; t < B.tiles; t += C::NT) {
#pragma unroll
          for (int q = 0; q < PCGB_NSLOT; ++q) {
            const double o = __ldcg(&B.partial[(long long)t * PCGB_NSLOT + q]);
            part[q] = slot_is_max(q) ? ((o > part[q] || o != o) ? o : part[q]) : part[q] + o;
          }
        }
#pragma unroll
        for (int q = 0; q < PCGB_NSLOT; ++q) {
          double vq = part[q];
#pragma unroll
          for (int o = 16; o > 0; o >>= 1) {
            const double other = __shfl_xor_sync(0xffffffffu, vq, o);
            vq = slot_is_max(q) ? ((other > vq || other != other) ? other : vq) : vq + other;
          }
          if (lane == 0) red[warp * PCGB_NSLOT + q] = vq;
        }
        __syncthreads();
        if (tid == 0) {
          double r[PCGB_NSLOT];
          for (int q = 0; q < PCGB_NSLOT; ++q) {
            r[q] = red[q];
            for (int wq = 1; wq < C::NWARP; ++wq) {
              const double o = red[wq * PCGB_NSLOT + q];
              r[q] = slot_is_max(q) ? ((o > r[q] || o != o) ? o : r[q]) : r[q] + o;
            }
          }
          if (want_cfl) {
            const double dtn = 1.0 / r[PCGB_S_DT1MAX];   // set_dt, sub.f90:4247
            if (!(dtn > 0.0) || !isfinite(dtn)) atomicOr(&S->err, PCGB_ERR_DT | PCGB_ERR_NONFINITE);
            if (mode_cfl) {
              if (B.dt_mode != PCGB_DT_FIXED) { S->dt = dtn; S->dt_next = dtn; }
            } else {
              S->dt_next = dtn;
            }
          }
          if (want_diag) {
            for (int q = 0; q < PCGB_NSLOT; ++q) S->diag[q] = r[q];
            S->diag_step = step;
            S->diag_request = 0;
          }
        }
      }
      if (tid == 0) {
        if (!mode_cfl) {
          // ds and time bookkeeping, timestep.f90:108-148, :201
          double ds = (s == 0) ? 0.0 : rk_alpha(s) * S->ds;
          ds = ds + 1.0;
          S->ds = ds;
          S->t = S->t + ds * (dt * rk_beta(s));
          if (s == 2 && B.dt_mode == PCGB_DT_LAGGED) S->dt = S->dt_next;
          S->nsub = nsub + 1ull;
        }
        S->done = 0u;
        __threadfence();
      }
    }
    __syncthreads();
  }
}

}  // namespace pcgb
