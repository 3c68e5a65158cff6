// cell_scalar.cuh -- cell policy with one value per field per cell (FP64, and
// FP32 in the field-major layout).  Shared memory holds NF field slices per
// plane; every stencil is a sequence of scalar loads.
#pragma once

#include "cell_physics.cuh"

namespace pcgb {

// UPW: compiled with the upwind corrections (lupw_uu, lupw_lnrho); the
// variants without them keep the registers of the plain advection terms.
template <typename TT, int NF, int TX, int TY, bool UPW = false>
struct ScalarCell {
  using T = TT;
  using Elem = TT;
  static constexpr int NSLICE = NF;
  static constexpr int BW = TX + 8, BH = TY + 6, FO = BW * BH;
  static constexpr int IUX = 0, ILNRHO = 3, ISS = 4, IAX = NF - 3;
  static constexpr bool ENTROPY = (NF == 8);

  // Stencils on the 7 staged planes (each pointer at field 0, row ty+3, col tx+4).
  struct St {
    const T* const* pl;
    const Fac<T>& F;
    __device__ __forceinline__ T v(int dz, int k, int dy, int dx) const { return pl[dz + 3][k * FO + dy * BW + dx]; }
    // der_main, deriv.f90:127-129 (x), :140-142 (y), :158-160 (z)
    __device__ __forceinline__ T der(int k, int j) const {
      if (j == 0)
        return F.fx * ((wmul<T>(45, v(0, k, 0, 1) - v(0, k, 0, -1)) - wmul<T>(9, v(0, k, 0, 2) - v(0, k, 0, -2))) +
                       (v(0, k, 0, 3) - v(0, k, 0, -3)));
      if (j == 1)
        return F.fy * ((wmul<T>(45, v(0, k, 1, 0) - v(0, k, -1, 0)) - wmul<T>(9, v(0, k, 2, 0) - v(0, k, -2, 0))) +
                       (v(0, k, 3, 0) - v(0, k, -3, 0)));
      return F.fz * ((wmul<T>(45, v(1, k, 0, 0) - v(-1, k, 0, 0)) - wmul<T>(9, v(2, k, 0, 0) - v(-2, k, 0, 0))) +
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
    // der6_main with upwind=T, deriv.f90:936-1010: (1/60) dx_1 (-20 f0 + 15 (f1 + f-1) - 6 (f2 + f-2) + (f3 + f-3))
    __device__ __forceinline__ T del6u(int k, int j) const {
      const T f0 = v(0, k, 0, 0);
      if (j == 0)
        return F.fx * (((wmul<T>(-20, f0) + wmul<T>(15, v(0, k, 0, 1) + v(0, k, 0, -1))) -
                        wmul<T>(6, v(0, k, 0, 2) + v(0, k, 0, -2))) + (v(0, k, 0, 3) + v(0, k, 0, -3)));
      if (j == 1)
        return F.fy * (((wmul<T>(-20, f0) + wmul<T>(15, v(0, k, 1, 0) + v(0, k, -1, 0))) -
                        wmul<T>(6, v(0, k, 2, 0) + v(0, k, -2, 0))) + (v(0, k, 3, 0) + v(0, k, -3, 0)));
      return F.fz * (((wmul<T>(-20, f0) + wmul<T>(15, v(1, k, 0, 0) + v(-1, k, 0, 0))) -
                      wmul<T>(6, v(2, k, 0, 0) + v(-2, k, 0, 0))) + (v(3, k, 0, 0) + v(-3, k, 0, 0)));
    }
    // calc_del6_for_upwind, sub.f90:7491-7539: sum_j |u_j| D6_j f
    __device__ __forceinline__ T upwind(int k, const T u[3]) const {
      return (tabs(u[0]) * del6u(k, 0) + tabs(u[1]) * del6u(k, 1)) + tabs(u[2]) * del6u(k, 2);
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
      return fac * ((wmul<T>(270, t[0]) - wmul<T>(27, t[1])) + wmul<T>(2, t[2]));
    }
  };

  struct Tile {
    Fac<T> F;
    Phys<T> P;
    T* fout;
    T* dfp;
    long long ps, fs;
    int px, xoff, nx, ny, nz;
    bool forcing, iso, vheat, oheat;
    T fsx, fcx, fsy, fcy;
    const T* sinz;
    const T* cosz;
    T fsz, fcz;   // sin/cos(kf z) of the current plane, prefetched one plane ahead
    T dfnext[NF];
    int upw;      // UPW_* bits

    __device__ __forceinline__ void begin(const PcgbBoxDev& B, int inb, int x, int y, int z0, bool active,
                                          bool mode_cfl, const StepFlags<T>& fl) {
      make_fac(F, B);
      make_phys(P, B);
      fout = reinterpret_cast<T*>(B.f[inb ^ 1]);
      dfp = reinterpret_cast<T*>(B.df);
      ps = B.ps; fs = B.fs; px = B.px; xoff = B.xoff; nx = B.nx; ny = B.ny; nz = B.nz;
      forcing = B.lforcing != 0; iso = B.isothermal != 0; vheat = B.lviscosity_heat != 0; oheat = B.lohmic_heat != 0;
      upw = UPW ? B.lupw : 0;
      const T* sinx = reinterpret_cast<const T*>(B.forc);
      const T* cosx = sinx + B.px;
      const T* siny = cosx + B.px;
      const T* cosy = siny + B.my;
      sinz = cosy + B.my;
      cosz = sinz + B.mz;
      fsx = fcx = fsy = fcy = fsz = fcz = T(0);
      if (forcing && active) {
        fsx = sinx[x + 3]; fcx = cosx[x + 3]; fsy = siny[y + 3]; fcy = cosy[y + 3];
        fsz = sinz[z0 + 3]; fcz = cosz[z0 + 3];
      }
#pragma unroll
      for (int k = 0; k < NF; ++k) dfnext[k] = T(0);
      if (fl.read_df && active && !mode_cfl) {
        const long long c0 = (long long)(z0 + 3) * ps + (long long)(y + 3) * px + xoff + x;
#pragma unroll
        for (int k = 0; k < NF; ++k) dfnext[k] = dfp[k * fs + c0];
      }
    }

    // Field values and stencil derivatives of one cell, fully unrolled.
    static __device__ __forceinline__ void upwinding(const St& st, CellIn<T>& c, int upw) {
      if (upw & UPW_UU) {
#pragma unroll
        for (int i = 0; i < 3; ++i) c.upw_u[i] = st.upwind(IUX + i, c.uu);
      }
      if (upw & UPW_LNRHO) c.upw_lnrho = st.upwind(ILNRHO, c.uu);
    }

    static __device__ __forceinline__ void gather(const St& st, CellIn<T>& c, bool want_diag) {
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        c.uu[i] = st.v(0, IUX + i, 0, 0);
#pragma unroll
        for (int jj = 0; jj < 3; ++jj) c.uij[i][jj] = st.der(IUX + i, jj);
      }
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        const T f0 = st.der2(IUX + i, 0), f1 = st.der2(IUX + i, 1), f2 = st.der2(IUX + i, 2);
        c.del2u[i] = (f0 + f1) + f2;
        // graddiv_i = sum_j d_i d_j u_j ; diagonal term from der2 (sub.f90:2646-2656)
        const T g0 = (i == 0) ? f0 : st.derij(IUX + 0, 0, i);
        const T g1 = (i == 1) ? f1 : st.derij(IUX + 1, 1 < i ? 1 : i, 1 < i ? i : 1);
        const T g2 = (i == 2) ? f2 : st.derij(IUX + 2, i, 2);
        c.graddivu[i] = (g0 + g1) + g2;
      }
      c.lnrho = st.v(0, ILNRHO, 0, 0);
#pragma unroll
      for (int jj = 0; jj < 3; ++jj) c.glnrho[jj] = st.der(ILNRHO, jj);
      if (ENTROPY) {
        c.ss = st.v(0, ISS, 0, 0);
#pragma unroll
        for (int jj = 0; jj < 3; ++jj) c.gss[jj] = st.der(ISS, jj);
        c.del2lnrho = (st.der2(ILNRHO, 0) + st.der2(ILNRHO, 1)) + st.der2(ILNRHO, 2);
        c.del2ss = (st.der2(ISS, 0) + st.der2(ISS, 1)) + st.der2(ISS, 2);
      } else {
        c.ss = T(0); c.gss[0] = c.gss[1] = c.gss[2] = T(0); c.del2lnrho = c.del2ss = T(0);
      }
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        c.aa[i] = st.v(0, IAX + i, 0, 0);
#pragma unroll
        for (int jj = 0; jj < 3; ++jj) {
          c.aij[i][jj] = st.der(IAX + i, jj);
          c.a2[i][jj] = st.der2(IAX + i, jj);
        }
      }
      c.a1xy = st.derij(IAX + 0, 0, 1); c.a2xy = st.derij(IAX + 1, 0, 1);
      c.a1xz = st.derij(IAX + 0, 0, 2); c.a3xz = st.derij(IAX + 2, 0, 2);
      c.a2yz = st.derij(IAX + 1, 1, 2); c.a3yz = st.derij(IAX + 2, 1, 2);
      c.a3xy = c.a2xz = c.a1yz = T(0);
      if (want_diag) {
        c.a3xy = st.derij(IAX + 2, 0, 1); c.a2xz = st.derij(IAX + 1, 0, 2); c.a1yz = st.derij(IAX + 0, 1, 2);
      }
    }

    // The same stencils and operation order with one copy of each stencil's
    // code, looped over fields and mixed-derivative jobs; results pass through
    // thread-local arrays (L1).  Fully unrolled, a double-float plane step is
    // about 7600 instructions (120 KB of code per z iteration), more than the
    // instruction caches hold, and its warps stall on instruction fetch.
    static __device__ __forceinline__ void gather_compact(const St& st, CellIn<T>& c, bool want_diag) {
      T d1[NF][3], d2[NF][3], m[15];
#pragma unroll 1
      for (int k = 0; k < NF; ++k) {
#pragma unroll
        for (int j = 0; j < 3; ++j) d1[k][j] = st.der(k, j);
        if (k < ILNRHO || k >= IAX || ENTROPY) {
#pragma unroll
          for (int j = 0; j < 3; ++j) d2[k][j] = st.der2(k, j);
        }
      }
      // (field, direction pair) of each mixed derivative; pair 0 = xy, 1 = yz, 2 = xz
      const int njob = want_diag ? 15 : 12;
#pragma unroll 1
      for (int q = 0; q < njob; ++q) {
        const int code = mixed_job(q);
        const int k = code >> 2, pr = code & 3;
        if (pr == 0) m[q] = st.derij(k, 0, 1);
        else if (pr == 1) m[q] = st.derij(k, 1, 2);
        else m[q] = st.derij(k, 0, 2);
      }
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        c.uu[i] = st.v(0, IUX + i, 0, 0);
        c.aa[i] = st.v(0, IAX + i, 0, 0);
#pragma unroll
        for (int jj = 0; jj < 3; ++jj) {
          c.uij[i][jj] = d1[IUX + i][jj];
          c.aij[i][jj] = d1[IAX + i][jj];
          c.a2[i][jj] = d2[IAX + i][jj];
        }
        c.del2u[i] = (d2[IUX + i][0] + d2[IUX + i][1]) + d2[IUX + i][2];
      }
      c.graddivu[0] = (d2[IUX + 0][0] + m[2]) + m[4];
      c.graddivu[1] = (m[0] + d2[IUX + 1][1]) + m[5];
      c.graddivu[2] = (m[1] + m[3]) + d2[IUX + 2][2];
      c.lnrho = st.v(0, ILNRHO, 0, 0);
#pragma unroll
      for (int jj = 0; jj < 3; ++jj) c.glnrho[jj] = d1[ILNRHO][jj];
      if (ENTROPY) {
        c.ss = st.v(0, ISS, 0, 0);
#pragma unroll
        for (int jj = 0; jj < 3; ++jj) c.gss[jj] = d1[ISS][jj];
        c.del2lnrho = (d2[ILNRHO][0] + d2[ILNRHO][1]) + d2[ILNRHO][2];
        c.del2ss = (d2[ISS][0] + d2[ISS][1]) + d2[ISS][2];
      } else {
        c.ss = T(0); c.gss[0] = c.gss[1] = c.gss[2] = T(0); c.del2lnrho = c.del2ss = T(0);
      }
      c.a1xy = m[6]; c.a2xy = m[7]; c.a1xz = m[8]; c.a3xz = m[9]; c.a2yz = m[10]; c.a3yz = m[11];
      c.a3xy = c.a2xz = c.a1yz = T(0);
      if (want_diag) { c.a3xy = m[12]; c.a2xz = m[13]; c.a1yz = m[14]; }
    }

    // job q of gather_compact: field * 4 + pair (0 xy, 1 yz, 2 xz)
    static __device__ __forceinline__ int mixed_job(int q) {
      switch (q) {
        case 0: return (IUX + 0) * 4 + 0;   // u_x,xy  (grad div u, y)
        case 1: return (IUX + 0) * 4 + 2;   // u_x,xz  (z)
        case 2: return (IUX + 1) * 4 + 0;   // u_y,xy  (x)
        case 3: return (IUX + 1) * 4 + 1;   // u_y,yz  (z)
        case 4: return (IUX + 2) * 4 + 2;   // u_z,xz  (x)
        case 5: return (IUX + 2) * 4 + 1;   // u_z,yz  (y)
        case 6: return (IAX + 0) * 4 + 0;   // A_1,xy
        case 7: return (IAX + 1) * 4 + 0;   // A_2,xy
        case 8: return (IAX + 0) * 4 + 2;   // A_1,xz
        case 9: return (IAX + 2) * 4 + 2;   // A_3,xz
        case 10: return (IAX + 1) * 4 + 1;  // A_2,yz
        case 11: return (IAX + 2) * 4 + 1;  // A_3,yz
        case 12: return (IAX + 2) * 4 + 0;  // A_3,xy (div B only)
        case 13: return (IAX + 1) * 4 + 2;  // A_2,xz (div B only)
        default: return (IAX + 0) * 4 + 1;  // A_1,yz (div B only)
      }
    }

    __device__ __forceinline__ void step(const T* const pl[7], int x, int y, int z, int z1, const StepFlags<T>& fl,
                                         typename AccOf<T>::type& acc, T& dt1max) {
      const St st{pl, F};
      const long long cidx = (long long)(z + 3) * ps + (long long)(y + 3) * px + xoff + x;
      T dfo[NF];
#pragma unroll
      for (int k = 0; k < NF; ++k) dfo[k] = dfnext[k];
      if (fl.read_df && z + 1 < z1) {
#pragma unroll
        for (int k = 0; k < NF; ++k) dfnext[k] = dfp[k * fs + cidx + ps];
      }
      if (fl.read_df && z + kDfPrefetch < z1) {
#pragma unroll
        for (int k = 0; k < NF; ++k) prefetch_l2(dfp + k * fs + cidx + kDfPrefetch * ps);
      }
      CellIn<T> c;
      if constexpr (is_dd<T>::value) gather_compact(st, c, fl.want_diag);
      else gather(st, c, fl.want_diag);
      if constexpr (UPW) {
        if (upw) upwinding(st, c, upw);
      }
      T fc[3] = {T(0), T(0), T(0)};
      if (forcing) {   // forcing_cont 'ABC', forcing.f90:5894-5896
        fc[0] = P.fact * (P.abc_c * fsz + (P.fact2 * P.abc_b) * fcy);
        fc[1] = P.fact * (P.abc_a * fsx + (P.fact2 * P.abc_c) * fcz);
        fc[2] = P.fact * (P.abc_b * fsy + (P.fact2 * P.abc_a) * fcx);
        if (z + 1 < z1) { fsz = sinz[z + 4]; fcz = cosz[z + 4]; }
      }
      T dfn[NF];
      cell_rhs<T, NF>(c, P, F, fc, forcing, iso, vheat, oheat, dfo, fl.alpha, dfn, fl.want_cfl, fl.want_diag, acc,
                      dt1max, UPW ? upw : 0);

      // ---- 2N update (timestep.f90:160) and periodic ghost images ----
      T fnew[NF], dsto[NF];
#pragma unroll
      for (int k = 0; k < NF; ++k) {
        const T fc0 = st.v(0, k, 0, 0);
        if (!fl.comp) {
          fnew[k] = fc0 + fl.dtb * dfn[k];
          dsto[k] = dfn[k];
        } else {
          // TwoSum of fc0 + y; on substep 1, y carries the previous step's compensation
          const T yv = (fl.s == 0) ? (fl.dtb * dfn[k] + dfo[k]) : fl.dtb * dfn[k];
          const T t = fc0 + yv;
          const T bp = t - fc0;
          const T e = (fc0 - (t - bp)) + (yv - bp);
          fnew[k] = t;
          dsto[k] = (fl.s < 2) ? (dfn[k] + e * fl.cinv) : e;
        }
      }
      if (fl.write_df) {
#pragma unroll
        for (int k = 0; k < NF; ++k) dfp[k * fs + cidx] = dsto[k];
      }
#pragma unroll
      for (int k = 0; k < NF; ++k) fout[k * fs + cidx] = fnew[k];
      const bool edge = (x < 3) | (x >= nx - 3) | (y < 3) | (y >= ny - 3) | (z < 3) | (z >= nz - 3);
      if (edge) {
        const Images ix(x, nx), iy(y, ny), iz(z, nz);
#pragma unroll
        for (int a = 0; a < 2; ++a)
#pragma unroll
          for (int b = 0; b < 2; ++b)
#pragma unroll
            for (int e = 0; e < 2; ++e) {
              if ((a == 0 && b == 0 && e == 0) || a >= iz.n || b >= iy.n || e >= ix.n) continue;
              const long long gi = (long long)(iz.v[a] + 3) * ps + (long long)(iy.v[b] + 3) * px + xoff + ix.v[e];
#pragma unroll
              for (int k = 0; k < NF; ++k) fout[k * fs + gi] = fnew[k];
            }
      }
    }

    __device__ __forceinline__ void cfl(const T* const pl[7], T& dt1max) {
      const St st{pl, F};
      const T uu[3] = {st.v(0, 0, 0, 0), st.v(0, 1, 0, 0), st.v(0, 2, 0, 0)};
      const T bb[3] = {st.der(IAX + 2, 1) - st.der(IAX + 1, 2), st.der(IAX + 0, 2) - st.der(IAX + 2, 0),
                       st.der(IAX + 1, 0) - st.der(IAX + 0, 1)};
      const T d = cell_cfl_only<T, NF>(P, F, uu, st.v(0, ILNRHO, 0, 0), ENTROPY ? st.v(0, ISS, 0, 0) : T(0), bb, iso);
      dt1max = (d > dt1max || d != d) ? d : dt1max;
    }
  };
};

}  // namespace pcgb
