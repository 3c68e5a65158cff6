// cell_ddpair.cuh -- double-float cell policy on field pairs packed as dd2.
//
// Same pairing as the FP32 pair layout (cell_pair.cuh): four slices per cell,
// P0 = (ux, ax), P1 = (uy, ay), P2 = (uz, az), P3 = (lnrho, ss) (or (lnrho, 0)),
// each element a 16-byte dd2 holding both members' hi and lo parts, so every
// stencil operation is one packed f32x2 double-float operation for two
// fields.  The stencil expressions mirror ScalarCell's operation by operation,
// and dd2 arithmetic equals dd arithmetic lane by lane: a pair tile gives the
// same bits as a field-major double-float tile.  The physics (cell_rhs) runs
// on scalar dd values taken from the lanes.  Stencil code is looped over pairs
// and mixed-derivative jobs (results in thread-local arrays) to keep the
// z-iteration's code within the instruction caches.
#pragma once

#include "cell_physics.cuh"

namespace pcgb {

// UPW: compiled with the upwind corrections (lupw_uu, lupw_lnrho).
template <int NF, int TX, int TY, bool UPW = false>
struct DDPairCell {
  using T = dd;
  using Elem = dd2;
  static constexpr int NSLICE = 4;
  static constexpr int BW = TX + 8, BH = TY + 6, FO = BW * BH;
  static constexpr int ILNRHO = 3, ISS = 4, IAX = NF - 3;
  static constexpr bool ENTROPY = (NF == 8);

  struct St {
    const dd2* const* pl;
    const Fac<dd>& F;
    __device__ __forceinline__ dd2 v(int dz, int p, int dy, int dx) const { return pl[dz + 3][p * FO + dy * BW + dx]; }
    // der_main, deriv.f90:127-129 (x), :140-142 (y), :158-160 (z)
    __device__ __forceinline__ dd2 der(int p, int j) const {
      dd2 a, b, c;
      dd fac;
      if (j == 0) {
        a = v(0, p, 0, 1) - v(0, p, 0, -1); b = v(0, p, 0, 2) - v(0, p, 0, -2); c = v(0, p, 0, 3) - v(0, p, 0, -3);
        fac = F.fx;
      } else if (j == 1) {
        a = v(0, p, 1, 0) - v(0, p, -1, 0); b = v(0, p, 2, 0) - v(0, p, -2, 0); c = v(0, p, 3, 0) - v(0, p, -3, 0);
        fac = F.fy;
      } else {
        a = v(1, p, 0, 0) - v(-1, p, 0, 0); b = v(2, p, 0, 0) - v(-2, p, 0, 0); c = v(3, p, 0, 0) - v(-3, p, 0, 0);
        fac = F.fz;
      }
      return dd2_splat(fac) * ((dd2_scale(a, 45.f) - dd2_scale(b, 9.f)) + c);
    }
    // der2_main 'standard', deriv.f90:39-41, :502-506
    __device__ __forceinline__ dd2 der2(int p, int j) const {
      const dd2 c0 = dd2_splat(dd(-490.0 / 180.0)), c1 = dd2_splat(dd(270.0 / 180.0));
      const dd2 c2 = dd2_splat(dd(-27.0 / 180.0)), c3 = dd2_splat(dd(2.0 / 180.0));
      const dd2 f0 = v(0, p, 0, 0);
      dd2 s1, s2, s3;
      dd fac;
      if (j == 0) {
        s1 = v(0, p, 0, 1) + v(0, p, 0, -1); s2 = v(0, p, 0, 2) + v(0, p, 0, -2); s3 = v(0, p, 0, 3) + v(0, p, 0, -3);
        fac = F.sx;
      } else if (j == 1) {
        s1 = v(0, p, 1, 0) + v(0, p, -1, 0); s2 = v(0, p, 2, 0) + v(0, p, -2, 0); s3 = v(0, p, 3, 0) + v(0, p, -3, 0);
        fac = F.sy;
      } else {
        s1 = v(1, p, 0, 0) + v(-1, p, 0, 0); s2 = v(2, p, 0, 0) + v(-2, p, 0, 0); s3 = v(3, p, 0, 0) + v(-3, p, 0, 0);
        fac = F.sz;
      }
      return dd2_splat(fac) * (((c0 * f0 + c1 * s1) + c2 * s2) + c3 * s3);
    }
    // der6_main with upwind=T, deriv.f90:936-1010, in ScalarCell::St::del6u's order
    __device__ __forceinline__ dd2 del6u(int p, int j) const {
      const dd2 f0 = v(0, p, 0, 0);
      dd2 s1, s2, s3;
      dd fac;
      if (j == 0) {
        s1 = v(0, p, 0, 1) + v(0, p, 0, -1); s2 = v(0, p, 0, 2) + v(0, p, 0, -2); s3 = v(0, p, 0, 3) + v(0, p, 0, -3);
        fac = F.fx;
      } else if (j == 1) {
        s1 = v(0, p, 1, 0) + v(0, p, -1, 0); s2 = v(0, p, 2, 0) + v(0, p, -2, 0); s3 = v(0, p, 3, 0) + v(0, p, -3, 0);
        fac = F.fy;
      } else {
        s1 = v(1, p, 0, 0) + v(-1, p, 0, 0); s2 = v(2, p, 0, 0) + v(-2, p, 0, 0); s3 = v(3, p, 0, 0) + v(-3, p, 0, 0);
        fac = F.fz;
      }
      return dd2_splat(fac) * (((dd2_scale(f0, -20.f) + dd2_scale(s1, 15.f)) - dd2_scale(s2, 6.f)) + s3);
    }
    // calc_del6_for_upwind, sub.f90:7491-7539, for the first member of pair p
    __device__ __forceinline__ dd upwind(int p, const dd u[3]) const {
      return (tabs(u[0]) * dd2_lane0(del6u(p, 0)) + tabs(u[1]) * dd2_lane0(del6u(p, 1))) +
             tabs(u[2]) * dd2_lane0(del6u(p, 2));
    }
    // derij_main bidiagonal, deriv.f90:1387-1447; pr: 0 = xy, 1 = yz, 2 = xz
    __device__ __forceinline__ dd2 derij(int p, int pr) const {
      dd2 t[3];
#pragma unroll
      for (int d = 1; d <= 3; ++d) {
        if (pr == 0)
          t[d - 1] = ((v(0, p, d, d) - v(0, p, d, -d)) + v(0, p, -d, -d)) - v(0, p, -d, d);
        else if (pr == 1)
          t[d - 1] = ((v(d, p, d, 0) - v(-d, p, d, 0)) + v(-d, p, -d, 0)) - v(d, p, -d, 0);
        else
          t[d - 1] = ((v(d, p, 0, d) - v(d, p, 0, -d)) + v(-d, p, 0, -d)) - v(-d, p, 0, d);
      }
      const dd fac = (pr == 0) ? F.mxy : ((pr == 1) ? F.myz : F.mxz);
      return dd2_splat(fac) * ((dd2_scale(t[0], 270.f) - dd2_scale(t[1], 27.f)) + dd2_scale(t[2], 2.f));
    }
  };

  struct Tile {
    Fac<dd> F;
    Phys<dd> P;
    dd2* fout;
    dd2* dfp;
    long long ps, fs;
    int px, xoff, nx, ny, nz;
    bool forcing, iso, vheat, oheat;
    dd fsx, fcx, fsy, fcy;
    const dd* sinz;
    const dd* cosz;
    dd fsz, fcz;   // sin/cos(kf z) of the current plane, prefetched one plane ahead
    dd2 dfnext[4];
    int upw;       // UPW_* bits

    __device__ __forceinline__ void begin(const PcgbBoxDev& B, int inb, int x, int y, int z0, bool active,
                                          bool mode_cfl, const StepFlags<dd>& fl) {
      make_fac(F, B);
      make_phys(P, B);
      fout = reinterpret_cast<dd2*>(B.f[inb ^ 1]);
      dfp = reinterpret_cast<dd2*>(B.df);
      ps = B.ps; fs = B.fs; px = B.px; xoff = B.xoff; nx = B.nx; ny = B.ny; nz = B.nz;
      forcing = B.lforcing != 0; iso = B.isothermal != 0; vheat = B.lviscosity_heat != 0; oheat = B.lohmic_heat != 0;
      upw = UPW ? B.lupw : 0;
      const dd* sinx = reinterpret_cast<const dd*>(B.forc);
      const dd* cosx = sinx + B.px;
      const dd* siny = cosx + B.px;
      const dd* cosy = siny + B.my;
      sinz = cosy + B.my;
      cosz = sinz + B.mz;
      fsx = fcx = fsy = fcy = fsz = fcz = dd(0);
      if (forcing && active) {
        fsx = sinx[x + 3]; fcx = cosx[x + 3]; fsy = siny[y + 3]; fcy = cosy[y + 3];
        fsz = sinz[z0 + 3]; fcz = cosz[z0 + 3];
      }
      const dd2 zero = dd2_pack(dd(0), dd(0));
#pragma unroll
      for (int p = 0; p < 4; ++p) dfnext[p] = zero;
      if (fl.read_df && active && !mode_cfl) {
        const long long c0 = (long long)(z0 + 3) * ps + (long long)(y + 3) * px + xoff + x;
#pragma unroll
        for (int p = 0; p < 4; ++p) dfnext[p] = dfp[p * fs + c0];
      }
    }

    // Field values and stencil derivatives of one cell into the scalar
    // inputs of cell_rhs, with ScalarCell::gather_compact's expressions.
    static __device__ __forceinline__ void gather(const St& st, CellIn<dd>& c, bool want_diag) {
      dd2 d1[4][3], d2[4][3], m[9];
#pragma unroll 1
      for (int p = 0; p < 4; ++p) {
#pragma unroll
        for (int j = 0; j < 3; ++j) d1[p][j] = st.der(p, j);
        if (p < 3 || ENTROPY) {
#pragma unroll
          for (int j = 0; j < 3; ++j) d2[p][j] = st.der2(p, j);
        }
      }
      // mixed-derivative jobs (pair, direction pair 0 xy / 1 yz / 2 xz):
      // 0 (P0,xy) 1 (P0,xz) 2 (P1,xy) 3 (P1,yz) 4 (P2,xz) 5 (P2,yz); div B only: 6 (P2,xy) 7 (P1,xz) 8 (P0,yz)
      const int njob = want_diag ? 9 : 6;
#pragma unroll 1
      for (int q = 0; q < njob; ++q) {
        const int code = (q == 0) ? 0 : (q == 1) ? 2 : (q == 2) ? 4 : (q == 3) ? 5 : (q == 4) ? 10 : (q == 5) ? 9
                       : (q == 6) ? 8 : (q == 7) ? 6 : 1;   // pair * 4 + direction pair
        m[q] = st.derij(code >> 2, code & 3);
      }
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        const dd2 f0 = st.v(0, i, 0, 0);
        c.uu[i] = dd2_lane0(f0);
        c.aa[i] = dd2_lane1(f0);
#pragma unroll
        for (int jj = 0; jj < 3; ++jj) {
          c.uij[i][jj] = dd2_lane0(d1[i][jj]);
          c.aij[i][jj] = dd2_lane1(d1[i][jj]);
          c.a2[i][jj] = dd2_lane1(d2[i][jj]);
        }
        c.del2u[i] = (dd2_lane0(d2[i][0]) + dd2_lane0(d2[i][1])) + dd2_lane0(d2[i][2]);
      }
      // grad div u (sub.f90:2646-2656): graddiv_i = (u_x,xi + u_y,yi) + u_z,zi
      c.graddivu[0] = (dd2_lane0(d2[0][0]) + dd2_lane0(m[2])) + dd2_lane0(m[4]);
      c.graddivu[1] = (dd2_lane0(m[0]) + dd2_lane0(d2[1][1])) + dd2_lane0(m[5]);
      c.graddivu[2] = (dd2_lane0(m[1]) + dd2_lane0(m[3])) + dd2_lane0(d2[2][2]);
      const dd2 f3 = st.v(0, 3, 0, 0);
      c.lnrho = dd2_lane0(f3);
#pragma unroll
      for (int jj = 0; jj < 3; ++jj) c.glnrho[jj] = dd2_lane0(d1[3][jj]);
      if (ENTROPY) {
        c.ss = dd2_lane1(f3);
#pragma unroll
        for (int jj = 0; jj < 3; ++jj) c.gss[jj] = dd2_lane1(d1[3][jj]);
        c.del2lnrho = (dd2_lane0(d2[3][0]) + dd2_lane0(d2[3][1])) + dd2_lane0(d2[3][2]);
        c.del2ss = (dd2_lane1(d2[3][0]) + dd2_lane1(d2[3][1])) + dd2_lane1(d2[3][2]);
      } else {
        c.ss = dd(0); c.gss[0] = c.gss[1] = c.gss[2] = dd(0); c.del2lnrho = c.del2ss = dd(0);
      }
      c.a1xy = dd2_lane1(m[0]); c.a2xy = dd2_lane1(m[2]); c.a1xz = dd2_lane1(m[1]);
      c.a3xz = dd2_lane1(m[4]); c.a2yz = dd2_lane1(m[3]); c.a3yz = dd2_lane1(m[5]);
      c.a3xy = c.a2xz = c.a1yz = dd(0);
      if (want_diag) { c.a3xy = dd2_lane1(m[6]); c.a2xz = dd2_lane1(m[7]); c.a1yz = dd2_lane1(m[8]); }
    }

    __device__ __forceinline__ void step(const dd2* const pl[7], int x, int y, int z, int z1,
                                         const StepFlags<dd>& fl, Acc& acc, dd& dt1max) {
      const St st{pl, F};
      const long long cidx = (long long)(z + 3) * ps + (long long)(y + 3) * px + xoff + x;
      dd2 dfo2[4];
#pragma unroll
      for (int p = 0; p < 4; ++p) dfo2[p] = dfnext[p];
      if (fl.read_df && z + 1 < z1) {
#pragma unroll
        for (int p = 0; p < 4; ++p) dfnext[p] = dfp[p * fs + cidx + ps];
      }
      if (fl.read_df && z + kDfPrefetch < z1) {
#pragma unroll
        for (int p = 0; p < 4; ++p) prefetch_l2(dfp + p * fs + cidx + kDfPrefetch * ps);
      }
      CellIn<dd> c;
      gather(st, c, fl.want_diag);
      if constexpr (UPW) {
        if (upw & UPW_UU) {
#pragma unroll
          for (int p = 0; p < 3; ++p) c.upw_u[p] = st.upwind(p, c.uu);
        }
        if (upw & UPW_LNRHO) c.upw_lnrho = st.upwind(3, c.uu);
      }
      dd fc[3] = {dd(0), dd(0), dd(0)};
      if (forcing) {   // forcing_cont 'ABC', forcing.f90:5894-5896
        fc[0] = P.fact * (P.abc_c * fsz + (P.fact2 * P.abc_b) * fcy);
        fc[1] = P.fact * (P.abc_a * fsx + (P.fact2 * P.abc_c) * fcz);
        fc[2] = P.fact * (P.abc_b * fsy + (P.fact2 * P.abc_a) * fcx);
        if (z + 1 < z1) { fsz = sinz[z + 4]; fcz = cosz[z + 4]; }
      }
      dd dfo[NF], dfn[NF];
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        dfo[i] = dd2_lane0(dfo2[i]);
        dfo[IAX + i] = dd2_lane1(dfo2[i]);
      }
      dfo[ILNRHO] = dd2_lane0(dfo2[3]);
      if (ENTROPY) dfo[ISS] = dd2_lane1(dfo2[3]);
      cell_rhs<dd, NF>(c, P, F, fc, forcing, iso, vheat, oheat, dfo, fl.alpha, dfn, fl.want_cfl, fl.want_diag, acc,
                       dt1max, UPW ? upw : 0);

      // ---- 2N update (timestep.f90:160), per pair, in ScalarCell's order ----
      dd2 dn[4];
#pragma unroll
      for (int i = 0; i < 3; ++i) dn[i] = dd2_pack(dfn[i], dfn[IAX + i]);
      dn[3] = dd2_pack(dfn[ILNRHO], ENTROPY ? dfn[ISS] : dd(0));
      const dd2 dtb2 = dd2_splat(fl.dtb);
      dd2 fnew[4];
#pragma unroll
      for (int p = 0; p < 4; ++p) fnew[p] = st.v(0, p, 0, 0) + dtb2 * dn[p];
      if (!ENTROPY) { fnew[3].hi.y = 0.f; fnew[3].lo.y = 0.f; }
      if (fl.write_df) {
#pragma unroll
        for (int p = 0; p < 4; ++p) dfp[p * fs + cidx] = dn[p];
      }
#pragma unroll
      for (int p = 0; p < 4; ++p) fout[p * fs + cidx] = fnew[p];
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
              for (int p = 0; p < 4; ++p) fout[p * fs + gi] = fnew[p];
            }
      }
    }

    __device__ __forceinline__ void cfl(const dd2* const pl[7], dd& dt1max) {
      const St st{pl, F};
      const dd uu[3] = {dd2_lane0(st.v(0, 0, 0, 0)), dd2_lane0(st.v(0, 1, 0, 0)), dd2_lane0(st.v(0, 2, 0, 0))};
      // B = curl A: the A lanes of the pair derivatives, ScalarCell::cfl's expressions
      const dd bb[3] = {dd2_lane1(st.der(2, 1)) - dd2_lane1(st.der(1, 2)),
                        dd2_lane1(st.der(0, 2)) - dd2_lane1(st.der(2, 0)),
                        dd2_lane1(st.der(1, 0)) - dd2_lane1(st.der(0, 1))};
      const dd2 f3 = st.v(0, 3, 0, 0);
      const dd d = cell_cfl_only<dd, NF>(P, F, uu, dd2_lane0(f3), ENTROPY ? dd2_lane1(f3) : dd(0), bb, iso);
      dt1max = (d > dt1max || d != d) ? d : dt1max;
    }
  };
};

}  // namespace pcgb
