// cell_pair.cuh -- FP32 cell policy on field pairs packed as float2.
//
// The device f and df arrays hold four slices of float2 per cell:
//   P0 = (ux, ax), P1 = (uy, ay), P2 = (uz, az), P3 = (lnrho, ss) (or (lnrho, 0)
// without entropy).  The members of P0..P2 need exactly the same stencils:
// ux and ax both need x, y, z, xx, yy, zz and the mixed xy and xz derivatives
// (u_x,xy / u_x,xz enter grad div u, A_1,xy / A_1,xz enter J = curl curl A);
// likewise (uy, ay) need xy and yz, (uz, az) need xz and yz.  So every stencil
// is one 8-byte shared load per point and packed f32x2 arithmetic
// (FADD2/FMUL2/FFMA2) for two fields at once, with no idle lane.
#pragma once

#include "cell_physics.cuh"
#include "helical_force.cuh"

namespace pcgb {

__device__ __forceinline__ float2 p_add(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 p_sub(float2 a, float2 b) { return __fadd2_rn(a, make_float2(-b.x, -b.y)); }
__device__ __forceinline__ float2 p_mul(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 p_fma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 p_splat(float v) { return make_float2(v, v); }

// UPW: compiled with the upwind corrections (lupw_uu, lupw_lnrho) and with the
// random helical force added in the last substep's update (the reference's
// timing-run physics); the plain variants keep their registers.
template <int NF, int TX, int TY, bool UPW = false>
struct PairCell {
  using T = float;
  using Elem = float2;
  static constexpr int NSLICE = 4;
  static constexpr int BW = TX + 8, BH = TY + 6, FO = BW * BH;
  static constexpr int ILNRHO = 3, ISS = 4, IAX = NF - 3;
  static constexpr bool ENTROPY = (NF == 8);

  struct St {
    const float2* const* pl;
    const Fac<float>& F;
    __device__ __forceinline__ float2 v(int dz, int p, int dy, int dx) const {
      return pl[dz + 3][p * FO + dy * BW + dx];
    }
    // der_main (deriv.f90:127-129) on both members of pair p
    __device__ __forceinline__ float2 der(int p, int j) const {
      float2 a, b, c;
      float fac;
      if (j == 0) {
        a = p_sub(v(0, p, 0, 1), v(0, p, 0, -1)); b = p_sub(v(0, p, 0, 2), v(0, p, 0, -2));
        c = p_sub(v(0, p, 0, 3), v(0, p, 0, -3)); fac = F.fx;
      } else if (j == 1) {
        a = p_sub(v(0, p, 1, 0), v(0, p, -1, 0)); b = p_sub(v(0, p, 2, 0), v(0, p, -2, 0));
        c = p_sub(v(0, p, 3, 0), v(0, p, -3, 0)); fac = F.fy;
      } else {
        a = p_sub(v(1, p, 0, 0), v(-1, p, 0, 0)); b = p_sub(v(2, p, 0, 0), v(-2, p, 0, 0));
        c = p_sub(v(3, p, 0, 0), v(-3, p, 0, 0)); fac = F.fz;
      }
      const float2 t = p_add(p_fma(p_splat(-9.f), b, p_mul(p_splat(45.f), a)), c);
      return p_mul(p_splat(fac), t);
    }
    // der2_main 'standard' (deriv.f90:39-41, :502-506)
    __device__ __forceinline__ float2 der2(int p, int j) const {
      float2 s1, s2, s3;
      float fac;
      if (j == 0) {
        s1 = p_add(v(0, p, 0, 1), v(0, p, 0, -1)); s2 = p_add(v(0, p, 0, 2), v(0, p, 0, -2));
        s3 = p_add(v(0, p, 0, 3), v(0, p, 0, -3)); fac = F.sx;
      } else if (j == 1) {
        s1 = p_add(v(0, p, 1, 0), v(0, p, -1, 0)); s2 = p_add(v(0, p, 2, 0), v(0, p, -2, 0));
        s3 = p_add(v(0, p, 3, 0), v(0, p, -3, 0)); fac = F.sy;
      } else {
        s1 = p_add(v(1, p, 0, 0), v(-1, p, 0, 0)); s2 = p_add(v(2, p, 0, 0), v(-2, p, 0, 0));
        s3 = p_add(v(3, p, 0, 0), v(-3, p, 0, 0)); fac = F.sz;
      }
      float2 t = p_mul(p_splat((float)(-490.0 / 180.0)), v(0, p, 0, 0));
      t = p_fma(p_splat((float)(270.0 / 180.0)), s1, t);
      t = p_fma(p_splat((float)(-27.0 / 180.0)), s2, t);
      t = p_fma(p_splat((float)(2.0 / 180.0)), s3, t);
      return p_mul(p_splat(fac), t);
    }
    // der6_main with upwind=T (deriv.f90:936-1010) on both members of pair p
    __device__ __forceinline__ float2 del6u(int p, int j) const {
      float2 s1, s2, s3;
      float fac;
      if (j == 0) {
        s1 = p_add(v(0, p, 0, 1), v(0, p, 0, -1)); s2 = p_add(v(0, p, 0, 2), v(0, p, 0, -2));
        s3 = p_add(v(0, p, 0, 3), v(0, p, 0, -3)); fac = F.fx;
      } else if (j == 1) {
        s1 = p_add(v(0, p, 1, 0), v(0, p, -1, 0)); s2 = p_add(v(0, p, 2, 0), v(0, p, -2, 0));
        s3 = p_add(v(0, p, 3, 0), v(0, p, -3, 0)); fac = F.fy;
      } else {
        s1 = p_add(v(1, p, 0, 0), v(-1, p, 0, 0)); s2 = p_add(v(2, p, 0, 0), v(-2, p, 0, 0));
        s3 = p_add(v(3, p, 0, 0), v(-3, p, 0, 0)); fac = F.fz;
      }
      float2 t = p_mul(p_splat(-20.f), v(0, p, 0, 0));
      t = p_fma(p_splat(15.f), s1, t);
      t = p_fma(p_splat(-6.f), s2, t);
      return p_mul(p_splat(fac), p_add(t, s3));
    }
    // calc_del6_for_upwind (sub.f90:7491-7539) for the first member of pair p: sum_j |u_j| D6_j
    __device__ __forceinline__ float upwind(int p, const float u[3]) const {
      return (fabsf(u[0]) * del6u(p, 0).x + fabsf(u[1]) * del6u(p, 1).x) + fabsf(u[2]) * del6u(p, 2).x;
    }
    // derij_main bidiagonal (deriv.f90:1387-1447); (a,b) with a<b: 0=x,1=y,2=z
    __device__ __forceinline__ float2 derij(int p, int a, int b) const {
      float2 t[3];
#pragma unroll
      for (int d = 1; d <= 3; ++d) {
        if (a == 0 && b == 1)
          t[d - 1] = p_sub(p_add(p_sub(v(0, p, d, d), v(0, p, d, -d)), v(0, p, -d, -d)), v(0, p, -d, d));
        else if (a == 1 && b == 2)
          t[d - 1] = p_sub(p_add(p_sub(v(d, p, d, 0), v(-d, p, d, 0)), v(-d, p, -d, 0)), v(d, p, -d, 0));
        else
          t[d - 1] = p_sub(p_add(p_sub(v(d, p, 0, d), v(d, p, 0, -d)), v(-d, p, 0, -d)), v(-d, p, 0, d));
      }
      const float fac = (a == 0 && b == 1) ? F.mxy : ((a == 1 && b == 2) ? F.myz : F.mxz);
      const float2 r = p_fma(p_splat(2.f), t[2], p_fma(p_splat(-27.f), t[1], p_mul(p_splat(270.f), t[0])));
      return p_mul(p_splat(fac), r);
    }
  };

  struct Tile {
    Fac<float> F;
    Phys<float> P;
    float2* fout;
    float2* dfp;
    long long ps, fs;
    int px, xoff, nx, ny, nz;
    bool forcing, iso, vheat, oheat;
    float fsx, fcx, fsy, fcy;
    const float* sinz;
    const float* cosz;
    float fsz, fcz;   // sin/cos(kf z) of the current plane, prefetched one plane ahead
    float2 dfnext[4];
    int upw;          // UPW_* bits
    const float* htab;    // helical forcing tables (float copy) fused into the last substep, or null
    int htarget;
    float hpr, hpi;       // fx fy of this column
    float hc1[3], hc2[3]; // coef1, coef2 of the step

    __device__ __forceinline__ void begin(const PcgbBoxDev& B, int inb, int x, int y, int z0, bool active,
                                          bool mode_cfl, const StepFlags<float>& fl) {
      make_fac(F, B);
      make_phys(P, B);
      fout = reinterpret_cast<float2*>(B.f[inb ^ 1]);
      dfp = reinterpret_cast<float2*>(B.df);
      ps = B.ps; fs = B.fs; px = B.px; xoff = B.xoff; nx = B.nx; ny = B.ny; nz = B.nz;
      forcing = B.lforcing != 0; iso = B.isothermal != 0; vheat = B.lviscosity_heat != 0; oheat = B.lohmic_heat != 0;
      upw = UPW ? B.lupw : 0;
      htab = UPW ? B.hel_tab : nullptr;
      htarget = B.hel_target;
      if constexpr (UPW) {
        if (htab != nullptr && fl.s == 2 && active) {   // the step's tables are in place before the last substep
          helical_fxy(htab, nx, x, y, hpr, hpi);
#pragma unroll
          for (int c = 0; c < 3; ++c) { hc1[c] = htab[c]; hc2[c] = htab[3 + c]; }
        }
      }
      const float* sinx = reinterpret_cast<const float*>(B.forc);
      const float* cosx = sinx + B.px;
      const float* siny = cosx + B.px;
      const float* cosy = siny + B.my;
      sinz = cosy + B.my;
      cosz = sinz + B.mz;
      fsx = fcx = fsy = fcy = fsz = fcz = 0.f;
      if (forcing && active) {
        fsx = sinx[x + 3]; fcx = cosx[x + 3]; fsy = siny[y + 3]; fcy = cosy[y + 3];
        fsz = sinz[z0 + 3]; fcz = cosz[z0 + 3];
      }
#pragma unroll
      for (int p = 0; p < 4; ++p) dfnext[p] = make_float2(0.f, 0.f);
      if (fl.read_df && active && !mode_cfl) {
        const long long c0 = (long long)(z0 + 3) * ps + (long long)(y + 3) * px + xoff + x;
#pragma unroll
        for (int p = 0; p < 4; ++p) dfnext[p] = dfp[p * fs + c0];
      }
    }

    __device__ __forceinline__ void step(const float2* const pl[7], int x, int y, int z, int z1,
                                         const StepFlags<float>& fl, AccF& acc, float& dt1max) {
      const St st{pl, F};
      const long long cidx = (long long)(z + 3) * ps + (long long)(y + 3) * px + xoff + x;
      float hzr = 0.f, hzi = 0.f;   // fz of this plane, loaded ahead of its use at the update
      if constexpr (UPW) {
        if (htab != nullptr && fl.s == 2) {
          const float* fz = htab + 8 + 2 * nx + 2 * ny;
          hzr = fz[2 * z];
          hzi = fz[2 * z + 1];
        }
      }
      float2 dfo2[4];
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
      // gather derivatives pair by pair
      const float2 c0 = st.v(0, 0, 0, 0), c1 = st.v(0, 1, 0, 0), c2 = st.v(0, 2, 0, 0), c3 = st.v(0, 3, 0, 0);
      CellIn<float> c;
      c.uu[0] = c0.x; c.uu[1] = c1.x; c.uu[2] = c2.x;
      c.aa[0] = c0.y; c.aa[1] = c1.y; c.aa[2] = c2.y;
      c.lnrho = c3.x;
      c.ss = ENTROPY ? c3.y : 0.f;
#pragma unroll
      for (int p = 0; p < 3; ++p) {
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          const float2 d1 = st.der(p, j);
          c.uij[p][j] = d1.x;
          c.aij[p][j] = d1.y;
          const float2 d2 = st.der2(p, j);
          c.a2[p][j] = d2.y;
          c.del2u[p] = (j == 0) ? d2.x : c.del2u[p] + d2.x;   // (f0 + f1) + f2
          // u_p,pp for the diagonal of grad div u
          if (j == p) c.graddivu[p] = d2.x;
        }
      }
      const float2 xy0 = st.derij(0, 0, 1);   // (u_x,xy, A_1,xy)
      const float2 xz0 = st.derij(0, 0, 2);   // (u_x,xz, A_1,xz)
      const float2 xy1 = st.derij(1, 0, 1);   // (u_y,xy, A_2,xy)
      const float2 yz1 = st.derij(1, 1, 2);   // (u_y,yz, A_2,yz)
      const float2 xz2 = st.derij(2, 0, 2);   // (u_z,xz, A_3,xz)
      const float2 yz2 = st.derij(2, 1, 2);   // (u_z,yz, A_3,yz)
      // grad div u (del2v_etc, sub.f90:2610): graddiv_i = (u_x,xi + u_y,yi) + u_z,zi
      const float gx = c.graddivu[0], gy = c.graddivu[1], gz = c.graddivu[2];
      c.graddivu[0] = (gx + xy1.x) + xz2.x;
      c.graddivu[1] = (xy0.x + gy) + yz2.x;
      c.graddivu[2] = (xz0.x + yz1.x) + gz;
      c.a1xy = xy0.y; c.a1xz = xz0.y; c.a2xy = xy1.y; c.a2yz = yz1.y; c.a3xz = xz2.y; c.a3yz = yz2.y;
      c.a3xy = c.a2xz = c.a1yz = 0.f;
      if (fl.want_diag) {
        c.a3xy = st.derij(2, 0, 1).y; c.a2xz = st.derij(1, 0, 2).y; c.a1yz = st.derij(0, 1, 2).y;
      }
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        const float2 g = st.der(3, j);   // (lnrho, ss)
        c.glnrho[j] = g.x;
        c.gss[j] = ENTROPY ? g.y : 0.f;
      }
      if (ENTROPY) {
        const float2 l0 = st.der2(3, 0), l1 = st.der2(3, 1), l2 = st.der2(3, 2);
        const float2 ls = p_add(p_add(l0, l1), l2);
        c.del2lnrho = ls.x;
        c.del2ss = ls.y;
      } else {
        c.del2lnrho = c.del2ss = 0.f;
      }
      if constexpr (UPW) {
        if (upw & UPW_UU) {
#pragma unroll
          for (int p = 0; p < 3; ++p) c.upw_u[p] = st.upwind(p, c.uu);
        }
        if (upw & UPW_LNRHO) c.upw_lnrho = st.upwind(3, c.uu);
      }
      float fc[3] = {0.f, 0.f, 0.f};
      if (forcing) {   // forcing_cont 'ABC', forcing.f90:5894-5896
        fc[0] = P.fact * (P.abc_c * fsz + (P.fact2 * P.abc_b) * fcy);
        fc[1] = P.fact * (P.abc_a * fsx + (P.fact2 * P.abc_c) * fcz);
        fc[2] = P.fact * (P.abc_b * fsy + (P.fact2 * P.abc_a) * fcx);
        if (z + 1 < z1) { fsz = sinz[z + 4]; fcz = cosz[z + 4]; }
      }
      float dfo[NF], dfn[NF];
      dfo[0] = dfo2[0].x; dfo[1] = dfo2[1].x; dfo[2] = dfo2[2].x; dfo[ILNRHO] = dfo2[3].x;
      if (ENTROPY) dfo[ISS] = dfo2[3].y;
      dfo[IAX] = dfo2[0].y; dfo[IAX + 1] = dfo2[1].y; dfo[IAX + 2] = dfo2[2].y;
      cell_rhs<float, NF>(c, P, F, fc, forcing, iso, vheat, oheat, dfo, fl.alpha, dfn, fl.want_cfl, fl.want_diag,
                          acc, dt1max, UPW ? upw : 0);

      // ---- 2N update (timestep.f90:160), compensated in FP32, per pair ----
      float2 dn[4];
      dn[0] = make_float2(dfn[0], dfn[IAX]);
      dn[1] = make_float2(dfn[1], dfn[IAX + 1]);
      dn[2] = make_float2(dfn[2], dfn[IAX + 2]);
      dn[3] = make_float2(dfn[ILNRHO], ENTROPY ? dfn[ISS] : 0.f);
      const float2 cur[4] = {c0, c1, c2, c3};
      const float2 dtb2 = p_splat(fl.dtb);
      float2 fnew[4], dsto[4];
#pragma unroll
      for (int p = 0; p < 4; ++p) {
        if (!fl.comp) {
          fnew[p] = p_fma(dtb2, dn[p], cur[p]);
          dsto[p] = dn[p];
        } else {
          const float2 yv = (fl.s == 0) ? p_fma(dtb2, dn[p], dfo2[p]) : p_mul(dtb2, dn[p]);
          const float2 t = p_add(cur[p], yv);
          const float2 bp = p_sub(t, cur[p]);
          const float2 e = p_add(p_sub(cur[p], p_sub(t, bp)), p_sub(yv, bp));
          fnew[p] = t;
          dsto[p] = (fl.s < 2) ? p_fma(e, p_splat(fl.cinv), dn[p]) : e;
        }
      }
      if (!ENTROPY) { fnew[3].y = 0.f; dsto[3].y = 0.f; }
      if constexpr (UPW) {
        if (htab != nullptr && fl.s == 2) {   // forcing_hel after the step (addforce, forcing.f90:1307)
          // (fx fy) fz and Re[(coef1 + i coef2) fxyz], as helical_fz computes them
          const float qr = rsub(rmul(hpr, hzr), rmul(hpi, hzi)), qi = radd(rmul(hpr, hzi), rmul(hpi, hzr));
#pragma unroll
          for (int p = 0; p < 3; ++p) {
            const float fh = rsub(rmul(hc1[p], qr), rmul(hc2[p], qi));
            if (htarget) fnew[p].y = __fadd_rn(fnew[p].y, fh);
            else fnew[p].x = __fadd_rn(fnew[p].x, fh);
          }
        }
      }
      if (fl.write_df) {
#pragma unroll
        for (int p = 0; p < 4; ++p) dfp[p * fs + cidx] = dsto[p];
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

    __device__ __forceinline__ void cfl(const float2* const pl[7], float& dt1max) {
      const St st{pl, F};
      const float2 c0 = st.v(0, 0, 0, 0), c1 = st.v(0, 1, 0, 0), c2 = st.v(0, 2, 0, 0), c3 = st.v(0, 3, 0, 0);
      const float uu[3] = {c0.x, c1.x, c2.x};
      // B = curl A needs A_3,y A_2,z A_1,z A_3,x A_2,x A_1,y (the .y lanes)
      const float bb[3] = {st.der(2, 1).y - st.der(1, 2).y, st.der(0, 2).y - st.der(2, 0).y,
                           st.der(1, 0).y - st.der(0, 1).y};
      const float d = cell_cfl_only<float, NF>(P, F, uu, c3.x, ENTROPY ? c3.y : 0.f, bb, iso);
      dt1max = (d > dt1max || d != d) ? d : dt1max;
    }
  };
};

}  // namespace pcgb
