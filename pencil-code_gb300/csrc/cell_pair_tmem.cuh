// cell_pair_tmem.cuh -- FP32 packed-pair cell policy whose z-direction data lives
// in tensor memory (TMEM) instead of the shared-memory plane ring.
//
// Each thread owns one TMEM lane (its column of the tile).  When a plane
// arrives at the leading edge of the stencil (plane z+3 of output plane z),
// the thread reads its centre values and the x / y differences
// A_d = f(+d) - f(-d) (d = 1..3) that the xz / yz mixed derivatives need from
// shared memory once, and keeps them in tensor memory.  Output plane z then
// takes its z-stencils (der, der2) from the centre values of planes z-3..z+3
// and the bidiagonal xz / yz derivatives
//   derij = fac (270 t1 - 27 t2 + 2 t3),  t_d = A_d(z+d) - A_d(z-d)
// (deriv.f90:1387-1447) from there, with plane z's x / y stencils and the xy
// derivative from shared memory as before.  Shared-memory loads per cell drop
// from 149 to 107 and shared-memory wavefronts from 9.6 to 6.9 per cell;
// tensor memory has its own data path.  The tcgen05 loads and stores are
// warp-collective, so the driver runs step() on every lane of a warp that has
// a live cell (kWholeWarp) and the cell masks its global accesses and
// reductions with `active`.
//
// Two layouts, by the warps of the CTA (the SM's 512 columns are shared by
// the warps w, w+4, w+8 of a lane quarter):
//  * full (up to 8 warps, 256 columns a thread): a ring of 8 plane slots of 32
//    columns, [0,8) centres, [8,16) A_1, [16,24) A_2, [24,32) A_3;
//  * compact (12 warps, 160 columns a thread): centres in a ring of 8 slots
//    [0,64), A_1 in a ring of 4 [64,96), A_2 in a ring of 8 [96,160); A_3 of
//    plane z-3 is taken from the shared-memory ring (8 more shared loads).  The
//    A_1 slot of plane z+3 is the one plane z-1 used, so it is written only
//    after this step's loads have completed.
// With 12 warps (168 registers) the SM issues from three warps per scheduler
// instead of two.
//
// UPW: the variant with the upwind corrections (lupw_uu, lupw_lnrho; the z part
// of each 6th difference from the tensor-memory centres, the x and y parts from
// shared memory, in St::del6u's arithmetic) and with the random helical force
// added in the last substep's update, as PairCell does it (the reference's
// timing-run physics).
#pragma once

#include "cell_pair.cuh"

namespace pcgb {

// tcgen05 wrappers: 32 lanes x 32-bit, x8 columns; the address is the warp's
// lane quarter (bits 31..16) and column (bits 15..0).
__device__ __forceinline__ void tm_st8(uint32_t taddr, const float v[8]) {
  asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};" ::"r"(taddr),
               "r"(__float_as_uint(v[0])), "r"(__float_as_uint(v[1])), "r"(__float_as_uint(v[2])),
               "r"(__float_as_uint(v[3])), "r"(__float_as_uint(v[4])), "r"(__float_as_uint(v[5])),
               "r"(__float_as_uint(v[6])), "r"(__float_as_uint(v[7]))
               : "memory");
}
__device__ __forceinline__ void tm_ld8(uint32_t taddr, uint32_t r[8]) {
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
               : "r"(taddr)
               : "memory");
}
__device__ __forceinline__ void tm_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }
// wait::ld, then tie the loaded registers to it so that no use moves above the wait
__device__ __forceinline__ void tm_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }
__device__ __forceinline__ void tm_tie8(uint32_t r[8]) {
  asm volatile("" : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7])
               :: "memory");
}
__device__ __forceinline__ float2 u2f2(uint32_t a, uint32_t b) { return make_float2(__uint_as_float(a), __uint_as_float(b)); }

template <int NF, int TX, int TY, bool UPW = false>
struct PairCellTM {
  using Base = PairCell<NF, TX, TY, UPW>;
  using T = float;
  using Elem = float2;
  static constexpr int NSLICE = 4;
  static constexpr int BW = TX + 8, BH = TY + 6, FO = BW * BH;
  static constexpr int ILNRHO = 3, ISS = 4, IAX = NF - 3;
  static constexpr bool ENTROPY = (NF == 8);
  static constexpr int NWARP = (TX * TY + 31) / 32;
  // each A group is (A^x of P0, A^x of P2, A^y of P1, A^y of P2) as float2
  static constexpr bool kCompact = NWARP > 8;
  static constexpr int kColsPerThread = kCompact ? 160 : 256;
  static constexpr int kGroups = (NWARP + 3) / 4;                  // warps sharing a lane quarter
  static_assert(kColsPerThread * kGroups <= 512, "tensor memory holds 512 columns");
  static constexpr int kTmemCols = (kColsPerThread * kGroups <= 256) ? 256 : 512;   // a power of two
  static constexpr bool kWholeWarp = true;   // the driver calls step() for every lane of a live warp

  struct Tile : Base::Tile {
    uint32_t tm;   // this warp's lane quarter and column base
    int zfirst;

    // TMEM address of plane zz's centres (part 0) or A_part differences
    __device__ __forceinline__ uint32_t slot(int zz, int part) const {
      if constexpr (kCompact)
        return tm + (uint32_t)(part == 0 ? ((zz & 7) << 3) : (part == 1 ? 64 + ((zz & 3) << 3) : 96 + ((zz & 7) << 3)));
      else
        return tm + (uint32_t)(((zz & 7) << 5) + (part << 3));
    }
    // leading plane of the stencil: centres and the x / y differences A_1..A_3 from shared memory
    __device__ __forceinline__ static void lead_read(const float2* q, float2 cen[4], float2 a[3][4]) {
      cen[0] = q[0]; cen[1] = q[FO]; cen[2] = q[2 * FO]; cen[3] = q[3 * FO];
#pragma unroll
      for (int d = 1; d <= 3; ++d) {
        a[d - 1][0] = p_sub(q[d], q[-d]);
        a[d - 1][1] = p_sub(q[2 * FO + d], q[2 * FO - d]);
        a[d - 1][2] = p_sub(q[FO + d * BW], q[FO - d * BW]);
        a[d - 1][3] = p_sub(q[2 * FO + d * BW], q[2 * FO - d * BW]);
      }
    }
    __device__ __forceinline__ static void put8(uint32_t taddr, const float2 v[4]) {
      const float w[8] = {v[0].x, v[0].y, v[1].x, v[1].y, v[2].x, v[2].y, v[3].x, v[3].y};
      tm_st8(taddr, w);
    }
    // full layout: the leading plane zz's centres and A differences into its slot as they are
    // formed; returns the centres and A_3 for the caller's use on this step
    __device__ __forceinline__ void lead_full(const float2* q, int zz, float2 cen[4], float2 a3[4]) const {
      cen[0] = q[0]; cen[1] = q[FO]; cen[2] = q[2 * FO]; cen[3] = q[3 * FO];
      put8(slot(zz, 0), cen);
#pragma unroll
      for (int d = 1; d <= 3; ++d) {
        const float2 a[4] = {p_sub(q[d], q[-d]), p_sub(q[2 * FO + d], q[2 * FO - d]),
                             p_sub(q[FO + d * BW], q[FO - d * BW]), p_sub(q[2 * FO + d * BW], q[2 * FO - d * BW])};
        put8(slot(zz, d), a);
        if (d == 3) { a3[0] = a[0]; a3[1] = a[1]; a3[2] = a[2]; a3[3] = a[3]; }
      }
    }

    __device__ __forceinline__ void step(const float2* const pl[7], int x, int y, int z, int z1,
                                         const StepFlags<float>& fl, AccF& acc, float& dt1max, bool active) {
      using St = typename Base::St;
      const St st{pl, this->F};
      const Fac<float>& F = this->F;
      const Phys<float>& P = this->P;
      // element offsets in 32 bits (the host keeps 2 fs + 8 ps below 2^32 for these tiles): slice p
      // of an array at base[p >> 1] + (p & 1) fs + offset, one wide multiply-add per access
      const uint32_t fs32 = (uint32_t)this->fs, ps32 = (uint32_t)this->ps;
      float hzr = 0.f, hzi = 0.f;   // helical fz of this plane, loaded ahead of its use at the update
      if constexpr (UPW) {
        if (this->htab != nullptr && fl.s == 2) {
          const float* fz = this->htab + 8 + 2 * this->nx + 2 * this->ny;
          hzr = fz[2 * z];
          hzi = fz[2 * z + 1];
        }
      }
      const uint32_t ci = (uint32_t)(z + 3) * ps32 + (uint32_t)((y + 3) * this->px + this->xoff + x);
      float2* const db[2] = {this->dfp, this->dfp + 2 * this->fs};
      float2* const fb[2] = {this->fout, this->fout + 2 * this->fs};
      auto at = [&](float2* const* b, int pp, uint32_t o) { return b[pp >> 1] + (uint32_t)((pp & 1) * fs32 + o); };
      float2 cL[4], aL[3][4];   // the leading plane z+3 (aL[0], aL[1]: compact layout only)
      if constexpr (!kCompact) {
        if (z == zfirst) {   // prologue of the tile: planes z-3..z+2 into their slots
          float2 c_[4], a_[4];
#pragma unroll
          for (int k = 0; k < 6; ++k) lead_full(pl[k], z - 3 + k, c_, a_);
        }
        tm_wait_st();   // earlier slots are written before they are read below
        lead_full(pl[6], z + 3, cL, aL[2]);
      } else {
        if (z == zfirst) {   // prologue: planes z-3..z+2, only the slots read later
#pragma unroll
          for (int k = 0; k < 6; ++k) {
            float2 c_[4], a_[3][4];
            lead_read(pl[k], c_, a_);
            put8(slot(z - 3 + k, 0), c_);
            if (k >= 2) put8(slot(z - 3 + k, 1), a_[0]);
            if (k >= 1) put8(slot(z - 3 + k, 2), a_[1]);
          }
        }
        tm_wait_st();
        lead_read(pl[6], cL, aL);
        put8(slot(z + 3, 0), cL);   // slots that no load of this step reads
        put8(slot(z + 3, 2), aL[1]);
      }
      // xz / yz mixed derivatives from the A slots of planes z+-1, z+-2, z-3 (and z+3 in registers)
      uint32_t ra1p[8], ra1m[8], ra2p[8], ra2m[8], ra3m[8];
      tm_ld8(slot(z + 1, 1), ra1p);
      tm_ld8(slot(z - 1, 1), ra1m);
      tm_ld8(slot(z + 2, 2), ra2p);
      tm_ld8(slot(z - 2, 2), ra2m);
      float2 a3m[4];   // A_3 of plane z-3
      if constexpr (!kCompact) {
        tm_ld8(slot(z - 3, 3), ra3m);
      } else {
        const float2* q = pl[0];
        a3m[0] = p_sub(q[3], q[-3]);
        a3m[1] = p_sub(q[2 * FO + 3], q[2 * FO - 3]);
        a3m[2] = p_sub(q[FO + 3 * BW], q[FO - 3 * BW]);
        a3m[3] = p_sub(q[2 * FO + 3 * BW], q[2 * FO - 3 * BW]);
      }
      float2 dfo2[4];
#pragma unroll
      for (int p = 0; p < 4; ++p) dfo2[p] = this->dfnext[p];
      if (fl.read_df && active && z + 1 < z1) {
#pragma unroll
        for (int p = 0; p < 4; ++p) this->dfnext[p] = *at(db, p, ci + ps32);
      }
      if (fl.read_df && active && z + kDfPrefetch < z1) {
#pragma unroll
        for (int p = 0; p < 4; ++p) prefetch_l2(at(db, p, ci + kDfPrefetch * ps32));
      }
      tm_wait_ld();
      tm_tie8(ra1p); tm_tie8(ra1m); tm_tie8(ra2p); tm_tie8(ra2m);
      if constexpr (!kCompact) {
        tm_tie8(ra3m);
#pragma unroll
        for (int g = 0; g < 4; ++g) a3m[g] = u2f2(ra3m[2 * g], ra3m[2 * g + 1]);
      } else {
        put8(slot(z + 3, 1), aL[0]);   // the A_1 slot just read for plane z-1
      }
      float2 mz[4];   // (u_x,xz A_1,xz) (u_z,xz A_3,xz) (u_y,yz A_2,yz) (u_z,yz A_3,yz)
#pragma unroll
      for (int g = 0; g < 4; ++g) {
        const float2 t1 = p_sub(u2f2(ra1p[2 * g], ra1p[2 * g + 1]), u2f2(ra1m[2 * g], ra1m[2 * g + 1]));
        const float2 t2 = p_sub(u2f2(ra2p[2 * g], ra2p[2 * g + 1]), u2f2(ra2m[2 * g], ra2m[2 * g + 1]));
        const float2 t3 = p_sub(aL[2][g], a3m[g]);
        const float fac = (g < 2) ? F.mxz : F.myz;
        const float2 r = p_fma(p_splat(2.f), t3, p_fma(p_splat(-27.f), t2, p_mul(p_splat(270.f), t1)));
        mz[g] = p_mul(p_splat(fac), r);
      }
      // centres of planes z-3..z+2 from their slots (z+3 is cL)
      uint32_t rc[6][8];
#pragma unroll
      for (int k = 0; k < 6; ++k) tm_ld8(slot(z - 3 + k, 0), rc[k]);
      tm_wait_ld();
#pragma unroll
      for (int k = 0; k < 6; ++k) tm_tie8(rc[k]);
      float2 cz[7][4];
#pragma unroll
      for (int k = 0; k < 6; ++k)
#pragma unroll
        for (int p = 0; p < 4; ++p) cz[k][p] = u2f2(rc[k][2 * p], rc[k][2 * p + 1]);
#pragma unroll
      for (int p = 0; p < 4; ++p) cz[6][p] = cL[p];
      const float2 c0 = cz[3][0], c1 = cz[3][1], c2 = cz[3][2], c3 = cz[3][3];
      auto derz = [&](int p) {
        const float2 a = p_sub(cz[4][p], cz[2][p]), b = p_sub(cz[5][p], cz[1][p]), c = p_sub(cz[6][p], cz[0][p]);
        return p_mul(p_splat(F.fz), p_add(p_fma(p_splat(-9.f), b, p_mul(p_splat(45.f), a)), c));
      };
      auto der2z = [&](int p) {
        const float2 s1 = p_add(cz[4][p], cz[2][p]), s2 = p_add(cz[5][p], cz[1][p]), s3 = p_add(cz[6][p], cz[0][p]);
        float2 t = p_mul(p_splat((float)(-490.0 / 180.0)), cz[3][p]);
        t = p_fma(p_splat((float)(270.0 / 180.0)), s1, t);
        t = p_fma(p_splat((float)(-27.0 / 180.0)), s2, t);
        t = p_fma(p_splat((float)(2.0 / 180.0)), s3, t);
        return p_mul(p_splat(F.sz), t);
      };

      CellIn<float> c;
      c.uu[0] = c0.x; c.uu[1] = c1.x; c.uu[2] = c2.x;
      c.aa[0] = c0.y; c.aa[1] = c1.y; c.aa[2] = c2.y;
      c.lnrho = c3.x;
      c.ss = ENTROPY ? c3.y : 0.f;
#pragma unroll
      for (int p = 0; p < 3; ++p) {
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          const float2 d1 = (j < 2) ? st.der(p, j) : derz(p);
          c.uij[p][j] = d1.x;
          c.aij[p][j] = d1.y;
          const float2 d2 = (j < 2) ? st.der2(p, j) : der2z(p);
          c.a2[p][j] = d2.y;
          c.del2u[p] = (j == 0) ? d2.x : c.del2u[p] + d2.x;
          if (j == p) c.graddivu[p] = d2.x;
        }
      }
      const float2 xy0 = st.derij(0, 0, 1);   // (u_x,xy, A_1,xy)
      const float2 xy1 = st.derij(1, 0, 1);   // (u_y,xy, A_2,xy)
      const float2 xz0 = mz[0], xz2 = mz[1], yz1 = mz[2], yz2 = mz[3];
      const float gx = c.graddivu[0], gy = c.graddivu[1], gz = c.graddivu[2];
      c.graddivu[0] = (gx + xy1.x) + xz2.x;
      c.graddivu[1] = (xy0.x + gy) + yz2.x;
      c.graddivu[2] = (xz0.x + yz1.x) + gz;
      c.a1xy = xy0.y; c.a1xz = xz0.y; c.a2xy = xy1.y; c.a2yz = yz1.y; c.a3xz = xz2.y; c.a3yz = yz2.y;
      c.a3xy = c.a2xz = c.a1yz = 0.f;
      if (fl.want_diag) {
        c.a3xy = st.derij(2, 0, 1).y; c.a2xz = st.derij(1, 0, 2).y; c.a1yz = st.derij(0, 1, 2).y;
      }
      {
        const float2 gxy0 = st.der(3, 0), gxy1 = st.der(3, 1), gz3 = derz(3);
        c.glnrho[0] = gxy0.x; c.glnrho[1] = gxy1.x; c.glnrho[2] = gz3.x;
        c.gss[0] = ENTROPY ? gxy0.y : 0.f; c.gss[1] = ENTROPY ? gxy1.y : 0.f; c.gss[2] = ENTROPY ? gz3.y : 0.f;
      }
      if (ENTROPY) {
        const float2 ls = p_add(p_add(st.der2(3, 0), st.der2(3, 1)), der2z(3));
        c.del2lnrho = ls.x;
        c.del2ss = ls.y;
      } else {
        c.del2lnrho = c.del2ss = 0.f;
      }
      if constexpr (UPW) {   // calc_del6_for_upwind, sub.f90:7491-7539
        auto del6z = [&](int p) {   // der6_main upwind=T along z (deriv.f90:936-1010)
          const float2 s1 = p_add(cz[4][p], cz[2][p]), s2 = p_add(cz[5][p], cz[1][p]), s3 = p_add(cz[6][p], cz[0][p]);
          float2 t = p_mul(p_splat(-20.f), cz[3][p]);
          t = p_fma(p_splat(15.f), s1, t);
          t = p_fma(p_splat(-6.f), s2, t);
          return p_mul(p_splat(F.fz), p_add(t, s3));
        };
        auto upwind = [&](int p) {
          return (fabsf(c.uu[0]) * st.del6u(p, 0).x + fabsf(c.uu[1]) * st.del6u(p, 1).x) + fabsf(c.uu[2]) * del6z(p).x;
        };
        if (this->upw & UPW_UU) {
#pragma unroll
          for (int p = 0; p < 3; ++p) c.upw_u[p] = upwind(p);
        }
        if (this->upw & UPW_LNRHO) c.upw_lnrho = upwind(3);
      }
      float fc[3] = {0.f, 0.f, 0.f};
      if (this->forcing) {   // forcing_cont 'ABC', forcing.f90:5894-5896
        fc[0] = P.fact * (P.abc_c * this->fsz + (P.fact2 * P.abc_b) * this->fcy);
        fc[1] = P.fact * (P.abc_a * this->fsx + (P.fact2 * P.abc_c) * this->fcz);
        fc[2] = P.fact * (P.abc_b * this->fsy + (P.fact2 * P.abc_a) * this->fcx);
        if (z + 1 < z1) { this->fsz = this->sinz[z + 4]; this->fcz = this->cosz[z + 4]; }
      }
      float dfo[NF], dfn[NF];
      dfo[0] = dfo2[0].x; dfo[1] = dfo2[1].x; dfo[2] = dfo2[2].x; dfo[ILNRHO] = dfo2[3].x;
      if (ENTROPY) dfo[ISS] = dfo2[3].y;
      dfo[IAX] = dfo2[0].y; dfo[IAX + 1] = dfo2[1].y; dfo[IAX + 2] = dfo2[2].y;
      DiagF dg;   // this cell's diagnostic terms, added to the column's sums only on a live lane
      float dt1_l = 0.f;
      cell_rhs<float, NF>(c, P, F, fc, this->forcing, this->iso, this->vheat, this->oheat, dfo, fl.alpha, dfn,
                          fl.want_cfl, fl.want_diag, dg, dt1_l, UPW ? this->upw : 0);
      if (active) {
        if (fl.want_diag) dg.add_to(acc);
        dt1max = (dt1_l > dt1max || dt1_l != dt1_l) ? dt1_l : dt1max;
      }

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
        if (this->htab != nullptr && fl.s == 2) {   // forcing_hel after the step (addforce, forcing.f90:1307)
          const float qr = rsub(rmul(this->hpr, hzr), rmul(this->hpi, hzi));
          const float qi = radd(rmul(this->hpr, hzi), rmul(this->hpi, hzr));
#pragma unroll
          for (int p = 0; p < 3; ++p) {
            const float fh = rsub(rmul(this->hc1[p], qr), rmul(this->hc2[p], qi));
            if (this->htarget) fnew[p].y = __fadd_rn(fnew[p].y, fh);
            else fnew[p].x = __fadd_rn(fnew[p].x, fh);
          }
        }
      }
      if (active) {
        if (fl.write_df) {
#pragma unroll
          for (int p = 0; p < 4; ++p) *at(db, p, ci) = dsto[p];
        }
#pragma unroll
        for (int p = 0; p < 4; ++p) *at(fb, p, ci) = fnew[p];
        const bool edge = (x < 3) | (x >= this->nx - 3) | (y < 3) | (y >= this->ny - 3) | (z < 3) | (z >= this->nz - 3);
        if (edge) {
          const Images ix(x, this->nx), iy(y, this->ny), iz(z, this->nz);
#pragma unroll
          for (int a = 0; a < 2; ++a)
#pragma unroll
            for (int b = 0; b < 2; ++b)
#pragma unroll
              for (int e = 0; e < 2; ++e) {
                if ((a == 0 && b == 0 && e == 0) || a >= iz.n || b >= iy.n || e >= ix.n) continue;
                const long long gi = (long long)(iz.v[a] + 3) * this->ps + (long long)(iy.v[b] + 3) * this->px +
                                     this->xoff + ix.v[e];
#pragma unroll
                for (int p = 0; p < 4; ++p) this->fout[p * this->fs + gi] = fnew[p];
              }
        }
      }
    }
  };
};

}  // namespace pcgb
