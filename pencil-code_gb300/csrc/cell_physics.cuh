// cell_physics.cuh -- the pencil algebra and right-hand sides of one cell,
// shared by the scalar and the packed-pair cell policies.  Inputs are the
// field values and stencil derivatives of the cell; outputs are the new df of
// every field (accumulated in the reference's module order) plus the CFL and
// diagnostic contributions.
#pragma once

#include <type_traits>
#include "mhd_common.cuh"

namespace pcgb {

template <typename T>
struct CellIn {
  T uu[3], uij[3][3];            // u and u_i,j (gij, sub.f90:1505)
  T del2u[3], graddivu[3];       // del2v_etc (sub.f90:2610)
  T lnrho, glnrho[3];
  T ss, gss[3], del2lnrho, del2ss;   // entropy only
  T aa[3], aij[3][3];
  T a2[3][3];                    // a2[i][j] = A_i,jj (der2)
  T a1xy, a2xy, a1xz, a3xz, a2yz, a3yz;   // mixed derivatives entering J
  T a3xy, a2xz, a1yz;                     // entering only the diagonal b_ii (div B)
  T upw_u[3], upw_lnrho;                  // upwind corrections sum_j |u_j| D6_j f (lupw_uu, lupw_lnrho)
};

// Upwinding flags (bits of PcgbBoxDev::lupw): hydro.f90:3662 lupw_uu, density.f90:2772 lupw_lnrho.
enum { UPW_UU = 1, UPW_LNRHO = 2 };

// Double-float product and sum of FP32 values (FMA TwoProd, TwoSum).
__device__ __forceinline__ void two_prod_f(float a, float b, float& h, float& l) {
  h = __fmul_rn(a, b);
  l = __fmaf_rn(a, b, -h);
}
__device__ __forceinline__ void add_df(float& h, float& l, float xh, float xl) {
  const float s = __fadd_rn(h, xh), bp = __fsub_rn(s, h);
  const float e = __fadd_rn(__fsub_rn(h, __fsub_rn(s, bp)), __fsub_rn(xh, bp));
  h = s;
  l = __fadd_rn(__fadd_rn(l, xl), e);
}

// RHS of one cell in the order of calc_all_rhs (equ.f90:1268-1274).
// dfo: df before the substep (already read); dfn: alpha*dfo + RHS.
// A: the diagnostic sink -- Acc (FP64 sums), AccF (FP32 cells' double-float sums) or
// DiagF (one FP32 cell's terms).
template <typename T, int NF, class A>
__device__ __forceinline__ void cell_rhs(const CellIn<T>& c, const Phys<T>& P, const Fac<T>& F, const T fc[3],
                                         bool forcing, bool iso, bool vheat, bool oheat, const T dfo[NF], T alpha,
                                         T dfn[NF], bool want_cfl, bool want_diag, A& acc, T& dt1max,
                                         int upw = 0) {
  constexpr int IUX = 0, ILNRHO = 3, ISS = 4, IAX = NF - 3;
  constexpr bool ENTROPY = (NF == 8);
  const T(&uu)[3] = c.uu;
  const T(&uij)[3][3] = c.uij;
  // ---- hydro pencils (hydro.f90:3564-3990, sub.f90) ----
  const T u2 = (uu[0] * uu[0] + uu[1] * uu[1]) + uu[2] * uu[2];          // dot2_mn, sub.f90:897
  const T divu = (uij[0][0] + uij[1][1]) + uij[2][2];                   // div_mn, sub.f90:1981
  T sij[3][3];                                                           // traceless_strain, sub.f90:8922
#pragma unroll
  for (int jj = 0; jj < 3; ++jj) {
    sij[jj][jj] = uij[jj][jj] - T(1.0 / 3.0) * divu;
#pragma unroll
    for (int i = jj + 1; i < 3; ++i) {
      sij[i][jj] = T(0.5) * (uij[i][jj] + uij[jj][i]);
      sij[jj][i] = sij[i][jj];
    }
  }
  T ugu[3];                                                              // u_dot_grad_vec, sub.f90:3482
#pragma unroll
  for (int jj = 0; jj < 3; ++jj) ugu[jj] = (uu[0] * uij[jj][0] + uu[1] * uij[jj][1]) + uu[2] * uij[jj][2];
  if (upw & UPW_UU) {                                                    // doupwind, sub.f90:7541
#pragma unroll
    for (int jj = 0; jj < 3; ++jj) ugu[jj] = ugu[jj] - c.upw_u[jj];
  }
  // ---- density pencils (density.f90:2747-2800) ----
  const T rho1 = texp(-c.lnrho);
  T uglnrho = (uu[0] * c.glnrho[0] + uu[1] * c.glnrho[1]) + uu[2] * c.glnrho[2];
  if (upw & UPW_LNRHO) uglnrho = uglnrho - c.upw_lnrho;                // density.f90:2772
  T sglnrho[3];                                                          // multmv_mn, sub.f90:1228
#pragma unroll
  for (int i = 0; i < 3; ++i) sglnrho[i] = (sij[i][0] * c.glnrho[0] + sij[i][1] * c.glnrho[1]) + sij[i][2] * c.glnrho[2];
  // ---- EOS (eos_idealgas.f90:842-887) ----
  T cs2, TT1 = T(0), glnTT[3] = {T(0), T(0), T(0)}, del2lnTT = T(0);
  if (ENTROPY) {
    cs2 = P.cs20 * texp(P.cv1 * c.ss + P.gamma_m1 * (c.lnrho - P.lnrho0));
    const T lnTT = (P.lnTT0 + P.cv1 * c.ss) + P.gamma_m1 * (c.lnrho - P.lnrho0);
    TT1 = texp(-lnTT);
#pragma unroll
    for (int jj = 0; jj < 3; ++jj) glnTT[jj] = P.gamma_m1 * c.glnrho[jj] + P.cv1 * c.gss[jj];
    del2lnTT = P.gamma_m1 * c.del2lnrho + P.cv1 * c.del2ss;
  } else if (iso) {
    cs2 = P.cs20;                                                        // noentropy.f90:100
  } else {
    cs2 = P.cs20 * texp(P.gamma_m1 * (c.lnrho - P.lnrho0));             // polytropic, noentropy.f90:102
  }
  // ---- magnetic pencils (magnetic.f90:4310-4900, gij_etc sub.f90:2945) ----
  T bb[3];                                                               // curl_mn, sub.f90:2058-2060
  bb[0] = c.aij[2][1] - c.aij[1][2];
  bb[1] = c.aij[0][2] - c.aij[2][0];
  bb[2] = c.aij[1][0] - c.aij[0][1];
  // off-diagonal b_ij = eps_ikl A_l,kj (sub.f90:3017-3019), with d2A[j][k][i] = A_i,jk
  const T b01 = c.a2[2][1] - c.a2yz;   // A_3,yy - A_2,zy
  const T b02 = c.a3yz - c.a2[1][2];   // A_3,yz - A_2,zz
  const T b10 = c.a1xz - c.a2[2][0];   // A_1,zx - A_3,xx
  const T b12 = c.a2[0][2] - c.a3xz;   // A_1,zz - A_3,xz
  const T b20 = c.a2[1][0] - c.a1xy;   // A_2,xx - A_1,yx
  const T b21 = c.a2xy - c.a2[0][1];   // A_2,xy - A_1,yy
  T del2a[3];                                                            // gij_etc del2, sub.f90:3085
#pragma unroll
  for (int i = 0; i < 3; ++i) del2a[i] = (c.a2[i][0] + c.a2[i][1]) + c.a2[i][2];
  bb[0] = bb[0] + P.bx; bb[1] = bb[1] + P.by; bb[2] = bb[2] + P.bz;     // B_ext, magnetic.f90:4366-4370
  T jj3[3];                                                              // jj = mu01*curl(bij), magnetic.f90:4735
  jj3[0] = P.mu01 * (b21 - b12);
  jj3[1] = P.mu01 * (b02 - b20);
  jj3[2] = P.mu01 * (b10 - b01);
  const T b2 = (bb[0] * bb[0] + bb[1] * bb[1]) + bb[2] * bb[2];
  const T j2 = (jj3[0] * jj3[0] + jj3[1] * jj3[1]) + jj3[2] * jj3[2];
  T jxbr[3], uxb[3];                                                     // cross_mn, multsv_mn
  jxbr[0] = rho1 * (jj3[1] * bb[2] - jj3[2] * bb[1]);
  jxbr[1] = rho1 * (jj3[2] * bb[0] - jj3[0] * bb[2]);
  jxbr[2] = rho1 * (jj3[0] * bb[1] - jj3[1] * bb[0]);
  uxb[0] = uu[1] * bb[2] - uu[2] * bb[1];
  uxb[1] = uu[2] * bb[0] - uu[0] * bb[2];
  uxb[2] = uu[0] * bb[1] - uu[1] * bb[0];

  // ---- right-hand sides in module order ----
  // duu_dt (hydro.f90:4421): -u.grad u, viscous force (viscosity.f90:1638), continuous forcing (:4609)
  T dfu[3];
#pragma unroll
  for (int jj = 0; jj < 3; ++jj) dfu[jj] = alpha * dfo[IUX + jj] - ugu[jj];
#pragma unroll
  for (int jj = 0; jj < 3; ++jj)
    dfu[jj] = dfu[jj] + P.nu * ((c.del2u[jj] + wmul<T>(2, sglnrho[jj])) + T(1.0 / 3.0) * c.graddivu[jj]);
  if (forcing) {
#pragma unroll
    for (int jj = 0; jj < 3; ++jj) dfu[jj] = dfu[jj] + P.ampl_fc * fc[jj];
  }
  // dlnrho_dt (density.f90:2929-2930, :3059)
  dfn[ILNRHO] = alpha * dfo[ILNRHO] + (-divu - uglnrho);
  // denergy_dt: pressure force (+ entropy equation)
  if (!ENTROPY) {
#pragma unroll
    for (int jj = 0; jj < 3; ++jj) dfu[jj] = dfu[jj] + (-(cs2 * c.glnrho[jj]));          // noentropy.f90:383
  } else {
#pragma unroll
    for (int jj = 0; jj < 3; ++jj)
      dfu[jj] = dfu[jj] + (-((cs2 * (c.glnrho[jj] + glnTT[jj])) * P.gamma1));             // entropy.f90:3599
    const T ugss = (uu[0] * c.gss[0] + uu[1] * c.gss[1]) + uu[2] * c.gss[2];
    T dfs = alpha * dfo[ISS] - ugss;                                                      // entropy.f90:3775
    if (vheat) {                                                                           // viscosity.f90:2765
      T sij2 = sij[0][0] * sij[0][0];                                                      // multm2_sym_mn
      sij2 = sij2 + sij[1][1] * sij[1][1];
      sij2 = sij2 + wmul<T>(2, sij[1][0] * sij[1][0]);
      sij2 = sij2 + sij[2][2] * sij[2][2];
      sij2 = sij2 + wmul<T>(2, sij[2][0] * sij[2][0]);
      sij2 = sij2 + wmul<T>(2, sij[2][1] * sij[2][1]);
      dfs = dfs + TT1 * (P.two_nu * sij2);
    }
    const T gs0 = c.glnrho[0] + glnTT[0], gs1 = c.glnrho[1] + glnTT[1], gs2 = c.glnrho[2] + glnTT[2];
    const T g2 = (gs0 * glnTT[0] + gs1 * glnTT[1]) + gs2 * glnTT[2];
    dfs = dfs + P.chi_cp * (del2lnTT + g2);                                                // entropy.f90:4886
    if (oheat) dfs = dfs + ((P.eta_mu0 * j2) * rho1) * TT1;                               // magnetic.f90:6141
    dfn[ISS] = dfs;
  }
  // daa_dt (magnetic.f90:5531, :5589, :6247, :6524)
#pragma unroll
  for (int jj = 0; jj < 3; ++jj) dfu[jj] = dfu[jj] + jxbr[jj];
#pragma unroll
  for (int jj = 0; jj < 3; ++jj) dfn[IAX + jj] = alpha * dfo[IAX + jj] + (uxb[jj] + P.eta * del2a[jj]);
#pragma unroll
  for (int jj = 0; jj < 3; ++jj) dfn[IUX + jj] = dfu[jj];

  if (want_cfl) {
    const T d = cfl_dt1(P, F, uu, bb, rho1, cs2);
    dt1max = (d > dt1max || d != d) ? d : dt1max;
  }
  if (want_diag) {
    const T b00 = c.a3xy - c.a2xz, b11 = c.a1yz - c.a3xy, b22 = c.a2xz - c.a1yz;
    // <A.B> uses the field before the imposed B_ext is added (p%bbb, magnetic.f90:4356,4451)
    const T bbb0 = c.aij[2][1] - c.aij[1][2], bbb1 = c.aij[0][2] - c.aij[2][0], bbb2 = c.aij[1][0] - c.aij[0][1];
    if constexpr (std::is_same<A, Acc>::value) {
      const double divb = (double)((b00 + b11) + b22);
      const double ab = ((double)c.aa[0] * (double)bbb0 + (double)c.aa[1] * (double)bbb1) +
                        (double)c.aa[2] * (double)bbb2;
      acc_diag(acc, (double)u2, (double)b2, (double)c.lnrho, divb, (double)j2, ab);
    } else {   // FP32 cell: the terms in FP32, <A.B> exactly as a double-float
      const float divb = (b00 + b11) + b22;
      float abh, abl, ph, pl;
      two_prod_f(c.aa[0], bbb0, abh, abl);
      two_prod_f(c.aa[1], bbb1, ph, pl);
      add_df(abh, abl, ph, pl);
      two_prod_f(c.aa[2], bbb2, ph, pl);
      add_df(abh, abl, ph, pl);
      const float rho = expf(c.lnrho);
      DiagF d{u2, b2, 0.5f * rho * u2, rho, divb * divb, j2, abh, abl};
      if constexpr (std::is_same<A, DiagF>::value) acc = d;
      else d.add_to(acc);
    }
  }
}

// CFL inverse timestep only (MODE_CFL pass): needs u, lnrho, [ss] and B.
template <typename T, int NF>
__device__ __forceinline__ T cell_cfl_only(const Phys<T>& P, const Fac<T>& F, const T uu[3], T lnrho, T ss,
                                           const T bb_noext[3], bool iso) {
  const T rho1 = texp(-lnrho);
  T cs2;
  if (NF == 8) cs2 = P.cs20 * texp(P.cv1 * ss + P.gamma_m1 * (lnrho - P.lnrho0));
  else if (iso) cs2 = P.cs20;
  else cs2 = P.cs20 * texp(P.gamma_m1 * (lnrho - P.lnrho0));
  T bb[3] = {bb_noext[0] + P.bx, bb_noext[1] + P.by, bb_noext[2] + P.bz};
  return cfl_dt1(P, F, uu, bb, rho1, cs2);
}

}  // namespace pcgb
