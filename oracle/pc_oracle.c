/*
 * pc_oracle.c -- CPU FP64 restatement of the Pencil Code compressible-MHD
 * pde() right-hand side and 2N-storage RK3 step.
 *
 * TEST INFRASTRUCTURE ONLY (the parity oracle; see pc_oracle.h).
 *
 * Every routine follows a reference routine, cited file:line (paths relative
 * to the pencil-code source tree).  Operand order of each sum follows the
 * Fortran expression it restates (left to right), and this file is compiled
 * with -ffp-contract=off so that results are identical on x86-64 and aarch64.
 */
#include "pc_oracle.h"

#include <math.h>
#include <stddef.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define NG ORC_NGHOST

typedef struct {
  int mx, my, mz, nf;
  int iux, iuy, iuz, ilnrho, iss, iax, iay, iaz;
  double dx_1, dy_1, dz_1, dxyz_2;
  /* EOS constants, src/eos_idealgas.f90:144-281 (units_eos) */
  double cs20, gamma_m1, gamma1, lnrho0, cp1, cv, cv1, lnTT0, cpp;
  double mu01;
  /* ABC forcing: src/forcing.f90:1100-1104 tables, :5869-5897 factors */
  double fact, fact2;
  double *sinx, *cosx, *siny, *cosy, *sinz, *cosz;
} ctx_t;

static inline size_t IDX(const ctx_t* c, int l, int m, int n, int k) {
  return (size_t)l + (size_t)c->mx * ((size_t)m + (size_t)c->my * ((size_t)n + (size_t)c->mz * (size_t)k));
}

int orc_nfields(const orc_params* p) { return p->lentropy ? 8 : 7; }

/* A direction is periodic when every field's code on both sides is 'p'. */
static int orc_periodic(const orc_params* p, int d) {
  for (int k = 0; k < orc_nfields(p); ++k)
    if (p->bc[d][k][0] != ORC_BC_PER || p->bc[d][k][1] != ORC_BC_PER) return 0;
  return 1;
}

/* Equidistant grid, src/grid.f90:123-151: on a periodic axis dx = Lx/nx and
   x(i) = x0 + (i - nghost - 1 + 1/2) dx (1-based i, cell centres); otherwise
   dx = Lx/(nx-1) and x(i) = x0 + (i - nghost - 1) dx (points on both boundaries). */
static double orc_spacing(const orc_params* p, int d) {
  const int n = d == 0 ? p->nx : d == 1 ? p->ny : p->nz;
  const double L = d == 0 ? p->Lx : d == 1 ? p->Ly : p->Lz;
  return L / (orc_periodic(p, d) ? n : n - 1);
}

void orc_grid(const orc_params* p, double* x, double* y, double* z) {
  const double dx = orc_spacing(p, 0), dy = orc_spacing(p, 1), dz = orc_spacing(p, 2);
  const double ox = orc_periodic(p, 0) ? 0.5 : 0.0, oy = orc_periodic(p, 1) ? 0.5 : 0.0,
               oz = orc_periodic(p, 2) ? 0.5 : 0.0;
  for (int i = 0; i < p->nx + 2 * NG; ++i) x[i] = p->x0 + ((double)(i - NG) + ox) * dx;
  for (int i = 0; i < p->ny + 2 * NG; ++i) y[i] = p->y0 + ((double)(i - NG) + oy) * dy;
  for (int i = 0; i < p->nz + 2 * NG; ++i) z[i] = p->z0 + ((double)(i - NG) + oz) * dz;
}

static void ctx_init(ctx_t* c, const orc_params* p) {
  memset(c, 0, sizeof(*c));
  c->mx = p->nx + 2 * NG; c->my = p->ny + 2 * NG; c->mz = p->nz + 2 * NG;
  c->nf = orc_nfields(p);
  c->iux = 0; c->iuy = 1; c->iuz = 2; c->ilnrho = 3;
  if (p->lentropy) { c->iss = 4; c->iax = 5; } else { c->iss = -1; c->iax = 4; }
  c->iay = c->iax + 1; c->iaz = c->iax + 2;
  c->dx_1 = 1.0 / orc_spacing(p, 0);
  c->dy_1 = 1.0 / orc_spacing(p, 1);
  c->dz_1 = 1.0 / orc_spacing(p, 2);
  /* dxyz_2 = dline_1(:,1)**2 + dline_1(:,2)**2 + dline_1(:,3)**2, grid.f90:3051 */
  c->dxyz_2 = (c->dx_1 * c->dx_1 + c->dy_1 * c->dy_1) + c->dz_1 * c->dz_1;
  /* units_eos, eos_idealgas.f90:158-268 */
  c->gamma_m1 = p->gamma - 1.0;
  c->gamma1 = 1.0 / p->gamma;
  c->lnrho0 = log(p->rho0);
  c->cs20 = p->cs0 * p->cs0;
  c->cp1 = 1.0 / p->cp;
  c->cv = c->gamma1 * p->cp;
  c->cv1 = p->gamma * c->cp1;
  c->lnTT0 = (c->gamma_m1 != 0.0) ? log(c->cs20 / (p->cp * c->gamma_m1)) : log(c->cs20 / p->cp);
  c->cpp = 1.0 / c->cp1;  /* p%cp = 1/cp1, eos_idealgas.f90:812 */
  c->mu01 = 1.0 / p->mu0;
  if (p->lforcing_cont) {
    /* forcing_cont 'ABC', forcing.f90:5869-5872 */
    c->fact2 = p->relhel;
    double fact1 = 0.5 * (1.0 + p->relhel * p->relhel);
    c->fact = p->ampl_ff / sqrt(fact1 * ((p->abc_a * p->abc_a + p->abc_b * p->abc_b) + p->abc_c * p->abc_c));
    double *x = malloc(sizeof(double) * c->mx), *y = malloc(sizeof(double) * c->my),
           *z = malloc(sizeof(double) * c->mz);
    orc_grid(p, x, y, z);
    c->sinx = malloc(sizeof(double) * c->mx); c->cosx = malloc(sizeof(double) * c->mx);
    c->siny = malloc(sizeof(double) * c->my); c->cosy = malloc(sizeof(double) * c->my);
    c->sinz = malloc(sizeof(double) * c->mz); c->cosz = malloc(sizeof(double) * c->mz);
    for (int i = 0; i < c->mx; ++i) { c->sinx[i] = sin(p->kf * x[i]); c->cosx[i] = cos(p->kf * x[i]); }
    for (int i = 0; i < c->my; ++i) { c->siny[i] = sin(p->kf * y[i]); c->cosy[i] = cos(p->kf * y[i]); }
    for (int i = 0; i < c->mz; ++i) { c->sinz[i] = sin(p->kf * z[i]); c->cosz[i] = cos(p->kf * z[i]); }
    free(x); free(y); free(z);
  }
}

static void ctx_free(ctx_t* c) {
  free(c->sinx); free(c->cosx); free(c->siny); free(c->cosy); free(c->sinz); free(c->cosz);
}

/* ------------------------------------------------------------------------ */
/* One field's ghosts on one side of direction d, over the full extent of the
   other two axes: bc_per_x/y/z (boundcond.f90:2387-2531) for 'p', bc_sym_x/y/z
   (:2637-2677, :3483-3530, :3842-3900) for 's' (sgn +1), 'a' (sgn -1, boundary
   value set to 0) and 'a2' (sgn -1, REL). */
static void bc_side(const orc_params* p, const ctx_t* c, double* f, int k, int d, int side) {
  const int code = p->bc[d][k][side];
  const int n = d == 0 ? p->nx : d == 1 ? p->ny : p->nz;
  const int na = d == 0 ? c->my : c->mx, nb = d == 0 ? c->mz : (d == 1 ? c->mz : c->my);
  const size_t st = d == 0 ? 1 : d == 1 ? (size_t)c->mx : (size_t)c->mx * c->my;
  const int b1 = NG, b2 = NG + n - 1;   /* n1, n2 (0-based array indices) */
  /* the lines normal to the boundary are independent: threads change nothing */
#ifdef _OPENMP
#pragma omp parallel for schedule(static) if ((size_t)na * nb > 4096)
#endif
  for (int ib = 0; ib < nb; ++ib)
    for (int ia = 0; ia < na; ++ia) {
      size_t base;   /* element at index 0 along d */
      if (d == 0) base = IDX(c, 0, ia, ib, k);
      else if (d == 1) base = IDX(c, ia, 0, ib, k);
      else base = IDX(c, ia, ib, 0, k);
      double* q = f + base;
      if (code == ORC_BC_PER) {
        for (int i = 1; i <= NG; ++i) {
          if (side == 0) q[(size_t)(b1 - i) * st] = q[(size_t)(b2 + 1 - i) * st];   /* f(n1-i) = f(n2+1-i) */
          else q[(size_t)(b2 + i) * st] = q[(size_t)(b1 - 1 + i) * st];              /* f(n2+i) = f(n1-1+i) */
        }
        continue;
      }
      const double sgn = (code == ORC_BC_SYM) ? 1.0 : -1.0;
      if (side == 0) {
        for (int i = 1; i <= NG; ++i) {
          const double fi = q[(size_t)(b1 + i) * st], f0 = q[(size_t)b1 * st];
          q[(size_t)(b1 - i) * st] = (code == ORC_BC_ASYM2) ? 2.0 * f0 + sgn * fi : sgn * fi;
        }
        if (code == ORC_BC_ASYM) q[(size_t)b1 * st] = 0.0;
      } else {
        for (int i = 1; i <= NG; ++i) {
          const double fi = q[(size_t)(b2 - i) * st], f0 = q[(size_t)b2 * st];
          double g;
          if (code != ORC_BC_ASYM2) g = sgn * fi;
          else if (d == 2) g = f0 + (f0 + sgn * fi);   /* bc_sym_z top, :3886 */
          else g = 2.0 * f0 + sgn * fi;
          q[(size_t)(b2 + i) * st] = g;
        }
        if (code == ORC_BC_ASYM) q[(size_t)b2 * st] = 0.0;
      }
    }
}

void orc_boundconds(const orc_params* p, double* f, int nf) {
  ctx_t c; ctx_init(&c, p);
  for (int d = 0; d < 3; ++d)          /* boundconds_x, then _y, then _z */
    for (int k = 0; k < nf; ++k)
      for (int side = 0; side < 2; ++side) bc_side(p, &c, f, k, d, side);
  ctx_free(&c);
}

/* ------------------------------------------------------------------------ */
/* der_main, deriv.f90:89-171 (equidistant Cartesian):
   df = fac*( 45*(f+1 - f-1) - 9*(f+2 - f-2) + (f+3 - f-3) ), fac = (1/60)*dx_1 */
static inline double der_c(const ctx_t* c, const double* f, int k, int j, int l, int m, int n) {
  const double a = 1.0 / 60.0;
  size_t s = (j == 0) ? 1 : (j == 1) ? (size_t)c->mx : (size_t)c->mx * c->my;
  double fac = a * ((j == 0) ? c->dx_1 : (j == 1) ? c->dy_1 : c->dz_1);
  const double* q = f + IDX(c, l, m, n, k);
  return fac * ((45.0 * (q[s] - q[-(ptrdiff_t)s]) - 9.0 * (q[2 * s] - q[-(ptrdiff_t)(2 * s)])) +
                (q[3 * s] - q[-(ptrdiff_t)(3 * s)]));
}

/* der2_main, deriv.f90:472-561, 'standard' coefficients (deriv.f90:39-41):
   df2 = fac*( c0 f0 + c1(f+1 + f-1) + c2(f+2 + f-2) + c3(f+3 + f-3) ), fac = dx_1**2 */
static inline double der2_c(const ctx_t* c, const double* f, int k, int j, int l, int m, int n) {
  const double c0 = -490.0 / 180.0, c1 = 270.0 / 180.0, c2 = -27.0 / 180.0, c3 = 2.0 / 180.0;
  size_t s = (j == 0) ? 1 : (j == 1) ? (size_t)c->mx : (size_t)c->mx * c->my;
  double d1 = (j == 0) ? c->dx_1 : (j == 1) ? c->dy_1 : c->dz_1;
  double fac = d1 * d1;
  const double* q = f + IDX(c, l, m, n, k);
  return fac * (((c0 * q[0] + c1 * (q[s] + q[-(ptrdiff_t)s])) + c2 * (q[2 * s] + q[-(ptrdiff_t)(2 * s)])) +
                c3 * (q[3 * s] + q[-(ptrdiff_t)(3 * s)]));
}

/* derij_main, bidiagonal scheme (deriv.f90:1367-1451; default
   lbidiagonal_derij=.true., cdata.f90:827).  Symmetric in (i,j). */
static inline double derij_c(const ctx_t* c, const double* f, int k, int i, int j, int l, int m, int n) {
  int a = i < j ? i : j, b = i < j ? j : i;   /* a < b, 0-based directions */
  size_t sa = (a == 0) ? 1 : (a == 1) ? (size_t)c->mx : (size_t)c->mx * c->my;
  size_t sb = (b == 0) ? 1 : (b == 1) ? (size_t)c->mx : (size_t)c->mx * c->my;
  double fac;
  if (a == 0 && b == 1) fac = ((1.0 / 720.0) * c->dx_1) * c->dy_1;        /* :1392 */
  else if (a == 1 && b == 2) fac = ((1.0 / 720.0) * c->dy_1) * c->dz_1;   /* :1408 */
  else fac = ((1.0 / 720.0) * c->dz_1) * c->dx_1;                         /* :1424 */
  const double* q = f + IDX(c, l, m, n, k);
  double t[3];
  for (int d = 1; d <= 3; ++d) {
    ptrdiff_t A = (ptrdiff_t)(d * sa), B = (ptrdiff_t)(d * sb);
    if (a == 1 && b == 2)   /* yz: f(m+d,n+d) - f(m+d,n-d) + f(m-d,n-d) - f(m-d,n+d), :1410-1415 */
      t[d - 1] = ((q[A + B] - q[A - B]) + q[-A - B]) - q[-A + B];
    else                    /* xy, xz: f(l+d,.+d) - f(l-d,.+d) + f(l-d,.-d) - f(l+d,.-d) */
      t[d - 1] = ((q[A + B] - q[-A + B]) + q[-A - B]) - q[A - B];
  }
  return fac * ((270.0 * t[0] - 27.0 * t[1]) + 2.0 * t[2]);
}

/* der6_main with upwind=T (deriv.f90:936-1010): the 6th difference times
   dx_1/60, (1/60) dx_1 (-20 f0 + 15 (f1 + f-1) - 6 (f2 + f-2) + (f3 + f-3)). */
static inline double der6_upwind_c(const ctx_t* c, const double* f, int k, int j, int l, int m, int n) {
  size_t s = (j == 0) ? 1 : (j == 1) ? (size_t)c->mx : (size_t)c->mx * c->my;
  const double fac = (j == 0) ? (1.0 / 60.0) * c->dx_1 : (j == 1) ? (1.0 / 60.0) * c->dy_1 : (1.0 / 60.0) * c->dz_1;
  const double* q = f + IDX(c, l, m, n, k);
  const ptrdiff_t a = (ptrdiff_t)s, b = 2 * (ptrdiff_t)s, d = 3 * (ptrdiff_t)s;
  return fac * (((-20.0 * q[0] + 15.0 * (q[a] + q[-a])) - 6.0 * (q[b] + q[-b])) + (q[d] + q[-d]));
}

/* calc_del6_for_upwind (sub.f90:7491-7539): sum_j |u_j| der6_j(f_k, upwind). */
static inline double del6_upwind(const ctx_t* c, const double* f, int k, const double uu[3], int l, int m, int n) {
  return (fabs(uu[0]) * der6_upwind_c(c, f, k, 0, l, m, n) + fabs(uu[1]) * der6_upwind_c(c, f, k, 1, l, m, n)) +
         fabs(uu[2]) * der6_upwind_c(c, f, k, 2, l, m, n);
}

double orc_der(const orc_params* p, const double* f, int k, int j, int l, int m, int n) {
  ctx_t c; ctx_init(&c, p); double r = der_c(&c, f, k, j, l, m, n); ctx_free(&c); return r;
}
double orc_der2(const orc_params* p, const double* f, int k, int j, int l, int m, int n) {
  ctx_t c; ctx_init(&c, p); double r = der2_c(&c, f, k, j, l, m, n); ctx_free(&c); return r;
}
double orc_derij(const orc_params* p, const double* f, int k, int i, int j, int l, int m, int n) {
  ctx_t c; ctx_init(&c, p); double r = derij_c(&c, f, k, i, j, l, m, n); ctx_free(&c); return r;
}

void orc_stencil_field(const orc_params* p, const double* f, int k, int kind, int i, int j, double* out) {
  ctx_t c; ctx_init(&c, p);
  for (int n = 0; n < p->nz; ++n)
    for (int m = 0; m < p->ny; ++m)
      for (int l = 0; l < p->nx; ++l) {
        double v;
        if (kind == 0) v = der_c(&c, f, k, i, l + NG, m + NG, n + NG);
        else if (kind == 1) v = der2_c(&c, f, k, i, l + NG, m + NG, n + NG);
        else v = derij_c(&c, f, k, i, j, l + NG, m + NG, n + NG);
        out[(size_t)l + (size_t)p->nx * ((size_t)m + (size_t)p->ny * n)] = v;
      }
  ctx_free(&c);
}

/* ------------------------------------------------------------------------ */
/* One interior cell of rhs_cpu (equ.f90:1386): calc_all_pencils then
   calc_all_rhs (equ.f90:1223) in module order hydro -> density -> energy ->
   magnetic, each adding into df.  Returns the CFL inverse timestep
   (set_dt1_max, equ.f90:1872) and accumulates diagnostics. */
static double cell(const orc_params* p, const ctx_t* c, const double* f, double* df, double alpha,
                   int l, int m, int n, double* dg) {
  const int iux = c->iux, ilnrho = c->ilnrho, iss = c->iss, iax = c->iax;
  double uu[3], uij[3][3];
  for (int i = 0; i < 3; ++i) {
    uu[i] = f[IDX(c, l, m, n, iux + i)];
    for (int j = 0; j < 3; ++j) uij[i][j] = der_c(c, f, iux + i, j, l, m, n);   /* gij, sub.f90:1505 */
  }
  /* u2: dot2_mn, sub.f90:897 */
  double u2 = (uu[0] * uu[0] + uu[1] * uu[1]) + uu[2] * uu[2];
  /* divu: div_mn, sub.f90:1981 */
  double divu = (uij[0][0] + uij[1][1]) + uij[2][2];
  /* sij: traceless_strain, sub.f90:8922 */
  double sij[3][3];
  for (int j = 0; j < 3; ++j) {
    sij[j][j] = uij[j][j] - (1.0 / 3.0) * divu;
    for (int i = j + 1; i < 3; ++i) {
      sij[i][j] = 0.5 * (uij[i][j] + uij[j][i]);
      sij[j][i] = sij[i][j];
    }
  }
  /* sij2: multm2_sym_mn, sub.f90:1207 */
  double sij2 = sij[0][0] * sij[0][0];
  for (int i = 1; i < 3; ++i) {
    sij2 = sij2 + sij[i][i] * sij[i][i];
    for (int j = 0; j < i; ++j) sij2 = sij2 + 2.0 * (sij[i][j] * sij[i][j]);
  }
  /* ugu: u_dot_grad_vec -> dot_mn(uu, uij(:,j,:)), sub.f90:3482/:599;
     with lupw_uu, minus the upwind correction (doupwind, sub.f90:7541) */
  double ugu[3];
  for (int j = 0; j < 3; ++j) {
    ugu[j] = (uu[0] * uij[j][0] + uu[1] * uij[j][1]) + uu[2] * uij[j][2];
    if (p->lupw_uu) ugu[j] = ugu[j] - del6_upwind(c, f, iux + j, uu, l, m, n);
  }
  /* del2u, graddivu: del2v_etc, sub.f90:2610 */
  double fijj[3][3], fjji[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      fijj[i][j] = der2_c(c, f, iux + i, j, l, m, n);
      fjji[i][j] = (i == j) ? fijj[i][j] : derij_c(c, f, iux + j, j, i, l, m, n);
    }
  double del2u[3], graddivu[3];
  for (int i = 0; i < 3; ++i) {
    del2u[i] = (fijj[i][0] + fijj[i][1]) + fijj[i][2];
    graddivu[i] = (fjji[i][0] + fjji[i][1]) + fjji[i][2];
  }
  /* density pencils, density.f90:2747-2800 */
  double lnrho = f[IDX(c, l, m, n, ilnrho)];
  double rho1 = exp(-lnrho);
  double glnrho[3];
  for (int j = 0; j < 3; ++j) glnrho[j] = der_c(c, f, ilnrho, j, l, m, n);
  double uglnrho = (uu[0] * glnrho[0] + uu[1] * glnrho[1]) + uu[2] * glnrho[2];
  if (p->lupw_lnrho) uglnrho = uglnrho - del6_upwind(c, f, ilnrho, uu, l, m, n);   /* density.f90:2772 */
  double sglnrho[3];
  for (int i = 0; i < 3; ++i)   /* multmv_mn, sub.f90:1228 */
    sglnrho[i] = (sij[i][0] * glnrho[0] + sij[i][1] * glnrho[1]) + sij[i][2] * glnrho[2];

  /* EOS, eos_idealgas.f90:842-887 */
  double cs2, ss = 0, gss[3] = {0, 0, 0}, lnTT = 0, TT1 = 0, glnTT[3] = {0, 0, 0}, del2lnTT = 0;
  if (p->lentropy) {
    ss = f[IDX(c, l, m, n, iss)];
    for (int j = 0; j < 3; ++j) gss[j] = der_c(c, f, iss, j, l, m, n);
    double del2lnrho = (der2_c(c, f, ilnrho, 0, l, m, n) + der2_c(c, f, ilnrho, 1, l, m, n)) +
                       der2_c(c, f, ilnrho, 2, l, m, n);
    double del2ss = (der2_c(c, f, iss, 0, l, m, n) + der2_c(c, f, iss, 1, l, m, n)) +
                    der2_c(c, f, iss, 2, l, m, n);
    cs2 = c->cs20 * exp(c->cv1 * ss + c->gamma_m1 * (lnrho - c->lnrho0));
    lnTT = (c->lnTT0 + c->cv1 * ss) + c->gamma_m1 * (lnrho - c->lnrho0);
    TT1 = exp(-lnTT);
    for (int j = 0; j < 3; ++j) glnTT[j] = c->gamma_m1 * glnrho[j] + c->cv1 * gss[j];
    del2lnTT = c->gamma_m1 * del2lnrho + c->cv1 * del2ss;
  } else if (c->gamma_m1 == 0.0) {
    cs2 = c->cs20;                                   /* isothermal, noentropy.f90:100 */
  } else {
    cs2 = c->cs20 * exp(c->gamma_m1 * (lnrho - c->lnrho0));   /* polytropic, noentropy.f90:102 */
  }

  /* magnetic pencils, magnetic.f90:4310-4900 and gij_etc, sub.f90:2945 */
  double aa[3], aij[3][3], d2A[3][3][3];
  for (int i = 0; i < 3; ++i) {
    aa[i] = f[IDX(c, l, m, n, iax + i)];
    for (int j = 0; j < 3; ++j) aij[i][j] = der_c(c, f, iax + i, j, l, m, n);
    for (int j = 0; j < 3; ++j) d2A[j][j][i] = der2_c(c, f, iax + i, j, l, m, n);
    d2A[1][2][i] = derij_c(c, f, iax + i, 1, 2, l, m, n); d2A[2][1][i] = d2A[1][2][i];
    d2A[2][0][i] = derij_c(c, f, iax + i, 2, 0, l, m, n); d2A[0][2][i] = d2A[2][0][i];
    d2A[0][1][i] = derij_c(c, f, iax + i, 0, 1, l, m, n); d2A[1][0][i] = d2A[0][1][i];
  }
  double bb[3];   /* curl_mn, sub.f90:2058-2060 */
  bb[0] = aij[2][1] - aij[1][2];
  bb[1] = aij[0][2] - aij[2][0];
  bb[2] = aij[1][0] - aij[0][1];
  double bij[3][3];   /* gij_etc, sub.f90:3017-3019 */
  for (int k = 0; k < 3; ++k) {
    bij[0][k] = d2A[1][k][2] - d2A[2][k][1];
    bij[1][k] = d2A[2][k][0] - d2A[0][k][2];
    bij[2][k] = d2A[0][k][1] - d2A[1][k][0];
  }
  double del2a[3];   /* gij_etc, sub.f90:3085 */
  for (int i = 0; i < 3; ++i) del2a[i] = (d2A[0][0][i] + d2A[1][1][i]) + d2A[2][2][i];
  const double bbb[3] = {bb[0], bb[1], bb[2]};   /* p%bbb: B before B_ext, magnetic.f90:4356 */
  for (int j = 0; j < 3; ++j) bb[j] = bb[j] + p->b_ext[j];   /* B_ext, magnetic.f90:4366-4370 */
  double jj[3];   /* jj = mu01*curl(bij), magnetic.f90:4735 */
  jj[0] = c->mu01 * (bij[2][1] - bij[1][2]);
  jj[1] = c->mu01 * (bij[0][2] - bij[2][0]);
  jj[2] = c->mu01 * (bij[1][0] - bij[0][1]);
  double b2 = (bb[0] * bb[0] + bb[1] * bb[1]) + bb[2] * bb[2];
  double j2 = (jj[0] * jj[0] + jj[1] * jj[1]) + jj[2] * jj[2];
  double jxb[3], jxbr[3], uxb[3];   /* cross_mn, sub.f90:1466-1468 */
  jxb[0] = jj[1] * bb[2] - jj[2] * bb[1];
  jxb[1] = jj[2] * bb[0] - jj[0] * bb[2];
  jxb[2] = jj[0] * bb[1] - jj[1] * bb[0];
  for (int i = 0; i < 3; ++i) jxbr[i] = rho1 * jxb[i];   /* multsv_mn, magnetic.f90:4888 */
  uxb[0] = uu[1] * bb[2] - uu[2] * bb[1];
  uxb[1] = uu[2] * bb[0] - uu[0] * bb[2];
  uxb[2] = uu[0] * bb[1] - uu[1] * bb[0];

  /* ---- duu_dt, hydro.f90:4421 ---- */
  double dfu[3];
  for (int j = 0; j < 3; ++j) dfu[j] = alpha * df[IDX(c, l, m, n, iux + j)];
  for (int j = 0; j < 3; ++j) dfu[j] = dfu[j] - ugu[j];                 /* advec_uu, :4384 */
  for (int j = 0; j < 3; ++j) {                                          /* viscosity.f90:1638 */
    double fvisc = p->nu * ((del2u[j] + 2.0 * sglnrho[j]) + (1.0 / 3.0) * graddivu[j]);
    dfu[j] = dfu[j] + fvisc;                                             /* viscosity.f90:2822 */
  }
  if (p->lforcing_cont) {                                                /* forcing.f90:5894-5896 */
    double fc[3];
    fc[0] = c->fact * (p->abc_c * c->sinz[n] + (c->fact2 * p->abc_b) * c->cosy[m]);
    fc[1] = c->fact * (p->abc_a * c->sinx[l] + (c->fact2 * p->abc_c) * c->cosz[n]);
    fc[2] = c->fact * (p->abc_b * c->siny[m] + (c->fact2 * p->abc_a) * c->cosx[l]);
    for (int j = 0; j < 3; ++j) dfu[j] = dfu[j] + p->ampl_fcont_uu * fc[j];   /* hydro.f90:4609 */
  }
  /* ---- dlnrho_dt, density.f90:3290 / continuity_eq :2929-2930, :3059 ---- */
  double density_rhs = -divu;
  density_rhs = density_rhs - 1.0 * uglnrho;
  df[IDX(c, l, m, n, ilnrho)] = alpha * df[IDX(c, l, m, n, ilnrho)] + density_rhs;
  /* ---- denergy_dt ---- */
  double dfs = 0.0;
  if (!p->lentropy) {
    for (int j = 0; j < 3; ++j) dfu[j] = dfu[j] + (-(cs2 * glnrho[j]));   /* noentropy.f90:316, :383 */
  } else {
    for (int j = 0; j < 3; ++j)                                          /* entropy.f90:3599, :3727 */
      dfu[j] = dfu[j] + (-((cs2 * (glnrho[j] + glnTT[j])) * c->gamma1));
    double ugss = (uu[0] * gss[0] + uu[1] * gss[1]) + uu[2] * gss[2];
    dfs = alpha * df[IDX(c, l, m, n, iss)];
    dfs = dfs - ugss;                                                    /* entropy.f90:3775 */
    if (p->lviscosity_heat) {                                            /* viscosity.f90:2765 */
      double visc_heat = (2.0 * p->nu) * sij2;
      dfs = dfs + TT1 * visc_heat;
    }
    double gs[3] = {glnrho[0] + glnTT[0], glnrho[1] + glnTT[1], glnrho[2] + glnTT[2]};
    double g2 = (gs[0] * glnTT[0] + gs[1] * glnTT[1]) + gs[2] * glnTT[2];
    double thdiff = (p->chi * c->cpp) * (del2lnTT + g2);                 /* entropy.f90:4886 */
    dfs = dfs + thdiff;
  }
  /* ---- daa_dt, magnetic.f90:5392 ---- */
  for (int j = 0; j < 3; ++j) dfu[j] = dfu[j] + jxbr[j];                /* Lorentz, :5531 */
  for (int j = 0; j < 3; ++j) {
    double fres = p->eta * del2a[j];                                     /* :5589 */
    double dAdt = uxb[j] + fres;                                         /* :6247 */
    df[IDX(c, l, m, n, iax + j)] = alpha * df[IDX(c, l, m, n, iax + j)] + dAdt;   /* :6524 */
  }
  if (p->lentropy) {
    if (p->lohmic_heat) dfs = dfs + (((p->eta * p->mu0) * j2) * rho1) * TT1;   /* :6141 */
    df[IDX(c, l, m, n, iss)] = dfs;
  }
  for (int j = 0; j < 3; ++j) df[IDX(c, l, m, n, iux + j)] = dfu[j];

  /* ---- CFL, equ.f90:1858-1971 ---- */
  double advec_uu = (fabs(uu[0]) * c->dx_1 + fabs(uu[1]) * c->dy_1) + fabs(uu[2]) * c->dz_1;   /* hydro.f90:3500 */
  double maxadvec = advec_uu > 0.0 ? advec_uu : 0.0;
  double t0 = bb[0] * c->dx_1, t1 = bb[1] * c->dy_1, t2 = bb[2] * c->dz_1;
  double advec_va2 = (((t0 * t0 + t1 * t1) + t2 * t2) * c->mu01) * rho1;   /* magnetic.f90:5180 */
  double advec_cs2 = cs2 * c->dxyz_2;                                    /* noentropy.f90:316 */
  double advec2 = (0.0 + advec_va2) + advec_cs2;
  maxadvec = maxadvec + sqrt(advec2);
  double maxdiffus = 0.0;
  double dn = p->nu * c->dxyz_2; if (dn > maxdiffus) maxdiffus = dn;      /* viscosity.f90:2436 */
  double de = p->eta * c->dxyz_2; if (de > maxdiffus) maxdiffus = de;     /* magnetic.f90:6541 */
  if (p->lentropy) { double dc = (p->gamma * p->chi) * c->dxyz_2; if (dc > maxdiffus) maxdiffus = dc; }
  double dt1_advec = maxadvec / p->cdt;
  double dt1_diffus = maxdiffus / p->cdtv;
  double dt1 = sqrt(dt1_advec * dt1_advec + dt1_diffus * dt1_diffus);

  if (dg) {
    double rho = exp(lnrho);
    double divb = (bij[0][0] + bij[1][1]) + bij[2][2];
    double ab = (aa[0] * bbb[0] + aa[1] * bbb[1]) + aa[2] * bbb[2];   /* p%ab = aa.bbb, magnetic.f90:4451 */
    dg[ORC_D_U2SUM] += u2;
    if (u2 > dg[ORC_D_U2MAX]) dg[ORC_D_U2MAX] = u2;
    dg[ORC_D_B2SUM] += b2;
    if (b2 > dg[ORC_D_B2MAX]) dg[ORC_D_B2MAX] = b2;
    dg[ORC_D_EKINSUM] += 0.5 * rho * u2;
    dg[ORC_D_RHOSUM] += rho;
    dg[ORC_D_DIVB2SUM] += divb * divb;
    dg[ORC_D_J2SUM] += j2;
    dg[ORC_D_ABSUM] += ab;
    dg[ORC_D_JBSUM] += (jj[0] * bbb[0] + jj[1] * bbb[1]) + jj[2] * bbb[2];   /* p%jb = jj.bbb, magnetic.f90:4781 */
    dg[ORC_D_EPSKSUM] += ((2.0 * p->nu) * sij2) * rho;                      /* visc_heat*rho, viscosity.f90:2908 */
  }
  return dt1;
}

void orc_pde(const orc_params* p, const double* f, double* df, double alpha, int want_dt,
             double* dt1_max, double* diag, int nthreads) {
  ctx_t c; ctx_init(&c, p);
  int ny = p->ny, nz = p->nz, nyz = ny * nz;
  double* pen_dt = malloc(sizeof(double) * nyz);
  double* pen_dg = diag ? calloc((size_t)nyz * ORC_D_N, sizeof(double)) : NULL;
  if (nthreads <= 0) nthreads = 1;
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(nthreads)
#endif
  for (int imn = 0; imn < nyz; ++imn) {     /* mn-loop, equ.f90:1443 */
    int m = NG + imn % ny, n = NG + imn / ny;
    double mx_dt = 0.0;
    double* dg = pen_dg ? pen_dg + (size_t)imn * ORC_D_N : NULL;
    for (int l = NG; l < NG + p->nx; ++l) {
      double d = cell(p, &c, f, df, alpha, l, m, n, dg);
      if (d > mx_dt) mx_dt = d;
    }
    pen_dt[imn] = mx_dt;
  }
  if (want_dt && dt1_max) {
    double mxv = 0.0;
    for (int i = 0; i < nyz; ++i) if (pen_dt[i] > mxv) mxv = pen_dt[i];
    *dt1_max = mxv;
  }
  if (diag) {
    for (int i = 0; i < nyz; ++i)
      for (int s = 0; s < ORC_D_N; ++s) {
        double v = pen_dg[(size_t)i * ORC_D_N + s];
        if (s == ORC_D_U2MAX || s == ORC_D_B2MAX) { if (v > diag[s]) diag[s] = v; }
        else diag[s] += v;
      }
  }
  free(pen_dt); free(pen_dg);
  ctx_free(&c);
}

/* time_step / advance_substeps, src/timestep.f90:77-202, itorder=3 with the
   Williamson (1980) coefficients of :43-44. */
void orc_time_step(const orc_params* p, double* f, double* df, double* t, double* dt, int ldt,
                   double* diag, int nthreads) {
  const double alpha_ts[3] = {0.0, -5.0 / 9.0, -153.0 / 128.0};
  const double beta_ts[3] = {1.0 / 3.0, 15.0 / 16.0, 8.0 / 15.0};
  int nf = orc_nfields(p);
  int mx = p->nx + 2 * NG, my = p->ny + 2 * NG;
  double ds = 0.0;
  for (int itsub = 0; itsub < 3; ++itsub) {
    double alpha = alpha_ts[itsub];
    if (itsub == 0) ds = 0.0; else ds = alpha * ds;
    orc_boundconds(p, f, nf);
    double dt1 = 0.0;
    /* substep 1 with df = 0 (alpha = 0 makes alpha*df = 0 for finite df) */
    if (itsub == 0) {
      const size_t nfield = (size_t)mx * my * (p->nz + 2 * NG);
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(nthreads > 0 ? nthreads : 1)
#endif
      for (int k = 0; k < nf * (p->nz + 2 * NG); ++k)
        memset(df + (size_t)k * (nfield / (p->nz + 2 * NG)), 0, nfield / (p->nz + 2 * NG) * sizeof(double));
    }
    orc_pde(p, f, df, alpha, ldt && itsub == 0, &dt1, itsub == 0 ? diag : NULL, nthreads);
    if (ldt && itsub == 0) *dt = 1.0 / dt1;          /* set_dt, sub.f90:4247 */
    ds = ds + 1.0;
    double dt_beta = *dt * beta_ts[itsub];
    double dtsub = ds * dt_beta;
    /* timestep.f90:160-161; every element is independent, so the threads
       change nothing in the result */
#ifdef _OPENMP
#pragma omp parallel for collapse(2) schedule(static) num_threads(nthreads > 0 ? nthreads : 1)
#endif
    for (int k = 0; k < nf; ++k)
      for (int n = NG; n < NG + p->nz; ++n)
        for (int m = NG; m < NG + p->ny; ++m) {
          size_t o = (size_t)mx * ((size_t)m + (size_t)my * ((size_t)n + (size_t)(p->nz + 2 * NG) * k));
          for (int l = NG; l < NG + p->nx; ++l) f[o + l] = f[o + l] + dt_beta * df[o + l];
        }
    *t = *t + dtsub;
  }
}

/* ran0, general.f90:867-889 ('Minimal Standard', Lewis-Goodman-Miller with
   the reference's XOR mask). */
double orc_ran0(int* dummy) {
  const int ia = 16807, im = 2147483647, iq = 127773, ir = 2836, mask = 123459876;
  const double am = 1.0 / (double)im;
  int k;
  *dummy = *dummy ^ mask;
  k = *dummy / iq;
  *dummy = ia * (*dummy - k * iq) - ir * k;
  if (*dummy < 0) *dummy = *dummy + im;
  double r = am * (double)(*dummy);
  *dummy = *dummy ^ mask;
  return r;
}

/* gaunoise_vect, initcond.f90:5005-5047: over the full ghosted volume,
   components i1..i2 (0-based), sin for even offsets (fresh r,p) and cos for
   odd offsets (reusing r,p). */
void orc_gaunoise_vect(const orc_params* p, double ampl, double* f, int i1, int i2, int* state) {
  int mx = p->nx + 2 * NG, my = p->ny + 2 * NG, mz = p->nz + 2 * NG;
  const double pi = 3.14159265358979323846264338327950;
  double* r = malloc(sizeof(double) * mx);
  double* q = malloc(sizeof(double) * mx);
  if (ampl == 0.0) { free(r); free(q); return; }
  for (int n = 0; n < mz; ++n)
    for (int m = 0; m < my; ++m)
      for (int i = i1; i <= i2; ++i) {
        size_t o = (size_t)mx * ((size_t)m + (size_t)my * ((size_t)n + (size_t)mz * i));
        if ((i - i1) % 2 == 0) {
          for (int l = 0; l < mx; ++l) r[l] = orc_ran0(state);
          for (int l = 0; l < mx; ++l) q[l] = orc_ran0(state);
          for (int l = 0; l < mx; ++l) f[o + l] = f[o + l] + ampl * (sqrt(-2.0 * log(r[l])) * sin((2.0 * pi) * q[l]));
        } else {
          for (int l = 0; l < mx; ++l) f[o + l] = f[o + l] + ampl * (sqrt(-2.0 * log(r[l])) * cos((2.0 * pi) * q[l]));
        }
      }
  free(r); free(q);
}

/* gaunoise_vect's draws and sin/cos pairing (initcond.f90:5026-5040) with
   volume arrays filled by random_number_wrapper_3 (general.f90:733-739): the
   loops run x outermost and z innermost, so consecutive draws step along z.
   The reference.out of samples/MHD-ABCforcing (brms 1.684E-01, jbm 2.24E-03,
   b1b32m 2.17E-04, epsM 8.11E-01, abm 9.67E-06 at it=0) is this realisation
   of seed -10; the pencil-wise fill of orc_gaunoise_vect is not. */
void orc_gaunoise_volume(const orc_params* p, double ampl, double* f, int i1, int i2, int* state) {
  const size_t mx = (size_t)p->nx + 2 * NG, my = (size_t)p->ny + 2 * NG, mz = (size_t)p->nz + 2 * NG;
  const size_t nv = mx * my * mz;
  const double pi = 3.14159265358979323846264338327950;
  if (ampl == 0.0) return;
  double* r = malloc(sizeof(double) * nv);
  double* q = malloc(sizeof(double) * nv);
  for (int i = i1; i <= i2; ++i) {
    double* fi = f + nv * (size_t)i;
    if ((i - i1) % 2 == 0) {
      for (size_t l = 0; l < mx; ++l)          /* random_number_wrapper_3(r) */
        for (size_t m = 0; m < my; ++m)
          for (size_t n = 0; n < mz; ++n) r[l + mx * (m + my * n)] = orc_ran0(state);
      for (size_t l = 0; l < mx; ++l)          /* random_number_wrapper_3(p) */
        for (size_t m = 0; m < my; ++m)
          for (size_t n = 0; n < mz; ++n) q[l + mx * (m + my * n)] = orc_ran0(state);
      for (size_t o = 0; o < nv; ++o) fi[o] = fi[o] + ampl * (sqrt(-2.0 * log(r[o])) * sin((2.0 * pi) * q[o]));
    } else {
      for (size_t o = 0; o < nv; ++o) fi[o] = fi[o] + ampl * (sqrt(-2.0 * log(r[o])) * cos((2.0 * pi) * q[o]));
    }
  }
  free(r); free(q);
}

/* fconst_coefs_hel, forcing.f90:1763-1880 (default options: no shear, no
   k-vector scaling, the new polarisation vectors, fda = 1, slope_ff = 0). */
void orc_helical_coefs(const orc_params* p, double force, const double* kkx, const double* kky, const double* kkz,
                       int nk, double kav, int* state, orc_helrec* rec) {
  const double pi = 3.14159265358979323846264338327950;
  const double fran1 = orc_ran0(state), fran2 = orc_ran0(state);
  const double phase = pi * (2.0 * fran1 - 1.0);
  const int ik = (int)((double)nk * (0.9999 * fran2) + 1.0);   /* 1-based */
  const double kx = kkx[ik - 1], ky = kky[ik - 1], kz = kkz[ik - 1];
  const double k2 = (kx * kx + ky * ky) + kz * kz;
  const double k = sqrt(k2);
  double ex, ey, ez;
  if (ky == 0.0 && kz == 0.0) { ex = 0.0; ey = 1.0; ez = 0.0; } else { ex = 1.0; ey = 0.0; ez = 0.0; }
  /* e1 = kk x ee, e2 = kk x e1, unit vectors (sub.f90 cross / dot2) */
  double e1[3] = {ky * ez - kz * ey, kz * ex - kx * ez, kx * ey - ky * ex};
  double norm = (e1[0] * e1[0] + e1[1] * e1[1]) + e1[2] * e1[2];
  for (int i = 0; i < 3; ++i) e1[i] = e1[i] / sqrt(norm);
  double e2[3] = {ky * e1[2] - kz * e1[1], kz * e1[0] - kx * e1[2], kx * e1[1] - ky * e1[0]};
  norm = (e2[0] * e2[0] + e2[1] * e2[1]) + e2[2] * e2[2];
  for (int i = 0; i < 3; ++i) e2[i] = e2[i] / sqrt(norm);
  const double phi = orc_ran0(state) * 2.0 * pi;
  ex = cos(phi) * e1[0] + sin(phi) * e2[0];
  ey = cos(phi) * e1[1] + sin(phi) * e2[1];
  ez = cos(phi) * e1[2] + sin(phi) * e2[2];
  const double kde = (kx * ex + ky * ey) + kz * ez;
  const double kex = ky * ez - kz * ey, key = kz * ex - kx * ez, kez = kx * ey - ky * ex;
  const double kkex = ky * kez - kz * key, kkey = kz * kex - kx * kez, kkez = kx * key - ky * kex;
  const double cs0eff = p->cs0;
  const double ffnorm = sqrt(1.0 + p->relhel * p->relhel) * k * sqrt(k2 - kde * kde) / sqrt(kav * (cs0eff * cs0eff * cs0eff));
  rec->kk[0] = kx; rec->kk[1] = ky; rec->kk[2] = kz;
  rec->phase = phase;
  rec->coef1[0] = k * kex; rec->coef1[1] = k * key; rec->coef1[2] = k * kez;
  rec->coef2[0] = p->relhel * kkex; rec->coef2[1] = p->relhel * kkey; rec->coef2[2] = p->relhel * kkez;
  rec->fact0 = force / ffnorm;
}

/* forcing_hel, forcing.f90:2066-2474, default path, with fxyz_coefs_hel
   (:1882-1930): fx = exp(i(kx k1 x + phase)) fact, fy = exp(i ky k1 y),
   fz = exp(i kz k1 z); f(uu_j) += Re[(coef1_j + i coef2_j) (fx fy) fz]. */
void orc_add_helical(const orc_params* p, double* f, const orc_helrec* rec, double dt, int target) {
  const int mx = p->nx + 2 * NG, my = p->ny + 2 * NG, mz = p->nz + 2 * NG;
  const int j0 = target ? (p->lentropy ? 5 : 4) : 0;   /* iax or iux, 0-based */
  const double fact = rec->fact0 * sqrt(dt);
  const double k1 = p->kf;
  double* x = malloc(sizeof(double) * (mx + my + mz));
  double* y = x + mx;
  double* z = y + my;
  orc_grid(p, x, y, z);
  for (int n = NG; n < NG + p->nz; ++n) {
    const double az = rec->kk[2] * k1 * z[n];
    const double fzr = cos(az), fzi = sin(az);
    for (int m = NG; m < NG + p->ny; ++m) {
      const double ay = rec->kk[1] * k1 * y[m];
      const double fyr = cos(ay), fyi = sin(ay);
      for (int l = NG; l < NG + p->nx; ++l) {
        const double ax = rec->kk[0] * k1 * x[l] + rec->phase;
        const double fxr = cos(ax) * fact, fxi = sin(ax) * fact;
        const double pr = fxr * fyr - fxi * fyi, pim = fxr * fyi + fxi * fyr;   /* fx fy */
        const double qr = pr * fzr - pim * fzi, qi = pr * fzi + pim * fzr;      /* (fx fy) fz */
        for (int j = 0; j < 3; ++j) {
          const size_t o = (size_t)l + (size_t)mx * ((size_t)m + (size_t)my * ((size_t)n + (size_t)mz * (j0 + j)));
          f[o] = f[o] + (rec->coef1[j] * qr - rec->coef2[j] * qi);
        }
      }
    }
  }
  free(x);
}
