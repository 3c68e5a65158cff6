/*
 * pc_oracle.h -- CPU FP64 restatement of the Pencil Code compressible-MHD
 * timestep (the pde() right-hand side + 2N-storage RK3 update).
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the parity oracle: it is linked
 * by tests/, by __graft_entry__.smoke() and by the CPU-baseline leg of
 * bench.py, always as the checker and never as the thing measured or shipped.
 * The product (libpcgb300.so) does not link it and has no CPU fallback.
 *
 * Layout: f(mx,my,mz,nf) Fortran column-major, x fastest, ghosts included
 * (nghost = 3), exactly the reference f-array (src/cparam.f90:19-59).
 * Variable order (src/register.f90:138-146): uu(1:3), lnrho, [ss], aa(1:3).
 */
#ifndef PC_ORACLE_H
#define PC_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_NGHOST 3

typedef struct {
  int nx, ny, nz;           /* interior cells */
  int lentropy;             /* 0: noentropy (7 fields), 1: entropy (8 fields) */
  double x0, y0, z0;        /* xyz0 (cdata.f90:211 default -pi) */
  double Lx, Ly, Lz;        /* Lxyz (default 2 pi) */
  double gamma, cs0, rho0, cp;
  double nu, eta, chi, mu0;
  int lforcing_cont;        /* ABC continuous forcing into duu */
  double ampl_ff, kf, relhel, abc_a, abc_b, abc_c, ampl_fcont_uu;
  double b_ext[3];
  int lohmic_heat, lviscosity_heat;
  double cdt, cdtv;
  int lupw_uu, lupw_lnrho;  /* upwinded advection (hydro.f90:3662, density.f90:2772) */
  int bc[3][8][2];          /* boundary condition of direction, field, side (0 lower, 1 upper):
                               0 'p', 1 's', 2 'a', 3 'a2' (boundcond.f90); all 0 = periodic */
} orc_params;

enum { ORC_BC_PER = 0, ORC_BC_SYM = 1, ORC_BC_ASYM = 2, ORC_BC_ASYM2 = 3 };

/* Diagnostic slots (FP64), evaluated on f at the start of a step. */
enum {
  ORC_D_U2SUM = 0, ORC_D_U2MAX, ORC_D_B2SUM, ORC_D_B2MAX, ORC_D_EKINSUM,
  ORC_D_RHOSUM, ORC_D_DIVB2SUM, ORC_D_J2SUM, ORC_D_ABSUM, ORC_D_JBSUM, ORC_D_EPSKSUM, ORC_D_N
};

int  orc_nfields(const orc_params* p);
void orc_grid(const orc_params* p, double* x, double* y, double* z);

/* Periodic ghost filling, x then y then z (src/boundcond.f90:2387-2531). */
/* Ghost zones as pde sets them before the RHS (equ.f90: boundconds_x, _y, _z),
   with bc_per_x/y/z (boundcond.f90:2387-2531) and bc_sym_x/y/z (:2637-2677,
   :3483-3530, :3842-3900) per field and side. */
void orc_boundconds(const orc_params* p, double* f, int nf);

/* Stencils on a single interior point (0-based ghosted indices l,m,n),
   field k, direction j (0,1,2).  deriv.f90:89 / :472 / :1367. */
double orc_der(const orc_params* p, const double* f, int k, int j, int l, int m, int n);
double orc_der2(const orc_params* p, const double* f, int k, int j, int l, int m, int n);
double orc_derij(const orc_params* p, const double* f, int k, int i, int j, int l, int m, int n);

/* Whole-interior stencil helpers used by the golden-vector tests:
   out is (nx,ny,nz) x fastest.  kind: 0 der, 1 der2, 2 derij(i,j). */
void orc_stencil_field(const orc_params* p, const double* f, int k, int kind, int i, int j,
                       double* out);

/* df(interior) = alpha*df + RHS(f).  f must have valid ghosts.
   When want_dt: *dt1_max = max over cells of the CFL inverse timestep.
   When diag != NULL: accumulates the ORC_D_* slots (sums and maxima). */
void orc_pde(const orc_params* p, const double* f, double* df, double alpha,
             int want_dt, double* dt1_max, double* diag, int nthreads);

/* One full RK3 step (src/timestep.f90:77-202):  fills ghosts, runs the three
   substeps, updates *t.  If ldt: dt is set from the CFL condition on substep
   1 (src/sub.f90:4223) and returned through *dt.  diag may be NULL. */
void orc_time_step(const orc_params* p, double* f, double* df, double* t, double* dt,
                   int ldt, double* diag, int nthreads);

/* Random helical forcing (iforce='helical'), default path: one record per
   time step from fconst_coefs_hel (src/forcing.f90:1763-1880) -- wavevector
   k drawn from the k.dat list, phase and polarisation angle from the random
   stream (two draws fran(1:2), then phi, as the reference draws them; here the
   stream is ran0) -- then forcing_hel (:2066-2474) with fxyz_coefs_hel
   (:1882-1930) adds Re[(coef1 + i coef2) fx fy fz] to uu after the step
   (addforce, :1307), fact = force/ffnorm*sqrt(dt).  k1_ff is p->kf, cs0eff
   is p->cs0 (initialize_forcing, :1075-1082), slope_ff = 0. */
typedef struct {
  double kk[3], phase, coef1[3], coef2[3], fact0;   /* fact0 = force/ffnorm (times sqrt(dt) on use) */
} orc_helrec;
void orc_helical_coefs(const orc_params* p, double force, const double* kkx, const double* kky, const double* kkz,
                       int nk, double kav, int* state, orc_helrec* rec);
/* f(uu) (target 0) or f(aa) (target 1, magnetic forcing) += forcing over the
   interior (ghosts are the caller's to refresh). */
void orc_add_helical(const orc_params* p, double* f, const orc_helrec* rec, double dt, int target);

/* The reference 'min_std' generator ran0 (src/general.f90:867-889) and
   gaunoise_vect (src/initcond.f90:5005-5047). */
double orc_ran0(int* state);
void orc_gaunoise_vect(const orc_params* p, double ampl, double* f, int i1, int i2, int* state);
/* The same Box-Muller pairing over whole volumes: per drawn component one
   (mx,my,mz) array of radii and one of phases, each filled by
   random_number_wrapper_3 (src/general.f90:733-739: z fastest, x slowest).
   This is the realisation printed in samples/MHD-ABCforcing/reference.out. */
void orc_gaunoise_volume(const orc_params* p, double ampl, double* f, int i1, int i2, int* state);

#ifdef __cplusplus
}
#endif
#endif
