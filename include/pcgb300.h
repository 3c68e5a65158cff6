/*
 * pcgb300.h -- C ABI of libpcgb300.so, the GB300-native replacement for the
 * Pencil Code GPU plug-in (the library the Fortran module `GPU`,
 * src/gpu_astaroth.f90, links through src/gpu_astaroth_ansi.c).
 *
 * Two groups of entry points:
 *
 *  1. The reference plug-in set, same names, argument meaning and void
 *     returns as the C-linkage prototypes of src/gpu_astaroth_ansi.c:23-55
 *     (implemented by src/astaroth/gpu_astaroth.cc in the reference), plus
 *     the Fortran-callable FTNIZE wrappers of src/gpu_astaroth_ansi.c:72-289
 *     (`name_`, gfortran convention, src/headers_c.h:30-37).  REAL is double
 *     (the REAL_PRECISION=double build, src/headers_c.h:11-25); FINT is int.
 *
 *  2. Native extensions (prefix pcgb_): the parameter block that stands in for
 *     the Fortran module variables the reference reads by address
 *     (src/global_pushpars.f90:6-60, gpu_astaroth_ansi.c:59-61), error
 *     reporting, and the box / batch / server API used for ensembles and
 *     serving.
 *
 * Errors: the reference prints and exits (gpu_astaroth.cc:2074-2078).  Here
 * every failure is recorded in a sticky code read by pcgb_last_error(); no
 * call blocks without a bound.
 */
#ifndef PCGB300_H
#define PCGB300_H

#include <stddef.h>
#include <stdbool.h>

#ifdef __cplusplus
extern "C" {
#endif

/* REAL of the Fortran build the plug-in entry points serve (headers_c.h:11-25):
   double in libpcgb300.so (REAL_PRECISION=double), float in libpcgb300_sgl.so,
   the same library compiled with PCGB_REAL_SINGLE for the single-precision
   build.  The device state's precision is pcgb_params.precision in both. */
#ifdef PCGB_REAL_SINGLE
typedef float REAL_PCGB;
#else
typedef double REAL_PCGB;
#endif

/* ---------------------------------------------------------------------------
 * Parameter block.  Field meanings follow the reference namelists:
 *   &init_pars xyz0, Lxyz (param_io.f90:82), grid sizes (cparam.local),
 *   &eos_init_pars gamma, cs0, rho0, cp (eos_idealgas.f90),
 *   &viscosity_run_pars nu (ivisc='nu-const'), &magnetic_run_pars eta, b_ext,
 *   &entropy_run_pars chi (iheatcond='chi-const'),
 *   &forcing_run_pars iforcing_cont='ABC', ampl_ff, k1_ff, relhel,
 *   &hydro_run_pars lforcing_cont_uu / ampl_fcont_uu,
 *   &run_pars dt, cdt, cdtv (cdata.f90:235-239).
 * ------------------------------------------------------------------------- */
typedef struct pcgb_params {
  int nx, ny, nz;          /* nxgrid, nygrid, nzgrid; each >= 6 */
  int lentropy;            /* 0: ENTROPY=noentropy (7 fields), 1: entropy (8 fields) */
  int precision;           /* device state: 8 = FP64, 4 = FP32 */
  int comp;                /* FP32 only: compensated 2N accumulation (1 = on) */
  double xyz0[3], Lxyz[3];
  double gamma, cs0, rho0, cp;
  double nu, eta, chi, mu0;
  int lforcing_cont;       /* continuous ABC forcing added to duu */
  double ampl_ff, kf, relhel, abc_a, abc_b, abc_c, ampl_fcont_uu;
  double b_ext[3];
  int lohmic_heat, lviscosity_heat;
  double cdt, cdtv;
  double dt;               /* fixed dt; 0 selects the CFL timestep (ldt) */
  int dt_mode;             /* with dt == 0: 1 = lagged (reference GPU default), 2 = current (CPU semantics) */
  int diag_every;          /* device diagnostics every diag_every steps (0: on request only) */
  int tile;                /* kernel tile variant, -1 = choose automatically.  FP32: 0-3 field-major
                              (32,4) (32,8) (16,8) (64,4); 4-7 packed pairs (32,4) (32,8) (16,8)
                              (32,12), 5 and 7 with the z data in tensor memory; FP64: (32,4)
                              (16,8) (24,8) (32,6); double-float pairs 4-7: (24,8) (16,12) (16,8)
                              (32,4).  Upwinding variants: FP32 tiles 1, 5, 6; FP64 1-3;
                              double-float 2, 3, 5, 6. */
  int zdepth;              /* z-sweep depth, 0 = choose automatically */
  int dfloat;              /* precision 8 only: 1 = FP64-class state and arithmetic as double-float
                              pairs (hi + lo FP32, 48-bit significand) on the FP32 pipes instead of
                              native FP64, whose rate on this GPU is 1/64 of FP32's */
  int lforcing_hel;        /* random helical forcing (&forcing_run_pars iforce='helical') added to uu
                              after every step; wavevectors from pcgb_box_set_kvectors / pcgb_set_kvectors */
  int seed_ff;             /* seed of the forcing's random stream (ran0, general.f90:867) */
  double force_hel;        /* &forcing_run_pars force (amplitude of the helical forcing) */
  int lupw_uu;             /* &hydro_run_pars lupw_uu: u.grad u minus sum_j |u_j| D6_j u (hydro.f90:3662,
                              sub.f90:7491); runs the upwinding kernel variant of the tile */
  int lupw_lnrho;          /* &density_run_pars lupw_lnrho: the same correction of u.grad lnrho
                              (density.f90:2772) */
  int lmagnetic_forcing;   /* &forcing_run_pars lmagnetic_forcing with iforce='helical': the force goes
                              into aa; each step also draws the secondary record of lmhd_forcing, whose
                              force on uu is zero for crosshel = 0 (forcing.f90:314-345, :2136-2311) */
  int pad_;                /* keeps the struct a multiple of 8 bytes; set to 0 */
  int bc[3][8][2];         /* boundary condition of direction x/y/z, field (f-array order), side
                              (0 lower, 1 upper): PCGB_BC_* codes (&init_pars bcx/bcy/bcz,
                              boundcond.f90); all 0 = periodic.  A direction is periodic when every
                              code is PCGB_BC_PER and non-periodic when none is; its grid then has
                              points on both boundaries, dx = L/(n-1) (grid.f90:123-151) */
} pcgb_params;

/* Boundary condition codes (boundcond.f90 bcx/bcy/bcz, bc_sym_x/y/z:2637,3483,3842). */
#define PCGB_BC_PER 0    /* 'p'  periodic */
#define PCGB_BC_SYM 1    /* 's'  f(n1-i) = f(n1+i) */
#define PCGB_BC_ASYM 2   /* 'a'  f(n1-i) = -f(n1+i), f(n1) = 0 */
#define PCGB_BC_ASYM2 3  /* 'a2' f(n1-i) = 2 f(n1) - f(n1+i) */

/* Defaults of the reference (cdata.f90:211,235,239; eos_idealgas.f90:47;
   forcing.f90:37,129; hydro.f90:283; magnetic.f90:247; entropy.f90:139). */
void pcgb_default_params(pcgb_params* p);

/* Set the parameters used by initializeGPU / reloadConfig (stands in for the
   Fortran module variables, src/global_pushpars.f90). Returns 0 or an error. */
int pcgb_set_params(const pcgb_params* p);

/* Sticky error code of the last failing call (0 = none) and its text. */
int pcgb_last_error(void);
const char* pcgb_error_string(int code);
void pcgb_clear_error(void);

/* Stream used for all device work (default: a library-owned stream).  Passing
   a cudaStream_t lets a caller time the kernels with its own events. */
void pcgb_set_stream(void* cuda_stream);
void* pcgb_get_stream(void);

/* ---------------------------------------------------------------------------
 * 1. Reference plug-in entry points (src/gpu_astaroth_ansi.c:23-55).
 * ------------------------------------------------------------------------- */

/* gpu_astaroth_ansi.c:23 -- registration hook (allocations happen in initializeGPU). */
void registerGPU(void);
/* gpu_astaroth_ansi.c:24 -- bind the host f-array f(mx,my,mz,mvar) (Fortran
   order, ghosts included), allocate device state for the parameter block set
   by pcgb_set_params, and set time t.  comm is ignored (one GPU).
   cpu_dt != 0 selects the CPU timestep semantics (lcpu_timestep_on_gpu,
   gpu_astaroth.f90:19-23); autotune != 0 runs the tile autotuner. */
void initializeGPU(REAL_PCGB* f, int comm, double t, int nt, int read_all, int cpu_dt, int autotune);
/* gpu_astaroth_ansi.c:25 -- free all device state. */
void finalizeGPU(void);
/* gpu_astaroth_ansi.c:26 -- device pointer of the input f buffer (getFArrayIn). */
void getFArrayIn(REAL_PCGB** p);
/* gpu_astaroth_ansi.c:27 -- one full RK substep (RHS, 2N update, ghosts, dt on
   substep 1), gpu_astaroth.cc:1672.  isubstep is 1-based and must follow the
   device's own substep counter. */
void substepGPU(int isubstep, double t);
/* gpu_astaroth_ansi.c:28 -- nothing to do for this physics (gpu_astaroth.cc:1320). */
void beforeBoundaryGPU(bool lrmv, int isubstep, double t, bool lsubstep);
/* gpu_astaroth_ansi.c:29 -- nothing to do for this physics (gpu_astaroth.cc:1515). */
void afterSubStepGPU(void);
/* gpu_astaroth_ansi.c:30 -- no radiative transfer on this path. */
void radTransfer(void);
/* gpu_astaroth_ansi.c:31 -- copy the device f (mvar fields, ghosts included)
   into the host array f (gpu_astaroth.cc:1719). */
void copyFarray(REAL_PCGB* f);
/* gpu_astaroth_ansi.c:32 -- copy the bound host f-array to the device and
   refresh periodic ghosts (gpu_astaroth.cc:1947). */
void loadFarray(void);
/* gpu_astaroth_ansi.c:33 -- re-read the parameter block into device state. */
void reloadConfig(void);
/* gpu_astaroth_ansi.c:34-39 -- parameter updates by index or name.  Index
   order is the field order of pcgb_params' double members starting at xyz0;
   names are the pcgb_params member names.  *Name variants return 0 on
   success and -1 for an unknown name. */
void updateInConfigArr(int index);
int updateInConfigArrName(char* name);
void updateInConfigScal(int index, REAL_PCGB value);
int updateInConfigScalName(char* name, REAL_PCGB value);
void updateInConfigVec(int index, REAL_PCGB* value);
int updateInConfigVecName(char* name, REAL_PCGB* value);
/* gpu_astaroth_ansi.c:40 -- compute the first timestep if none is known
   (GpuCalcDt, gpu_astaroth.cc:546). */
void prepareForFirstSubstep(double t);
/* gpu_astaroth_ansi.c:41 -- not provided by the reference either. */
void random_initial_condition(void);
/* gpu_astaroth_ansi.c:42 -- reduced diagnostics of the last diagnostic step:
   dst[0..11] = urms, umax, brms, bmax, ekin, rhom, divbrms, jrms, abm, dt, t,
   step.  (The reference returns module-specific sums, gpu_astaroth.cc:2486.) */
void getGPUReducedVars(REAL_PCGB* dst);
/* gpu_astaroth_ansi.c:43 -- compare device ghost cells with a periodic fill
   of the device interior; prints the maximum difference (gpu_astaroth.cc:2283). */
void testBCs(void);
/* gpu_astaroth_ansi.c:44 -- split updates are not part of this path (no-op). */
void splitUpdate(const REAL_PCGB eps, const int max_iter);
/* gpu_astaroth_ansi.c:45 -- device pointers of the input and output f buffers.
   They point at this library's device layout, not at the reference's field
   buffers of stride mw = mx*my*mz (gpu_astaroth.cc:1833-1848): element
   (i, j, k, slice), interior i in [0,nx), sits at
     slice*fs + (k+3)*ps + (j+3)*px + xoff + i
   with xoff, px, ps = px*(ny+6), fs = ps*(nz+6) as pcgb_box_info reports them,
   and the element is the device state's type whatever REAL_PCGB is: float for
   precision 4, double for precision 8, a 16-byte (hi_a, hi_b, lo_a, lo_b) float
   quadruple for the double-float state.  Field-major tiles (0-3) hold one
   slice per field in f-array order; the pair tiles (4-7 of the FP32 and
   double-float states) hold four slices of field pairs (ux,ax) (uy,ay) (uz,az)
   (lnrho, ss or 0), interleaved per element.  copyFarray gives the reference
   layout on the host. */
void copyVBApointers(REAL_PCGB** in, REAL_PCGB** out);

/* gpu_astaroth_ansi.c:48-56 -- TorchFort hooks: not part of this path (no-ops). */
void tf_save_checkpoint_c_api(const char* a, const char* b);
void tf_save_model_c_api(const char* a, const char* b);
void tf_load_model_c_api(const char* a, const char* b);
void tf_load_model_checkpoint_c_api(const char* a, const char* b);
void tf_create_model_c_api(const char* a, const char* b, int comm, bool lmpicomm);
void tf_train_c_api(const char* a, REAL_PCGB* loss, int itsub, double t);
void tf_infer_c_api(const char* a, int itsub);
void print_debug(void);

/* Fortran-callable wrappers, gpu_astaroth_ansi.c:72-289 (gfortran: name_). */
void initialize_gpu_c_(REAL_PCGB* f, int* comm, double* t, int* nt, int* read_all, int* cpu_dt, int* autotune);
void register_gpu_c_(void);
void finalize_gpu_c_(void);
void get_farray_ptr_gpu_c_(REAL_PCGB** in, REAL_PCGB** out);
void before_boundary_gpu_c_(int* lrmv, int* isubstep, double* t, int* lsubstepping);
void update_after_substep_gpu_c_(void);
void rhs_gpu_c_(int* isubstep, double* t);
void copy_farray_c_(REAL_PCGB* f);
void load_farray_c_(void);
void reload_gpu_config_c_(void);
void update_on_gpu_scal_by_ind_c_(int* index, REAL_PCGB* value);
void update_on_gpu_vec_by_ind_c_(int* index, REAL_PCGB* value);
void update_on_gpu_arr_by_ind_c_(int* index);
int update_on_gpu_scal_by_name_c_(char* name, REAL_PCGB* value);
int update_on_gpu_vec_by_name_c_(char* name, REAL_PCGB* value);
int update_on_gpu_arr_by_name_c_(char* name);
void gpu_prepare_for_first_substep_c_(double* t);
void radtransfer_gpu_c_(void);
void get_gpu_reduced_vars_c_(REAL_PCGB* dst);
void test_bcs_c_(void);
void split_update_gpu_c_(void);
/* gpu_astaroth_ansi.c:72-108 -- TorchFort wrappers (no-ops, present for linking). */
void tf_train_c_(const char* model_name, REAL_PCGB* loss, int* itsub, double* t);
void tf_infer_c_(const char* model_name, int* itsub);
void tf_create_model_c_(const char* model_name, const char* config_file_path, int* comm, int* lmpicomm);
void print_snapshot_c_(void);
void tf_load_model_c_(const char* model_name, const char* fname);
void tf_load_model_checkpoint_c_(const char* model_name, const char* checkpoint_dir);
void tf_save_model_c_(const char* model_name, const char* fname);
void tf_save_checkpoint_c_(const char* model_name, const char* checkpoint_dir);

/* Timestep of the plug-in's box: the value Fortran's set_dt would receive
   (gpu_astaroth.cc:1618-1634 calls set_dt from C++; a C caller reads it). */
/* k.dat for the plug-in's box (see pcgb_box_set_kvectors); call before initializeGPU. */
int pcgb_set_kvectors(const double* kxyz, int nk, double kav);
double pcgb_get_dt(void);
double pcgb_get_time(void);
/* Request device diagnostics (urms, brms, ...) on the next substep 1. */
void pcgb_request_diagnostics(void);

/* Timestep driver mirroring Timestep.time_step with lgpu=T
   (src/timestep.f90:206 -> advance_substeps :77): nsteps full RK3 steps of
   the plug-in box, substepGPU(1..3) each.  Returns 0 or an error code. */
int pcgb_time_step(int nsteps);

/* ---------------------------------------------------------------------------
 * 2. Boxes, batches and serving (no reference counterpart: the reference
 *    drives one domain per process).
 * ------------------------------------------------------------------------- */
typedef struct pcgb_box pcgb_box;
typedef struct pcgb_batch pcgb_batch;

pcgb_box* pcgb_box_create(const pcgb_params* p);
void pcgb_box_destroy(pcgb_box* b);
/* f(mx,my,mz,nf) double, Fortran order, ghosts included (ghosts are refreshed on device).
   Page-locked host arrays are read or written in place by the layout kernels. */
int pcgb_box_load(pcgb_box* b, const double* f_host, double t);
int pcgb_box_store(pcgb_box* b, double* f_host);
/* The same with a float host f-array (the single-precision Fortran build).  The
   store rounds f (+ the FP32 compensation carry, summed in double) once to float. */
int pcgb_box_load_f32(pcgb_box* b, const float* f_host, double t);
int pcgb_box_store_f32(pcgb_box* b, float* f_host);
/* Seeded initial condition written on the device (for boxes too large to
   stage through host memory): kind 0 sets field to zero, 1 adds ampl*N(0,1)
   from a counter-based generator seeded by seed, 2 adds component `field`
   (0..2) of the ABC flow (hydro.f90:2214-2220) ampl*(a,b,c) at wavenumber k.
   Ghosts, df and the step bookkeeping are reset as after pcgb_box_load. */
int pcgb_box_init_field(pcgb_box* b, int field, int kind, double ampl, double a, double bb, double c, double k,
                        unsigned long long seed);
/* Run nsteps RK3 steps (3 launches each, or 4 with dt_mode = 2). */
int pcgb_box_steps(pcgb_box* b, int nsteps);
int pcgb_box_sync(pcgb_box* b);
/* out[0..PCGB_NSLOT-1] raw reduced slots, then t, dt, step of the diagnostics. */
int pcgb_box_diag(pcgb_box* b, double* out, int nout);
int pcgb_box_time(pcgb_box* b, double* t, double* dt, long long* nsub);
int pcgb_box_set_dt(pcgb_box* b, double dt);
/* Wavevector list of the random helical forcing, the content of the reference's
   k.dat (forcing.f90:888-900): kxyz = kkx[0..nk), kky[0..nk), kkz[0..nk); kav
   the average |k| given there.  Required before stepping a box with
   lforcing_hel; boxes with helical forcing step through the box API and the
   plug-in set (a batch refuses them). */
int pcgb_box_set_kvectors(pcgb_box* b, const double* kxyz, int nk, double kav);
/* Device bytes held by the box. */
size_t pcgb_box_bytes(const pcgb_box* b);
/* Device bytes a box with these parameters would hold (admission control). */
size_t pcgb_params_bytes(const pcgb_params* p);
/* Cells, fields, precision and tile of the box. */
int pcgb_box_info(const pcgb_box* b, int* info, int ninfo);

/* A batch advances many boxes of one class (precision, field count, tile)
   in one persistent launch per substep.  Each box's result is bitwise the one
   it has stepped alone when the boxes also agree in the FP32 compensated mode
   (comp): a batch mixing comp and plain FP32 boxes runs the kernel with the
   mode read at run time, which can differ from the single-box kernels in the
   last bits. */
pcgb_batch* pcgb_batch_create(pcgb_box** boxes, int n, int persistent);
void pcgb_batch_destroy(pcgb_batch* b);
/* nsteps RK3 steps for every box; use_graph != 0 captures the substep loop
   of graph_steps steps in a CUDA graph and replays it. */
int pcgb_batch_steps(pcgb_batch* b, int nsteps, int use_graph, int graph_steps);

/* Request server with continuous batching.  Requests (a parameter block,
   a step count and a seeded initial condition) are admitted in arrival order
   while their device memory fits the budget.  Each round advances the oldest
   request together with the younger requests of its class (precision, field
   count, kernel variant, state mode, tile) that fit into the kernel waves the oldest one fills
   alone, and, while less than one wave of the GPU is busy, younger requests of
   other classes: one persistent launch per substep per class, the classes on
   streams of their own, in rounds of at most round_steps RK3 steps.  Boxes that
   finish leave and waiting requests join between rounds.  While it runs, the
   server's thread drives the library's engine (its stream is the server's).
   max_active = 1 gives FIFO one-at-a-time service.  Times are seconds since the
   server was created. */
typedef struct pcgb_server pcgb_server;
pcgb_server* pcgb_server_create(size_t mem_budget_bytes, int max_active, int round_steps);
/* init: Gaussian noise of amplitude noise_ampl on aa (seeded), ABC flow of
   amplitude abc_ampl on uu when abc_ampl != 0.  f_out, if not NULL, receives
   the final f(mx,my,mz,nf) (double, Fortran order).  Returns a request id >= 0,
   or -1 for a bad request (requests with lforcing_hel or non-periodic
   boundaries are refused: those run through the box API).  A request with
   tile < 0 gets its tiling by size: FP32 on tile 7 from 152 column tiles of
   (32,8) up (tile 6 below, and with upwinding), double-float on tile 5, FP64
   on tile 1; zdepth <= 0 becomes nz/4 within [16, 64]. */
long long pcgb_server_submit(pcgb_server* s, const pcgb_params* p, int nsteps, unsigned long long seed,
                             double noise_ampl, double abc_ampl, double* f_out);
/* 1 when request id is done (times[0..2] = submitted, started, finished;
   diag[0..PCGB_NSLOT+2] = the box's last reduced slots, t, dt, step), 0 while
   pending, < 0 on error. */
int pcgb_server_poll(pcgb_server* s, long long id, double* times, double* diag);
/* Wait until every submitted request is done or timeout_s passes (0: done). */
int pcgb_server_drain(pcgb_server* s, double timeout_s);
/* stats[0..5] = submitted, completed, active now, peak active, peak device bytes, rounds. */
int pcgb_server_stats(pcgb_server* s, double* stats, int nstats);
void pcgb_server_destroy(pcgb_server* s);

/* Autotuner: times each tile variant and z-depth for a box of this shape and
   returns the best (tile, zdepth); results are cached per (precision, nf, n). */
int pcgb_autotune(const pcgb_params* p, int* tile, int* zdepth, double* ms_per_substep);

/* ---------------------------------------------------------------------------
 * 3. Allocation-free substep (no counterpart in the reference).
 *
 * For callers that cannot allocate device memory at this point: a host code
 * whose device memory belongs to another allocator (a caching pool holding the
 * free memory, an application that reserves every buffer at start-up), or a
 * time loop that must not incur the device-wide synchronisation that
 * cudaMalloc/cudaFree can imply.  The caller owns f_in, f_out and df; the call
 * allocates nothing (no cudaMalloc/cudaFree, no library allocator).
 *
 * Buffers use the library's device layout for the parameter block p:
 * element (i, j, k, field), interior i in [0,nx), at
 *   field*fs + (k+3)*ps + (j+3)*px + xoff + i,
 *   xoff = 128/precision, px = xoff + roundup(nx+8, xoff), ps = px*(ny+6),
 *   fs = ps*(nz+6)   (the same layout pcgb_box_info reports),
 * each buffer fs*nf*precision bytes, 16-byte aligned.  f_in must hold valid
 * periodic ghosts (every f_out written by this call does).  One call performs
 * substep isubstep (1..3) of the 2N-RK3 scheme with timestep dt (FP64 or FP32
 * state, without the FP32 carry): df is written on substeps 1-2 and read on
 * 2-3.  If reductions != NULL (host array of PCGB_NOALLOC_NRED doubles) the
 * call waits for the kernel and returns, on substep 1, the CFL inverse
 * timestep in [0] and the diagnostic slots (sums/maxima of u^2, B^2, ...) in
 * [1..9]; only such a call reads back the kernel's error flags (return 5).  A
 * call without reductions returns once its kernel is queued.  The parameter
 * block is checked as pcgb_box_create checks it.  Each call uploads its
 * descriptor, step state and forcing tables with cudaMemcpyAsync from host
 * memory of the call.  stream is a cudaStream_t (NULL: the default stream).
 *
 * Its scratch (descriptor, step state, forcing tables, per-tile partials) is
 * a fixed file-scope device array of about 1.5 MB that every GPU using the
 * library keeps until exit; limits: nx, ny, nz <= PCGB_NOALLOC_MAX_EXTENT and
 * at most PCGB_NOALLOC_MAX_TILES tiles (larger requests return 7).  The first
 * call on each device looks up the scratch address; make it before any stream
 * capture.  All calls share the scratch: calls that overlap on the GPU race.
 * Returns 0, or 2 (bad argument), 7 (size limit), 1 (CUDA error), 5 (device
 * error flag). */
#define PCGB_NOALLOC_MAX_EXTENT 4096
#define PCGB_NOALLOC_MAX_TILES 16384
#define PCGB_NOALLOC_NRED 10   /* doubles in the reductions array */
int pcgb_substep_noalloc(const pcgb_params* p, int isubstep, double dt, const void* f_in, void* f_out, void* df,
                         double* reductions, void* stream);

/* Iteration limit of every bounded wait on a TMA copy inside the substep
   kernel; one iteration is a suspended wait of at most 1 microsecond (0
   restores the default, 2^21 iterations: about two seconds).  When a wait runs out the
   kernel records PCGB_ERR_TIMEOUT in the box state, waits for its own copies
   still in flight, and returns; the next pcgb_box_sync/store reports the
   error and the box must be reloaded.  Used by the failure-detection tests. */
void pcgb_set_wait_limit(unsigned int iterations);
/* Test hook: when on, every plane wait of the substep kernel also waits (with
   the same bound) on a shared-memory barrier that nothing ever arrives on, so
   the bounded wait runs out and the timeout path above is taken. */
void pcgb_inject_wait_failure(int on);

/* Number of kernel launches issued by this process (all entry points). */
long long pcgb_launch_count(void);
/* Name of the compiled device architecture and library version. */
const char* pcgb_version(void);

#ifdef __cplusplus
}
#endif
#endif
