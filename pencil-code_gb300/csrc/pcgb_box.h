// pcgb_box.h -- per-box descriptors shared by host runtime and device kernels.
//
// A "box" is one periodic MHD domain (the reference's f-array on one GPU).
// Its device state is fully described by PcgbBoxDev (read-only during a
// launch) and PcgbBoxState (mutated on device at the end of each substep),
// so that a time loop is a sequence of identical launches that a CUDA graph
// can replay without host involvement.
#pragma once

#include <cuda.h>
#include <stdint.h>

#define PCGB_NGHOST 3
#define PCGB_NSLOT 10  // per-tile reduction slots, see PcgbSlot

// Reduction slots (FP64 on device).  Diagnostics follow the reference's
// print.in quantities: urms/umax (hydro.f90:4709,4743), brms/bmax
// (magnetic.f90:6879,6894), ekin (hydro.f90:4859), rhom (density.f90:3519),
// divB, jrms, abm (magnetic.f90:6908).
enum PcgbSlot {
  PCGB_S_DT1MAX = 0, PCGB_S_U2SUM, PCGB_S_U2MAX, PCGB_S_B2SUM, PCGB_S_B2MAX,
  PCGB_S_EKINSUM, PCGB_S_RHOSUM, PCGB_S_DIVB2SUM, PCGB_S_J2SUM, PCGB_S_ABSUM
};

// Timestep modes (how dt is chosen on substep 1).
enum PcgbDtMode {
  PCGB_DT_FIXED = 0,    // dt from run.in, never changed
  PCGB_DT_LAGGED = 1,   // CFL reduced on substep 1 of step n, used from step n+1
                        // (the reference GPU default, gpu_astaroth.f90:24-29)
  PCGB_DT_CURRENT = 2   // CFL of the current f before substep 1 (CPU semantics,
                        // lcpu_timestep_on_gpu=T): one extra read-only pass
};

struct PcgbBoxState;

struct alignas(128) PcgbBoxDev {
  CUtensorMap tmap[2];   // TMA maps over f buffer 0 / 1 (4-D: x, y, z, field)
  void* f[2];            // ghosted f buffers (T*), ping-pong
  void* df;              // df, same geometry as f (T*); holds the RK carry in comp mode
  const void* forc;      // forcing tables T: sinx[px] cosx[px] siny[my] cosy[my] sinz[mz] cosz[mz]
  double* partial;       // [tiles][PCGB_NSLOT] per-tile reductions
  PcgbBoxState* state;   // mutable per-box state (device)
  int nx, ny, nz;        // interior cells
  int px, my, mz;        // row pitch (elements), ghosted y/z extents
  int xoff;              // element offset of interior x = 0 within a row
  int nf;                // 7 or 8
  long long ps, fs;      // plane stride px*my, field stride px*my*mz
  int ntx, nty, ntz, zd; // tile counts and z-sweep depth
  int tiles;             // ntx*nty*ntz
  int tile0;             // first global work index of this box in its launch
  // physics (double; kernels convert to their arithmetic type)
  double dx_1, dy_1, dz_1, dxyz_2;
  double nu, eta, chi, mu0, mu01;
  double cs20, gamma, gamma_m1, gamma1, lnrho0, cv1, lnTT0, cpp;
  double b_ext[3];
  double fact, fact2, abc_a, abc_b, abc_c, ampl_fcont_uu;
  double cdt, cdtv;
  int lforcing, lohmic_heat, lviscosity_heat, lentropy;
  int dt_mode;           // PcgbDtMode
  int comp;              // FP32 compensated 2N accumulation
  int diag_every;        // diagnostics at steps with step % diag_every == 0 (0: never)
  int isothermal;        // gamma == 1 without entropy
  int lupw;              // upwinding of u.grad u / u.grad lnrho (UPW_* bits)
  // random helical forcing added in the last substep's update (FP32 pair layout):
  // the float copy of the step's tables (helical.h: coef1[3] coef2[3] 2 spare, fx,
  // fy, fz as (re, im) pairs), or null; the forced lane: 0 uu, 1 aa
  const float* hel_tab;
  int hel_target;
};

struct alignas(64) PcgbBoxState {
  unsigned long long nsub;   // substeps completed since load
  unsigned long long step0;  // step index at load (for diagnostics cadence)
  double t;                  // simulation time
  double dt;                 // dt used by the current step
  double dt_next;            // CFL dt reduced on the last substep 1 (lagged mode)
  double ds;                 // RK ds accumulator (timestep.f90:108-148)
  unsigned int done;         // tiles of this box finished in the current launch
  int err;                   // sticky error flags (PCGB_ERR_*)
  unsigned long long diag_step;  // step of the last diagnostics (or ~0)
  double diag[PCGB_NSLOT];   // last reduced diagnostics (sums and maxima)
  int diag_request;          // host request: diagnostics at the next substep 1
  int pad_[3];
  double dt_last;            // dt of the last completed step (the step-end helical forcing scales with it)
};

#define PCGB_ERR_NONFINITE 1   // NaN/Inf seen in dt1
#define PCGB_ERR_TIMEOUT 2     // a bounded wait gave up
#define PCGB_ERR_DT 4          // dt <= 0 or not finite
#define PCGB_ERR_NORED 8       // a CFL or diagnostic reduction was due in a launch of the reduction-free kernel
#define PCGB_ERR_VARIANT 16    // a kernel specialised for another substep or state mode was launched for the box
