// params_check.h -- the one validity check of a pcgb_params block, shared by
// the box/plug-in runtime and the allocation-free substep entry point.
#pragma once

#include <cstdio>

#include "../../include/pcgb300.h"

namespace pcgb {

// Iteration limit of the kernel's bounded waits as pcgb_set_wait_limit set it
// (defined by the runtime of each library).
unsigned int current_wait_limit();
// CTAs in one full wave of a box's substep kernel (occupancy x SMs).
int box_wave(const pcgb_box* b);
// Make s the engine's stream and return the previous one (nothing is destroyed).
void* engine_swap_stream(void* s);

// Returns nullptr when p is valid, else a message (written into buf when it
// carries numbers).
inline const char* params_problem(const pcgb_params* p, char* buf, size_t n) {
  if (!p) return "null parameter block";
  // >= 2 x nghost cells: the substep kernel writes each cell's periodic ghost
  // image on one side of an axis (Images in mhd_common.cuh)
  if (p->nx < 6 || p->ny < 6 || p->nz < 6) {
    snprintf(buf, n, "grid %dx%dx%d: each axis needs >= 6 cells", p->nx, p->ny, p->nz);
    return buf;
  }
  if (p->precision != 4 && p->precision != 8) return "precision must be 4 or 8";
  if (p->dfloat != 0 && p->dfloat != 1) return "dfloat must be 0 or 1";
  if (p->dfloat && p->precision != 8) return "dfloat needs precision 8 (FP64-class state)";
  if (!(p->Lxyz[0] > 0 && p->Lxyz[1] > 0 && p->Lxyz[2] > 0)) return "Lxyz must be positive";
  if (!(p->cs0 > 0 && p->rho0 > 0 && p->cp > 0 && p->gamma > 0 && p->mu0 > 0))
    return "cs0, rho0, cp, gamma, mu0 must be positive";
  if (!(p->cdt > 0 && p->cdtv > 0)) return "cdt and cdtv must be positive";
  if (p->dt < 0) return "dt must be >= 0";
  if (p->lforcing_hel != 0 && p->lforcing_hel != 1) return "lforcing_hel must be 0 or 1";
  if (p->lforcing_hel && !(p->force_hel >= 0.0)) return "force_hel must be >= 0";
  if (p->lmagnetic_forcing != 0 && p->lmagnetic_forcing != 1) return "lmagnetic_forcing must be 0 or 1";
  if (p->lmagnetic_forcing && !p->lforcing_hel)
    return "lmagnetic_forcing applies to random helical forcing (lforcing_hel)";
  if ((p->lupw_uu != 0 && p->lupw_uu != 1) || (p->lupw_lnrho != 0 && p->lupw_lnrho != 1))
    return "lupw_uu and lupw_lnrho must be 0 or 1";
  const int nf = p->lentropy ? 8 : 7;
  for (int d = 0; d < 3; ++d) {
    int nper = 0;
    for (int k = 0; k < nf; ++k)
      for (int side = 0; side < 2; ++side) {
        const int c = p->bc[d][k][side];
        if (c < PCGB_BC_PER || c > PCGB_BC_ASYM2) {
          snprintf(buf, n, "boundary condition code %d (direction %d, field %d) is not one of p, s, a, a2", c, d, k);
          return buf;
        }
        nper += (c == PCGB_BC_PER);
      }
    if (nper != 0 && nper != 2 * nf) {
      snprintf(buf, n, "direction %d mixes periodic and non-periodic boundary conditions", d);
      return buf;
    }
  }
  return nullptr;
}

}  // namespace pcgb
