// mhd_driver.cuh -- the fused RK substep kernel (sm_103a): work distribution,
// TMA plane ring, reductions and step bookkeeping, generic over a cell policy.
//
// One launch advances every box of a batch by one 2N-RK3 substep
// (timestep.f90:77-202).  The cell policy evaluates, for one output cell,
// the compressible-MHD right-hand side of pde() (equ.f90:1386 rhs_cpu: duu_dt,
// dlnrho_dt, denergy_dt, daa_dt) with the 6th-order der/der2/bidiagonal derij
// stencils (deriv.f90:89,472,1367), applies df = alpha*df + RHS and
// f_out = f_in + dt*beta*df, and writes f_out's periodic ghost images
// (boundcond.f90:2387-2531) in the same pass.
//
// Work decomposition: a tile is TX x TY columns of one box swept over zd
// z-planes.  Every field slice of one ghosted plane (TX+8) x (TY+6) is staged
// into a ring of RING shared-memory slots by one 4-D TMA load per plane,
// tracked by one mbarrier per slot; output plane z reads planes z-3..z+3.
// Warps are not held in lock step: each warp counts itself off a ring plane
// when it no longer needs it, and the last warp to do so refills the slot
// with the plane RING ahead, so a warp only waits for data, never for the
// other warps of its CTA (there is one CTA barrier per tile, not per plane).
// Work items come from blockIdx (one tile per CTA) or, for persistent batched
// launches, from an atomic tile counter.
//
// Reductions (CFL inverse timestep and diagnostics) are accumulated in FP64,
// written per tile, and reduced in fixed tile order by the last CTA of each
// box, which also advances the box's bookkeeping (substep index, time, dt)
// in device memory, so a time loop is a sequence of identical launches.
#pragma once

#include "mhd_common.cuh"

namespace pcgb {

// Bound of the wait for copies still in flight after a failed wait: long
// enough for any TMA load to land, so a CTA never leaves with copies pending.
constexpr unsigned int kDrainWaitLimit = 1u << 22;

// Cells that keep state in tensor memory declare kTmemCols (columns the CTA
// allocates) and kColsPerThread; the others use none.
template <class C, class = void>
struct CellTmem {
  static constexpr int cols = 0, per_thread = 0;
  static constexpr bool whole_warp = false;
};
template <class C>
struct CellTmem<C, decltype((void)C::kTmemCols, void())> {
  static constexpr int cols = C::kTmemCols, per_thread = C::kColsPerThread;
  static constexpr bool whole_warp = C::kWholeWarp;
};

template <class CELL, int TX, int TY, int RING>
struct DriverCfg {
  using Elem = typename CELL::Elem;
  static constexpr int NT = TX * TY;
  static constexpr int NWARP = (NT + 31) / 32;
  static constexpr int BW = TX + 8;   // TMA box width: x0-4 .. x0+TX+4
  static constexpr int BH = TY + 6;   // TMA box rows:  y0-3 .. y0+TY+3
  static constexpr int PLANE_BYTES = CELL::NSLICE * BW * BH * (int)sizeof(Elem);
  static constexpr int SLOT_BYTES = (PLANE_BYTES + 127) / 128 * 128;
  static constexpr int BAR_OFF = RING * SLOT_BYTES;                  // RING slot barriers + one never armed
  static constexpr int CNT_OFF = BAR_OFF + (RING + 1) * 8;           // RING release counters, a spare word, issued
  static constexpr int RED_OFF = CNT_OFF + ((RING + 2) * 4 + 7) / 8 * 8;
  static constexpr int SMEM_BYTES = RED_OFF + NWARP * PCGB_NSLOT * 8 + 64;
};

// RED = false: the variant for launches in which no box reduces (substeps 2
// and 3, and substep 1 with a fixed dt and no diagnostics due): no per-thread
// FP64 accumulators, no reduction code.  The host picks it; a box that
// nevertheless finds a reduction due flags PCGB_ERR_NORED.
// KIND = 1..3: specialised at compile time for substep KIND-1 of boxes in the
// FP32 compensated mode, so that the substep's branches of the update (df read
// and written, the carry's form) fold away -- reduction-free, or with RED for
// substep 1 (the substep that reduces); the host picks it for such launches, a
// box in another substep or mode flags PCGB_ERR_VARIANT.  KIND = 0: the substep
// and mode are read at run time.
template <class CELL, int TX, int TY, int RING, int MINB, bool RED, int KIND = 0>
__global__ void __launch_bounds__(TX* TY, MINB) mhd_substep_kernel(LaunchArgs args) {
  static_assert(KIND == 0 || !RED || KIND == 1, "reductions happen on substep 1 only");
  using C = DriverCfg<CELL, TX, TY, RING>;
  using T = typename CELL::T;
  using Elem = typename CELL::Elem;
  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + C::BAR_OFF);
  unsigned int* released = reinterpret_cast<unsigned int*>(smem + C::CNT_OFF);   // [RING]
  unsigned int* issued = reinterpret_cast<unsigned int*>(smem + C::CNT_OFF + (RING + 1) * 4);
  double* red = reinterpret_cast<double*>(smem + C::RED_OFF);
  int* sh = reinterpret_cast<int*>(smem + C::RED_OFF + C::NWARP * PCGB_NSLOT * 8);

  const int tid = threadIdx.x;
  const int tx = tid % TX, ty = tid / TX;
  const int lane = tid & 31, warp = tid >> 5;

  constexpr int TMC = CellTmem<CELL>::cols;
  if constexpr (TMC > 0) {
    if (warp == 0) {
      asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&sh[2])),
                   "n"(TMC) : "memory");
      asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
  }
  if (tid == 0) {
    for (int r = 0; r <= RING; ++r) mbar_init(&full[r], 1);   // full[RING]: never arrived on
    for (int r = 0; r < RING; ++r) released[r] = 0u;
    fence_mbar_init();
  }
  if constexpr (TMC > 0) asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  uint32_t tm_thread = 0;
  if constexpr (TMC > 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    tm_thread = (uint32_t)sh[2] + ((uint32_t)(32 * (warp & 3)) << 16) +
                (uint32_t)((warp >> 2) * CellTmem<CELL>::per_thread);
  }

  unsigned int gplane = 0;   // planes loaded by this CTA in this launch (ring slot and phase tracking)
  int iter = 0;
  int failed = 0;

  while (true) {
    int w;
    if (args.work_counter) {
      if (tid == 0) sh[0] = (int)atomicAdd(args.work_counter, 1u);
      __syncthreads();
      w = sh[0];
      __syncthreads();
    } else {
      w = (iter == 0) ? (int)blockIdx.x : args.total_tiles;
    }
    ++iter;
    if (w >= args.total_tiles) break;

    // locate the box of work item w (binary search over tile0)
    int lo = 0, hi = args.nboxes - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (args.boxes[mid].tile0 <= w) lo = mid; else hi = mid - 1;
    }
    const PcgbBoxDev& B = args.boxes[lo];
    PcgbBoxState* const S = B.state;
    const int btiles = B.tiles;
    double* const bpartial = B.partial;
    const int bdt_mode = B.dt_mode;

    const int lt = w - B.tile0;
    const int ntx = B.ntx, nty = B.nty;
    const int tix = lt % ntx, tiy = (lt / ntx) % nty, tiz = lt / (ntx * nty);
    const int x0 = tix * TX, y0 = tiy * TY, z0 = tiz * B.zd;
    const int z1 = min(z0 + B.zd, B.nz);
    const int nplanes = (z1 - z0) + 6;

    const unsigned long long nsub = __ldcg(&S->nsub);
    const int s = KIND > 0 ? KIND - 1 : (int)(nsub % 3ull);
    if (KIND > 0 && ((int)(nsub % 3ull) != s || B.comp == 0) && threadIdx.x == 0) atomicOr(&S->err, PCGB_ERR_VARIANT);
    const int inb = (int)(nsub & 1ull);
    const CUtensorMap* tmap = &B.tmap[inb];
    const double dt = __ldcg(&S->dt);
    const bool mode_cfl = KIND == 0 && args.mode == MODE_CFL;   // specialised kernels run substeps only
    const unsigned long long step = nsub / 3ull + __ldcg(&S->step0);
    StepFlags<T> fl;
    fl.s = s;
    fl.want_diag = !mode_cfl && s == 0 &&
                   ((B.diag_every > 0 && (step % (unsigned long long)B.diag_every) == 0ull) ||
                    __ldcg(&S->diag_request) != 0);
    fl.want_cfl = mode_cfl || (s == 0 && B.dt_mode == PCGB_DT_LAGGED);
    fl.comp = KIND > 0 || B.comp != 0;
    fl.read_df = (s > 0) || fl.comp;
    fl.write_df = (s < 2) || fl.comp;
    fl.alpha = T(rk_alpha(s));
    fl.dtb = T(dt * rk_beta(s));
    // compensated mode: df_stored = df + e / (dt*beta_{s+1}*alpha_{s+1})
    fl.cinv = (fl.comp && s < 2) ? T(1.0 / (dt * rk_beta(s + 1) * rk_alpha(s + 1))) : T(0);
    if (!RED) {
      if ((fl.want_cfl || fl.want_diag) && threadIdx.x == 0) atomicOr(&S->err, PCGB_ERR_NORED);
      fl.want_cfl = false;
      fl.want_diag = false;
    }
    const bool need_red = RED && (fl.want_cfl || fl.want_diag);

    // plane j of this tile is ring plane gplane + j: slot (sbase + j) % RING and
    // fill phase ((sbase + j) / RING + pbase) & 1
    const unsigned int sbase = gplane % RING, pbase = gplane / RING;
    // producer: prologue (TMA box origin held in a register: stores through the
    // cell's output pointers would otherwise force a reload from the descriptor)
    // (16-byte dd2 elements travel as two 8-byte TMA elements)
    const int tma_x = (B.xoff + x0 - 4) * (sizeof(Elem) == 16 ? 2 : 1);
    if (tid == 0) {
      prefetch_tensormap(tmap);
      const int npro = nplanes < RING ? nplanes : RING;
      *issued = (unsigned int)npro;
      for (int j = 0; j < npro; ++j) {
        const unsigned int slot = (sbase + j) % RING;
        fence_proxy_async_smem();
        mbar_arrive_expect_tx(&full[slot], C::PLANE_BYTES);
        tma_load_4d(smem + slot * C::SLOT_BYTES, tmap, &full[slot], tma_x, y0, z0 + j, 0);
      }
    }

    const int x = x0 + tx, y = y0 + ty;
    const bool active = (x < B.nx) && (y < B.ny);
    typename CELL::Tile cell;
    cell.begin(B, inb, x, y, z0, active, mode_cfl, fl);
    if constexpr (TMC > 0) { cell.tm = tm_thread; cell.zfirst = z0; }
    const bool warp_live = __any_sync(0xffffffffu, active);

    typename AccOf<T>::type acc;
    acc.reset();
    T dt1max = T(0);

    // rolling ring positions: ws/wp = slot and phase of plane j+6 (the newest this
    // output needs), rs = slot of plane j (released after it), po = offsets of the
    // seven planes z-3..z+3 of this thread's column
    unsigned int ws = 0u, wp = 0u, rs = sbase;
    unsigned int po[7];
    for (int z = z0; z < z1; ++z) {
      const int j = z - z0;
      int lfail = 0;
      if (j == 0) {
        for (int jw = 0; jw <= 6; ++jw) {
          const unsigned int r = sbase + (unsigned int)jw;
          if (!mbar_wait_bounded(&full[r % RING], ((r / RING) + pbase) & 1u, args.wait_limit)) lfail = 1;
        }
        const unsigned int r6 = sbase + 6u;
        ws = r6 % RING;
        wp = ((r6 / RING) + pbase) & 1u;
      } else {
        if (++ws == (unsigned int)RING) { ws = 0u; wp ^= 1u; }
        if (!mbar_wait_bounded(&full[ws], wp, args.wait_limit)) lfail = 1;
      }
      // failure-detection test hook: a flag that nothing sets, waited for with the same bound
      if (args.inject_wait_failure && !mbar_wait_bounded(&full[RING], 0u, args.wait_limit)) lfail = 1;
      // a warp whose wait failed leaves the tile; the others stop at their next wait, which
      // then fails too (that warp no longer releases planes), and the CTA agrees below
      if (__any_sync(0xffffffffu, lfail)) {
        failed = 1;
        break;
      }

      if (CellTmem<CELL>::whole_warp && !mode_cfl ? warp_live : active) {
        if (j == 0) {
          const unsigned int cb = ((ty + 3) * C::BW + (tx + 4)) * (int)sizeof(Elem);
#pragma unroll
          for (int dd = 0; dd < 7; ++dd) po[dd] = cb + ((sbase + dd) % RING) * C::SLOT_BYTES;
        } else {
#pragma unroll
          for (int dd = 0; dd < 6; ++dd) po[dd] = po[dd + 1];
          const unsigned int n6 = po[5] + C::SLOT_BYTES;
          po[6] = n6 >= (unsigned int)(RING * C::SLOT_BYTES) ? n6 - RING * C::SLOT_BYTES : n6;
        }
        const Elem* pl[7];
#pragma unroll
        for (int dd = 0; dd < 7; ++dd) pl[dd] = reinterpret_cast<const Elem*>(smem + po[dd]);
        if constexpr (CellTmem<CELL>::whole_warp) {
          if (!mode_cfl) cell.step(pl, x, y, z, z1, fl, acc, dt1max, active);
          else cell.cfl(pl, dt1max);
        } else {
          if (!mode_cfl) cell.step(pl, x, y, z, z1, fl, acc, dt1max);
          else cell.cfl(pl, dt1max);
        }
      }

      // this warp is done with ring plane j; the last warp to say so refills its slot
      __syncwarp();
      if (lane == 0) {
        const unsigned int slot = rs;
        __threadfence_block();
        const unsigned int prev = atomicAdd(&released[slot], 1u);
        if (prev == (unsigned int)(C::NWARP - 1)) {
          __threadfence_block();
          released[slot] = 0u;
          if (j + RING < nplanes) {
            *issued = (unsigned int)(j + RING + 1);
            fence_proxy_async_smem();
            mbar_arrive_expect_tx(&full[slot], C::PLANE_BYTES);
            tma_load_4d(smem + slot * C::SLOT_BYTES, tmap, &full[slot], tma_x, y0, z0 + j + RING, 0);
          }
        }
      }
      rs = (rs + 1u == (unsigned int)RING) ? 0u : rs + 1u;
    }
    failed = __syncthreads_or(failed);
    if (failed && tid == 0) {
      // drain: wait (bounded) for the newest plane of every slot before leaving
      const int hi2 = (int)*issued;
      for (int jw = (hi2 > RING ? hi2 - RING : 0); jw < hi2; ++jw) {
        const unsigned int r = sbase + (unsigned int)jw;
        mbar_wait_bounded(&full[r % RING], ((r / RING) + pbase) & 1u, kDrainWaitLimit);
      }
    }
    gplane += (unsigned int)nplanes;
    if (failed) {
      if (tid == 0) atomicOr(&S->err, PCGB_ERR_TIMEOUT);
      break;
    }

    // ---- per-tile reduction (fixed order: lanes, then warps) ----
    if (need_red) {
#pragma unroll
      for (int q = 0; q < PCGB_NSLOT; ++q) {
        double vq = (q == PCGB_S_DT1MAX) ? (double)dt1max : acc.get(q);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) vq = red_op(q, vq, __shfl_xor_sync(0xffffffffu, vq, o));
        if (lane == 0) red[warp * PCGB_NSLOT + q] = vq;
      }
      __syncthreads();
      if (tid < PCGB_NSLOT) {
        double r = red[tid];
        for (int wq = 1; wq < C::NWARP; ++wq) r = red_op(tid, r, red[wq * PCGB_NSLOT + tid]);
        bpartial[(long long)lt * PCGB_NSLOT + tid] = r;
      }
    }

    // ---- last CTA of the box: reduce tiles in order, advance bookkeeping ----
    __threadfence();
    __syncthreads();
    if (tid == 0) {
      const unsigned int prev = atomicAdd(&S->done, 1u);
      sh[1] = (prev == (unsigned int)(btiles - 1)) ? 1 : 0;
    }
    __syncthreads();
    if (sh[1]) {
      __threadfence();
      if (need_red) {
        double part[PCGB_NSLOT];
#pragma unroll
        for (int q = 0; q < PCGB_NSLOT; ++q) part[q] = 0.0;
        for (int t = tid; t < btiles; t += C::NT) {
#pragma unroll
          for (int q = 0; q < PCGB_NSLOT; ++q)
            part[q] = red_op(q, part[q], __ldcg(&bpartial[(long long)t * PCGB_NSLOT + q]));
        }
#pragma unroll
        for (int q = 0; q < PCGB_NSLOT; ++q) {
          double vq = part[q];
#pragma unroll
          for (int o = 16; o > 0; o >>= 1) vq = red_op(q, vq, __shfl_xor_sync(0xffffffffu, vq, o));
          if (lane == 0) red[warp * PCGB_NSLOT + q] = vq;
        }
        __syncthreads();
        if (tid == 0) {
          double r[PCGB_NSLOT];
          for (int q = 0; q < PCGB_NSLOT; ++q) {
            r[q] = red[q];
            for (int wq = 1; wq < C::NWARP; ++wq) r[q] = red_op(q, r[q], red[wq * PCGB_NSLOT + q]);
          }
          if (fl.want_cfl) {
            const double dtn = 1.0 / r[PCGB_S_DT1MAX];   // set_dt, sub.f90:4247
            if (!(dtn > 0.0) || !isfinite(dtn)) atomicOr(&S->err, PCGB_ERR_DT | PCGB_ERR_NONFINITE);
            if (mode_cfl) {
              if (bdt_mode != PCGB_DT_FIXED) { S->dt = dtn; S->dt_next = dtn; }
            } else {
              S->dt_next = dtn;
            }
          }
          if (fl.want_diag) {
            for (int q = 0; q < PCGB_NSLOT; ++q) S->diag[q] = r[q];
            S->diag_step = step;
            S->diag_request = 0;
          }
        }
      }
      if (tid == 0) {
        if (!mode_cfl) {
          // ds and time bookkeeping, timestep.f90:108-148, :201
          double ds = (s == 0) ? 0.0 : rk_alpha(s) * S->ds;
          ds = ds + 1.0;
          S->ds = ds;
          S->t = S->t + ds * (dt * rk_beta(s));
          if (s == 2) S->dt_last = dt;
          if (s == 2 && bdt_mode == PCGB_DT_LAGGED) S->dt = S->dt_next;
          S->nsub = nsub + 1ull;
        }
        S->done = 0u;
        __threadfence();
      }
    }
    __syncthreads();
  }
  if constexpr (TMC > 0) {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (warp == 0)
      asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"((uint32_t)sh[2]), "n"(TMC)
                   : "memory");
  }
}

}  // namespace pcgb
