// noalloc.cu -- one RK substep on caller-owned device buffers, with no device
// memory allocation of any kind.
//
// Who needs this: a host program whose device memory is owned by another
// allocator (for example a caching pool that already holds the free memory,
// or a Fortran/C++ application that reserves all its buffers at start-up and
// forbids later allocations), or a time loop that must never trigger the
// device-wide synchronisation that cudaMalloc/cudaFree may imply.  Such a
// caller allocates f_in, f_out and df itself and calls pcgb_substep_noalloc.
//
// The substep kernel needs scratch beyond its inputs and outputs: the box
// descriptor with its TMA maps, the per-box step state, the ABC forcing
// tables and the per-tile FP64 reduction partials.  Here all of it lives in
// one file-scope __device__ array of fixed size, g_noalloc_scratch, which every
// GPU that loads this library keeps until the process exits.  Host code never
// dereferences that symbol: its device address is looked up once per device
// with cudaGetSymbolAddress (while that device is current) on the first call
// made on that device, so make that first call before any stream capture.
//
// Every call reuses the same scratch and leaves the last call's contents in
// it; each call rewrites the descriptor, the state (including the tile
// counter that must start at zero) and the forcing tables before launching,
// by cudaMemcpyAsync from host memory of the call.  Calls whose kernels
// overlap on the GPU (several streams, or several host threads) race on the
// scratch and must be serialised by the caller.
//
// Device-side errors (a bounded wait that ran out, a non-finite state) are
// read back only by a call given a reductions array: such a call waits for
// its kernel and returns 5 when the kernel flagged one.  A call without
// reductions returns as soon as its kernel is queued, and the next call's
// state upload clears the flags.
#include <cuda.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <cmath>
#include <cstdio>
#include <cstring>

#include "boundcond.h"
#include "../../include/pcgb300.h"
#include "kernels.cuh"
#include "params_check.h"
#include "pcgb_box.h"

using namespace pcgb;

namespace {

constexpr int kMaxTiles = PCGB_NOALLOC_MAX_TILES;
constexpr int kMaxExtent = PCGB_NOALLOC_MAX_EXTENT;                      // nx, ny, nz <= this
constexpr size_t kDescBytes = (sizeof(PcgbBoxDev) + 255) / 256 * 256;
constexpr size_t kStateBytes = (sizeof(PcgbBoxState) + 255) / 256 * 256;
constexpr size_t kForcElems = 6 * (size_t)(kMaxExtent + 72);             // 2 px + 2 my + 2 mz, px <= extent + 72
constexpr size_t kForcBytes = (kForcElems * sizeof(double) + 255) / 256 * 256;
constexpr size_t kPartialBytes = (size_t)kMaxTiles * PCGB_NSLOT * sizeof(double);
constexpr size_t kScratchBytes = kDescBytes + kStateBytes + kForcBytes + kPartialBytes;

__device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
unsigned char* g_scratch_dev[kMaxDevices] = {nullptr};
PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;

int fail(int code, const char* msg) {
  if (getenv("PCGB_VERBOSE")) fprintf(stderr, "pcgb_substep_noalloc: %s\n", msg);
  return code;
}

}  // namespace

extern "C" int pcgb_substep_noalloc(const pcgb_params* p, int isubstep, double dt, const void* f_in, void* f_out,
                                    void* df, double* reductions, void* stream) {
  if (!p || !f_in || !f_out || !df || isubstep < 1 || isubstep > 3 || !(dt > 0.0))
    return fail(2, "invalid argument");
  if (p->nx > kMaxExtent || p->ny > kMaxExtent || p->nz > kMaxExtent)
    return fail(7, "grid extent above PCGB_NOALLOC_MAX_EXTENT");
  {
    char buf[160];
    const char* msg = params_problem(p, buf, sizeof(buf));   // the box path's checks
    if (msg) return fail(2, msg);
  }
  if (p->dfloat) return fail(2, "double-float state is not available here (use the box API)");
  if (p->lforcing_hel) return fail(2, "the step-end helical forcing is applied by the box API only");
  for (int d = 0; d < 3; ++d)
    if (!axis_periodic(*p, d)) return fail(2, "non-periodic boundaries are applied by the box API only");
  cudaStream_t s = static_cast<cudaStream_t>(stream);

  // set-up once per device, with the device current
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return fail(1, "no current device");
  if (!g_scratch_dev[dev]) {
    void* ptr = nullptr;
    if (cudaGetSymbolAddress(&ptr, g_noalloc_scratch) != cudaSuccess || !ptr)
      return fail(1, "cudaGetSymbolAddress of the scratch array failed");
    g_scratch_dev[dev] = static_cast<unsigned char*>(ptr);
  }
  if (!g_encode) {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        !fn || q != cudaDriverEntryPointSuccess)
      return fail(1, "cuTensorMapEncodeTiled unavailable");
    g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  }
  unsigned char* base = g_scratch_dev[dev];
  PcgbBoxDev* d_desc = reinterpret_cast<PcgbBoxDev*>(base);
  PcgbBoxState* d_state = reinterpret_cast<PcgbBoxState*>(base + kDescBytes);
  void* d_forc = base + kDescBytes + kStateBytes;
  double* d_partial = reinterpret_cast<double*>(base + kDescBytes + kStateBytes + kForcBytes);

  // geometry: the library's device layout (see pcgb_box_info)
  const int tb = p->precision, nf = p->lentropy ? 8 : 7;
  const int xoff = 128 / tb;
  const int px = xoff + ((p->nx + 8 + xoff - 1) / xoff) * xoff;
  const int my = p->ny + 6, mz = p->nz + 6, mx = p->nx + 6;
  const bool upw = p->lupw_uu || p->lupw_lnrho;
  const int tile = p->tile >= 0 ? p->tile : (upw ? 1 : 0);   // tile 1 has an upwinding variant in FP32 and FP64
  // the documented layout is field-major: only the field-major tile variants apply
  if (tile >= kNumScalarTiles) return fail(2, "tile variant out of range");
  const TileShape ts = tile_shape(tb, tile);
  const KernelHandle kh = get_kernel(tb, nf, tile, 0, upw);
  if (!kh.fn) return fail(2, upw ? "no upwinding kernel for this tile variant" : "no kernel for this tile variant");
  int zd = p->zdepth > 0 ? std::min(p->zdepth, p->nz) : p->nz;

  PcgbBoxDev h;
  memset(&h, 0, sizeof(h));
  h.nx = p->nx; h.ny = p->ny; h.nz = p->nz; h.px = px; h.my = my; h.mz = mz; h.xoff = xoff; h.nf = nf;
  h.ps = (long long)px * my; h.fs = h.ps * mz;
  h.ntx = (p->nx + ts.tx - 1) / ts.tx; h.nty = (p->ny + ts.ty - 1) / ts.ty;
  h.zd = zd; h.ntz = (p->nz + zd - 1) / zd;
  h.tiles = h.ntx * h.nty * h.ntz; h.tile0 = 0;
  if (h.tiles > kMaxTiles) return fail(7, "more tiles than PCGB_NOALLOC_MAX_TILES; raise zdepth or use a larger tile");
  // buffers: index 0 is the input, 1 the output (the state below selects index 0)
  h.f[0] = const_cast<void*>(f_in); h.f[1] = f_out; h.df = df; h.forc = d_forc; h.partial = d_partial;
  h.state = d_state;
  // physics, as in the box path (eos_idealgas.f90:158-268, forcing.f90:5869-5872)
  const double dx = p->Lxyz[0] / p->nx, dy = p->Lxyz[1] / p->ny, dz = p->Lxyz[2] / p->nz;
  h.dx_1 = 1.0 / dx; h.dy_1 = 1.0 / dy; h.dz_1 = 1.0 / dz;
  h.dxyz_2 = (h.dx_1 * h.dx_1 + h.dy_1 * h.dy_1) + h.dz_1 * h.dz_1;
  h.nu = p->nu; h.eta = p->eta; h.chi = p->chi; h.mu0 = p->mu0; h.mu01 = 1.0 / p->mu0;
  h.gamma = p->gamma; h.gamma_m1 = p->gamma - 1.0; h.gamma1 = 1.0 / p->gamma;
  h.lnrho0 = std::log(p->rho0); h.cs20 = p->cs0 * p->cs0;
  const double cp1 = 1.0 / p->cp;
  h.cv1 = p->gamma * cp1;
  h.lnTT0 = (h.gamma_m1 != 0.0) ? std::log(h.cs20 / (p->cp * h.gamma_m1)) : std::log(h.cs20 / p->cp);
  h.cpp = 1.0 / cp1;
  for (int i = 0; i < 3; ++i) h.b_ext[i] = p->b_ext[i];
  h.lforcing = p->lforcing_cont;
  h.fact2 = p->relhel;
  const double fact1 = 0.5 * (1.0 + p->relhel * p->relhel);
  h.fact = p->ampl_ff / std::sqrt(fact1 * ((p->abc_a * p->abc_a + p->abc_b * p->abc_b) + p->abc_c * p->abc_c));
  h.abc_a = p->abc_a; h.abc_b = p->abc_b; h.abc_c = p->abc_c; h.ampl_fcont_uu = p->ampl_fcont_uu;
  h.cdt = p->cdt; h.cdtv = p->cdtv;
  h.lohmic_heat = p->lohmic_heat; h.lviscosity_heat = p->lviscosity_heat; h.lentropy = p->lentropy;
  // dt is the caller's; a CFL reduction on substep 1 is returned, not applied
  h.dt_mode = reductions ? PCGB_DT_LAGGED : PCGB_DT_FIXED;
  h.comp = 0;   // the FP32 carry would need state across calls; plain 2N update here
  h.diag_every = reductions ? 1 : 0;
  h.isothermal = (!p->lentropy && h.gamma_m1 == 0.0) ? 1 : 0;
  h.lupw = (p->lupw_uu ? UPW_UU : 0) | (p->lupw_lnrho ? UPW_LNRHO : 0);

  cuuint64_t dims[4] = {(cuuint64_t)px, (cuuint64_t)my, (cuuint64_t)mz, (cuuint64_t)nf};
  cuuint64_t strides[3] = {(cuuint64_t)px * tb, (cuuint64_t)h.ps * tb, (cuuint64_t)h.fs * tb};
  cuuint32_t box[4] = {(cuuint32_t)(ts.tx + 8), (cuuint32_t)(ts.ty + 6), 1u, (cuuint32_t)nf};
  cuuint32_t es[4] = {1, 1, 1, 1};
  for (int q = 0; q < 2; ++q) {
    CUresult r = g_encode(&h.tmap[q], tb == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 4,
                          h.f[q], dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                          CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(2, "cuTensorMapEncodeTiled rejected the buffers (need 16-byte alignment)");
  }

  // forcing tables on the host stack-free path: computed into a static host buffer
  static double hforc[kForcElems];
  static float hforcf[kForcElems];
  const size_t nforc = 2 * (size_t)px + 2 * (size_t)my + 2 * (size_t)mz;
  {
    double* sx = hforc; double* cx = sx + px; double* sy = cx + px; double* cy = sy + my;
    double* sz = cy + my; double* cz = sz + mz;
    for (size_t i = 0; i < nforc; ++i) hforc[i] = 0.0;
    for (int i = 0; i < mx; ++i) { double x = p->xyz0[0] + ((double)(i - 3) + 0.5) * dx; sx[i] = std::sin(p->kf * x); cx[i] = std::cos(p->kf * x); }
    for (int i = 0; i < my; ++i) { double y = p->xyz0[1] + ((double)(i - 3) + 0.5) * dy; sy[i] = std::sin(p->kf * y); cy[i] = std::cos(p->kf * y); }
    for (int i = 0; i < mz; ++i) { double z = p->xyz0[2] + ((double)(i - 3) + 0.5) * dz; sz[i] = std::sin(p->kf * z); cz[i] = std::cos(p->kf * z); }
  }
  if (tb == 4) {
    for (size_t i = 0; i < nforc; ++i) hforcf[i] = (float)hforc[i];
    if (cudaMemcpyAsync(d_forc, hforcf, nforc * 4, cudaMemcpyHostToDevice, s) != cudaSuccess)
      return fail(1, "forcing table upload failed");
  } else if (cudaMemcpyAsync(d_forc, hforc, nforc * 8, cudaMemcpyHostToDevice, s) != cudaSuccess) {
    return fail(1, "forcing table upload failed");
  }

  // state: everything that must start at zero is rewritten here (done counter, flags)
  PcgbBoxState st;
  memset(&st, 0, sizeof(st));
  static const unsigned long long nsub_of[3] = {0ull, 4ull, 2ull};   // substep index with even parity
  st.nsub = nsub_of[isubstep - 1];
  st.step0 = 0;
  st.dt = dt; st.dt_next = dt;
  st.diag_step = ~0ull;
  if (cudaMemcpyAsync(d_desc, &h, sizeof(h), cudaMemcpyHostToDevice, s) != cudaSuccess ||
      cudaMemcpyAsync(d_state, &st, sizeof(st), cudaMemcpyHostToDevice, s) != cudaSuccess)
    return fail(1, "descriptor upload failed");

  LaunchArgs a;
  a.boxes = d_desc; a.nboxes = 1; a.total_tiles = h.tiles; a.work_counter = nullptr;
  a.mode = MODE_SUBSTEP; a.wait_limit = current_wait_limit(); a.inject_wait_failure = 0;
  void* args[] = {&a};
  // the dynamic shared-memory allowance is an attribute of the current device's context
  if (cudaFuncSetAttribute(kh.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, kh.smem) != cudaSuccess)
    return fail(1, "cudaFuncSetAttribute failed");
  if (cudaLaunchKernel(kh.fn, dim3(h.tiles), dim3(kh.threads), args, (size_t)kh.smem, s) != cudaSuccess)
    return fail(1, "kernel launch failed");
  if (reductions) {
    PcgbBoxState out;
    if (cudaMemcpyAsync(&out, d_state, sizeof(out), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
      return fail(1, "reduction read-back failed");
    if (out.err) return fail(5, "device reported error flags");
    // [0] CFL inverse timestep max (substep 1), [1..] diagnostic sums and maxima (substep 1)
    for (int q = 0; q < PCGB_NSLOT; ++q) reductions[q] = out.diag[q];
    reductions[PCGB_S_DT1MAX] = (isubstep == 1) ? 1.0 / out.dt_next : 0.0;
  }
  return 0;
}
