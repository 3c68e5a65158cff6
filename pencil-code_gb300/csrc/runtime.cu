// runtime.cu -- host runtime of libpcgb300.so: boxes, batches, the reference
// GPU plug-in ABI (src/gpu_astaroth_ansi.c) and the timestep driver.
//
// Device layout of one box (all buffers ghosted, Fortran field order
// uu(1:3), lnrho, [ss], aa(1:3) as in src/register.f90:138-146):
//   element (i, j, k, fld), interior i in [0,nx) ... at
//   fld*fs + (k+3)*ps + (j+3)*px + xoff + i,  ps = px*my, fs = ps*mz,
//   xoff = 128 bytes / sizeof(T) so every interior row starts 128-byte aligned,
//   px = xoff + roundup(nx + 8, xoff) so a TMA box [x0-4, x0+TX+4) stays in the row.
#include <cuda.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cstdarg>
#include <cstddef>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/pcgb300.h"
#include "aux_kernels.h"
#include "boundcond.h"
#include "cfl_pair.h"
#include "helical.h"
#include "params_check.h"
#include "kernels.cuh"
#include "pcgb_box.h"

using namespace pcgb;

// ---------------------------------------------------------------------------
// errors
enum {
  PCGB_OK = 0,
  PCGB_E_CUDA = 1,
  PCGB_E_ARG = 2,
  PCGB_E_STATE = 3,
  PCGB_E_NOMEM = 4,
  PCGB_E_DEVICE = 5,
  PCGB_E_TIMEOUT = 6,
  PCGB_E_UNSUPPORTED = 7,
};

static int g_err = 0;
static char g_errmsg[512] = "";
static std::mutex g_mu;

static int set_err(int code, const char* fmt, ...) __attribute__((format(printf, 2, 3)));
static int set_err(int code, const char* fmt, ...) {
  if (code == PCGB_OK) return 0;
  g_err = code;
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_errmsg, sizeof(g_errmsg), fmt, ap);
  va_end(ap);
  if (getenv("PCGB_VERBOSE")) fprintf(stderr, "pcgb: error %d: %s\n", code, g_errmsg);
  return code;
}

#define CK(call)                                                                              \
  do {                                                                                        \
    cudaError_t e_ = (call);                                                                  \
    if (e_ != cudaSuccess)                                                                    \
      return set_err(PCGB_E_CUDA, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_),     \
                     __FILE__, __LINE__);                                                     \
  } while (0)

// ---------------------------------------------------------------------------
// engine
struct Engine {
  bool init = false;
  int dev = 0;
  int nsm = 0;
  int max_smem = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
  long long launches = 0;
  double* stage[2] = {nullptr, nullptr};   // host-layout staging buffers (copies of one overlap kernels on the other)
  size_t stage_elems = 0;
  cudaStream_t xfer = nullptr;             // copy stream of the staged transfers
  cudaEvent_t ev_copied[2] = {nullptr, nullptr}, ev_free[2] = {nullptr, nullptr};
  int host_mode = 0;                       // 0 auto, 1 always staged, 2 direct when possible (PCGB_HOST_TRANSFER)
  unsigned int wait_limit = 1u << 21;   // suspended waits of up to 1 us each: about two seconds
  int inject_wait_failure = 0;
};
static Engine g;

static int engine_init() {
  if (g.init) return 0;
  int ndev = 0;
  CK(cudaGetDeviceCount(&ndev));
  if (ndev < 1) return set_err(PCGB_E_CUDA, "no CUDA device");
  CK(cudaGetDevice(&g.dev));
  cudaDeviceProp prop;
  CK(cudaGetDeviceProperties(&prop, g.dev));
  if (prop.major != 10 || prop.minor != 3)
    return set_err(PCGB_E_UNSUPPORTED, "device %s is sm_%d%d; this library is built for sm_103a", prop.name,
                   prop.major, prop.minor);
  g.nsm = prop.multiProcessorCount;
  g.max_smem = (int)prop.sharedMemPerBlockOptin;
  if (!g.stream) {
    CK(cudaStreamCreateWithFlags(&g.stream, cudaStreamNonBlocking));
    g.own_stream = true;
  }
  void* fn = nullptr;
  cudaDriverEntryPointQueryResult q;
  CK(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q));
  if (!fn || q != cudaDriverEntryPointSuccess) return set_err(PCGB_E_CUDA, "cuTensorMapEncodeTiled unavailable");
  g.encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  g.stage_elems = (size_t)16 << 20;  // 2 x 128 MiB of doubles
  for (int i = 0; i < 2; ++i) {
    CK(cudaMalloc(&g.stage[i], g.stage_elems * sizeof(double)));
    CK(cudaEventCreateWithFlags(&g.ev_copied[i], cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&g.ev_free[i], cudaEventDisableTiming));
  }
  CK(cudaStreamCreateWithFlags(&g.xfer, cudaStreamNonBlocking));
  if (const char* e = getenv("PCGB_HOST_TRANSFER")) {
    if (!strcmp(e, "staged")) g.host_mode = 1;
    else if (!strcmp(e, "direct")) g.host_mode = 2;
  }
  g.init = true;
  return 0;
}

// ---------------------------------------------------------------------------
// box
struct pcgb_box {
  pcgb_params p;
  int nf = 7, tb = 8, tile = 0, zd = 0, tx = 32, ty = 4;
  int pairs = 0;   // packed field-pair layout (FP32 tiles 4..7)
  int dfl = 0;     // FP64-class state as double-float pairs (precision 8, dfloat = 1)
  int eb = 8;      // bytes per device element (T, or float2 with pairs)
  int ns = 7;      // slices per plane (nf, or 4 pairs)
  int nx = 0, ny = 0, nz = 0, mx = 0, my = 0, mz = 0, px = 0, xoff = 0;
  long long ps = 0, fs = 0;
  size_t fbytes = 0;    // bytes of one f buffer
  void* f[2] = {nullptr, nullptr};
  void* df = nullptr;
  void* forc = nullptr;
  double* partial = nullptr;
  PcgbBoxState* dstate = nullptr;
  PcgbBoxDev hdev;
  PcgbBoxDev* ddev = nullptr;
  int tiles = 0;
  unsigned long long nsub = 0;  // host mirror of the device substep counter
  bool dt_known = false;
  bool nonper = false;   // some direction has non-periodic boundary conditions
  bool diag_pending = false;    // a diagnostics request not yet served by a substep-1 launch
  KernelHandle kh;
  // random helical forcing: wavevector list (kkx, kky, kkz), its mean |k|, the
  // ran0 stream, the device record ring and factor tables
  std::vector<double> kvec;
  double kav = 0.0;
  int rng = 0;
  HelRec* dring = nullptr;
  double* dtab = nullptr;
  // the CFL pass of the FP32 pair layout (cfl_pair.cu): per-block maxima and its counter
  double* cfl_partial = nullptr;
  unsigned int* cfl_done = nullptr;
};

// Element code of the layout kernels: float, double or double-float.
static int elem_code(const pcgb_box* b) { return b->dfl ? (b->pairs ? kElemDDPair : kElemDD) : b->tb; }

// Element layout code of the helical forcing and boundary kernels (HelLayout).
static int hel_layout(const pcgb_box* b) {
  if (b->tb == 4) return b->pairs ? HEL_F32_PAIR : HEL_F32;
  if (b->dfl) return b->pairs ? HEL_DD_PAIR : HEL_DD;
  return HEL_F64;
}

// Ghost zones of the non-periodic directions of the current f (boundconds_x/y/z
// at the start of pde, equ.f90; update_ghosts before a snapshot).
static int box_boundconds(pcgb_box* b) {
  // the FP32 carry lives in df between steps (substep counter at a step boundary)
  void* carry = (b->hdev.comp && (b->nsub % 3) == 0) ? b->df : nullptr;
  CK(launch_boundconds(hel_layout(b), b->f[b->nsub & 1ull], carry, b->p, b->nx, b->ny, b->nz, b->px, b->my, b->mz,
                       b->xoff, b->ps, b->fs, b->nf, g.stream));
  g.launches += !axis_periodic(b->p, 0) + !axis_periodic(b->p, 1) + !axis_periodic(b->p, 2);
  return 0;
}

static void fill_physics(pcgb_box* b) {
  const pcgb_params& p = b->p;
  PcgbBoxDev& d = b->hdev;
  const double dx = axis_spacing(p, 0), dy = axis_spacing(p, 1), dz = axis_spacing(p, 2);
  d.dx_1 = 1.0 / dx; d.dy_1 = 1.0 / dy; d.dz_1 = 1.0 / dz;
  d.dxyz_2 = (d.dx_1 * d.dx_1 + d.dy_1 * d.dy_1) + d.dz_1 * d.dz_1;   // grid.f90:3051
  d.nu = p.nu; d.eta = p.eta; d.chi = p.chi; d.mu0 = p.mu0; d.mu01 = 1.0 / p.mu0;
  // units_eos, eos_idealgas.f90:158-268
  d.gamma = p.gamma; d.gamma_m1 = p.gamma - 1.0; d.gamma1 = 1.0 / p.gamma;
  d.lnrho0 = std::log(p.rho0); d.cs20 = p.cs0 * p.cs0;
  const double cp1 = 1.0 / p.cp;
  d.cv1 = p.gamma * cp1;
  d.lnTT0 = (d.gamma_m1 != 0.0) ? std::log(d.cs20 / (p.cp * d.gamma_m1)) : std::log(d.cs20 / p.cp);
  d.cpp = 1.0 / cp1;
  for (int i = 0; i < 3; ++i) d.b_ext[i] = p.b_ext[i];
  d.lforcing = p.lforcing_cont;
  // forcing_cont 'ABC', forcing.f90:5869-5872
  d.fact2 = p.relhel;
  const double fact1 = 0.5 * (1.0 + p.relhel * p.relhel);
  d.fact = p.ampl_ff / std::sqrt(fact1 * ((p.abc_a * p.abc_a + p.abc_b * p.abc_b) + p.abc_c * p.abc_c));
  d.abc_a = p.abc_a; d.abc_b = p.abc_b; d.abc_c = p.abc_c; d.ampl_fcont_uu = p.ampl_fcont_uu;
  d.cdt = p.cdt; d.cdtv = p.cdtv;
  d.lohmic_heat = p.lohmic_heat; d.lviscosity_heat = p.lviscosity_heat; d.lentropy = p.lentropy;
  d.dt_mode = (p.dt > 0.0) ? PCGB_DT_FIXED : (p.dt_mode == PCGB_DT_CURRENT ? PCGB_DT_CURRENT : PCGB_DT_LAGGED);
  d.comp = (b->tb == 4 && p.comp) ? 1 : 0;
  d.diag_every = p.diag_every;
  d.isothermal = (!p.lentropy && d.gamma_m1 == 0.0) ? 1 : 0;
  d.lupw = (p.lupw_uu ? UPW_UU : 0) | (p.lupw_lnrho ? UPW_LNRHO : 0);
  // FP32 pairs with the upwinding kernel variant: the helical force is added in the
  // last substep's update (otherwise by the apply kernel after the step)
  d.hel_tab = (p.lforcing_hel && b->tb == 4 && b->pairs && d.lupw)
                  ? reinterpret_cast<const float*>(b->dtab + hel_tab_doubles(b->nx, b->ny, b->nz))
                  : nullptr;
  d.hel_target = p.lmagnetic_forcing ? 1 : 0;
}

// ABC forcing tables sin/cos(kf*x) over the ghosted grid, forcing.f90:1100-1104,
// grid x_i = x0 + (i - 3 + o) dx, o = 1/2 on a periodic axis, 0 otherwise (grid.f90:123-151).
static int upload_forcing(pcgb_box* b) {
  const pcgb_params& p = b->p;
  const size_t n = 2 * (size_t)b->px + 2 * (size_t)b->my + 2 * (size_t)b->mz;
  std::vector<double> h(n, 0.0);
  const double dx = axis_spacing(p, 0), dy = axis_spacing(p, 1), dz = axis_spacing(p, 2);
  const double ox = axis_offset(p, 0), oy = axis_offset(p, 1), oz = axis_offset(p, 2);
  double* sx = h.data(); double* cx = sx + b->px; double* sy = cx + b->px; double* cy = sy + b->my;
  double* sz = cy + b->my; double* cz = sz + b->mz;
  for (int i = 0; i < b->mx; ++i) { double x = p.xyz0[0] + ((double)(i - 3) + ox) * dx; sx[i] = std::sin(p.kf * x); cx[i] = std::cos(p.kf * x); }
  for (int i = 0; i < b->my; ++i) { double y = p.xyz0[1] + ((double)(i - 3) + oy) * dy; sy[i] = std::sin(p.kf * y); cy[i] = std::cos(p.kf * y); }
  for (int i = 0; i < b->mz; ++i) { double z = p.xyz0[2] + ((double)(i - 3) + oz) * dz; sz[i] = std::sin(p.kf * z); cz[i] = std::cos(p.kf * z); }
  if (b->dfl) {   // double-float pairs: hi = nearest float, lo = nearest float to the rest
    std::vector<float> hf(2 * n);
    for (size_t i = 0; i < n; ++i) {
      hf[2 * i] = (float)h[i];
      hf[2 * i + 1] = (float)(h[i] - (double)hf[2 * i]);
    }
    CK(cudaMemcpyAsync(b->forc, hf.data(), n * 8, cudaMemcpyHostToDevice, g.stream));
  } else if (b->tb == 8) {
    CK(cudaMemcpyAsync(b->forc, h.data(), n * 8, cudaMemcpyHostToDevice, g.stream));
  } else {
    std::vector<float> hf(n);
    for (size_t i = 0; i < n; ++i) hf[i] = (float)h[i];
    CK(cudaMemcpyAsync(b->forc, hf.data(), n * 4, cudaMemcpyHostToDevice, g.stream));
  }
  CK(cudaStreamSynchronize(g.stream));
  return 0;
}

static int encode_maps(pcgb_box* b) {
  for (int q = 0; q < 2; ++q) {
    // a 16-byte double-float pair travels as two 8-byte TMA elements
    const int sub = b->eb == 16 ? 2 : 1;
    cuuint64_t dims[4] = {(cuuint64_t)b->px * sub, (cuuint64_t)b->my, (cuuint64_t)b->mz, (cuuint64_t)b->ns};
    cuuint64_t strides[3] = {(cuuint64_t)b->px * b->eb, (cuuint64_t)b->ps * b->eb, (cuuint64_t)b->fs * b->eb};
    cuuint32_t box[4] = {(cuuint32_t)((b->tx + 8) * sub), (cuuint32_t)(b->ty + 6), 1u, (cuuint32_t)b->ns};
    cuuint32_t es[4] = {1, 1, 1, 1};
    // TMA moves bytes: a float2 pair travels as one 8-byte element
    CUresult r = g.encode(&b->hdev.tmap[q], b->eb == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64,
                          4, b->f[q], dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                          CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return set_err(PCGB_E_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
  }
  return 0;
}

static int default_zdepth(const pcgb_box* b) {
  const int ntx = (b->nx + b->tx - 1) / b->tx, nty = (b->ny + b->ty - 1) / b->ty;
  const long long cols = (long long)ntx * nty;
  const long long wave = pcgb::box_wave(b);
  if (cols >= wave) {
    // at least a wave of column tiles: among the splits of z into k sweeps (z-depth
    // 16 or more) that give four waves of tiles or more, the one of least cost =
    // waves x (planes of a tile + 10 for the ring prologue and the tile's
    // bookkeeping); it evens out the last wave (1024^3 on tile 7: z-depth 512,
    // +1.2 % over whole columns; 384^3: 128, +8.8 % over 192; 320^3: 64, +4.8 % over 80)
    int best = 0;
    long long best_cost = -1;
    for (int k = 1; k <= 64; ++k) {
      const int zd = (b->nz + k - 1) / k;
      if (k > 1 && zd < 16) break;
      const long long tiles = cols * ((b->nz + zd - 1) / zd);
      if (tiles < 4 * wave) continue;
      const long long cost = ((tiles + wave - 1) / wave) * (zd + 10);
      if (best_cost < 0 || cost < best_cost) { best_cost = cost; best = zd; }
    }
    if (best > 0) return best;
  }
  int zd = b->nz;
  // split z until there are enough tiles for ~4 waves of one CTA per SM
  while (zd > 16 && cols * ((b->nz + zd - 1) / zd) < 4LL * g.nsm) zd = (zd + 1) / 2;
  return zd;
}

// FP32: packed pairs on (32,12) tiles, one 12-warp CTA per SM (on (32,8)
// tiles, 8 warps, with upwinding), when a box has at least a wave
// of (32,8) column tiles, else on (16,8) tiles with two CTAs per SM (more,
// smaller work items for small boxes); double-float: packed
// pairs on (16,12) tiles, one 6-warp CTA per SM; FP64: one 6-warp CTA per SM,
// (32,6) with 7 fields, (24,8) with 8 (an 8-field ring of (32,6) planes needs
// 246 KB of shared memory)
static int default_tile(int tb, int nf, int dfl, int nx, int ny, int nz, bool upw) {
  if (tb == 4) {
    if ((long long)((nx + 31) / 32) * ((ny + 7) / 8) < 152) return 6;
    const long long px = 16 + (nx + 8 + 15) / 16 * 16, ps = px * (ny + 6);   // the FP32 pair layout
    if (!offsets32_fit(ps * (nz + 6), ps)) return 6;
    return upw ? 5 : 7;
  }
  return dfl ? 5 : (nf == 8 ? 2 : 3);
}

static int set_tiling(pcgb_box* b, int tile, int zd) {
  if (tile < 0) tile = default_tile(b->tb, b->nf, b->dfl, b->nx, b->ny, b->nz, b->hdev.lupw != 0);
  if (tile >= num_tiles(b->tb, b->dfl)) return set_err(PCGB_E_ARG, "tile variant %d out of range", tile);
  if ((int)tile_is_pair(b->tb, tile, b->dfl) != b->pairs)
    return set_err(PCGB_E_ARG, "tile %d needs a different device layout than this box was created with", tile);
  TileShape ts = tile_shape(b->tb, tile, b->dfl);
  const bool upw = b->hdev.lupw != 0;
  KernelHandle kh = get_kernel(b->tb, b->nf, tile, b->dfl, upw);
  if (!kh.fn && upw) return set_err(PCGB_E_UNSUPPORTED, "tile %d has no upwinding variant", tile);
  if (tile_uses_offsets32(b->tb, tile) && !offsets32_fit(b->fs, b->ps))
    return set_err(PCGB_E_UNSUPPORTED, "tile %d addresses a box with 32-bit offsets; one this large needs tile 4 or 6",
                   tile);
  if (!kh.fn) return set_err(PCGB_E_ARG, "no kernel for tile %d", tile);
  if (kh.smem > g.max_smem) return set_err(PCGB_E_UNSUPPORTED, "tile %d needs %d B shared memory", tile, kh.smem);
  b->tile = tile; b->tx = ts.tx; b->ty = ts.ty; b->kh = kh;
  b->zd = (zd > 0) ? std::min(zd, b->nz) : default_zdepth(b);
  PcgbBoxDev& d = b->hdev;
  d.ntx = (b->nx + b->tx - 1) / b->tx;
  d.nty = (b->ny + b->ty - 1) / b->ty;
  d.zd = b->zd;
  d.ntz = (b->nz + b->zd - 1) / b->zd;
  d.tiles = d.ntx * d.nty * d.ntz;
  d.tile0 = 0;
  if (b->partial && d.tiles > b->tiles) { cudaFree(b->partial); b->partial = nullptr; }
  if (!b->partial) CK(cudaMalloc(&b->partial, (size_t)d.tiles * PCGB_NSLOT * sizeof(double)));
  b->tiles = d.tiles;
  d.partial = b->partial;
  int rc = encode_maps(b);
  if (rc) return rc;
  CK(cudaMemcpyAsync(b->ddev, &b->hdev, sizeof(PcgbBoxDev), cudaMemcpyHostToDevice, g.stream));
  CK(cudaStreamSynchronize(g.stream));
  return 0;
}

static void box_free(pcgb_box* b) {
  if (!b) return;
  cudaFree(b->f[0]); cudaFree(b->f[1]); cudaFree(b->df); cudaFree(b->forc); cudaFree(b->partial);
  cudaFree(b->dstate); cudaFree(b->ddev); cudaFree(b->dring); cudaFree(b->dtab);
  cudaFree(b->cfl_partial); cudaFree(b->cfl_done);
  delete b;
}

static int validate(const pcgb_params* p) {
  char buf[160];
  const char* msg = params_problem(p, buf, sizeof(buf));
  return msg ? set_err(PCGB_E_ARG, "%s", msg) : 0;
}

// The wait limit the box path uses, for the allocation-free entry point.
unsigned int pcgb::current_wait_limit() { return g.wait_limit; }

// For the request server: CTAs of one full wave of a box's substep kernel, and
// a stream switch that never destroys the stream it replaces.
int pcgb::box_wave(const pcgb_box* b) {
  int occ = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, b->kh.fn, b->kh.threads, (size_t)b->kh.smem) != cudaSuccess)
    occ = 1;
  return std::max(occ, 1) * std::max(g.nsm, 1);
}
void* pcgb::engine_swap_stream(void* s) {
  if (!g.init) engine_init();
  void* old = (void*)g.stream;
  g.stream = (cudaStream_t)s;
  return old;
}

extern "C" pcgb_box* pcgb_box_create(const pcgb_params* p) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (engine_init() || validate(p)) return nullptr;
  pcgb_box* b = new pcgb_box();
  b->p = *p;
  b->nf = p->lentropy ? 8 : 7;
  b->tb = p->precision;
  b->dfl = (p->precision == 8 && p->dfloat) ? 1 : 0;
  b->nx = p->nx; b->ny = p->ny; b->nz = p->nz;
  b->mx = p->nx + 6; b->my = p->ny + 6; b->mz = p->nz + 6;
  {
    const int t0 = p->tile >= 0 ? p->tile : default_tile(b->tb, b->nf, b->dfl, p->nx, p->ny, p->nz, p->lupw_uu || p->lupw_lnrho);
    b->pairs = (t0 < num_tiles(b->tb, b->dfl) && tile_is_pair(b->tb, t0, b->dfl)) ? 1 : 0;
  }
  b->eb = b->pairs ? (b->dfl ? 16 : 8) : b->tb;
  b->ns = b->pairs ? 4 : b->nf;
  b->xoff = 128 / b->eb;
  b->px = b->xoff + ((b->nx + 8 + b->xoff - 1) / b->xoff) * b->xoff;
  b->ps = (long long)b->px * b->my;
  b->fs = b->ps * b->mz;
  b->fbytes = (size_t)b->fs * b->ns * b->eb;
  memset(&b->hdev, 0, sizeof(b->hdev));
  auto fail = [&](const char* what) {
    set_err(PCGB_E_NOMEM, "device allocation of %s failed (%zu bytes per f buffer)", what, b->fbytes);
    box_free(b);
    return (pcgb_box*)nullptr;
  };
  if (cudaMalloc(&b->f[0], b->fbytes) != cudaSuccess) return fail("f0");
  if (cudaMalloc(&b->f[1], b->fbytes) != cudaSuccess) return fail("f1");
  if (cudaMalloc(&b->df, b->fbytes) != cudaSuccess) return fail("df");
  const size_t nforc = 2 * (size_t)b->px + 2 * (size_t)b->my + 2 * (size_t)b->mz;
  if (cudaMalloc(&b->forc, nforc * b->tb) != cudaSuccess) return fail("forcing tables");
  if (cudaMalloc(&b->dstate, sizeof(PcgbBoxState)) != cudaSuccess) return fail("state");
  if (cudaMalloc(&b->ddev, sizeof(PcgbBoxDev)) != cudaSuccess) return fail("descriptor");
  if (cudaMalloc(&b->dring, sizeof(HelRec) * kHelRing) != cudaSuccess ||
      cudaMalloc(&b->dtab, hel_tab_bytes(b->nx, b->ny, b->nz)) != cudaSuccess)
    return fail("helical forcing tables");
  if (b->tb == 4 && b->pairs) {
    if (cudaMalloc(&b->cfl_partial, sizeof(double) * cfl_pair_blocks(b->nx, b->ny, b->nz)) != cudaSuccess ||
        cudaMalloc(&b->cfl_done, sizeof(unsigned int)) != cudaSuccess)
      return fail("CFL pass");
    cudaMemsetAsync(b->cfl_done, 0, sizeof(unsigned int), g.stream);
  }
  b->rng = p->seed_ff;
  cudaMemsetAsync(b->f[0], 0, b->fbytes, g.stream);
  cudaMemsetAsync(b->f[1], 0, b->fbytes, g.stream);
  cudaMemsetAsync(b->df, 0, b->fbytes, g.stream);
  PcgbBoxState st;
  memset(&st, 0, sizeof(st));
  st.dt = p->dt; st.dt_next = p->dt; st.diag_step = ~0ull;
  cudaMemcpyAsync(b->dstate, &st, sizeof(st), cudaMemcpyHostToDevice, g.stream);
  b->dt_known = p->dt > 0;
  PcgbBoxDev& d = b->hdev;
  d.f[0] = b->f[0]; d.f[1] = b->f[1]; d.df = b->df; d.forc = b->forc; d.state = b->dstate;
  d.nx = b->nx; d.ny = b->ny; d.nz = b->nz; d.px = b->px; d.my = b->my; d.mz = b->mz; d.xoff = b->xoff;
  d.nf = b->nf; d.ps = b->ps; d.fs = b->fs;
  b->nonper = !(axis_periodic(*p, 0) && axis_periodic(*p, 1) && axis_periodic(*p, 2));
  fill_physics(b);
  if (upload_forcing(b) || set_tiling(b, p->tile, p->zdepth)) { box_free(b); return nullptr; }
  return b;
}

extern "C" void pcgb_box_destroy(pcgb_box* b) {
  if (!b) return;
  cudaStreamSynchronize(g.stream);
  box_free(b);
}

// Device bytes a box with these parameters will hold (same layout as pcgb_box_create).
extern "C" size_t pcgb_params_bytes(const pcgb_params* p) {
  if (!p || p->nx < 1 || p->ny < 1 || p->nz < 1 || (p->precision != 4 && p->precision != 8)) return 0;
  const int tb = p->precision, nf = p->lentropy ? 8 : 7;
  const int dfl = (tb == 8 && p->dfloat) ? 1 : 0;
  const int t0 = p->tile >= 0 ? p->tile : default_tile(tb, nf, dfl, p->nx, p->ny, p->nz, p->lupw_uu || p->lupw_lnrho);
  const int pairs = (t0 < num_tiles(tb, dfl) && tile_is_pair(tb, t0, dfl)) ? 1 : 0;
  const int eb = pairs ? (dfl ? 16 : 8) : tb, ns = pairs ? 4 : nf;
  const int xoff = 128 / eb;
  const long long px = xoff + ((p->nx + 8 + xoff - 1) / xoff) * xoff;
  const long long fs = px * (p->ny + 6) * (p->nz + 6);
  const size_t fbytes = (size_t)fs * ns * eb;
  const long long ntiles = (long long)((p->nx + 15) / 16) * ((p->ny + 1) / 2) * 64;   // upper bound on tiles
  return 3 * fbytes + (size_t)ntiles * PCGB_NSLOT * 8 / 64 + 4096 +
         (2 * (size_t)px + 2 * (size_t)(p->ny + 6) + 2 * (size_t)(p->nz + 6)) * tb;
}

extern "C" size_t pcgb_box_bytes(const pcgb_box* b) {
  if (!b) return 0;
  return 3 * b->fbytes + (size_t)b->tiles * PCGB_NSLOT * 8 + sizeof(PcgbBoxState) + sizeof(PcgbBoxDev) +
         (2 * (size_t)b->px + 2 * (size_t)b->my + 2 * (size_t)b->mz) * b->tb;
}

extern "C" int pcgb_box_info(const pcgb_box* b, int* info, int ninfo) {
  if (!b || !info) return set_err(PCGB_E_ARG, "null argument");
  int v[12] = {b->nx, b->ny, b->nz, b->nf, b->tb, b->tile, b->zd, b->tiles, b->px, b->xoff, b->pairs, b->dfl};
  for (int i = 0; i < ninfo && i < 12; ++i) info[i] = v[i];
  return 0;
}

static int cur_in(const pcgb_box* b) { return (int)(b->nsub & 1ull); }

// Launch one substep (or CFL pass) over boxes[0..n) of one class; s (0..2, or -1 when
// the boxes differ) and comp (every box compensated FP32) select a specialised kernel.
static int launch(const PcgbBoxDev* dboxes, int nboxes, int total_tiles, unsigned int* counter, int mode,
                  const KernelHandle& kh, int grid, bool red, int s = -1, bool comp = false) {
  LaunchArgs a;
  a.boxes = dboxes;
  a.nboxes = nboxes;
  a.total_tiles = total_tiles;
  a.work_counter = counter;
  a.mode = mode;
  a.wait_limit = g.wait_limit;
  a.inject_wait_failure = g.inject_wait_failure;
  if (counter) CK(cudaMemsetAsync(counter, 0, sizeof(unsigned int), g.stream));
  void* args[] = {&a};
  CK(cudaLaunchKernel(kh.pick(red || mode == MODE_CFL, s, comp, mode == MODE_SUBSTEP), dim3(grid), dim3(kh.threads), args,
                      (size_t)kh.smem,
                      g.stream));
  ++g.launches;
  return 0;
}

// Whether a launch of this box may reduce (CFL dt or diagnostics): the CFL
// pass, or substep 1 with the lagged CFL dt, periodic diagnostics or a pending
// request.  Every other launch runs the reduction-free kernel variant.
static bool box_needs_red(const pcgb_box* b, int mode) {
  if (mode == MODE_CFL) return true;
  if (b->nsub % 3 != 0) return false;
  return b->hdev.dt_mode == PCGB_DT_LAGGED || b->hdev.diag_every > 0 || b->diag_pending;
}

static int box_launch(pcgb_box* b, int mode) {
  if (b->nonper) {   // ghosts of the non-periodic directions before every pass that reads f
    const int rc = box_boundconds(b);
    if (rc) return rc;
  }
  if (mode == MODE_CFL && b->cfl_partial) {   // FP32 pairs: the light CFL pass
    CK(launch_cfl_pair(b->ddev, b->nf, b->nx, b->ny, b->nz, b->cfl_partial, b->cfl_done, g.stream));
    ++g.launches;
    return 0;
  }
  const int rc = launch(b->ddev, 1, b->tiles, nullptr, mode, b->kh, b->tiles, box_needs_red(b, mode),
                        (int)(b->nsub % 3), b->hdev.comp != 0);
  if (mode == MODE_SUBSTEP && b->nsub % 3 == 0) b->diag_pending = false;
  return rc;
}

// First timestep when the CFL condition decides it (GpuCalcDt, gpu_astaroth.cc:546).
static int box_ensure_dt(pcgb_box* b) {
  if (b->dt_known) return 0;
  int rc = box_launch(b, MODE_CFL);
  if (rc) return rc;
  b->dt_known = true;
  return 0;
}

static int box_check_state(pcgb_box* b) {
  PcgbBoxState st;
  CK(cudaMemcpyAsync(&st, b->dstate, sizeof(st), cudaMemcpyDeviceToHost, g.stream));
  CK(cudaStreamSynchronize(g.stream));
  if (st.err & PCGB_ERR_TIMEOUT) return set_err(PCGB_E_TIMEOUT, "a bounded device wait gave up (flags %d)", st.err);
  if (st.err & PCGB_ERR_VARIANT)
    return set_err(PCGB_E_DEVICE, "a kernel variant for another substep or state mode ran on the box (flags %d)", st.err);
  if (st.err) return set_err(PCGB_E_DEVICE, "device reported error flags %d (non-finite dt or state)", st.err);
  return 0;
}

// After new data is in the input buffer: refresh ghosts, zero df (and the
// FP32 carry), restart the step bookkeeping at substep 1 with time t.
static int box_reset(pcgb_box* b, double t) {
  const int in = cur_in(b);
  CK(launch_ghost_fill(b->eb, b->f[in], b->nx, b->ny, b->nz, b->px, b->my, b->mz, b->xoff, b->ns, g.stream));
  ++g.launches;
  CK(cudaMemsetAsync(b->df, 0, b->fbytes, g.stream));
  PcgbBoxState st;
  CK(cudaMemcpyAsync(&st, b->dstate, sizeof(st), cudaMemcpyDeviceToHost, g.stream));
  CK(cudaStreamSynchronize(g.stream));
  st.t = t; st.ds = 0.0; st.done = 0; st.err = 0; st.diag_request = 0;
  // nsub % 3 == 0 and nsub parity == in; step numbering restarts at 0
  unsigned long long base = b->nsub - (b->nsub % 3);
  if ((base & 1ull) != (unsigned long long)in) base += 3;
  st.step0 = (unsigned long long)(-(long long)(base / 3));
  st.nsub = base;
  b->nsub = base;
  if (b->p.dt > 0) { st.dt = b->p.dt; st.dt_next = b->p.dt; }
  CK(cudaMemcpyAsync(b->dstate, &st, sizeof(st), cudaMemcpyHostToDevice, g.stream));
  b->dt_known = b->p.dt > 0;
  CK(cudaStreamSynchronize(g.stream));
  return 0;
}

// Device-visible alias of a host f-array, or nullptr when it has to be staged.
// Page-locked host memory (cudaHostAlloc / cudaHostRegister) is mapped into the
// device address space: the layout kernels then read or write it directly
// over the host link, with no staging copy.  Pageable memory is staged.
static const void* host_alias(const void* h) {
  if (g.host_mode == 1) return nullptr;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, h) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (a.type == cudaMemoryTypeHost && a.devicePointer) return a.devicePointer;
  return nullptr;
}

// Host f-array of REAL type (hb = 8: double, 4: float) into the box.
static int box_load_host(pcgb_box* b, const void* fh, int hb, double t) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!b || !fh) return set_err(PCGB_E_ARG, "null argument");
  const long long rows = (long long)b->my * b->mz * b->nf;
  const int in = cur_in(b);
  if (const void* dh = host_alias(fh)) {
    CK(launch_load_rows(elem_code(b), hb, b->f[in], dh, 0, rows, b->mx, b->my, b->mz, b->px, b->xoff, b->nf, b->pairs,
                        g.stream));
    ++g.launches;
    return box_reset(b, t);
  }
  // staged: copy chunk c into buffer c&1 on the copy stream while the layout
  // kernel of chunk c-1 runs on the compute stream
  const long long chunk = (long long)(g.stage_elems / b->mx);
  CK(cudaEventRecord(g.ev_free[0], g.stream));
  CK(cudaEventRecord(g.ev_free[1], g.stream));
  int c = 0;
  for (long long r0 = 0; r0 < rows; r0 += chunk, ++c) {
    const int k = c & 1;
    const long long nr = std::min(chunk, rows - r0);
    CK(cudaStreamWaitEvent(g.xfer, g.ev_free[k], 0));
    CK(cudaMemcpyAsync(g.stage[k], static_cast<const char*>(fh) + (size_t)(r0 * b->mx) * hb, (size_t)(nr * b->mx) * hb,
                       cudaMemcpyHostToDevice, g.xfer));
    CK(cudaEventRecord(g.ev_copied[k], g.xfer));
    CK(cudaStreamWaitEvent(g.stream, g.ev_copied[k], 0));
    CK(launch_load_rows(elem_code(b), hb, b->f[in], g.stage[k], r0, nr, b->mx, b->my, b->mz, b->px, b->xoff, b->nf,
                        b->pairs, g.stream));
    CK(cudaEventRecord(g.ev_free[k], g.stream));
    ++g.launches;
  }
  return box_reset(b, t);
}

extern "C" int pcgb_box_load(pcgb_box* b, const double* fh, double t) { return box_load_host(b, fh, 8, t); }
extern "C" int pcgb_box_load_f32(pcgb_box* b, const float* fh, double t) { return box_load_host(b, fh, 4, t); }

// Seeded initial condition on the device (kind 0 zero, 1 Gaussian noise of
// amplitude ampl, 2 ABC flow component `field` 0..2 with a,b,c,k), then the
// same reset as after a load.  Fields are indexed in f-array order.
extern "C" int pcgb_box_init_field(pcgb_box* b, int field, int kind, double ampl, double a, double bb, double c,
                                   double k, unsigned long long seed) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!b || field < 0 || field >= b->nf || kind < 0 || kind > 2) return set_err(PCGB_E_ARG, "bad argument");
  const int in = cur_in(b);
  // slice and lane of the field: field-major, or P0=(ux,ax) P1=(uy,ay) P2=(uz,az) P3=(lnrho,ss)
  int slice = field, lane = 0;
  if (b->pairs) {
    const int iax = b->nf - 3;
    if (field < 4) { slice = field; lane = 0; }
    else if (b->nf == 8 && field == 4) { slice = 3; lane = 1; }
    else { slice = field - iax; lane = 1; }
  }
  // lane offset in bytes: one value (field-major / FP32 pairs) or one float of the
  // double-float pair's hi half (its lo half is 8 bytes further)
  const size_t lane_bytes = (b->dfl && b->pairs) ? 4 : (size_t)b->tb;
  char* base = static_cast<char*>(b->f[in]) + (size_t)slice * b->fs * b->eb + (size_t)lane * lane_bytes;
  const pcgb_params& p = b->p;
  const int comp = (field < 3) ? field : 0;   // ABC component of uu
  CK(launch_init_field(elem_code(b), base, kind, kind == 2 ? comp : 0, ampl, a, bb, c, k, seed, b->nx, b->ny, b->nz, b->px,
                       b->my, b->xoff, p.xyz0[0], p.xyz0[1], p.xyz0[2], axis_spacing(p, 0), axis_spacing(p, 1),
                       axis_spacing(p, 2), axis_offset(p, 0), axis_offset(p, 1), axis_offset(p, 2),
                       b->pairs ? 2 : 1, g.stream));
  ++g.launches;
  return box_reset(b, 0.0);
}

// The box's f into a host f-array of REAL type (hb = 8: double, 4: float).
static int box_store_host(pcgb_box* b, void* fh, int hb) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!b || !fh) return set_err(PCGB_E_ARG, "null argument");
  const long long rows = (long long)b->my * b->mz * b->nf;
  const int in = cur_in(b);
  // the FP32 carry lives in df between steps (substep counter at a step boundary)
  const void* carry = (b->hdev.comp && (b->nsub % 3) == 0) ? b->df : nullptr;
  if (b->nonper) {   // update_ghosts before the snapshot (snapshot.f90:363)
    const int rc = box_boundconds(b);
    if (rc) return rc;
  }
  const int permask = (axis_periodic(b->p, 0) ? 1 : 0) | (axis_periodic(b->p, 1) ? 2 : 0) | (axis_periodic(b->p, 2) ? 4 : 0);
  if (void* dh = const_cast<void*>(host_alias(fh))) {
    CK(launch_store_rows(elem_code(b), hb, dh, b->f[in], carry, 0, rows, b->nx, b->ny, b->nz, b->px,
                         b->my, b->mz, b->xoff, b->nf, b->pairs, permask, g.stream));
    ++g.launches;
    CK(cudaStreamSynchronize(g.stream));
    return box_check_state(b);
  }
  // staged: the layout kernel of chunk c fills buffer c&1 while chunk c-1 is copied out
  const long long chunk = (long long)(g.stage_elems / b->mx);
  CK(cudaEventRecord(g.ev_free[0], g.xfer));
  CK(cudaEventRecord(g.ev_free[1], g.xfer));
  int c = 0;
  for (long long r0 = 0; r0 < rows; r0 += chunk, ++c) {
    const int k = c & 1;
    const long long nr = std::min(chunk, rows - r0);
    CK(cudaStreamWaitEvent(g.stream, g.ev_free[k], 0));
    CK(launch_store_rows(elem_code(b), hb, g.stage[k], b->f[in], carry, r0, nr, b->nx, b->ny, b->nz, b->px, b->my, b->mz,
                         b->xoff, b->nf, b->pairs, permask, g.stream));
    ++g.launches;
    CK(cudaEventRecord(g.ev_copied[k], g.stream));
    CK(cudaStreamWaitEvent(g.xfer, g.ev_copied[k], 0));
    CK(cudaMemcpyAsync(static_cast<char*>(fh) + (size_t)(r0 * b->mx) * hb, g.stage[k], (size_t)(nr * b->mx) * hb,
                       cudaMemcpyDeviceToHost, g.xfer));
    CK(cudaEventRecord(g.ev_free[k], g.xfer));
  }
  CK(cudaStreamSynchronize(g.xfer));
  CK(cudaStreamSynchronize(g.stream));
  return box_check_state(b);
}

extern "C" int pcgb_box_store(pcgb_box* b, double* fh) { return box_store_host(b, fh, 8); }
extern "C" int pcgb_box_store_f32(pcgb_box* b, float* fh) { return box_store_host(b, fh, 4); }

// Random helical forcing of the step that starts now: draw its record into the
// device ring (forcing.f90 fconst_coefs_hel), applied when the step ends.  With
// magnetic forcing the step also draws the secondary record of lmhd_forcing
// (forcing_hel, forcing.f90:2136-2141), whose force on uu is zero by default,
// so the stream advances as the reference's does.
static int helical_begin_step(pcgb_box* b) {
  if (b->kvec.empty()) return set_err(PCGB_E_STATE, "helical forcing needs wavevectors (pcgb_box_set_kvectors)");
  HelRec rec, secondary;
  const int nk = (int)(b->kvec.size() / 3);
  helical_record(b->p.cs0, b->p.relhel, b->p.force_hel, b->kvec.data(), nk, b->kav, &b->rng, &rec);
  if (b->p.lmagnetic_forcing)
    helical_record(b->p.cs0, b->p.relhel, b->p.force_hel, b->kvec.data(), nk, b->kav, &b->rng, &secondary);
  CK(cudaMemcpyAsync(b->dring + (b->nsub / 3) % kHelRing, &rec, sizeof(rec), cudaMemcpyHostToDevice, g.stream));
  return 0;
}

static HelGeom helical_geom(const pcgb_box* b) {
  const pcgb_params& p = b->p;
  HelGeom hg;
  hg.nx = b->nx; hg.ny = b->ny; hg.nz = b->nz; hg.px = b->px; hg.my = b->my; hg.xoff = b->xoff;
  hg.ps = b->ps; hg.fs = b->fs;
  hg.x0 = p.xyz0[0]; hg.y0 = p.xyz0[1]; hg.z0 = p.xyz0[2];
  hg.dx = axis_spacing(p, 0); hg.dy = axis_spacing(p, 1); hg.dz = axis_spacing(p, 2);
  hg.ox = axis_offset(p, 0); hg.oy = axis_offset(p, 1); hg.oz = axis_offset(p, 2);
  hg.k1 = p.kf;
  hg.iax = b->nf - 3;
  hg.magnetic = p.lmagnetic_forcing ? 1 : 0;
  return hg;
}

// addforce (forcing.f90:1307) after the step: uu (aa with magnetic forcing) of the new state += the force.
static int helical_end_step(pcgb_box* b) {
  CK(launch_helical(hel_layout(b), b->f[cur_in(b)], b->dring, b->dstate, b->dtab, helical_geom(b), g.stream));
  g.launches += 2;
  return 0;
}

// The same force added by the last substep's update itself (FP32 pairs): its tables first.
static int helical_before_last_substep(pcgb_box* b) {
  CK(launch_helical_tables_pre(b->dring, b->dstate, b->dtab, helical_geom(b), g.stream));
  g.launches += 1;
  return 0;
}

static int box_substep(pcgb_box* b) {
  const int s = (int)(b->nsub % 3);
  int rc;
  if (s == 0) {
    if ((rc = box_ensure_dt(b))) return rc;
    if (b->hdev.dt_mode == PCGB_DT_CURRENT && (rc = box_launch(b, MODE_CFL))) return rc;
    if (b->p.lforcing_hel && (rc = helical_begin_step(b))) return rc;
  }
  const bool fused = b->hdev.hel_tab != nullptr;
  if (s == 2 && b->p.lforcing_hel && fused && (rc = helical_before_last_substep(b))) return rc;
  if ((rc = box_launch(b, MODE_SUBSTEP))) return rc;
  b->nsub++;
  if (s == 2 && b->p.lforcing_hel && !fused && (rc = helical_end_step(b))) return rc;
  return 0;
}

extern "C" int pcgb_box_set_kvectors(pcgb_box* b, const double* kxyz, int nk, double kav) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!b || !kxyz || nk < 1 || !(kav > 0.0)) return set_err(PCGB_E_ARG, "bad wavevector list");
  for (int i = 0; i < nk; ++i) {
    const double kx = kxyz[i], ky = kxyz[nk + i], kz = kxyz[2 * nk + i];
    if (kx * kx + ky * ky + kz * kz == 0.0) return set_err(PCGB_E_ARG, "wavevector %d is zero", i);
  }
  b->kvec.assign(kxyz, kxyz + 3 * (size_t)nk);
  b->kav = kav;
  return 0;
}

extern "C" int pcgb_box_steps(pcgb_box* b, int nsteps) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!b || nsteps < 0) return set_err(PCGB_E_ARG, "bad argument");
  if (b->nsub % 3 != 0) return set_err(PCGB_E_STATE, "box is in the middle of a step");
  for (int i = 0; i < 3 * nsteps; ++i) {
    int rc = box_substep(b);
    if (rc) return rc;
  }
  return 0;
}

extern "C" int pcgb_box_sync(pcgb_box* b) {
  CK(cudaStreamSynchronize(g.stream));
  return b ? box_check_state(b) : 0;
}

extern "C" int pcgb_box_diag(pcgb_box* b, double* out, int nout) {
  if (!b || !out) return set_err(PCGB_E_ARG, "null argument");
  PcgbBoxState st;
  CK(cudaMemcpyAsync(&st, b->dstate, sizeof(st), cudaMemcpyDeviceToHost, g.stream));
  CK(cudaStreamSynchronize(g.stream));
  double v[PCGB_NSLOT + 3];
  for (int i = 0; i < PCGB_NSLOT; ++i) v[i] = st.diag[i];
  v[PCGB_NSLOT] = st.t; v[PCGB_NSLOT + 1] = st.dt; v[PCGB_NSLOT + 2] = (double)(long long)st.diag_step;
  for (int i = 0; i < nout && i < PCGB_NSLOT + 3; ++i) out[i] = v[i];
  return 0;
}

extern "C" int pcgb_box_time(pcgb_box* b, double* t, double* dt, long long* nsub) {
  if (!b) return set_err(PCGB_E_ARG, "null box");
  PcgbBoxState st;
  CK(cudaMemcpyAsync(&st, b->dstate, sizeof(st), cudaMemcpyDeviceToHost, g.stream));
  CK(cudaStreamSynchronize(g.stream));
  if (t) *t = st.t;
  if (dt) *dt = st.dt;
  if (nsub) *nsub = (long long)st.nsub;
  return 0;
}

extern "C" int pcgb_box_set_dt(pcgb_box* b, double dt) {
  if (!b || !(dt > 0)) return set_err(PCGB_E_ARG, "bad argument");
  PcgbBoxState st;
  CK(cudaMemcpyAsync(&st, b->dstate, sizeof(st), cudaMemcpyDeviceToHost, g.stream));
  CK(cudaStreamSynchronize(g.stream));
  st.dt = dt; st.dt_next = dt;
  CK(cudaMemcpyAsync(b->dstate, &st, sizeof(st), cudaMemcpyHostToDevice, g.stream));
  CK(cudaStreamSynchronize(g.stream));
  b->dt_known = true;
  return 0;
}

static int box_request_diag(pcgb_box* b) {
  b->diag_pending = true;
  int one = 1;
  CK(cudaMemcpyAsync(reinterpret_cast<char*>(b->dstate) + offsetof(PcgbBoxState, diag_request), &one, sizeof(int),
                     cudaMemcpyHostToDevice, g.stream));
  CK(cudaStreamSynchronize(g.stream));
  return 0;
}

// ---------------------------------------------------------------------------
// batches
struct pcgb_batch {
  std::vector<pcgb_box*> boxes;   // sorted by descending work
  PcgbBoxDev* ddev = nullptr;
  unsigned int* counter = nullptr;
  int total_tiles = 0;
  int persistent = 1;
  int grid = 0;
  KernelHandle kh;
  bool any_current = false;
  bool red0 = false;   // some box reduces on every substep 1 (lagged CFL dt or periodic diagnostics)
  bool all_comp = true;   // every box holds the compensated FP32 state
  cudaGraphExec_t gexec = nullptr;
  int gsteps = 0;
};

extern "C" pcgb_batch* pcgb_batch_create(pcgb_box** boxes, int n, int persistent) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!boxes || n < 1) { set_err(PCGB_E_ARG, "empty batch"); return nullptr; }
  pcgb_batch* B = new pcgb_batch();
  B->boxes.assign(boxes, boxes + n);
  for (auto* b : B->boxes) {
    if (!b || b->tb != boxes[0]->tb || b->dfl != boxes[0]->dfl || b->nf != boxes[0]->nf ||
        b->tile != boxes[0]->tile || b->kh.fn != boxes[0]->kh.fn) {
      set_err(PCGB_E_ARG, "a batch needs boxes of one class (precision, fields, tile, upwinding)");
      delete B;
      return nullptr;
    }
    if (b->nsub % 3 != 0) { set_err(PCGB_E_STATE, "box in the middle of a step"); delete B; return nullptr; }
    if (b->p.lforcing_hel || b->nonper) {
      set_err(PCGB_E_UNSUPPORTED, "random helical forcing and non-periodic boundaries step through the box API, "
                                  "not in a batch");
      delete B;
      return nullptr;
    }
  }
  std::stable_sort(B->boxes.begin(), B->boxes.end(), [](const pcgb_box* a, const pcgb_box* c) {
    return (long long)a->nx * a->ny * a->nz > (long long)c->nx * c->ny * c->nz;
  });
  std::vector<PcgbBoxDev> h(n);
  int t0 = 0;
  for (int i = 0; i < n; ++i) {
    h[i] = B->boxes[i]->hdev;
    h[i].tile0 = t0;
    t0 += h[i].tiles;
    if (B->boxes[i]->hdev.dt_mode == PCGB_DT_CURRENT) B->any_current = true;
    if (B->boxes[i]->hdev.dt_mode == PCGB_DT_LAGGED || B->boxes[i]->hdev.diag_every > 0) B->red0 = true;
    if (B->boxes[i]->hdev.comp == 0) B->all_comp = false;
  }
  B->total_tiles = t0;
  B->kh = boxes[0]->kh;
  B->persistent = persistent;
  if (cudaMalloc(&B->ddev, sizeof(PcgbBoxDev) * n) != cudaSuccess ||
      cudaMalloc(&B->counter, sizeof(unsigned int)) != cudaSuccess) {
    set_err(PCGB_E_NOMEM, "batch descriptor allocation failed");
    cudaFree(B->ddev); delete B; return nullptr;
  }
  cudaMemcpyAsync(B->ddev, h.data(), sizeof(PcgbBoxDev) * n, cudaMemcpyHostToDevice, g.stream);
  int occ = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, B->kh.fn, B->kh.threads, (size_t)B->kh.smem);
  if (occ < 1) occ = 1;
  B->grid = persistent ? std::min(B->total_tiles, occ * g.nsm) : B->total_tiles;
  if (cudaStreamSynchronize(g.stream) != cudaSuccess) { set_err(PCGB_E_CUDA, "batch upload failed"); }
  return B;
}

extern "C" void pcgb_batch_destroy(pcgb_batch* B) {
  if (!B) return;
  cudaStreamSynchronize(g.stream);
  if (B->gexec) cudaGraphExecDestroy(B->gexec);
  cudaFree(B->ddev); cudaFree(B->counter);
  delete B;
}

static bool batch_diag_pending(const pcgb_batch* B) {
  for (const auto* b : B->boxes)
    if (b->diag_pending) return true;
  return false;
}

static int batch_substep(pcgb_batch* B, int s) {
  int rc;
  unsigned int* ctr = B->persistent ? B->counter : nullptr;
  if (s == 0 && B->any_current &&
      (rc = launch(B->ddev, (int)B->boxes.size(), B->total_tiles, ctr, MODE_CFL, B->kh, B->grid, true)))
    return rc;
  const bool red = (s == 0) && (B->red0 || batch_diag_pending(B));
  rc = launch(B->ddev, (int)B->boxes.size(), B->total_tiles, ctr, MODE_SUBSTEP, B->kh, B->grid, red, s, B->all_comp);
  if (s == 0)
    for (auto* b : B->boxes) b->diag_pending = false;
  return rc;
}

extern "C" int pcgb_batch_steps(pcgb_batch* B, int nsteps, int use_graph, int graph_steps) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!B || nsteps < 0) return set_err(PCGB_E_ARG, "bad argument");
  int rc;
  for (auto* b : B->boxes)
    if ((rc = box_ensure_dt(b))) return rc;
  int done = 0;
  // a pending diagnostics request is served by direct launches (the captured
  // graph's substep-1 launches reduce only when the batch always does)
  if (use_graph && graph_steps > 0 && nsteps >= graph_steps && !batch_diag_pending(B)) {
    if (!B->gexec || B->gsteps != graph_steps) {
      if (B->gexec) { cudaGraphExecDestroy(B->gexec); B->gexec = nullptr; }
      cudaGraph_t graph;
      CK(cudaStreamBeginCapture(g.stream, cudaStreamCaptureModeThreadLocal));
      long long l0 = g.launches;
      for (int i = 0; i < graph_steps; ++i)
        for (int s = 0; s < 3; ++s)
          if ((rc = batch_substep(B, s))) { cudaStreamEndCapture(g.stream, &graph); return rc; }
      g.launches = l0;   // captured launches are counted when replayed
      CK(cudaStreamEndCapture(g.stream, &graph));
      CK(cudaGraphInstantiate(&B->gexec, graph, 0));
      cudaGraphDestroy(graph);
      B->gsteps = graph_steps;
    }
    while (nsteps - done >= graph_steps) {
      CK(cudaGraphLaunch(B->gexec, g.stream));
      g.launches += (long long)graph_steps * (3 + (B->any_current ? 1 : 0));
      done += graph_steps;
    }
  }
  for (; done < nsteps; ++done)
    for (int s = 0; s < 3; ++s)
      if ((rc = batch_substep(B, s))) return rc;
  for (auto* b : B->boxes) b->nsub += 3ull * (unsigned long long)nsteps;
  return 0;
}

// ---------------------------------------------------------------------------
// autotuner: tile variant and z-sweep depth per (precision, fields, grid)
static std::map<std::tuple<int, int, int, int, int, int>, std::tuple<int, int, double>> g_tune;

extern "C" int pcgb_autotune(const pcgb_params* p, int* tile, int* zdepth, double* ms) {
  if (validate(p)) return g_err;
  auto key = std::make_tuple(p->precision, p->dfloat, p->lentropy ? 8 : 7, p->nx, p->ny, p->nz);
  auto it = g_tune.find(key);
  if (it != g_tune.end()) {
    if (tile) *tile = std::get<0>(it->second);
    if (zdepth) *zdepth = std::get<1>(it->second);
    if (ms) *ms = std::get<2>(it->second);
    return 0;
  }
  pcgb_params q = *p;
  q.dt = (p->dt > 0) ? p->dt : 1e-4;
  q.diag_every = 0;
  q.tile = -1; q.zdepth = 0;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0); cudaEventCreate(&e1);
  double best = 1e30; int bt = -1, bz = 0;
  const int ntile = num_tiles(p->precision, p->dfloat);
  for (int fam = 0; fam < ((p->precision == 4 || p->dfloat) ? 2 : 1); ++fam) {
  q.tile = fam * kNumScalarTiles;
  pcgb_box* b = pcgb_box_create(&q);
  if (!b) { cudaEventDestroy(e0); cudaEventDestroy(e1); return g_err; }
  if (bt < 0) { bt = b->tile; bz = b->zd; }
  for (int t = fam * kNumScalarTiles; t < (fam + 1) * kNumScalarTiles && t < ntile; ++t) {
    KernelHandle kh = get_kernel(b->tb, b->nf, t, b->dfl, b->hdev.lupw != 0);
    if (!kh.fn || kh.smem > g.max_smem) continue;
    std::vector<int> zs = {b->nz, 256, 128, 64, 32, 16};
    std::sort(zs.begin(), zs.end());
    zs.erase(std::unique(zs.begin(), zs.end()), zs.end());
    for (int zd : zs) {
      if (zd > b->nz) continue;
      std::lock_guard<std::mutex> lk(g_mu);
      if (set_tiling(b, t, zd)) continue;
      for (int w = 0; w < 2; ++w) box_launch(b, MODE_SUBSTEP), b->nsub++;
      cudaEventRecord(e0, g.stream);
      const int reps = 3;
      for (int r = 0; r < reps; ++r) box_launch(b, MODE_SUBSTEP), b->nsub++;
      cudaEventRecord(e1, g.stream);
      cudaEventSynchronize(e1);
      float el = 0;
      cudaEventElapsedTime(&el, e0, e1);
      const double per = el / reps;
      if (per < best) { best = per; bt = t; bz = zd; }
    }
  }
  pcgb_box_destroy(b);
  }
  cudaEventDestroy(e0); cudaEventDestroy(e1);
  g_tune[key] = std::make_tuple(bt, bz, best);
  if (tile) *tile = bt;
  if (zdepth) *zdepth = bz;
  if (ms) *ms = best;
  return 0;
}

// ---------------------------------------------------------------------------
// library-wide
extern "C" void pcgb_default_params(pcgb_params* p) {
  if (!p) return;
  memset(p, 0, sizeof(*p));
  p->nx = p->ny = p->nz = 32;
  p->lentropy = 0;
  p->precision = 8;
  p->comp = 1;
  for (int i = 0; i < 3; ++i) { p->xyz0[i] = -M_PI; p->Lxyz[i] = 2.0 * M_PI; }
  p->gamma = 5.0 / 3.0; p->cs0 = 1.0; p->rho0 = 1.0; p->cp = 1.0;
  p->nu = 0.0; p->eta = 0.0; p->chi = 0.0; p->mu0 = 1.0;
  p->lforcing_cont = 0; p->ampl_ff = 0.0; p->kf = 1.0; p->relhel = 1.0;
  p->abc_a = p->abc_b = p->abc_c = 1.0; p->ampl_fcont_uu = 1.0;
  p->lohmic_heat = 1; p->lviscosity_heat = 1;
  p->cdt = 0.9; p->cdtv = 0.25;
  p->dt = 0.0; p->dt_mode = PCGB_DT_LAGGED; p->diag_every = 0;
  p->tile = -1; p->zdepth = 0;
  p->lforcing_hel = 0; p->force_hel = 0.0; p->seed_ff = 1812;   // seed0, cdata.f90:743
}

extern "C" int pcgb_last_error(void) { return g_err; }
extern "C" void pcgb_clear_error(void) { g_err = 0; g_errmsg[0] = 0; }
extern "C" const char* pcgb_error_string(int code) {
  if (code == g_err && g_errmsg[0]) return g_errmsg;
  switch (code) {
    case PCGB_OK: return "no error";
    case PCGB_E_CUDA: return "CUDA error";
    case PCGB_E_ARG: return "invalid argument";
    case PCGB_E_STATE: return "invalid call sequence";
    case PCGB_E_NOMEM: return "out of device memory";
    case PCGB_E_DEVICE: return "device reported a non-finite state";
    case PCGB_E_TIMEOUT: return "bounded device wait expired";
    case PCGB_E_UNSUPPORTED: return "unsupported configuration";
  }
  return "unknown error";
}
extern "C" void pcgb_set_stream(void* s) {
  if (g.own_stream && g.stream) { cudaStreamSynchronize(g.stream); cudaStreamDestroy(g.stream); }
  g.stream = (cudaStream_t)s;
  g.own_stream = false;
}
extern "C" void* pcgb_get_stream(void) {
  if (!g.init) engine_init();
  return (void*)g.stream;
}
extern "C" long long pcgb_launch_count(void) { return g.launches; }
extern "C" void pcgb_set_wait_limit(unsigned int iterations) {
  g.wait_limit = iterations ? iterations : (1u << 21);
}
extern "C" void pcgb_inject_wait_failure(int on) { g.inject_wait_failure = on ? 1 : 0; }
extern "C" const char* pcgb_version(void) { return "pcgb300 1.0 sm_103a"; }

// ---------------------------------------------------------------------------
// 1. reference plug-in ABI (src/gpu_astaroth_ansi.c:23-55) over one box
static pcgb_params g_par;
static bool g_par_set = false;
static pcgb_box* g_box = nullptr;
static std::vector<double> g_kvec;   // k.dat of the plug-in's box
static double g_kav = 0.0;
static REAL_PCGB* g_hostf = nullptr;

// The plug-in's host f-array is the Fortran build's REAL (double, or float in
// the single-precision library).
#ifdef PCGB_REAL_SINGLE
static int host_load(pcgb_box* b, const float* f, double t) { return pcgb_box_load_f32(b, f, t); }
static int host_store(pcgb_box* b, float* f) { return pcgb_box_store_f32(b, f); }
#else
static int host_load(pcgb_box* b, const double* f, double t) { return pcgb_box_load(b, f, t); }
static int host_store(pcgb_box* b, double* f) { return pcgb_box_store(b, f); }
#endif

extern "C" int pcgb_set_params(const pcgb_params* p) {
  if (validate(p)) return g_err;
  g_par = *p;
  g_par_set = true;
  return 0;
}

extern "C" void registerGPU(void) {}

extern "C" void initializeGPU(REAL_PCGB* f, int comm, double t, int nt, int read_all, int cpu_dt, int autotune) {
  (void)comm; (void)read_all;
  if (!g_par_set) { set_err(PCGB_E_STATE, "initializeGPU before pcgb_set_params"); return; }
  if (g_box) finalizeGPU();
  pcgb_params p = g_par;
  if (cpu_dt) p.dt_mode = PCGB_DT_CURRENT;
  if (autotune && p.tile < 0) {
    int t = -1, z = 0;
    if (pcgb_autotune(&p, &t, &z, nullptr) == 0) { p.tile = t; p.zdepth = z; }
  }
  g_box = pcgb_box_create(&p);
  if (!g_box) return;
  if (!g_kvec.empty()) pcgb_box_set_kvectors(g_box, g_kvec.data(), (int)(g_kvec.size() / 3), g_kav);
  g_hostf = f;
  if (f && nt > 0) host_load(g_box, f, t);   // gpu_astaroth.f90:236 load_farray_to_GPU
  else if (g_box) {
    PcgbBoxState st;
    cudaMemcpy(&st, g_box->dstate, sizeof(st), cudaMemcpyDeviceToHost);
    st.t = t;
    cudaMemcpy(g_box->dstate, &st, sizeof(st), cudaMemcpyHostToDevice);
  }
}

extern "C" void finalizeGPU(void) {
  if (g_box) pcgb_box_destroy(g_box);
  g_box = nullptr;
  g_hostf = nullptr;
}

extern "C" void getFArrayIn(REAL_PCGB** p) {
  if (!p) return;
  *p = g_box ? (REAL_PCGB*)g_box->f[cur_in(g_box)] : nullptr;
}

extern "C" void substepGPU(int isubstep, double t) {
  (void)t;
  if (!g_box) { set_err(PCGB_E_STATE, "substepGPU before initializeGPU"); return; }
  if (isubstep < 1 || isubstep > 3 || (int)(g_box->nsub % 3) != isubstep - 1) {
    set_err(PCGB_E_STATE, "substepGPU(%d) out of sequence (device is at substep %d)", isubstep,
            (int)(g_box->nsub % 3) + 1);
    return;
  }
  std::lock_guard<std::mutex> lk(g_mu);
  box_substep(g_box);
}

extern "C" void beforeBoundaryGPU(bool lrmv, int isubstep, double t, bool lsubstep) {
  (void)lrmv; (void)isubstep; (void)t; (void)lsubstep;
}
extern "C" void afterSubStepGPU(void) {}
extern "C" void radTransfer(void) {}

extern "C" void copyFarray(REAL_PCGB* f) {
  if (!g_box) { set_err(PCGB_E_STATE, "copyFarray before initializeGPU"); return; }
  if (!f) f = g_hostf;
  if (f) host_store(g_box, f);
}

extern "C" void loadFarray(void) {
  if (!g_box || !g_hostf) { set_err(PCGB_E_STATE, "loadFarray without a bound host f-array"); return; }
  double t = 0;
  pcgb_box_time(g_box, &t, nullptr, nullptr);
  host_load(g_box, g_hostf, t);
}

static int box_reload(pcgb_box* b, const pcgb_params& p) {
  if (p.nx != b->p.nx || p.ny != b->p.ny || p.nz != b->p.nz || p.lentropy != b->p.lentropy ||
      p.precision != b->p.precision || p.dfloat != b->p.dfloat)
    return set_err(PCGB_E_ARG, "reloadConfig cannot change grid, field count or precision");
  const int upw_was = b->hdev.lupw;
  b->p = p;
  b->nonper = !(axis_periodic(p, 0) && axis_periodic(p, 1) && axis_periodic(p, 2));
  fill_physics(b);
  int rc = upload_forcing(b);
  if (rc) return rc;
  // kernel variant; a box on the default tile takes the default tile of its new physics
  // (the default FP32 tile has no upwinding variant)
  if ((b->hdev.lupw != 0) != (upw_was != 0) &&
      (rc = p.tile >= 0 ? set_tiling(b, b->tile, b->zd) : set_tiling(b, -1, p.zdepth)))
    return rc;
  CK(cudaMemcpyAsync(b->ddev, &b->hdev, sizeof(PcgbBoxDev), cudaMemcpyHostToDevice, g.stream));
  if (p.dt > 0) return pcgb_box_set_dt(b, p.dt);
  CK(cudaStreamSynchronize(g.stream));
  return 0;
}

extern "C" void reloadConfig(void) {
  if (!g_box) return;
  std::lock_guard<std::mutex> lk(g_mu);
  box_reload(g_box, g_par);
}

// parameter table for updateInConfig*: the double members of pcgb_params
struct ParEntry { const char* name; size_t off; int n; };
static const ParEntry kPar[] = {
    {"xyz0", offsetof(pcgb_params, xyz0), 3}, {"Lxyz", offsetof(pcgb_params, Lxyz), 3},
    {"gamma", offsetof(pcgb_params, gamma), 1}, {"cs0", offsetof(pcgb_params, cs0), 1},
    {"rho0", offsetof(pcgb_params, rho0), 1}, {"cp", offsetof(pcgb_params, cp), 1},
    {"nu", offsetof(pcgb_params, nu), 1}, {"eta", offsetof(pcgb_params, eta), 1},
    {"chi", offsetof(pcgb_params, chi), 1}, {"mu0", offsetof(pcgb_params, mu0), 1},
    {"ampl_ff", offsetof(pcgb_params, ampl_ff), 1}, {"kf", offsetof(pcgb_params, kf), 1},
    {"relhel", offsetof(pcgb_params, relhel), 1}, {"abc_a", offsetof(pcgb_params, abc_a), 1},
    {"abc_b", offsetof(pcgb_params, abc_b), 1}, {"abc_c", offsetof(pcgb_params, abc_c), 1},
    {"ampl_fcont_uu", offsetof(pcgb_params, ampl_fcont_uu), 1}, {"b_ext", offsetof(pcgb_params, b_ext), 3},
    {"cdt", offsetof(pcgb_params, cdt), 1}, {"cdtv", offsetof(pcgb_params, cdtv), 1},
    {"dt", offsetof(pcgb_params, dt), 1},
};
static const int kNPar = sizeof(kPar) / sizeof(kPar[0]);

static int par_find(const char* name) {
  if (!name) return -1;
  for (int i = 0; i < kNPar; ++i)
    if (strcmp(kPar[i].name, name) == 0) return i;
  return -1;
}
// values of the Fortran REAL type (double or float) into the double parameters
static void par_set(int i, const REAL_PCGB* v, int n) {
  double* dst = reinterpret_cast<double*>(reinterpret_cast<char*>(&g_par) + kPar[i].off);
  for (int k = 0; k < kPar[i].n && k < n; ++k) dst[k] = (double)v[k];
  if (g_box) box_reload(g_box, g_par);
}

extern "C" void updateInConfigArr(int index) { (void)index; reloadConfig(); }
extern "C" int updateInConfigArrName(char* name) { (void)name; reloadConfig(); return 0; }
extern "C" void updateInConfigScal(int index, REAL_PCGB value) {
  if (index < 0 || index >= kNPar) { set_err(PCGB_E_ARG, "parameter index %d out of range", index); return; }
  par_set(index, &value, 1);
}
extern "C" int updateInConfigScalName(char* name, REAL_PCGB value) {
  int i = par_find(name);
  if (i < 0) return -1;
  par_set(i, &value, 1);
  return 0;
}
extern "C" void updateInConfigVec(int index, REAL_PCGB* value) {
  if (index < 0 || index >= kNPar || !value) { set_err(PCGB_E_ARG, "parameter index %d out of range", index); return; }
  par_set(index, value, 3);
}
extern "C" int updateInConfigVecName(char* name, REAL_PCGB* value) {
  int i = par_find(name);
  if (i < 0 || !value) return -1;
  par_set(i, value, 3);
  return 0;
}

extern "C" void prepareForFirstSubstep(double t) {
  (void)t;
  if (!g_box) return;
  std::lock_guard<std::mutex> lk(g_mu);
  box_ensure_dt(g_box);
}

extern "C" void random_initial_condition(void) {}

extern "C" void getGPUReducedVars(REAL_PCGB* dst) {
  if (!g_box || !dst) return;
  double v[PCGB_NSLOT + 3];
  if (pcgb_box_diag(g_box, v, PCGB_NSLOT + 3)) return;
  const double nw = (double)g_box->nx * g_box->ny * g_box->nz;   // diagnostics.f90:274
  dst[0] = std::sqrt(v[PCGB_S_U2SUM] / nw);
  dst[1] = std::sqrt(v[PCGB_S_U2MAX]);
  dst[2] = std::sqrt(v[PCGB_S_B2SUM] / nw);
  dst[3] = std::sqrt(v[PCGB_S_B2MAX]);
  dst[4] = v[PCGB_S_EKINSUM] / nw;
  dst[5] = v[PCGB_S_RHOSUM] / nw;
  dst[6] = std::sqrt(v[PCGB_S_DIVB2SUM] / nw);
  dst[7] = std::sqrt(v[PCGB_S_J2SUM] / nw);
  dst[8] = v[PCGB_S_ABSUM] / nw;
  double t = 0, dt = 0;
  pcgb_box_time(g_box, &t, &dt, nullptr);
  dst[9] = dt;
  dst[10] = t;
  dst[11] = v[PCGB_NSLOT + 2];
}

extern "C" void testBCs(void) {
  if (!g_box) return;
  const pcgb_box* b = g_box;
  std::vector<double> h((size_t)b->mx * b->my * b->mz * b->nf);
  if (pcgb_box_store(g_box, h.data())) return;
  auto at = [&](int i, int j, int k, int f) -> double& {
    return h[(size_t)i + (size_t)b->mx * ((size_t)j + (size_t)b->my * ((size_t)k + (size_t)b->mz * f))];
  };
  auto wr = [](int i, int n) { int v = i - 3; if (v < 0) v += n; else if (v >= n) v -= n; return v + 3; };
  double maxd = 0.0;
  for (int f = 0; f < b->nf; ++f)
    for (int k = 0; k < b->mz; ++k)
      for (int j = 0; j < b->my; ++j)
        for (int i = 0; i < b->mx; ++i) {
          double d = std::fabs(at(i, j, k, f) - at(wr(i, b->nx), wr(j, b->ny), wr(k, b->nz), f));
          if (d > maxd) maxd = d;
        }
  printf("testBCs: max |ghost - periodic image| = %.3e\n", maxd);
}

extern "C" void splitUpdate(const REAL_PCGB eps, const int max_iter) { (void)eps; (void)max_iter; }

extern "C" void copyVBApointers(REAL_PCGB** in, REAL_PCGB** out) {
  if (!g_box) { if (in) *in = nullptr; if (out) *out = nullptr; return; }
  const int c = cur_in(g_box);
  if (in) *in = (REAL_PCGB*)g_box->f[c];
  if (out) *out = (REAL_PCGB*)g_box->f[c ^ 1];
}

extern "C" void tf_save_checkpoint_c_api(const char*, const char*) {}
extern "C" void tf_save_model_c_api(const char*, const char*) {}
extern "C" void tf_load_model_c_api(const char*, const char*) {}
extern "C" void tf_load_model_checkpoint_c_api(const char*, const char*) {}
extern "C" void tf_create_model_c_api(const char*, const char*, int, bool) {}
extern "C" void tf_train_c_api(const char*, REAL_PCGB*, int, double) {}
extern "C" void tf_infer_c_api(const char*, int) {}
extern "C" void print_debug(void) {}

extern "C" int pcgb_set_kvectors(const double* kxyz, int nk, double kav) {
  if (!kxyz || nk < 1 || !(kav > 0.0)) return set_err(PCGB_E_ARG, "bad wavevector list");
  g_kvec.assign(kxyz, kxyz + 3 * (size_t)nk);
  g_kav = kav;
  if (g_box) return pcgb_box_set_kvectors(g_box, kxyz, nk, kav);
  return 0;
}

extern "C" double pcgb_get_dt(void) {
  double dt = 0;
  if (g_box) pcgb_box_time(g_box, nullptr, &dt, nullptr);
  return dt;
}
extern "C" double pcgb_get_time(void) {
  double t = 0;
  if (g_box) pcgb_box_time(g_box, &t, nullptr, nullptr);
  return t;
}
extern "C" void pcgb_request_diagnostics(void) {
  if (g_box) box_request_diag(g_box);
}

// Timestep.time_step with lgpu=T (timestep.f90:206 -> advance_substeps :77).
extern "C" int pcgb_time_step(int nsteps) {
  if (!g_box) return set_err(PCGB_E_STATE, "pcgb_time_step before initializeGPU");
  for (int it = 0; it < nsteps; ++it) {
    prepareForFirstSubstep(0.0);
    for (int itsub = 1; itsub <= 3; ++itsub) {
      beforeBoundaryGPU(false, itsub, 0.0, false);
      substepGPU(itsub, 0.0);
      afterSubStepGPU();
      if (g_err) return g_err;
    }
  }
  return 0;
}

// Fortran-callable wrappers, gpu_astaroth_ansi.c:72-289.
extern "C" void initialize_gpu_c_(REAL_PCGB* f, int* comm, double* t, int* nt, int* read_all, int* cpu_dt, int* autotune) {
  initializeGPU(f, *comm, *t, *nt, *read_all, *cpu_dt, *autotune);
}
extern "C" void register_gpu_c_(void) { registerGPU(); }
extern "C" void finalize_gpu_c_(void) { finalizeGPU(); }
extern "C" void get_farray_ptr_gpu_c_(REAL_PCGB** in, REAL_PCGB** out) { copyVBApointers(in, out); }
extern "C" void before_boundary_gpu_c_(int* lrmv, int* isubstep, double* t, int* lsubstepping) {
  beforeBoundaryGPU(*lrmv == 1, *isubstep, *t, *lsubstepping != 0);
}
extern "C" void update_after_substep_gpu_c_(void) { afterSubStepGPU(); }
extern "C" void rhs_gpu_c_(int* isubstep, double* t) { substepGPU(*isubstep, *t); }
extern "C" void copy_farray_c_(REAL_PCGB* f) { copyFarray(f); }
extern "C" void load_farray_c_(void) { loadFarray(); }
extern "C" void reload_gpu_config_c_(void) { reloadConfig(); }
extern "C" void update_on_gpu_scal_by_ind_c_(int* index, REAL_PCGB* value) { updateInConfigScal(*index, *value); }
extern "C" void update_on_gpu_vec_by_ind_c_(int* index, REAL_PCGB* value) { updateInConfigVec(*index, value); }
extern "C" void update_on_gpu_arr_by_ind_c_(int* index) { updateInConfigArr(*index); }
extern "C" int update_on_gpu_scal_by_name_c_(char* name, REAL_PCGB* value) { return updateInConfigScalName(name, *value); }
extern "C" int update_on_gpu_vec_by_name_c_(char* name, REAL_PCGB* value) { return updateInConfigVecName(name, value); }
extern "C" int update_on_gpu_arr_by_name_c_(char* name) { return updateInConfigArrName(name); }
extern "C" void gpu_prepare_for_first_substep_c_(double* t) { prepareForFirstSubstep(*t); }
extern "C" void radtransfer_gpu_c_(void) { radTransfer(); }
extern "C" void get_gpu_reduced_vars_c_(REAL_PCGB* dst) { getGPUReducedVars(dst); }
extern "C" void test_bcs_c_(void) { testBCs(); }
extern "C" void split_update_gpu_c_(void) { splitUpdate(1e-15, 1000000); }
// TorchFort wrappers (gpu_astaroth_ansi.c:72-108): gpu_astaroth.f90 names them as
// externals, so a link in place of the reference's plug-in needs them; no-ops here.
extern "C" void tf_train_c_(const char* m, REAL_PCGB* loss, int* itsub, double* t) { tf_train_c_api(m, loss, *itsub, *t); }
extern "C" void tf_infer_c_(const char* m, int* itsub) { tf_infer_c_api(m, *itsub); }
extern "C" void tf_create_model_c_(const char* m, const char* cfg, int* comm, int* lmpicomm) {
  tf_create_model_c_api(m, cfg, *comm, *lmpicomm == 1);
}
extern "C" void print_snapshot_c_(void) { print_debug(); }
extern "C" void tf_load_model_c_(const char* m, const char* f) { tf_load_model_c_api(m, f); }
extern "C" void tf_load_model_checkpoint_c_(const char* m, const char* d) { tf_load_model_checkpoint_c_api(m, d); }
extern "C" void tf_save_model_c_(const char* m, const char* f) { tf_save_model_c_api(m, f); }
extern "C" void tf_save_checkpoint_c_(const char* m, const char* d) { tf_save_checkpoint_c_api(m, d); }
