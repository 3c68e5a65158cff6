// kernels.cuh -- host-side view of the compiled substep kernel variants.
#pragma once
#include <cuda_runtime.h>
#include "cell_ddpair.cuh"
#include "cell_pair.cuh"
#include "cell_pair_tmem.cuh"
#include "cell_scalar.cuh"
#include "mhd_driver.cuh"

namespace pcgb {

// Tile variants.  Ids 0..3 use the field-major layout (one value per field per
// cell); for FP32 and double-float, ids 4..7 use the packed field-pair layout
// (cell_pair.cuh: float2 elements; cell_ddpair.cuh: 16-byte dd2 elements).  The
// FP32 pair tiles 5 (8 warps) and 7 (12 warps, the default for large boxes)
// keep their z-direction data in tensor memory (cell_pair_tmem.cuh), as does
// the upwinding variant of tile 5; tile 7 has no upwinding variant.
//   FP32: 0 (32,4)x2  1 (32,8)  2 (16,8)x2  3 (64,4)  4 pair(32,4)x2  5 pair(32,8)  6 pair(16,8)x2  7 pair(32,12)
//   FP64: 0 (32,4)  1 (16,8)  2 (24,8)  3 (32,6)
//   double-float: 0..3 as FP64, 4 pair(24,8)  5 pair(16,12)  6 pair(16,8)  7 pair(32,4)
// (FP64-family rings of 8 planes fit one CTA per SM; the 192-thread tiles
// give 6 warps per SM instead of 4.)  "x2" variants ask for two resident CTAs per SM.
// dfl: the box holds the double-float state.
struct TileShape { int tx, ty; };
constexpr int kNumScalarTiles = 4;
constexpr int kNumTiles = 8;
inline int num_tiles(int dtype_bytes, int dfl = 0) {
  return (dtype_bytes == 4 || dfl) ? kNumTiles : kNumScalarTiles;
}
inline bool tile_is_pair(int dtype_bytes, int tile, int dfl = 0) {
  return (dtype_bytes == 4 || dfl) && tile >= kNumScalarTiles;
}
// Namespace-scope constexpr tables have internal linkage.  (Static locals of an
// inline function would be one process-wide "unique" symbol, shared by every
// library built from these sources that a process loads.)
constexpr TileShape kF32Tiles[kNumScalarTiles] = {{32, 4}, {32, 8}, {16, 8}, {64, 4}};
constexpr TileShape kF32PairTiles[kNumScalarTiles] = {{32, 4}, {32, 8}, {16, 8}, {32, 12}};
constexpr TileShape kF64Tiles[kNumScalarTiles] = {{32, 4}, {16, 8}, {24, 8}, {32, 6}};
constexpr TileShape kDdPairTiles[kNumScalarTiles] = {{24, 8}, {16, 12}, {16, 8}, {32, 4}};
inline TileShape tile_shape(int dtype_bytes, int tile, int dfl = 0) {
  if (dtype_bytes == 4) return tile >= kNumScalarTiles ? kF32PairTiles[tile - kNumScalarTiles] : kF32Tiles[tile];
  return (dfl && tile >= kNumScalarTiles) ? kDdPairTiles[tile - kNumScalarTiles] : kF64Tiles[tile % kNumScalarTiles];
}

struct KernelHandle {
  const void* fn = nullptr;        // with CFL / diagnostic reductions
  const void* fn_nored = nullptr;  // without (same shared memory and block)
  const void* fn_comp[3] = {nullptr, nullptr, nullptr};   // reduction-free, compensated, substep s (FP32 tiles 5-7)
  const void* fn_comp_red = nullptr;                        // with reductions, compensated, substep 1
  int smem = 0;
  int threads = 0;
  // the kernel for a launch; s (0..2) and comp describe every box of the launch, s < 0 if they
  // differ; substep: a substep launch (not the CFL pass)
  const void* pick(bool red, int s = -1, bool comp = false, bool substep = true) const {
    if (comp && substep && s >= 0 && s < 3) {
      if (!red && fn_comp[s]) return fn_comp[s];
      if (red && s == 0 && fn_comp_red) return fn_comp_red;
    }
    return red ? fn : fn_nored;
  }
};

// Defined in kernels_<type>_<nf>.cu.
KernelHandle kernel_f32_7(int tile);
KernelHandle kernel_f32_8(int tile);
KernelHandle kernel_f64_7(int tile);
KernelHandle kernel_f64_8(int tile);
KernelHandle kernel_dd_7(int tile);
KernelHandle kernel_dd_8(int tile);
// Variants with the upwind corrections, defined in kernels_upw_<type>.cu for the
// tiles upw_tile() names (an empty handle for the others).
KernelHandle kernel_f32_7_upw(int tile);
KernelHandle kernel_f32_8_upw(int tile);
KernelHandle kernel_f64_7_upw(int tile);
KernelHandle kernel_f64_8_upw(int tile);
KernelHandle kernel_dd_7_upw(int tile);
KernelHandle kernel_dd_8_upw(int tile);

// Tiles compiled with upwinding: the default tiles of the box and server
// paths for each element type, and the field-major (32,8) FP32 tile.
inline bool upw_tile(int dtype_bytes, int tile, int dfl = 0) {
  if (dtype_bytes == 4) return tile == 1 || tile == 5 || tile == 6;
  if (dfl) return tile == 2 || tile == 3 || tile == 5 || tile == 6;
  return tile == 1 || tile == 2 || tile == 3;
}

// The tensor-memory cell (FP32 pair tiles 5 and 7) addresses the arrays with 32-bit
// element offsets of up to 2 fs + 8 ps (fs, ps: elements per slice and per plane).
inline bool tile_uses_offsets32(int dtype_bytes, int tile) {
  return dtype_bytes == 4 && (tile == 5 || tile == 7);
}
inline bool offsets32_fit(long long fs, long long ps) { return 2 * fs + 8 * ps < (1LL << 32); }

// dfl: FP64-class state held as double-float pairs (8-byte elements, same tiles as FP64)
// upw: the variant with the upwind corrections
inline KernelHandle get_kernel(int dtype_bytes, int nf, int tile, int dfl = 0, bool upw = false) {
  if (upw) {
    if (dtype_bytes == 4) return nf == 8 ? kernel_f32_8_upw(tile) : kernel_f32_7_upw(tile);
    if (dfl) return nf == 8 ? kernel_dd_8_upw(tile) : kernel_dd_7_upw(tile);
    return nf == 8 ? kernel_f64_8_upw(tile) : kernel_f64_7_upw(tile);
  }
  if (dtype_bytes == 4) return nf == 8 ? kernel_f32_8(tile) : kernel_f32_7(tile);
  if (dfl) return nf == 8 ? kernel_dd_8(tile) : kernel_dd_7(tile);
  return nf == 8 ? kernel_f64_8(tile) : kernel_f64_7(tile);
}

template <class CELL, int TX, int TY, int R, int MB, bool SPEC = false>
static KernelHandle make_kernel_handle();

// Pair tiles of the double-float family (no kernel for the other element types).
template <typename T, int NF, int TX, int TY, bool UPW = false>
static KernelHandle make_dd_pair_handle() {
  if constexpr (is_dd<T>::value) return make_kernel_handle<DDPairCell<NF, TX, TY, UPW>, TX, TY, 8, 1>();
  else return KernelHandle();
}

// SPEC: also the substep-specialised compensated variants (KIND 1..3)
template <class CELL, int TX, int TY, int R, int MB, bool SPEC>
static KernelHandle make_kernel_handle() {
  KernelHandle h;
  h.fn = reinterpret_cast<const void*>(&mhd_substep_kernel<CELL, TX, TY, R, MB, true>);
  h.fn_nored = reinterpret_cast<const void*>(&mhd_substep_kernel<CELL, TX, TY, R, MB, false>);
  h.smem = DriverCfg<CELL, TX, TY, R>::SMEM_BYTES;
  h.threads = TX * TY;
  cudaFuncSetAttribute(&mhd_substep_kernel<CELL, TX, TY, R, MB, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       h.smem);
  cudaFuncSetAttribute(&mhd_substep_kernel<CELL, TX, TY, R, MB, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       h.smem);
  if constexpr (SPEC) {
    h.fn_comp[0] = reinterpret_cast<const void*>(&mhd_substep_kernel<CELL, TX, TY, R, MB, false, 1>);
    h.fn_comp[1] = reinterpret_cast<const void*>(&mhd_substep_kernel<CELL, TX, TY, R, MB, false, 2>);
    h.fn_comp[2] = reinterpret_cast<const void*>(&mhd_substep_kernel<CELL, TX, TY, R, MB, false, 3>);
    h.fn_comp_red = reinterpret_cast<const void*>(&mhd_substep_kernel<CELL, TX, TY, R, MB, true, 1>);
    for (const void* fn : h.fn_comp) cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, h.smem);
    cudaFuncSetAttribute(h.fn_comp_red, cudaFuncAttributeMaxDynamicSharedMemorySize, h.smem);
  }
  return h;
}

}  // namespace pcgb

// Instantiation helper used by the kernels_*.cu translation units.
#define PCGB_DEFINE_KERNELS(NAME, T, NF)                                                           \
  namespace pcgb {                                                                                 \
  KernelHandle NAME(int tile) {                                                                    \
    static KernelHandle cache[kNumTiles];                                                          \
    static bool init[kNumTiles] = {false, false, false, false, false, false, false, false};        \
    if (tile < 0 || tile >= num_tiles(sizeof(T), is_dd<T>::value)) return KernelHandle();          \
    if (!init[tile]) {                                                                             \
      if constexpr (sizeof(T) == 4) {                                                              \
        switch (tile) {                                                                            \
          case 0: cache[0] = make_kernel_handle<ScalarCell<T, NF, 32, 4>, 32, 4, 9, 2>(); break;   \
          case 1: cache[1] = make_kernel_handle<ScalarCell<T, NF, 32, 8>, 32, 8, 9, 1>(); break;   \
          case 2: cache[2] = make_kernel_handle<ScalarCell<T, NF, 16, 8>, 16, 8, 9, 2>(); break;   \
          case 3: cache[3] = make_kernel_handle<ScalarCell<T, NF, 64, 4>, 64, 4, 9, 1>(); break;   \
          case 4: cache[4] = make_kernel_handle<PairCell<NF, 32, 4>, 32, 4, 8, 2>(); break;        \
          case 5: cache[5] = make_kernel_handle<PairCellTM<NF, 32, 8>, 32, 8, 9, 1, true>(); break; \
          case 6: cache[6] = make_kernel_handle<PairCell<NF, 16, 8>, 16, 8, 8, 2, true>(); break;  \
          default: cache[7] = make_kernel_handle<PairCellTM<NF, 32, 12>, 32, 12, 9, 1, true>(); break; \
        }                                                                                          \
      } else {                                                                                     \
        switch (tile) {                                                                            \
          case 4: cache[4] = make_dd_pair_handle<T, NF, 24, 8>(); break;                           \
          case 5: cache[5] = make_dd_pair_handle<T, NF, 16, 12>(); break;                          \
          case 6: cache[6] = make_dd_pair_handle<T, NF, 16, 8>(); break;                           \
          case 7: cache[7] = make_dd_pair_handle<T, NF, 32, 4>(); break;                           \
          case 0: cache[0] = make_kernel_handle<ScalarCell<T, NF, 32, 4>, 32, 4, 8, 1>(); break;   \
          case 1: cache[1] = make_kernel_handle<ScalarCell<T, NF, 16, 8>, 16, 8, 8, 1>(); break;   \
          case 2: cache[2] = make_kernel_handle<ScalarCell<T, NF, 24, 8>, 24, 8, 8, 1>(); break;   \
          default: cache[3] = make_kernel_handle<ScalarCell<T, NF, 32, 6>, 32, 6, 8, 1>(); break;  \
        }                                                                                          \
      }                                                                                            \
      init[tile] = true;                                                                           \
    }                                                                                              \
    return cache[tile];                                                                            \
  }                                                                                                \
  }

// Upwinding variants of the tiles upw_tile() names, same shapes, rings and
// residency as the plain ones.
#define PCGB_DEFINE_UPW_KERNELS(NAME, T, NF)                                                       \
  namespace pcgb {                                                                                 \
  KernelHandle NAME(int tile) {                                                                    \
    static KernelHandle cache[kNumTiles];                                                          \
    static bool init[kNumTiles] = {false, false, false, false, false, false, false, false};        \
    if (tile < 0 || tile >= num_tiles(sizeof(T), is_dd<T>::value) ||                               \
        !upw_tile(sizeof(T), tile, is_dd<T>::value))                                               \
      return KernelHandle();                                                                       \
    if (!init[tile]) {                                                                             \
      if constexpr (sizeof(T) == 4) {                                                              \
        switch (tile) {                                                                            \
          case 1: cache[1] = make_kernel_handle<ScalarCell<T, NF, 32, 8, true>, 32, 8, 9, 1>(); break; \
          case 5: cache[5] = make_kernel_handle<PairCellTM<NF, 32, 8, true>, 32, 8, 9, 1, true>(); break; \
          default: cache[6] = make_kernel_handle<PairCell<NF, 16, 8, true>, 16, 8, 8, 2>(); break; \
        }                                                                                          \
      } else {                                                                                     \
        switch (tile) {                                                                            \
          case 5: cache[5] = make_dd_pair_handle<T, NF, 16, 12, true>(); break;                    \
          case 6: cache[6] = make_dd_pair_handle<T, NF, 16, 8, true>(); break;                     \
          case 1: cache[1] = make_kernel_handle<ScalarCell<T, NF, 16, 8, true>, 16, 8, 8, 1>(); break; \
          case 2: cache[2] = make_kernel_handle<ScalarCell<T, NF, 24, 8, true>, 24, 8, 8, 1>(); break; \
          default: cache[3] = make_kernel_handle<ScalarCell<T, NF, 32, 6, true>, 32, 6, 8, 1>(); break; \
        }                                                                                          \
      }                                                                                            \
      init[tile] = true;                                                                           \
    }                                                                                              \
    return cache[tile];                                                                            \
  }                                                                                                \
  }
