// kernels.cuh -- host-side view of the compiled substep kernel variants.
#pragma once
#include <cuda_runtime.h>
#include "mhd_substep.cuh"

namespace pcgb {

// Tile variants (TX, TY).  The ring depth is fixed per precision.
struct TileShape { int tx, ty; };
constexpr int kNumTiles = 4;
// FP32 variants: (32,4) (32,8) (16,8) (64,4); FP64 variants: (32,4) (16,8) (16,4) (32,2).
// FP32 (32,4) and (16,8) ask for two resident CTAs per SM.
inline TileShape tile_shape(int dtype_bytes, int tile) {
  static const TileShape f32[kNumTiles] = {{32, 4}, {32, 8}, {16, 8}, {64, 4}};
  static const TileShape f64[kNumTiles] = {{32, 4}, {16, 8}, {16, 4}, {32, 2}};
  return dtype_bytes == 4 ? f32[tile] : f64[tile];
}
constexpr int ring_depth(int dtype_bytes) { return dtype_bytes == 4 ? 9 : 8; }

struct KernelHandle {
  const void* fn = nullptr;
  int smem = 0;
  int threads = 0;
};

// Defined in kernels_<type>_<nf>.cu.
KernelHandle kernel_f32_7(int tile);
KernelHandle kernel_f32_8(int tile);
KernelHandle kernel_f64_7(int tile);
KernelHandle kernel_f64_8(int tile);

inline KernelHandle get_kernel(int dtype_bytes, int nf, int tile) {
  if (dtype_bytes == 4) return nf == 8 ? kernel_f32_8(tile) : kernel_f32_7(tile);
  return nf == 8 ? kernel_f64_8(tile) : kernel_f64_7(tile);
}

}  // namespace pcgb

// Instantiation helper used by the kernels_*.cu translation units.
#define PCGB_DEFINE_KERNELS(NAME, T, NF)                                                   \
  namespace pcgb {                                                                         \
  template <int TX, int TY, int MB>                                                        \
  static KernelHandle make_##NAME() {                                                      \
    constexpr int R = ring_depth(sizeof(T));                                               \
    KernelHandle h;                                                                        \
    h.fn = reinterpret_cast<const void*>(&mhd_substep_kernel<T, NF, TX, TY, R, MB>);       \
    h.smem = TileCfg<T, NF, TX, TY, R>::SMEM_BYTES;                                        \
    h.threads = TX * TY;                                                                   \
    cudaFuncSetAttribute(&mhd_substep_kernel<T, NF, TX, TY, R, MB>,                        \
                         cudaFuncAttributeMaxDynamicSharedMemorySize, h.smem);             \
    return h;                                                                              \
  }                                                                                        \
  KernelHandle NAME(int tile) {                                                            \
    static KernelHandle cache[kNumTiles];                                                  \
    static bool init[kNumTiles] = {false, false, false, false};                            \
    if (tile < 0 || tile >= kNumTiles) return KernelHandle();                              \
    if (!init[tile]) {                                                                     \
      if constexpr (sizeof(T) == 4) {                                                      \
        switch (tile) {                                                                    \
          case 0: cache[0] = make_##NAME<32, 4, 2>(); break;                               \
          case 1: cache[1] = make_##NAME<32, 8, 1>(); break;                               \
          case 2: cache[2] = make_##NAME<16, 8, 2>(); break;                               \
          default: cache[3] = make_##NAME<64, 4, 1>(); break;                              \
        }                                                                                  \
      } else {                                                                             \
        switch (tile) {                                                                    \
          case 0: cache[0] = make_##NAME<32, 4, 1>(); break;                               \
          case 1: cache[1] = make_##NAME<16, 8, 1>(); break;                               \
          case 2: cache[2] = make_##NAME<16, 4, 1>(); break;                               \
          default: cache[3] = make_##NAME<32, 2, 1>(); break;                              \
        }                                                                                  \
      }                                                                                    \
      init[tile] = true;                                                                   \
    }                                                                                      \
    return cache[tile];                                                                    \
  }                                                                                        \
  }
