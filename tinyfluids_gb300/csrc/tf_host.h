// Host-side helpers of the C ABI: error reporting and launch checks.
#pragma once
#include <cuda_runtime.h>
#include <stdarg.h>
#include <stdio.h>

#include "../../include/tinyfluids_gb300.h"

namespace tf {

// Records a message for tf_last_error() on this thread and returns `status`.
int set_error(int status, const char* fmt, ...);

inline int cuda_check(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return TF_OK;
  return set_error(TF_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

// Status of the launches just enqueued.
inline int launch_check(const char* what) { return cuda_check(cudaGetLastError(), what); }

int sm_count();  // multiprocessors of the current device (cached per device)

// Launch shape of a for_each_cell kernel: threads along z (a multiple of 32,
// at most 256), blocks over the (x, y) rows, at most 16 per SM.
struct RowLaunch {
  int blocks, threads;
};
inline RowLaunch row_launch(int nx, int ny, int nz) {
  RowLaunch l;
  l.threads = nz >= 256 ? 256 : ((nz + 31) / 32) * 32;
  const long long rows = (long long)nx * ny, cap = (long long)sm_count() * 16;
  l.blocks = (int)(rows < cap ? rows : cap);
  return l;
}

}  // namespace tf

// Tile heights (grid rows incl. the one-cell ring) the fused kernel is
// instantiated for; the kernel uses rows/2 warps.
inline bool valid_tile_rows(int rows) { return rows == 8 || rows == 16 || rows == 32; }

// CTAs per SM the fused kernels are register-bounded for: TF_WARPS_PER_SM
// (16 by default) warps per SM for every tile height.
#ifndef TF_WARPS_PER_SM
#define TF_WARPS_PER_SM 16
#endif
__host__ __device__ constexpr int min_ctas_per_sm(int nwp) {
  return nwp >= TF_WARPS_PER_SM ? 1 : TF_WARPS_PER_SM / nwp;
}

// Launch bounds of the fused-step kernels (single step, TMA form, batch).
#define TF_FUSED_BOUNDS(NWP) __launch_bounds__((NWP) * 32, min_ctas_per_sm(NWP))

#define TF_DISPATCH_ROWS(rows, NWP, ...)          \
  switch (rows) {                                 \
    case 8: {                                     \
      constexpr int NWP = 4;                      \
      __VA_ARGS__;                                \
    } break;                                      \
    case 16: {                                    \
      constexpr int NWP = 8;                      \
      __VA_ARGS__;                                \
    } break;                                      \
    default: {                                    \
      constexpr int NWP = 16;                     \
      __VA_ARGS__;                                \
    } break;                                      \
  }

#define TF_TRY(expr)              \
  do {                            \
    int _st = (expr);             \
    if (_st != TF_OK) return _st; \
  } while (0)
