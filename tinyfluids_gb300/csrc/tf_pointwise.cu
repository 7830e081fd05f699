// The reference's building blocks as standalone device functions
// (fluid.py:105-413): sound speed, HLL wave speeds and their maximum, the
// Euler flux, the HLL interface flux and the open-boundary copy.  All use the
// reference's op order (ExactPolicy), so each is bit-identical to the
// float32 oracle.  The fused step does not call these; they complete the
// drop-in surface for code that uses the reference's helpers directly.
#include <math.h>

#include "tf_common.cuh"
#include "tf_host.h"
#include "tf_math.cuh"

namespace tf {

static int pw_grid(long long n) {
  long long b = (n + 255) / 256;
  long long cap = (long long)sm_count() * 8;
  return (int)(b < 1 ? 1 : (b < cap ? b : cap));
}

static StepConsts<float> pw_consts(float gamma) {
  StepConsts<float> k;
  k.g = gamma;
  k.gm1 = gamma - 1.f;
  k.igm1 = 1.f / k.gm1;
  k.inv_dx = 1.f;
  k.dt = 0.f;
  k.k = 0.f;
  return k;
}

#define TF_GRID_LOOP(i, n)                                                  \
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < (n); \
       i += (long long)gridDim.x * blockDim.x)

__global__ void sound_kernel(const float* __restrict__ rho, const float* __restrict__ p,
                             float* __restrict__ c, long long n, float g) {
  TF_GRID_LOOP(i, n) c[i] = exact_sound(rho[i], p[i], g);
}

__device__ __forceinline__ void load5(const float* W, long long n, long long i, float w[5]) {
#pragma unroll
  for (int v = 0; v < 5; ++v) w[v] = W[v * n + i];
}

template <int VEL>
__global__ void euler_flux_kernel(const float* __restrict__ W, float* __restrict__ F, long long n,
                                  StepConsts<float> k) {
  TF_GRID_LOOP(i, n) {
    float w[5];
    load5(W, n, i, w);
    Cell<float> c;
    ExactPolicy<float>::derive<VEL>(w, c, k);
#pragma unroll
    for (int v = 0; v < 5; ++v) F[v * n + i] = c.F[v];
  }
}

template <int VEL>
__global__ void wave_speeds_kernel(const float* __restrict__ WL, const float* __restrict__ WR,
                                   float* __restrict__ sm, float* __restrict__ sp, long long n,
                                   float g) {
  using O = IEEE<float>;
  TF_GRID_LOOP(i, n) {
    float cl = exact_sound(WL[i], WL[4 * n + i], g), cr = exact_sound(WR[i], WR[4 * n + i], g);
    float ul = WL[VEL * n + i], ur = WR[VEL * n + i];
    sp[i] = O::mx(O::mx(O::add(ul, cl), O::add(ur, cr)), 0.f);
    sm[i] = O::mn(O::mn(O::sub(ul, cl), O::sub(ur, cr)), 0.f);
  }
}

// max(max|S+|, max|S-|) over all cells (fluid.py:192-195) into ctl->max_speed
template <int VEL>
__global__ void __launch_bounds__(256) max_wave_speeds_kernel(const float* __restrict__ WL,
                                                              const float* __restrict__ WR,
                                                              long long n, float g, tf_ctl* ctl) {
  using O = IEEE<float>;
  __shared__ float red[8];
  float m = 0.f;
  TF_GRID_LOOP(i, n) {
    float cl = exact_sound(WL[i], WL[4 * n + i], g), cr = exact_sound(WR[i], WR[4 * n + i], g);
    float ul = WL[VEL * n + i], ur = WR[VEL * n + i];
    float sp = O::mx(O::mx(O::add(ul, cl), O::add(ur, cr)), 0.f);
    float sm = O::mn(O::mn(O::sub(ul, cl), O::sub(ur, cr)), 0.f);
    m = speed_max(m, speed_max(fabsf(sp), fabsf(sm)));
  }
  float bm = block_max(m, red);
  if (threadIdx.x == 0) ctl_finish_cta(ctl, bm, gridDim.x, 0.f, false);
}

template <int VEL>
__global__ void hll_kernel(const float* __restrict__ WL, const float* __restrict__ WR,
                           float* __restrict__ F, long long n, StepConsts<float> k) {
  TF_GRID_LOOP(i, n) {
    float wl[5], wr[5], f[5];
    load5(WL, n, i, wl);
    load5(WR, n, i, wr);
    Cell<float> L, R;
    ExactPolicy<float>::derive<VEL>(wl, L, k);
    ExactPolicy<float>::derive<VEL>(wr, R, k);
    ExactPolicy<float>::hll(L, R, f);
#pragma unroll
    for (int v = 0; v < 5; ++v) F[v * n + i] = f[v];
  }
}

// Open boundaries with g ghost cells (fluid.py:335-413): per axis, cells
// [0,g) take cell g, then cells [n-g,n) take cell n-g-1 of the left-copied
// array; axes x, y, z in turn.  As a remap: out(i) = in(left(right(i))).
__device__ __forceinline__ int open_remap(int i, int n, int g, bool lo, bool hi) {
  if (hi && i >= n - g) i = n - g - 1;
  if (lo && i < g) i = g;
  return i;
}

__global__ void open_boundaries_kernel(const float* __restrict__ W, float* __restrict__ out,
                                       int nx, int ny, int nz, int g, unsigned lo_mask,
                                       unsigned hi_mask) {
  const long long n = (long long)nx * ny * nz;
  TF_GRID_LOOP(i, n) {
    int z = (int)(i % nz);
    long long r = i / nz;
    int y = (int)(r % ny), x = (int)(r / ny);
    int sx = open_remap(x, nx, g, lo_mask & 1u, hi_mask & 1u);
    int sy = open_remap(y, ny, g, lo_mask & 2u, hi_mask & 2u);
    int sz = open_remap(z, nz, g, lo_mask & 4u, hi_mask & 4u);
    long long j = ((long long)sx * ny + sy) * nz + sz;
#pragma unroll
    for (int v = 0; v < 5; ++v) out[v * n + i] = W[v * n + j];
  }
}

#define TF_DISPATCH_VEL(vel, ...)           \
  switch (vel) {                            \
    case 1: {                               \
      constexpr int VEL = 1;                \
      __VA_ARGS__;                          \
    } break;                                \
    case 2: {                               \
      constexpr int VEL = 2;                \
      __VA_ARGS__;                          \
    } break;                                \
    default: {                              \
      constexpr int VEL = 3;                \
      __VA_ARGS__;                          \
    } break;                                \
  }

static int check_pw(long long n, int vel, float gamma) {
  if (n < 0) return set_error(TF_ERR_ARG, "ncells must be >= 0");
  if (vel < 1 || vel > 3) return set_error(TF_ERR_ARG, "flux_direction_index must be 1, 2 or 3");
  if (!isfinite(gamma) || gamma == 1.f) return set_error(TF_ERR_ARG, "gamma must be finite and != 1");
  return TF_OK;
}

}  // namespace tf

using namespace tf;

extern "C" {

int tf_speed_of_sound(const float* rho, const float* p, float* c, long long n, float gamma,
                      void* stream) {
  if (!rho || !p || !c) return set_error(TF_ERR_ARG, "null pointer");
  TF_TRY(check_pw(n, 1, gamma));
  if (n == 0) return TF_OK;
  sound_kernel<<<pw_grid(n), 256, 0, (cudaStream_t)stream>>>(rho, p, c, n, gamma);
  return launch_check("sound_kernel");
}

int tf_euler_flux(const float* W, float* F, long long ncells, float gamma, int vel, void* stream) {
  if (!W || !F || W == F) return set_error(TF_ERR_ARG, "bad state pointers");
  TF_TRY(check_pw(ncells, vel, gamma));
  if (ncells == 0) return TF_OK;
  StepConsts<float> k = pw_consts(gamma);
  cudaStream_t s = (cudaStream_t)stream;
  TF_DISPATCH_VEL(vel, euler_flux_kernel<VEL><<<pw_grid(ncells), 256, 0, s>>>(W, F, ncells, k));
  return launch_check("euler_flux_kernel");
}

int tf_wave_speeds(const float* WL, const float* WR, float* s_minus, float* s_plus, long long ncells,
                   float gamma, int vel, void* stream) {
  if (!WL || !WR || !s_minus || !s_plus) return set_error(TF_ERR_ARG, "null pointer");
  TF_TRY(check_pw(ncells, vel, gamma));
  if (ncells == 0) return TF_OK;
  cudaStream_t s = (cudaStream_t)stream;
  TF_DISPATCH_VEL(vel, wave_speeds_kernel<VEL><<<pw_grid(ncells), 256, 0, s>>>(
                           WL, WR, s_minus, s_plus, ncells, gamma));
  return launch_check("wave_speeds_kernel");
}

int tf_max_wave_speeds(const float* WL, const float* WR, long long ncells, float gamma, int vel,
                       tf_ctl* ctl, void* stream) {
  if (!WL || !WR || !ctl) return set_error(TF_ERR_ARG, "null pointer");
  TF_TRY(check_pw(ncells, vel, gamma));
  if (ncells < 1) return set_error(TF_ERR_ARG, "the maximum of no interfaces is undefined");
  cudaStream_t s = (cudaStream_t)stream;
  TF_TRY(cuda_check(cudaMemsetAsync(ctl, 0, sizeof(tf_ctl), s), "cudaMemsetAsync(ctl)"));
  TF_DISPATCH_VEL(vel, max_wave_speeds_kernel<VEL><<<pw_grid(ncells), 256, 0, s>>>(
                           WL, WR, ncells, gamma, ctl));
  return launch_check("max_wave_speeds_kernel");
}

int tf_hll_flux(const float* WL, const float* WR, float* F, long long ncells, float gamma, int vel,
                void* stream) {
  if (!WL || !WR || !F || F == WL || F == WR) return set_error(TF_ERR_ARG, "bad state pointers");
  TF_TRY(check_pw(ncells, vel, gamma));
  if (ncells == 0) return TF_OK;
  StepConsts<float> k = pw_consts(gamma);
  cudaStream_t s = (cudaStream_t)stream;
  TF_DISPATCH_VEL(vel, hll_kernel<VEL><<<pw_grid(ncells), 256, 0, s>>>(WL, WR, F, ncells, k));
  return launch_check("hll_kernel");
}

int tf_open_boundaries(const float* W, float* out, int nx, int ny, int nz, int num_ghost_cells,
                       unsigned lo_axes, unsigned hi_axes, void* stream) {
  if (!W || !out || W == out) return set_error(TF_ERR_ARG, "bad state pointers");
  if (nx < 1 || ny < 1 || nz < 1) return set_error(TF_ERR_ARG, "grid dims must be >= 1");
  const int g = num_ghost_cells;
  if (g < 0) return set_error(TF_ERR_ARG, "num_ghost_cells must be >= 0");
  const int dims[3] = {nx, ny, nz};
  for (int a = 0; a < 3; ++a)
    if (((lo_axes | hi_axes) >> a & 1u) && g >= dims[a])
      return set_error(TF_ERR_ARG, "num_ghost_cells %d out of range for an axis of %d cells", g,
                       dims[a]);
  long long n = (long long)nx * ny * nz;
  open_boundaries_kernel<<<pw_grid(n), 256, 0, (cudaStream_t)stream>>>(W, out, nx, ny, nz, g,
                                                                       lo_axes, hi_axes);
  return launch_check("open_boundaries_kernel");
}

}  // extern "C"
