// Single-instance kernels and their C ABI: conversions, the CFL dt, the
// fused step, the per-axis sweep and the run-to-time loop.
#include <cuda.h>  // CUtensorMap and its enums (the encoder is fetched at run time)
#include <math.h>
#include <string.h>

#include <atomic>
#include <mutex>
#include <vector>

#include "tf_common.cuh"
#include "tf_fused.cuh"
#include "tf_fused_ym.cuh"
#include "tf_host.h"
#include "tf_math.cuh"

namespace tf {

// ---------------------------------------------------------------------------
// error reporting
// ---------------------------------------------------------------------------
static thread_local char g_err[512] = "";

int set_error(int status, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof g_err, fmt, ap);
  va_end(ap);
  return status;
}

int sm_count() {
  static std::mutex mu;
  static std::vector<int> cache;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 148;
  std::lock_guard<std::mutex> lk(mu);
  if ((int)cache.size() <= dev) cache.resize(dev + 1, 0);
  if (cache[dev] == 0) {
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0)
      n = 148;
    cache[dev] = n;
  }
  return cache[dev];
}

template <typename T>
static StepConsts<T> make_consts(T gamma, T dx, T dt) {
  StepConsts<T> k;
  k.g = gamma;
  k.gm1 = gamma - T(1);
  k.igm1 = T(1) / k.gm1;
  k.inv_dx = T(1) / dx;
  k.dt = dt;
  k.k = dt * k.inv_dx;
  return k;
}

// ---------------------------------------------------------------------------
// conversions (fluid.py:30-103), exact arithmetic
// ---------------------------------------------------------------------------
// Cell-wise map of a [5][n] state: 16-byte loads and stores of four cells per
// variable when n % 4 == 0 and both arrays are 16-byte aligned, else one
// cell per thread.  `f(in[5], out[5])` maps one cell.
template <class F>
__device__ __forceinline__ void map_cells(const float* __restrict__ in, float* __restrict__ out,
                                          long long n, F f) {
  const long long t0 = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const long long stride = (long long)gridDim.x * blockDim.x;
  if ((n & 3) == 0 &&
      ((reinterpret_cast<uintptr_t>(in) | reinterpret_cast<uintptr_t>(out)) & 15) == 0) {
    const float4* in4 = reinterpret_cast<const float4*>(in);
    float4* out4 = reinterpret_cast<float4*>(out);
    const long long n4 = n >> 2;
    for (long long i = t0; i < n4; i += stride) {
      float4 v[5], r[5];
#pragma unroll
      for (int k = 0; k < 5; ++k) v[k] = __ldg(in4 + k * n4 + i);
      float a[5], b[5];
#pragma unroll
      for (int k = 0; k < 5; ++k) a[k] = v[k].x;
      f(a, b);
#pragma unroll
      for (int k = 0; k < 5; ++k) r[k].x = b[k], a[k] = v[k].y;
      f(a, b);
#pragma unroll
      for (int k = 0; k < 5; ++k) r[k].y = b[k], a[k] = v[k].z;
      f(a, b);
#pragma unroll
      for (int k = 0; k < 5; ++k) r[k].z = b[k], a[k] = v[k].w;
      f(a, b);
#pragma unroll
      for (int k = 0; k < 5; ++k) {
        r[k].w = b[k];
        out4[k * n4 + i] = r[k];
      }
    }
  } else {
    for (long long i = t0; i < n; i += stride) {
      float a[5], b[5];
#pragma unroll
      for (int k = 0; k < 5; ++k) a[k] = in[k * n + i];
      f(a, b);
#pragma unroll
      for (int k = 0; k < 5; ++k) out[k * n + i] = b[k];
    }
  }
}

__global__ void cons_from_prim_kernel(const float* __restrict__ W, float* __restrict__ U,
                                      long long n, StepConsts<float> k) {
  map_cells(W, U, n, [&](const float w[5], float u[5]) { exact_cons_from_prim(w, u, k); });
}

__global__ void prim_from_cons_kernel(const float* __restrict__ U, float* __restrict__ W,
                                      long long n, StepConsts<float> k) {
  map_cells(U, W, n, [&](const float u[5], float w[5]) { exact_prim_from_cons(u, w, k); });
}

static int elementwise_grid(long long n) {
  long long b = (n + 255) / 256;
  long long cap = (long long)sm_count() * 8;
  return (int)(b < cap ? (b < 1 ? 1 : b) : cap);
}

// ---------------------------------------------------------------------------
// control block
// ---------------------------------------------------------------------------
__global__ void ctl_init_kernel(tf_ctl* ctl, float t_final, float cfl_dx, int max_steps,
                                float t0 = 0.f) {
  ctl->t = t0;
  ctl->dt = 0.f;
  ctl->t_final = t_final;
  ctl->cfl_dx = cfl_dx;
  ctl->ws_bits = 0u;
  ctl->done = 0u;
  ctl->iter = 0;
  ctl->active = 0;
  ctl->max_steps = max_steps;
  ctl->status = TF_OK;
  ctl->max_speed = 0.f;
  for (int i = 0; i < 5; ++i) ctl->reserved[i] = 0;
}

// Condition of the device-side t_final loop (a CUDA graph while node): the
// loop condition the last step left in ctl->active, stopped early when
// float32 t did not advance since the previous evaluation (a stalled loop
// the reference would never leave) or after `cap` steps.  The loop's
// control block carries max_steps = cap, so the step kernels themselves stop
// after exactly `cap` steps; a loop that stopped there short of t_final is
// reported as TF_ERR_TIMEOUT.  Every body iteration runs this kernel once,
// and `cap` evaluations also end the loop, so it is bounded whatever the step
// kernel does.  ctl->reserved[0] counts evaluations, reserved[1] holds the
// bits of t at the previous one.
constexpr int kGraphLoopCap = 1 << 24;
// the step cap of the device-side t_final loops started from now on
// (tf_debug_set_graph_loop_cap lowers it so a test can run into it)
static std::atomic<int> g_graph_loop_cap{kGraphLoopCap};
// the time a tf_time_integration loop starts from: 0 as in the reference
// (time_integration.py:66); tf_debug_set_loop_start_time changes it so a
// test can drive a loop into its float32 stall guard
static std::atomic<float> g_loop_t0{0.f};
// the fused steps of grids under 2^31 cells address with 32-bit offsets from
// per-variable bases; tf_debug_force_64bit_offsets makes them take the 64-bit
// form that larger grids use, so a test can check it on small grids
static std::atomic<bool> g_force_64bit{false};

#ifndef TF_PDL
#define TF_PDL 1
#endif
// Programmatic dependent launch: a step kernel waits for the grid before it
// in the stream to complete (and its writes to be visible) before it reads
// anything, then lets the next step's grid launch as soon as every one of its
// own CTAs has started, so the next launch's latency and CTA setup overlap
// this grid's last wave (6-16% per step on 32^3-128^3 grids, under 1% from
// 256^3 up).  Build with -DTF_PDL=0 for plain stream-ordered launches.
__device__ __forceinline__ void pdl_wait_and_release() {
#if TF_PDL
  asm volatile("griddepcontrol.wait;" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
#endif
}

__global__ void loop_cond_kernel(tf_ctl* ctl, cudaGraphConditionalHandle h, int cap) {
  pdl_wait_and_release();
  const int evals = ctl->reserved[0] + 1;
  const float t = ld_volatile(&ctl->t);
  const float t_prev = __int_as_float(ctl->reserved[1]);
  int active = ld_volatile(&ctl->active);
  if (active && evals > 1 && t == t_prev) {
    ctl->status = TF_ERR_NONFINITE;
    active = 0;
  }
  if (active && evals > cap) {
    ctl->status = TF_ERR_TIMEOUT;
    active = 0;
  }
  if (!active && ctl->status == TF_OK && ld_volatile(&ctl->iter) >= cap &&
      t < ld_volatile(&ctl->t_final))
    ctl->status = TF_ERR_TIMEOUT;
  ctl->active = active;
  ctl->reserved[0] = evals;
  ctl->reserved[1] = __float_as_int(t);
  cudaGraphSetConditional(h, active ? 1u : 0u);
}

// Max wave speed of a primitive state (fluid.py:427-500 in per-cell form);
// the last CTA sets ctl->dt and the loop condition.  `fast` selects the fast
// policy's speed formula (the one its fused epilogue uses) for loops run with
// the fast arithmetic; otherwise the reference's.
__global__ void __launch_bounds__(256) maxspeed_kernel(const float* __restrict__ W, long long n,
                                                       float g, tf_ctl* ctl, int fast) {
  __shared__ float red[8];
  float m = 0.f;
  auto speed = [&](const float w[5]) {
    return fast ? FastPolicy::cell_speed(w, g) : exact_cell_speed(w, g);
  };
  const long long t0 = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const long long stride = (long long)gridDim.x * blockDim.x;
  if ((n & 3) == 0 && (reinterpret_cast<uintptr_t>(W) & 15) == 0) {
    // four cells per thread and variable with 16-byte loads: more bytes in
    // flight per thread (the maximum does not depend on the visiting order)
    const float4* W4 = reinterpret_cast<const float4*>(W);
    const long long n4 = n >> 2;
    for (long long i = t0; i < n4; i += stride) {
      float4 v[5];
#pragma unroll
      for (int k = 0; k < 5; ++k) v[k] = __ldg(W4 + k * n4 + i);
      const float a[5] = {v[0].x, v[1].x, v[2].x, v[3].x, v[4].x};
      const float b[5] = {v[0].y, v[1].y, v[2].y, v[3].y, v[4].y};
      const float c[5] = {v[0].z, v[1].z, v[2].z, v[3].z, v[4].z};
      const float d[5] = {v[0].w, v[1].w, v[2].w, v[3].w, v[4].w};
      m = speed_max(m, speed_max(speed_max(speed(a), speed(b)), speed_max(speed(c), speed(d))));
    }
  } else {
    for (long long i = t0; i < n; i += stride) {
      float w[5];
#pragma unroll
      for (int v = 0; v < 5; ++v) w[v] = __ldg(W + v * n + i);
      m = speed_max(m, speed(w));
    }
  }
  float bm = block_max(m, red);
  if (threadIdx.x == 0) ctl_finish_cta(ctl, bm, gridDim.x, 0.f, false);
}

// Copies the final state of a loop into `out` unless it already is there.
// After `iter` steps the state is in src0 (iter == 0) or buf[iter & 1].
__global__ void final_select_kernel(const tf_ctl* ctl, const float* __restrict__ src0,
                                    const float* buf0, const float* buf1, float* out,
                                    long long n) {
  int iter = ld_volatile(&ctl->iter);
  const float* from = iter == 0 ? src0 : ((iter & 1) ? buf1 : buf0);
  if (from == out) return;
  const float4* f4 = reinterpret_cast<const float4*>(from);
  float4* o4 = reinterpret_cast<float4*>(out);
  long long n4 = n / 4;
  long long i0 = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  long long st = (long long)gridDim.x * blockDim.x;
  bool vec = ((reinterpret_cast<uintptr_t>(from) | reinterpret_cast<uintptr_t>(out)) & 15) == 0;
  if (vec) {
    for (long long i = i0; i < n4; i += st) o4[i] = f4[i];
    for (long long i = n4 * 4 + i0; i < n; i += st) out[i] = from[i];
  } else {
    for (long long i = i0; i < n; i += st) out[i] = from[i];
  }
}

// Diagnostics of a stored primitive state in one pass: sums of the conserved
// variables (fluid.py:30-67 per cell; compensated float32 per thread, float64
// across threads) and the rho / p plane z == z_slice ([2][nx][ny], skipped
// when slice is null).  Blocks stride over (x, y) rows, threads along z, so no
// cell index is divided.
__global__ void __launch_bounds__(256) diagnostics_kernel(const float* __restrict__ W, int nx,
                                                          int ny, int nz, StepConsts<float> k,
                                                          double* totals, float* slice,
                                                          int z_slice) {
  __shared__ double red[8 * 5];
  const long long n = (long long)nx * ny * nz;
  const long long rows = (long long)nx * ny;
  CSum acc[5];
#pragma unroll
  for (int v = 0; v < 5; ++v) acc[v] = CSum{0.f, 0.f};
  auto cell = [&](const float w[5], long long r, int z) {
    float u[5];
    exact_cons_from_prim(w, u, k);
#pragma unroll
    for (int v = 0; v < 5; ++v) csum_add(acc[v], u[v]);
    if (slice && z == z_slice) {
      slice[r] = w[0];
      slice[rows + r] = w[4];
    }
  };
  if ((nz & 3) == 0 && (reinterpret_cast<uintptr_t>(W) & 15) == 0) {
    // four cells of a row per thread with 16-byte loads
    const int nz4 = nz >> 2;
    for (long long r = blockIdx.x; r < rows; r += gridDim.x) {
      const float4* row = reinterpret_cast<const float4*>(W + r * nz);
      const long long n4 = n >> 2;
      for (int z4 = threadIdx.x; z4 < nz4; z4 += blockDim.x) {
        float4 q[5];
#pragma unroll
        for (int v = 0; v < 5; ++v) q[v] = __ldg(row + v * n4 + z4);
        const float a[5] = {q[0].x, q[1].x, q[2].x, q[3].x, q[4].x};
        const float b[5] = {q[0].y, q[1].y, q[2].y, q[3].y, q[4].y};
        const float c[5] = {q[0].z, q[1].z, q[2].z, q[3].z, q[4].z};
        const float d[5] = {q[0].w, q[1].w, q[2].w, q[3].w, q[4].w};
        cell(a, r, 4 * z4);
        cell(b, r, 4 * z4 + 1);
        cell(c, r, 4 * z4 + 2);
        cell(d, r, 4 * z4 + 3);
      }
    }
  } else {
    for (long long r = blockIdx.x; r < rows; r += gridDim.x) {
      const float* row = W + r * nz;
      for (int z = threadIdx.x; z < nz; z += blockDim.x) {
        float w[5];
#pragma unroll
        for (int v = 0; v < 5; ++v) w[v] = __ldg(row + v * n + z);
        cell(w, r, z);
      }
    }
  }
  block_add_totals(acc, red, totals);
}

// ---------------------------------------------------------------------------
// fused step
// ---------------------------------------------------------------------------
struct FusedArgs {
  // The buffers of this launch.  A run loop passes, per launch, the source
  // and destination of that step (the ping-pong parity is known on the host),
  // so the kernel's addresses derive from launch arguments only and are the
  // same for every thread of a CTA.
  const float* src;
  float* dst;
  VarPtrs vp;  // per-variable bases of src and dst (set by launch_fused)
  FusedGeom geo;
  float gamma, inv_dx, gm1, igm1;
  float dt_host;
  const float* dt_dev;
  float fixed_dt;  // loop mode: > 0 replaces ctl->dt
  tf_ctl* ctl;     // fixed mode: optional; loop mode: required
  int loop;        // 1: a step of a run loop (predicated on ctl->active, dt from ctl)
  double* totals;  // diagnostics instantiation: conserved totals (zeroed before)
  DiagArgs diag;   // diagnostics instantiation: optional slice
  int conserved_io;  // fast policy on conserved input and output (16-row tiles)
  int layout;        // 0: x-marching tile (fused_tile), 1: y-marching tile (fused_tile_ym)
};

// dt of a launch: a loop step reads the loop's dt (or its fixed dt) and runs
// only while the loop is active; a single step takes the caller's dt.
__device__ __forceinline__ bool launch_dt(const FusedArgs& a, float* dt) {
  if (a.loop) {
    if (!ld_volatile(&a.ctl->active)) return false;
    *dt = a.fixed_dt > 0.f ? a.fixed_dt : ld_volatile(&a.ctl->dt);
  } else {
    *dt = a.dt_dev ? *a.dt_dev : a.dt_host;
  }
  return true;
}

__device__ __forceinline__ StepConsts<float> launch_consts(const FusedArgs& a, float dt) {
  StepConsts<float> K;
  K.g = a.gamma;
  K.gm1 = a.gm1;
  K.igm1 = a.igm1;
  K.inv_dx = a.inv_dx;
  K.dt = dt;
  K.k = dt * a.inv_dx;
  return K;
}

// VP: per-variable bases from the launch parameters and 32-bit element
// offsets (grids of fewer than 2^31 cells; the fast arithmetic's plain step).
template <class P, int NWP, bool DIAG = false, bool VP = false>
__global__ void TF_FUSED_BOUNDS(NWP) fused_step_kernel(const __grid_constant__ FusedArgs a) {
  __shared__ FusedSmem<NWP> sm;
  __shared__ double dred[DIAG ? NWP * 5 : 1];
  pdl_wait_and_release();
  float dt;
  if (!launch_dt(a, &dt)) return;
  const StepConsts<float> K = launch_consts(a, dt);
  CSum acc[5];
  float m = fused_tile<P, NWP, false, DIAG, VP && !DIAG && !P::kExact>(a.src, a.dst, a.geo, blockIdx.x, blockIdx.y,
                                                blockIdx.z, K, sm, a.diag, acc, &a.vp);
  if constexpr (DIAG) block_add_totals(acc, dred, a.totals);
  if (a.ctl) {
    float bm = block_max(m, sm.red);
    if (threadIdx.x == 0)
      ctl_finish_cta(a.ctl, bm, gridDim.x * gridDim.y * gridDim.z, dt, a.loop != 0);
  }
}

// The y-marching fused step (fused_tile_ym): NW x rows per CTA, grid
// (x tiles, z tiles, y chunks).
template <class P, int NW, bool DIAG = false, bool VP = false, int VEC = 0>
__global__ void __launch_bounds__(NW * 32, min_ctas_per_sm(NW))
    fused_step_ym_kernel(const __grid_constant__ FusedArgs a) {
  extern __shared__ __align__(16) unsigned char ym_smem[];
  YmSmem<NW>& sm = *reinterpret_cast<YmSmem<NW>*>(ym_smem);
  __shared__ double dred[DIAG ? NW * 5 : 1];
  pdl_wait_and_release();
  float dt;
  if (!launch_dt(a, &dt)) return;
  const StepConsts<float> K = launch_consts(a, dt);
  CSum acc[5];
  float m = fused_tile_ym<P, NW, DIAG, VP, VEC>(a.src, a.dst, a.geo, blockIdx.x, blockIdx.y,
                                                blockIdx.z, K, sm, a.diag, acc, &a.vp);
  if constexpr (DIAG) block_add_totals(acc, dred, a.totals);
  if (a.ctl) {
    float bm = block_max(m, sm.red);
    if (threadIdx.x == 0)
      ctl_finish_cta(a.ctl, bm, gridDim.x * gridDim.y * gridDim.z, dt, a.loop != 0);
  }
}

// The fused step with TMA-staged planes (fused_tile_tma); the tensor map
// describes a.src.
template <class P, int NWP>
__global__ void TF_FUSED_BOUNDS(NWP)
    fused_step_tma_kernel(FusedArgs a, const __grid_constant__ CUtensorMap tm_src) {
  __shared__ FusedSmem<NWP> sm;
  __shared__ __align__(8) unsigned long long bars[kStages];
  extern __shared__ unsigned char dyn_smem[];
  float* stages = reinterpret_cast<float*>(
      (reinterpret_cast<uintptr_t>(dyn_smem) + 127) & ~static_cast<uintptr_t>(127));
  float dt;
  if (!launch_dt(a, &dt)) return;
  const StepConsts<float> K = launch_consts(a, dt);
  bool timed_out = false;
  float m = fused_tile_tma<P, NWP>(a.src, a.dst, &tm_src, a.geo, blockIdx.x, blockIdx.y,
                                   blockIdx.z, K, sm, stages, bars, &timed_out);
  if (a.ctl) {
    float bm = block_max(m, sm.red);
    if (threadIdx.x == 0) {
      if (timed_out) atomicExch(&a.ctl->status, TF_ERR_TIMEOUT);
      ctl_finish_cta(a.ctl, bm, gridDim.x * gridDim.y * gridDim.z, dt, a.loop != 0);
    }
  }
}

// cuTensorMapEncodeTiled, fetched from the driver through the runtime so
// that the library does not link libcuda.
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                  const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                  const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_tiled() {
  static std::once_flag once;
  static EncodeTiledFn fn = nullptr;
  std::call_once(once, []() {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
  });
  return fn;
}

// A [5][nx][ny][nz] float state as a 4D tensor (z, y, x, var) with the tile
// box (kBoxZ, rows, 1, 5); false if the encoder rejects it.
static bool make_state_tmap(CUtensorMap* m, const float* base, int nx, int ny, int nz, int rows) {
  EncodeTiledFn fn = encode_tiled();
  if (!fn) return false;
  cuuint64_t dims[4] = {(cuuint64_t)nz, (cuuint64_t)ny, (cuuint64_t)nx, 5};
  cuuint64_t strides[3] = {(cuuint64_t)nz * 4, (cuuint64_t)ny * nz * 4,
                           (cuuint64_t)nx * ny * nz * 4};
  cuuint32_t box[4] = {(cuuint32_t)kBoxZ, (cuuint32_t)rows, 1, 5};
  cuuint32_t es[4] = {1, 1, 1, 1};
  return fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, const_cast<float*>(base), dims, strides, box,
            es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
            CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

static bool tma_usable(const FusedArgs& a, int rows) {
  if (rows != 8 && rows != 16 && rows != 32) return false;
  if (a.geo.nz % 4 != 0) return false;  // tensor strides must be multiples of 16 bytes
  if ((reinterpret_cast<uintptr_t>(a.src) | reinterpret_cast<uintptr_t>(a.dst)) & 15) return false;
  return encode_tiled() != nullptr;
}

static int check_dims(int nx, int ny, int nz, unsigned flags) {
  if (nx < 1 || ny < 1 || nz < 1)
    return set_error(TF_ERR_ARG, "grid dims must be >= 1 (got %d,%d,%d)", nx, ny, nz);
  if ((flags & TF_FLAG_OPEN_BOUNDARIES) && (nx < 2 || ny < 2 || nz < 2))
    return set_error(TF_ERR_ARG, "open boundaries need >= 2 cells per axis (fluid.py:349,374)");
  if ((long long)nx * ny * nz > (1LL << 40))
    return set_error(TF_ERR_ARG, "grid too large");
  return TF_OK;
}

static int check_scalars(float dx, float gamma) {
  if (!(dx > 0.f) || !isfinite(dx)) return set_error(TF_ERR_ARG, "dx must be finite and > 0");
  if (!isfinite(gamma) || gamma == 1.f) return set_error(TF_ERR_ARG, "gamma must be finite and != 1");
  return TF_OK;
}

// Tile grid of a fused step.  layout 0 (x-marching): tiles_z x tiles_y tiles
// of 30 x (rows-2) stored cells, marching along x in chunks of lx planes.
// layout 1 (y-marching): tiles_x x tiles_z tiles of rows/2 x rows and 62 z
// cells, marching along y in chunks of lx planes (tiles_y chunks); the chunk
// rule is the same with the axes' roles exchanged.
static FusedGeom make_geom(int nx, int ny, int nz, unsigned flags, int rows, int lx,
                           int layout = 0) {
  FusedGeom g;
  g.nx = nx;
  g.ny = ny;
  g.nz = nz;
  g.open_bc = (flags & TF_FLAG_OPEN_BOUNDARIES) ? 1 : 0;
  if (layout == 1) {
    const int nw = rows / 2;
    g.tiles_x = (nx + nw - 1) / nw;
    g.tiles_z = (nz + kYmZ - 1) / kYmZ;
    if (lx <= 0) {
      const long long tiles_xz = (long long)g.tiles_x * g.tiles_z;
      const long long resident = (long long)sm_count() * min_ctas_per_sm(nw);
      long long min_planes;
      if (tiles_xz * (ny / 16) >= resident) {
        min_planes = 16;
      } else if (tiles_xz * (ny / 8) >= resident) {
        min_planes = 8;
      } else {
        min_planes = (ny * tiles_xz + resident - 1) / resident;
        if (min_planes < 2) min_planes = 2;
      }
      // about 9 waves, and chunks of at most 64 planes (measured at 512^3 to
      // 1024^3: 32-64 planes beat longer chunks by 2-7%)
      long long ty = (9 * resident + tiles_xz - 1) / tiles_xz;
      if (ty < (ny + 63) / 64) ty = (ny + 63) / 64;
      long long max_ty = ny / min_planes > 0 ? ny / min_planes : 1;
      if (ty > max_ty) ty = max_ty;
      if (ty < 1) ty = 1;
      lx = (int)((ny + ty - 1) / ty);
    }
    if (lx > ny) lx = ny;
    g.lx = lx;
    g.tiles_y = (ny + lx - 1) / lx;
    return g;
  }
  g.tiles_z = (nz + kTileZ - 1) / kTileZ;
  g.tiles_y = (ny + (rows - 2) - 1) / (rows - 2);
  if (lx <= 0) {
    // About 9 waves of resident CTAs, in chunks of >= 32 planes where those
    // still make 1.5 waves, else >= 16 planes (each chunk re-reads one plane
    // and warms up its carry); grids too small for one wave at 16 planes take
    // 8-plane chunks, and grids too small for one wave even then are
    // latency-bound and take the chunk length that makes one wave, but at
    // least 2 planes.  Measured on GB300 (shear layer, 16-row tiles, chunk
    // length: Gcell-updates/s): 160^3 16: 58.5, 32: 50.6; 192^3 16: 66.2, 32:
    // 68.6; 256^3 16: 73.0, 32: 75.6; the reference's benchmark states: 32^3
    // -> 2 planes, 64^3 -> 4, 96^3 -> 8, 128^3 -> 16, 512^3 -> 103.
    const long long tiles_yz = (long long)g.tiles_z * g.tiles_y;
    const long long resident = (long long)sm_count() * min_ctas_per_sm(rows / 2);
    long long min_planes;
    if (2 * tiles_yz * (nx / 32) >= 3 * resident) {
      min_planes = 32;
    } else if (tiles_yz * (nx / 16) >= resident) {
      min_planes = 16;
    } else if (tiles_yz * (nx / 8) >= resident) {
      min_planes = 8;
    } else {
      min_planes = (nx * tiles_yz + resident - 1) / resident;
      if (min_planes < 2) min_planes = 2;
    }
    long long tx = (9 * resident + tiles_yz - 1) / tiles_yz;
    long long max_tx = nx / min_planes > 0 ? nx / min_planes : 1;
    if (tx > max_tx) tx = max_tx;
    if (tx < 1) tx = 1;
    lx = (int)((nx + tx - 1) / tx);
  }
  if (lx > nx) lx = nx;
  g.lx = lx;
  g.tiles_x = (nx + lx - 1) / lx;
  return g;
}

// Cells a layout computes per stored cell for a grid (ring and ragged
// tiles): the x-marching 16-row tile stores 30 x 14 of 32 x 16 cells; the
// y-marching 8-row tile stores 60 of 64 z cells and derives two halo rows per
// 4 rows (about 7.8% more arithmetic, from the FP32 pipe counters).
static double overlap_xmarch(int ny, int nz) {
  const double y = (double)((ny + 13) / 14) * 16 / ny;
  const double z = (double)((nz + kTileZ - 1) / kTileZ) * kTileLanes / nz;
  return y * z;
}
static double overlap_ymarch(int nz) {
  return (double)((nz + kYmZ - 1) / kYmZ) * 64 / nz * 1.078;
}

// The tile of a fused step.  With no tile given, the fast and diagnostics
// steps on a periodic grid with an even nz and at least 4 x rows take the
// y-marching 8-row tile when it computes no more cells than the x-marching
// 16-row tile, else the x-marching tile: 8 rows for grids of at most 128^3
// cells, 16 rows above (two CTAs per SM interleave their barrier phases).  Measured on GB300 (shear layer, Gcell-updates/s,
// x-marching / y-marching): 128^3 46.4 / 42.3, 192^3 66.2 / 63.7, 256^3
// 72.8 / 73.7, 320^3 80.5 / 80.2, 384^3 81.6 / 84.6, 448^3 87.6 / 87.0,
// 512^3 83.7 / 89.3, 640^3 86.7 / 89.9, 768^3 87.6 / 91.9, 1024^3 84.9 /
// 85.6; the rule picks the faster one except at the near-ties 256^3 and
// 320^3.  loader 3 selects the y-marching tile explicitly.
static int resolve_tile(const tf_tile_config* tile, int nx, int ny, int nz, unsigned flags,
                        int* rows, int* lx, int* loader) {
  *rows = 16;
  *lx = 0;
  *loader = 0;
  if (tile) {
    if (!valid_tile_rows(tile->rows))
      return set_error(TF_ERR_ARG, "tile rows must be 8, 16 or 32 (got %d)", tile->rows);
    *rows = tile->rows;
    *lx = tile->lx;
    if (*lx < 0) return set_error(TF_ERR_ARG, "tile lx must be >= 0");
    if (tile->loader < 0 || tile->loader > 3)
      return set_error(TF_ERR_ARG,
                       "tile loader must be 0 (auto), 1 (loads), 2 (TMA) or 3 (y-marching)");
    if (tile->loader == 3 && tile->rows == 32)
      return set_error(TF_ERR_ARG, "the y-marching tile takes 8 or 16 rows");
    *loader = tile->loader;
    return TF_OK;
  }
  // the y-marching tile from 2^17 cells up: below, a step is a few
  // microseconds of latency and the x-marching tile's shorter chains win
  // (32^3 4.9 vs 4.5, 48^3 13.7 vs 13.2 Gcell-updates/s); with open
  // boundaries (its 8-byte pairs fixed up at the z edges) from 2^27 cells
  // (512^3 87.5 vs 84.3, 768^3 88.7 vs 88.1; 384^3 79.4 vs 82.3)
  const long long cells = (long long)nx * ny * nz;
  const bool open = (flags & TF_FLAG_OPEN_BOUNDARIES) != 0;
  const bool fit =
      !(flags & TF_FLAG_EXACT) && (nz & 1) == 0 && nx >= 4 && cells >= (1LL << 17) &&
      (!open || (cells >= (1LL << 27) && nz >= 4 &&
                 !(flags & (TF_FLAG_IN_CONSERVED | TF_FLAG_OUT_CONSERVED))));
  if (fit && overlap_xmarch(ny, nz) >= overlap_ymarch(nz)) {
    *rows = 8;
    *loader = 3;
  } else if ((long long)nx * ny * nz <= (1LL << 21) &&
             !(flags & (TF_FLAG_IN_CONSERVED | TF_FLAG_OUT_CONSERVED))) {
    // grids of at most 128^3 cells: 8-row x-marching tiles (four CTAs per SM
    // fill the GPU better; measured 96^3 34.6 vs 34.0, 128^3 49.0 vs 47.4
    // Gcell-updates/s against 16 rows, equal below); the conserved-state step
    // keeps its 16-row tile
    *rows = 8;
  }
  return TF_OK;
}

template <int NWP>
static int launch_tma(const FusedArgs& a, dim3 grid, const CUtensorMap& tm, bool exact,
                      cudaStream_t s) {
  const size_t smem = tma_smem_bytes(NWP) + 128;
  auto k = exact ? fused_step_tma_kernel<ExactPair, NWP> : fused_step_tma_kernel<FastPair, NWP>;
  TF_TRY(cuda_check(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem),
                    "cudaFuncSetAttribute"));
  k<<<grid, NWP * 32, smem, s>>>(a, tm);
  return TF_OK;
}

// Launches a step (or loop condition) kernel; with TF_PDL, as a programmatic
// dependent of the work before it in the stream (the kernel waits for that
// work itself).
template <class... KArgs, class... Args>
static void launch_step(void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem,
                        cudaStream_t s, Args... args) {
#if TF_PDL
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, kern, args...);
#else
  kern<<<grid, block, smem, s>>>(args...);
#endif
}

// Template arguments of one y-marching kernel instantiation.
template <class P_, int NW_, bool DIAG_, bool VP_, int VEC_ = 0>
struct YmTag {
  using P = P_;
  static constexpr int nw = NW_;
  static constexpr bool diag = DIAG_, vp = VP_;
  static constexpr int vec = VEC_;
};

// Dynamic shared memory of the y-marching kernel with NW warps.
static size_t ym_smem_bytes(int nw) {
  return nw == 4 ? sizeof(YmSmem<4>) : sizeof(YmSmem<8>);
}

// Raises a kernel's dynamic shared-memory limit once per device (the flag
// is per kernel instantiation: Tag is the kernel's template arguments).
template <class Tag, class Kern>
static int ym_smem_attr(Kern kern, size_t bytes) {
  static std::atomic<unsigned long long> done{0};
  int dev = 0;
  TF_TRY(cuda_check(cudaGetDevice(&dev), "cudaGetDevice"));
  const unsigned long long bit = 1ull << (dev & 63);
  if (done.load() & bit) return TF_OK;
  TF_TRY(cuda_check(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)bytes),
                    "cudaFuncSetAttribute"));
  done.fetch_or(bit);
  return TF_OK;
}

// Launches one fused step.  loader: 0 auto, 1 per-thread loads, 2 TMA-staged
// planes (falls back to loads when not usable).  Auto takes the per-thread
// loads: on GB300 at 256^3-512^3 they measured faster (80 vs 64 Gcell/s at
// 512^3 with 16-row tiles).
static int launch_fused(const FusedArgs& a_in, int rows, bool exact, cudaStream_t s,
                        int loader = 1) {
  if (a_in.geo.tiles_y > 65535 || a_in.geo.tiles_x > 65535)
    return set_error(TF_ERR_ARG, "grid too large for the tile grid");
  FusedArgs a = a_in;
  const size_t vs = (size_t)a.geo.nx * a.geo.ny * a.geo.nz;
  for (int i = 0; i < 5; ++i) {
    a.vp.s[i] = a.src + i * vs;
    a.vp.d[i] = a.dst ? a.dst + i * vs : nullptr;
  }
  if (a.layout == 1) {
    if (a.geo.tiles_z > 65535) return set_error(TF_ERR_ARG, "grid too large for the tile grid");
    a.geo.pairs8 = ((reinterpret_cast<uintptr_t>(a.src) | reinterpret_cast<uintptr_t>(a.dst)) &
                    7) == 0 && (vs & 1) == 0 && (a.geo.nz & 1) == 0;
    const dim3 g(a.geo.tiles_x, a.geo.tiles_z, a.geo.tiles_y);
    const bool vp = vs < (1ull << 31) && !g_force_64bit.load();
    // 8-byte pair accesses: periodic wrap keeps every pair whole when nz is
    // even; with open boundaries the fast step fixes up the two pairs the
    // clamp changes (nz >= 4)
    const bool vec = a.geo.pairs8 && !a.geo.open_bc;
    const bool vec_open = a.geo.pairs8 && a.geo.open_bc && a.geo.nz >= 4;
    int st = TF_OK;
    auto go = [&](auto nw_c) {
      constexpr int NW = decltype(nw_c)::value;
      auto launch = [&](auto tag) {
        using T = decltype(tag);
        auto kern = fused_step_ym_kernel<typename T::P, NW, T::diag, T::vp, T::vec>;
        const size_t smem = ym_smem_bytes(NW);
        st = ym_smem_attr<T>(kern, smem);
        if (st == TF_OK) launch_step(kern, g, dim3(NW * 32), smem, s, a);
      };
      if (a.totals) {
        if (exact) launch(YmTag<ExactPair, NW, true, false>{});
        else launch(YmTag<FastPair, NW, true, false>{});
      } else if (a.conserved_io) {
        if (vp && vec) launch(YmTag<FastPairConserved, NW, false, true, 1>{});
        else if (vp) launch(YmTag<FastPairConserved, NW, false, true>{});
        else launch(YmTag<FastPairConserved, NW, false, false>{});
      } else if (exact) {
        launch(YmTag<ExactPair, NW, false, false>{});
      } else if (vp && vec) {
        launch(YmTag<FastPair, NW, false, true, 1>{});
      } else if (vp && vec_open) {
        launch(YmTag<FastPair, NW, false, true, 2>{});
      } else if (vp) {
        launch(YmTag<FastPair, NW, false, true>{});
      } else if (vec) {
        launch(YmTag<FastPair, NW, false, false, 1>{});
      } else {
        launch(YmTag<FastPair, NW, false, false>{});
      }
    };
    if (rows == 8) go(std::integral_constant<int, 4>{});
    else if (rows == 16) go(std::integral_constant<int, 8>{});
    else return set_error(TF_ERR_ARG, "the y-marching tile takes 8 or 16 rows");
    TF_TRY(st);
    return launch_check("fused_step_ym_kernel");
  }
  dim3 grid(a.geo.tiles_z, a.geo.tiles_y, a.geo.tiles_x);
  if (loader == 2 && tma_usable(a, rows)) {
    CUtensorMap tm;
    if (make_state_tmap(&tm, a.src, a.geo.nx, a.geo.ny, a.geo.nz, rows)) {
      TF_DISPATCH_ROWS(rows, NWP, TF_TRY((launch_tma<NWP>(a, grid, tm, exact, s))));
      return launch_check("fused_step_tma_kernel");
    }
  }
  if (a.totals) {
    TF_DISPATCH_ROWS(rows, NWP, {
      if (exact)
        launch_step(fused_step_kernel<ExactPair, NWP, true>, grid, dim3(NWP * 32), 0, s, a);
      else
        launch_step(fused_step_kernel<FastPair, NWP, true>, grid, dim3(NWP * 32), 0, s, a);
    });
    return launch_check("fused_step_kernel (diagnostics)");
  }
  if (a.conserved_io) {
    if (exact || rows != 16)
      return set_error(TF_ERR_UNSUPPORTED,
                       "conserved input/output: fast arithmetic and 16-row tiles only");
    if (vs < (1ull << 31) && !g_force_64bit.load())
      launch_step(fused_step_kernel<FastPairConserved, 8, false, true>, grid, dim3(8 * 32), 0, s,
                  a);
    else
      launch_step(fused_step_kernel<FastPairConserved, 8>, grid, dim3(8 * 32), 0, s, a);
    return launch_check("fused_step_kernel (conserved)");
  }
  const bool vp32 = vs < (1ull << 31) && !g_force_64bit.load();
  TF_DISPATCH_ROWS(rows, NWP, {
    if (exact) launch_step(fused_step_kernel<ExactPair, NWP>, grid, dim3(NWP * 32), 0, s, a);
    else if (vp32)
      launch_step(fused_step_kernel<FastPair, NWP, false, true>, grid, dim3(NWP * 32), 0, s, a);
    else launch_step(fused_step_kernel<FastPair, NWP>, grid, dim3(NWP * 32), 0, s, a);
  });
  return launch_check("fused_step_kernel");
}

// The buffers of a run loop.  Step i (1-based) reads `in` for i == 1, else
// buf[(i - 1) & 1], and writes buf[i & 1]; after n steps the state is in
// `in` (n == 0) or buf[n & 1].
struct LoopBufs {
  const float* in;
  float* buf[2];
};

static FusedArgs step_args(FusedArgs a, const LoopBufs& b, long long i) {
  a.src = i == 1 ? b.in : b.buf[(i - 1) & 1];
  a.dst = b.buf[i & 1];
  return a;
}

// The t_final loop as a CUDA graph: {condition, step 1, condition} and then a
// while node whose body is an even number of steps and one condition, so
// every step launch carries its own buffers.  Each step is predicated on the
// loop condition the previous step's last CTA (or the condition kernel) left
// in the control block, so the steps of the last body past the end of the
// loop only launch and exit.  Small grids take 8 steps per body: the
// per-iteration cost of the while node and the condition kernel (~3 us)
// then falls on every eighth step instead of every second.  The kernel arguments bake in the buffers and scalars,
// so executable graphs are cached by (device, arguments, buffers, tile): a
// repeated call on the same buffers launches the cached graph.  An evicted
// graph is destroyed at once; CUDA frees it after any in-flight launch
// completes.
struct GraphKey {
  int device, rows, exact, cap;
  FusedArgs a;  // with src / dst cleared; zero-initialised, so padding compares equal
  LoopBufs b;
};
struct GraphEntry {
  GraphKey key;
  cudaGraphExec_t exec;
};
static std::mutex g_graph_mu;
static std::vector<GraphEntry> g_graphs;  // most recently used last
constexpr size_t kGraphCacheSize = 8;

static int build_graph_loop(const FusedArgs& a, const LoopBufs& b, int rows, bool exact,
                            tf_ctl* ctl, int cap, cudaGraphExec_t* out);

// steps per while-node body of a t_final loop graph (even)
static int body_steps(const FusedGeom& g) {
  return (long long)g.nx * g.ny * g.nz <= (1LL << 22) ? 8 : 2;
}

static int graph_loop(const FusedArgs& a, const LoopBufs& b, int rows, bool exact, tf_ctl* ctl,
                      int cap, cudaStream_t s) {
  GraphKey k;
  memset(&k, 0, sizeof k);
  TF_TRY(cuda_check(cudaGetDevice(&k.device), "cudaGetDevice"));
  k.rows = rows;
  k.exact = exact ? 1 : 0;
  k.cap = cap;
  k.a = a;
  k.a.src = nullptr;
  k.a.dst = nullptr;
  k.b = b;
  std::lock_guard<std::mutex> lk(g_graph_mu);
  for (size_t i = 0; i < g_graphs.size(); ++i) {
    if (memcmp(&g_graphs[i].key, &k, sizeof k) == 0) {
      GraphEntry e = g_graphs[i];
      g_graphs.erase(g_graphs.begin() + i);
      g_graphs.push_back(e);
      return cuda_check(cudaGraphLaunch(e.exec, s), "cudaGraphLaunch");
    }
  }
  cudaGraphExec_t exec = nullptr;
  TF_TRY(build_graph_loop(a, b, rows, exact, ctl, k.cap, &exec));
  int st = cuda_check(cudaGraphLaunch(exec, s), "cudaGraphLaunch");
  if (st != TF_OK) {
    cudaGraphExecDestroy(exec);
    return st;
  }
  if (g_graphs.size() >= kGraphCacheSize) {
    cudaGraphExecDestroy(g_graphs.front().exec);
    g_graphs.erase(g_graphs.begin());
  }
  g_graphs.push_back(GraphEntry{k, exec});
  return TF_OK;
}

static int build_graph_loop(const FusedArgs& a, const LoopBufs& b, int rows, bool exact,
                            tf_ctl* ctl, int cap, cudaGraphExec_t* out) {
  cudaGraph_t g = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaStream_t cs = nullptr;
  int st = TF_OK;
  bool capturing = false;
  auto fail = [&](cudaError_t e, const char* what) {
    if (st == TF_OK && e != cudaSuccess) st = cuda_check(e, what);
    return st != TF_OK;
  };
  auto end_capture = [&]() {
    cudaGraph_t captured = nullptr;
    cudaError_t ce = cudaStreamEndCapture(cs, &captured);
    capturing = false;
    return ce;
  };
  do {
    if (fail(cudaGraphCreate(&g, 0), "cudaGraphCreate")) break;
    cudaGraphConditionalHandle h;
    if (fail(cudaGraphConditionalHandleCreate(&h, g, 0, 0), "cudaGraphConditionalHandleCreate"))
      break;
    if (fail(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking), "cudaStreamCreate")) break;
    // prologue: condition (t_final may already be reached), step 1, condition
    if (fail(cudaStreamBeginCaptureToGraph(cs, g, nullptr, nullptr, 0,
                                           cudaStreamCaptureModeThreadLocal),
             "cudaStreamBeginCaptureToGraph"))
      break;
    capturing = true;
    launch_step(loop_cond_kernel, dim3(1), dim3(1), 0, cs, ctl, h, cap);
    int lst = launch_check("loop_cond_kernel");
    if (lst == TF_OK) lst = launch_fused(step_args(a, b, 1), rows, exact, cs, 1);
    if (lst == TF_OK) {
      launch_step(loop_cond_kernel, dim3(1), dim3(1), 0, cs, ctl, h, cap);
      lst = launch_check("loop_cond_kernel");
    }
    if (lst != TF_OK) {
      st = lst;
      break;
    }
    // the while node after the prologue
    cudaStreamCaptureStatus cst;
    cudaGraph_t cg = nullptr;
    const cudaGraphNode_t* deps = nullptr;
    size_t ndeps = 0;
    if (fail(cudaStreamGetCaptureInfo(cs, &cst, nullptr, &cg, &deps, nullptr, &ndeps),
             "cudaStreamGetCaptureInfo"))
      break;
    cudaGraphNodeParams np = {cudaGraphNodeTypeConditional};  // other members zero
    np.conditional.handle = h;
    np.conditional.type = cudaGraphCondTypeWhile;
    np.conditional.size = 1;
    cudaGraphNode_t loop;
    if (fail(cudaGraphAddNode(&loop, cg, deps, nullptr, ndeps, &np), "cudaGraphAddNode(while)"))
      break;
    if (fail(cudaStreamUpdateCaptureDependencies(cs, &loop, nullptr, 1,
                                                 cudaStreamSetCaptureDependencies),
             "cudaStreamUpdateCaptureDependencies"))
      break;
    if (fail(end_capture(), "cudaStreamEndCapture")) break;
    // the body: steps 2k .. 2k + m - 1, then the condition
    cudaGraph_t body = np.conditional.phGraph_out[0];
    if (fail(cudaStreamBeginCaptureToGraph(cs, body, nullptr, nullptr, 0,
                                           cudaStreamCaptureModeThreadLocal),
             "cudaStreamBeginCaptureToGraph(body)"))
      break;
    capturing = true;
    const int m = body_steps(a.geo);
    for (int i = 2; i <= 1 + m && lst == TF_OK; ++i)
      lst = launch_fused(step_args(a, b, i), rows, exact, cs, 1);
    if (lst == TF_OK) {
      launch_step(loop_cond_kernel, dim3(1), dim3(1), 0, cs, ctl, h, cap);
      lst = launch_check("loop_cond_kernel");
    }
    if (lst != TF_OK) {
      st = lst;
      break;
    }
    if (fail(end_capture(), "cudaStreamEndCapture(body)")) break;
    if (fail(cudaGraphInstantiate(&exec, g, 0), "cudaGraphInstantiate")) break;
  } while (false);
  if (capturing) end_capture();
  if (cs) cudaStreamDestroy(cs);
  if (g) cudaGraphDestroy(g);
  if (st != TF_OK && exec) {
    cudaGraphExecDestroy(exec);
    exec = nullptr;
  }
  *out = exec;
  return st;
}

static FusedArgs make_fused_args(const float* src, float* dst, const FusedGeom& geo, float dx,
                                 float gamma) {
  FusedArgs a;
  memset(&a, 0, sizeof a);
  a.src = src;
  a.dst = dst;
  a.geo = geo;
  StepConsts<float> k = make_consts<float>(gamma, dx, 0.f);
  a.gamma = k.g;
  a.gm1 = k.gm1;
  a.igm1 = k.igm1;
  a.inv_dx = k.inv_dx;
  return a;
}

// ---------------------------------------------------------------------------
// per-axis sweep (one thread per cell, both faces recomputed): the
// reference's structure, used to cross-check the fused kernel and by the
// adjoint's forward recomputation.
// ---------------------------------------------------------------------------
template <class P, int VEL>
__global__ void __launch_bounds__(256) sweep_kernel(const float* __restrict__ src,
                                                    float* __restrict__ dst, int nx, int ny,
                                                    int nz, int open_bc, int in_prim,
                                                    int out_prim, StepConsts<float> K) {
  const long long n = (long long)nx * ny * nz;
  const bool open = open_bc != 0;
  for_each_cell(nx, ny, nz, [&](long long i, int x, int y, int z) {
    Cell<float> c[3];
#pragma unroll
    for (int d = -1; d <= 1; ++d) {
      int xx = x, yy = y, zz = z;
      if (VEL == 1) xx += d;
      if (VEL == 2) yy += d;
      if (VEL == 3) zz += d;
      long long j = ((long long)src_index(xx, nx, open) * ny + src_index(yy, ny, open)) * nz +
                    src_index(zz, nz, open);
      float w[5];
#pragma unroll
      for (int v = 0; v < 5; ++v) w[v] = __ldg(src + v * n + j);
      if (in_prim) P::template derive_in<VEL>(w, c[d + 1], K);
      else P::template derive<VEL>(w, c[d + 1], K);
    }
    float flo[5], fhi[5], s[5], o[5];
    P::hll(c[0], c[1], flo);
    P::hll(c[1], c[2], fhi);
    P::update(c[1], flo, fhi, s, K);
    if (out_prim) P::to_prim(s, o, K);
    else {
#pragma unroll
      for (int v = 0; v < 5; ++v) o[v] = s[v];
    }
#pragma unroll
    for (int v = 0; v < 5; ++v) dst[v * n + i] = o[v];
  });
}

// Per-axis sweep along x or y (VEL 1 or 2) that marches: a thread owns one
// (other in-plane coordinate, z) column and walks a chunk of the sweep axis,
// keeping the previous cell's quantities and the flux of the face behind it,
// so each cell is loaded and derived once and each face is solved once.  The
// operations on every face and cell are those of sweep_kernel, so the result
// is the same bits.  z stays with sweep_kernel (a z march would not coalesce).
template <class P, int VEL>
__global__ void __launch_bounds__(256) march_sweep_kernel(const float* __restrict__ src,
                                                          float* __restrict__ dst, int nx, int ny,
                                                          int nz, int chunk, int open_bc,
                                                          int in_prim, int out_prim,
                                                          StepConsts<float> K) {
  static_assert(VEL == 1 || VEL == 2, "x or y sweeps only");
  const long long n = (long long)nx * ny * nz;
  const bool open = open_bc != 0;
  const int z = blockIdx.x * blockDim.x + threadIdx.x;
  if (z >= nz) return;
  const int o = blockIdx.y;                        // y for an x sweep, x for a y sweep
  const int na = VEL == 1 ? nx : ny;               // length of the sweep axis
  const int a0 = blockIdx.z * chunk, a_end = min(a0 + chunk, na);
  const int zs = src_index(z, nz, open);
  const int os = src_index(o, VEL == 1 ? ny : nx, open);
  auto index = [&](int a) {  // linear index of cell a of this column
    return VEL == 1 ? ((long long)a * ny + o) * nz + z : ((long long)o * ny + a) * nz + z;
  };
  auto derive_src = [&](int a, Cell<float>& c) {  // cell a read as the sweep reads it
    const int as = src_index(a, na, open);
    const long long j = VEL == 1 ? ((long long)as * ny + os) * nz + zs
                                 : ((long long)os * ny + as) * nz + zs;
    float w[5];
#pragma unroll
    for (int v = 0; v < 5; ++v) w[v] = __ldg(src + v * n + j);
    if (in_prim) P::template derive_in<VEL>(w, c, K);
    else P::template derive<VEL>(w, c, K);
  };
  Cell<float> prev, cur, next;
  float flo[5], fhi[5];
  derive_src(a0 - 1, prev);
  derive_src(a0, cur);
  P::hll(prev, cur, flo);
  for (int a = a0; a < a_end; ++a) {
    derive_src(a + 1, next);
    P::hll(cur, next, fhi);
    float st[5], out[5];
    P::update(cur, flo, fhi, st, K);
    if (out_prim) P::to_prim(st, out, K);
    else {
#pragma unroll
      for (int v = 0; v < 5; ++v) out[v] = st[v];
    }
    const long long i = index(a);
#pragma unroll
    for (int v = 0; v < 5; ++v) dst[v * n + i] = out[v];
    cur = next;
#pragma unroll
    for (int v = 0; v < 5; ++v) flo[v] = fhi[v];
  }
}

}  // namespace tf

using namespace tf;

// ===========================================================================
// C ABI
// ===========================================================================
extern "C" {

int tf_abi_version(void) { return TF_ABI_VERSION; }

const char* tf_status_string(int status) {
  switch (status) {
    case TF_OK: return "ok";
    case TF_ERR_ARG: return "invalid argument";
    case TF_ERR_CUDA: return "CUDA error";
    case TF_ERR_NONFINITE: return "non-finite or zero max wave speed";
    case TF_ERR_TIMEOUT: return "device-side wait timed out";
    case TF_ERR_UNSUPPORTED: return "unsupported";
    default: return "unknown status";
  }
}

const char* tf_last_error(void) { return g_err; }

unsigned long long tf_ctl_bytes(void) { return sizeof(tf_ctl); }

int tf_conserved_from_primitive(const float* W, float* U, long long ncells, float gamma,
                                void* stream) {
  if (!W || !U || ncells < 0) return set_error(TF_ERR_ARG, "bad arguments");
  if (W == U) return set_error(TF_ERR_ARG, "output must not alias input");
  if (ncells == 0) return TF_OK;
  StepConsts<float> k = make_consts<float>(gamma, 1.f, 0.f);
  cons_from_prim_kernel<<<elementwise_grid(ncells), 256, 0, (cudaStream_t)stream>>>(W, U, ncells, k);
  return launch_check("cons_from_prim_kernel");
}

int tf_primitive_from_conserved(const float* U, float* W, long long ncells, float gamma,
                                void* stream) {
  if (!W || !U || ncells < 0) return set_error(TF_ERR_ARG, "bad arguments");
  if (W == U) return set_error(TF_ERR_ARG, "output must not alias input");
  if (ncells == 0) return TF_OK;
  StepConsts<float> k = make_consts<float>(gamma, 1.f, 0.f);
  prim_from_cons_kernel<<<elementwise_grid(ncells), 256, 0, (cudaStream_t)stream>>>(U, W, ncells, k);
  return launch_check("prim_from_cons_kernel");
}

int tf_cfl_time_step(const float* W, int nx, int ny, int nz, float dx, float gamma, float cfl,
                     tf_ctl* ctl, void* stream) {
  if (!W || !ctl) return set_error(TF_ERR_ARG, "null pointer");
  TF_TRY(check_dims(nx, ny, nz, 0));
  TF_TRY(check_scalars(dx, gamma));
  if (!(cfl > 0.f) || !isfinite(cfl)) return set_error(TF_ERR_ARG, "C_CFL must be finite and > 0");
  cudaStream_t s = (cudaStream_t)stream;
  long long n = (long long)nx * ny * nz;
  float cfl_dx = cfl * dx;  // fluid.py:502, rounded to float like the traced product
  ctl_init_kernel<<<1, 1, 0, s>>>(ctl, 0.f, cfl_dx, 0);
  maxspeed_kernel<<<elementwise_grid(n), 256, 0, s>>>(W, n, gamma, ctl, 0);
  return launch_check("maxspeed_kernel");
}

int tf_evolve_state(const float* W_in, float* W_out, int nx, int ny, int nz, float dx,
                    float dt_host, const float* dt_dev, float gamma, unsigned flags,
                    const tf_tile_config* tile, void* stream) {
  if (!W_in || !W_out) return set_error(TF_ERR_ARG, "null state pointer");
  if (W_in == W_out) return set_error(TF_ERR_ARG, "W_out must not alias W_in");
  TF_TRY(check_dims(nx, ny, nz, flags));
  TF_TRY(check_scalars(dx, gamma));
  if (!dt_dev && !isfinite(dt_host)) return set_error(TF_ERR_ARG, "dt must be finite");
  int rows, lx, loader;
  TF_TRY(resolve_tile(tile, nx, ny, nz, flags, &rows, &lx, &loader));
  FusedGeom geo = make_geom(nx, ny, nz, flags, rows, lx, loader == 3 ? 1 : 0);
  FusedArgs a = make_fused_args(W_in, W_out, geo, dx, gamma);
  a.layout = loader == 3 ? 1 : 0;
  a.dt_host = dt_host;
  a.dt_dev = dt_dev;
  a.loop = 0;
  a.ctl = nullptr;
  const unsigned cons = TF_FLAG_IN_CONSERVED | TF_FLAG_OUT_CONSERVED;
  if (flags & cons) {
    if ((flags & cons) != cons)
      return set_error(TF_ERR_UNSUPPORTED, "the fused step takes conserved input and output together");
    a.conserved_io = 1;
    if (loader != 3) loader = 1;
  }
  return launch_fused(a, rows, (flags & TF_FLAG_EXACT) != 0, (cudaStream_t)stream, loader);
}

int tf_evolve_state_diag(const float* W_in, float* W_out, int nx, int ny, int nz, float dx,
                         float dt_host, const float* dt_dev, float gamma, unsigned flags,
                         const tf_tile_config* tile, double* totals, float* slice, int z_slice,
                         void* stream) {
  if (!W_in || !W_out || !totals) return set_error(TF_ERR_ARG, "null pointer");
  if (W_in == W_out) return set_error(TF_ERR_ARG, "W_out must not alias W_in");
  TF_TRY(check_dims(nx, ny, nz, flags));
  TF_TRY(check_scalars(dx, gamma));
  if (!dt_dev && !isfinite(dt_host)) return set_error(TF_ERR_ARG, "dt must be finite");
  if (slice && (z_slice < 0 || z_slice >= nz))
    return set_error(TF_ERR_ARG, "z_slice %d outside [0, %d)", z_slice, nz);
  int rows, lx, loader;
  TF_TRY(resolve_tile(tile, nx, ny, nz, flags, &rows, &lx, &loader));
  FusedGeom geo = make_geom(nx, ny, nz, flags, rows, lx, loader == 3 ? 1 : 0);
  FusedArgs a = make_fused_args(W_in, W_out, geo, dx, gamma);
  a.layout = loader == 3 ? 1 : 0;
  a.dt_host = dt_host;
  a.dt_dev = dt_dev;
  a.loop = 0;
  a.ctl = nullptr;
  a.totals = totals;
  a.diag.slice = slice;
  a.diag.z_slice = slice ? z_slice : -1;
  cudaStream_t s = (cudaStream_t)stream;
  TF_TRY(cuda_check(cudaMemsetAsync(totals, 0, 5 * sizeof(double), s), "cudaMemsetAsync"));
  return launch_fused(a, rows, (flags & TF_FLAG_EXACT) != 0, s, 1);
}

int tf_resolve_tile(int nx, int ny, int nz, unsigned flags, const tf_tile_config* tile,
                    tf_tile_config* out) {
  if (!out) return set_error(TF_ERR_ARG, "null output");
  TF_TRY(check_dims(nx, ny, nz, flags));
  int rows, lx, loader;
  TF_TRY(resolve_tile(tile, nx, ny, nz, flags, &rows, &lx, &loader));
  const FusedGeom g = make_geom(nx, ny, nz, flags, rows, lx, loader == 3 ? 1 : 0);
  out->rows = rows;
  out->lx = g.lx;
  out->loader = loader;
  return TF_OK;
}

int tf_debug_checked(void) { return TF_CHECKED; }

int tf_debug_set_graph_loop_cap(int cap) {
  g_graph_loop_cap.store(cap > 0 && cap < kGraphLoopCap ? cap : kGraphLoopCap);
  return TF_OK;
}

int tf_debug_force_64bit_offsets(int on) {
  g_force_64bit.store(on != 0);
  return TF_OK;
}

int tf_debug_set_loop_start_time(float t0) {
  if (!isfinite(t0) || t0 < 0.f) return set_error(TF_ERR_ARG, "start time must be finite and >= 0");
  g_loop_t0.store(t0);
  return TF_OK;
}

int tf_debug_reset(int* write_counts, long long ncells) {
#if TF_CHECKED
  unsigned long long zero = 0;
  TF_TRY(cuda_check(cudaMemcpyToSymbol(g_chk_oob, &zero, sizeof zero), "cudaMemcpyToSymbol"));
  TF_TRY(cuda_check(cudaMemcpyToSymbol(g_chk_writes, &write_counts, sizeof write_counts),
                    "cudaMemcpyToSymbol"));
  TF_TRY(cuda_check(cudaMemcpyToSymbol(g_chk_ncells, &ncells, sizeof ncells),
                    "cudaMemcpyToSymbol"));
  return TF_OK;
#else
  (void)write_counts;
  (void)ncells;
  return set_error(TF_ERR_UNSUPPORTED, "not a checked build (TF_CHECKED=0)");
#endif
}

long long tf_debug_oob_count(void) {
#if TF_CHECKED
  unsigned long long v = 0;
  if (cudaMemcpyFromSymbol(&v, g_chk_oob, sizeof v) != cudaSuccess) return -1;
  return (long long)v;
#else
  return -1;
#endif
}

int tf_diagnostics(const float* W, int nx, int ny, int nz, float gamma, double* totals,
                   float* slice, int z_slice, void* stream) {
  if (!W || !totals) return set_error(TF_ERR_ARG, "null pointer");
  TF_TRY(check_dims(nx, ny, nz, 0));
  TF_TRY(check_scalars(1.f, gamma));
  if (slice && (z_slice < 0 || z_slice >= nz))
    return set_error(TF_ERR_ARG, "z_slice %d outside [0, %d)", z_slice, nz);
  cudaStream_t s = (cudaStream_t)stream;
  TF_TRY(cuda_check(cudaMemsetAsync(totals, 0, 5 * sizeof(double), s), "cudaMemsetAsync"));
  const long long rows = (long long)nx * ny;
  const long long cap = (long long)sm_count() * 16;
  const int per_row = (nz & 3) == 0 ? nz / 4 : nz;  // threads' work items per row
  const int threads = per_row >= 256 ? 256 : ((per_row + 31) / 32) * 32;
  diagnostics_kernel<<<(int)(rows < cap ? rows : cap), threads, 0, s>>>(W, nx, ny, nz,
                                                         make_consts<float>(gamma, 1.f, 0.f),
                                                         totals, slice, z_slice);
  return launch_check("diagnostics_kernel");
}

int tf_time_integration(const float* W_in, float* W_out, float* work, tf_ctl* ctl, int nx, int ny,
                        int nz, float dx, float t_final, float gamma, float cfl, int max_steps,
                        float fixed_dt, unsigned flags, const tf_tile_config* tile,
                        int* iters_host, void* stream) {
  if (!W_in || !W_out || !work || !ctl) return set_error(TF_ERR_ARG, "null pointer");
  if (W_in == W_out || W_in == work || W_out == work)
    return set_error(TF_ERR_ARG, "W_in, W_out and work must be distinct buffers");
  TF_TRY(check_dims(nx, ny, nz, flags));
  TF_TRY(check_scalars(dx, gamma));
  if (!(cfl > 0.f) || !isfinite(cfl)) return set_error(TF_ERR_ARG, "C_CFL must be finite and > 0");
  if (isnan(t_final)) return set_error(TF_ERR_ARG, "t_final is NaN");
  if (!(fixed_dt >= 0.f) || !isfinite(fixed_dt)) return set_error(TF_ERR_ARG, "fixed_dt must be >= 0");
  if (max_steps < 0 && !isfinite(t_final))
    return set_error(TF_ERR_ARG, "an unbounded loop needs a finite t_final or max_steps >= 0");
  int rows, lx, loader;
  TF_TRY(resolve_tile(tile, nx, ny, nz, flags, &rows, &lx, &loader));
  cudaStream_t s = (cudaStream_t)stream;
  const long long n = (long long)nx * ny * nz;
  const bool exact = (flags & TF_FLAG_EXACT) != 0;

  // the device-side t_final loop stops its steps after `cap` of them
  const bool graph = max_steps < 0 && !(flags & TF_FLAG_HOST_LOOP);
  const int cap = g_graph_loop_cap.load();
  ctl_init_kernel<<<1, 1, 0, s>>>(ctl, t_final, cfl * dx, graph ? cap : max_steps,
                                  g_loop_t0.load());
  maxspeed_kernel<<<elementwise_grid(n), 256, 0, s>>>(W_in, n, gamma, ctl, exact ? 0 : 1);
  TF_TRY(launch_check("maxspeed_kernel"));

  FusedGeom geo = make_geom(nx, ny, nz, flags, rows, lx, loader == 3 ? 1 : 0);
  // with a known step count, choose the ping-pong roles so that the last
  // step writes W_out (step i writes buf[i & 1], i = 1..max_steps)
  float* b0 = work;
  float* b1 = W_out;
  if (max_steps >= 0 && (max_steps & 1) == 0) {
    b0 = W_out;
    b1 = work;
  }
  FusedArgs a = make_fused_args(W_in, nullptr, geo, dx, gamma);
  a.layout = loader == 3 ? 1 : 0;
  a.loop = 1;
  a.ctl = ctl;
  a.fixed_dt = fixed_dt;
  const LoopBufs bufs{W_in, {b0, b1}};

  if (max_steps >= 0) {
    // step count known: enqueue exactly that many predicated steps
    for (int i = 1; i <= max_steps; ++i)
      TF_TRY(launch_fused(step_args(a, bufs, i), rows, exact, s, loader));
  } else if (graph) {
    TF_TRY(graph_loop(a, bufs, rows, exact, ctl, cap, s));
  } else {
    // run to t_final: chunks of predicated steps, one host check per chunk
    static thread_local tf_ctl* pinned = nullptr;
    if (!pinned) TF_TRY(cuda_check(cudaMallocHost(&pinned, sizeof(tf_ctl)), "cudaMallocHost"));
    int chunk = 8;
    long long launched = 0;
    float t_prev = -1.f;
    for (;;) {
      for (int i = 1; i <= chunk; ++i)
        TF_TRY(launch_fused(step_args(a, bufs, launched + i), rows, exact, s, loader));
      launched += chunk;
      TF_TRY(cuda_check(cudaMemcpyAsync(pinned, ctl, sizeof(tf_ctl), cudaMemcpyDeviceToHost, s),
                        "cudaMemcpyAsync(ctl)"));
      TF_TRY(cuda_check(cudaStreamSynchronize(s), "cudaStreamSynchronize"));
      if (!pinned->active) break;
      // float32 t no longer advances (t + dt == t): the reference would loop
      // forever here; report it instead
      if (pinned->t == t_prev)
        return set_error(TF_ERR_NONFINITE, "time stalled at t=%g (dt=%g below float spacing)",
                         (double)pinned->t, (double)pinned->dt);
      t_prev = pinned->t;
      if (launched > (1LL << 28)) return set_error(TF_ERR_ARG, "loop did not terminate");
      // remaining steps at the current dt, with margin; predicated steps past
      // the end cost only a launch
      double rem = pinned->dt > 0.f ? ((double)t_final - pinned->t) / pinned->dt : 8.0;
      double want = rem * 1.1 + 2.0;
      chunk = want < 4 ? 4 : (want > 512 ? 512 : (int)want);
    }
  }
  final_select_kernel<<<elementwise_grid(5 * n / 4 + 1), 256, 0, s>>>(ctl, W_in, b0, b1, W_out,
                                                                       5 * n);
  TF_TRY(launch_check("final_select_kernel"));
  if (iters_host) {
    tf_ctl h;
    TF_TRY(cuda_check(cudaMemcpyAsync(&h, ctl, sizeof(tf_ctl), cudaMemcpyDeviceToHost, s),
                      "cudaMemcpyAsync(ctl)"));
    TF_TRY(cuda_check(cudaStreamSynchronize(s), "cudaStreamSynchronize"));
    *iters_host = h.iter;
    if (h.status != TF_OK)
      return set_error(h.status, "device reported %s after %d steps", tf_status_string(h.status),
                       h.iter);
  }
  return TF_OK;
}

int tf_evolve_along_axis(const float* W_in, float* W_out, int nx, int ny, int nz, float dx,
                         float dt_host, const float* dt_dev, float gamma, int axis, unsigned flags,
                         void* stream) {
  if (!W_in || !W_out) return set_error(TF_ERR_ARG, "null state pointer");
  if (W_in == W_out) return set_error(TF_ERR_ARG, "W_out must not alias W_in");
  if (axis < 0 || axis > 2) return set_error(TF_ERR_ARG, "axis must be 0, 1 or 2");
  TF_TRY(check_dims(nx, ny, nz, flags));
  TF_TRY(check_scalars(dx, gamma));
  if (dt_dev) {
    float h = 0.f;
    TF_TRY(cuda_check(cudaMemcpyAsync(&h, dt_dev, sizeof(float), cudaMemcpyDeviceToHost,
                                      (cudaStream_t)stream), "cudaMemcpyAsync(dt)"));
    TF_TRY(cuda_check(cudaStreamSynchronize((cudaStream_t)stream), "cudaStreamSynchronize"));
    dt_host = h;
  }
  StepConsts<float> K = make_consts<float>(gamma, dx, dt_host);
  long long n = (long long)nx * ny * nz;
  int open = (flags & TF_FLAG_OPEN_BOUNDARIES) ? 1 : 0;
  int in_prim = (flags & TF_FLAG_IN_CONSERVED) ? 0 : 1;
  int out_prim = (flags & TF_FLAG_OUT_CONSERVED) ? 0 : 1;
  if ((flags & TF_FLAG_EXACT) && !(in_prim && out_prim))
    return set_error(TF_ERR_ARG, "the exact sweep works on primitive states only");
  cudaStream_t s = (cudaStream_t)stream;
  const bool exact = (flags & TF_FLAG_EXACT) != 0;
  if (axis == 2) {
    const RowLaunch rl = row_launch(nx, ny, nz);
    if (exact) sweep_kernel<ExactPolicy<float>, 3><<<rl.blocks, rl.threads, 0, s>>>(W_in, W_out, nx, ny, nz, open, 1, 1, K);
    else sweep_kernel<FastPolicy, 3><<<rl.blocks, rl.threads, 0, s>>>(W_in, W_out, nx, ny, nz, open, in_prim, out_prim, K);
    return launch_check("sweep_kernel");
  }
  // x / y: march along the axis in chunks sized for ~8 waves of 256 threads
  const int na = axis == 0 ? nx : ny, other = axis == 0 ? ny : nx;
  const int threads = nz >= 256 ? 256 : ((nz + 31) / 32) * 32;
  const long long zblocks = (nz + threads - 1) / threads;
  if (other > 65535) return set_error(TF_ERR_ARG, "grid too large for the sweep launch");
  const long long want = 8LL * sm_count() * (2048 / threads);
  long long chunks = (want + zblocks * other - 1) / (zblocks * other);
  const long long max_chunks = na / 4 > 0 ? na / 4 : 1;  // chunks of >= 4 cells
  if (chunks > max_chunks) chunks = max_chunks;
  if (chunks > 65535) chunks = 65535;
  const int chunk = (int)((na + chunks - 1) / chunks);
  const dim3 grid((unsigned)zblocks, (unsigned)other, (unsigned)((na + chunk - 1) / chunk));
  if (exact) {
    if (axis == 0) march_sweep_kernel<ExactPolicy<float>, 1><<<grid, threads, 0, s>>>(W_in, W_out, nx, ny, nz, chunk, open, 1, 1, K);
    else march_sweep_kernel<ExactPolicy<float>, 2><<<grid, threads, 0, s>>>(W_in, W_out, nx, ny, nz, chunk, open, 1, 1, K);
  } else {
    if (axis == 0) march_sweep_kernel<FastPolicy, 1><<<grid, threads, 0, s>>>(W_in, W_out, nx, ny, nz, chunk, open, in_prim, out_prim, K);
    else march_sweep_kernel<FastPolicy, 2><<<grid, threads, 0, s>>>(W_in, W_out, nx, ny, nz, chunk, open, in_prim, out_prim, K);
  }
  return launch_check("march_sweep_kernel");
}

}  // extern "C"

// ===========================================================================
// Allocation-free run (tf_time_integration_noalloc)
// ===========================================================================
// Some callers cannot allocate device memory at the point where they step a
// simulation: code running inside a host runtime that owns the device heap and
// forbids outside cudaMalloc/cudaFree, callbacks that must not block on the
// allocator, or programs that reserved all memory up front.  For them the run
// loop's scratch -- one control block and one work state -- lives in a
// file-scope device array instead of caller or library allocations.  Every GPU
// that loads this library holds the array (about 5 MiB) until the process
// exits.
namespace tf {
constexpr size_t kNoallocCtlBytes = 256;
constexpr size_t kNoallocBytes =
    kNoallocCtlBytes + 5 * sizeof(float) * (size_t)TF_NOALLOC_MAX_CELLS;
static __device__ __align__(256) unsigned char tf_noalloc_scratch[kNoallocBytes];

// Device address of the scratch on the current device.  In host code the
// array's name is only a host-side handle, so it is looked up once per device
// (with that device current) and cached for the life of the process; a
// cudaDeviceReset unloads the module and invalidates the cached address, so
// the entry point must not be used across one.
constexpr int kNoallocMaxDevices = 64;
static std::mutex g_noalloc_mu;
static void* g_noalloc_addr[kNoallocMaxDevices] = {};

static int noalloc_scratch(unsigned char** out) {
  int dev = 0;
  TF_TRY(cuda_check(cudaGetDevice(&dev), "cudaGetDevice"));
  if (dev < 0 || dev >= kNoallocMaxDevices)
    return set_error(TF_ERR_UNSUPPORTED, "device ordinal %d out of range", dev);
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_addr[dev]) {
    void* p = nullptr;
    TF_TRY(cuda_check(cudaGetSymbolAddress(&p, tf_noalloc_scratch),
                      "cudaGetSymbolAddress(tf_noalloc_scratch)"));
    g_noalloc_addr[dev] = p;
  }
  *out = (unsigned char*)g_noalloc_addr[dev];
  return TF_OK;
}
}  // namespace tf

extern "C" int tf_time_integration_noalloc(const float* W_in, float* W_out, int nx, int ny,
                                           int nz, float dx, float t_final, float gamma,
                                           float cfl, int max_steps, float fixed_dt,
                                           unsigned flags, int* iters_host, void* stream) {
  if (!W_in || !W_out) return set_error(TF_ERR_ARG, "null state pointer");
  if (W_in == W_out) return set_error(TF_ERR_ARG, "W_out must not alias W_in");
  TF_TRY(check_dims(nx, ny, nz, flags));
  const long long n = (long long)nx * ny * nz;
  if (n > (long long)TF_NOALLOC_MAX_CELLS)
    return set_error(TF_ERR_ARG,
                     "grid of %lld cells exceeds the allocation-free scratch of %d cells "
                     "(use tf_time_integration with a caller-provided work buffer)",
                     n, (int)TF_NOALLOC_MAX_CELLS);
  TF_TRY(check_scalars(dx, gamma));
  if (!(cfl > 0.f) || !isfinite(cfl)) return set_error(TF_ERR_ARG, "C_CFL must be finite and > 0");
  if (isnan(t_final)) return set_error(TF_ERR_ARG, "t_final is NaN");
  if (!(fixed_dt >= 0.f) || !isfinite(fixed_dt)) return set_error(TF_ERR_ARG, "fixed_dt must be >= 0");
  if (max_steps < 0 && !isfinite(t_final))
    return set_error(TF_ERR_ARG, "an unbounded loop needs a finite t_final or max_steps >= 0");
  unsigned char* scratch = nullptr;
  TF_TRY(noalloc_scratch(&scratch));
  tf_ctl* ctl = (tf_ctl*)scratch;
  float* work = (float*)(scratch + kNoallocCtlBytes);
  // byte ranges of the two states and of the scratch must be disjoint
  const uintptr_t state_bytes = (uintptr_t)(5 * n) * sizeof(float);
  auto overlap = [](uintptr_t a, uintptr_t na, uintptr_t b, uintptr_t nb) {
    return a < b + nb && b < a + na;
  };
  const uintptr_t in_p = (uintptr_t)W_in, out_p = (uintptr_t)W_out, sc_p = (uintptr_t)scratch;
  if (overlap(in_p, state_bytes, out_p, state_bytes))
    return set_error(TF_ERR_ARG, "W_in and W_out overlap");
  if (overlap(in_p, state_bytes, sc_p, kNoallocBytes) ||
      overlap(out_p, state_bytes, sc_p, kNoallocBytes))
    return set_error(TF_ERR_ARG, "W_in / W_out overlap the library's allocation-free scratch");

  cudaStream_t s = (cudaStream_t)stream;
  const bool exact = (flags & TF_FLAG_EXACT) != 0;
  // tf_time_integration's built-in tile choice (rows, layout, chunk length)
  int rows, lx, loader;
  TF_TRY(resolve_tile(nullptr, nx, ny, nz, flags, &rows, &lx, &loader));
  // the control block keeps the previous call's contents: re-initialise all of it
  ctl_init_kernel<<<1, 1, 0, s>>>(ctl, t_final, cfl * dx, max_steps);
  maxspeed_kernel<<<elementwise_grid(n), 256, 0, s>>>(W_in, n, gamma, ctl, exact ? 0 : 1);
  TF_TRY(launch_check("maxspeed_kernel"));
  FusedGeom geo = make_geom(nx, ny, nz, flags, rows, lx, loader == 3 ? 1 : 0);
  float* b0 = work;
  float* b1 = W_out;
  if (max_steps >= 0 && (max_steps & 1) == 0) {
    b0 = W_out;
    b1 = work;
  }
  FusedArgs a = make_fused_args(W_in, nullptr, geo, dx, gamma);
  a.layout = loader == 3 ? 1 : 0;
  a.loop = 1;
  a.ctl = ctl;
  a.fixed_dt = fixed_dt;
  const LoopBufs bufs{W_in, {b0, b1}};
  if (max_steps >= 0) {
    for (int i = 1; i <= max_steps; ++i)
      TF_TRY(launch_fused(step_args(a, bufs, i), rows, exact, s, loader));
  } else {
    tf_ctl h;  // host copy of the loop state (pageable, on the stack)
    int chunk = 8;
    long long launched = 0;
    float t_prev = -1.f;
    for (;;) {
      for (int i = 1; i <= chunk; ++i)
        TF_TRY(launch_fused(step_args(a, bufs, launched + i), rows, exact, s, loader));
      launched += chunk;
      TF_TRY(cuda_check(cudaMemcpyAsync(&h, ctl, sizeof h, cudaMemcpyDeviceToHost, s),
                        "cudaMemcpyAsync(ctl)"));
      TF_TRY(cuda_check(cudaStreamSynchronize(s), "cudaStreamSynchronize"));
      if (h.status != TF_OK)  // reported whether or not iters_host is given
        return set_error(h.status, "device reported %s after %d steps",
                         tf_status_string(h.status), h.iter);
      if (!h.active) break;
      if (h.t == t_prev)
        return set_error(TF_ERR_NONFINITE, "time stalled at t=%g", (double)h.t);
      t_prev = h.t;
      if (launched > (1LL << 28)) return set_error(TF_ERR_ARG, "loop did not terminate");
      double rem = h.dt > 0.f ? ((double)t_final - h.t) / h.dt : 8.0;
      double want = rem * 1.1 + 2.0;
      chunk = want < 4 ? 4 : (want > 512 ? 512 : (int)want);
    }
  }
  final_select_kernel<<<elementwise_grid(5 * n / 4 + 1), 256, 0, s>>>(ctl, W_in, b0, b1, W_out,
                                                                       5 * n);
  TF_TRY(launch_check("final_select_kernel"));
  if (iters_host) {
    tf_ctl h;
    TF_TRY(cuda_check(cudaMemcpyAsync(&h, ctl, sizeof h, cudaMemcpyDeviceToHost, s),
                      "cudaMemcpyAsync(ctl)"));
    TF_TRY(cuda_check(cudaStreamSynchronize(s), "cudaStreamSynchronize"));
    *iters_host = h.iter;
    if (h.status != TF_OK)
      return set_error(h.status, "device reported %s after %d steps", tf_status_string(h.status),
                       h.iter);
  }
  return TF_OK;
}
