// Shared device helpers: the control block, index maps, reductions.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/tinyfluids_gb300.h"

namespace tf {

// Periodic wrap of a (possibly negative or >= n) index into [0, n).
__device__ __forceinline__ int wrap_index(int i, int n) {
  if ((unsigned)i < (unsigned)n) return i;
  int r = i % n;
  return r < 0 ? r + n : r;
}

// Source index of logical cell i along an axis of n cells.  Periodic wrap
// (the jnp.roll neighbours of fluid.py:528,548), then, with open boundaries,
// the clamp to [1, n-2] that the x/y/z slab copies of fluid.py:384-413
// amount to: after copying x=0 <- 1, x=n-1 <- n-2, then the same along y and
// z, cell (x,y,z) holds the input value at (cx(x), cy(y), cz(z)).
__device__ __forceinline__ int src_index(int i, int n, bool open) {
  int j = wrap_index(i, n);
  if (open) {
    int hi = n - 2;
    if (hi < 1) hi = 1;  // n == 2: both cells take cell 1 (left copy first)
    j = j < 1 ? 1 : (j > hi ? hi : j);
  }
  return j;
}

// Warp and block maxima of wave speeds (>= 0 or NaN), NaN-propagating via
// the unsigned order of the bit patterns.
__device__ __forceinline__ unsigned warp_max_bits(unsigned v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// Maximum over the block of the speed v; valid in thread 0.  `red` needs one
// float per warp.
__device__ __forceinline__ float block_max(float v, float* red) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int nw = (blockDim.x + 31) >> 5;
  unsigned b = warp_max_bits(__float_as_uint(v));
  __syncthreads();
  if (lane == 0) red[w] = __uint_as_float(b);
  __syncthreads();
  if (w == 0) {
    b = lane < nw ? __float_as_uint(red[lane]) : 0u;
    b = warp_max_bits(b);
  }
  return __uint_as_float(b);
}

// Compensated float32 sum (Knuth's TwoSum): s + c carries the running sum
// to about twice float32 precision, so per-thread partials need no float64
// arithmetic (a small fraction of the float32 rate on this GPU).  The
// operations must not be reassociated: they contain no products, so no FMA
// contraction applies either.
struct CSum {
  float s, c;
};
__device__ __forceinline__ void csum_add(CSum& a, float x) {
  const float t = a.s + x;
  const float z = t - a.s;
  a.c += (a.s - (t - z)) + (x - z);
  a.s = t;
}

// Sums five per-thread partials over the block in float64 and adds them to
// totals[0..4] (one atomic per component per CTA).  `red` needs 5 doubles per
// warp.  Every thread of the block must call it.
__device__ __forceinline__ void block_add_totals(const CSum acc[5], double* red,
                                                 double* totals) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int nw = (blockDim.x + 31) >> 5;
  double v[5];
#pragma unroll
  for (int i = 0; i < 5; ++i) {
    v[i] = (double)acc[i].s + (double)acc[i].c;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v[i] += __shfl_xor_sync(0xffffffffu, v[i], o);
  }
  __syncthreads();
  if (lane == 0) {
#pragma unroll
    for (int i = 0; i < 5; ++i) red[w * 5 + i] = v[i];
  }
  __syncthreads();
  if (threadIdx.x < 5) {
    double sum = 0.0;
    for (int k = 0; k < nw; ++k) sum += red[k * 5 + threadIdx.x];
    atomicAdd(totals + threadIdx.x, sum);
  }
}

// Visits every cell (x, y, z) of an nx*ny*nz grid once: blocks stride over
// the (x, y) rows, threads over z, so a cell's coordinates need no division
// (one per row).  f(i, x, y, z) with i the linear index (x*ny + y)*nz + z.
template <class F>
__device__ __forceinline__ void for_each_cell(int nx, int ny, int nz, F f) {
  const long long rows = (long long)nx * ny;
  for (long long r = blockIdx.x; r < rows; r += gridDim.x) {
    const int y = (int)(r % ny), x = (int)(r / ny);
    for (int z = threadIdx.x; z < nz; z += blockDim.x) f(r * nz + z, x, y, z);
  }
}

// Volatile reads of control fields written by other kernels/CTAs.
__device__ __forceinline__ int ld_volatile(const int* p) { return *(const volatile int*)p; }
__device__ __forceinline__ float ld_volatile(const float* p) { return *(const volatile float*)p; }

// Adds this CTA's max wave speed to ctl and, in the CTA that finishes last,
// closes the step: t += dt, iter += 1, next dt = (C_CFL*dx)/max_speed, the
// loop condition, and the device-side error status.  Called by thread 0
// only, after the CTA's last store.  `nblocks` is the number of CTAs that
// contribute to this ctl in this launch.
__device__ __forceinline__ bool ctl_finish_cta(tf_ctl* ctl, float cta_max, unsigned nblocks,
                                               float dt_used, bool advance_time) {
  atomicMax(&ctl->ws_bits, __float_as_uint(cta_max));
  __threadfence();
  unsigned prev = atomicAdd(&ctl->done, 1u);
  if (prev != nblocks - 1) return false;
  __threadfence();
  float ms = __uint_as_float(atomicAdd(&ctl->ws_bits, 0u));
  float cfl_dx = ld_volatile(&ctl->cfl_dx);
  int iter = ld_volatile(&ctl->iter);
  float t = ld_volatile(&ctl->t);
  if (advance_time) {
    t = __fadd_rn(t, dt_used);  // time_integration.py:80
    iter += 1;                  // time_integration.py:81
  }
  float dt_next = __fdiv_rn(cfl_dx, ms);  // fluid.py:502
  int status = ld_volatile(&ctl->status);
  if (!(ms > 0.f) || !isfinite(ms) || !isfinite(dt_next)) status = TF_ERR_NONFINITE;
  int max_steps = ld_volatile(&ctl->max_steps);
  float t_final = ld_volatile(&ctl->t_final);
  int active = (t < t_final) && (max_steps < 0 || iter < max_steps) && status == TF_OK;
  ctl->max_speed = ms;
  ctl->dt = dt_next;
  ctl->t = t;
  ctl->status = status;
  ctl->active = active;
  ctl->ws_bits = 0u;
  ctl->done = 0u;
  __threadfence();
  // iter is written last: a CTA that waits for this step (the persistent
  // batch kernel) polls iter and then reads the other fields after a fence
  *(volatile int*)&ctl->iter = iter;
  return true;
}

}  // namespace tf
