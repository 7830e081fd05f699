// Device builders of initial states: the reference's injection cube
// (scaling_jax.py:23-41) and the two benchmark states (spherical
// overpressure, shear layer), filled in place on the GPU so that large
// states never pass through host memory.  Random numbers come from a
// counter-based hash of (seed, stream, cell index): the fill is independent of
// the launch shape and reproducible across runs and devices.
#include <math.h>
#include <stdint.h>

#include "tf_host.h"

namespace tf {

// SplitMix64 finaliser (Steele, Lea & Flood, 2014) over a 64-bit counter.
__device__ __forceinline__ uint64_t mix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

// Uniform float in [0, 1) from the top 24 hash bits.
__device__ __forceinline__ float hash_uniform(uint64_t seed, uint64_t stream, uint64_t i) {
  uint64_t h = mix64(mix64(seed ^ (stream * 0xD1B54A32D192ED03ull)) + i);
  return (float)(h >> 40) * (1.0f / 16777216.0f);
}

// Standard normal by Box-Muller from two hash uniforms (float32: the fill is
// bandwidth-bound, and GB300's FP64 rate is a small fraction of its FP32 rate).
__device__ __forceinline__ float hash_normal(uint64_t seed, uint64_t stream, uint64_t i) {
  float u1 = 1.0f - hash_uniform(seed, stream, 2 * i);  // (0, 1]
  float u2 = hash_uniform(seed, stream, 2 * i + 1);
  return sqrtf(-2.0f * logf(u1)) * cospif(2.0f * u2);
}

// Launch shape of the fills: blockIdx.y = y row, blockIdx.z = x plane,
// threads stride over z -- no index division per cell.
struct FillIdx {
  int x, y;
  long long row;  // linear index of (x, y, 0)
};
__device__ __forceinline__ FillIdx fill_idx(int n) {
  FillIdx f;
  f.y = blockIdx.y;
  f.x = blockIdx.z;
  f.row = ((long long)f.x * n + f.y) * n;
  return f;
}

__global__ void ics_cube_kernel(float* W, int n, int lo, int hi) {
  const long long n3 = (long long)n * n * n;
  const FillIdx f = fill_idx(n);
  const bool in_xy = f.x >= lo && f.x < hi && f.y >= lo && f.y < hi;
  for (int z = threadIdx.x; z < n; z += blockDim.x) {
    const long long i = f.row + z;
    const bool in = in_xy && z >= lo && z < hi;
    W[i] = in ? 1.0f : 0.125f;
    W[n3 + i] = 0.f;
    W[2 * n3 + i] = 0.f;
    W[3 * n3 + i] = 0.f;
    W[4 * n3 + i] = in ? 1.0f : 0.1f;
  }
}

__global__ void ics_overpressure_kernel(float* W, int n, uint64_t seed, float radius, float p_in,
                                        float p_out, float rho0, float noise) {
  const long long n3 = (long long)n * n * n;
  const FillIdx f = fill_idx(n);
  const float inv_n = 1.0f / (float)n;
  const float cx = (f.x + 0.5f) * inv_n - 0.5f, cy = (f.y + 0.5f) * inv_n - 0.5f;
  const float r2xy = cx * cx + cy * cy;
  for (int z = threadIdx.x; z < n; z += blockDim.x) {
    const long long i = f.row + z;
    const float cz = (z + 0.5f) * inv_n - 0.5f;
    const float r2 = r2xy + cz * cz;
    const float u = hash_uniform(seed, 1, (uint64_t)i);
    W[i] = rho0 * (1.0f + noise * (2.0f * u - 1.0f));
    W[n3 + i] = 0.f;
    W[2 * n3 + i] = 0.f;
    W[3 * n3 + i] = 0.f;
    W[4 * n3 + i] = r2 < radius * radius ? p_in : p_out;
  }
}

__global__ void ics_shear_kernel(float* W, int n, uint64_t seed, float amplitude) {
  const long long n3 = (long long)n * n * n;
  const FillIdx f = fill_idx(n);
  const float inv_n = 1.0f / (float)n;
  const float yc = (f.y + 0.5f) * inv_n, xc = (f.x + 0.5f) * inv_n;
  const bool band = fabsf(yc - 0.5f) < 0.25f;
  const float vy_scale = amplitude * sinpif(4.0f * xc);
  for (int z = threadIdx.x; z < n; z += blockDim.x) {
    const long long i = f.row + z;
    const float a = hash_normal(seed, 2, (uint64_t)i);
    W[i] = band ? 2.0f : 1.0f;
    W[n3 + i] = band ? 0.5f : -0.5f;
    W[2 * n3 + i] = vy_scale * a;
    W[3 * n3 + i] = 0.f;
    W[4 * n3 + i] = 2.5f;
  }
}

static dim3 fill_grid(int n) { return dim3(1, (unsigned)n, (unsigned)n); }
static int fill_threads(int n) { return n >= 256 ? 256 : ((n + 31) / 32) * 32; }
static int check_fill(float* W, int n) {
  if (!W || n < 1) return set_error(TF_ERR_ARG, "bad arguments");
  if (n > 65535) return set_error(TF_ERR_ARG, "grid size %d above 65535", n);
  return TF_OK;
}


}  // namespace tf

using namespace tf;

extern "C" {

// scaling_jax.py:23-41 setup_ics: rho = 0.125, p = 0.1, u = 0, and rho = p = 1
// on the cube [n/2 - k, n/2 + k)^3.  W: 5*n^3 floats.
int tf_ics_injection_cube(float* W, int n, int num_injection_cells, void* stream) {
  TF_TRY(check_fill(W, n));
  int c = n / 2;
  int lo = c - num_injection_cells, hi = c + num_injection_cells;
  // a Python slice with negative start counts from the end; the reference's
  // callers use k = n // 16, so lo >= 0 there; reject the wrap-around case
  if (lo < 0) return set_error(TF_ERR_ARG, "num_injection_cells larger than n/2");
  if (hi > n) hi = n;
  ics_cube_kernel<<<fill_grid(n), fill_threads(n), 0, (cudaStream_t)stream>>>(W, n, lo, hi);
  return launch_check("ics_cube_kernel");
}

// Spherical overpressure on the unit periodic cube, cell centres (i+0.5)/n:
// p = p_in for r < radius around (0.5,0.5,0.5), else p_out; u = 0;
// rho = rho0 * (1 + noise * U(-1, 1)) from the seeded hash.
int tf_ics_overpressure(float* W, int n, unsigned long long seed, double radius, double p_in,
                        double p_out, double rho0, double noise, void* stream) {
  TF_TRY(check_fill(W, n));
  ics_overpressure_kernel<<<fill_grid(n), fill_threads(n), 0, (cudaStream_t)stream>>>(
      W, n, seed, (float)radius, (float)p_in, (float)p_out, (float)rho0, (float)noise);
  return launch_check("ics_overpressure_kernel");
}

// Shear layer: rho = 2, vx = +0.5 for |y - 0.5| < 0.25, else rho = 1,
// vx = -0.5; p = 2.5; vy = amplitude * sin(4 pi x) * a, a ~ N(0, 1) per cell
// from the seeded hash; vz = 0.
int tf_ics_shear_layer(float* W, int n, unsigned long long seed, double amplitude, void* stream) {
  TF_TRY(check_fill(W, n));
  ics_shear_kernel<<<fill_grid(n), fill_threads(n), 0, (cudaStream_t)stream>>>(W, n, seed,
                                                                             (float)amplitude);
  return launch_check("ics_shear_kernel");
}

}  // extern "C"
