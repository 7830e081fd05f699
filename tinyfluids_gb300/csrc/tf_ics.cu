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

// Uniform double in [0, 1) from 53 hash bits.
__device__ __forceinline__ double hash_uniform(uint64_t seed, uint64_t stream, uint64_t i) {
  uint64_t h = mix64(mix64(seed ^ (stream * 0xD1B54A32D192ED03ull)) + i);
  return (double)(h >> 11) * (1.0 / 9007199254740992.0);
}

// Standard normal by Box-Muller from two hash uniforms.
__device__ __forceinline__ double hash_normal(uint64_t seed, uint64_t stream, uint64_t i) {
  double u1 = hash_uniform(seed, stream, 2 * i);
  double u2 = hash_uniform(seed, stream, 2 * i + 1);
  u1 = 1.0 - u1;  // (0, 1]
  return sqrt(-2.0 * log(u1)) * cospi(2.0 * u2);
}

__global__ void ics_cube_kernel(float* W, int n, int lo, int hi) {
  long long n3 = (long long)n * n * n;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n3;
       i += (long long)gridDim.x * blockDim.x) {
    int z = (int)(i % n), y = (int)((i / n) % n), x = (int)(i / ((long long)n * n));
    bool in = x >= lo && x < hi && y >= lo && y < hi && z >= lo && z < hi;
    W[i] = in ? 1.0f : 0.125f;
    W[n3 + i] = 0.f;
    W[2 * n3 + i] = 0.f;
    W[3 * n3 + i] = 0.f;
    W[4 * n3 + i] = in ? 1.0f : 0.1f;
  }
}

__global__ void ics_overpressure_kernel(float* W, int n, uint64_t seed, double radius, double p_in,
                                        double p_out, double rho0, double noise) {
  long long n3 = (long long)n * n * n;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n3;
       i += (long long)gridDim.x * blockDim.x) {
    int z = (int)(i % n), y = (int)((i / n) % n), x = (int)(i / ((long long)n * n));
    double cx = (x + 0.5) / n - 0.5, cy = (y + 0.5) / n - 0.5, cz = (z + 0.5) / n - 0.5;
    double r2 = cx * cx + cy * cy + cz * cz;
    double u = hash_uniform(seed, 1, (uint64_t)i);
    W[i] = (float)(rho0 * (1.0 + noise * (2.0 * u - 1.0)));
    W[n3 + i] = 0.f;
    W[2 * n3 + i] = 0.f;
    W[3 * n3 + i] = 0.f;
    W[4 * n3 + i] = (float)(r2 < radius * radius ? p_in : p_out);
  }
}

__global__ void ics_shear_kernel(float* W, int n, uint64_t seed, double amplitude) {
  long long n3 = (long long)n * n * n;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n3;
       i += (long long)gridDim.x * blockDim.x) {
    int y = (int)((i / n) % n), x = (int)(i / ((long long)n * n));
    double yc = (y + 0.5) / n, xc = (x + 0.5) / n;
    bool band = fabs(yc - 0.5) < 0.25;
    double a = hash_normal(seed, 2, (uint64_t)i);
    W[i] = band ? 2.0f : 1.0f;
    W[n3 + i] = band ? 0.5f : -0.5f;
    W[2 * n3 + i] = (float)(amplitude * sinpi(4.0 * xc) * a);
    W[3 * n3 + i] = 0.f;
    W[4 * n3 + i] = 2.5f;
  }
}

static int ics_grid(long long n3) {
  long long b = (n3 + 255) / 256;
  long long cap = (long long)sm_count() * 16;
  return (int)(b < 1 ? 1 : (b < cap ? b : cap));
}

}  // namespace tf

using namespace tf;

extern "C" {

// scaling_jax.py:23-41 setup_ics: rho = 0.125, p = 0.1, u = 0, and rho = p = 1
// on the cube [n/2 - k, n/2 + k)^3.  W: 5*n^3 floats.
int tf_ics_injection_cube(float* W, int n, int num_injection_cells, void* stream) {
  if (!W || n < 1) return set_error(TF_ERR_ARG, "bad arguments");
  int c = n / 2;
  int lo = c - num_injection_cells, hi = c + num_injection_cells;
  // a Python slice with negative start counts from the end; the reference's
  // callers use k = n // 16, so lo >= 0 there; reject the wrap-around case
  if (lo < 0) return set_error(TF_ERR_ARG, "num_injection_cells larger than n/2");
  if (hi > n) hi = n;
  long long n3 = (long long)n * n * n;
  ics_cube_kernel<<<ics_grid(n3), 256, 0, (cudaStream_t)stream>>>(W, n, lo, hi);
  return launch_check("ics_cube_kernel");
}

// Spherical overpressure on the unit periodic cube, cell centres (i+0.5)/n:
// p = p_in for r < radius around (0.5,0.5,0.5), else p_out; u = 0;
// rho = rho0 * (1 + noise * U(-1, 1)) from the seeded hash.
int tf_ics_overpressure(float* W, int n, unsigned long long seed, double radius, double p_in,
                        double p_out, double rho0, double noise, void* stream) {
  if (!W || n < 1) return set_error(TF_ERR_ARG, "bad arguments");
  long long n3 = (long long)n * n * n;
  ics_overpressure_kernel<<<ics_grid(n3), 256, 0, (cudaStream_t)stream>>>(W, n, seed, radius, p_in,
                                                                          p_out, rho0, noise);
  return launch_check("ics_overpressure_kernel");
}

// Shear layer: rho = 2, vx = +0.5 for |y - 0.5| < 0.25, else rho = 1,
// vx = -0.5; p = 2.5; vy = amplitude * sin(4 pi x) * a, a ~ N(0, 1) per cell
// from the seeded hash; vz = 0.
int tf_ics_shear_layer(float* W, int n, unsigned long long seed, double amplitude, void* stream) {
  if (!W || n < 1) return set_error(TF_ERR_ARG, "bad arguments");
  long long n3 = (long long)n * n * n;
  ics_shear_kernel<<<ics_grid(n3), 256, 0, (cudaStream_t)stream>>>(W, n, seed, amplitude);
  return launch_check("ics_shear_kernel");
}

}  // extern "C"
