// Hand-written adjoint (reverse-mode derivative) of the fixed-dt split step
// in conserved variables.
//
// One sweep along axis d maps U to U' with
//   U'_i = U_i + k (H(U_{i-1}, U_i) - H(U_i, U_{i+1})),   k = dt/dx,
// H the HLL flux (fluid.py:263-305) written in conserved variables.  Given
// lam' = dL/dU', the adjoint sweep returns lam = dL/dU:
//   g_{i-1/2} = k (lam'_i - lam'_{i-1})            (dL/dH at face i-1/2)
//   lam_i = lam'_i + g_{i-1/2}^T dH/dU_R(U_{i-1}, U_i) + g_{i+1/2}^T dH/dU_L(U_i, U_{i+1})
// The VJP of H below is derived by hand from the forward formulas (rho, m,
// E -> u, p, c, F -> S+, S- -> H).  At ties of the max/min in the wave speeds
// the gradient is split evenly between the tied arguments, the convention of
// both JAX (lax.max) and PyTorch (torch.maximum), so it matches their
// automatic derivatives of the reference step.
//
// A step's adjoint is the z, y, x adjoint sweeps in that order, each given the
// input state of the corresponding forward sweep (recomputed from the step's
// input); tinyfluids_gb300/adjoint.py drives it with sqrt(N) checkpointing.
#include <math.h>

#include "tf_common.cuh"
#include "tf_host.h"
#include "tf_math.cuh"

namespace tf {

template <typename T> struct AdjMath;
template <> struct AdjMath<float> {
  static __device__ __forceinline__ float rcp(float x) { return FastPolicy::rcp(x); }
  static __device__ __forceinline__ float sqrt_(float x) { return FastPolicy::sqrt_(x); }
};
template <> struct AdjMath<double> {
  static __device__ __forceinline__ double rcp(double x) { return 1.0 / x; }
  static __device__ __forceinline__ double sqrt_(double x) { return sqrt(x); }
};

// Forward quantities of one side (conserved input), as FastPolicy::derive.
template <typename T>
struct Side {
  T U[5], F[5];
  T ir, u, q, p, c;
};

template <typename T, int VEL>
__device__ __forceinline__ void side_forward(const T U[5], T g, T gm1, Side<T>& s) {
  using M = AdjMath<T>;
#pragma unroll
  for (int i = 0; i < 5; ++i) s.U[i] = U[i];
  s.ir = M::rcp(U[0]);
  s.u = U[VEL] * s.ir;
  s.q = fma(U[1], U[1], fma(U[2], U[2], U[3] * U[3]));
  s.p = gm1 * fma(T(-0.5) * s.q, s.ir, U[4]);
  s.F[0] = U[VEL];
  s.F[1] = U[1] * s.u;
  s.F[2] = U[2] * s.u;
  s.F[3] = U[3] * s.u;
  s.F[4] = (U[4] + s.p) * s.u;
  s.F[VEL] = fma(U[VEL], s.u, s.p);
  s.c = M::sqrt_(g * s.p * s.ir);
}

// HLL flux of (L, R), as FastPolicy::hll.
template <typename T>
__device__ __forceinline__ void hll_forward(const Side<T>& L, const Side<T>& R, T H[5]) {
  using M = AdjMath<T>;
  T sp = fmax(fmax(L.u + L.c, R.u + R.c), T(0));
  T sm = fmin(fmin(L.u - L.c, R.u - R.c), T(0));
  T inv = M::rcp(sp - sm);
  T a = sp * inv, b = sm * inv, s = sm * a;
#pragma unroll
  for (int i = 0; i < 5; ++i) H[i] = fma(a, L.F[i], fma(-b, R.F[i], s * (R.U[i] - L.U[i])));
}

// d max(x, y) split evenly at ties: weight of x
template <typename T>
__device__ __forceinline__ T wmax_x(T x, T y) { return x > y ? T(1) : (x == y ? T(0.5) : T(0)); }
template <typename T>
__device__ __forceinline__ T wmin_x(T x, T y) { return x < y ? T(1) : (x == y ? T(0.5) : T(0)); }

// Reverse through one side: given the adjoints of its F, u and c, add dL/dU.
template <typename T, int VEL>
__device__ __forceinline__ void side_backward(const Side<T>& s, const T Fb[5], T ub, T cb,
                                              T g, T gm1, T Ub[5]) {
  // F = [m_d, m_x u, m_y u, m_z u, (E + p) u] + p e_d
  T mb[4] = {T(0), T(0), T(0), T(0)};  // adjoints of m_x, m_y, m_z (index 1..3)
  T Eb = T(0), pb = T(0), irb = T(0);
  mb[VEL] += Fb[0];
  mb[1] += Fb[1] * s.u;
  mb[2] += Fb[2] * s.u;
  mb[3] += Fb[3] * s.u;
  ub += Fb[1] * s.U[1] + Fb[2] * s.U[2] + Fb[3] * s.U[3] + Fb[4] * (s.U[4] + s.p);
  Eb += Fb[4] * s.u;
  pb += Fb[4] * s.u + Fb[VEL];
  // c = sqrt(g p ir)
  if (s.c > T(0)) {
    T xb = cb / (T(2) * s.c);
    pb += xb * g * s.ir;
    irb += xb * g * s.p;
  }
  // u = m_d ir
  mb[VEL] += ub * s.ir;
  irb += ub * s.U[VEL];
  // p = gm1 (E - 0.5 q ir)
  Eb += pb * gm1;
  T qb = T(-0.5) * gm1 * s.ir * pb;
  irb += T(-0.5) * gm1 * s.q * pb;
  // q = m_x^2 + m_y^2 + m_z^2
  mb[1] += T(2) * s.U[1] * qb;
  mb[2] += T(2) * s.U[2] * qb;
  mb[3] += T(2) * s.U[3] * qb;
  // ir = 1/rho
  Ub[0] += -irb * s.ir * s.ir;
  Ub[1] += mb[1];
  Ub[2] += mb[2];
  Ub[3] += mb[3];
  Ub[4] += Eb;
}

// VJP of the HLL flux: given gb = dL/dH, add dL/dU_L to ULb and dL/dU_R to URb.
template <typename T, int VEL>
__device__ __forceinline__ void hll_vjp(const Side<T>& L, const Side<T>& R, const T gb[5], T g,
                                        T gm1, T ULb[5], T URb[5]) {
  using M = AdjMath<T>;
  const T aL = L.u + L.c, aR = R.u + R.c, bL = L.u - L.c, bR = R.u - R.c;
  const T sp_in = fmax(aL, aR), sm_in = fmin(bL, bR);
  const T sp = fmax(sp_in, T(0)), sm = fmin(sm_in, T(0));
  const T inv = M::rcp(sp - sm);
  const T a = sp * inv, b = sm * inv, s = sm * a;
  T ab = T(0), bb = T(0), sb = T(0);
  T FLb[5], FRb[5];
#pragma unroll
  for (int i = 0; i < 5; ++i) {
    FLb[i] = a * gb[i];
    FRb[i] = -b * gb[i];
    ULb[i] += -s * gb[i];
    URb[i] += s * gb[i];
    ab += gb[i] * L.F[i];
    bb -= gb[i] * R.F[i];
    sb += gb[i] * (R.U[i] - L.U[i]);
  }
  // a = sp/D, b = sm/D, s = sm sp/D with D = sp - sm
  const T inv2 = inv * inv;
  const T spb = (-(ab + bb) * sm - sb * sm * sm) * inv2;
  const T smb = ((ab + bb) * sp + sb * sp * sp) * inv2;
  // S+ = max(max(aL, aR), 0), S- = min(min(bL, bR), 0), ties split evenly
  const T sp_inb = spb * wmax_x(sp_in, T(0));
  const T sm_inb = smb * wmin_x(sm_in, T(0));
  const T aLb = sp_inb * wmax_x(aL, aR), aRb = sp_inb - aLb;
  const T bLb = sm_inb * wmin_x(bL, bR), bRb = sm_inb - bLb;
  side_backward<T, VEL>(L, FLb, aLb + bLb, aLb - bLb, g, gm1, ULb);
  side_backward<T, VEL>(R, FRb, aRb + bRb, aRb - bRb, g, gm1, URb);
}

struct AdjGeom {
  int nx, ny, nz;
};

// Linear index of the periodic neighbour at offset d along velocity index vel.
__device__ __forceinline__ long long nb_index(int x, int y, int z, const AdjGeom& G, int vel,
                                              int d) {
  if (vel == 1) x = wrap_index(x + d, G.nx);
  if (vel == 2) y = wrap_index(y + d, G.ny);
  if (vel == 3) z = wrap_index(z + d, G.nz);
  return ((long long)x * G.ny + y) * G.nz + z;
}

// Adjoint of one periodic sweep along VEL (one thread per cell).
template <typename T, int VEL>
__global__ void __launch_bounds__(256) adjoint_sweep_kernel(const T* __restrict__ U,
                                                            const T* __restrict__ lam_out,
                                                            T* __restrict__ lam_in, AdjGeom G, T k,
                                                            T g) {
  const long long n = (long long)G.nx * G.ny * G.nz;
  const T gm1 = g - T(1);
  for_each_cell(G.nx, G.ny, G.nz, [&](long long i, int x, int y, int z) {
    const long long im = nb_index(x, y, z, G, VEL, -1), ip = nb_index(x, y, z, G, VEL, +1);
    T u0[5], u1[5], u2[5], l0[5], l1[5], l2[5];
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      u0[v] = U[v * n + im];
      u1[v] = U[v * n + i];
      u2[v] = U[v * n + ip];
      l0[v] = lam_out[v * n + im];
      l1[v] = lam_out[v * n + i];
      l2[v] = lam_out[v * n + ip];
    }
    Side<T> s0, s1, s2;
    side_forward<T, VEL>(u0, g, gm1, s0);
    side_forward<T, VEL>(u1, g, gm1, s1);
    side_forward<T, VEL>(u2, g, gm1, s2);
    T glo[5], ghi[5], dummy[5], acc[5];
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      glo[v] = k * (l1[v] - l0[v]);  // face i-1/2
      ghi[v] = k * (l2[v] - l1[v]);  // face i+1/2
      acc[v] = l1[v];
      dummy[v] = T(0);
    }
    hll_vjp<T, VEL>(s0, s1, glo, g, gm1, dummy, acc);  // cell i is the right state
#pragma unroll
    for (int v = 0; v < 5; ++v) dummy[v] = T(0);
    hll_vjp<T, VEL>(s1, s2, ghi, g, gm1, acc, dummy);  // cell i is the left state
#pragma unroll
    for (int v = 0; v < 5; ++v) lam_in[v * n + i] = acc[v];
  });
}

// Adjoint of one periodic sweep along x or y (VEL 1 or 2) that marches: a
// thread owns one (y or x, z) column and walks a chunk of the sweep axis,
// carrying the previous cell's forward quantities and its partly accumulated
// lam_in, so each cell's forward side is computed once and each face's VJP
// once.  Every cell's lam_in receives the same additions in the same order
// as in adjoint_sweep_kernel (its lam_out, then its left face, then its right
// face), so the result is the same bits.
template <typename T, int VEL>
__global__ void __launch_bounds__(256) march_adjoint_kernel(const T* __restrict__ U,
                                                            const T* __restrict__ lam_out,
                                                            T* __restrict__ lam_in, AdjGeom G, T k,
                                                            T g, int chunk) {
  static_assert(VEL == 1 || VEL == 2, "x or y sweeps only");
  const long long n = (long long)G.nx * G.ny * G.nz;
  const T gm1 = g - T(1);
  const int z = blockIdx.x * blockDim.x + threadIdx.x;
  if (z >= G.nz) return;
  const int o = blockIdx.y;  // y for an x sweep, x for a y sweep
  const int na = VEL == 1 ? G.nx : G.ny;
  const int a0 = blockIdx.z * chunk, a_end = min(a0 + chunk, na);
  auto index = [&](int a) {
    a = wrap_index(a, na);
    return VEL == 1 ? ((long long)a * G.ny + o) * G.nz + z : ((long long)o * G.ny + a) * G.nz + z;
  };
  auto load = [&](int a, Side<T>& sd, T l[5]) {
    const long long j = index(a);
    T u[5];
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      u[v] = U[v * n + j];
      l[v] = lam_out[v * n + j];
    }
    side_forward<T, VEL>(u, g, gm1, sd);
  };
  Side<T> prev, cur, next;
  T l_prev[5], l_cur[5], l_next[5], acc_cur[5], acc_next[5], gb[5], dummy[5];
  load(a0 - 1, prev, l_prev);
  load(a0, cur, l_cur);
#pragma unroll
  for (int v = 0; v < 5; ++v) {
    gb[v] = k * (l_cur[v] - l_prev[v]);  // face a0-1/2
    acc_cur[v] = l_cur[v];
    dummy[v] = T(0);
  }
  hll_vjp<T, VEL>(prev, cur, gb, g, gm1, dummy, acc_cur);
  for (int a = a0; a < a_end; ++a) {
    load(a + 1, next, l_next);
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      gb[v] = k * (l_next[v] - l_cur[v]);  // face a+1/2
      acc_next[v] = l_next[v];
    }
    hll_vjp<T, VEL>(cur, next, gb, g, gm1, acc_cur, acc_next);
    const long long i = index(a);
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      lam_in[v * n + i] = acc_cur[v];
      acc_cur[v] = acc_next[v];
      l_cur[v] = l_next[v];
    }
    cur = next;
  }
}

// Forward sweep in conserved variables, for the FP64 finite-difference check
// (float runs use the fast sweep kernel of tf_step.cu with conserved I/O).
template <typename T, int VEL>
__global__ void __launch_bounds__(256) cons_sweep_kernel(const T* __restrict__ U,
                                                         T* __restrict__ out, AdjGeom G, T k,
                                                         T g) {
  const long long n = (long long)G.nx * G.ny * G.nz;
  const T gm1 = g - T(1);
  for_each_cell(G.nx, G.ny, G.nz, [&](long long i, int x, int y, int z) {
    const long long idx[3] = {nb_index(x, y, z, G, VEL, -1), i, nb_index(x, y, z, G, VEL, +1)};
    Side<T> s[3];
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      T u[5];
#pragma unroll
      for (int v = 0; v < 5; ++v) u[v] = U[v * n + idx[j]];
      side_forward<T, VEL>(u, g, gm1, s[j]);
    }
    T flo[5], fhi[5];
    hll_forward(s[0], s[1], flo);
    hll_forward(s[1], s[2], fhi);
#pragma unroll
    for (int v = 0; v < 5; ++v) out[v * n + i] = fma(k, flo[v] - fhi[v], s[1].U[v]);
  });
}

template <typename T>
static int launch_adj(bool adjoint, const T* U, const T* lam_out, T* out, int nx, int ny, int nz,
                      double dx, double dt, double gamma, int axis, cudaStream_t s,
                      bool per_cell = false) {
  if (!U || !out || (adjoint && !lam_out)) return set_error(TF_ERR_ARG, "null pointer");
  if (out == U || (adjoint && out == lam_out)) return set_error(TF_ERR_ARG, "output aliases input");
  if (nx < 1 || ny < 1 || nz < 1) return set_error(TF_ERR_ARG, "grid dims must be >= 1");
  if (axis < 0 || axis > 2) return set_error(TF_ERR_ARG, "axis must be 0, 1 or 2");
  if (!(dx > 0) || !isfinite(dt) || !isfinite(gamma) || gamma == 1.0)
    return set_error(TF_ERR_ARG, "bad scalar parameter");
  AdjGeom G{nx, ny, nz};
  const RowLaunch rl = row_launch(nx, ny, nz);
  T k = (T)(dt / dx), g = (T)gamma;
  if (sizeof(T) == 4) k = (T)((float)dt * (1.f / (float)dx));  // as the fast sweep: dt * (1/dx)
  if (adjoint) {
    if (axis == 2 || per_cell) {
      if (axis == 0) adjoint_sweep_kernel<T, 1><<<rl.blocks, rl.threads, 0, s>>>(U, lam_out, out, G, k, g);
      if (axis == 1) adjoint_sweep_kernel<T, 2><<<rl.blocks, rl.threads, 0, s>>>(U, lam_out, out, G, k, g);
      if (axis == 2) adjoint_sweep_kernel<T, 3><<<rl.blocks, rl.threads, 0, s>>>(U, lam_out, out, G, k, g);
      return launch_check("adjoint_sweep_kernel");
    }
    // x / y: march in chunks sized for ~8 waves of 256 threads
    const int na = axis == 0 ? nx : ny, other = axis == 0 ? ny : nx;
    const int threads = nz >= 256 ? 256 : ((nz + 31) / 32) * 32;
    const long long zblocks = (nz + threads - 1) / threads;
    if (other > 65535) return set_error(TF_ERR_ARG, "grid too large for the adjoint launch");
    const long long want = 8LL * sm_count() * (2048 / threads);
    long long chunks = (want + zblocks * other - 1) / (zblocks * other);
    const long long max_chunks = na / 4 > 0 ? na / 4 : 1;
    if (chunks > max_chunks) chunks = max_chunks;
    if (chunks > 65535) chunks = 65535;
    const int chunk = (int)((na + chunks - 1) / chunks);
    const dim3 grid((unsigned)zblocks, (unsigned)other, (unsigned)((na + chunk - 1) / chunk));
    if (axis == 0) march_adjoint_kernel<T, 1><<<grid, threads, 0, s>>>(U, lam_out, out, G, k, g, chunk);
    else march_adjoint_kernel<T, 2><<<grid, threads, 0, s>>>(U, lam_out, out, G, k, g, chunk);
    return launch_check("march_adjoint_kernel");
  }
  if (axis == 0) cons_sweep_kernel<T, 1><<<rl.blocks, rl.threads, 0, s>>>(U, out, G, k, g);
  if (axis == 1) cons_sweep_kernel<T, 2><<<rl.blocks, rl.threads, 0, s>>>(U, out, G, k, g);
  if (axis == 2) cons_sweep_kernel<T, 3><<<rl.blocks, rl.threads, 0, s>>>(U, out, G, k, g);
  return launch_check("cons_sweep_kernel");
}

}  // namespace tf

using namespace tf;

extern "C" {

int tf_adjoint_sweep(const float* U, const float* lam_out, float* lam_in, int nx, int ny, int nz,
                     float dx, float dt, float gamma, int axis, void* stream) {
  return launch_adj<float>(true, U, lam_out, lam_in, nx, ny, nz, dx, dt, gamma, axis,
                           (cudaStream_t)stream);
}

int tf_debug_adjoint_sweep_per_cell(const float* U, const float* lam_out, float* lam_in, int nx,
                                    int ny, int nz, float dx, float dt, float gamma, int axis,
                                    void* stream) {
  return launch_adj<float>(true, U, lam_out, lam_in, nx, ny, nz, dx, dt, gamma, axis,
                           (cudaStream_t)stream, true);
}

int tf_adjoint_sweep_f64(const double* U, const double* lam_out, double* lam_in, int nx, int ny,
                         int nz, double dx, double dt, double gamma, int axis, void* stream) {
  return launch_adj<double>(true, U, lam_out, lam_in, nx, ny, nz, dx, dt, gamma, axis,
                            (cudaStream_t)stream);
}

int tf_sweep_conserved_f64(const double* U, double* out, int nx, int ny, int nz, double dx,
                           double dt, double gamma, int axis, void* stream) {
  return launch_adj<double>(false, U, nullptr, out, nx, ny, nz, dx, dt, gamma, axis,
                            (cudaStream_t)stream);
}

}  // extern "C"
