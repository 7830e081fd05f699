// Per-cell and per-interface arithmetic of the tinyfluids step, in two
// policies that every kernel of this library is templated on.
//
//  * ExactPolicy<T>: the reference's float arithmetic, op for op
//    (tinyfluids/jax_tinyfluids/fluid.py).  Each +,-,*,/,sqrt is an explicit
//    IEEE round-to-nearest intrinsic, so nothing is contracted into an FMA and
//    the result is bit-identical to a NumPy float32 evaluation of the same
//    expressions.  The state between directional sweeps is PRIMITIVE, rounded
//    through conserved -> primitive at the end of every sweep exactly like
//    fluid.py:517 and :555.
//  * FastPolicy: the same scheme, restructured for throughput.  The state
//    between sweeps is CONSERVED (no prim/cons round trip inside the step),
//    each cell's 1/rho, pressure and sound speed are computed once, the HLL
//    quotient uses one reciprocal per interface, and products/sums fuse into
//    FMAs.  Results differ from the reference in the last bits; the tests
//    state the tolerance.
//
// Variable order of a state: rho, vx, vy, vz, p (primitive) or
// rho, mx, my, mz, E (conserved), fluid.py:14-18.
#pragma once
#include <cuda_runtime.h>
#include <math.h>

namespace tf {

// Quantities of one cell for a sweep along velocity index VEL (1, 2, 3):
// conserved U, physical flux F along VEL (fluid.py:208-259) and two wave
// quantities that only the policy's own hll() reads: the exact policy keeps
// the normal velocity u and the sound speed c (fluid.py:106-117), the fast
// policies keep the wave-speed bounds u + c and c - u, which every face of
// the cell needs and which are then computed once per cell instead of once
// per face.
template <typename T>
struct Cell {
  T U[5];
  T F[5];
  T wa;  // exact: u      fast: u + c
  T wb;  // exact: c      fast: c - u
};

// ---------------------------------------------------------------------------
// IEEE round-to-nearest operations that the compiler may not contract.
// ---------------------------------------------------------------------------
template <typename T> struct IEEE;
template <> struct IEEE<float> {
  static __device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
  static __device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
  static __device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
  static __device__ __forceinline__ float div(float a, float b) { return __fdiv_rn(a, b); }
  static __device__ __forceinline__ float sqrt(float a) { return __fsqrt_rn(a); }
  static __device__ __forceinline__ float mx(float a, float b) { return fmaxf(a, b); }
  static __device__ __forceinline__ float mn(float a, float b) { return fminf(a, b); }
  static __device__ __forceinline__ float ab(float a) { return fabsf(a); }
};
template <> struct IEEE<double> {
  static __device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
  static __device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
  static __device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
  static __device__ __forceinline__ double div(double a, double b) { return __ddiv_rn(a, b); }
  static __device__ __forceinline__ double sqrt(double a) { return __dsqrt_rn(a); }
  static __device__ __forceinline__ double mx(double a, double b) { return fmax(a, b); }
  static __device__ __forceinline__ double mn(double a, double b) { return fmin(a, b); }
  static __device__ __forceinline__ double ab(double a) { return fabs(a); }
};

// Scalars of one step.  gm1 = gamma - 1 rounded in T (the reference traces
// gamma as a float32 and evaluates gamma - 1 in float32, fluid.py:53).
template <typename T>
struct StepConsts {
  T g;       // gamma
  T gm1;     // gamma - 1
  T igm1;    // 1 / (gamma - 1)       (FastPolicy only)
  T inv_dx;  // 1 / dx, fluid.py:547
  T dt;      // time step
  T k;       // dt * inv_dx           (FastPolicy only)
};

// fluid.py:47-53 / :231-237: E = p/(g-1) + 0.5*rho*sqrt(vx^2+vy^2+vz^2)**2
template <typename T>
__device__ __forceinline__ T exact_energy(T rho, T vx, T vy, T vz, T p, const StepConsts<T>& k) {
  using O = IEEE<T>;
  T ut = O::sqrt(O::add(O::add(O::mul(vx, vx), O::mul(vy, vy)), O::mul(vz, vz)));
  return O::add(O::div(p, k.gm1), O::mul(O::mul(T(0.5), rho), O::mul(ut, ut)));
}

// fluid.py:117: c = sqrt(gamma*p/rho)
template <typename T>
__device__ __forceinline__ T exact_sound(T rho, T p, T g) {
  using O = IEEE<T>;
  return O::sqrt(O::div(O::mul(g, p), rho));
}

// Maximum of two wave speeds that keeps NaN, like jnp.max/jnp.maximum.
// Speeds are >= +0 or NaN, so the unsigned order of their bit patterns is
// their numeric order with every NaN above +Inf.
__device__ __forceinline__ float speed_max(float a, float b) {
  return __uint_as_float(max(__float_as_uint(a), __float_as_uint(b)));
}
__device__ __forceinline__ double speed_max(double a, double b) {
  return __longlong_as_double((long long)max((unsigned long long)__double_as_longlong(a),
                                             (unsigned long long)__double_as_longlong(b)));
}

// max over the three axes of |v_d| + c for one primitive cell.  Its maximum
// over all cells equals the interface maximum of fluid.py:457-500 bit for bit
// (each cell is the right state of one periodic interface and the left state
// of the next, c >= 0, and max(u+c, c-u) rounds to |u|+c).
template <typename T>
__device__ __forceinline__ T exact_cell_speed(const T w[5], T g) {
  using O = IEEE<T>;
  T c = exact_sound(w[0], w[4], g);
  T m = O::add(O::ab(w[1]), c);
  m = speed_max(m, O::add(O::ab(w[2]), c));
  m = speed_max(m, O::add(O::ab(w[3]), c));
  return m;
}

// fluid.py:30-67
template <typename T>
__device__ __forceinline__ void exact_cons_from_prim(const T w[5], T U[5], const StepConsts<T>& k) {
  using O = IEEE<T>;
  T rho = w[0];
  U[4] = exact_energy(rho, w[1], w[2], w[3], w[4], k);
  U[0] = rho;
  U[1] = O::mul(rho, w[1]);
  U[2] = O::mul(rho, w[2]);
  U[3] = O::mul(rho, w[3]);
}

// fluid.py:71-103
template <typename T>
__device__ __forceinline__ void exact_prim_from_cons(const T U[5], T w[5], const StepConsts<T>& k) {
  using O = IEEE<T>;
  T rho = U[0], E = U[4];
  T ux = O::div(U[1], rho), uy = O::div(U[2], rho), uz = O::div(U[3], rho);
  T u = O::sqrt(O::add(O::add(O::mul(ux, ux), O::mul(uy, uy)), O::mul(uz, uz)));
  T p = O::mul(O::mul(k.gm1, rho), O::sub(O::div(E, rho), O::mul(T(0.5), O::mul(u, u))));
  w[0] = rho;
  w[1] = ux;
  w[2] = uy;
  w[3] = uz;
  w[4] = p;
}

// ---------------------------------------------------------------------------
// ExactPolicy: reference op order; state = primitive.
// ---------------------------------------------------------------------------
template <typename T>
struct ExactPolicy {
  using real = T;
  static constexpr bool kExact = true;

  static __device__ __forceinline__ void to_state(const T w[5], T s[5], const StepConsts<T>&) {
#pragma unroll
    for (int i = 0; i < 5; ++i) s[i] = w[i];
  }
  static __device__ __forceinline__ void to_prim(const T s[5], T w[5], const StepConsts<T>&) {
#pragma unroll
    for (int i = 0; i < 5; ++i) w[i] = s[i];
  }

  // fluid.py:517 (U = cons(W)) and fluid.py:225-257 (_euler_flux)
  template <int VEL>
  static __device__ __forceinline__ void derive(const T w[5], Cell<T>& o, const StepConsts<T>& k) {
    using O = IEEE<T>;
    T rho = w[0], p = w[4];
    T E = exact_energy(rho, w[1], w[2], w[3], p, k);
    T ud = w[VEL];
    o.U[0] = rho;
    o.U[1] = O::mul(rho, w[1]);
    o.U[2] = O::mul(rho, w[2]);
    o.U[3] = O::mul(rho, w[3]);
    o.U[4] = E;
    o.F[0] = O::mul(ud, rho);
    o.F[1] = O::mul(ud, O::mul(w[1], rho));
    o.F[2] = O::mul(ud, O::mul(w[2], rho));
    o.F[3] = O::mul(ud, O::mul(w[3], rho));
    o.F[4] = O::mul(ud, O::add(p, E));
    o.F[VEL] = O::add(o.F[VEL], p);
    o.wa = ud;
    o.wb = exact_sound(rho, p, k.g);
  }

  // derive() of an input cell: the state is primitive, like the input
  template <int VEL>
  static __device__ __forceinline__ void derive_in(const T w[5], Cell<T>& o,
                                                   const StepConsts<T>& k) {
    derive<VEL>(w, o, k);
  }

  // fluid.py:282-303
  static __device__ __forceinline__ void hll(const Cell<T>& L, const Cell<T>& R, T F[5]) {
    using O = IEEE<T>;
    T sp = O::mx(O::mx(O::add(L.wa, L.wb), O::add(R.wa, R.wb)), T(0));
    T sm = O::mn(O::mn(O::sub(L.wa, L.wb), O::sub(R.wa, R.wb)), T(0));
    T smsp = O::mul(sm, sp);
    T den = O::sub(sp, sm);
#pragma unroll
    for (int i = 0; i < 5; ++i) {
      T num = O::add(O::sub(O::mul(sp, L.F[i]), O::mul(sm, R.F[i])),
                     O::mul(smsp, O::sub(R.U[i], L.U[i])));
      F[i] = O::div(num, den);
    }
  }

  // fluid.py:547-555: U + (1/dx)*(F_lo - F_hi)*dt, then back to primitive.
  static __device__ __forceinline__ void update(const Cell<T>& C, const T flo[5], const T fhi[5],
                                                T s_out[5], const StepConsts<T>& k) {
    using O = IEEE<T>;
    T U[5];
#pragma unroll
    for (int i = 0; i < 5; ++i)
      U[i] = O::add(C.U[i], O::mul(O::mul(k.inv_dx, O::sub(flo[i], fhi[i])), k.dt));
    exact_prim_from_cons(U, s_out, k);
  }

  // Primitive output (the state itself) and its CFL speed, fluid.py:427-500.
  static __device__ __forceinline__ T finish(const T s[5], T w[5], const StepConsts<T>& k) {
#pragma unroll
    for (int i = 0; i < 5; ++i) w[i] = s[i];
    return exact_cell_speed(w, k.g);
  }
};

// ---------------------------------------------------------------------------
// FastPolicy: conserved state between sweeps, FMAs, one reciprocal per cell
// and per interface.
// ---------------------------------------------------------------------------
struct FastPolicy {
  using real = float;
  static constexpr bool kExact = false;

  // Single-instruction (MUFU) reciprocal and square root from the PTX ISA:
  // rcp.approx / sqrt.approx, max error about 1 ulp; operands here are normal
  // positive floats (densities, pressures, wave-speed sums).
  static __device__ __forceinline__ float rcp(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
  }
  static __device__ __forceinline__ float sqrt_(float x) {
    float r;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
  }

  static __device__ __forceinline__ void to_state(const float w[5], float U[5],
                                                  const StepConsts<float>& k) {
    float rho = w[0];
    float q = fmaf(w[1], w[1], fmaf(w[2], w[2], w[3] * w[3]));
    U[0] = rho;
    U[1] = rho * w[1];
    U[2] = rho * w[2];
    U[3] = rho * w[3];
    U[4] = fmaf(w[4], k.igm1, 0.5f * rho * q);
  }
  static __device__ __forceinline__ void to_prim(const float U[5], float w[5],
                                                 const StepConsts<float>& k) {
    float ir = rcp(U[0]);
    float vx = U[1] * ir, vy = U[2] * ir, vz = U[3] * ir;
    float ke = 0.5f * fmaf(U[1], vx, fmaf(U[2], vy, U[3] * vz));
    w[0] = U[0];
    w[1] = vx;
    w[2] = vy;
    w[3] = vz;
    w[4] = k.gm1 * (U[4] - ke);
  }

  template <int VEL>
  static __device__ __forceinline__ void derive(const float U[5], Cell<float>& o,
                                                const StepConsts<float>& k) {
    float ir = rcp(U[0]);
    float ud = U[VEL] * ir;
    float q = fmaf(U[1], U[1], fmaf(U[2], U[2], U[3] * U[3]));
    float p = k.gm1 * fmaf(-0.5f * q, ir, U[4]);
#pragma unroll
    for (int i = 0; i < 5; ++i) o.U[i] = U[i];
    o.F[0] = U[VEL];
    o.F[1] = U[1] * ud;
    o.F[2] = U[2] * ud;
    o.F[3] = U[3] * ud;
    o.F[4] = (U[4] + p) * ud;
    o.F[VEL] = fmaf(U[VEL], ud, p);
    const float c = sqrt_(k.g * p * ir);
    o.wa = ud + c;
    o.wb = c - ud;
  }

  // derive() of a PRIMITIVE input cell (the first sweep of a step): U is
  // to_state(w), and the normal velocity and the pressure are the input's own
  // (no reconstruction from U).
  template <int VEL>
  static __device__ __forceinline__ void derive_in(const float w[5], Cell<float>& o,
                                                   const StepConsts<float>& k) {
    to_state(w, o.U, k);
    const float ud = w[VEL], p = w[4];
    o.F[0] = o.U[VEL];
    o.F[1] = o.U[1] * ud;
    o.F[2] = o.U[2] * ud;
    o.F[3] = o.U[3] * ud;
    o.F[4] = (o.U[4] + p) * ud;
    o.F[VEL] = fmaf(o.U[VEL], ud, p);
    const float c = sqrt_(k.g * p * rcp(w[0]));
    o.wa = ud + c;
    o.wb = c - ud;
  }

  // HLL with ns = -S- = max(c_L - u_L, c_R - u_R, 0) (exactly the negated
  // min of the reference's form): F = a F_L + b F_R + s (U_L - U_R) with
  // a = S+/(S+ + ns), b = ns/(S+ + ns), s = ns a.
  static __device__ __forceinline__ void hll(const Cell<float>& L, const Cell<float>& R,
                                             float F[5]) {
    float sp = fmaxf(fmaxf(L.wa, R.wa), 0.f);
    float ns = fmaxf(fmaxf(L.wb, R.wb), 0.f);
    float inv = rcp(sp + ns);
    float a = sp * inv, b = ns * inv, s = ns * a;
#pragma unroll
    for (int i = 0; i < 5; ++i)
      F[i] = fmaf(a, L.F[i], fmaf(b, R.F[i], s * (L.U[i] - R.U[i])));
  }

  static __device__ __forceinline__ void update(const Cell<float>& C, const float flo[5],
                                                const float fhi[5], float s_out[5],
                                                const StepConsts<float>& k) {
#pragma unroll
    for (int i = 0; i < 5; ++i) s_out[i] = fmaf(k.k, flo[i] - fhi[i], C.U[i]);
  }

  // CFL speed max_d |v_d| + c of a stored primitive cell, computed exactly
  // as finish() computes it for the cell it stores (same ir and p), so a run
  // restarted from a stored state reproduces the uninterrupted dt sequence.
  static __device__ __forceinline__ float cell_speed(const float w[5], float g) {
    float ir = rcp(w[0]);
    float c = sqrt_(g * w[4] * ir);
    return speed_max(speed_max(fabsf(w[1]), fabsf(w[2])), fabsf(w[3])) + c;
  }

  // Primitive output of a conserved state and its CFL speed max_d |v_d| + c.
  static __device__ __forceinline__ float finish(const float U[5], float w[5],
                                                 const StepConsts<float>& k) {
    float ir = rcp(U[0]);
    float vx = U[1] * ir, vy = U[2] * ir, vz = U[3] * ir;
    float ke = 0.5f * fmaf(U[1], vx, fmaf(U[2], vy, U[3] * vz));
    float p = k.gm1 * (U[4] - ke);
    w[0] = U[0];
    w[1] = vx;
    w[2] = vy;
    w[3] = vz;
    w[4] = p;
    float c = sqrt_(k.g * p * ir);
    return speed_max(speed_max(fabsf(vx), fabsf(vy)), fabsf(vz)) + c;
  }
};

}  // namespace tf
