// Two-cell ("pair") form of the step arithmetic.  Every thread of the fused
// kernel owns two vertically adjacent cells (rows y and y+1 of one z column)
// and evaluates both with the same instruction stream:
//
//  * FastPair: sm_100+ packed float32x2 instructions (fma/add/mul .f32x2)
//    carry both cells at once, halving the issue slots of the FP32 math;
//    min/max and the MUFU reciprocal/square root act per component.  The op
//    sequence is exactly FastPolicy's (tf_math.cuh), so results are
//    bit-identical to evaluating FastPolicy on each cell.
//  * ExactPair: the reference's op order per component with IEEE intrinsics
//    (ExactPolicy), bit-identical to the float32 oracle.
#pragma once
#include <cuda_runtime.h>

#include "tf_math.cuh"

namespace tf {

typedef float2 V2;

// Cell<float> of two cells (see Cell in tf_math.cuh for wa / wb).
struct Cell2 {
  V2 U[5];
  V2 F[5];
  V2 wa;
  V2 wb;
};

__device__ __forceinline__ V2 v2(float x, float y) { return make_float2(x, y); }
__device__ __forceinline__ V2 splat(float x) { return make_float2(x, x); }

// Accessor view of a Cell2 in registers (the left cell of hll_from).
struct CellRef2 {
  const Cell2& c;
  __device__ __forceinline__ V2 wa() const { return c.wa; }
  __device__ __forceinline__ V2 wb() const { return c.wb; }
  __device__ __forceinline__ V2 U(int i) const { return c.U[i]; }
  __device__ __forceinline__ V2 F(int i) const { return c.F[i]; }
};

// ---------------------------------------------------------------------------
// FastPair
// ---------------------------------------------------------------------------
struct FastPair {
  static constexpr bool kExact = false;
  static __device__ __forceinline__ V2 add(V2 a, V2 b) { return __fadd2_rn(a, b); }
  static __device__ __forceinline__ V2 mul(V2 a, V2 b) { return __fmul2_rn(a, b); }
  static __device__ __forceinline__ V2 fma(V2 a, V2 b, V2 c) { return __ffma2_rn(a, b, c); }
  // a - b rounded once: b * (-1) is exact
  static __device__ __forceinline__ V2 sub(V2 a, V2 b) { return __ffma2_rn(b, splat(-1.f), a); }
  static __device__ __forceinline__ V2 vmax(V2 a, V2 b) { return v2(fmaxf(a.x, b.x), fmaxf(a.y, b.y)); }
  static __device__ __forceinline__ V2 vmin(V2 a, V2 b) { return v2(fminf(a.x, b.x), fminf(a.y, b.y)); }
  static __device__ __forceinline__ V2 rcp(V2 a) { return v2(FastPolicy::rcp(a.x), FastPolicy::rcp(a.y)); }
  static __device__ __forceinline__ V2 sqrt_(V2 a) {
    return v2(FastPolicy::sqrt_(a.x), FastPolicy::sqrt_(a.y));
  }

  static __device__ __forceinline__ void to_state(const V2 w[5], V2 U[5], const StepConsts<float>& k) {
    V2 rho = w[0];
    V2 q = fma(w[1], w[1], fma(w[2], w[2], mul(w[3], w[3])));
    U[0] = rho;
    U[1] = mul(rho, w[1]);
    U[2] = mul(rho, w[2]);
    U[3] = mul(rho, w[3]);
    U[4] = fma(w[4], splat(k.igm1), mul(mul(splat(0.5f), rho), q));
  }

  template <int VEL>
  static __device__ __forceinline__ void derive(const V2 U[5], Cell2& o, const StepConsts<float>& k) {
    V2 ir = rcp(U[0]);
    V2 ud = mul(U[VEL], ir);
    V2 q = fma(U[1], U[1], fma(U[2], U[2], mul(U[3], U[3])));
    V2 p = mul(splat(k.gm1), fma(mul(splat(-0.5f), q), ir, U[4]));
#pragma unroll
    for (int i = 0; i < 5; ++i) o.U[i] = U[i];
    o.F[0] = U[VEL];
    o.F[1] = mul(U[1], ud);
    o.F[2] = mul(U[2], ud);
    o.F[3] = mul(U[3], ud);
    o.F[4] = mul(add(U[4], p), ud);
    o.F[VEL] = fma(U[VEL], ud, p);
    const V2 c = sqrt_(mul(mul(splat(k.g), p), ir));
    o.wa = add(ud, c);
    o.wb = sub(c, ud);
  }

  // FastPolicy::derive_in on both cells (primitive input)
  template <int VEL>
  static __device__ __forceinline__ void derive_in(const V2 w[5], Cell2& o,
                                                   const StepConsts<float>& k) {
    to_state(w, o.U, k);
    const V2 ud = w[VEL], p = w[4];
    o.F[0] = o.U[VEL];
    o.F[1] = mul(o.U[1], ud);
    o.F[2] = mul(o.U[2], ud);
    o.F[3] = mul(o.U[3], ud);
    o.F[4] = mul(add(o.U[4], p), ud);
    o.F[VEL] = fma(o.U[VEL], ud, p);
    const V2 c = sqrt_(mul(mul(splat(k.g), p), rcp(w[0])));
    o.wa = add(ud, c);
    o.wb = sub(c, ud);
  }

  // FastPolicy::hll on both cells
  static __device__ __forceinline__ void hll(const Cell2& L, const Cell2& R, V2 F[5]) {
    hll_from(CellRef2{L}, CellRef2{R}, F);
  }
  // The same, with the cells read through accessors (wa(), wb(), U(i), F(i))
  // at the point of use -- for cells held in shared memory or in another
  // lane, so that their values need registers only briefly.
  template <class LC, class RC>
  static __device__ __forceinline__ void hll_from(const LC& L, const RC& R, V2 F[5]) {
    V2 sp = vmax(vmax(L.wa(), R.wa()), splat(0.f));
    V2 ns = vmax(vmax(L.wb(), R.wb()), splat(0.f));
    V2 inv = rcp(add(sp, ns));
    V2 a = mul(sp, inv), b = mul(ns, inv);
    V2 s = mul(ns, a);
#pragma unroll
    for (int i = 0; i < 5; ++i) F[i] = fma(a, L.F(i), fma(b, R.F(i), mul(s, sub(L.U(i), R.U(i)))));
  }

  static __device__ __forceinline__ void update(const Cell2& C, const V2 flo[5], const V2 fhi[5],
                                                V2 s_out[5], const StepConsts<float>& k) {
#pragma unroll
    for (int i = 0; i < 5; ++i) s_out[i] = fma(splat(k.k), sub(flo[i], fhi[i]), C.U[i]);
  }

  // primitive output and the CFL speed of each cell (FastPolicy::finish)
  static __device__ __forceinline__ V2 finish(const V2 U[5], V2 w[5], const StepConsts<float>& k) {
    V2 ir = rcp(U[0]);
    V2 vx = mul(U[1], ir), vy = mul(U[2], ir), vz = mul(U[3], ir);
    V2 ke = mul(splat(0.5f), fma(U[1], vx, fma(U[2], vy, mul(U[3], vz))));
    V2 p = mul(splat(k.gm1), sub(U[4], ke));
    w[0] = U[0];
    w[1] = vx;
    w[2] = vy;
    w[3] = vz;
    w[4] = p;
    V2 c = sqrt_(mul(mul(splat(k.g), p), ir));
    V2 m = v2(speed_max(speed_max(fabsf(vx.x), fabsf(vy.x)), fabsf(vz.x)),
              speed_max(speed_max(fabsf(vx.y), fabsf(vy.y)), fabsf(vz.y)));
    return add(m, c);
  }
};

// FastPair on conserved input and output: the fused step on states that are
// already conserved (the adjoint's forward passes).  Same operations as
// FastPair between the two conversions, so a step equals the three
// conserved-in/out fast sweeps bit for bit.  The CFL speed is not formed.
struct FastPairConserved : FastPair {
  static __device__ __forceinline__ void to_state(const V2 w[5], V2 U[5], const StepConsts<float>&) {
#pragma unroll
    for (int i = 0; i < 5; ++i) U[i] = w[i];
  }
  template <int VEL>
  static __device__ __forceinline__ void derive_in(const V2 U[5], Cell2& o,
                                                   const StepConsts<float>& k) {
    FastPair::derive<VEL>(U, o, k);
  }
  static __device__ __forceinline__ V2 finish(const V2 U[5], V2 w[5], const StepConsts<float>&) {
#pragma unroll
    for (int i = 0; i < 5; ++i) w[i] = U[i];
    return splat(0.f);
  }
};

// ---------------------------------------------------------------------------
// ExactPair: ExactPolicy<float> on each component.
// ---------------------------------------------------------------------------
struct ExactPair {
  static constexpr bool kExact = true;
  typedef ExactPolicy<float> E;

  static __device__ __forceinline__ Cell<float> lo(const Cell2& c) {
    Cell<float> r;
#pragma unroll
    for (int i = 0; i < 5; ++i) { r.U[i] = c.U[i].x; r.F[i] = c.F[i].x; }
    r.wa = c.wa.x;
    r.wb = c.wb.x;
    return r;
  }
  static __device__ __forceinline__ Cell<float> hi(const Cell2& c) {
    Cell<float> r;
#pragma unroll
    for (int i = 0; i < 5; ++i) { r.U[i] = c.U[i].y; r.F[i] = c.F[i].y; }
    r.wa = c.wa.y;
    r.wb = c.wb.y;
    return r;
  }
  static __device__ __forceinline__ void join(Cell2& o, const Cell<float>& a, const Cell<float>& b) {
#pragma unroll
    for (int i = 0; i < 5; ++i) { o.U[i] = v2(a.U[i], b.U[i]); o.F[i] = v2(a.F[i], b.F[i]); }
    o.wa = v2(a.wa, b.wa);
    o.wb = v2(a.wb, b.wb);
  }
  static __device__ __forceinline__ void split(const V2 s[5], float a[5], float b[5]) {
#pragma unroll
    for (int i = 0; i < 5; ++i) { a[i] = s[i].x; b[i] = s[i].y; }
  }
  static __device__ __forceinline__ void merge(V2 s[5], const float a[5], const float b[5]) {
#pragma unroll
    for (int i = 0; i < 5; ++i) s[i] = v2(a[i], b[i]);
  }

  static __device__ __forceinline__ void to_state(const V2 w[5], V2 U[5], const StepConsts<float>&) {
#pragma unroll
    for (int i = 0; i < 5; ++i) U[i] = w[i];
  }
  template <int VEL>
  static __device__ __forceinline__ void derive_in(const V2 s[5], Cell2& o,
                                                   const StepConsts<float>& k) {
    derive<VEL>(s, o, k);
  }
  template <int VEL>
  static __device__ __forceinline__ void derive(const V2 s[5], Cell2& o, const StepConsts<float>& k) {
    float a[5], b[5];
    split(s, a, b);
    Cell<float> ca, cb;
    E::template derive<VEL>(a, ca, k);
    E::template derive<VEL>(b, cb, k);
    join(o, ca, cb);
  }
  static __device__ __forceinline__ void hll(const Cell2& L, const Cell2& R, V2 F[5]) {
    float fa[5], fb[5];
    E::hll(lo(L), lo(R), fa);
    E::hll(hi(L), hi(R), fb);
    merge(F, fa, fb);
  }
  template <class LC, class RC>
  static __device__ __forceinline__ void hll_from(const LC& L, const RC& R, V2 F[5]) {
    Cell2 l, r;
#pragma unroll
    for (int i = 0; i < 5; ++i) {
      l.U[i] = L.U(i);
      l.F[i] = L.F(i);
      r.U[i] = R.U(i);
      r.F[i] = R.F(i);
    }
    l.wa = L.wa();
    l.wb = L.wb();
    r.wa = R.wa();
    r.wb = R.wb();
    hll(l, r, F);
  }
  static __device__ __forceinline__ void update(const Cell2& C, const V2 flo[5], const V2 fhi[5],
                                                V2 s_out[5], const StepConsts<float>& k) {
    float la[5], lb[5], ha[5], hb[5], oa[5], ob[5];
    split(flo, la, lb);
    split(fhi, ha, hb);
    E::update(lo(C), la, ha, oa, k);
    E::update(hi(C), lb, hb, ob, k);
    merge(s_out, oa, ob);
  }
  static __device__ __forceinline__ V2 finish(const V2 s[5], V2 w[5], const StepConsts<float>& k) {
#pragma unroll
    for (int i = 0; i < 5; ++i) w[i] = s[i];
    float a[5], b[5];
    split(s, a, b);
    return v2(exact_cell_speed(a, k.g), exact_cell_speed(b, k.g));
  }
};

}  // namespace tf
