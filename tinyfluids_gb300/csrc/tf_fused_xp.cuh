// The fused time step with PLANE PAIRS: each thread owns one (y, z) column of
// a tile and advances two consecutive x planes per iteration, evaluating both
// with one packed (f32x2) instruction stream.
//
// Compared with the row-pair tile of tf_fused.cuh (a thread owns two rows of
// one plane):
//  * the x sweep carries one cell's quantities and one face flux (17 values,
//    not 34) from iteration to iteration; the face between the iteration's
//    two planes is local;
//  * each warp is one tile row, so every y face is between two warps: a warp
//    publishes its cells in shared memory and reads its upper neighbour's as
//    ready-made (plane x, plane x+1) pairs -- no re-pairing of registers --
//    and two CTA barriers serve two planes;
//  * the tile's two ring rows are whole warps (the first and the last), which
//    sweep along x and provide the edge y faces but skip the y update, the z
//    sweep and the stores.
// A CTA of NW warps covers NW rows (NW - 2 stored) by 32 lanes (30 stored),
// the same tile shape as the row-pair tile of NW / 2 warps, so the launch
// geometry (make_geom) is shared.  Per cell the operations are those of the
// row-pair tile (the same policy functions in the same order), so the results
// are the same bits.
#pragma once
#include "tf_fused.cuh"

namespace tf {

template <int NW>
struct FusedSmemXP {
  float4 cy[6][NW][kTileLanes];  // each warp's cells after the x sweep, y form (12 pairs)
  float4 fy[2][NW][kTileLanes];  // face above each warp's row, components 0..3 (pairs)
  float2 fy4[NW][kTileLanes];    // face above, component 4
  float red[NW];
};

// Cell2 <-> 6 float4 (pairs of the two planes, 2 values per float4)
__device__ __forceinline__ void pack_cell2(const Cell2& c, float4 q[6]) {
  q[0] = make_float4(c.U[0].x, c.U[0].y, c.U[1].x, c.U[1].y);
  q[1] = make_float4(c.U[2].x, c.U[2].y, c.U[3].x, c.U[3].y);
  q[2] = make_float4(c.U[4].x, c.U[4].y, c.F[0].x, c.F[0].y);
  q[3] = make_float4(c.F[1].x, c.F[1].y, c.F[2].x, c.F[2].y);
  q[4] = make_float4(c.F[3].x, c.F[3].y, c.F[4].x, c.F[4].y);
  q[5] = make_float4(c.wa.x, c.wa.y, c.wb.x, c.wb.y);
}
__device__ __forceinline__ void unpack_cell2(const float4 q[6], Cell2& c) {
  c.U[0] = v2(q[0].x, q[0].y); c.U[1] = v2(q[0].z, q[0].w);
  c.U[2] = v2(q[1].x, q[1].y); c.U[3] = v2(q[1].z, q[1].w);
  c.U[4] = v2(q[2].x, q[2].y); c.F[0] = v2(q[2].z, q[2].w);
  c.F[1] = v2(q[3].x, q[3].y); c.F[2] = v2(q[3].z, q[3].w);
  c.F[3] = v2(q[4].x, q[4].y); c.F[4] = v2(q[4].z, q[4].w);
  c.wa = v2(q[5].x, q[5].y);   c.wb = v2(q[5].z, q[5].w);
}

// One cell's quantities (the carried plane of the x sweep).
struct Cell1 {
  float U[5], F[5], wa, wb;
};
__device__ __forceinline__ void take_hi(const Cell2& c, Cell1& o) {
#pragma unroll
  for (int i = 0; i < 5; ++i) {
    o.U[i] = c.U[i].y;
    o.F[i] = c.F[i].y;
  }
  o.wa = c.wa.y;
  o.wb = c.wb.y;
}

// The fused tile with plane pairs.  Returns this thread's running maximum of
// the stored cells' wave speeds (0 for threads that store nothing).
// COHERENT: L2-only loads for kernels that read data other CTAs wrote in the
// same launch (not used by the single-step kernels).
template <class P, int NW, bool COHERENT = false>
__device__ __forceinline__ float fused_tile_xp(const float* __restrict__ src,
                                               float* __restrict__ dst, const FusedGeom& G,
                                               int tz, int ty, int tx,
                                               const StepConsts<float>& K,
                                               FusedSmemXP<NW>& sm) {
  const int lane = threadIdx.x & 31;
  const int w = threadIdx.x >> 5;
  const bool open = G.open_bc != 0;
  const int z0 = tz * kTileZ, y0 = ty * (NW - 2);
  const int x0 = tx * G.lx, x_end = min(x0 + G.lx, G.nx);
  const int z = z0 - 1 + lane, y = y0 - 1 + w;
  const size_t plane = (size_t)G.ny * G.nz, vstride = plane * G.nx;
  const size_t col = (size_t)src_index(y, G.ny, open) * G.nz + src_index(z, G.nz, open);
  const bool ring = w == 0 || w == NW - 1;  // warp-uniform
  const bool store = !ring && lane >= 1 && lane <= kTileLanes - 2 && z < G.nz && y < G.ny;
  const size_t dcol = store ? (size_t)y * G.nz + z : 0;
  float wmax = 0.f;

  auto ld = [&](const float* p) { return COHERENT ? __ldcg(p) : __ldg(p); };
  // planes (xa, xb) of this column as pairs
  auto load2 = [&](int xa, int xb, V2 v[5]) {
    const float* pa = src + (size_t)src_index(xa, G.nx, open) * plane + col;
    const float* pb = src + (size_t)src_index(xb, G.nx, open) * plane + col;
#pragma unroll
    for (int i = 0; i < 5; ++i) {
      v[i].x = ld(pa + i * vstride);
      v[i].y = ld(pb + i * vstride);
    }
  };

  // prologue: planes x0-1 and x0, the face x0 - 1/2, the carry (plane x0)
  Cell1 c;  // carried plane x: derived quantities for the x sweep
  float fm[5];  // flux at x - 1/2
  V2 pr[5];     // raw planes of the next iteration (x+1, x+2)
  {
    V2 r[5], s[5];
    load2(x0 - 1, x0, r);
    load2(x0 + 1, x0 + 2, pr);
    P::to_state(r, s, K);
    Cell2 d;
    P::template derive<1>(s, d, K);
    Cell2 L, R;
#pragma unroll
    for (int i = 0; i < 5; ++i) {
      L.U[i] = splat(d.U[i].x); L.F[i] = splat(d.F[i].x);
      R.U[i] = splat(d.U[i].y); R.F[i] = splat(d.F[i].y);
    }
    L.wa = splat(d.wa.x); L.wb = splat(d.wb.x);
    R.wa = splat(d.wa.y); R.wb = splat(d.wb.y);
    V2 f[5];
    P::hll(L, R, f);
#pragma unroll
    for (int i = 0; i < 5; ++i) fm[i] = f[i].x;
    take_hi(d, c);
  }

  for (int x = x0; x < x_end; x += 2) {
    // ---- x sweep of planes (x, x+1) ----
    V2 s[5];
    P::to_state(pr, s, K);
    Cell2 D;  // planes (x+1, x+2)
    P::template derive<1>(s, D, K);
    if (x + 2 < x_end) load2(x + 3, x + 4, pr);
    Cell2 L;  // planes (x, x+1)
#pragma unroll
    for (int i = 0; i < 5; ++i) {
      L.U[i] = v2(c.U[i], D.U[i].x);
      L.F[i] = v2(c.F[i], D.F[i].x);
    }
    L.wa = v2(c.wa, D.wa.x);
    L.wb = v2(c.wb, D.wb.x);
    V2 fx[5];  // faces (x + 1/2, x + 3/2)
    P::hll(L, D, fx);
    V2 flo[5], s1[5];
#pragma unroll
    for (int i = 0; i < 5; ++i) flo[i] = v2(fm[i], fx[i].x);
    P::update(L, flo, fx, s1, K);
    take_hi(D, c);
#pragma unroll
    for (int i = 0; i < 5; ++i) fm[i] = fx[i].y;

    // ---- y sweep ----
    Cell2 Y;
    P::template derive<2>(s1, Y, K);
    {
      float4 q[6];
      pack_cell2(Y, q);
#pragma unroll
      for (int k = 0; k < 6; ++k) sm.cy[k][w][lane] = q[k];
    }
    __syncthreads();
    V2 fa[5];  // face above this row
    if (w >= 1) {
      float4 q[6];
#pragma unroll
      for (int k = 0; k < 6; ++k) q[k] = sm.cy[k][w - 1][lane];
      Cell2 A;
      unpack_cell2(q, A);
      P::hll(A, Y, fa);
      sm.fy[0][w][lane] = make_float4(fa[0].x, fa[0].y, fa[1].x, fa[1].y);
      sm.fy[1][w][lane] = make_float4(fa[2].x, fa[2].y, fa[3].x, fa[3].y);
      sm.fy4[w][lane] = fa[4];
    }
    __syncthreads();
    if (ring) continue;  // warp-uniform: ring rows are not updated
    V2 fb[5];  // face below this row: the next row's face above
    {
      const float4 a = sm.fy[0][w + 1][lane], b = sm.fy[1][w + 1][lane];
      fb[0] = v2(a.x, a.y);
      fb[1] = v2(a.z, a.w);
      fb[2] = v2(b.x, b.y);
      fb[3] = v2(b.z, b.w);
      fb[4] = sm.fy4[w + 1][lane];
    }
    V2 s2[5];
    P::update(Y, fa, fb, s2, K);

    // ---- z sweep ----
    Cell2 cz, nb;
    P::template derive<3>(s2, cz, K);
    shfl_up_cell2(cz, nb);
    V2 fzl[5], fzh[5];
    P::hll(nb, cz, fzl);  // faces between lanes l-1 and l, both planes
#pragma unroll
    for (int i = 0; i < 5; ++i) {
      fzh[i].x = __shfl_down_sync(0xffffffffu, fzl[i].x, 1);
      fzh[i].y = __shfl_down_sync(0xffffffffu, fzl[i].y, 1);
    }
    V2 s3[5], wo[5];
    P::update(cz, fzl, fzh, s3, K);
    const V2 sp = P::finish(s3, wo, K);
    if (store) {
      float* q = dst + (size_t)x * plane + dcol;
#pragma unroll
      for (int i = 0; i < 5; ++i) q[i * vstride] = wo[i].x;
      wmax = speed_max(wmax, sp.x);
      if (x + 1 < x_end) {
#pragma unroll
        for (int i = 0; i < 5; ++i) q[plane + i * vstride] = wo[i].y;
        wmax = speed_max(wmax, sp.y);
      }
    }
  }
  return wmax;
}

}  // namespace tf
