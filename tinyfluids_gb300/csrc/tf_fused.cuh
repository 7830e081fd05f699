// The fused time-step kernel: open-BC remap, the x, y and z HLL sweeps of
// fluid.py:562-578 and the max-wave-speed reduction of the next dt
// (fluid.py:427-504) in ONE pass over the state.
//
// Decomposition.  Dimensional splitting means the y sweep reads x-updated
// neighbours and the z sweep reads y-updated ones, but each dependency is one
// cell wide.  A CTA owns a (y, z) tile and MARCHES along x (the slowest axis)
// through a chunk of planes.  Each thread owns a PAIR of cells -- rows 2w and
// 2w+1 of the tile in one z column -- and evaluates both with one instruction
// stream (tf_pair.cuh: packed f32x2 arithmetic in the fast policy).
//
//  * x sweep: a thread keeps, in registers, the previous plane's cell
//    quantities and the flux at the face x-1/2 of its two columns.  A plane
//    costs one load per cell, one new face flux and one update; nothing is
//    exchanged between threads.  Planes x+2 and x+3 are in flight while x is
//    computed.
//  * y sweep: the face between a thread's two rows is local; the face above
//    needs the previous warp's lower cell and the face below is computed by
//    the next warp, both through shared memory (two barriers per plane).
//  * z sweep: lane l holds column z0-1+l, so z neighbours are one lane apart
//    and are exchanged with warp shuffles.
//
// The tile is 32 lanes wide and 2*NWP rows high, including a one-cell ring
// (lanes 0 and 31, the first and last row) that is swept but not stored; the
// CTA stores 30 x (2*NWP-2) cells per plane.  Every load index is wrapped
// periodically in-kernel (and clamped for open boundaries), so ragged edge
// tiles and any nx, ny, nz >= 1 need no padding.
//
// The epilogue of each stored cell computes max_d |v_d| + c of the NEW state
// (the next step's CFL speed).  Its CTA maximum goes to the control block; the
// CTA that finishes last turns it into the next dt.
#pragma once
#include "tf_common.cuh"
#include "tf_math.cuh"
#include "tf_pair.cuh"

namespace tf {

constexpr int kTileLanes = 32;          // lanes per tile row (z)
constexpr int kTileZ = kTileLanes - 2;  // stored z cells per tile row

struct FusedGeom {
  int nx, ny, nz;
  int tiles_z, tiles_y, tiles_x;  // tile grid
  int lx;                         // planes per x chunk
  int open_bc;                    // TF_FLAG_OPEN_BOUNDARIES set
};

// stored rows per tile for NWP warps (two rows per warp, minus the ring)
__host__ __device__ constexpr int tile_rows_out(int nwp) { return 2 * nwp - 2; }

template <int NWP>
struct FusedSmem {
  float4 cy[3][NWP][kTileLanes];  // lower cell of each thread's pair (U, F, u, c)
  float4 fy4[NWP][kTileLanes];    // face above each pair, components 0..3
  float fy1[NWP][kTileLanes];     // face above each pair, component 4
  float red[NWP];                 // block reduction
};

__device__ __forceinline__ void shfl_up_cell2(const Cell2& in, Cell2& out) {
#pragma unroll
  for (int i = 0; i < 5; ++i) {
    out.U[i].x = __shfl_up_sync(0xffffffffu, in.U[i].x, 1);
    out.U[i].y = __shfl_up_sync(0xffffffffu, in.U[i].y, 1);
    out.F[i].x = __shfl_up_sync(0xffffffffu, in.F[i].x, 1);
    out.F[i].y = __shfl_up_sync(0xffffffffu, in.F[i].y, 1);
  }
  out.u.x = __shfl_up_sync(0xffffffffu, in.u.x, 1);
  out.u.y = __shfl_up_sync(0xffffffffu, in.u.y, 1);
  out.c.x = __shfl_up_sync(0xffffffffu, in.c.x, 1);
  out.c.y = __shfl_up_sync(0xffffffffu, in.c.y, 1);
}

// One CTA-tile of the fused step.  Returns this thread's running maximum of
// the stored cells' wave speeds (0 for threads that store nothing).
// COHERENT selects L2-only loads (ld.global.cg) for kernels that read data
// other CTAs wrote earlier in the same launch (the persistent batch kernel);
// otherwise loads use the read-only path.
template <class P, int NWP, bool COHERENT = false>
__device__ __forceinline__ float fused_tile(const float* __restrict__ src, float* __restrict__ dst,
                                            const FusedGeom& G, int tz, int ty, int tx,
                                            const StepConsts<float>& K, FusedSmem<NWP>& sm) {
  const int lane = threadIdx.x & 31;
  const int w = threadIdx.x >> 5;
  const bool open = G.open_bc != 0;
  const int z0 = tz * kTileZ, y0 = ty * tile_rows_out(NWP);
  const int x0 = tx * G.lx;
  const int x_end = min(x0 + G.lx, G.nx);
  const int z = z0 - 1 + lane;
  const int ya = y0 - 1 + 2 * w, yb = ya + 1;  // the thread's two rows
  const size_t plane = (size_t)G.ny * G.nz;
  const size_t vstride = plane * G.nx;
  const int zs = src_index(z, G.nz, open);
  const size_t col_a = (size_t)src_index(ya, G.ny, open) * G.nz + zs;
  const size_t col_b = (size_t)src_index(yb, G.ny, open) * G.nz + zs;
  const bool store_lane = lane >= 1 && lane <= kTileLanes - 2 && z < G.nz;
  const bool store_a = store_lane && w >= 1 && ya < G.ny;
  const bool store_b = store_lane && w <= NWP - 2 && yb < G.ny;
  const size_t dcol_a = store_a ? (size_t)ya * G.nz + z : 0;
  const size_t dcol_b = store_b ? (size_t)yb * G.nz + z : 0;

  auto load = [&](int x, V2 v[5]) {
    const float* p = src + (size_t)src_index(x, G.nx, open) * plane;
#pragma unroll
    for (int i = 0; i < 5; ++i) {
      const float* q = p + i * vstride;
      v[i].x = COHERENT ? __ldcg(q + col_a) : __ldg(q + col_a);
      v[i].y = COHERENT ? __ldcg(q + col_b) : __ldg(q + col_b);
    }
  };

  float wmax = 0.f;
  Cell2 cur;
  V2 fm[5];
  V2 pa[5], pb[5];
  {
    V2 w0[5], s[5];
    load(x0 - 1, w0);
    load(x0, pa);
    load(x0 + 1, pb);
    P::to_state(w0, s, K);
    P::template derive<1>(s, cur, K);
    Cell2 nx_;
    P::to_state(pa, s, K);
    P::template derive<1>(s, nx_, K);
    if (x0 + 2 <= x_end) load(x0 + 2, pa);
    P::hll(cur, nx_, fm);  // flux at face x0 - 1/2
    cur = nx_;
  }

  // One plane: x sweep from registers, then y and z sweeps, store, epilogue.
  // `pf` holds plane x+1 on entry and receives plane x+3.
  auto plane_step = [&](int x, V2 pf[5]) {
    V2 s[5];
    Cell2 nxt;
    P::to_state(pf, s, K);
    P::template derive<1>(s, nxt, K);
    if (x + 3 <= x_end) load(x + 3, pf);
    V2 fp[5];
    P::hll(cur, nxt, fp);  // face x + 1/2
    V2 s1[5];
    P::update(cur, fm, fp, s1, K);

    // ---- y sweep ----
    Cell2 cy;
    P::template derive<2>(s1, cy, K);
    sm.cy[0][w][lane] = make_float4(cy.U[0].y, cy.U[1].y, cy.U[2].y, cy.U[3].y);
    sm.cy[1][w][lane] = make_float4(cy.U[4].y, cy.F[0].y, cy.F[1].y, cy.F[2].y);
    sm.cy[2][w][lane] = make_float4(cy.F[3].y, cy.F[4].y, cy.u.y, cy.c.y);
    __syncthreads();
    // L = (cell above the pair, upper cell), R = (upper cell, lower cell):
    // faces (ya - 1/2, ya + 1/2).  Warp 0 has no cell above (its upper row
    // is the ring); it uses its own upper cell, and that face is never used.
    Cell2 L;
    {
      float4 a, b, d;
      if (w >= 1) {
        a = sm.cy[0][w - 1][lane];
        b = sm.cy[1][w - 1][lane];
        d = sm.cy[2][w - 1][lane];
      } else {
        a = make_float4(cy.U[0].x, cy.U[1].x, cy.U[2].x, cy.U[3].x);
        b = make_float4(cy.U[4].x, cy.F[0].x, cy.F[1].x, cy.F[2].x);
        d = make_float4(cy.F[3].x, cy.F[4].x, cy.u.x, cy.c.x);
      }
      L.U[0] = v2(a.x, cy.U[0].x); L.U[1] = v2(a.y, cy.U[1].x);
      L.U[2] = v2(a.z, cy.U[2].x); L.U[3] = v2(a.w, cy.U[3].x);
      L.U[4] = v2(b.x, cy.U[4].x); L.F[0] = v2(b.y, cy.F[0].x);
      L.F[1] = v2(b.z, cy.F[1].x); L.F[2] = v2(b.w, cy.F[2].x);
      L.F[3] = v2(d.x, cy.F[3].x); L.F[4] = v2(d.y, cy.F[4].x);
      L.u = v2(d.z, cy.u.x);       L.c = v2(d.w, cy.c.x);
    }
    V2 fy[5];
    P::hll(L, cy, fy);
    sm.fy4[w][lane] = make_float4(fy[0].x, fy[1].x, fy[2].x, fy[3].x);
    sm.fy1[w][lane] = fy[4].x;
    __syncthreads();
    // face below the pair = the next warp's face above its pair; the last
    // warp's lower row is the ring and takes its own value (unused)
    V2 fyh[5];
    {
      float4 f4;
      float f1;
      if (w <= NWP - 2) {
        f4 = sm.fy4[w + 1][lane];
        f1 = sm.fy1[w + 1][lane];
      } else {
        f4 = make_float4(fy[0].x, fy[1].x, fy[2].x, fy[3].x);
        f1 = fy[4].x;
      }
      fyh[0] = v2(fy[0].y, f4.x);
      fyh[1] = v2(fy[1].y, f4.y);
      fyh[2] = v2(fy[2].y, f4.z);
      fyh[3] = v2(fy[3].y, f4.w);
      fyh[4] = v2(fy[4].y, f1);
    }
    V2 s2[5];
    P::update(cy, fy, fyh, s2, K);

    // ---- z sweep ----
    Cell2 cz, nb;
    P::template derive<3>(s2, cz, K);
    shfl_up_cell2(cz, nb);
    V2 fzl[5], fzh[5];
    P::hll(nb, cz, fzl);  // faces between lanes l-1 and l, both rows
#pragma unroll
    for (int i = 0; i < 5; ++i) {
      fzh[i].x = __shfl_down_sync(0xffffffffu, fzl[i].x, 1);
      fzh[i].y = __shfl_down_sync(0xffffffffu, fzl[i].y, 1);
    }
    V2 s3[5], wo[5];
    P::update(cz, fzl, fzh, s3, K);
    const V2 sp = P::finish(s3, wo, K);
    float* q = dst + (size_t)x * plane;
    if (store_a) {
#pragma unroll
      for (int i = 0; i < 5; ++i) q[i * vstride + dcol_a] = wo[i].x;
      wmax = speed_max(wmax, sp.x);
    }
    if (store_b) {
#pragma unroll
      for (int i = 0; i < 5; ++i) q[i * vstride + dcol_b] = wo[i].y;
      wmax = speed_max(wmax, sp.y);
    }
#pragma unroll
    for (int i = 0; i < 5; ++i) fm[i] = fp[i];
    cur = nxt;
  };

  // Two planes per trip so the two prefetch buffers alternate without moves.
  for (int x = x0; x < x_end; x += 2) {
    plane_step(x, pb);
    if (x + 1 < x_end) plane_step(x + 1, pa);
  }
  return wmax;
}

}  // namespace tf
