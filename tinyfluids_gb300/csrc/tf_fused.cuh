// The fused time-step kernel: open-BC remap, the x, y and z HLL sweeps of
// fluid.py:562-578 and the max-wave-speed reduction of the next dt
// (fluid.py:427-504) in ONE pass over the state.
//
// Decomposition.  Dimensional splitting means the y sweep reads x-updated
// neighbours and the z sweep reads y-updated ones, but each dependency is one
// cell wide.  A CTA owns a (y, z) tile and MARCHES along x (the slowest axis)
// through a chunk of planes:
//
//  * x sweep: every thread owns one (y, z) column and keeps, in registers,
//    the previous plane's cell quantities and the flux at the face x-1/2.  A
//    plane costs one load per cell, one new face flux and one update; nothing
//    is exchanged between threads.  Planes x+2 and x+3 are in flight while x
//    is computed.
//  * y sweep: warp w holds row y0-1+w of the tile, so the y neighbours of a
//    cell live in the warps above and below; cell quantities and face fluxes
//    go through shared memory (two barriers per plane).
//  * z sweep: lane l holds column z0-1+l, so z neighbours are one lane apart
//    and are exchanged with warp shuffles.
//
// The tile is 32 lanes wide and NW rows high, including a one-cell ring
// (lanes 0 and 31, warps 0 and NW-1) that is swept but not stored; the CTA
// stores 30 x (NW-2) cells per plane.  Every load index is wrapped
// periodically in-kernel (and clamped for open boundaries), so ragged edge
// tiles and any nx, ny, nz >= 1 need no padding.
//
// The epilogue of each stored cell computes max_d |v_d| + c of the NEW state
// (the next step's CFL speed).  Its CTA maximum goes to the control block; the
// CTA that finishes last turns it into the next dt.
#pragma once
#include "tf_common.cuh"
#include "tf_math.cuh"

namespace tf {

constexpr int kTileLanes = 32;              // lanes per tile row (z)
constexpr int kTileZ = kTileLanes - 2;      // stored z cells per tile row

struct FusedGeom {
  int nx, ny, nz;
  int tiles_z, tiles_y, tiles_x;  // tile grid
  int lx;                         // planes per x chunk
  int open_bc;                    // TF_FLAG_OPEN_BOUNDARIES set
};

template <int NW>
struct FusedSmem {
  float4 cy[3][NW][kTileLanes];  // y-sweep cell quantities (U, F, u, c)
  float4 fy4[NW][kTileLanes];    // y face flux, components 0..3
  float fy1[NW][kTileLanes];     // y face flux, component 4
  float red[NW];                 // block reduction
};

template <typename T>
__device__ __forceinline__ void pack_cell(const Cell<T>& c, float4& a, float4& b, float4& d) {
  a = make_float4(c.U[0], c.U[1], c.U[2], c.U[3]);
  b = make_float4(c.U[4], c.F[0], c.F[1], c.F[2]);
  d = make_float4(c.F[3], c.F[4], c.u, c.c);
}
template <typename T>
__device__ __forceinline__ void unpack_cell(Cell<T>& c, const float4& a, const float4& b,
                                            const float4& d) {
  c.U[0] = a.x; c.U[1] = a.y; c.U[2] = a.z; c.U[3] = a.w;
  c.U[4] = b.x; c.F[0] = b.y; c.F[1] = b.z; c.F[2] = b.w;
  c.F[3] = d.x; c.F[4] = d.y; c.u = d.z;    c.c = d.w;
}

template <typename T>
__device__ __forceinline__ void shfl_up_cell(const Cell<T>& in, Cell<T>& out) {
#pragma unroll
  for (int i = 0; i < 5; ++i) {
    out.U[i] = __shfl_up_sync(0xffffffffu, in.U[i], 1);
    out.F[i] = __shfl_up_sync(0xffffffffu, in.F[i], 1);
  }
  out.u = __shfl_up_sync(0xffffffffu, in.u, 1);
  out.c = __shfl_up_sync(0xffffffffu, in.c, 1);
}

// One CTA-tile of the fused step.  Returns this thread's running maximum of
// the stored cells' wave speeds (0 for threads that store nothing).
// COHERENT selects L2-only loads (ld.global.cg) for kernels that read data
// other CTAs wrote earlier in the same launch (the persistent batch kernel);
// otherwise loads use the read-only path.
template <class P, int NW, bool COHERENT = false>
__device__ __forceinline__ float fused_tile(const float* __restrict__ src, float* __restrict__ dst,
                                            const FusedGeom& G, int tz, int ty, int tx,
                                            const StepConsts<float>& K, FusedSmem<NW>& sm) {
  const int lane = threadIdx.x & 31;
  const int w = threadIdx.x >> 5;
  const bool open = G.open_bc != 0;
  const int z0 = tz * kTileZ, y0 = ty * (NW - 2);
  const int x0 = tx * G.lx;
  const int x_end = min(x0 + G.lx, G.nx);
  const int z = z0 - 1 + lane, y = y0 - 1 + w;
  const size_t plane = (size_t)G.ny * G.nz;
  const size_t vstride = plane * G.nx;
  const size_t col_src = (size_t)src_index(y, G.ny, open) * G.nz + src_index(z, G.nz, open);
  const bool store_lane = lane >= 1 && lane <= kTileLanes - 2 && z < G.nz;
  const bool store_row = w >= 1 && w <= NW - 2 && y < G.ny;
  const bool stores = store_lane && store_row;
  const size_t col_dst = stores ? (size_t)y * G.nz + z : 0;

  auto load = [&](int x, float v[5]) {
    const float* p = src + (size_t)src_index(x, G.nx, open) * plane + col_src;
#pragma unroll
    for (int i = 0; i < 5; ++i) v[i] = COHERENT ? __ldcg(p + i * vstride) : __ldg(p + i * vstride);
  };

  float wmax = 0.f;
  Cell<float> cur;
  float fm[5];
  float pa[5], pb[5];
  {
    float w0[5], s[5];
    load(x0 - 1, w0);
    load(x0, pa);
    load(x0 + 1, pb);
    P::to_state(w0, s, K);
    P::template derive<1>(s, cur, K);
    Cell<float> nx_;
    P::to_state(pa, s, K);
    P::template derive<1>(s, nx_, K);
    if (x0 + 2 <= x_end) load(x0 + 2, pa);
    P::hll(cur, nx_, fm);  // flux at face x0 - 1/2
    cur = nx_;
  }

  // One plane: x sweep from registers, then y and z sweeps, store, epilogue.
  // `pf` holds plane x+1 on entry and receives plane x+3.
  auto plane_step = [&](int x, float pf[5]) {
    float s[5];
    Cell<float> nxt;
    P::to_state(pf, s, K);
    P::template derive<1>(s, nxt, K);
    if (x + 3 <= x_end) load(x + 3, pf);
    float fp[5];
    P::hll(cur, nxt, fp);  // face x + 1/2
    float s1[5];
    P::update(cur, fm, fp, s1, K);

    // ---- y sweep ----
    Cell<float> cy;
    P::template derive<2>(s1, cy, K);
    pack_cell(cy, sm.cy[0][w][lane], sm.cy[1][w][lane], sm.cy[2][w][lane]);
    __syncthreads();
    float fyl[5];
    if (w >= 1) {
      Cell<float> nb;
      unpack_cell(nb, sm.cy[0][w - 1][lane], sm.cy[1][w - 1][lane], sm.cy[2][w - 1][lane]);
      P::hll(nb, cy, fyl);  // face between rows w-1 and w
      sm.fy4[w][lane] = make_float4(fyl[0], fyl[1], fyl[2], fyl[3]);
      sm.fy1[w][lane] = fyl[4];
    }
    __syncthreads();
    if (w >= 1 && w <= NW - 2) {
      float fyh[5];
      float4 f4 = sm.fy4[w + 1][lane];
      fyh[0] = f4.x; fyh[1] = f4.y; fyh[2] = f4.z; fyh[3] = f4.w;
      fyh[4] = sm.fy1[w + 1][lane];
      float s2[5];
      P::update(cy, fyl, fyh, s2, K);

      // ---- z sweep ----
      Cell<float> cz, nb;
      P::template derive<3>(s2, cz, K);
      shfl_up_cell(cz, nb);
      float fzl[5], fzh[5];
      P::hll(nb, cz, fzl);  // face between lanes l-1 and l
#pragma unroll
      for (int i = 0; i < 5; ++i) fzh[i] = __shfl_down_sync(0xffffffffu, fzl[i], 1);
      float s3[5], wo[5];
      P::update(cz, fzl, fzh, s3, K);
      const float sp = P::finish(s3, wo, K);
      if (stores) {
        float* q = dst + (size_t)x * plane + col_dst;
#pragma unroll
        for (int i = 0; i < 5; ++i) q[i * vstride] = wo[i];
        wmax = speed_max(wmax, sp);
      }
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
