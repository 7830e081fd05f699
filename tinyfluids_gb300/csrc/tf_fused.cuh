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
  int pairs8;  // y-marching tile: source and destination rows move z pairs as 8-byte units
};

// Per-variable base pointers of a launch's source and destination states
// (variable i of a [5][nx][ny][nz] state starts i * nx*ny*nz floats in), for
// kernels that receive them as launch parameters: an access is then a 32-bit
// element offset within one variable added to a parameter-space base, with
// no 64-bit address arithmetic per access.  Needs nx*ny*nz < 2^31.
struct VarPtrs {
  const float* s[5];
  float* d[5];
};

// The warp index through a shuffle from lane 0: provably the same in every
// lane of the warp, so branches on it need no convergence barriers.
__device__ __forceinline__ int uniform_warp_index() {
  return __shfl_sync(0xffffffffu, (int)(threadIdx.x >> 5), 0);
}

// stored rows per tile for NWP warps (two rows per warp, minus the ring)
__host__ __device__ constexpr int tile_rows_out(int nwp) { return 2 * nwp - 2; }

template <int NWP>
struct FusedSmem {
  float4 cy[3][NWP][kTileLanes];  // lower cell of each thread's pair (U, F, wa, wb)
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
  out.wa.x = __shfl_up_sync(0xffffffffu, in.wa.x, 1);
  out.wa.y = __shfl_up_sync(0xffffffffu, in.wa.y, 1);
  out.wb.x = __shfl_up_sync(0xffffffffu, in.wb.x, 1);
  out.wb.y = __shfl_up_sync(0xffffffffu, in.wb.y, 1);
}

// Per-thread context of one tile: store targets and the running CFL speed.
struct TileOut {
  const VarPtrs* vp;  // per-variable bases (launch parameters), or null
  float* dst;
  size_t plane, vstride, dcol_a, dcol_b;
  bool store_a, store_b;
  float wmax;
  // diagnostics (set only by the diagnostics instantiation)
  CSum acc[5];         // running sums of the stored cells' conserved variables
  float* slice;        // [2][nx][ny]: rho and p of the plane z == z_slice, or null
  size_t slice_plane;  // nx * ny
  int ny, sy_a, sy_b;  // y of cell a / b if it lies on the slice plane, else -1
};

// Diagnostics output of a fused step: conserved totals and, optionally, the
// density and pressure of one z plane (the reference's plot_results slice,
// scaling_jax.py:75-82).
struct DiagArgs {
  float* slice;
  int z_slice;
};

// Conserved variables of one stored primitive cell (the reference's
// conversion, fluid.py:30-67) into the running totals, and its slice values.
__device__ __forceinline__ void diag_cell(TileOut& o, int x, int sy, const V2 wo[5], bool hi,
                                          const StepConsts<float>& K) {
  float w[5], u[5];
#pragma unroll
  for (int i = 0; i < 5; ++i) w[i] = hi ? wo[i].y : wo[i].x;
  exact_cons_from_prim(w, u, K);
#pragma unroll
  for (int i = 0; i < 5; ++i) csum_add(o.acc[i], u[i]);
  if (sy >= 0) {
    const size_t j = (size_t)x * o.ny + sy;
    o.slice[j] = w[0];
    o.slice[o.slice_plane + j] = w[4];
  }
}

// Checked build (TF_CHECKED=1, a separate library used by the tests): every
// global load and store of the fused tile is range-checked -- an access
// outside the state is counted and skipped, never performed -- and every
// stored cell increments its entry of a caller-provided write-count array,
// so a test sees that each cell of a step is written exactly once (no two
// tiles store the same cell, none is missed).  The product build compiles
// none of this.
#ifndef TF_CHECKED
#define TF_CHECKED 0
#endif
#if TF_CHECKED
static __device__ unsigned long long g_chk_oob;
static __device__ int* g_chk_writes;
static __device__ long long g_chk_ncells;
#endif

template <bool VP = false>
__device__ __forceinline__ void store5(const TileOut& o, int x, size_t dcol, const V2 wo[5],
                                       bool hi) {
  if constexpr (VP && !TF_CHECKED) {
    const unsigned oc = (unsigned)x * (unsigned)o.plane + (unsigned)dcol;
#pragma unroll
    for (int i = 0; i < 5; ++i) o.vp->d[i][oc] = hi ? wo[i].y : wo[i].x;
    return;
  }
  float* q = o.dst + (size_t)x * o.plane + dcol;
#if TF_CHECKED
  const size_t cell = (size_t)x * o.plane + dcol;
  if (cell >= o.vstride) {
    atomicAdd(&g_chk_oob, 1ull);
    return;
  }
  if (g_chk_writes && (long long)cell < g_chk_ncells) atomicAdd(g_chk_writes + cell, 1);
#endif
#pragma unroll
  for (int i = 0; i < 5; ++i) q[i * o.vstride] = hi ? wo[i].y : wo[i].x;
}

// One plane of the fused step for the thread's pair of cells: the x sweep
// from registers (cur = plane x, pf = plane x+1, fm = flux at x-1/2), then
// the y and z sweeps, the store and the CFL epilogue.  `consumed()` runs as
// soon as pf has been read (the register-prefetch loader refills pf there);
// `after_sync()` runs after the plane's first CTA barrier, when every thread
// has read plane x+1 (the TMA loader refills its stage there) and returns
// true if the CTA must stop (a bounded wait gave up).
template <class P, int NWP, bool DIAG = false, bool VP = false, class Consumed,
          class AfterSync>
__device__ __forceinline__ bool plane_update(int x, V2 pf[5], const Cell2& cur, const V2 fm[5],
                                             Cell2& nxt, V2 fp[5], const StepConsts<float>& K,
                                             FusedSmem<NWP>& sm, TileOut& o, Consumed consumed,
                                             AfterSync after_sync) {
  // cur / fm: plane x and the flux at x-1/2; nxt / fp receive plane x+1 and
  // the flux at x+1/2 (the caller copies them into cur / fm for the next plane)
  const int lane = threadIdx.x & 31;
  // fast tiles: the warp index through a lane-0 shuffle (measured +0.5-1%);
  // the exact tile keeps threadIdx.x >> 5 (the shuffle costs it a register
  // spill and 9%)
  const int w = P::kExact ? (int)(threadIdx.x >> 5) : uniform_warp_index();
  P::template derive_in<1>(pf, nxt, K);
  consumed();
  P::hll(cur, nxt, fp);  // face x + 1/2
  V2 s1[5];
  P::update(cur, fm, fp, s1, K);

  // ---- y sweep ----
  Cell2 cy;
  P::template derive<2>(s1, cy, K);
  sm.cy[0][w][lane] = make_float4(cy.U[0].y, cy.U[1].y, cy.U[2].y, cy.U[3].y);
  sm.cy[1][w][lane] = make_float4(cy.U[4].y, cy.F[0].y, cy.F[1].y, cy.F[2].y);
  sm.cy[2][w][lane] = make_float4(cy.F[3].y, cy.F[4].y, cy.wa.y, cy.wb.y);
  const bool stop = after_sync();
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
      d = make_float4(cy.F[3].x, cy.F[4].x, cy.wa.x, cy.wb.x);
    }
    L.U[0] = v2(a.x, cy.U[0].x); L.U[1] = v2(a.y, cy.U[1].x);
    L.U[2] = v2(a.z, cy.U[2].x); L.U[3] = v2(a.w, cy.U[3].x);
    L.U[4] = v2(b.x, cy.U[4].x); L.F[0] = v2(b.y, cy.F[0].x);
    L.F[1] = v2(b.z, cy.F[1].x); L.F[2] = v2(b.w, cy.F[2].x);
    L.F[3] = v2(d.x, cy.F[3].x); L.F[4] = v2(d.y, cy.F[4].x);
    L.wa = v2(d.z, cy.wa.x);     L.wb = v2(d.w, cy.wb.x);
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
  if (o.store_a) {
    store5<VP>(o, x, o.dcol_a, wo, false);
    o.wmax = speed_max(o.wmax, sp.x);
    if constexpr (DIAG) diag_cell(o, x, o.sy_a, wo, false, K);
  }
  if (o.store_b) {
    store5<VP>(o, x, o.dcol_b, wo, true);
    o.wmax = speed_max(o.wmax, sp.y);
    if constexpr (DIAG) diag_cell(o, x, o.sy_b, wo, true, K);
  }
  return stop;
}

// Geometry of the thread's two cells within a tile.
struct TileCols {
  int x0, x_end, z, ya, yb;
  size_t col_a, col_b;  // source columns (wrapped / clamped)
};

template <int NWP>
__device__ __forceinline__ TileCols tile_cols(const FusedGeom& G, int tz, int ty, int tx,
                                              const float* src, float* dst, TileOut& o) {
  const int lane = threadIdx.x & 31;
  const int w = threadIdx.x >> 5;
  const bool open = G.open_bc != 0;
  TileCols t;
  const int z0 = tz * kTileZ, y0 = ty * tile_rows_out(NWP);
  t.x0 = tx * G.lx;
  t.x_end = min(t.x0 + G.lx, G.nx);
  t.z = z0 - 1 + lane;
  t.ya = y0 - 1 + 2 * w;
  t.yb = t.ya + 1;
  const int zs = src_index(t.z, G.nz, open);
  t.col_a = (size_t)src_index(t.ya, G.ny, open) * G.nz + zs;
  t.col_b = (size_t)src_index(t.yb, G.ny, open) * G.nz + zs;
  o.dst = dst;
  o.plane = (size_t)G.ny * G.nz;
  o.vstride = o.plane * G.nx;
  const bool store_lane = lane >= 1 && lane <= kTileLanes - 2 && t.z < G.nz;
  o.store_a = store_lane && w >= 1 && t.ya < G.ny;
  o.store_b = store_lane && w <= NWP - 2 && t.yb < G.ny;
  o.dcol_a = o.store_a ? (size_t)t.ya * G.nz + t.z : 0;
  o.dcol_b = o.store_b ? (size_t)t.yb * G.nz + t.z : 0;
  o.wmax = 0.f;
  return t;
}

// One CTA-tile of the fused step, planes loaded by each thread with
// register prefetch.  Returns this thread's running maximum of the stored
// cells' wave speeds (0 for threads that store nothing).  COHERENT selects
// L2-only loads (ld.global.cg) for kernels that read data other CTAs wrote
// earlier in the same launch (the persistent batch kernel); otherwise loads
// use the read-only path.
// DIAG: also accumulate the stored cells' conserved totals into acc[5] and
// write the slice of `d` (the diagnostics instantiation of the single step).
// VP: `vp` holds the per-variable bases of src and dst as launch parameters.
template <class P, int NWP, bool COHERENT = false, bool DIAG = false, bool VP = false>
__device__ __forceinline__ float fused_tile(const float* __restrict__ src, float* __restrict__ dst,
                                            const FusedGeom& G, int tz, int ty, int tx,
                                            const StepConsts<float>& K, FusedSmem<NWP>& sm,
                                            DiagArgs d = DiagArgs{nullptr, -1},
                                            CSum* acc = nullptr, const VarPtrs* vp = nullptr) {
  TileOut o;
  const TileCols t = tile_cols<NWP>(G, tz, ty, tx, src, dst, o);
  o.vp = vp;
  if constexpr (DIAG) {
#pragma unroll
    for (int i = 0; i < 5; ++i) o.acc[i] = CSum{0.f, 0.f};
    o.slice = d.slice;
    o.slice_plane = (size_t)G.nx * G.ny;
    o.ny = G.ny;
    const bool on = d.slice != nullptr && t.z == d.z_slice;
    o.sy_a = on && o.store_a ? t.ya : -1;
    o.sy_b = on && o.store_b ? t.yb : -1;
  }
  const bool open = G.open_bc != 0;
#if TF_CHECKED
  const size_t total = 5 * o.vstride;
  auto ld = [&](const float* p) {
    if ((size_t)(p - src) >= total) {
      atomicAdd(&g_chk_oob, 1ull);
      return 0.f;
    }
    return COHERENT ? __ldcg(p) : __ldg(p);
  };
#else
  auto ld = [&](const float* p) { return COHERENT ? __ldcg(p) : __ldg(p); };
#endif
  const unsigned ca32 = (unsigned)t.col_a, cb32 = (unsigned)t.col_b;
  auto load = [&](int x, V2 v[5]) {
    if constexpr (VP && !TF_CHECKED) {
      const unsigned xo = (unsigned)src_index(x, G.nx, open) * (unsigned)o.plane;
      const unsigned oa = xo + ca32, ob = xo + cb32;
#pragma unroll
      for (int i = 0; i < 5; ++i) {
        v[i].x = ld(vp->s[i] + oa);
        v[i].y = ld(vp->s[i] + ob);
      }
    } else {
      const float* p = src + (size_t)src_index(x, G.nx, open) * o.plane;
#pragma unroll
      for (int i = 0; i < 5; ++i) {
        const float* q = p + i * o.vstride;
        v[i].x = ld(q + t.col_a);
        v[i].y = ld(q + t.col_b);
      }
    }
  };
  // Loop form: the fast arithmetic's plain tile keeps one plane in flight and
  // alternates the carried plane quantities between two register sets (two
  // planes per trip, no copy); measured 3.6% faster at 512^3 than the form
  // below, which the other instantiations keep because the alternating form
  // spills registers there: two planes in flight and the carry copied back
  // after every plane.
  constexpr bool kAlt = !DIAG && !P::kExact;
  Cell2 c0, c1;  // c0 = plane x, c1 receives plane x+1
  V2 f0[5], f1[5];
  V2 pa[5], pb[5];
  {
    V2 w0[5];
    load(t.x0 - 1, w0);
    load(t.x0, pa);
    load(t.x0 + 1, pb);
    P::template derive_in<1>(w0, c1, K);
    P::template derive_in<1>(pa, c0, K);
    if (!kAlt && t.x0 + 2 <= t.x_end) load(t.x0 + 2, pa);
    P::hll(c1, c0, f0);  // flux at face x0 - 1/2; c0 = plane x0
  }
  auto sync_only = []() {
    __syncthreads();
    return false;
  };
  if constexpr (kAlt) {
    // pb holds plane x+1 on entry and receives plane x+2; after the trip's
    // second plane the carry is back in c0 / f0
    for (int x = t.x0; x < t.x_end; x += 2) {
      plane_update<P, NWP, DIAG, VP>(x, pb, c0, f0, c1, f1, K, sm, o,
                                     [&]() { if (x + 2 <= t.x_end) load(x + 2, pb); }, sync_only);
      if (x + 1 < t.x_end)
        plane_update<P, NWP, DIAG, VP>(x + 1, pb, c1, f1, c0, f0, K, sm, o,
                                   [&]() { if (x + 3 <= t.x_end) load(x + 3, pb); },
                                   sync_only);
    }
  } else {
    // Two planes per trip so the prefetch buffers alternate without moves;
    // `pf` holds plane x+1 on entry and receives plane x+3.
    for (int x = t.x0; x < t.x_end; x += 2) {
      plane_update<P, NWP, DIAG>(x, pb, c0, f0, c1, f1, K, sm, o,
                                 [&]() { if (x + 3 <= t.x_end) load(x + 3, pb); }, sync_only);
      c0 = c1;
#pragma unroll
      for (int i = 0; i < 5; ++i) f0[i] = f1[i];
      if (x + 1 < t.x_end) {
        plane_update<P, NWP, DIAG>(x + 1, pa, c0, f0, c1, f1, K, sm, o,
                                   [&]() { if (x + 4 <= t.x_end) load(x + 4, pa); },
                                   sync_only);
        c0 = c1;
#pragma unroll
        for (int i = 0; i < 5; ++i) f0[i] = f1[i];
      }
    }
  }
  if constexpr (DIAG) {
#pragma unroll
    for (int i = 0; i < 5; ++i) acc[i] = o.acc[i];
  }
  return o.wmax;
}

// ---------------------------------------------------------------------------
// TMA-staged planes
// ---------------------------------------------------------------------------
// One elected thread copies each x plane of the tile -- all five variables,
// the tile's rows including the ring, and a 40-float window of z rounded
// down to a 16-byte boundary -- from HBM into a shared-memory ring of
// kStages stages with one cp.async.bulk.tensor per plane; an mbarrier per
// stage signals its arrival.  Threads then read their two cells with
// constant-offset shared loads.  The tensor copy does not wrap, so threads
// whose source column is wrapped (periodic) or clamped (open boundaries) --
// only in tiles on the domain edge -- read that column directly from HBM.
constexpr int kStages = 3;
constexpr int kBoxZ = 40;  // z window: 32 lanes + up to 3 cells of 16-byte rounding, padded

__host__ __device__ constexpr size_t tma_stage_floats(int nwp) { return (size_t)5 * 2 * nwp * kBoxZ; }
__host__ __device__ constexpr size_t tma_smem_bytes(int nwp) {
  return kStages * tma_stage_floats(nwp) * sizeof(float);
}

__device__ __forceinline__ unsigned smem_u32(const void* p) {
  return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

__device__ __forceinline__ unsigned long long tf_global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Waits for an mbarrier phase; gives up after `limit_ns` and returns false.
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long* bar, unsigned parity,
                                                  unsigned long long limit_ns) {
  if (mbar_try_wait(bar, parity)) return true;
  const unsigned long long t0 = tf_global_ns();
  for (;;) {
    if (mbar_try_wait(bar, parity)) return true;
    if (tf_global_ns() - t0 > limit_ns) return false;
  }
}

__device__ __forceinline__ void tma_load_plane(void* dst, const void* tmap, unsigned long long* bar,
                                               int zc, int yc, int xc) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4, %5}], [%6];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<unsigned long long>(tmap)), "r"(zc), "r"(yc), "r"(xc), "r"(0),
      "r"(smem_u32(bar))
      : "memory");
}

constexpr unsigned long long kTmaWaitNs = 2000000000ull;  // 2 s per stage wait

// The fused tile with TMA-staged planes.  `tmap` describes `src` as a 4D
// tensor (z, y, x, var) with box (kBoxZ, 2*NWP, 1, 5).  Sets *timed_out (the
// CTA stopped early because a stage never arrived) and returns the running
// CFL speed like fused_tile.
template <class P, int NWP>
__device__ __forceinline__ float fused_tile_tma(const float* __restrict__ src,
                                                float* __restrict__ dst, const void* tmap,
                                                const FusedGeom& G, int tz, int ty, int tx,
                                                const StepConsts<float>& K, FusedSmem<NWP>& sm,
                                                float* stages, unsigned long long* bars,
                                                bool* timed_out) {
  constexpr int ROWS = 2 * NWP;
  constexpr size_t SF = tma_stage_floats(NWP);
  constexpr unsigned STAGE_BYTES = (unsigned)(SF * sizeof(float));
  const int w = threadIdx.x >> 5;
  const bool open = G.open_bc != 0;
  TileOut o;
  const TileCols t = tile_cols<NWP>(G, tz, ty, tx, src, dst, o);
  const int z0 = tz * kTileZ, y0 = ty * tile_rows_out(NWP);
  const int zb = (z0 - 1) >= 0 ? ((z0 - 1) & ~3) : -4;  // 16-byte aligned window start
  const int scol = t.z - zb;                              // 0..34
  // a cell whose source column is not its own (wrapped or clamped) reads HBM
  const bool direct_a = t.col_a != (size_t)t.ya * G.nz + t.z || t.ya < 0 || t.ya >= G.ny ||
                        t.z < 0 || t.z >= G.nz;
  const bool direct_b = t.col_b != (size_t)t.yb * G.nz + t.z || t.yb < 0 || t.yb >= G.ny ||
                        t.z < 0 || t.z >= G.nz;
  const int L = t.x_end - t.x0 + 1;  // planes consumed: x0-1 .. x_end (relative 0..L)
  bool bad = false;
  int issued_hi = -1, read_lo = 0;    // thread 0's view of the copies in flight

  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) mbar_init(&bars[s], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  auto issue = [&](int r) {  // plane x0-1+r into stage r % kStages (thread 0)
    const int s = r % kStages;
    issued_hi = r;
    mbar_expect_tx(&bars[s], STAGE_BYTES);
    tma_load_plane(stages + s * SF, tmap, &bars[s], zb, y0 - 1,
                   src_index(t.x0 - 1 + r, G.nx, open));
  };
  if (threadIdx.x == 0) {
    for (int r = 0; r < kStages && r <= L; ++r) issue(r);
  }
  // warps with no wrapped or clamped cell (every warp of an interior tile)
  // read shared memory only
  const bool warp_direct = __any_sync(0xffffffffu, direct_a || direct_b);
  auto read = [&](int r, V2 v[5]) {
    const int s = r % kStages;
    read_lo = r;
    if (!mbar_wait_bounded(&bars[s], (unsigned)((r / kStages) & 1), kTmaWaitNs)) bad = true;
    const float* st = stages + s * SF;
    const float* pa_ = st + (2 * w) * kBoxZ + scol;
    const float* pb_ = pa_ + kBoxZ;
    if (!warp_direct) {
#pragma unroll
      for (int i = 0; i < 5; ++i) {
        v[i].x = pa_[i * ROWS * kBoxZ];
        v[i].y = pb_[i * ROWS * kBoxZ];
      }
    } else {
      const float* g = src + (size_t)src_index(t.x0 - 1 + r, G.nx, open) * o.plane;
#pragma unroll
      for (int i = 0; i < 5; ++i) {
        v[i].x = direct_a ? __ldg(g + i * o.vstride + t.col_a) : pa_[i * ROWS * kBoxZ];
        v[i].y = direct_b ? __ldg(g + i * o.vstride + t.col_b) : pb_[i * ROWS * kBoxZ];
      }
    }
  };

  Cell2 c0, c1;  // carried plane quantities, alternating roles
  V2 f0[5], f1[5];
  {
    V2 w0[5], w1[5];
    read(0, w0);
    read(1, w1);
    P::template derive_in<1>(w0, c1, K);
    P::template derive_in<1>(w1, c0, K);
    P::hll(c1, c0, f0);  // flux at face x0 - 1/2; c0 = plane x0
  }
  if (__syncthreads_or(bad)) {
    *timed_out = true;
  } else {
    if (threadIdx.x == 0) {
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      for (int r = kStages; r < kStages + 2 && r <= L; ++r) issue(r);
    }
    auto step = [&](int x, const Cell2& cur, const V2* fm, Cell2& nxt, V2* fp) {
      const int r = x - t.x0 + 2;  // plane x+1
      V2 pf[5];
      read(r, pf);
      return plane_update<P, NWP>(
          x, pf, cur, fm, nxt, fp, K, sm, o, []() {},
          [&]() {
            if (__syncthreads_or(bad)) return true;
            if (threadIdx.x == 0 && r + kStages <= L) {
              asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
              issue(r + kStages);
            }
            return false;
          });
    };
    for (int x = t.x0; x < t.x_end; x += 2) {
      if (step(x, c0, f0, c1, f1)) {
        *timed_out = true;
        break;
      }
      if (x + 1 < t.x_end && step(x + 1, c1, f1, c0, f0)) {
        *timed_out = true;
        break;
      }
    }
  }
  if (*timed_out && threadIdx.x == 0) {
    // let the copies this CTA issued land before its shared memory is released
    for (int r = read_lo; r <= issued_hi; ++r)
      mbar_wait_bounded(&bars[r % kStages], (unsigned)((r / kStages) & 1), kTmaWaitNs);
  }
  return o.wmax;
}

}  // namespace tf
