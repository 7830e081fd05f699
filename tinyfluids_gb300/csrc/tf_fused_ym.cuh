// The y-marching form of the fused time step ("ym" tile): the same x, y and z
// HLL sweeps of fluid.py:562-578 and the same CFL epilogue as fused_tile
// (tf_fused.cuh), with the axes given other roles so that fewer cells are
// computed twice.
//
// Decomposition.  A CTA owns NW consecutive x rows (one per warp) of 60 z
// cells and MARCHES along y through a chunk of planes.  Lane l of a warp owns
// the PAIR of z-adjacent cells 60*tz-2+2l and 60*tz-1+2l (packed f32x2
// arithmetic, tf_pair.cuh), so a warp spans 64 cells of z: lanes 0 and 31
// hold the ring (swept, not stored) and a pair starts at an even z, so it
// moves as one 8-byte access when the grid allows.
//
//  * x sweep (the first sweep) across the warps: every warp derives its own
//    row, writes it to shared memory, and solves the face above its row from
//    the row above; the face below is the next warp's.  The rows just outside
//    the tile (x0-1, x0+NW) are needed only as the left / right state of the
//    tile's two edge faces, i.e. DERIVED from the input, never updated, so the
//    x ring costs one derive per edge instead of a swept row.  Warp 0 and the
//    last warp derive them.  Every row's input (the tile's rows and the
//    two halo rows) arrives in a shared-memory ring by per-lane cp.async two
//    planes ahead.
//  * y sweep (the second sweep) along the march: a thread keeps the previous
//    plane's x-updated cell quantities and the flux at the face y-1/2 in
//    registers; each plane adds one face and one update.
//  * z sweep (the third sweep) within the lane pair and with warp shuffles:
//    the face between the pair's cells is local, the face below the pair needs
//    the previous lane's upper cell, the face above is the next lane's.
//
// Compared with the x-marching tile (32 lanes x 2 rows per warp, 30 x 14
// cells stored of 32 x 16 computed) the only recomputed cells are the z ring
// (60 stored of 64) and the two derived halo rows per CTA, the z exchange
// shuffles half as many values and the global accesses move 8-byte pairs.  Every load index is wrapped periodically
// in-kernel (and clamped for open boundaries), so any nx, ny, nz >= 1 works.
// Results equal the x-marching tile's bit for bit: each face and each update
// is the same operation sequence on the same operands.
#pragma once
#include <type_traits>

#include "tf_fused.cuh"

namespace tf {


constexpr int kYmZ = 60;  // stored z cells per tile: lanes 1..30 (lanes 0 and 31 are the ring)

template <int NW>
struct YmSmem {
  // x-derived cell pair of each row: (U0, wa), (U1, F1) .. (U4, F4) and wb
  float4 cx[5][NW][32];
  float2 cw[NW][32];
  float4 fx[2][NW][32];      // flux at the face above each row, components 0..3
  float2 fx4[NW][32];        // component 4
  // input pairs landing by cp.async, two planes ahead: [stage][slot][variable][lane],
  // slot 0 = row x0-1, 1..NW = the tile's rows, NW+1 = row x0+NW
  float2 ring[2][NW + 2][5][32];
  float red[NW];  // block reduction
};

__device__ __forceinline__ float4 pack_v2(V2 a, V2 b) { return make_float4(a.x, a.y, b.x, b.y); }

// A cell of the x sweep travels without F[0]: the mass flux along the sweep
// axis is the momentum U[1] itself (both policies form it as the same
// product, fluid.py:225-228).
template <int NW>
__device__ __forceinline__ void ym_put_cell(YmSmem<NW>& sm, int s, int l, const Cell2& c) {
  sm.cx[0][s][l] = pack_v2(c.U[0], c.wa);
#pragma unroll
  for (int i = 1; i < 5; ++i) sm.cx[i][s][l] = pack_v2(c.U[i], c.F[i]);
  sm.cw[s][l] = c.wb;
}

// Accessor view of a row's cell in shared memory (the left cell of
// hll_from): each value is read where the face formula uses it.
template <int NW>
struct SmemCell {
  const YmSmem<NW>& sm;
  int s, l;
  __device__ __forceinline__ V2 wa() const {
    const float4 t = sm.cx[0][s][l];
    return v2(t.z, t.w);
  }
  __device__ __forceinline__ V2 wb() const { return sm.cw[s][l]; }
  __device__ __forceinline__ V2 U(int i) const {
    const float4 t = sm.cx[i][s][l];
    return v2(t.x, t.y);
  }
  __device__ __forceinline__ V2 F(int i) const {
    const float4 t = sm.cx[i == 0 ? 1 : i][s][l];
    return i == 0 ? v2(t.x, t.y) : v2(t.z, t.w);
  }
};

template <int NW>
__device__ __forceinline__ void ym_put_face(YmSmem<NW>& sm, int s, int l, const V2 f[5]) {
  sm.fx[0][s][l] = pack_v2(f[0], f[1]);
  sm.fx[1][s][l] = pack_v2(f[2], f[3]);
  sm.fx4[s][l] = f[4];
}

template <int NW>
__device__ __forceinline__ void ym_get_face(const YmSmem<NW>& sm, int s, int l, V2 f[5]) {
  float4 t = sm.fx[0][s][l];
  f[0] = v2(t.x, t.y);
  f[1] = v2(t.z, t.w);
  t = sm.fx[1][s][l];
  f[2] = v2(t.x, t.y);
  f[3] = v2(t.z, t.w);
  f[4] = sm.fx4[s][l];
}

// Per-lane asynchronous 4- and 8-byte copies global -> shared (cached in
// L1) and their group bookkeeping (PTX ISA: cp.async, cp.async.commit_group,
// cp.async.wait_group).
__device__ __forceinline__ void cp_async4(void* smem, const float* gmem) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(smem_u32(smem)), "l"(gmem)
               : "memory");
}
__device__ __forceinline__ void cp_async8(void* smem, const float* gmem) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(smem_u32(smem)), "l"(gmem)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;" ::: "memory");
}
// waits until at most one group (the most recent) is pending
__device__ __forceinline__ void cp_async_wait_prev() {
  asm volatile("cp.async.wait_group 1;" ::: "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.wait_group 0;" ::: "memory");
}

// Left cell of the z sweep's lane pair, read through shuffles at the point of
// use: (previous lane's upper cell, own lower cell), so hll_from(ShflLower{c},
// c) solves the faces below and between the pair's two cells.  F[0] is the
// z momentum U[3] (the mass flux along z).
struct ShflLower {
  const Cell2& c;
  static __device__ __forceinline__ V2 lo(V2 v) {
    return v2(__shfl_up_sync(0xffffffffu, v.y, 1), v.x);
  }
  __device__ __forceinline__ V2 wa() const { return lo(c.wa); }
  __device__ __forceinline__ V2 wb() const { return lo(c.wb); }
  __device__ __forceinline__ V2 U(int i) const { return lo(c.U[i]); }
  __device__ __forceinline__ V2 F(int i) const { return lo(i == 0 ? c.U[3] : c.F[i]); }
};

// One CTA-tile of the y-marching fused step: x rows x0 .. x0+NW-1 (tile tx),
// the 64 z cells 60*tz-2 .. 60*tz+61 (tile tz) of which lanes 1..30 store
// 60*tz .. 60*tz+59, planes y0 .. y0+ly-1 (chunk ty, ly = G.lx).  Lane pairs
// start at even z: with VEC (even nz, 8-byte aligned states) every pair moves
// as one 8-byte access.  VEC 1: periodic wrap; VEC 2: open boundaries, where
// the clamp of the source index to [1, nz-2] turns exactly two pairs into
// repeats of one cell, (0,1) into (1,1) and (nz-2,nz-1) into (nz-2,nz-2):
// those pairs load whole from their wrapped address and are fixed up after
// the y sweep (nz >= 4).  Returns this thread's running maximum of the stored cells'
// wave speeds (0 for threads that store nothing).  DIAG and VP as in
// fused_tile.
template <class P, int NW, bool DIAG = false, bool VP = false, int VEC = 0>
__device__ __forceinline__ float fused_tile_ym(const float* __restrict__ src,
                                               float* __restrict__ dst, const FusedGeom& G,
                                               int tx, int tz, int ty,
                                               const StepConsts<float>& K, YmSmem<NW>& sm,
                                               DiagArgs d = DiagArgs{nullptr, -1},
                                               CSum* acc = nullptr,
                                               const VarPtrs* vp = nullptr) {
  static_assert(NW >= 2, "the two halo rows need two distinct warps");
  using Off = typename std::conditional<VP && !TF_CHECKED, unsigned, size_t>::type;
  const int lane = threadIdx.x & 31;
  // the warp index through a shuffle from lane 0: provably the same in every
  // lane, so branches on it need no convergence barriers (measured +0.5%)
  const int w = __shfl_sync(0xffffffffu, (int)(threadIdx.x >> 5), 0);
  // VEC 1 runs periodic grids only: the clamp code is compiled out
  const bool open = VEC != 1 && G.open_bc != 0;
  const int x0 = tx * NW;
  const int y0 = ty * G.lx;
  const int y_end = min(y0 + G.lx, G.ny);
  const int x = x0 + w;
  const int za = tz * kYmZ - 2 + 2 * lane, zb = za + 1;
  const Off nz = (Off)G.nz;
  const Off xstride = (Off)G.ny * (Off)G.nz;
  const size_t vstride = (size_t)G.nx * G.ny * G.nz;
  // pairs move from their wrapped address (the checked build reads cells one
  // by one, through the full source-index map)
  constexpr bool kPairAddr = VEC != 0 && !TF_CHECKED;
  const int zwa = wrap_index(za, G.nz);
  const Off zsa = (Off)(kPairAddr ? zwa : src_index(za, G.nz, open));
  const Off zsb = (Off)(kPairAddr ? zwa + 1 : src_index(zb, G.nz, open));
  // open boundaries: does this warp hold one of the two pairs the clamp
  // turns into repeated cells (warp-uniform)
  const bool zfix = VEC == 2 && __any_sync(0xffffffffu, zwa == 0 || zwa == G.nz - 2);
  const Off rs = (Off)src_index(x, G.nx, open) * xstride;
  const Off ra = rs + zsa;
  const Off rb = rs + zsb;
  // the halo row this warp derives: warp 0 the row above, the last warp the
  // row below the tile
  const bool halo_warp = w == 0 || w == NW - 1;
  const int hslot = w == 0 ? 0 : NW + 1;
  const Off hs = (Off)src_index(w == 0 ? x0 - 1 : x0 + NW, G.nx, open) * xstride;
  const Off ha = hs + zsa;
  const Off hb = hs + zsb;
  // stored cells
  const bool st_lane = x < G.nx && lane >= 1 && lane <= 30;
  const bool st_a = st_lane && za < G.nz;
  const bool st_b = st_lane && zb < G.nz;
  const Off da = st_a ? (Off)x * xstride + (Off)za : 0;
  const Off db = da + 1;
  float wmax = 0.f;
  CSum dacc[5];
  if constexpr (DIAG) {
#pragma unroll
    for (int i = 0; i < 5; ++i) dacc[i] = CSum{0.f, 0.f};
  }
  const bool on_a = DIAG && d.slice != nullptr && st_a && za == d.z_slice;
  const bool on_b = DIAG && d.slice != nullptr && st_b && zb == d.z_slice;

  auto gsrc = [&](int i, Off off) -> const float* {
    if constexpr (VP && !TF_CHECKED) return vp->s[i] + off;
    else return src + i * vstride + off;
  };
  auto stage_of = [&](int y) { return (y - y0 + 1) & 1; };
#if TF_CHECKED
  // the checked build reads every row directly, range-checked
  auto ld = [&](int i, Off off) {
    if ((size_t)off >= vstride) {
      atomicAdd(&g_chk_oob, 1ull);
      return 0.f;
    }
    return __ldg(src + i * vstride + off);
  };
  auto issue = [&](int) {};
  auto read = [&](int y, bool halo, V2 v[5]) {
    const Off yo = (Off)src_index(y, G.ny, open) * nz;
    const Off oa = (halo ? ha : ra) + yo, ob = (halo ? hb : rb) + yo;
#pragma unroll
    for (int i = 0; i < 5; ++i) {
      v[i].x = ld(i, oa);
      v[i].y = ld(i, ob);
    }
  };
  auto wait_plane = []() {};
#else
  // plane y of the thread's row (and of its halo row) into the ring
  auto issue_row = [&](float2 (*slot)[32], Off oa, Off ob) {
#pragma unroll
    for (int i = 0; i < 5; ++i) {
      if constexpr (VEC) {
        cp_async8(&slot[i][lane], gsrc(i, oa));
      } else {
        cp_async4(&slot[i][lane].x, gsrc(i, oa));
        cp_async4(&slot[i][lane].y, gsrc(i, ob));
      }
    }
  };
  auto issue = [&](int y) {
    if (y <= y_end) {
      const Off yo = (Off)src_index(y, G.ny, open) * nz;
      issue_row(sm.ring[stage_of(y)][w + 1], ra + yo, rb + yo);
      if (halo_warp) issue_row(sm.ring[stage_of(y)][hslot], ha + yo, hb + yo);
    }
    cp_async_commit();  // an empty group past the chunk keeps the count uniform
  };
  auto read = [&](int y, bool halo, V2 v[5]) {
    const float2(*slot)[32] = sm.ring[stage_of(y)][halo ? hslot : w + 1];
#pragma unroll
    for (int i = 0; i < 5; ++i) v[i] = slot[i][lane];
  };
  // this plane's copies have landed; the next plane's may still be in flight
  auto wait_plane = []() { cp_async_wait_prev(); };
#endif

  // x sweep of plane y; s1 receives the x-updated state of the thread's pair
  auto xsweep = [&](int y, V2 s1[5]) {
    wait_plane();
    Cell2 cx;
    {
      V2 in[5];
      read(y, false, in);
      P::template derive_in<1>(in, cx, K);
    }
    ym_put_cell(sm, w, lane, cx);
    // the halo warps solve their tile-edge face before the barrier, so the
    // halo cell is dead before the row above is read (handing the edge work
    // to other warps through shared memory measured slower)
    V2 fxm[5], fxp[5];
    if (halo_warp) {
      V2 hin[5];
      Cell2 hc;
      read(y, true, hin);
      P::template derive_in<1>(hin, hc, K);
      if (w == 0) P::hll(hc, cx, fxm);
      else P::hll(cx, hc, fxp);
    }
    issue(y + 2);  // into this plane's stage, whose values are consumed
    __syncthreads();
    if (w != 0) {
      P::hll_from(SmemCell<NW>{sm, w - 1, lane}, CellRef2{cx}, fxm);
      ym_put_face(sm, w, lane, fxm);
    }
    __syncthreads();
    if (w != NW - 1) ym_get_face(sm, w + 1, lane, fxp);
    P::update(cx, fxm, fxp, s1, K);
  };

  auto put = [&](Off o, int i, float v) {
#if TF_CHECKED
    if ((size_t)o >= vstride) {
      atomicAdd(&g_chk_oob, 1ull);
      return;
    }
    dst[i * vstride + o] = v;
#else
    if constexpr (VP) vp->d[i][o] = v;
    else dst[i * vstride + o] = v;
#endif
  };
  auto store = [&](int y, const V2 wo[5], V2 sp) {
    const Off yo = (Off)y * nz;
#if TF_CHECKED
    if (g_chk_writes) {
      if (st_a && (long long)(da + yo) < g_chk_ncells) atomicAdd(g_chk_writes + da + yo, 1);
      if (st_b && (long long)(db + yo) < g_chk_ncells) atomicAdd(g_chk_writes + db + yo, 1);
    }
#endif
    if constexpr (VEC && !TF_CHECKED) {
      if (st_a) {  // nz is even: the pair is stored whole
#pragma unroll
        for (int i = 0; i < 5; ++i) {
          float* q;
          if constexpr (VP) q = vp->d[i] + (da + yo);
          else q = dst + i * vstride + (da + yo);
          *reinterpret_cast<float2*>(q) = wo[i];
        }
      }
    } else {
      if (st_a) {
#pragma unroll
        for (int i = 0; i < 5; ++i) put(da + yo, i, wo[i].x);
      }
      if (st_b) {
#pragma unroll
        for (int i = 0; i < 5; ++i) put(db + yo, i, wo[i].y);
      }
    }
    if (st_a) wmax = speed_max(wmax, sp.x);
    if (st_b) wmax = speed_max(wmax, sp.y);
    if constexpr (DIAG) {
      const size_t j = (size_t)x * G.ny + y;
      const size_t splane = (size_t)G.nx * G.ny;
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        if (h == 0 ? !st_a : !st_b) continue;
        float wv[5], u[5];
#pragma unroll
        for (int i = 0; i < 5; ++i) wv[i] = h == 0 ? wo[i].x : wo[i].y;
        exact_cons_from_prim(wv, u, K);
#pragma unroll
        for (int i = 0; i < 5; ++i) csum_add(dacc[i], u[i]);
        if (h == 0 ? on_a : on_b) {
          d.slice[j] = wv[0];
          d.slice[splane + j] = wv[4];
        }
      }
    }
  };

  // One plane y: x sweep of plane y+1, the y face y+1/2, the y update of
  // plane y, its z sweep, store and CFL speed.  cur / fm: plane y (derived
  // for the y sweep) and the flux at y-1/2; nxt / fp receive plane y+1 and
  // the flux at y+1/2.
  auto plane = [&](int y, const Cell2& cur, const V2 fm[5], Cell2& nxt, V2 fp[5]) {
    {
      V2 s1[5];
      xsweep(y + 1, s1);
      P::template derive<2>(s1, nxt, K);
    }
    P::hll(cur, nxt, fp);  // face y + 1/2
    V2 s2[5];
    P::update(cur, fm, fp, s2, K);
    if constexpr (VEC == 2) {
      // open boundaries: a cell whose input the clamp replaces by its z
      // neighbour's, z = 0 by z = 1 and z = nz-1 by nz-2, has x and y
      // neighbours replaced the same way, so after the x and y sweeps it
      // equals that neighbour bit for bit; the pair loaded whole from the
      // wrapped address takes it now, before the z sweep (its x and y sweeps
      // ran on the unclamped cell and reach no other cell)
      if (zfix) {
        const int zw = wrap_index(tz * kYmZ - 2 + 2 * lane, G.nz);
        const bool lo = zw == 0, hi = zw == G.nz - 2;
#pragma unroll
        for (int i = 0; i < 5; ++i) {
          if (lo) s2[i].x = s2[i].y;
          if (hi) s2[i].y = s2[i].x;
        }
      }
    }
    // ---- z sweep ----
    Cell2 cz;
    P::template derive<3>(s2, cz, K);
    V2 fzl[5], fzh[5];
    P::hll_from(ShflLower{cz}, CellRef2{cz}, fzl);  // faces za - 1/2 (.x) and za + 1/2 (.y)
#pragma unroll
    for (int i = 0; i < 5; ++i) fzh[i] = v2(fzl[i].y, __shfl_down_sync(0xffffffffu, fzl[i].x, 1));
    V2 s3[5], wo[5];
    P::update(cz, fzl, fzh, s3, K);
    const V2 sp = P::finish(s3, wo, K);
    store(y, wo, sp);
  };

  // warm-up: x sweeps of planes y0-1 and y0, the face y0 - 1/2
  Cell2 c0, c1;
  V2 f0[5], f1[5];
  issue(y0 - 1);
  issue(y0);
  {
    V2 s1[5];
    xsweep(y0 - 1, s1);
    P::template derive<2>(s1, c1, K);
    xsweep(y0, s1);
    P::template derive<2>(s1, c0, K);
    P::hll(c1, c0, f0);  // c0 = plane y0, f0 = face y0 - 1/2
  }
  // two planes per trip: the face fluxes alternate between f0 and f1, the
  // carried cell is copied back (alternating it too spills registers here)
  for (int y = y0; y < y_end; y += 2) {
    plane(y, c0, f0, c1, f1);
    c0 = c1;
    if (y + 1 < y_end) {
      plane(y + 1, c0, f1, c1, f0);
      c0 = c1;
    }
  }
#if !TF_CHECKED
  cp_async_wait_all();
#endif
  if constexpr (DIAG) {
#pragma unroll
    for (int i = 0; i < 5; ++i) acc[i] = dacc[i];
  }
  return wmax;
}

}  // namespace tf
