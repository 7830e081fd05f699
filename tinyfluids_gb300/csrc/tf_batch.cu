// Batched time stepping of many independent instances of uneven size, each
// with its own CFL dt: one persistent launch advances every instance through
// all its steps (or one launch per step in the non-persistent form).
//
// Work items are (step s, instance i, tile t), enumerated step-major.  A CTA
// takes the next item from a global counter, waits until instance i has
// completed s steps (its control block's `iter`), runs the fused tile
// (tf_fused.cuh) and reports its tile's max wave speed; the CTA finishing an
// instance's step last closes it (t, dt, iter) exactly like a single-instance
// step.  An item only waits on items with smaller queue positions, which were
// taken earlier by running CTAs, so the queue cannot deadlock for any grid
// size; every wait is also bounded and ends with TF_ERR_TIMEOUT.
#include <string.h>

#include <mutex>
#include <unordered_map>
#include <vector>

#include "tf_common.cuh"
#include "tf_fused.cuh"
#include "tf_host.h"
#include "tf_math.cuh"

namespace tf {

constexpr long long kChunkCells = 1 << 16;  // cells per item of the init/final kernels

struct BatchInst {
  const float* src0;
  float* buf[2];
  float* out;
  tf_ctl* ctl;
  FusedGeom geo;
  float gamma, gm1, igm1, inv_dx, fixed_dt, cfl_dx, t_final;
  int max_steps;
  int ntiles;  // tiles per step
  int nchunks;
  long long ncells;
};

struct BatchHeader {
  unsigned long long queue;  // next work item
  int error;                 // batch-level tf_status (timeout)
  int count;
  int tiles_per_step;
  int chunks_total;
  int pad[2];
};

struct BatchPlan {  // host mirror of a prepared workspace
  int count = 0;
  int rows = 16;
  int exact = 0;
  int persistent = 1;
  int ctas_per_sm = 0;
  unsigned long long wait_limit = 0;
  int tiles_per_step = 0;
  int chunks_total = 0;
};

static std::mutex g_plan_mu;
static std::unordered_map<const void*, BatchPlan> g_plans;

static size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

struct Layout {
  size_t hdr, inst, tile_prefix, chunk_prefix, total;
};

static Layout layout(int count) {
  Layout L;
  L.hdr = 0;
  L.inst = align_up(sizeof(BatchHeader), 256);
  L.tile_prefix = align_up(L.inst + sizeof(BatchInst) * (size_t)count, 256);
  L.chunk_prefix = align_up(L.tile_prefix + sizeof(int) * (size_t)(count + 1), 256);
  L.total = align_up(L.chunk_prefix + sizeof(int) * (size_t)(count + 1), 256);
  return L;
}

// index i with prefix[i] <= r < prefix[i+1]
__device__ __forceinline__ int find_instance(const int* __restrict__ prefix, int count, int r) {
  int lo = 0, hi = count;  // prefix[lo] <= r < prefix[hi]
  while (hi - lo > 1) {
    int mid = (lo + hi) >> 1;
    if (__ldg(prefix + mid) <= r) lo = mid;
    else hi = mid;
  }
  return lo;
}

__global__ void batch_init_kernel(BatchHeader* hdr, const BatchInst* __restrict__ inst, int count) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0) {
    hdr->queue = 0ull;
    hdr->error = TF_OK;
  }
  if (i >= count) return;
  tf_ctl* c = inst[i].ctl;
  c->t = 0.f;
  c->dt = 0.f;
  c->t_final = inst[i].t_final;
  c->cfl_dx = inst[i].cfl_dx;
  c->ws_bits = 0u;
  c->done = 0u;
  c->iter = 0;
  c->active = 0;
  c->max_steps = inst[i].max_steps;
  c->status = TF_OK;
  c->max_speed = 0.f;
}

// Max wave speed of every instance's initial state; sets each ctl's dt.
__global__ void __launch_bounds__(256) batch_maxspeed_kernel(const BatchInst* __restrict__ inst,
                                                             const int* __restrict__ chunk_prefix,
                                                             int count, int chunks_total,
                                                             int fast) {
  __shared__ float red[8];
  for (int c = blockIdx.x; c < chunks_total; c += gridDim.x) {
    int i = find_instance(chunk_prefix, count, c);
    const BatchInst& I = inst[i];
    long long k = c - __ldg(chunk_prefix + i);
    long long b = k * kChunkCells, e = min(b + kChunkCells, I.ncells);
    float m = 0.f;
    for (long long j = b + threadIdx.x; j < e; j += blockDim.x) {
      float w[5];
#pragma unroll
      for (int v = 0; v < 5; ++v) w[v] = __ldg(I.src0 + v * I.ncells + j);
      m = speed_max(m, fast ? FastPolicy::cell_speed(w, I.gamma) : exact_cell_speed(w, I.gamma));
    }
    float bm = block_max(m, red);
    if (threadIdx.x == 0) ctl_finish_cta(I.ctl, bm, (unsigned)I.nchunks, 0.f, false);
  }
}

// Copies each instance's final state into its W_out unless it is there.
__global__ void batch_final_kernel(const BatchInst* __restrict__ inst,
                                   const int* __restrict__ chunk_prefix, int count,
                                   int chunks_total) {
  for (int c = blockIdx.x; c < chunks_total; c += gridDim.x) {
    int i = find_instance(chunk_prefix, count, c);
    const BatchInst& I = inst[i];
    int iter = ld_volatile(&I.ctl->iter);
    const float* from = iter == 0 ? I.src0 : ((iter & 1) ? I.buf[1] : I.buf[0]);
    if (from == I.out) continue;
    long long k = c - __ldg(chunk_prefix + i);
    long long b = k * kChunkCells, e = min(b + kChunkCells, I.ncells);
    for (int v = 0; v < 5; ++v)
      for (long long j = b + threadIdx.x; j < e; j += blockDim.x)
        I.out[v * I.ncells + j] = __ldcg(from + v * I.ncells + j);
  }
}

__device__ __forceinline__ void setup_step(const BatchInst& I, int iter, float dt,
                                           const float*& src, float*& dst,
                                           StepConsts<float>& K) {
  src = iter == 0 ? I.src0 : ((iter & 1) ? I.buf[1] : I.buf[0]);
  dst = (iter & 1) ? I.buf[0] : I.buf[1];
  K.g = I.gamma;
  K.gm1 = I.gm1;
  K.igm1 = I.igm1;
  K.inv_dx = I.inv_dx;
  K.dt = dt;
  K.k = dt * I.inv_dx;
}

__device__ __forceinline__ void tile_coords(const FusedGeom& g, int t, int& tz, int& ty, int& tx) {
  tz = t % g.tiles_z;
  int r = t / g.tiles_z;
  ty = r % g.tiles_y;
  tx = r / g.tiles_y;
}

// One step of every active instance: one CTA per (instance, tile).
template <class P, int NWP>
__global__ void TF_FUSED_BOUNDS(NWP) batch_step_kernel(const BatchInst* __restrict__ inst,
                                                                const int* __restrict__ tile_prefix,
                                                                int count) {
  __shared__ FusedSmem<NWP> sm;
  int r = blockIdx.x;
  int i = find_instance(tile_prefix, count, r);
  const BatchInst& I = inst[i];
  if (!ld_volatile(&I.ctl->active)) return;
  int iter = ld_volatile(&I.ctl->iter);
  float dt = I.fixed_dt > 0.f ? I.fixed_dt : ld_volatile(&I.ctl->dt);
  const float* src;
  float* dst;
  StepConsts<float> K;
  setup_step(I, iter, dt, src, dst, K);
  int tz, ty, tx;
  tile_coords(I.geo, r - __ldg(tile_prefix + i), tz, ty, tx);
  float m = fused_tile<P, NWP, false>(src, dst, I.geo, tz, ty, tx, K, sm);
  float bm = block_max(m, sm.red);
  if (threadIdx.x == 0) ctl_finish_cta(I.ctl, bm, (unsigned)I.ntiles, dt, true);
}

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// All steps of all instances in one launch (see the file comment).
template <class P, int NWP>
__global__ void TF_FUSED_BOUNDS(NWP)
    batch_persistent_kernel(BatchHeader* hdr, const BatchInst* __restrict__ inst,
                            const int* __restrict__ tile_prefix, int count, int tiles_per_step,
                            int step_base, int steps, unsigned long long wait_limit) {
  __shared__ FusedSmem<NWP> sm;
  __shared__ unsigned long long s_item;
  __shared__ int s_go, s_iter;
  __shared__ float s_dt;
  const unsigned long long total = (unsigned long long)steps * tiles_per_step;
  for (;;) {
    if (threadIdx.x == 0) {
      s_item = ld_volatile(&hdr->error) != TF_OK ? total : atomicAdd(&hdr->queue, 1ull);
    }
    __syncthreads();
    const unsigned long long q = s_item;
    if (q >= total) break;
    const int s = step_base + (int)(q / tiles_per_step);
    const int r = (int)(q % tiles_per_step);
    const int i = find_instance(tile_prefix, count, r);
    const BatchInst& I = inst[i];
    if (threadIdx.x == 0) {
      // wait until instance i has completed s steps, or has stopped
      int go = 0;
      unsigned long long spins = 0;
      unsigned ns = 32;
      for (;;) {
        int it = ld_volatile(&I.ctl->iter);
        if (it >= s) {
          __threadfence();
          go = ld_volatile(&I.ctl->active) && it == s ? 1 : 0;
          s_iter = it;
          break;
        }
        if (!ld_volatile(&I.ctl->active)) break;  // stopped before reaching s
        if (ld_volatile(&hdr->error) != TF_OK) break;
        if (++spins > wait_limit) {
          atomicExch(&hdr->error, TF_ERR_TIMEOUT);
          atomicExch(&I.ctl->status, TF_ERR_TIMEOUT);
          break;
        }
        __nanosleep(ns);
        if (ns < 1024) ns <<= 1;
      }
      s_go = go;
      if (go) s_dt = I.fixed_dt > 0.f ? I.fixed_dt : ld_volatile(&I.ctl->dt);
    }
    __syncthreads();
    if (!s_go) continue;  // uniform across the CTA
    const float dt = s_dt;
    const float* src;
    float* dst;
    StepConsts<float> K;
    setup_step(I, s_iter, dt, src, dst, K);
    int tz, ty, tx;
    tile_coords(I.geo, r - __ldg(tile_prefix + i), tz, ty, tx);
    float m = fused_tile<P, NWP, true>(src, dst, I.geo, tz, ty, tx, K, sm);
    __threadfence();  // this thread's stores before the CTA's completion count
    float bm = block_max(m, sm.red);
    if (threadIdx.x == 0) ctl_finish_cta(I.ctl, bm, (unsigned)I.ntiles, dt, true);
    __syncthreads();
  }
}

template <class P, int NWP>
static int occupancy_persistent(int* per_sm) {
  return cuda_check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                        per_sm, batch_persistent_kernel<P, NWP>, NWP * 32, 0),
                    "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
}

template <class P, int NWP>
static int launch_batch(const BatchPlan& p, void* ws, int step_base, int steps, cudaStream_t s) {
  Layout L = layout(p.count);
  char* base = (char*)ws;
  BatchHeader* hdr = (BatchHeader*)(base + L.hdr);
  const BatchInst* inst = (const BatchInst*)(base + L.inst);
  const int* tp = (const int*)(base + L.tile_prefix);
  if (p.persistent) {
    int per_sm = p.ctas_per_sm;
    if (per_sm <= 0) {
      TF_TRY((occupancy_persistent<P, NWP>(&per_sm)));
      if (per_sm < 1) per_sm = 1;
    }
    long long grid = (long long)per_sm * sm_count();
    long long total = (long long)steps * p.tiles_per_step;
    if (grid > total) grid = total;
    if (grid < 1) return TF_OK;
    unsigned long long lim = p.wait_limit ? p.wait_limit : (1ull << 24);
    batch_persistent_kernel<P, NWP><<<(int)grid, NWP * 32, 0, s>>>(
        hdr, inst, tp, p.count, p.tiles_per_step, step_base, steps, lim);
    return launch_check("batch_persistent_kernel");
  }
  for (int k = 0; k < steps; ++k) {
    batch_step_kernel<P, NWP><<<p.tiles_per_step, NWP * 32, 0, s>>>(inst, tp, p.count);
    TF_TRY(launch_check("batch_step_kernel"));
  }
  return TF_OK;
}

}  // namespace tf

using namespace tf;

extern "C" {

unsigned long long tf_batch_workspace_bytes(int count) {
  if (count < 1) return 0;
  return layout(count).total;
}

int tf_batch_prepare(const tf_instance* inst, int count, const tf_batch_config* cfg,
                     void* workspace, unsigned long long workspace_bytes, void* stream) {
  if (!inst || count < 1 || !workspace) return set_error(TF_ERR_ARG, "bad batch arguments");
  Layout L = layout(count);
  if (workspace_bytes < L.total)
    return set_error(TF_ERR_ARG, "workspace too small: %llu < %llu bytes",
                     (unsigned long long)workspace_bytes, (unsigned long long)L.total);
  if ((uintptr_t)workspace % 256) return set_error(TF_ERR_ARG, "workspace must be 256-byte aligned");
  BatchPlan plan;
  plan.count = count;
  if (cfg) {
    if (!valid_tile_rows(cfg->rows))
      return set_error(TF_ERR_ARG, "batch rows must be 8, 16 or 32 (got %d)", cfg->rows);
    plan.rows = cfg->rows;
    plan.exact = cfg->exact ? 1 : 0;
    plan.persistent = cfg->persistent ? 1 : 0;
    plan.ctas_per_sm = cfg->ctas_per_sm;
    plan.wait_limit = cfg->wait_limit;
  }
  std::vector<char> host(L.total, 0);
  BatchInst* bi = (BatchInst*)(host.data() + L.inst);
  int* tp = (int*)(host.data() + L.tile_prefix);
  int* cp = (int*)(host.data() + L.chunk_prefix);
  long long tiles = 0, chunks = 0;
  for (int i = 0; i < count; ++i) {
    const tf_instance& q = inst[i];
    if (!q.W_in || !q.W_out || !q.work || !q.ctl)
      return set_error(TF_ERR_ARG, "instance %d: null pointer", i);
    if (q.W_in == q.W_out || q.W_out == q.work)
      return set_error(TF_ERR_ARG, "instance %d: W_out must differ from W_in and work", i);
    if (q.nx < 1 || q.ny < 1 || q.nz < 1) return set_error(TF_ERR_ARG, "instance %d: bad dims", i);
    if ((q.flags & TF_FLAG_OPEN_BOUNDARIES) && (q.nx < 2 || q.ny < 2 || q.nz < 2))
      return set_error(TF_ERR_ARG, "instance %d: open boundaries need >= 2 cells per axis", i);
    if (!(q.dx > 0.f) || !isfinite(q.dx) || !isfinite(q.gamma) || q.gamma == 1.f ||
        !(q.cfl > 0.f) || isnan(q.t_final) || !(q.fixed_dt >= 0.f) || q.lx < 0)
      return set_error(TF_ERR_ARG, "instance %d: bad scalar parameter", i);
    if (q.max_steps < 0 && !isfinite(q.t_final))
      return set_error(TF_ERR_ARG, "instance %d: needs a finite t_final or max_steps >= 0", i);
    BatchInst& b = bi[i];
    int lx = q.lx > 0 ? q.lx : (q.nx < 64 ? q.nx : 64);
    if (lx > q.nx) lx = q.nx;
    FusedGeom g;
    g.nx = q.nx;
    g.ny = q.ny;
    g.nz = q.nz;
    g.open_bc = (q.flags & TF_FLAG_OPEN_BOUNDARIES) ? 1 : 0;
    g.tiles_z = (q.nz + kTileZ - 1) / kTileZ;
    g.tiles_y = (q.ny + plan.rows - 3) / (plan.rows - 2);
    g.lx = lx;
    g.tiles_x = (q.nx + lx - 1) / lx;
    b.geo = g;
    b.src0 = q.W_in;
    // with a known step count the last step writes W_out directly; when work
    // aliases W_in (the input may be overwritten), step 1 must write W_out
    bool even = q.work != q.W_in && q.max_steps >= 0 && (q.max_steps & 1) == 0;
    b.buf[0] = even ? q.W_out : q.work;
    b.buf[1] = even ? q.work : q.W_out;
    b.out = q.W_out;
    b.ctl = q.ctl;
    b.gamma = q.gamma;
    b.gm1 = q.gamma - 1.f;
    b.igm1 = 1.f / b.gm1;
    b.inv_dx = 1.f / q.dx;
    b.fixed_dt = q.fixed_dt;
    b.cfl_dx = q.cfl * q.dx;
    b.t_final = q.t_final;
    b.max_steps = q.max_steps;
    b.ncells = (long long)q.nx * q.ny * q.nz;
    long long nt = (long long)g.tiles_z * g.tiles_y * g.tiles_x;
    b.ntiles = (int)nt;
    b.nchunks = (int)((b.ncells + kChunkCells - 1) / kChunkCells);
    tp[i] = (int)tiles;
    cp[i] = (int)chunks;
    tiles += nt;
    chunks += b.nchunks;
    if (tiles > (1LL << 30) || chunks > (1LL << 30))
      return set_error(TF_ERR_ARG, "batch too large");
  }
  tp[count] = (int)tiles;
  cp[count] = (int)chunks;
  BatchHeader* h = (BatchHeader*)(host.data() + L.hdr);
  h->count = count;
  h->tiles_per_step = (int)tiles;
  h->chunks_total = (int)chunks;
  plan.tiles_per_step = (int)tiles;
  plan.chunks_total = (int)chunks;
  cudaStream_t s = (cudaStream_t)stream;
  TF_TRY(cuda_check(cudaMemcpyAsync(workspace, host.data(), L.total, cudaMemcpyHostToDevice, s),
                    "cudaMemcpyAsync(batch plan)"));
  // the host vector dies on return: wait for the copy to finish
  TF_TRY(cuda_check(cudaStreamSynchronize(s), "cudaStreamSynchronize"));
  std::lock_guard<std::mutex> lk(g_plan_mu);
  g_plans[workspace] = plan;
  return TF_OK;
}

int tf_batch_run(void* workspace, int step_base, int steps, void* stream) {
  if (!workspace || steps < 0 || step_base < 0) return set_error(TF_ERR_ARG, "bad arguments");
  BatchPlan p;
  {
    std::lock_guard<std::mutex> lk(g_plan_mu);
    auto it = g_plans.find(workspace);
    if (it == g_plans.end()) return set_error(TF_ERR_ARG, "workspace was not prepared");
    p = it->second;
  }
  cudaStream_t s = (cudaStream_t)stream;
  Layout L = layout(p.count);
  char* base = (char*)workspace;
  BatchHeader* hdr = (BatchHeader*)(base + L.hdr);
  const BatchInst* inst = (const BatchInst*)(base + L.inst);
  const int* cp = (const int*)(base + L.chunk_prefix);
  int grid_chunks = p.chunks_total < sm_count() * 8 ? p.chunks_total : sm_count() * 8;
  if (step_base == 0) {
    batch_init_kernel<<<(p.count + 255) / 256, 256, 0, s>>>(hdr, inst, p.count);
    TF_TRY(launch_check("batch_init_kernel"));
    batch_maxspeed_kernel<<<grid_chunks, 256, 0, s>>>(inst, cp, p.count, p.chunks_total,
                                                      p.exact ? 0 : 1);
    TF_TRY(launch_check("batch_maxspeed_kernel"));
  } else {
    // continuation: only the queue restarts
    TF_TRY(cuda_check(cudaMemsetAsync(hdr, 0, sizeof(unsigned long long), s), "cudaMemsetAsync"));
  }
  TF_DISPATCH_ROWS(p.rows, NWP, {
    if (p.exact) TF_TRY((launch_batch<ExactPair, NWP>(p, workspace, step_base, steps, s)));
    else TF_TRY((launch_batch<FastPair, NWP>(p, workspace, step_base, steps, s)));
  });
  batch_final_kernel<<<grid_chunks, 256, 0, s>>>(inst, cp, p.count, p.chunks_total);
  return launch_check("batch_final_kernel");
}

int tf_batch_error(void* workspace, int* error_host, void* stream) {
  if (!workspace || !error_host) return set_error(TF_ERR_ARG, "bad arguments");
  BatchHeader h;
  cudaStream_t s = (cudaStream_t)stream;
  TF_TRY(cuda_check(cudaMemcpyAsync(&h, workspace, sizeof h, cudaMemcpyDeviceToHost, s),
                    "cudaMemcpyAsync(batch header)"));
  TF_TRY(cuda_check(cudaStreamSynchronize(s), "cudaStreamSynchronize"));
  *error_host = h.error;
  return TF_OK;
}

int tf_batch_release(void* workspace) {
  std::lock_guard<std::mutex> lk(g_plan_mu);
  g_plans.erase(workspace);
  return TF_OK;
}

}  // extern "C"
