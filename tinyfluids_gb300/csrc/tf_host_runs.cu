// Runs of tf_time_integration over states held in host memory.
//
// The reference's time_integration (time_integration.py:94-128) takes any
// array the caller has, a host array included: JAX copies it to the device,
// runs the loop and hands back a device array the caller copies out.  Here a
// whole stream of such states goes through one call: each state is copied in,
// run with exactly tf_time_integration's loop, and copied back out, and the
// copies of one state overlap the steps of its neighbours.  Two device slots
// (input, work and output states each) alternate between consecutive states;
// host-to-device copies go on one stream, device-to-host copies on another,
// the runs on the caller's stream, ordered by events:
//
//   up:    [in k]   waits run k-2 (the slot's input was read by it)
//   run:   [run k]  waits in k and out k-2 (the slot's output was copied out)
//   down:  [out k]  waits run k
//
// With pinned host memory a stream of states then takes about one copy in,
// the runs back to back and one copy out, instead of the sum of all copies
// and runs.
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <mutex>
#include <utility>
#include <vector>

#include "tf_host.h"

namespace tf {

static unsigned long long align256(unsigned long long x) { return (x + 255ull) & ~255ull; }

// Bytes of one state, rounded up so every state of the workspace starts on
// a 256-byte boundary; 0 for invalid dimensions.
static unsigned long long slot_state_bytes(int nx, int ny, int nz) {
  if (nx < 1 || ny < 1 || nz < 1) return 0;
  const unsigned long long n = (unsigned long long)nx * ny * nz;
  if (n > (1ull << 40)) return 0;
  return align256(5ull * sizeof(float) * n);
}

// The two copy streams of a device (host-to-device, device-to-host), created
// on first use and kept for the life of the process, so a call creates no
// streams.  Calls on one device share them, which only orders their copies.
static std::mutex g_copy_mu;
static std::vector<std::pair<cudaStream_t, cudaStream_t>> g_copy_streams;

static int copy_streams(cudaStream_t* up, cudaStream_t* down) {
  int dev = 0;
  TF_TRY(cuda_check(cudaGetDevice(&dev), "cudaGetDevice"));
  std::lock_guard<std::mutex> lk(g_copy_mu);
  if ((int)g_copy_streams.size() <= dev) g_copy_streams.resize((size_t)dev + 1, {nullptr, nullptr});
  auto& p = g_copy_streams[(size_t)dev];
  if (!p.first) {
    // non-blocking: no implicit ordering against the legacy default stream
    TF_TRY(cuda_check(cudaStreamCreateWithFlags(&p.first, cudaStreamNonBlocking),
                      "cudaStreamCreate"));
    if (cuda_check(cudaStreamCreateWithFlags(&p.second, cudaStreamNonBlocking),
                   "cudaStreamCreate") != TF_OK) {
      cudaStreamDestroy(p.first);
      p.first = nullptr;
      return TF_ERR_CUDA;
    }
  }
  *up = p.first;
  *down = p.second;
  return TF_OK;
}

}  // namespace tf

using namespace tf;

extern "C" unsigned long long tf_host_runs_workspace_bytes(int nx, int ny, int nz, int count) {
  const unsigned long long sb = slot_state_bytes(nx, ny, nz);
  if (sb == 0 || count < 1) return 0;
  return 6ull * sb + align256((unsigned long long)count * sizeof(tf_ctl));
}

extern "C" int tf_time_integration_host(const float* const* W_in_host, float* const* W_out_host,
                                        int count, int nx, int ny, int nz, float dx,
                                        float t_final, float gamma, float cfl, int max_steps,
                                        float fixed_dt, unsigned flags,
                                        const tf_tile_config* tile, void* workspace,
                                        unsigned long long workspace_bytes, int* iters_host,
                                        void* stream) {
  if (!W_in_host || !W_out_host || !workspace)
    return set_error(TF_ERR_ARG, "null pointer (host state lists or workspace)");
  if (count < 1) return set_error(TF_ERR_ARG, "count must be >= 1 (got %d)", count);
  for (int k = 0; k < count; ++k)
    if (!W_in_host[k] || !W_out_host[k])
      return set_error(TF_ERR_ARG, "null host state pointer at index %d", k);
  const unsigned long long sb = slot_state_bytes(nx, ny, nz);
  if (sb == 0)
    return set_error(TF_ERR_ARG, "grid dims must be >= 1 and at most 2^40 cells (got %d,%d,%d)",
                     nx, ny, nz);
  const unsigned long long need = tf_host_runs_workspace_bytes(nx, ny, nz, count);
  if (workspace_bytes < need)
    return set_error(TF_ERR_ARG, "workspace of %llu bytes, %llu needed", workspace_bytes, need);
  if (reinterpret_cast<uintptr_t>(workspace) & 255)
    return set_error(TF_ERR_ARG, "workspace must be 256-byte aligned");
  // the run's own argument checks, before any copy is queued
  if (!(dx > 0.f) || !isfinite(dx)) return set_error(TF_ERR_ARG, "dx must be finite and > 0");
  if (!isfinite(gamma) || gamma == 1.f)
    return set_error(TF_ERR_ARG, "gamma must be finite and != 1");
  if (!(cfl > 0.f) || !isfinite(cfl)) return set_error(TF_ERR_ARG, "C_CFL must be finite and > 0");
  if (isnan(t_final)) return set_error(TF_ERR_ARG, "t_final is NaN");
  if (!(fixed_dt >= 0.f) || !isfinite(fixed_dt))
    return set_error(TF_ERR_ARG, "fixed_dt must be >= 0");
  if (max_steps < 0 && !isfinite(t_final))
    return set_error(TF_ERR_ARG, "an unbounded loop needs a finite t_final or max_steps >= 0");
  tf_tile_config resolved;
  const int ts = tf_resolve_tile(nx, ny, nz, flags, tile, &resolved);
  if (ts != TF_OK) return ts;
  const size_t bytes = 5ull * sizeof(float) * (size_t)nx * ny * nz;
  // an output is copied back while later inputs may still be copied in: it
  // may share memory with its own or earlier inputs (in place), not later
  // ones.  Inputs sorted by address: the ones overlapping an output start
  // within `bytes` of it on either side.
  {
    std::vector<std::pair<uintptr_t, int>> ins((size_t)count);
    for (int j = 0; j < count; ++j) ins[(size_t)j] = {reinterpret_cast<uintptr_t>(W_in_host[j]), j};
    std::sort(ins.begin(), ins.end());
    for (int k = 0; k < count; ++k) {
      const uintptr_t o = reinterpret_cast<uintptr_t>(W_out_host[k]);
      const uintptr_t lo = o >= bytes ? o - bytes + 1 : 0;
      auto it = std::lower_bound(ins.begin(), ins.end(), std::make_pair(lo, -1));
      for (; it != ins.end() && it->first < o + bytes; ++it)
        if (it->second > k)
          return set_error(TF_ERR_ARG, "output %d overlaps the input of later state %d", k,
                           it->second);
    }
  }
  unsigned char* base = static_cast<unsigned char*>(workspace);
  auto state = [&](int slot, int j) {
    return reinterpret_cast<float*>(base + (3 * slot + j) * sb);
  };
  tf_ctl* ctls = reinterpret_cast<tf_ctl*>(base + 6 * sb);

  cudaStream_t s = (cudaStream_t)stream;
  cudaStream_t up = nullptr, down = nullptr;
  cudaEvent_t ev[7] = {};  // start, in[2], run[2], out[2]
  int st = TF_OK;
  auto fail = [&](cudaError_t e, const char* what) {
    if (st == TF_OK && e != cudaSuccess) st = cuda_check(e, what);
    return st != TF_OK;
  };
  do {
    if ((st = copy_streams(&up, &down)) != TF_OK) break;
    bool ok = true;
    for (int i = 0; i < 7 && ok; ++i)
      ok = !fail(cudaEventCreateWithFlags(&ev[i], cudaEventDisableTiming), "cudaEventCreate");
    if (!ok) break;
    cudaEvent_t* ev_in = ev + 1;
    cudaEvent_t* ev_run = ev + 3;
    cudaEvent_t* ev_out = ev + 5;
    // the copies come after whatever the caller queued on its stream (which
    // may still use the workspace)
    if (fail(cudaEventRecord(ev[0], s), "cudaEventRecord")) break;
    if (fail(cudaStreamWaitEvent(up, ev[0], 0), "cudaStreamWaitEvent")) break;
    if (fail(cudaStreamWaitEvent(down, ev[0], 0), "cudaStreamWaitEvent")) break;
    for (int k = 0; k < count && st == TF_OK; ++k) {
      const int slot = k & 1;
      float* in = state(slot, 0);
      float* work = state(slot, 1);
      float* out = state(slot, 2);
      if (k >= 2 && fail(cudaStreamWaitEvent(up, ev_run[slot], 0), "cudaStreamWaitEvent")) break;
      if (fail(cudaMemcpyAsync(in, W_in_host[k], bytes, cudaMemcpyHostToDevice, up),
               "cudaMemcpyAsync(host state -> device)"))
        break;
      if (fail(cudaEventRecord(ev_in[slot], up), "cudaEventRecord")) break;
      if (fail(cudaStreamWaitEvent(s, ev_in[slot], 0), "cudaStreamWaitEvent")) break;
      if (k >= 2 && fail(cudaStreamWaitEvent(s, ev_out[slot], 0), "cudaStreamWaitEvent")) break;
      st = tf_time_integration(in, out, work, ctls + k, nx, ny, nz, dx, t_final, gamma, cfl,
                               max_steps, fixed_dt, flags, tile, nullptr, stream);
      if (st != TF_OK) break;
      if (fail(cudaEventRecord(ev_run[slot], s), "cudaEventRecord")) break;
      if (fail(cudaStreamWaitEvent(down, ev_run[slot], 0), "cudaStreamWaitEvent")) break;
      if (fail(cudaMemcpyAsync(W_out_host[k], out, bytes, cudaMemcpyDeviceToHost, down),
               "cudaMemcpyAsync(device state -> host)"))
        break;
      if (fail(cudaEventRecord(ev_out[slot], down), "cudaEventRecord")) break;
    }
    if (st != TF_OK) break;
    // the caller's stream orders after the last copy out
    if (fail(cudaStreamWaitEvent(s, ev_out[(count - 1) & 1], 0), "cudaStreamWaitEvent")) break;
  } while (false);
  // every copy reads or writes the caller's host memory: nothing may be in
  // flight when the call returns, on success or error
  if (up) cudaStreamSynchronize(up);
  if (down) cudaStreamSynchronize(down);
  const cudaError_t se = cudaStreamSynchronize(s);
  if (st == TF_OK) st = cuda_check(se, "cudaStreamSynchronize");
  if (st == TF_OK) {
    std::vector<tf_ctl> h((size_t)count);
    st = cuda_check(cudaMemcpy(h.data(), ctls, sizeof(tf_ctl) * (size_t)count,
                               cudaMemcpyDeviceToHost),
                    "cudaMemcpy(control blocks)");
    for (int k = 0; k < count && st == TF_OK; ++k) {
      if (iters_host) iters_host[k] = h[(size_t)k].iter;
      if (h[(size_t)k].status != TF_OK)
        st = set_error(h[(size_t)k].status, "state %d: device reported %s after %d steps", k,
                       tf_status_string(h[(size_t)k].status), h[(size_t)k].iter);
    }
  }
  for (int i = 0; i < 7; ++i)
    if (ev[i]) cudaEventDestroy(ev[i]);
  return st;
}
