"""Benchmark of the tinyfluids time step on GB300.

Default workload (the headline): 512^3 shear layer, float32, gamma=5/3,
CFL 0.4, `--steps` time steps (default 200) per timed run.  Reports
Gcell-updates/s, the HBM roofline fraction of the fused step kernel, an
end-to-end figure through the public API with host buffers, and the CPU
baseline (the C restatement of the reference step on the host cores).

`--impl reference` times the reference's CPU path instead: the reference is a
JAX program that cannot be installed here, so its C restatement (the oracle
port, all host threads) runs a bounded sample of the same workload.

Multi-GPU (`--gpus N` under torchrun): the step does not shard (the
reference's single-GPU path); every rank runs an independent replica and the
reported value is the sum of all ranks' cell updates over the slowest rank's
time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GAMMA = 5.0 / 3.0
BYTES_PER_CELL = 40  # 5 float32 read + 5 float32 written per cell-update
METRIC = "Gcell-updates/s & %HBM roofline @512^3 fp32"
UNIT = "Gcell-updates/s"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=200)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--n", type=int, default=512, help="grid size per axis")
    p.add_argument("--exact", action="store_true", help="reference op order (slower)")
    p.add_argument("--e2e-repeats", type=int, default=8,
                   help="host states per end-to-end call (>= 2)")
    p.add_argument("--cpu-sample-seconds", type=float, default=20.0)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--tile", default=None,
                   help="rows,lx[,layout] of the fused kernel (layout: ldg, tma or ym)")
    p.add_argument("--out", default=None, help="also write the JSON line here")
    p.add_argument("--workload", default="plain", choices=["plain", "batch", "serve", "adjoint"],
                   help="plain: 512^3 step (default); batch: 256 uneven instances in one "
                        "persistent launch; serve: continuous batching vs one-at-a-time; "
                        "adjoint: 128^3 fixed-dt gradient")
    p.add_argument("--instances", type=int, default=256)
    p.add_argument("--requests", type=int, default=120)
    p.add_argument("--rates", default="10,50,100,200,500")
    p.add_argument("--serve-rate", type=float, default=200.0,
                   help="arrival rate of the serving part of the default line")
    p.add_argument("--serve-requests", type=int, default=300)
    p.add_argument("--serve-rate-light", type=float, default=40.0,
                   help="a second arrival rate of the default line, below the GPU's "
                        "capacity for this request mix (about 60 solves/s), where "
                        "latencies are not dominated by the backlog")
    p.add_argument("--no-extras", action="store_true",
                   help="skip the serving and batching parts of the default line")
    return p.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def init_dist(world, backend):
    import torch.distributed as dist
    if world > 1 and not dist.is_initialized():
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group(backend)
    return dist if world > 1 else None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms.

    Started before the warm-up so that nvidia-smi's own start-up never overlaps
    the timed region; only samples inside [mark_start, mark_stop] are kept."""

    QUERY = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None
        self.t0 = self.t1 = None

    def start(self, wait_s=15.0):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
            return
        end = time.time() + wait_s
        while time.time() < end and os.path.getsize(self.path) == 0:
            time.sleep(0.05)

    def mark_start(self):
        self.t0 = time.time()

    def mark_stop(self):
        self.t1 = time.time() + 0.25

    def stop(self):
        if self.proc is None:
            return None
        time.sleep(0.3)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        from datetime import datetime
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 10:
                continue
            try:
                ts = datetime.strptime(parts[0], "%Y/%m/%d %H:%M:%S.%f").timestamp()
                rows.append((ts, float(parts[2]), float(parts[3]), parts[6:10]))
            except ValueError:
                continue
        os.unlink(self.path)
        if not rows:
            return None
        win = [r for r in rows if self.t0 is None or (self.t0 <= r[0] <= self.t1)] or rows[-3:]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in win for i, v in enumerate(r[3])
                          if v.lower() == "active"})
        return {"sm_mhz": statistics.median(r[1] for r in win),
                "sm_max_mhz": max(r[2] for r in rows), "reasons": reasons,
                "samples": len(win)}


def cpu_baseline(n, seconds_budget, steps_cap, warmup=3):
    """The C restatement of the reference step (all host threads) on an n^3
    shear layer: `warmup` untimed steps, then up to steps_cap timed steps,
    bounded by the time budget.  The returned dict's "steps" is the number of
    steps timed."""
    import numpy as np
    from oracle import build as ob
    from oracle import fluid_c
    from oracle import ics_np
    ob.build()
    threads = fluid_c.max_threads()
    W, dx = ics_np.shear_layer(n, seed=0)
    # warm-up steps (also measure the per-step cost)
    warmup = max(1, int(warmup))
    t0 = time.perf_counter()
    W1, _ = fluid_c.run_steps(W, dx, GAMMA, warmup)
    per = (time.perf_counter() - t0) / warmup
    k = int(max(1, min(steps_cap, seconds_budget // max(per, 1e-9))))
    t0 = time.perf_counter()
    fluid_c.run_steps(W1, dx, GAMMA, k)
    el = time.perf_counter() - t0
    del np
    return {"value": n ** 3 * k / el / 1e9, "unit": UNIT, "cores": threads, "kind": "port",
            "steps": k, "warmup": warmup, "seconds": el,
            "sample": f"{k} CFL steps of the {n}^3 shear layer timed (after {warmup} untimed "
                      f"warm-up steps), C restatement of fluid.py/time_integration.py, "
                      f"{threads} OpenMP threads"}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    # every requested step is timed unless that would take more than ~90 s
    cb = cpu_baseline(args.n, 90.0, max(1, args.steps), warmup=max(3, args.warmup))
    line = {"metric": METRIC, "value": cb["value"], "unit": UNIT, "impl": "reference",
            "n_gpus": args.gpus, "steps": cb["steps"], "warmup": cb["warmup"],
            "steps_requested": args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "ms_per_step": 1e3 * cb["seconds"] / cb["steps"],
            "config": {"workload": f"shear layer {args.n}^3, gamma=5/3, CFL 0.4, periodic",
                       "instances": 1, "parallelism": "cpu"},
            "cpu_baseline": cb,
            "e2e": {"value": cb["value"], "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "note": "the reference (JAX) is not installable offline; its C restatement "
                    "(oracle/fluid_ref.c, bit-identical to the float32 NumPy restatement) is "
                    "timed on a bounded sample of the workload"}
    emit(line, args.out)
    return 0


def emit(line, out):
    s = json.dumps(line)
    print(s, flush=True)
    if out:
        with open(out, "w") as f:
            f.write(s + "\n")


def run_gpu(args):
    import torch

    import tinyfluids_gb300 as tg
    from tinyfluids_gb300 import build, replicas

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    dist = init_dist(world, "nccl")
    build.build()
    tg._lib.load()
    if args.exact:
        tg.set_exact(True)
    tile = (tuple(int(x) if x.isdigit() else x for x in args.tile.split(","))
            if args.tile else None)

    n, K, Wu = args.n, args.steps, args.warmup
    W, dx = tg.shear_layer(n, seed=rank, device=dev)
    state_bytes = W.numel() * 4

    def run(k):
        return tg.run_steps(W, dx, GAMMA, k, tile=tile)

    clocks = ClockSampler(local)
    clocks.start()
    # warm-up (W >= 3 enforced)
    for _ in range(max(3, Wu)):
        out = run(2)
    torch.cuda.synchronize()

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    # ---- kernel throughput: K steps, inputs resident, state (2.7 GB) >> L2 ----
    stream = torch.cuda.current_stream(dev)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    barrier()
    clocks.mark_start()
    e0.record(stream)
    out, ctl = tg.run_steps(W, dx, GAMMA, K, tile=tile, return_ctl=True)
    e1.record(stream)
    barrier()
    clocks.mark_stop()
    ms = e0.elapsed_time(e1)
    clk = clocks.stop()
    summ = tg.time_integration.ctl_summary(ctl)
    if summ["status"] != 0 or summ["iter"] != K:
        raise RuntimeError(f"run failed: {summ}")
    cells = n ** 3
    # the fused kernel's own launch duration: a second run of K - K/2 fewer
    # steps, timed the same way; the per-run work (control block, CFL
    # reduction of the initial state, final buffer choice) cancels in the
    # difference
    Kh = K // 2
    e2 = torch.cuda.Event(enable_timing=True)
    e3 = torch.cuda.Event(enable_timing=True)
    barrier()
    e2.record(stream)
    tg.run_steps(W, dx, GAMMA, Kh, tile=tile)
    e3.record(stream)
    barrier()
    ms_half = e2.elapsed_time(e3)
    kernel_ms = (ms - ms_half) / (K - Kh) if K > Kh else ms / max(K, 1)
    value, ms = replicas.job_throughput(cells, K, ms, world, dev)

    # ---- end to end: public API with pinned host buffers ----
    Wh = W.cpu().pin_memory()
    Oh = torch.empty_like(Wh).pin_memory()
    # (1) one state: copy in, K steps, copy out, nothing overlapped
    single_ms = []
    # one untimed pass first: the device buffers of a call come from torch's
    # caching allocator, which reaches its steady state after one call
    for rep in range(3):
        barrier()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        Wd = Wh.to(dev, non_blocking=True)
        Od = tg.run_steps(Wd, dx, GAMMA, K, tile=tile)
        Oh.copy_(Od, non_blocking=True)
        b.record(stream)
        barrier()
        if rep > 0:
            single_ms.append(a.elapsed_time(b))
        del Wd, Od
    single_value, _ = replicas.job_throughput(cells, K, min(single_ms), world, dev)
    # (2) R host states per call of time_integration_host (the C-ABI call with
    # host buffers): each copied in, K steps, copied out; the copies of one
    # state overlap the steps of its neighbours
    R = max(2, args.e2e_repeats)
    Oh2 = torch.empty_like(Wh).pin_memory()
    outs_h = [Oh if k % 2 == 0 else Oh2 for k in range(R)]
    # the call's device workspace, allocated once (repeated calls allocate nothing)
    ws = torch.empty(tg.host_runs_workspace_bytes(W.shape, R), dtype=torch.uint8, device=dev)
    e2e_ms = []
    for rep in range(6):
        barrier()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        _, its = tg.time_integration_host([Wh] * R, dx, None, GAMMA, False, num_steps=K,
                                          tile=tile, out=outs_h, workspace=ws)
        b.record(stream)
        barrier()
        assert its == [K] * R
        if rep > 0:
            e2e_ms.append(a.elapsed_time(b))
    e2e_value, e2e = replicas.job_throughput(cells, K * R, min(e2e_ms), world, dev)
    del Oh2, outs_h, ws
    torch.cuda.empty_cache()  # the host-run workspace (six states) is not needed again

    if rank != 0:
        return 0
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except OSError:
        pass
    peak = float(peaks.get("hbm_gbs", 6800.0))
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"
    per_launch_ms = kernel_ms
    rt = tg.resolved_tile((n, n, n), exact=args.exact, tile=tile)
    kernel_label = ("fused_step_ym_kernel (y-marching tile, %d x rows per CTA, %d y planes per "
                    "CTA)" % (rt[0] // 2, rt[1]) if rt[2] == "ym" else
                    "fused_step_kernel (x-marching tile, %d rows, %d x planes per CTA)"
                    % (rt[0], rt[1])) + "; 40 B/cell algorithmic"
    achieved = BYTES_PER_CELL * cells / (per_launch_ms * 1e-3) / 1e9
    traffic = None
    prof = os.path.join(ROOT, "profiles", "fused_step_traffic.json")
    if os.path.exists(prof):
        try:
            pj = json.load(open(prof))
            if int(pj.get("n", 0)) == n:
                traffic = pj.get("bytes_per_launch")
        except (OSError, ValueError):
            pass
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": K,
        "warmup": max(3, Wu), "ms_per_step": ms / K, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"shear layer {n}^3, gamma=5/3, CFL 0.4, periodic",
                   "steps_per_run": K,
                   "instances": world,
                   "parallelism": "replicas" if world > 1 else "single",
                   "arithmetic": "exact" if args.exact else "fast",
                   "l2": f"state {20 * n ** 3 / 1e9:.2f} GB vs 129 MB L2"
                         + (" (no flush needed)" if 2 * 20 * n ** 3 > 129e6 else
                            " (state fits in L2: not a DRAM measurement)"),
                   "tile": list(tile) if tile else "heuristic"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "peak_source": peak_src,
                     "kernel": kernel_label,
                     "launch_ms": per_launch_ms,
                     "launch_ms_definition": f"(time of {K} steps - time of {Kh} steps) / "
                                             f"{K - Kh}, CUDA events on the launching stream"},
        "e2e": {"value": e2e_value, "unit": UNIT,
                "h2d_bytes_per_step": state_bytes / K, "d2h_bytes_per_step": state_bytes / K,
                "definition": f"{R} pinned host states per call of time_integration_host "
                              f"(C ABI tf_time_integration_host): each copied to the GPU, "
                              f"{K} steps, copied back to pinned host memory; the copies of "
                              "one state overlap the steps of the others; bytes per time step",
                "states_per_call": R,
                "single_state": {"value": single_value, "unit": UNIT,
                                 "definition": f"one pinned host state -> device, {K} steps "
                                               "(run_steps), state -> pinned host, nothing "
                                               "overlapped"}},
        "gpu_launches": K + 3,
        "clocks": clk,
    }
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(min(n, 512), args.cpu_sample_seconds, K)
    if world == 1 and not args.no_extras:
        # the other two parts of the headline metric, measured on the same GPU
        # after the timed region: served solves/s with p50/p99 latency (config
        # 4 at one arrival rate) and batched solves/s (config 3)
        del W, out, ctl, Wh, Oh
        torch.cuda.empty_cache()
        line["serving"] = measure_serving(torch, tg, dev, args.serve_rate, args.serve_requests)
        line["serving_light_load"] = measure_serving(torch, tg, dev, args.serve_rate_light,
                                                     args.serve_requests)
        line["batching"] = measure_batching(torch, tg, dev, 256, 100, 3)
    emit(line, args.out)
    return 0


def _gpu_setup():
    import torch
    import tinyfluids_gb300 as tg
    from tinyfluids_gb300 import build
    build.build()
    tg._lib.load()
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", "0")))
    torch.cuda.set_device(dev)
    return torch, tg, dev


def measure_batching(torch, tg, dev, instances=256, K=100, warmup=3):
    """Config 3: `instances` overpressure spheres, N uniform in {32,48,64,96,128},
    radius U[0.05,0.2], pressure ratio U[10,100] (p_out 0.1), +-1% rho noise,
    K CFL steps each with its own dt, in one persistent graph-captured launch;
    against the plain loop of one run_steps call per instance."""
    import numpy as np
    from tinyfluids_gb300.batching import Batch, InstanceSpec
    rng = np.random.default_rng(0)
    specs = []
    for i in range(instances):
        n = int(rng.choice([32, 48, 64, 96, 128]))
        ratio = float(rng.uniform(10, 100))
        W, dx = tg.overpressure(n, seed=i, radius=float(rng.uniform(0.05, 0.2)),
                               p_in=0.1 * ratio, p_out=0.1, device=dev)
        specs.append(InstanceSpec(W, dx, GAMMA, num_steps=K))
    cells = sum(sp.state[0].numel() for sp in specs) * K
    t_tune = time.perf_counter()
    b = Batch(specs, autotune=True, capture_graph=True)
    t_tune = time.perf_counter() - t_tune
    for _ in range(max(3, warmup)):
        b.run()
    torch.cuda.synchronize()
    st = torch.cuda.current_stream(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    outs = b.run()
    e1.record(st)
    torch.cuda.synchronize()
    ms_batch = e0.elapsed_time(e1)
    assert b.error() == 0 and all(s["iter"] == K for s in b.summaries())
    # plain loops: one run_steps per instance (tuned tile per size), (a) all
    # enqueued asynchronously, (b) one solve at a time with its result read
    # back before the next starts (how the reference's API is driven: each
    # time_integration call returns its state)
    for sp in specs[:8]:
        tg.run_steps(sp.state, sp.grid_spacing, GAMMA, K, tile="auto")
    torch.cuda.synchronize()
    e0.record(st)
    alone = [tg.run_steps(sp.state, sp.grid_spacing, GAMMA, K, tile="auto") for sp in specs]
    e1.record(st)
    torch.cuda.synchronize()
    ms_plain = e0.elapsed_time(e1)
    same = all(torch.equal(o, a) for o, a in zip(outs, alone))
    del alone
    t0 = time.perf_counter()
    for sp in specs:
        r = tg.run_steps(sp.state, sp.grid_spacing, GAMMA, K, tile="auto")
        float(r[0, 0, 0, 0])  # the solve's result reaches the host
    ms_sync = (time.perf_counter() - t0) * 1e3
    res = {"solves_per_s": instances / (ms_batch * 1e-3), "ms": ms_batch,
           "gcell_updates_per_s": cells / (ms_batch * 1e-3) / 1e9,
           "workload": f"{instances} overpressure instances, N in {{32,48,64,96,128}}, "
                       f"{K} CFL steps each, one persistent graph-captured launch",
           "rows": b.rows, "tuning_s": t_tune,
           "plain_loop_async": {"solves_per_s": instances / (ms_plain * 1e-3), "ms": ms_plain,
                                "gcell_updates_per_s": cells / (ms_plain * 1e-3) / 1e9},
           "plain_loop_one_at_a_time": {"solves_per_s": instances / (ms_sync * 1e-3),
                                        "ms": ms_sync,
                                        "gcell_updates_per_s": cells / (ms_sync * 1e-3) / 1e9},
           "speedup_vs_plain_loop_async": ms_plain / ms_batch,
           "speedup_vs_plain_loop_one_at_a_time": ms_sync / ms_batch,
           "results_equal_alone": bool(same)}
    b.close()
    return res


def measure_serving(torch, tg, dev, rate, requests):
    """Config 4 at one arrival rate: Poisson arrivals, N uniform in [32,256],
    steps uniform in [50,500], seeded overpressure or shear states, 120 GB
    budget; the continuous-batching server (SRPT ticks) against the plain
    one-solve-at-a-time loop on the same requests."""
    from tinyfluids_gb300 import serving

    def fresh(reqs):
        return [serving.Request(r.rid, r.n, r.steps, r.ic, r.seed, r.arrival) for r in reqs]

    # warm-up: first use of the kernels, batch plans and allocator in this
    # process, outside the measurement (both arms)
    warm = serving.poisson_requests(12, 200.0, seed=12345)
    serving.Server(hbm_budget=120e9, device=dev, policy="srpt").serve(fresh(warm))
    serving.serve_one_at_a_time(fresh(warm), device=dev)
    torch.cuda.synchronize()
    reqs = serving.poisson_requests(requests, rate, seed=int(rate))
    srv = serving.Server(hbm_budget=120e9, device=dev, policy="srpt")
    st = serving.latency_stats(srv.serve(fresh(reqs)))
    bt = serving.latency_stats(serving.serve_one_at_a_time(fresh(reqs), device=dev))
    return {"rate_req_per_s": rate, "requests": requests,
            "workload": f"{requests} Poisson requests at {rate:g} req/s, N U[32,256], steps "
                        "U[50,500], overpressure or shear, 120 GB admission budget",
            "served": st, "one_at_a_time": bt, "ticks": srv.ticks,
            "solves_per_s_ratio": st["solves_per_s"] / bt["solves_per_s"],
            "p50_ratio": bt["p50_s"] / st["p50_s"], "p99_ratio": bt["p99_s"] / st["p99_s"]}


def measure_batch_classes(torch, tg, dev, K=100, count=32, sizes=(32, 48, 64, 96, 128)):
    """Per size class: a batch of `count` overpressure instances of one grid
    size (one persistent launch, tuned) against one instance of that size
    run alone (run_steps, tuned tile), both in Gcell-updates/s."""
    from tinyfluids_gb300.batching import Batch, InstanceSpec
    st = torch.cuda.current_stream(dev)
    out = {}
    for n in sizes:
        specs = [InstanceSpec(*tg.overpressure(n, seed=i, device=dev), GAMMA, num_steps=K)
                 for i in range(count)]
        b = Batch(specs, autotune=True, capture_graph=True)
        for _ in range(3):
            b.run()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        b.run()
        e1.record(st)
        torch.cuda.synchronize()
        ms_b = e0.elapsed_time(e1)
        W, dx = specs[0].state, specs[0].grid_spacing
        for _ in range(3):
            tg.run_steps(W, dx, GAMMA, K, tile="auto")
        e0.record(st)
        tg.run_steps(W, dx, GAMMA, K, tile="auto")
        e1.record(st)
        torch.cuda.synchronize()
        ms_a = e0.elapsed_time(e1)
        out[str(n)] = {"batch_gcell_updates_per_s": count * n ** 3 * K / (ms_b * 1e-3) / 1e9,
                       "alone_gcell_updates_per_s": n ** 3 * K / (ms_a * 1e-3) / 1e9,
                       "instances": count, "lx": sorted({sp.lx for sp in b.specs}),
                       "rows": b.rows}
        b.close()
    return out


def run_batch_workload(args):
    torch, tg, dev = _gpu_setup()
    K = args.steps if args.steps != 200 else 100
    r = measure_batching(torch, tg, dev, args.instances, K, args.warmup)
    r["per_size_class"] = measure_batch_classes(torch, tg, dev, K)
    line = {"metric": f"batched solves/s ({args.instances} uneven instances, {K} CFL steps each)",
            "value": r["solves_per_s"], "unit": "solves/s", "higher_is_better": True,
            "n_gpus": 1, "dtype": "f32", "data": "synthetic",
            "config": {"workload": r["workload"], "rows": r["rows"]}, **r}
    emit(line, args.out)
    return 0


def run_serve_workload(args):
    """Config 4 over a rate sweep."""
    torch, tg, dev = _gpu_setup()
    rates = [float(r) for r in args.rates.split(",")]
    sweep = [measure_serving(torch, tg, dev, rate, args.requests) for rate in rates]
    top = sweep[-1]
    line = {"metric": "served solves/s, p50/p99 latency (continuous batching, SRPT ticks)",
            "value": top["served"]["solves_per_s"], "unit": "solves/s", "higher_is_better": True,
            "n_gpus": 1, "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"{args.requests} requests per rate, N U[32,256], steps "
                                   "U[50,500], 120 GB budget", "rates": rates},
            "sweep": sweep}
    emit(line, args.out)
    return 0


def run_adjoint_workload(args):
    """Config 5: 128^3 shear layer, fixed dt 2e-4, 100 steps, loss = mean squared
    density difference to a seeded +-5% perturbation; gradient w.r.t. the five
    initial conserved fields by the hand-written adjoint (sqrt(N) checkpoints),
    checked by central differences (FP64 runs) on 32 random cells."""
    import numpy as np
    torch, tg, dev = _gpu_setup()
    from tinyfluids_gb300 import adjoint as A
    n, K, dt = 128, (args.steps if args.steps != 200 else 100), 2e-4
    W, dx = tg.shear_layer(n, seed=0, device=dev)
    U0 = tg.conserved_state_from_primitive(W, GAMMA)
    g = torch.Generator(device="cpu").manual_seed(1)
    noise = (torch.rand(W.shape[1:], generator=g) * 2 - 1).to(dev)
    rho_t = W[0] * (1 + 0.05 * noise)

    def grad(U):
        U = U.clone().requires_grad_(True)
        loss = A.density_mse_loss(U, rho_t.to(U.dtype), dx, dt, GAMMA, K)
        loss.backward()
        return U.grad, float(loss)

    grad(U0)  # warm-up
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    g32, loss32 = grad(U0)
    torch.cuda.synchronize()
    t_grad = time.perf_counter() - t0
    U64 = U0.double()
    g64, loss64 = grad(U64)
    rng = np.random.default_rng(2)
    errs32, errs64 = [], []
    scale = float(g64.abs().max())
    with torch.no_grad():
        for _ in range(32):
            f = int(rng.integers(5))
            i, j, k = (int(v) for v in rng.integers(n, size=3))
            h = 1e-6 * max(1.0, abs(float(U64[f, i, j, k])))
            Up, Um = U64.clone(), U64.clone()
            Up[f, i, j, k] += h
            Um[f, i, j, k] -= h
            fd = (float(A.density_mse_loss(Up, rho_t.double(), dx, dt, GAMMA, K))
                  - float(A.density_mse_loss(Um, rho_t.double(), dx, dt, GAMMA, K))) / (2 * h)
            errs64.append(abs(fd - float(g64[f, i, j, k])) / scale)
            errs32.append(abs(fd - float(g32[f, i, j, k])) / scale)
    line = {"metric": "adjoint gradient, 128^3 x 100 fixed-dt steps", "value": t_grad,
            "unit": "s per loss+gradient", "higher_is_better": False, "n_gpus": 1,
            "dtype": "f32", "data": "synthetic",
            "config": {"workload": "shear layer 128^3, dt=2e-4, 100 steps, sqrt(N) checkpoints"},
            "loss_f32": loss32, "loss_f64": loss64,
            "fd_check": {"cells": 32, "max_err_f64_adjoint": max(errs64),
                         "max_err_f32_adjoint": max(errs32),
                         "relative_to": "max |dL/dU0| (FP64)"},
            "gcell_updates_per_s_fwd_bwd": n ** 3 * K / t_grad / 1e9}
    emit(line, args.out)
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "batch":
        return run_batch_workload(args)
    if args.workload == "serve":
        return run_serve_workload(args)
    if args.workload == "adjoint":
        return run_adjoint_workload(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
