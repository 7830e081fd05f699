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
    p.add_argument("--e2e-repeats", type=int, default=2)
    p.add_argument("--cpu-sample-seconds", type=float, default=20.0)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--tile", default=None, help="rows,lx of the fused kernel")
    p.add_argument("--out", default=None, help="also write the JSON line here")
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


def cpu_baseline(n, seconds_budget, steps_cap):
    """The C restatement of the reference step (all host threads) on an n^3
    shear layer; times up to steps_cap steps, bounded by the time budget."""
    import numpy as np
    from oracle import build as ob
    from oracle import fluid_c
    from oracle import ics_np
    ob.build()
    threads = fluid_c.max_threads()
    W, dx = ics_np.shear_layer(n, seed=0)
    # warm-up: one step (also measures the per-step cost)
    t0 = time.perf_counter()
    W1, _ = fluid_c.run_steps(W, dx, GAMMA, 1)
    per = time.perf_counter() - t0
    k = int(max(1, min(steps_cap, seconds_budget // max(per, 1e-9))))
    t0 = time.perf_counter()
    fluid_c.run_steps(W1, dx, GAMMA, k)
    el = time.perf_counter() - t0
    del np
    return {"value": n ** 3 * k / el / 1e9, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{k} CFL steps of the {n}^3 shear layer (after 1 warm-up step), "
                      f"C restatement of fluid.py/time_integration.py, {threads} OpenMP threads"}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    budget = min(args.cpu_sample_seconds, 60.0)
    cb = cpu_baseline(args.n, budget, max(1, args.steps))
    line = {"metric": METRIC, "value": cb["value"], "unit": UNIT, "impl": "reference",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "ms_per_step": 1e3 * args.n ** 3 / (cb["value"] * 1e9),
            "config": {"workload": f"shear layer {args.n}^3, gamma=5/3, CFL 0.4, periodic",
                       "global_batch": 1, "seq_len": None, "parallelism": "cpu"},
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
    from tinyfluids_gb300 import build

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    dist = init_dist(world, "nccl")
    build.build()
    tg._lib.load()
    if args.exact:
        tg.set_exact(True)
    tile = tuple(int(x) for x in args.tile.split(",")) if args.tile else None

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
    if dist is not None:
        t = torch.tensor([ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t)
    cells = n ** 3
    value = world * cells * K / (ms * 1e-3) / 1e9

    # ---- end to end: public API with pinned host buffers ----
    Wh = W.cpu().pin_memory()
    Oh = torch.empty_like(Wh).pin_memory()
    e2e_ms = []
    for _ in range(max(1, args.e2e_repeats)):
        barrier()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        Wd = Wh.to(dev, non_blocking=True)
        Od = tg.run_steps(Wd, dx, GAMMA, K, tile=tile)
        Oh.copy_(Od, non_blocking=True)
        b.record(stream)
        barrier()
        e2e_ms.append(a.elapsed_time(b))
    e2e = min(e2e_ms)
    if dist is not None:
        t = torch.tensor([e2e], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e = float(t)
    e2e_value = world * cells * K / (e2e * 1e-3) / 1e9

    if rank != 0:
        return 0
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except OSError:
        pass
    peak = float(peaks.get("hbm_gbs", 6800.0))
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"
    per_launch_ms = ms / K
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
        "config": {"workload": f"shear layer {n}^3, gamma=5/3, CFL 0.4, periodic, "
                               f"{K} steps per run",
                   "global_batch": world, "seq_len": None,
                   "parallelism": "replicas" if world > 1 else "single",
                   "arithmetic": "exact" if args.exact else "fast",
                   "l2": "state 2.7 GB >> 129 MB L2 (no flush needed)",
                   "tile": list(tile) if tile else "heuristic"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "peak_source": peak_src,
                     "kernel": "fused_step_kernel (40 B/cell algorithmic; duration = run "
                               "time / steps, incl. the one-off dt init)"},
        "e2e": {"value": e2e_value, "unit": UNIT,
                "h2d_bytes_per_step": state_bytes / K, "d2h_bytes_per_step": state_bytes / K,
                "definition": f"pinned host state -> device, {K} steps, state -> pinned host; "
                              "bytes per time step"},
        "gpu_launches": K + 3,
        "clocks": clk,
    }
    if not args.no_cpu_baseline and world == 1 or (not args.no_cpu_baseline and rank == 0):
        line["cpu_baseline"] = cpu_baseline(min(n, 512), args.cpu_sample_seconds, 5)
    emit(line, args.out)
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
