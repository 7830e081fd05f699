"""Continuous-batching simulation server on one GPU.

Requests (grid size, step count, initial state) arrive over time.  The server
keeps every admitted simulation's state resident in HBM and advances all of
them together in TICKS: one persistent batch launch (``batching.Batch``)
moves every active request by up to ``tick_steps`` steps; between ticks,
finished requests are retired (their buffers freed) and waiting requests are
admitted as long as their two state buffers fit in the HBM budget.  Requests
that arrive while others are on the GPU therefore share the device with them
instead of queueing behind them.

Each request's result is bit-identical to running it alone with
``time_integration.run_steps``: a request's dt sequence depends only on its
own state, and a tick boundary restarts from the stored state with the same
CFL formula the fused kernel's epilogue uses.

The reference has no serving layer; this is an addition on top of the
drop-in step (its unit of work is one ``time_integration`` call per state).
"""
from __future__ import annotations

import math
import time
from collections import deque
from dataclasses import dataclass, field

import numpy as np
import torch

from . import initial_conditions as ics
from .batching import Batch, InstanceSpec

STATE_BYTES_PER_CELL = 20  # 5 float32


@dataclass
class Request:
    """One simulation: an n^3 grid, `steps` CFL steps from a seeded initial state."""
    rid: int
    n: int
    steps: int
    ic: str = "overpressure"       # "overpressure" | "shear"
    seed: int = 0
    arrival: float = 0.0           # seconds after the start of serving
    gamma: float = 5.0 / 3.0
    # filled in by the server
    admitted: float | None = None
    finished: float | None = None
    result: dict = field(default_factory=dict)

    @property
    def latency(self):
        return None if self.finished is None else self.finished - self.arrival


def request_bytes(n: int) -> int:
    """HBM a request holds while admitted: two state buffers (ping-pong)."""
    return 2 * STATE_BYTES_PER_CELL * n ** 3 + 64


def build_initial_state(req: Request, device):
    if req.ic == "overpressure":
        return ics.overpressure(req.n, seed=req.seed, device=device)
    if req.ic == "shear":
        return ics.shear_layer(req.n, seed=req.seed, device=device)
    raise ValueError(f"unknown initial state {req.ic!r}")


class _Active:
    def __init__(self, req, cur, other, dx):
        self.req = req
        self.cur = cur      # holds the current state
        self.other = other  # free buffer of the same size
        self.dx = dx
        self.remaining = req.steps


class Server:
    """Admits requests by free HBM budget and advances admitted ones together.

    hbm_budget: bytes of request state the server may hold (two state buffers
    per request); None takes 90% of the HBM free when the server is created.

    A tick advances a set of active requests by min(tick_steps, remaining)
    steps each, in one persistent batch launch.  policy "all" puts every
    active request in every tick (processor sharing).  policy "srpt" (the
    default) takes active requests in order of least remaining work
    (cells x remaining steps) until the tick holds `tick_budget`
    cell-updates, so the GPU stays full while short requests finish first
    instead of sharing the device with long ones; long requests run
    whenever the short ones leave room.  tick_steps is odd: a request's two
    buffers alternate as input and output, and with the input doubling as the
    work buffer an odd step count ends in the output buffer (no copy).  Batch
    plans are cached by the tick's buffers and step counts, which recur every
    other tick while the set is stable, and at most two ticks are in flight
    on the GPU."""

    # defaults from a sweep on GB300 (60 Poisson requests, N U[32,256], steps
    # U[50,500]): ticks of 31 steps and 2^29 cell-updates keep the throughput
    # of putting every request in every tick while cutting the median latency
    # about 5x
    def __init__(self, hbm_budget=120e9, device=None, tick_steps=31, rows=16,
                 cfl=0.4, keep_states=False, max_active=4096, plan_cache=4, policy="srpt",
                 tick_budget=2 ** 29):
        if policy not in ("srpt", "all"):
            raise ValueError("policy must be 'srpt' or 'all'")
        self.policy = policy
        self.tick_budget = int(tick_budget)
        self.device = torch.device(device if device is not None else "cuda")
        if hbm_budget is None:
            # admit by the HBM actually free now, keeping 10% for the batch
            # plans' workspaces and the allocator's slack
            free, _ = torch.cuda.mem_get_info(self.device)
            hbm_budget = 0.9 * free
        self.budget = int(hbm_budget)
        self.tick_steps = int(tick_steps) | 1
        self.rows = rows
        self.cfl = cfl
        self.keep_states = keep_states
        self.max_active = max_active
        self.queue: deque[Request] = deque()
        self.active: list[_Active] = []
        self.done: list[Request] = []
        self.used = 0
        self.ticks = 0
        self._plans: dict = {}
        self._plan_cache = int(plan_cache)
        self._inflight: deque = deque()

    # -- admission ----------------------------------------------------------
    def submit(self, req: Request):
        if request_bytes(req.n) > self.budget:
            raise ValueError(f"request {req.rid} needs more HBM than the whole budget")
        self.queue.append(req)

    def _admit(self, now):
        while self.queue and len(self.active) < self.max_active:
            req = self.queue[0]
            if req.arrival > now:
                break
            need = request_bytes(req.n)
            if self.used + need > self.budget:
                break  # FIFO: the head waits for memory, nobody overtakes it
            self.queue.popleft()
            W, dx = build_initial_state(req, self.device)
            self.active.append(_Active(req, W, torch.empty_like(W), dx))
            self.used += need
            req.admitted = now

    # -- one tick -----------------------------------------------------------
    def _select(self):
        """The requests of the next tick."""
        if self.policy == "all" or len(self.active) <= 1:
            return list(self.active)
        chosen, work = [], 0
        for a in sorted(self.active, key=lambda a: (a.req.n ** 3 * a.remaining, a.req.rid)):
            chosen.append(a)
            work += a.req.n ** 3 * min(self.tick_steps, a.remaining)
            if work >= self.tick_budget:
                break
        return chosen

    def _plan(self, group):
        key = tuple((a.cur.data_ptr(), a.other.data_ptr(), min(self.tick_steps, a.remaining))
                    for a in group)
        b = self._plans.pop(key, None)
        if b is None:
            specs = [InstanceSpec(a.cur, a.dx, a.req.gamma,
                                  num_steps=min(self.tick_steps, a.remaining), C_CFL=self.cfl,
                                  out=a.other, consume_input=True) for a in group]
            # a tick of one request runs as one launch per step (measured a
            # few ms lower latency for lone requests); several share one
            # persistent launch
            b = Batch(specs, rows=self.rows, persistent=len(group) > 1)
            while len(self._plans) >= self._plan_cache:
                old = self._plans.pop(next(iter(self._plans)))
                old.close()
        self._plans[key] = b  # most recently used last
        return b

    def _tick(self):
        group = self._select()
        if len(group) == 1 and self._lone_fits(group[0]):
            self._tick_lone(group[0])
            return
        b = self._plan(group)
        b.run()
        ev = torch.cuda.Event()
        ev.record(torch.cuda.current_stream(self.device))
        self._inflight.append(ev)
        while len(self._inflight) > 2:
            self._inflight.popleft().synchronize()
        self.ticks += 1
        for a, sp in zip(group, b.specs):
            a.cur, a.other = a.other, a.cur  # the result is in `out`
            a.remaining -= sp.num_steps

    def _lone_fits(self, a):
        # the single-grid run takes a work buffer and a fresh output besides
        # the request's two buffers
        return self.used + request_bytes(a.req.n) <= self.budget

    def _tick_lone(self, a):
        """A tick of one request runs the single-grid step loop (``run_steps``:
        the single-grid kernel and tile choice, no batch plan), measured faster
        than a one-instance batch when the server is lightly loaded; the result
        is the same bits.  Like a tick of several requests it holds up to
        `tick_budget` cell-updates (at least tick_steps steps), so a small
        request finishes in one tick instead of paying a tick's fixed cost
        every tick_steps steps."""
        from .time_integration import run_steps
        k = min(a.remaining, max(self.tick_steps, self.tick_budget // a.req.n ** 3))
        out = run_steps(a.cur, a.dx, a.req.gamma, k, C_CFL=self.cfl)
        a.other, a.cur = a.cur, out
        a.remaining -= k
        ev = torch.cuda.Event()
        ev.record(torch.cuda.current_stream(self.device))
        self._inflight.append(ev)
        while len(self._inflight) > 2:
            self._inflight.popleft().synchronize()
        self.ticks += 1

    def _retire(self):
        finishing = [a for a in self.active if a.remaining <= 0]
        if not finishing:
            return
        self.active = [a for a in self.active if a.remaining > 0]
        masses = [a.cur[0].double().sum() for a in finishing]
        rmax = [a.cur[0].max() for a in finishing]
        torch.cuda.current_stream(self.device).synchronize()
        self._inflight.clear()
        now = self._now()
        for a, m, r in zip(finishing, masses, rmax):
            a.req.result = {"mass": float(m) * a.dx ** 3, "rho_max": float(r)}
            if self.keep_states:
                a.req.result["state"] = a.cur
            a.req.finished = now
            self.used -= request_bytes(a.req.n)
            self.done.append(a.req)
        # plans that refer to retired buffers can never recur
        self._plans.clear()

    # -- event loop ---------------------------------------------------------
    def serve(self, requests, clock=None, idle_sleep=2e-4):
        """Serve `requests` (arrival times relative to the start); returns them."""
        for r in sorted(requests, key=lambda r: r.arrival):
            self.submit(r)
        t0 = time.perf_counter()
        self._now = (lambda: time.perf_counter() - t0) if clock is None else clock
        while self.queue or self.active:
            n_before = len(self.active)
            self._admit(self._now())
            if len(self.active) != n_before:
                self._plans.clear()
            if not self.active:
                nxt = self.queue[0].arrival
                while self._now() < nxt:
                    time.sleep(min(idle_sleep, max(0.0, nxt - self._now())))
                continue
            self._tick()
            self._retire()
        for b in self._plans.values():
            b.close()
        self._plans.clear()
        return self.done


def serve_one_at_a_time(requests, device=None, cfl=0.4):
    """The plain loop: each request alone (``run_steps``), first come first served."""
    from .time_integration import run_steps
    device = torch.device(device if device is not None else "cuda")
    reqs = sorted(requests, key=lambda r: r.arrival)
    t0 = time.perf_counter()
    for r in reqs:
        while time.perf_counter() - t0 < r.arrival:
            time.sleep(1e-4)
        r.admitted = time.perf_counter() - t0
        W, dx = build_initial_state(r, device)
        out = run_steps(W, dx, r.gamma, r.steps, C_CFL=cfl)
        r.result = {"mass": float(out[0].double().sum()) * dx ** 3,
                    "rho_max": float(out[0].max())}
        r.finished = time.perf_counter() - t0
    return reqs


def poisson_requests(count, rate, seed=0, n_range=(32, 256), steps_range=(50, 500),
                     ics_kinds=("overpressure", "shear")):
    """`count` requests with Poisson arrivals at `rate` per second, n and steps
    uniform in the given inclusive ranges, seeded initial states."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate, size=count)
    t = np.cumsum(gaps) - gaps[0]
    reqs = []
    for i in range(count):
        reqs.append(Request(rid=i, n=int(rng.integers(n_range[0], n_range[1] + 1)),
                            steps=int(rng.integers(steps_range[0], steps_range[1] + 1)),
                            ic=str(ics_kinds[int(rng.integers(len(ics_kinds)))]),
                            seed=int(rng.integers(2 ** 31)), arrival=float(t[i])))
    return reqs


def latency_stats(reqs):
    lat = np.array([r.latency for r in reqs if r.latency is not None])
    span = max(r.finished for r in reqs) - min(r.arrival for r in reqs)
    cells = sum(r.n ** 3 * r.steps for r in reqs)
    return {"solves": len(lat), "p50_s": float(np.percentile(lat, 50)),
            "p99_s": float(np.percentile(lat, 99)), "mean_s": float(lat.mean()),
            "solves_per_s": len(lat) / span if span > 0 else math.inf,
            "gcell_updates_per_s": cells / span / 1e9 if span > 0 else math.inf,
            "makespan_s": span}
