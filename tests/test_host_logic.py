"""Host-side logic that needs no GPU: serving's admission arithmetic and tick
selection, request generation and latency statistics, the autotuner's
candidate sets, the control-block reader, and the replica timing combiner
without a process group."""
import math

import numpy as np
import pytest
import torch

from tinyfluids_gb300 import autotune, replicas, serving
from tinyfluids_gb300.fluid import CTL_ITER, CTL_STATUS, CTL_T
from tinyfluids_gb300.serving import Request, Server
from tinyfluids_gb300.time_integration import ctl_summary


def test_request_bytes_counts_two_state_buffers():
    assert serving.request_bytes(32) == 2 * 20 * 32 ** 3 + 64
    assert serving.request_bytes(256) > 2 * 20 * 256 ** 3


def test_server_arguments_and_oversized_request():
    srv = Server(hbm_budget=1e6, device="cpu")
    assert srv.tick_steps % 2 == 1  # odd: results end in the output buffer
    assert Server(hbm_budget=1e6, device="cpu", tick_steps=4).tick_steps == 5
    with pytest.raises(ValueError):
        srv.submit(Request(0, 64, 10))
    with pytest.raises(ValueError):
        Server(hbm_budget=1e6, device="cpu", policy="lifo")


class _FakeActive:
    def __init__(self, rid, n, remaining):
        self.req = Request(rid, n, remaining)
        self.remaining = remaining


def test_srpt_tick_takes_least_remaining_work_until_the_budget():
    srv = Server(hbm_budget=1e12, device="cpu", tick_steps=31, tick_budget=40_000_000)
    a = _FakeActive(0, 128, 500)   # remaining work 128^3*500 = 1049 M
    b = _FakeActive(1, 64, 20)     # 64^3*20 = 5.2 M (least)
    c = _FakeActive(2, 64, 400)    # 64^3*400 = 104.9 M
    d = _FakeActive(3, 96, 60)     # 96^3*60 = 53.1 M
    srv.active = [a, b, c, d]
    # order b, d, c, a; tick work b 5.2 M, + d 96^3*31 = 32.7 M, + c 64^3*31
    # = 40.9 M >= 40 M: stop after c
    assert [x.req.rid for x in srv._select()] == [1, 3, 2]
    srv.policy = "all"
    assert [x.req.rid for x in srv._select()] == [0, 1, 2, 3]
    srv.policy = "srpt"
    srv.tick_budget = 1
    assert [x.req.rid for x in srv._select()] == [1]
    srv.active = [a]
    assert srv._select() == [a]


def test_poisson_requests_are_seeded_and_in_range():
    r1 = serving.poisson_requests(50, 100.0, seed=3)
    r2 = serving.poisson_requests(50, 100.0, seed=3)
    assert [(r.n, r.steps, r.ic, r.seed, r.arrival) for r in r1] == \
        [(r.n, r.steps, r.ic, r.seed, r.arrival) for r in r2]
    assert r1[0].arrival == 0.0 and all(b.arrival >= a.arrival for a, b in zip(r1, r1[1:]))
    assert all(32 <= r.n <= 256 and 50 <= r.steps <= 500 for r in r1)
    assert {r.ic for r in r1} <= {"overpressure", "shear"}
    gaps = np.diff([r.arrival for r in serving.poisson_requests(4000, 50.0, seed=1)])
    assert abs(gaps.mean() - 1 / 50.0) < 0.1 / 50.0


def test_latency_stats():
    reqs = []
    for i, (arr, fin) in enumerate([(0.0, 1.0), (0.5, 1.5), (1.0, 4.0)]):
        r = Request(i, 32, 10, arrival=arr)
        r.finished = fin
        reqs.append(r)
    st = serving.latency_stats(reqs)
    assert st["solves"] == 3 and st["p50_s"] == 1.0 and st["makespan_s"] == 4.0
    assert math.isclose(st["solves_per_s"], 0.75)
    assert math.isclose(st["gcell_updates_per_s"], 3 * 32 ** 3 * 10 / 4.0 / 1e9)


def test_autotune_candidates_and_size_classes():
    c = autotune.candidates((64, 64, 64))
    assert (16, 0, "ldg") in c and (16, 64, "ldg") in c and (8, 2, "ldg") in c
    assert (8, 0, "ym") in c and (16, 32, "ym") in c
    assert all(r in (8, 16, 32) and lx <= 64 for r, lx, _ in c)
    assert all(r in (8, 16) for r, _, lay in c if lay == "ym")
    assert autotune.size_class(1) == 16 and autotune.size_class(33) == 48
    assert autotune.size_class(512) == 512 and autotune.size_class(5000) == 1024


def test_ctl_summary_reads_the_control_block():
    ctl = torch.zeros(16, dtype=torch.int32)
    ctl.view(torch.float32)[CTL_T] = 0.25
    ctl[CTL_ITER] = 17
    ctl[CTL_STATUS] = 3
    assert ctl_summary(ctl) == {"t": 0.25, "iter": 17, "status": 3}


def test_job_throughput_without_a_process_group():
    value, ms = replicas.job_throughput(512 ** 3, 200, 330.0, 1)
    assert ms == 330.0 and math.isclose(value, 512 ** 3 * 200 / 0.33 / 1e9)
