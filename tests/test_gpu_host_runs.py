"""Runs of host-resident states (tf_time_integration_host): every output is
bit-identical to the same run on a device state, whatever the overlap of the
copies with the runs of neighbouring states."""
import json
import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

GAMMA = 5.0 / 3.0
GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden",
                                     "iteration_counts.json")))


@pytest.fixture(scope="module")
def tg():
    import tinyfluids_gb300 as m
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    return m


def random_state(shape, seed):
    rng = np.random.default_rng(seed)
    W = np.empty((5,) + tuple(shape), np.float32)
    W[0] = rng.uniform(0.5, 2.0, shape)
    W[1:4] = rng.uniform(-1.0, 1.0, (3,) + tuple(shape))
    W[4] = rng.uniform(0.2, 3.0, shape)
    return torch.from_numpy(W)


@pytest.mark.parametrize("shape,count", [((40, 31, 64), 5), ((64, 64, 120), 3),
                                         ((13, 9, 33), 1)])
@pytest.mark.parametrize("exact", [False, True])
def test_fixed_steps_match_device_runs(tg, shape, count, exact):
    states = [random_state(shape, 100 + k).pin_memory() for k in range(count)]
    outs, its = tg.time_integration_host(states, 0.05, None, GAMMA, False, num_steps=6,
                                         exact=exact)
    assert its == [6] * count
    for st, o in zip(states, outs):
        ref = tg.run_steps(st.cuda(), 0.05, GAMMA, 6, exact=exact)
        assert torch.equal(o, ref.cpu())


@pytest.mark.parametrize("exact", [False, True])
def test_t_final_runs_reproduce_the_golden_counts(tg, exact):
    """The reference's benchmark (setup_ics, open boundaries, t = 0.2) for
    several host states at once: the golden iteration counts, and the states
    of time_integration."""
    for n in (32, 64):
        W, dx = tg.setup_ics(n, n // 16)
        states = [W.cpu().pin_memory() for _ in range(3)]
        outs, its = tg.time_integration_host(states, dx, 0.2, GAMMA, True, exact=exact)
        assert its == [GOLDEN["counts"][str(n)]] * 3
        ref, it = tg.time_integration_fn(W, dx, 0.2, GAMMA, True, False, exact=exact)
        assert int(it) == its[0]
        for o in outs:
            assert torch.equal(o, ref.cpu())


def test_in_place_pageable_and_repeated_inputs(tg):
    """Outputs written over their own inputs; pageable host memory (no
    overlap, same results); one input repeated."""
    shape = (24, 20, 36)
    base = [random_state(shape, 7 + k) for k in range(4)]
    refs = [tg.run_steps(b.cuda(), 0.05, GAMMA, 3).cpu() for b in base]
    states = [b.clone() for b in base]  # pageable
    outs, its = tg.time_integration_host(states, 0.05, None, GAMMA, False, num_steps=3,
                                         out=states)
    assert its == [3] * 4
    for s, r, o in zip(states, refs, outs):
        assert o.data_ptr() == s.data_ptr() and torch.equal(s, r)
    one = base[0].pin_memory()
    outs, _ = tg.time_integration_host([one] * 3, 0.05, None, GAMMA, False, num_steps=3)
    for o in outs:
        assert torch.equal(o, refs[0])
    # a numpy array, alone
    o, it = tg.time_integration_host(base[1].numpy(), 0.05, None, GAMMA, False, num_steps=3)
    assert it == 3 and torch.equal(o, refs[1])


def test_device_errors_name_their_state(tg):
    """A state whose sound speed is NaN is reported with its index; an output
    over a later state's input is rejected before any copy."""
    shape = (16, 16, 16)
    states = [random_state(shape, 30 + k) for k in range(3)]
    states[1][4, 3, 3, 3] = -1.0  # negative pressure: sound speed is NaN
    with pytest.raises(tg.TinyfluidsError) as e:
        tg.time_integration_host(states, 0.05, None, GAMMA, False, num_steps=2)
    assert e.value.status == 3 and "state 1" in str(e.value)
    with pytest.raises(tg.TinyfluidsError) as e:  # an output over a later state's input
        tg.time_integration_host(states, 0.05, None, GAMMA, False, num_steps=2,
                                 out=[states[1], states[2], states[0]])
    assert e.value.status == 1


def test_runs_on_the_callers_stream(tg):
    """The runs go on the caller's current stream (here a side stream), after
    the work queued there before the call."""
    shape = (32, 32, 32)
    states = [random_state(shape, 50 + k).pin_memory() for k in range(3)]
    refs = [tg.run_steps(s.cuda(), 0.05, GAMMA, 4).cpu() for s in states]
    side = torch.cuda.Stream()
    with torch.cuda.stream(side):
        prior = torch.ones(1 << 22, device="cuda").cumsum(0)
        outs, _ = tg.time_integration_host(states, 0.05, None, GAMMA, False, num_steps=4)
    torch.cuda.synchronize()
    assert float(prior[-1]) == float(1 << 22)
    for o, r in zip(outs, refs):
        assert torch.equal(o, r)


def test_caller_workspace_is_reused(tg):
    """A workspace passed by the caller serves repeated calls (no device
    allocation per call) with the same results; one too small is rejected."""
    shape = (20, 18, 32)
    states = [random_state(shape, 70 + k).pin_memory() for k in range(3)]
    ws = torch.empty(tg.host_runs_workspace_bytes(shape, 3), dtype=torch.uint8, device="cuda")
    first, _ = tg.time_integration_host(states, 0.05, None, GAMMA, False, num_steps=4,
                                        workspace=ws)
    again, _ = tg.time_integration_host(states, 0.05, None, GAMMA, False, num_steps=4,
                                        workspace=ws)
    for a, b, s in zip(first, again, states):
        assert torch.equal(a, b)
        assert torch.equal(a, tg.run_steps(s.cuda(), 0.05, GAMMA, 4).cpu())
    with pytest.raises(ValueError):
        tg.time_integration_host(states, 0.05, None, GAMMA, False, num_steps=4,
                                 workspace=ws[:1024])
