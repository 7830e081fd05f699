"""Batched stepping through the C ABI: every instance's result equals the same
instance run alone (bit for bit), in persistent and per-step launch forms,
with the exact policy also equal to the oracle."""
import math

import numpy as np
import pytest
import torch

from oracle import fluid_np as F
from tinyfluids_gb300.batching import Batch, InstanceSpec

pytestmark = pytest.mark.gpu
GAMMA = 5.0 / 3.0


def rand_state(shape, seed):
    rng = np.random.default_rng(seed)
    W = np.empty((5,) + tuple(shape), np.float32)
    W[0] = rng.uniform(0.5, 2.0, shape)
    W[1:4] = rng.uniform(-0.5, 0.5, (3,) + tuple(shape))
    W[4] = rng.uniform(0.2, 3.0, shape)
    return torch.from_numpy(W).cuda()


SHAPES = [(24, 24, 24), (32, 32, 32), (17, 20, 33), (40, 9, 31), (5, 64, 7), (48, 48, 48)]


def make_specs(tg, hb_index=None):
    specs = []
    for k, sh in enumerate(SHAPES):
        W = rand_state(sh, 100 + k)
        specs.append(InstanceSpec(W, 0.02 + 0.001 * k, GAMMA, num_steps=3 + k,
                                  handle_boundaries=(k == hb_index)))
    return specs


@pytest.mark.parametrize("persistent", [True, False])
@pytest.mark.parametrize("exact", [False, True])
@pytest.mark.parametrize("rows", [16, 8])
def test_batch_equals_instances_alone(tg, persistent, exact, rows):
    specs = make_specs(tg, hb_index=2)
    b = Batch(specs, rows=rows, exact=exact, persistent=persistent)
    outs = [o.clone() for o in b.run()]
    assert b.error() == 0
    for sp, o, s in zip(specs, outs, b.summaries()):
        alone = tg.run_steps(sp.state, sp.grid_spacing, GAMMA, sp.num_steps,
                             sp.handle_boundaries, exact=exact)
        assert s["iter"] == sp.num_steps and s["status"] == 0
        assert torch.equal(o, alone)
        if exact and sp.state.shape[1] <= 24:
            ref, _ = F.run_steps(sp.state.cpu().numpy(), sp.grid_spacing, GAMMA, sp.num_steps,
                                 sp.handle_boundaries)
            assert np.array_equal(o.cpu().numpy(), ref)


def test_batch_mixed_fixed_dt_and_t_final(tg):
    a = rand_state((20, 22, 24), 1)
    b_ = rand_state((30, 12, 40), 2)
    c = rand_state((16, 16, 16), 3)
    specs = [InstanceSpec(a, 0.05, GAMMA, num_steps=6, fixed_dt=1e-3),
             InstanceSpec(b_, 0.05, GAMMA, t_final=0.02),
             InstanceSpec(c, 0.05, GAMMA, num_steps=4, t_final=0.004)]
    b = Batch(specs, steps=64)
    outs = [o.clone() for o in b.run()]
    s = b.summaries()
    ra = tg.run_steps(a, 0.05, GAMMA, 6, dt=1e-3)
    assert torch.equal(outs[0], ra) and s[0]["iter"] == 6
    rb, itb = tg.time_integration_fn(b_, 0.05, 0.02, GAMMA, False, False)
    assert s[1]["iter"] == int(itb) and torch.equal(outs[1], rb)
    rc, itc = tg.time_integration_fn(c, 0.05, 0.004, GAMMA, False, False)
    assert s[2]["iter"] == min(4, int(itc))
    if int(itc) <= 4:
        assert torch.equal(outs[2], rc)


def test_batch_graph_replay(tg):
    specs = make_specs(tg)
    b = Batch(specs, capture_graph=True)
    first = [o.clone() for o in b.run()]
    second = [o.clone() for o in b.run()]
    for x, y, sp in zip(first, second, specs):
        assert torch.equal(x, y)
        assert torch.equal(x, tg.run_steps(sp.state, sp.grid_spacing, GAMMA, sp.num_steps))


def test_batch_continuation(tg):
    W = rand_state((28, 28, 28), 9)
    b = Batch([InstanceSpec(W, 0.05, GAMMA, t_final=0.03)], steps=3)
    b.run()
    s = b.summaries()[0]
    base = 3
    while s["status"] == 0 and s["iter"] == base:  # still running: more slots
        b.continue_run(base, 3)
        base += 3
        s = b.summaries()[0]
    ref, it = tg.time_integration_fn(W, 0.05, 0.03, GAMMA, False, False)
    assert s["iter"] == int(it)
    assert torch.equal(b.outputs[0], ref)


def test_bounded_wait_times_out_and_context_survives(tg):
    """A continuation at step 5 of instances that have taken 0 steps waits on
    a counter nothing advances: the bounded wait gives up with TF_ERR_TIMEOUT
    and the kernel returns."""
    specs = [InstanceSpec(rand_state((32, 32, 32), 4), 0.05, GAMMA, num_steps=10)]
    b = Batch(specs, wait_limit=2000)
    b._enqueue(0, 0)  # initialise ctl (iter 0, active) without stepping
    b.continue_run(5, 1)
    assert b.error() == 4
    assert b.summaries()[0]["status"] == 4
    # the context is still usable
    x = torch.ones(10, device="cuda") * 2
    assert float(x.sum()) == 20.0
    W = rand_state((8, 8, 8), 5)
    assert torch.isfinite(tg.run_steps(W, 0.1, GAMMA, 2)).all()


def test_batch_rejects_bad_specs(tg):
    W = rand_state((8, 8, 8), 1)
    with pytest.raises(ValueError):
        Batch([InstanceSpec(W, 0.1, GAMMA)])  # neither num_steps nor t_final
    with pytest.raises(tg.TinyfluidsError):
        Batch([InstanceSpec(W, -0.1, GAMMA, num_steps=2)])
    with pytest.raises(tg.TinyfluidsError):
        Batch([InstanceSpec(W, 0.1, GAMMA, num_steps=2)], rows=12)
