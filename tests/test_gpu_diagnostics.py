"""In-pass diagnostics (conserved totals, rho/p slice) on the GPU.

The diagnostics step must return the same state as the plain step (bitwise),
slices equal to the stored state's plane, and totals equal to float64 sums of
the reference conversion of the stored state (fluid.py:30-67, applied by the
oracle).  Both kernels sum with compensated float32 per thread and float64
across threads, so the bar is TOTALS_RTOL relative to the sum of magnitudes.
"""
import numpy as np
import pytest
import torch

from oracle import fluid_np as F

pytestmark = pytest.mark.gpu

GAMMA = 5.0 / 3.0
TOTALS_RTOL = 1e-10
SHAPES = [(1, 1, 1), (5, 7, 33), (33, 17, 61), (40, 31, 64)]


def random_state(shape, seed):
    rng = np.random.default_rng(seed)
    W = np.empty((5,) + tuple(shape), np.float32)
    W[0] = rng.uniform(0.5, 2.0, shape)
    W[1:4] = rng.uniform(-1.0, 1.0, (3,) + tuple(shape))
    W[4] = rng.uniform(0.2, 3.0, shape)
    return W


def oracle_totals(W):
    U = F.conserved_state_from_primitive(W, GAMMA)
    return U.reshape(5, -1).astype(np.float64).sum(axis=1)


def scale_of(W):
    """Sum of |conserved| per variable: the scale of the summation error."""
    U = F.conserved_state_from_primitive(W, GAMMA)
    return np.abs(U.reshape(5, -1).astype(np.float64)).sum(axis=1)


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("exact", [False, True])
@pytest.mark.parametrize("hb", [False, True])
def test_step_with_diagnostics(tg, shape, exact, hb):
    if hb and min(shape) < 2:
        pytest.skip("open boundaries need two cells per axis")
    W = torch.from_numpy(random_state(shape, 3)).cuda()
    dx, dt = 0.05, 0.004
    plain = tg._evolve_state(W, dx, dt, GAMMA, hb, exact=exact)
    for tile in (None, (8, 3), (32, 2)):
        out, totals, sl = tg.diagnostics.step_with_diagnostics(W, dx, dt, GAMMA, hb,
                                                               exact=exact, tile=tile)
        assert torch.equal(out, plain), (shape, tile)
        z = shape[2] // 2
        assert torch.equal(sl[0], out[0, :, :, z]) and torch.equal(sl[1], out[4, :, :, z])
        h = out.cpu().numpy()
        ref = oracle_totals(h)
        err = np.abs(totals.cpu().numpy() - ref) / scale_of(h)
        assert err.max() < TOTALS_RTOL, (shape, tile, err)


@pytest.mark.parametrize("shape", SHAPES)
def test_read_pass_diagnostics(tg, shape):
    Wn = random_state(shape, 4)
    W = torch.from_numpy(Wn).cuda()
    z = shape[2] - 1
    totals, sl = tg.diagnostics.diagnostics(W, GAMMA, z=z)
    err = np.abs(totals.cpu().numpy() - oracle_totals(Wn)) / scale_of(Wn)
    assert err.max() < TOTALS_RTOL, err
    assert torch.equal(sl[0], W[0, :, :, z]) and torch.equal(sl[1], W[4, :, :, z])
    t2, none = tg.diagnostics.diagnostics(W, GAMMA, slices=False)
    assert none is None and torch.equal(t2, totals)


@pytest.mark.parametrize("steps", [1, 2, 7])
@pytest.mark.parametrize("fixed_dt", [None, 2e-3])
def test_run_with_final_diagnostics_matches_run_steps(tg, steps, fixed_dt):
    W, dx = tg.overpressure(40, seed=2)
    ref = tg.run_steps(W, dx, GAMMA, steps, dt=fixed_dt)
    out, totals, sl = tg.diagnostics.run_steps_with_diagnostics(W, dx, GAMMA, steps, dt=fixed_dt)
    assert torch.equal(out, ref)
    t_read, sl_read = tg.diagnostics.diagnostics(out, GAMMA)
    assert torch.equal(sl, sl_read)
    rel = (totals - t_read).abs() / t_read.abs().clamp_min(1e-30)
    assert float(rel[[0, 4]].max()) < TOTALS_RTOL


def test_periodic_run_conserves_totals(tg):
    W, dx = tg.shear_layer(48, seed=1, amplitude=0.05)
    t0, _ = tg.diagnostics.diagnostics(W, GAMMA, slices=False)
    out, t1, _ = tg.diagnostics.run_steps_with_diagnostics(W, dx, GAMMA, 30, slices=False)
    scale = tg.diagnostics.diagnostics(out.abs(), GAMMA, slices=False)[0].abs()
    drift = ((t1 - t0).abs() / scale.clamp_min(1e-30)).cpu().numpy()
    # mass, momentum and energy telescope under periodic wrap; what is left is
    # float32 rounding of the stored state
    assert drift.max() < 1e-5, drift


def test_diagnostics_arguments(tg):
    W = torch.from_numpy(random_state((4, 4, 6), 1)).cuda()
    with pytest.raises(ValueError):
        tg.diagnostics.diagnostics(W, GAMMA, z=6)
    with pytest.raises(ValueError):
        tg.diagnostics.step_with_diagnostics(W, 0.1, 0.001, GAMMA, z=-1)
    with pytest.raises(ValueError):
        tg.diagnostics.run_steps_with_diagnostics(W, 0.1, GAMMA, 0)
