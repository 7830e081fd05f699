"""The reference's helper functions (fluid.py:105-413) through the C ABI:
bit-identical to the float32 oracle."""
import numpy as np
import pytest
import torch

from oracle import fluid_np as F

pytestmark = pytest.mark.gpu
GAMMA = 5.0 / 3.0


def random_state(shape, seed):
    rng = np.random.default_rng(seed)
    W = np.empty((5,) + tuple(shape), np.float32)
    W[0] = rng.uniform(0.5, 2.0, shape)
    W[1:4] = rng.uniform(-1.0, 1.0, (3,) + tuple(shape))
    W[4] = rng.uniform(0.2, 3.0, shape)
    return W


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    return t.cpu().numpy()


SHAPES = [(7, 5, 9), (16, 16, 16), (1, 3, 2)]


@pytest.mark.parametrize("shape", SHAPES)
def test_speed_of_sound(tg, shape):
    W = random_state(shape, 1)
    c = tg.speed_of_sound(dev(W[0]), dev(W[4]), GAMMA)
    assert np.array_equal(host(c), F.speed_of_sound(W[0], W[4], GAMMA))


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("vel", [1, 2, 3])
def test_euler_flux_wave_speeds_hll(tg, shape, vel):
    W = random_state(shape, 2 + vel)
    axis = vel  # X_AXIS == VELOCITY_X_INDEX etc. (fluid.py:15-21)
    L = np.roll(W, 1, axis)
    assert np.array_equal(host(tg._euler_flux(dev(W), GAMMA, vel)),
                          F._euler_flux(W, GAMMA, vel))
    sm, sp = tg.get_wave_speeds(dev(L), dev(W), GAMMA, vel)
    rsm, rsp = F.get_wave_speeds(L, W, GAMMA, vel)
    assert np.array_equal(host(sm), rsm) and np.array_equal(host(sp), rsp)
    m = tg.get_max_wave_speeds(dev(L), dev(W), GAMMA, vel)
    assert float(m) == float(F.get_max_wave_speeds(L, W, GAMMA, vel))
    assert np.array_equal(host(tg._hll_solver(dev(L), dev(W), GAMMA, vel)),
                          F._hll_solver(L, W, GAMMA, vel))


@pytest.mark.parametrize("shape", [(6, 5, 7), (2, 4, 3), (9, 9, 9)])
@pytest.mark.parametrize("g", [1, 2])
def test_open_boundaries(tg, shape, g):
    if g >= min(shape):
        pytest.skip("ghost cells must fit the axis")
    W = random_state(shape, 5)
    assert np.array_equal(host(tg._open_boundaries(dev(W), g)), F._open_boundaries(W, g))
    for axis in (1, 2, 3):
        assert np.array_equal(host(tg.fluid._open_left_boundary(dev(W), g, axis)),
                              F._open_left_boundary(W, g, axis))
        assert np.array_equal(host(tg.fluid._open_right_boundary(dev(W), g, axis)),
                              F._open_right_boundary(W, g, axis))
