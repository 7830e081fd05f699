"""The oracle against the reference's golden data and the scheme's invariants (CPU)."""
import json
import os

import numpy as np
import pytest

from oracle import fluid_np as F
from oracle import ics_np as I

GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden",
                                     "iteration_counts.json")))
GAMMA = 5.0 / 3.0


def random_state(shape, seed, dtype=np.float32):
    rng = np.random.default_rng(seed)
    W = np.empty((5,) + tuple(shape), dtype)
    W[0] = rng.uniform(0.5, 2.0, shape)
    W[1:4] = rng.uniform(-1.0, 1.0, (3,) + tuple(shape))
    W[4] = rng.uniform(0.2, 3.0, shape)
    return W


@pytest.mark.parametrize("n", [32, 64])
def test_numpy_oracle_reproduces_reference_iteration_counts(n):
    """results/scaling_data.npz pins the number of CFL steps to t=0.2."""
    W, dx = I.setup_ics(n, n // 16)
    _, it = F.time_integration(W, dx, 0.2, GAMMA, True, False)
    assert it == GOLDEN["counts"][str(n)]


@pytest.mark.parametrize("n", [32, 64, 96])
def test_c_oracle_reproduces_reference_iteration_counts(oracle_lib, n):
    W, dx = I.setup_ics(n, n // 16)
    _, it = oracle_lib.time_integration(W, dx, 0.2, GAMMA, True)
    assert it == GOLDEN["counts"][str(n)]


@pytest.mark.slow
@pytest.mark.parametrize("n", [128])
def test_c_oracle_iteration_count_128(oracle_lib, n):
    W, dx = I.setup_ics(n, n // 16)
    _, it = oracle_lib.time_integration(W, dx, 0.2, GAMMA, True)
    assert it == GOLDEN["counts"][str(n)]


def test_golden_counts_agree_across_reference_runs():
    """The unsharded and GSPMD-sharded reference runs took the same steps."""
    assert GOLDEN["counts"] == GOLDEN["cross_check"]["scaling_data_sharding.npz"]


@pytest.mark.parametrize("shape", [(7, 5, 9), (16, 16, 16), (3, 1, 4), (1, 1, 1), (2, 6, 3)])
@pytest.mark.parametrize("hb", [False, True])
@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_c_oracle_bit_identical_to_numpy(oracle_lib, shape, hb, dtype):
    if hb and min(shape) < 2:
        pytest.skip("open boundaries need two cells per axis")
    W = random_state(shape, 7, dtype)
    dt_np = F._cfl_time_step(W, 0.1, GAMMA)
    dt_c = oracle_lib._cfl_time_step(W, 0.1, GAMMA)
    assert dt_np == dt_c
    a = F._evolve_state(W, 0.1, dt_np, GAMMA, hb)
    b = oracle_lib._evolve_state(W, 0.1, dt_c, GAMMA, hb)
    assert np.array_equal(a, b)


@pytest.mark.parametrize("seed", range(10))
def test_per_cell_max_speed_equals_interface_max(seed):
    """max_d |v_d|+c over cells == the reference's interface maximum, bitwise."""
    shape = (5 + seed % 3, 4 + seed % 5, 6)
    W = random_state(shape, seed)
    ref = F._cfl_time_step(W, 1.0, GAMMA, 1.0)  # = 1/max_speed
    m = F.max_wave_speed_per_cell(W, GAMMA)
    assert np.float32(1.0) / m == ref


def test_periodic_step_conserves_totals():
    W = random_state((12, 10, 8), 3, np.float64)
    dt = F._cfl_time_step(W, 0.05, GAMMA)
    W2 = F._evolve_state(W, 0.05, dt, GAMMA)
    U1 = F.conserved_state_from_primitive(W, GAMMA).sum(axis=(1, 2, 3))
    U2 = F.conserved_state_from_primitive(W2, GAMMA).sum(axis=(1, 2, 3))
    assert np.allclose(U1, U2, rtol=1e-12, atol=1e-10)


def test_uniform_state_stays_uniform():
    W = np.empty((5, 6, 5, 4), np.float32)
    W[0], W[1], W[2], W[3], W[4] = 1.3, 0.2, -0.1, 0.05, 0.7
    dt = F._cfl_time_step(W, 0.1, GAMMA)
    W2 = F._evolve_state(W, 0.1, dt, GAMMA)
    for v in range(5):
        assert np.all(W2[v] == W2[v].flat[0])
    assert np.allclose(W2, W, rtol=1e-6)


@pytest.mark.parametrize("axis,shift", [(1, 3), (2, -2), (3, 5)])
def test_roll_equivariance(axis, shift):
    W = random_state((8, 7, 6), 11)
    dt = np.float32(0.01)
    a = F._evolve_state(np.roll(W, shift, axis), 0.1, dt, GAMMA)
    b = np.roll(F._evolve_state(W, 0.1, dt, GAMMA), shift, axis)
    assert np.array_equal(a, b)


def test_open_boundaries_are_an_index_clamp():
    """x, y, z slab copies (fluid.py:384-413) == reading W at clamp(i, 1, n-2)."""
    W = random_state((6, 5, 7), 4)
    a = F._open_boundaries(W, 1)
    cl = [np.clip(np.arange(n), 1, n - 2) for n in W.shape[1:]]
    b = W[:, cl[0]][:, :, cl[1]][:, :, :, cl[2]]
    assert np.array_equal(a, b)


def test_float32_error_vs_float64_is_small():
    """The float32 scheme tracks the FP64 oracle (64^3-like but small)."""
    W, dx = I.overpressure(16, seed=1)
    W32, _ = F.run_steps(W, dx, GAMMA, 10)
    W64, _ = F.run_steps(W.astype(np.float64), dx, GAMMA, 10)
    err = np.abs(W32[0] - W64[0]).max()
    assert err < 1e-4


def test_time_integration_rejects_shard_map():
    W, dx = I.setup_ics(8, 1)
    with pytest.raises(NotImplementedError):
        F.time_integration(W, dx, 0.1, GAMMA, False, True)
