"""Parity of the CUDA path (through the C ABI) with the oracle.

Bar: the exact policy (TF_FLAG_EXACT, the reference's op order) is
bit-identical to the float32 oracle; the fast policy agrees with it to
FAST_STEP_RTOL per step (relative to each variable's max magnitude) and its
density error against the FP64 oracle stays within 2x the reference float32
scheme's own error.
"""
import ctypes
import json
import os

import numpy as np
import pytest
import torch

from oracle import fluid_np as F
from oracle import ics_np as I

pytestmark = pytest.mark.gpu

GAMMA = 5.0 / 3.0
FAST_STEP_RTOL = 2e-6   # one fast step vs the float32 reference scheme
GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden",
                                     "iteration_counts.json")))

SHAPES = [(1, 1, 1), (2, 3, 5), (5, 7, 33), (16, 16, 16), (33, 17, 61), (40, 31, 64),
          (3, 64, 29), (64, 15, 2)]


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
    return t.detach().cpu().numpy()


def rel_err(a, b):
    scale = np.abs(b).reshape(5, -1).max(axis=1).reshape(5, 1, 1, 1) + 1e-30
    return float((np.abs(a - b) / scale).max())


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("hb", [False, True])
def test_exact_fused_step_bit_identical(tg, shape, hb):
    if hb and min(shape) < 2:
        pytest.skip("open boundaries need two cells per axis")
    W = random_state(shape, hash(shape) % 1000)
    dx = 0.05
    dt = F._cfl_time_step(W, dx, GAMMA)
    ref = F._evolve_state(W, dx, dt, GAMMA, hb)
    for tile in (None, (8, 3), (16, 1), (32, 2), (32, 5, "tma"), (8, 3, "ym"), (16, 1, "ym")):
        out = host(tg._evolve_state(dev(W), dx, float(dt), GAMMA, hb, exact=True, tile=tile))
        assert np.array_equal(out, ref), (shape, hb, tile, np.abs(out - ref).max())


@pytest.mark.parametrize("shape", [(5, 7, 33), (16, 16, 16), (9, 1, 4)])
@pytest.mark.parametrize("axis", [1, 2, 3])
def test_exact_sweep_bit_identical(tg, shape, axis):
    W = random_state(shape, 5)
    dt = np.float32(0.003)
    ref = F._evolve_state_along_axis(W, 0.05, dt, GAMMA, axis)
    out = host(tg._evolve_state_along_axis(dev(W), 0.05, float(dt), GAMMA, axis, exact=True))
    assert np.array_equal(out, ref)


@pytest.mark.parametrize("shape", SHAPES)
def test_cfl_time_step_bit_identical(tg, shape):
    W = random_state(shape, 9)
    ref = F._cfl_time_step(W, 0.02, GAMMA)
    out = tg._cfl_time_step(dev(W), 0.02, GAMMA)
    assert out.shape == () and out.dtype == torch.float32
    assert float(out) == float(ref)


def test_conversions_bit_identical(tg):
    W = random_state((7, 9, 11), 2)
    U = F.conserved_state_from_primitive(W, GAMMA)
    assert np.array_equal(host(tg.conserved_state_from_primitive(dev(W), GAMMA)), U)
    assert np.array_equal(host(tg.primitive_state_from_conserved(dev(U), GAMMA)),
                          F.primitive_state_from_conserved(U, GAMMA))


def test_dt_from_device_tensor(tg):
    W = random_state((12, 10, 8), 4)
    dt = tg._cfl_time_step(dev(W), 0.05, GAMMA)
    a = host(tg._evolve_state(dev(W), 0.05, dt, GAMMA, exact=True))
    b = F._evolve_state(W, 0.05, F._cfl_time_step(W, 0.05, GAMMA), GAMMA)
    assert np.array_equal(a, b)


_ORACLE_RUNS = {}


@pytest.mark.parametrize("n", [32, 64, 96, 128, 196, 256])
@pytest.mark.parametrize("host_loop", [False, True])
def test_exact_time_integration_reproduces_reference_counts(tg, oracle_lib, n, host_loop):
    """The reference's golden data: steps to t=0.2 for setup_ics(n, n//16),
    with the loop as a device-side graph while node and as host-checked chunks."""
    W, dx = tg.setup_ics(n, n // 16)
    Wf, it = tg.time_integration_fn(W, dx, 0.2, GAMMA, True, False, exact=True,
                                    host_loop=host_loop)
    assert int(it) == GOLDEN["counts"][str(n)]
    # the final state against the C oracle's (up to 226 steps of 256^3; one
    # oracle run per size serves both loop forms)
    if n not in _ORACLE_RUNS:
        _ORACLE_RUNS[n] = oracle_lib.time_integration(host(W), dx, 0.2, GAMMA, True)
    ref, rit = _ORACLE_RUNS[n]
    assert rit == int(it)
    assert np.array_equal(host(Wf), ref)


@pytest.mark.parametrize("n", [32, 64, 96, 128, 196, 256])
def test_fast_time_integration_reproduces_reference_counts(tg, n):
    W, dx = tg.setup_ics(n, n // 16)
    _, it = tg.time_integration_fn(W, dx, 0.2, GAMMA, True, False)
    assert int(it) == GOLDEN["counts"][str(n)]


@pytest.mark.parametrize("shape,t_final", [((48, 48, 48), 0.05), ((33, 17, 61), 0.02),
                                           ((1, 1, 1), 0.3)])
def test_graph_loop_matches_host_loop(tg, shape, t_final):
    W = dev(random_state(shape, 8))
    a, ia = tg.time_integration_fn(W, 0.05, t_final, GAMMA, False, False)
    b, ib = tg.time_integration_fn(W, 0.05, t_final, GAMMA, False, False, host_loop=True)
    assert int(ia) == int(ib) > 0
    assert torch.equal(a, b)
    # repeated calls build a fresh graph each time and give the same result
    c, ic = tg.time_integration_fn(W, 0.05, t_final, GAMMA, False, False)
    assert int(ic) == int(ia) and torch.equal(c, a)


@pytest.mark.parametrize("hb", [False, True])
def test_step_is_one_loop_iteration(tg, oracle_lib, hb):
    W = dev(random_state((20, 24, 28), 13))
    out, dt = tg.step(W, 0.05, GAMMA, 0.4, hb, return_dt=True)
    assert torch.equal(out, tg.run_steps(W, 0.05, GAMMA, 1, hb))
    assert torch.equal(out, tg._evolve_state(W, 0.05, dt, GAMMA, hb))
    ex, dte = tg.step(W, 0.05, GAMMA, 0.4, hb, exact=True, return_dt=True)
    ref, rit = oracle_lib.time_integration(host(W), 0.05, float("inf"), GAMMA, hb, max_steps=1)
    assert rit == 1 and np.array_equal(host(ex), ref)
    assert float(dte) == float(oracle_lib._cfl_time_step(host(W), 0.05, GAMMA))


def test_setup_ics_matches_reference_builder(tg):
    W, dx = tg.setup_ics(40, 40 // 16)
    Wn, dxn = I.setup_ics(40, 40 // 16)
    assert dx == dxn and np.array_equal(host(W), Wn)


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("hb", [False, True])
def test_fast_step_close_to_reference(tg, shape, hb):
    if hb and min(shape) < 2:
        pytest.skip("open boundaries need two cells per axis")
    W = random_state(shape, 21)
    dt = F._cfl_time_step(W, 0.05, GAMMA)
    ref = F._evolve_state(W, 0.05, dt, GAMMA, hb)
    out = host(tg._evolve_state(dev(W), 0.05, float(dt), GAMMA, hb))
    assert rel_err(out, ref) < FAST_STEP_RTOL


@pytest.mark.parametrize("shape", [(70, 45, 77), (37, 29, 124)])
def test_fast_step_independent_of_tile_shape(tg, shape):
    """Every tile layout, height and chunk length gives the same bits (odd nz:
    the y-marching tile's 4-byte path; even nz: its 8-byte pair path)."""
    W = dev(random_state(shape, 8))
    outs = [host(tg._evolve_state(W, 0.05, 1e-3, GAMMA, tile=t))
            for t in (None, (16, 64), (16, 5), (8, 1), (8, 70), (32, 7), (32, 70, "tma"), (32, 1),
                      (8, 0, "ym"), (8, 1, "ym"), (8, 7, "ym"), (16, 0, "ym"), (16, 3, "ym"))]
    for o in outs[1:]:
        assert np.array_equal(o, outs[0])


YM_SHAPES = [(1, 1, 1), (2, 3, 5), (5, 7, 33), (4, 9, 60), (9, 13, 62), (13, 5, 121),
             (40, 31, 64), (3, 64, 29), (64, 15, 2), (17, 2, 130), (6, 5, 4), (5, 6, 6),
             (7, 3, 120), (3, 4, 122)]


@pytest.mark.parametrize("shape", YM_SHAPES)
@pytest.mark.parametrize("hb", [False, True])
@pytest.mark.parametrize("exact", [False, True])
def test_y_marching_tile_bitwise(tg, shape, hb, exact):
    """The y-marching tile (x rows across warps, z pairs in lanes, derived
    x halo rows, cp.async input ring) equals the x-marching tile bit for bit
    for ragged shapes, both boundary modes, both policies and every chunk
    length; the exact form also equals the oracle."""
    if hb and min(shape) < 2:
        pytest.skip("open boundaries need two cells per axis")
    W = random_state(shape, 53)
    dt = F._cfl_time_step(W, 0.05, GAMMA)
    Wd = dev(W)
    ref = tg._evolve_state(Wd, 0.05, float(dt), GAMMA, hb, exact=exact, tile=(16, 0, "ldg"))
    for tile in ((8, 0, "ym"), (8, 1, "ym"), (8, 2, "ym"), (16, 0, "ym"), (16, 3, "ym")):
        out = tg._evolve_state(Wd, 0.05, float(dt), GAMMA, hb, exact=exact, tile=tile)
        assert torch.equal(out, ref), (shape, hb, exact, tile)
    if exact:
        assert np.array_equal(host(ref), F._evolve_state(W, 0.05, dt, GAMMA, hb))


@pytest.mark.parametrize("shape", [(40, 31, 64), (9, 13, 62)])
def test_y_marching_conserved_and_diagnostics(tg, shape):
    """The conserved-in/out step (the adjoint's forward pass) and the
    diagnostics step in the y-marching tile equal their x-marching forms."""
    W = dev(random_state(shape, 61))
    U = tg.conserved_state_from_primitive(W, GAMMA)
    a = tg._evolve_state(U, 0.05, 2e-3, GAMMA, conserved=True)
    b = tg._evolve_state(U, 0.05, 2e-3, GAMMA, conserved=True, tile=(8, 0, "ym"))
    assert torch.equal(a, b)
    nz = shape[2]
    ra = tg.diagnostics.step_with_diagnostics(W, 0.05, 2e-3, GAMMA, z=nz // 2,
                                              tile=(16, 0, "ldg"))
    rb = tg.diagnostics.step_with_diagnostics(W, 0.05, 2e-3, GAMMA, z=nz // 2,
                                              tile=(8, 3, "ym"))
    assert torch.equal(ra[0], rb[0])  # the state
    assert torch.equal(ra[2], rb[2])  # the rho / p slice
    # the totals are summed in another order: equal to float64 rounding
    assert torch.allclose(ra[1], rb[1], rtol=1e-10, atol=0)


def test_y_marching_loops_match(tg):
    """Run loops (fixed step count and the device-side t_final loop) in the
    y-marching tile reproduce the x-marching tile's states."""
    W, dx = tg.shear_layer(64, seed=2)
    a = tg.run_steps(W, dx, GAMMA, 9, tile=(16, 16, "ldg"))
    b = tg.run_steps(W, dx, GAMMA, 9, tile=(8, 16, "ym"))
    assert torch.equal(a, b)
    c, ic = tg.time_integration_fn(W, dx, 0.01, GAMMA, False, False, tile=(16, 0, "ldg"))
    d, id_ = tg.time_integration_fn(W, dx, 0.01, GAMMA, False, False, tile=(8, 0, "ym"))
    assert int(ic) == int(id_) and torch.equal(c, d)


@pytest.mark.parametrize("shape", [(5, 7, 33), (40, 31, 64), (17, 66, 3)])
@pytest.mark.parametrize("hb", [False, True])
def test_fast_fused_step_equals_fast_sweeps(tg, shape, hb):
    """The fused kernel (packed pairs, conserved state between sweeps) and three
    per-axis fast sweeps run the same op sequence: equal bit for bit."""
    W = dev(random_state(shape, 31))
    dt = 2e-3
    fused = tg._evolve_state(W, 0.05, dt, GAMMA, hb)
    a = tg._evolve_state_along_axis(W, 0.05, dt, GAMMA, 1, open_boundaries=hb,
                                    conserved_out=True)
    b = tg._evolve_state_along_axis(a, 0.05, dt, GAMMA, 2, conserved_in=True,
                                    conserved_out=True)
    c = tg._evolve_state_along_axis(b, 0.05, dt, GAMMA, 3, conserved_in=True)
    assert torch.equal(fused, c)


@pytest.mark.parametrize("shape", [(5, 7, 33), (40, 31, 64), (1, 1, 1)])
def test_fused_conserved_step_equals_conserved_sweeps(tg, shape):
    """The conserved-in/out fused step (the adjoint's forward pass) equals the
    three conserved fast sweeps bit for bit."""
    U = tg.conserved_state_from_primitive(dev(random_state(shape, 41)), GAMMA)
    dt = 2e-3
    fused = tg._evolve_state(U, 0.05, dt, GAMMA, conserved=True)
    a = tg._evolve_state_along_axis(U, 0.05, dt, GAMMA, 1, conserved_in=True, conserved_out=True)
    b = tg._evolve_state_along_axis(a, 0.05, dt, GAMMA, 2, conserved_in=True, conserved_out=True)
    c = tg._evolve_state_along_axis(b, 0.05, dt, GAMMA, 3, conserved_in=True, conserved_out=True)
    assert torch.equal(fused, c)
    with pytest.raises(tg.TinyfluidsError):
        tg._evolve_state(U, 0.05, dt, GAMMA, conserved=True, exact=True)
    with pytest.raises(tg.TinyfluidsError):
        tg._evolve_state(U, 0.05, dt, GAMMA, conserved=True, tile=(8, 4))
    with pytest.raises(tg.TinyfluidsError):
        tg._evolve_state(U, 0.05, dt, GAMMA, tile=(32, 0, "ym"))


@pytest.mark.parametrize("axis,shift", [(1, 3), (2, -5), (3, 31)])
def test_fast_step_roll_equivariant(tg, axis, shift):
    W = random_state((40, 36, 70), 12)
    a = host(tg._evolve_state(dev(np.roll(W, shift, axis)), 0.05, 2e-3, GAMMA))
    b = np.roll(host(tg._evolve_state(dev(W), 0.05, 2e-3, GAMMA)), shift, axis)
    assert np.array_equal(a, b)


def test_fast_run_conserves_totals(tg):
    W, dx = tg.overpressure(48, seed=5)
    U0 = F.conserved_state_from_primitive(host(W).astype(np.float64), GAMMA).sum(axis=(1, 2, 3))
    Wf = tg.run_steps(W, dx, GAMMA, 20)
    U1 = F.conserved_state_from_primitive(host(Wf).astype(np.float64), GAMMA).sum(axis=(1, 2, 3))
    assert np.allclose(U0, U1, rtol=2e-5, atol=1e-3)


def test_overpressure_64_accuracy_vs_fp64(tg, oracle_lib):
    """Config 1: 64^3 overpressure, CFL 0.4, 100 steps.  The fast path's density
    error against the FP64 oracle is within 2x the reference float32 scheme's."""
    W, dx = tg.overpressure(64, seed=0)
    W0 = host(W)
    ref32, dts32 = oracle_lib.run_steps(W0, dx, GAMMA, 100)
    ref64, _ = oracle_lib.run_steps(W0.astype(np.float64), dx, GAMMA, 100)
    fast = host(tg.run_steps(W, dx, GAMMA, 100))
    exact = host(tg.run_steps(W, dx, GAMMA, 100, exact=True))
    assert np.array_equal(exact, ref32)
    e_ref_l1 = np.abs(ref32[0] - ref64[0]).mean()
    e_ref_inf = np.abs(ref32[0] - ref64[0]).max()
    e_fast_l1 = np.abs(fast[0] - ref64[0]).mean()
    e_fast_inf = np.abs(fast[0] - ref64[0]).max()
    print(f"density error vs FP64: reference-f32 L1 {e_ref_l1:.3e} Linf {e_ref_inf:.3e}; "
          f"fast L1 {e_fast_l1:.3e} Linf {e_fast_inf:.3e}")
    assert e_fast_l1 <= 2 * e_ref_l1 and e_fast_inf <= 2 * e_ref_inf


@pytest.mark.parametrize("n", [64, 128])
def test_reference_benchmark_accuracy_vs_fp64(tg, oracle_lib, n):
    """The reference's own benchmark state (setup_ics(n, n//16), open
    boundaries) over its golden number of steps to t = 0.2: the fast path's
    density error against the FP64 oracle is within 2x the reference float32
    scheme's, and the exact path equals the float32 oracle bit for bit."""
    W, dx = tg.setup_ics(n, n // 16)
    steps = GOLDEN["counts"][str(n)]
    W0 = host(W)
    ref32, _ = oracle_lib.run_steps(W0, dx, GAMMA, steps, True)
    ref64, _ = oracle_lib.run_steps(W0.astype(np.float64), dx, GAMMA, steps, True)
    fast = host(tg.run_steps(W, dx, GAMMA, steps, True))
    exact = host(tg.run_steps(W, dx, GAMMA, steps, True, exact=True))
    assert np.array_equal(exact, ref32)
    e_ref = np.abs(ref32[0] - ref64[0])
    e_fast = np.abs(fast[0] - ref64[0])
    print(f"{n}^3 density error vs FP64: reference-f32 L1 {e_ref.mean():.3e} "
          f"Linf {e_ref.max():.3e}; fast L1 {e_fast.mean():.3e} Linf {e_fast.max():.3e}")
    assert e_fast.mean() <= 2 * e_ref.mean() and e_fast.max() <= 2 * e_ref.max()


@pytest.mark.parametrize("host_loop", [False, True])
def test_nonfinite_state_is_reported(tg, host_loop):
    W = random_state((8, 8, 8), 1)
    W[4, 3, 3, 3] = -1.0  # negative pressure: sound speed is NaN
    with pytest.raises(tg.TinyfluidsError) as e:
        tg.time_integration_fn(dev(W), 0.1, 0.5, GAMMA, False, False, host_loop=host_loop)
    assert e.value.status == 3


@pytest.mark.parametrize("n,cap", [(32, 5), (32, 10), (32, 17), (168, 5)])
def test_graph_loop_stops_at_its_step_cap(tg, n, cap):
    """The device-side while loop ends after `cap` steps even though t_final
    is not reached: TF_ERR_TIMEOUT, exactly cap steps, wherever the cap falls
    in a while-node body (8 steps per body at 32^3, 2 at 168^3)."""
    W, dx = tg.setup_ics(n, 2)
    lib = tg._lib.load()
    lib.tf_debug_set_graph_loop_cap(cap)
    try:
        with pytest.raises(tg.TinyfluidsError) as e:
            tg.time_integration_fn(W, dx, 0.2, GAMMA, True, False)
        assert e.value.status == 4 and ("after %d steps" % cap) in str(e.value)
    finally:
        lib.tf_debug_set_graph_loop_cap(0)
    if n == 32:
        _, it = tg.time_integration_fn(W, dx, 0.2, GAMMA, True, False)
        assert int(it) == GOLDEN["counts"]["32"]


@pytest.mark.parametrize("host_loop", [False, True])
def test_stalled_time_is_reported(tg, host_loop):
    """A loop whose float32 t no longer advances (t + dt == t: the reference
    would loop forever) stops with TF_ERR_NONFINITE, in the device-side graph
    loop and in the host-checked loop; the loop starts at t = 1e7 through the
    test hook, where the ~1e-3 CFL steps of this state round away."""
    W, dx = tg.setup_ics(32, 2)
    lib = tg._lib.load()
    assert lib.tf_debug_set_loop_start_time(ctypes.c_float(1e7)) == 0
    try:
        with pytest.raises(tg.TinyfluidsError) as e:
            tg.time_integration_fn(W, dx, 2e7, GAMMA, True, False, host_loop=host_loop)
        assert e.value.status == 3, str(e.value)
    finally:
        assert lib.tf_debug_set_loop_start_time(ctypes.c_float(0.0)) == 0
    _, it = tg.time_integration_fn(W, dx, 0.2, GAMMA, True, False, host_loop=host_loop)
    assert int(it) == GOLDEN["counts"]["32"]


@pytest.mark.parametrize("shape", [(40, 31, 64), (13, 9, 121), (9, 13, 62)])
def test_64bit_addressing_form_bitwise(tg, shape):
    """The addressing form of grids of 2^31 or more cells (64-bit offsets),
    forced on small grids through the test hook, gives the same bits as the
    32-bit form in both tiles, fast and conserved."""
    W = dev(random_state(shape, 71))
    U = tg.conserved_state_from_primitive(W, GAMMA)
    tiles = (None, (16, 0, "ldg"), (8, 0, "ym"), (16, 3, "ym"))
    ref = [tg._evolve_state(W, 0.05, 2e-3, GAMMA, tile=t) for t in tiles]
    refc = tg._evolve_state(U, 0.05, 2e-3, GAMMA, conserved=True)
    lib = tg._lib.load()
    assert lib.tf_debug_force_64bit_offsets(1) == 0
    try:
        out = [tg._evolve_state(W, 0.05, 2e-3, GAMMA, tile=t) for t in tiles]
        outc = tg._evolve_state(U, 0.05, 2e-3, GAMMA, conserved=True)
    finally:
        assert lib.tf_debug_force_64bit_offsets(0) == 0
    for t, a, b in zip(tiles, ref, out):
        assert torch.equal(a, b), t
    assert torch.equal(refc, outc)


def test_empty_axis_rejected(tg):
    with pytest.raises(ValueError):
        tg._evolve_state(torch.zeros(5, 0, 4, 4, device="cuda"), 0.1, 1e-3, GAMMA)
    with pytest.raises(ValueError):
        tg.time_integration_fn(torch.zeros(5, 4, 4, 0, device="cuda"), 0.1, 0.1, GAMMA, False,
                               False)


def test_time_integration_zero_and_negative_t_final(tg):
    W = dev(random_state((6, 6, 6), 3))
    Wf, it = tg.time_integration_fn(W, 0.1, 0.0, GAMMA, False, False)
    assert int(it) == 0 and torch.equal(Wf, W)


@pytest.mark.parametrize("shape", [(16, 16, 16), (40, 31, 64), (7, 9, 4), (5, 45, 8),
                                   (33, 17, 60), (2, 2, 12), (130, 3, 4), (1, 5, 8), (3, 3, 33)])
@pytest.mark.parametrize("hb", [False, True])
@pytest.mark.parametrize("exact", [False, True])
def test_tma_and_load_planes_agree_bitwise(tg, shape, hb, exact):
    """TMA-staged planes (shared-memory ring) and per-thread loads feed the same
    arithmetic: identical results, for every tile height, ragged and wrapped
    edges included; the exact form also equals the oracle."""
    if hb and min(shape) < 2:
        pytest.skip("open boundaries need two cells per axis")
    W = random_state(shape, 41)
    dt = F._cfl_time_step(W, 0.05, GAMMA)
    Wd = dev(W)
    for rows, lx in ((8, 3), (16, 0), (32, 5)):
        a = tg._evolve_state(Wd, 0.05, float(dt), GAMMA, hb, exact=exact, tile=(rows, lx, "ldg"))
        b = tg._evolve_state(Wd, 0.05, float(dt), GAMMA, hb, exact=exact, tile=(rows, lx, "tma"))
        assert torch.equal(a, b), (rows, lx)
    if exact:
        assert np.array_equal(host(b), F._evolve_state(W, 0.05, dt, GAMMA, hb))


def test_tma_loop_matches_load_loop(tg):
    W, dx = tg.shear_layer(64, seed=2)
    a = tg.run_steps(W, dx, GAMMA, 9, tile=(16, 16, "ldg"))
    b = tg.run_steps(W, dx, GAMMA, 9, tile=(16, 16, "tma"))
    assert torch.equal(a, b)


@pytest.mark.parametrize("shape", [(40, 36, 64), (64, 64, 120)])
def test_run_steps_inside_user_graph_capture(tg, shape):
    """A step loop captured into the caller's own CUDA graph (the steps are
    launched as programmatic dependents of one another) replays to the same
    bits as the eager loop, twice over, in both tile layouts."""
    W = dev(random_state(shape, 91))
    ref = tg.run_steps(W, 0.05, GAMMA, 7)
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        tg.run_steps(W, 0.05, GAMMA, 7)  # warm-up outside the capture
    torch.cuda.current_stream().wait_stream(side)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        out = tg.run_steps(W, 0.05, GAMMA, 7)
    for _ in range(2):
        out.zero_()
        g.replay()
        torch.cuda.synchronize()
        assert torch.equal(out, ref)
