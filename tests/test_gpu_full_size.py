"""The 512^3 benchmark workload (shear layer, the bench's default) at full size.

Size-independent properties of the fused step on the full grid; one exact
step against the C oracle bit for bit (the oracle finishes a 512^3 step in a
couple of seconds on the host cores); and the accuracy bar of the benchmark
on this very configuration: over 10 CFL steps the fast default's density
error against the FP64 oracle stays within 2x the reference float32 scheme's.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

GAMMA = 5.0 / 3.0
N = 512
FAST_STEP_RTOL = 2e-6  # one fast step vs the float32 reference scheme (test_gpu_parity.py)
K_ACCURACY = 10


@pytest.fixture(scope="module")
def shear(tg):
    W, dx = tg.shear_layer(N, seed=0)
    dt = float(tg._cfl_time_step(W, dx, GAMMA))
    return W, dx, dt


def test_exact_step_bit_identical_to_oracle(tg, oracle_lib, shear):
    W, dx, dt = shear
    out = tg._evolve_state(W, dx, dt, GAMMA, exact=True)
    ref = oracle_lib._evolve_state(W.cpu().numpy(), dx, np.float32(dt), GAMMA)
    assert np.array_equal(out.cpu().numpy(), ref)


def test_cfl_dt_matches_oracle(tg, oracle_lib, shear):
    W, dx, dt = shear
    assert np.float32(dt) == oracle_lib._cfl_time_step(W.cpu().numpy(), dx, GAMMA)


def test_tile_shapes_agree(tg, shear):
    W, dx, dt = shear
    ref = tg._evolve_state(W, dx, dt, GAMMA)
    for tile in ((8, 64), (32, 128), (16, 7), (16, 0, "ldg"), (8, 0, "ym"), (16, 64, "ym")):
        assert torch.equal(tg._evolve_state(W, dx, dt, GAMMA, tile=tile), ref), tile


def test_open_boundary_tiles_agree(tg, shear):
    """Open boundaries at 512^3 (the built-in choice: the y-marching tile
    with its z-edge pair fix-up) equal the x-marching tile bit for bit, and
    one exact step with open boundaries equals the exact x-marching step."""
    W, dx, dt = shear
    assert tg.resolved_tile((N, N, N), True, exact=False)[2] == "ym"
    ref = tg._evolve_state(W, dx, dt, GAMMA, True, tile=(16, 0, "ldg"))
    for tile in (None, (8, 0, "ym"), (8, 37, "ym"), (16, 0, "ym")):
        assert torch.equal(tg._evolve_state(W, dx, dt, GAMMA, True, tile=tile), ref), tile


def test_fused_equals_three_sweeps(tg, shear):
    W, dx, dt = shear
    fused = tg._evolve_state(W, dx, dt, GAMMA)
    a = tg._evolve_state_along_axis(W, dx, dt, GAMMA, 1, conserved_out=True)
    b = tg._evolve_state_along_axis(a, dx, dt, GAMMA, 2, conserved_in=True, conserved_out=True)
    del a
    c = tg._evolve_state_along_axis(b, dx, dt, GAMMA, 3, conserved_in=True)
    assert torch.equal(fused, c)


def test_roll_equivariance(tg, shear):
    W, dx, dt = shear
    shifts, dims = (7, -13, 29), (1, 2, 3)
    a = tg._evolve_state(torch.roll(W, shifts, dims), dx, dt, GAMMA)
    b = torch.roll(tg._evolve_state(W, dx, dt, GAMMA), shifts, dims)
    assert torch.equal(a, b)


def test_run_conserves_totals(tg, shear):
    W, dx, _ = shear
    t0, _ = tg.diagnostics.diagnostics(W, GAMMA, slices=False)
    out, t1, sl = tg.diagnostics.run_steps_with_diagnostics(W, dx, GAMMA, 10)
    scale, _ = tg.diagnostics.diagnostics(out.abs(), GAMMA, slices=False)
    drift = ((t1 - t0).abs() / scale).cpu().numpy()
    assert drift.max() < 1e-6, drift
    assert torch.equal(sl[0], out[0, :, :, N // 2])


def test_long_run_stays_finite_and_conservative(tg, shear):
    """2000 CFL steps of the benchmark state (about 0.6 time units): the run
    reports no device error and mass and energy stay conserved to float32
    rounding of the stored state (the per-step drift is ~1e-10 of the total;
    a non-conservative update would drift by orders of magnitude more)."""
    W, dx, _ = shear
    t0, _ = tg.diagnostics.diagnostics(W, GAMMA, slices=False)
    out, ctl = tg.run_steps(W, dx, GAMMA, 2000, return_ctl=True)
    summ = tg.time_integration.ctl_summary(ctl)
    assert summ["status"] == 0 and summ["iter"] == 2000 and summ["t"] > 0.3
    t1, _ = tg.diagnostics.diagnostics(out, GAMMA, slices=False)
    rel = ((t1 - t0).abs() / t0.abs()).cpu().numpy()
    print(f"relative drift after 2000 steps: mass {rel[0]:.2e}, energy {rel[4]:.2e}")
    assert rel[0] < 5e-6 and rel[4] < 1e-4, rel
    assert bool(torch.isfinite(out).all())


def test_fast_default_accuracy_vs_fp64(tg, oracle_lib, shear):
    """The benchmark's accuracy bar at 512^3: K CFL steps of the shear layer in
    the fast default (what bench.py times), in the exact mode, and with the C
    oracle in float32 (the reference scheme) and float64 (the FP64 oracle),
    each with its own CFL dt sequence from the same initial state.  The fast
    density L1 and Linf errors against FP64 must be within 2x the float32
    scheme's; the exact mode must equal the float32 oracle bit for bit over
    all K steps; one fast step must agree with one oracle step to
    FAST_STEP_RTOL (rho and p relative to their maxima, velocities relative to
    the largest speed component)."""
    W, dx, dt = shear
    W0 = W.cpu().numpy()
    # one step
    one_fast = tg._evolve_state(W, dx, dt, GAMMA).cpu().numpy()
    one_ref = oracle_lib._evolve_state(W0, dx, np.float32(dt), GAMMA)
    # error scale per variable: rho and p their own maxima, the three velocity
    # components the largest speed component (vz is zero initially and only
    # rounding-sized after a step, so its own maximum is no scale for it)
    mx = np.abs(one_ref).reshape(5, -1).max(axis=1)
    scale = np.array([mx[0], mx[1:4].max(), mx[1:4].max(), mx[1:4].max(), mx[4]])
    errs = [float(np.abs(one_fast[v] - one_ref[v]).max() / scale[v]) for v in range(5)]
    step_err = max(errs)
    del one_fast, one_ref
    assert step_err < FAST_STEP_RTOL, errs
    # K steps
    fast = tg.run_steps(W, dx, GAMMA, K_ACCURACY).cpu().numpy()[0]
    exact = tg.run_steps(W, dx, GAMMA, K_ACCURACY, exact=True).cpu().numpy()
    ref32, _ = oracle_lib.run_steps(W0, dx, GAMMA, K_ACCURACY)
    assert np.array_equal(exact, ref32)
    del exact
    rho32 = ref32[0].copy()
    del ref32
    ref64, _ = oracle_lib.run_steps(W0.astype(np.float64), dx, GAMMA, K_ACCURACY)
    rho64 = ref64[0].copy()
    del ref64
    d_ref = np.abs(rho32.astype(np.float64) - rho64)
    d_fast = np.abs(fast.astype(np.float64) - rho64)
    e_ref_l1, e_ref_inf = float(d_ref.mean()), float(d_ref.max())
    e_fast_l1, e_fast_inf = float(d_fast.mean()), float(d_fast.max())
    print(f"512^3 shear layer, {K_ACCURACY} CFL steps, density error vs FP64: "
          f"reference-f32 L1 {e_ref_l1:.3e} Linf {e_ref_inf:.3e}; "
          f"fast L1 {e_fast_l1:.3e} Linf {e_fast_inf:.3e}; one fast step vs f32 oracle "
          f"{step_err:.2e} (rho, v, p relative to their maxima)")
    assert e_fast_l1 <= 2 * e_ref_l1 and e_fast_inf <= 2 * e_ref_inf
