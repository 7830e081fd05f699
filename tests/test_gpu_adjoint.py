"""The hand-written adjoint of the fixed-dt step.

Checked against (1) torch.autograd of the FP64 restatement of the reference
step (oracle/torch_ref.py, the stand-in for JAX's gradient), (2) central
finite differences of the FP64 forward run, and (3) itself across checkpoint
segment lengths; the float32 adjoint is checked against the float64 one."""
import numpy as np
import pytest
import torch

from oracle import torch_ref
from tinyfluids_gb300 import adjoint as A

pytestmark = pytest.mark.gpu
GAMMA = 5.0 / 3.0


def shear_conserved(tg, n, seed, dtype=torch.float64):
    W, dx = tg.shear_layer(n, seed=seed, amplitude=0.05)
    U = tg.conserved_state_from_primitive(W, GAMMA)
    return U.to(dtype), dx


def target_from(U, seed):
    g = torch.Generator(device="cpu").manual_seed(seed)
    noise = (torch.rand(U.shape[1:], generator=g, dtype=torch.float64) * 2 - 1).to(U.device)
    return (U[0] * (1 + 0.05 * noise)).to(U.dtype)


def grad_of(loss_fn, U0):
    U = U0.clone().requires_grad_(True)
    loss = loss_fn(U)
    loss.backward()
    return U.grad, float(loss.detach())


def test_adjoint_matches_autograd_of_reference_restatement(tg):
    U0, _ = shear_conserved(tg, 12, 1)
    U0 = U0[:, :12, :10, :8].contiguous()
    rho_t = target_from(U0, 2)
    dx, dt, steps = 1 / 12, 2e-3, 3
    g_ours, l_ours = grad_of(lambda U: A.density_mse_loss(U, rho_t, dx, dt, GAMMA, steps), U0)
    g_ref, l_ref = grad_of(lambda U: torch_ref.density_mse_loss(U.cpu(), rho_t.cpu(), dx, dt,
                                                                GAMMA, steps), U0)
    assert abs(l_ours - l_ref) <= 1e-12 * abs(l_ref)
    err = float((g_ours.cpu() - g_ref.cpu()).abs().max() / g_ref.abs().max())
    assert err < 1e-9, err


def _fd_check(tg, U0, rho_t, dx, dt, steps, cells, rtol, seed, rel_h=1e-6):
    g, _ = grad_of(lambda U: A.density_mse_loss(U, rho_t, dx, dt, GAMMA, steps), U0)
    gmax = float(g.abs().max())
    rng = np.random.default_rng(seed)
    worst = 0.0
    with torch.no_grad():
        for _ in range(cells):
            f = int(rng.integers(5))
            i, j, k = (int(v) for v in (rng.integers(s) for s in U0.shape[1:]))
            h = rel_h * max(1.0, abs(float(U0[f, i, j, k])))
            Up, Um = U0.clone(), U0.clone()
            Up[f, i, j, k] += h
            Um[f, i, j, k] -= h
            fd = (float(A.density_mse_loss(Up, rho_t, dx, dt, GAMMA, steps))
                  - float(A.density_mse_loss(Um, rho_t, dx, dt, GAMMA, steps))) / (2 * h)
            worst = max(worst, abs(fd - float(g[f, i, j, k])) / gmax)
    assert worst < rtol, worst
    return worst


def test_adjoint_matches_central_differences_smooth_state(tg):
    """A noisy overpressure state has no tied wave speeds, so the loss is smooth
    around it and central differences match the adjoint tightly."""
    W, dx = tg.overpressure(16, seed=3, noise=0.05)
    W[1] += 0.1 * torch.rand_like(W[1])  # break the remaining symmetries
    U0 = tg.conserved_state_from_primitive(W, GAMMA).double()
    _fd_check(tg, U0, target_from(U0, 4), dx, 2e-3, 6, 16, 1e-5, 5, rel_h=1e-7)


def test_adjoint_matches_central_differences_shear_layer(tg):
    """The shear layer (the differentiation benchmark's state) has exactly tied
    wave speeds in its uniform bands: the loss has kinks there, the adjoint
    splits the gradient evenly at ties (like JAX and PyTorch), and a central
    difference straddling a near-tie mixes the two slopes.  The bound is
    therefore looser (relative to the largest gradient entry)."""
    U0, dx = shear_conserved(tg, 16, 3)
    _fd_check(tg, U0, target_from(U0, 4), dx, 2e-3, 6, 16, 1e-3, 5)


def test_checkpoint_segments_give_identical_gradients(tg):
    U0, dx = shear_conserved(tg, 20, 6, torch.float32)
    rho_t = target_from(U0, 7)
    grads = [grad_of(lambda U: A.density_mse_loss(U, rho_t, dx, 1e-3, GAMMA, 7, seg), U0)[0]
             for seg in (1, 3, None, 7)]
    for g in grads[1:]:
        assert torch.equal(g, grads[0])


def test_float32_adjoint_close_to_float64(tg):
    U64, dx = shear_conserved(tg, 24, 8)
    rho_t = target_from(U64, 9)
    g64, _ = grad_of(lambda U: A.density_mse_loss(U, rho_t, dx, 2e-3, GAMMA, 10), U64)
    g32, _ = grad_of(lambda U: A.density_mse_loss(U, rho_t.float(), dx, 2e-3, GAMMA, 10),
                     U64.float())
    err = float((g32.double() - g64).abs().max() / g64.abs().max())
    assert err < 1e-3, err


def test_zero_steps_is_identity(tg):
    U0, dx = shear_conserved(tg, 8, 1, torch.float32)
    g, _ = grad_of(lambda U: A.fixed_dt_run(U, dx, 1e-3, GAMMA, 0).sum(), U0)
    assert torch.equal(g, torch.ones_like(U0))


@pytest.mark.parametrize("shape", [(13, 9, 33), (40, 7, 5), (6, 50, 17)])
@pytest.mark.parametrize("axis", [0, 1])
def test_marching_adjoint_equals_per_cell_adjoint(tg, shape, axis):
    """The marching x / y adjoint kernels (each cell's forward side and each
    face's VJP computed once, carried along the sweep axis in chunks) give
    the same bits as the per-cell kernel that recomputes both faces, on odd
    sizes where the sweep axis splits into several chunks."""
    lib = tg._lib.load()
    W, _ = tg.shear_layer(max(shape), seed=3, amplitude=0.05)
    U = tg.conserved_state_from_primitive(
        W[:, :shape[0], :shape[1], :shape[2]].contiguous(), GAMMA)
    g = torch.Generator(device="cpu").manual_seed(7)
    lam = torch.randn(U.shape, generator=g, dtype=torch.float32).cuda()
    a = torch.empty_like(U)
    b = torch.empty_like(U)
    nx, ny, nz = shape
    s = torch.cuda.current_stream().cuda_stream
    dx, dt = 1.0 / 64, 2e-4
    assert lib.tf_adjoint_sweep(U.data_ptr(), lam.data_ptr(), a.data_ptr(), nx, ny, nz, dx, dt,
                                GAMMA, axis, s) == 0
    assert lib.tf_debug_adjoint_sweep_per_cell(U.data_ptr(), lam.data_ptr(), b.data_ptr(), nx,
                                               ny, nz, dx, dt, GAMMA, axis, s) == 0
    assert torch.equal(a, b)
