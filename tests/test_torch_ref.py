"""The torch FP64 restatement (gradient oracle) equals the NumPy oracle (CPU)."""
import numpy as np
import torch

from oracle import fluid_np as F
from oracle import torch_ref as T


def test_torch_restatement_matches_numpy_oracle():
    rng = np.random.default_rng(0)
    shape = (6, 5, 7)
    W = np.empty((5,) + shape)
    W[0] = rng.uniform(0.5, 2.0, shape)
    W[1:4] = rng.uniform(-1, 1, (3,) + shape)
    W[4] = rng.uniform(0.2, 3.0, shape)
    a = F._evolve_state(W, 0.1, 0.01, 5 / 3)
    b = T._evolve_state(torch.from_numpy(W), 0.1, 0.01, 5 / 3).numpy()
    assert np.allclose(a, b, rtol=1e-13, atol=1e-14)
    U = F.conserved_state_from_primitive(W, 5 / 3)
    assert np.allclose(T.conserved_state_from_primitive(torch.from_numpy(W), 5 / 3).numpy(), U,
                       rtol=1e-14)


def test_torch_restatement_gradient_is_finite_on_moving_flow():
    W = torch.ones(5, 4, 4, 4, dtype=torch.float64)
    W[1] = 0.3
    U = T.conserved_state_from_primitive(W, 5 / 3).requires_grad_(True)
    loss = T.density_mse_loss(U, torch.zeros(4, 4, 4, dtype=torch.float64), 0.1, 0.01, 5 / 3, 2)
    loss.backward()
    assert torch.isfinite(U.grad).all()
