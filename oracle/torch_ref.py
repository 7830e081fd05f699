"""PyTorch FP64 restatement of the reference step -- TEST INFRASTRUCTURE ONLY.

The gradient oracle: the same op-for-op restatement of fluid.py as
oracle/fluid_np.py, written with torch ops so that ``torch.autograd`` gives
the derivative of the reference step.  It stands in for JAX's own gradient of
the reference (JAX is not installed here).  torch.maximum/minimum split the
gradient evenly at ties, as JAX's lax.max/min do.
"""
from __future__ import annotations

import torch


def conserved_state_from_primitive(W, gamma):
    """fluid.py:30-67."""
    rho, p = W[0], W[4]
    utotal = torch.sqrt(W[1] ** 2 + W[2] ** 2 + W[3] ** 2)
    E = p / (gamma - 1) + 0.5 * rho * utotal ** 2
    return torch.stack([rho, rho * W[1], rho * W[2], rho * W[3], E])


def primitive_state_from_conserved(U, gamma):
    """fluid.py:71-103."""
    rho, E = U[0], U[4]
    ux, uy, uz = U[1] / rho, U[2] / rho, U[3] / rho
    u = torch.sqrt(ux ** 2 + uy ** 2 + uz ** 2)
    p = (gamma - 1) * rho * (E / rho - 0.5 * u ** 2)
    return torch.stack([rho, ux, uy, uz, p])


def _euler_flux(W, gamma, d):
    """fluid.py:208-259."""
    rho, p = W[0], W[4]
    utotal = torch.sqrt(W[1] ** 2 + W[2] ** 2 + W[3] ** 2)
    E = p / (gamma - 1) + 0.5 * rho * utotal ** 2
    fv = [rho, W[1] * rho, W[2] * rho, W[3] * rho, p + E]
    fv = [W[d] * f for f in fv]
    fv[d] = fv[d] + p
    return torch.stack(fv)


def _hll_solver(L, R, gamma, d):
    """fluid.py:263-305."""
    FL, FR = _euler_flux(L, gamma, d), _euler_flux(R, gamma, d)
    cL = torch.sqrt(gamma * L[4] / L[0])
    cR = torch.sqrt(gamma * R[4] / R[0])
    zero = torch.zeros_like(cL)
    sp = torch.maximum(torch.maximum(L[d] + cL, R[d] + cR), zero)
    sm = torch.minimum(torch.minimum(L[d] - cL, R[d] - cR), zero)
    UL = conserved_state_from_primitive(L, gamma)
    UR = conserved_state_from_primitive(R, gamma)
    return (sp * FL - sm * FR + sm * sp * (UR - UL)) / (sp - sm)


def _evolve_state_along_axis(W, dx, dt, gamma, axis):
    """fluid.py:508-557."""
    U = conserved_state_from_primitive(W, gamma)
    F = _hll_solver(torch.roll(W, 1, axis), W, gamma, axis)
    U = U + 1 / dx * (F - torch.roll(F, -1, axis)) * dt
    return primitive_state_from_conserved(U, gamma)


def _evolve_state(W, dx, dt, gamma):
    """fluid.py:562-578 (periodic)."""
    for axis in (1, 2, 3):
        W = _evolve_state_along_axis(W, dx, dt, gamma, axis)
    return W


def density_mse_loss(U0, rho_target, dx, dt, gamma, num_steps):
    """mean((rho_N - rho_target)^2) of a fixed-dt run started from conserved U0."""
    W = primitive_state_from_conserved(U0, gamma)
    for _ in range(num_steps):
        W = _evolve_state(W, dx, dt, gamma)
    return ((W[0] - rho_target) ** 2).mean()
