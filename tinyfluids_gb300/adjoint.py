"""Differentiation through a fixed-dt run with a hand-written adjoint.

``FixedDtRun`` is a ``torch.autograd.Function`` for ``U_N = S^N(U_0)``: N
steps of the split HLL scheme (fluid.py:562-578) with a fixed dt, acting on
CONSERVED states (rho, m, E) -- the reference's primitive round trips between
sweeps are the identity map, so this is the same function as the reference
step, differentiated directly in the variables the scheme updates.

Forward: one fused step per step on conserved states (float32; FP64 runs
three per-axis sweeps); every ``segment``-th state (segment =
ceil(sqrt(N))) is kept.
Backward: for each segment, last to first, the segment's states are
recomputed from its checkpoint, then each step is reversed with the adjoint
sweep kernels (``tf_adjoint_sweep``: z, then y, then x, each with the input
state of that forward sweep, recomputed from the step's input).  Peak memory
is about 2*sqrt(N) states instead of N.

float32 inputs use the fast arithmetic (the fused kernel's op sequence);
float64 inputs use an FP64 sweep of the same formulas, which the tests use
for central finite differences.
"""
from __future__ import annotations

import math

import torch

from . import _lib
from .fluid import _evolve_state, _evolve_state_along_axis, _stream, check_state


def _check(U):
    if not isinstance(U, torch.Tensor) or U.dim() != 4 or U.shape[0] != 5 or not U.is_cuda:
        raise TypeError("U must be a [5, nx, ny, nz] CUDA tensor")
    if U.dtype not in (torch.float32, torch.float64):
        raise TypeError("U must be float32 or float64")
    return U.contiguous()


def sweep_conserved(U, dx, dt, gamma, axis):
    """One forward sweep (axis 1, 2, 3) on a conserved state."""
    U = _check(U)
    if U.dtype == torch.float32:
        return _evolve_state_along_axis(U, dx, dt, gamma, axis, exact=False,
                                        conserved_in=True, conserved_out=True)
    _, nx, ny, nz = U.shape
    with torch.cuda.device(U.device):
        out = torch.empty_like(U)
        _lib.call("tf_sweep_conserved_f64", U.data_ptr(), out.data_ptr(), nx, ny, nz,
                  float(dx), float(dt), float(gamma), axis - 1, _stream(U))
    return out


def step_conserved(U, dx, dt, gamma):
    """One split step (x, y, z sweeps) on a conserved state: float32 in one
    fused kernel pass (equal bit for bit to the three sweeps), float64 as
    three FP64 sweeps."""
    U = _check(U)
    if U.dtype == torch.float32:
        return _evolve_state(U, dx, dt, gamma, exact=False, conserved=True)
    for axis in (1, 2, 3):
        U = sweep_conserved(U, dx, dt, gamma, axis)
    return U


def adjoint_sweep(U, lam_out, dx, dt, gamma, axis):
    """dL/dU of one sweep given its input U and dL/dU' (axis 1, 2, 3)."""
    U = _check(U)
    lam_out = lam_out.contiguous()
    if lam_out.shape != U.shape or lam_out.dtype != U.dtype:
        raise TypeError("lam_out must match U")
    _, nx, ny, nz = U.shape
    name = "tf_adjoint_sweep" if U.dtype == torch.float32 else "tf_adjoint_sweep_f64"
    with torch.cuda.device(U.device):
        out = torch.empty_like(U)
        _lib.call(name, U.data_ptr(), lam_out.data_ptr(), out.data_ptr(), nx, ny, nz,
                  float(dx), float(dt), float(gamma), axis - 1, _stream(U))
    return out


def adjoint_step(U, lam, dx, dt, gamma):
    """dL/dU_n of one step given U_n and dL/dU_{n+1}."""
    ux = sweep_conserved(U, dx, dt, gamma, 1)
    uxy = sweep_conserved(ux, dx, dt, gamma, 2)
    lam = adjoint_sweep(uxy, lam, dx, dt, gamma, 3)
    lam = adjoint_sweep(ux, lam, dx, dt, gamma, 2)
    return adjoint_sweep(U, lam, dx, dt, gamma, 1)


class FixedDtRun(torch.autograd.Function):
    """U_N = S^N(U_0) with a hand-written adjoint and sqrt(N) checkpoints."""

    @staticmethod
    def forward(ctx, U0, dx, dt, gamma, num_steps, segment=None):
        U0 = _check(U0)
        n = int(num_steps)
        seg = int(segment) if segment else max(1, math.ceil(math.sqrt(max(n, 1))))
        ckpts = [U0]
        U = U0
        for i in range(n):
            U = step_conserved(U, dx, dt, gamma)
            if (i + 1) % seg == 0 and i + 1 < n:
                ckpts.append(U)
        ctx.save_for_backward(*ckpts)
        ctx.args = (dx, dt, gamma, n, seg)
        return U.clone() if n == 0 else U

    @staticmethod
    def backward(ctx, lam):
        dx, dt, gamma, n, seg = ctx.args
        ckpts = ctx.saved_tensors
        lam = lam.contiguous()
        if n == 0:
            return lam, None, None, None, None, None
        for c in range(len(ckpts) - 1, -1, -1):
            start = c * seg
            stop = min(start + seg, n)
            states = [ckpts[c]]
            for _ in range(start, stop - 1):
                states.append(step_conserved(states[-1], dx, dt, gamma))
            for U in reversed(states):
                lam = adjoint_step(U, lam, dx, dt, gamma)
            del states
        return lam, None, None, None, None, None


def fixed_dt_run(U0, grid_spacing, dt, gamma, num_steps, segment=None):
    """Differentiable N-step run on a conserved state (see module doc)."""
    return FixedDtRun.apply(U0, grid_spacing, dt, gamma, num_steps, segment)


def density_mse_loss(U0, rho_target, grid_spacing, dt, gamma, num_steps, segment=None):
    """mean((rho_N - rho_target)^2), differentiable w.r.t. U0."""
    UN = fixed_dt_run(U0, grid_spacing, dt, gamma, num_steps, segment)
    return ((UN[0] - rho_target) ** 2).mean()
