"""Drop-in for ``tinyfluids.jax_tinyfluids.time_integration`` on a GB300.

``time_integration`` keeps the reference's signature and loop semantics
(time_integration.py:35-128): ``while t < t_final: dt = CFL dt(W);
W = evolve(W, dt); t += dt; num_iterations += 1``, with ``t`` accumulated in
float32 and the last step not clamped.  The loop runs on the device: each
step is one fused kernel that also produces the next dt and the loop
condition, and the loop itself is a CUDA graph with a device-side while node
(the counterpart of the reference's ``lax.while_loop``), so the host waits
only for the result.  ``host_loop=True`` selects the older form that tests
the condition on the host once per chunk of predicated steps.
"""
from __future__ import annotations

import math

import torch

from . import _lib
from .fluid import (CTL_ITER, CTL_STATUS, CTL_T, _flags, _scalar, _stream, _tile_arg,
                    check_state, new_ctl)


def time_integration(primitive_state, grid_spacing, t_final, gamma, handle_boundaries,
                     shard_mapped, padding=None, split=None, *, C_CFL=0.4, exact=None,
                     tile=None, host_loop=False):
    """time_integration.py:94-128.  Returns ``(state, num_iterations)``;
    ``num_iterations`` is a 0-d int32 CUDA tensor like the reference's traced
    counter.  ``shard_mapped=True`` (the multi-GPU shard_map branch) is out of
    scope and raises."""
    if shard_mapped or padding is not None or split is not None:
        raise NotImplementedError(
            "the shard_map branch (shard_mapped/padding/split) is not part of this "
            "single-GPU implementation")
    W, _, ctl = _run(primitive_state, grid_spacing, gamma, float(t_final), -1, 0.0,
                     handle_boundaries, C_CFL, exact, tile, wait=True, host_loop=host_loop)
    return W, ctl[CTL_ITER].clone()


def run_steps(primitive_state, grid_spacing, gamma, num_steps, handle_boundaries=False, *,
              C_CFL=0.4, dt=None, exact=None, tile=None, return_ctl=False):
    """``num_steps`` iterations of the same loop body (CFL dt, or a fixed ``dt``),
    fully asynchronous: nothing waits for the device.  Returns the state (and
    the control block tensor with t, dt, iter, status when ``return_ctl``)."""
    if int(num_steps) < 0:
        raise ValueError("num_steps must be >= 0")
    fixed = 0.0 if dt is None else float(dt)
    if dt is not None and not (fixed > 0 and math.isfinite(fixed)):
        raise ValueError("a fixed dt must be finite and > 0")
    W, _, ctl = _run(primitive_state, grid_spacing, gamma, math.inf, int(num_steps), fixed,
                     handle_boundaries, C_CFL, exact, tile, wait=False)
    return (W, ctl) if return_ctl else W


def step(primitive_state, grid_spacing, gamma, C_CFL=0.4, handle_boundaries=False, *,
         exact=None, tile=None, return_dt=False):
    """One loop iteration: dt = CFL dt of the state (fluid.py:427-504), then
    the split step (fluid.py:562-578); the same bits as ``run_steps(..., 1)``.
    With ``return_dt`` also returns the dt used (0-d float32 CUDA tensor)."""
    W, ctl = run_steps(primitive_state, grid_spacing, gamma, 1, handle_boundaries, C_CFL=C_CFL,
                       exact=exact, tile=tile, return_ctl=True)
    if not return_dt:
        return W
    # the loop's t after one step is the dt it took
    return W, ctl.view(torch.float32)[CTL_T].clone()


def _run(primitive_state, grid_spacing, gamma, t_final, max_steps, fixed_dt,
         handle_boundaries, C_CFL, exact, tile, wait, host_loop=False):
    W = check_state(primitive_state)
    _, nx, ny, nz = W.shape
    with torch.cuda.device(W.device):
        out = torch.empty_like(W)
        work = torch.empty_like(W)
        ctl = new_ctl(W.device)
        it = _lib.ctypes.c_int(0)
        _lib.call("tf_time_integration", W.data_ptr(), out.data_ptr(), work.data_ptr(),
                  ctl.data_ptr(), nx, ny, nz, float(grid_spacing), float(t_final),
                  _scalar(gamma, "gamma"), _scalar(C_CFL, "C_CFL"), int(max_steps),
                  float(fixed_dt),
                  _flags(handle_boundaries, exact) | (_lib.TF_FLAG_HOST_LOOP if host_loop else 0),
                  _tile_arg(tile, W, exact),
                  _lib.ctypes.byref(it) if wait else None, _stream(W))
    return out, (it.value if wait else None), ctl


def ctl_summary(ctl: torch.Tensor) -> dict:
    """Host copy of a control block: t, iter, status (synchronises)."""
    h = ctl.cpu()
    return {"t": float(h.view(torch.float32)[CTL_T]), "iter": int(h[CTL_ITER]),
            "status": int(h[CTL_STATUS])}
