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

import numpy as np
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


def time_integration_host(primitive_states, grid_spacing, t_final, gamma, handle_boundaries,
                          *, num_steps=None, C_CFL=0.4, dt=None, exact=None, tile=None,
                          out=None, device=None, workspace=None):
    """time_integration.py:94-128 for host-resident states: each CPU state of
    ``primitive_states`` (a list of [5, nx, ny, nz] float32 CPU tensors or
    numpy arrays of one shape, or one such state) is copied to the GPU, run with exactly
    ``time_integration``'s loop (to ``t_final``, or ``num_steps`` steps when
    given) and copied back.  The copies of one state overlap the runs of its
    neighbours, so for pinned host tensors a list of states runs at about the
    device's step rate.  Returns ``(states, num_iterations)``: lists of CPU
    tensors (pinned; ``out`` may name them, including the inputs themselves
    for an in-place update) and ints.  Blocks until the outputs are in host
    memory.  ``workspace``: a uint8 CUDA tensor of at least
    ``host_runs_workspace_bytes(shape, count)`` bytes to use instead of one
    allocated per call (repeated calls then allocate nothing on the device)."""
    single = isinstance(primitive_states, (torch.Tensor, np.ndarray))
    states = [primitive_states] if single else list(primitive_states)
    if not states:
        raise ValueError("no states given")
    # numpy arrays are viewed, not copied
    states = [torch.from_numpy(st) if isinstance(st, np.ndarray) else st for st in states]
    shape = None
    for i, st in enumerate(states):
        if not isinstance(st, torch.Tensor) or st.dtype != torch.float32:
            raise TypeError(f"state {i} must be a float32 torch.Tensor")
        if st.dim() != 4 or st.shape[0] != 5 or min(st.shape[1:]) < 1:
            raise TypeError(f"state {i} must have shape [5, nx, ny, nz], got {tuple(st.shape)}")
        if st.is_cuda:
            raise ValueError(f"state {i} is on the GPU: use time_integration for device states")
        if not st.is_contiguous():
            raise ValueError(f"state {i} must be contiguous")
        if shape is None:
            shape = tuple(st.shape)
        elif tuple(st.shape) != shape:
            raise ValueError(f"state {i} has shape {tuple(st.shape)}, state 0 {shape}")
    if num_steps is None:
        max_steps, tf = -1, float(t_final)
    else:
        if int(num_steps) < 0:
            raise ValueError("num_steps must be >= 0")
        max_steps = int(num_steps)
        tf = math.inf if t_final is None else float(t_final)
    fixed = 0.0 if dt is None else float(dt)
    if dt is not None and not (fixed > 0 and math.isfinite(fixed)):
        raise ValueError("a fixed dt must be finite and > 0")
    if out is None:
        outs = [torch.empty(shape, dtype=torch.float32, pin_memory=True) for _ in states]
    else:
        outs = [out] if isinstance(out, torch.Tensor) else list(out)
        if len(outs) != len(states):
            raise ValueError("out must hold one tensor per state")
        for i, o in enumerate(outs):
            if (not isinstance(o, torch.Tensor) or o.is_cuda or o.dtype != torch.float32
                    or tuple(o.shape) != shape or not o.is_contiguous()):
                raise ValueError(f"out[{i}] must be a contiguous float32 CPU tensor of shape "
                                 f"{shape}")
    dev = torch.device("cuda", torch.cuda.current_device()) if device is None else \
        torch.device(device)
    _, nx, ny, nz = shape
    n = len(states)
    with torch.cuda.device(dev):
        lib = _lib.load()
        nbytes = int(lib.tf_host_runs_workspace_bytes(nx, ny, nz, n))
        if nbytes == 0:
            raise ValueError(f"invalid grid {shape[1:]}")
        if workspace is None:
            ws = torch.empty(nbytes, dtype=torch.uint8, device=dev)
        else:
            ws = workspace
            if (not isinstance(ws, torch.Tensor) or not ws.is_cuda or ws.device != dev
                    or not ws.is_contiguous() or ws.numel() * ws.element_size() < nbytes):
                raise ValueError(f"workspace must be a contiguous CUDA tensor on {dev} of at "
                                 f"least {nbytes} bytes")
            nbytes = ws.numel() * ws.element_size()
        ins = (_lib.vp * n)(*[st.data_ptr() for st in states])
        ous = (_lib.vp * n)(*[o.data_ptr() for o in outs])
        its = (_lib.c_int * n)()
        _lib.call("tf_time_integration_host", ins, ous, n, nx, ny, nz, float(grid_spacing), tf,
                  _scalar(gamma, "gamma"), _scalar(C_CFL, "C_CFL"), max_steps, fixed,
                  _flags(handle_boundaries, exact), _tile_arg(tile, None, exact), ws.data_ptr(),
                  nbytes, its, torch.cuda.current_stream(dev).cuda_stream)
    iters = list(its)
    return (outs[0], iters[0]) if single else (outs, iters)


def host_runs_workspace_bytes(shape, count):
    """Device workspace bytes ``time_integration_host`` needs for ``count``
    states of ``shape`` ([5,] nx, ny, nz)."""
    nx, ny, nz = (int(v) for v in tuple(shape)[-3:])
    return int(_lib.load().tf_host_runs_workspace_bytes(nx, ny, nz, int(count)))


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
