"""Many independent simulations advanced together on one GPU.

``Batch`` wraps the C ABI's batch entry points (tf_batch_prepare /
tf_batch_run): every instance keeps its own grid size, CFL dt, step count or
end time and control block, and one persistent kernel launch (optionally
replayed from a CUDA graph) advances all of them through all their steps.
Each instance's result is bit-identical to running it alone with
``time_integration.run_steps`` / ``time_integration`` (same arithmetic, same
per-instance dt), which the tests check.
"""
from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass
from dataclasses import replace as _replace

import torch

from . import _lib
from .fluid import _flags, check_state, new_ctl
from .time_integration import ctl_summary


@dataclass
class InstanceSpec:
    """One member of a batch: the primitive state and its run parameters."""
    state: torch.Tensor
    grid_spacing: float
    gamma: float = 5.0 / 3.0
    num_steps: int | None = None    # bound on steps (None: t_final only)
    t_final: float = math.inf       # loop while t < t_final
    fixed_dt: float | None = None   # fixed dt instead of the CFL dt
    C_CFL: float = 0.4
    handle_boundaries: bool = False
    lx: int = 0                     # x planes per tile (0: default)
    out: torch.Tensor | None = None   # preallocated result buffer (else allocated)
    consume_input: bool = False     # use the input as scratch (it is overwritten)


class Batch:
    """A prepared batch; ``run()`` advances every instance and returns the
    final states (new tensors, inputs untouched)."""

    def __init__(self, specs, *, rows=16, exact=None, persistent=True, ctas_per_sm=0,
                 wait_limit=0, capture_graph=False, steps=None, autotune=False):
        self._closed = True
        if not specs:
            raise ValueError("a batch needs at least one instance")
        self.specs = list(specs)
        dev = check_state(self.specs[0].state).device
        self.device = dev
        ex = _flags(False, exact) & _lib.TF_FLAG_EXACT
        self.exact = bool(ex)
        caps = []
        for sp in self.specs:
            W = check_state(sp.state)
            if W.device != dev:
                raise ValueError("all instances must be on the same device")
            if sp.num_steps is None and not math.isfinite(sp.t_final):
                raise ValueError("each instance needs num_steps or a finite t_final")
            caps.append(sp.num_steps)
        if steps is None:
            if any(c is None for c in caps):
                raise ValueError("instances bounded only by t_final need `steps` "
                                 "(an upper bound on their step count)")
            steps = max(caps)
        self.steps = int(steps)
        if autotune:
            from . import autotune as _at
            rows, lxs = _at.tune_batch(self.specs, exact=self.exact, device=dev)
            self.specs = [sp if sp.lx else _replace(sp, lx=lx) for sp, lx in zip(self.specs, lxs)]
        self.rows = int(rows)
        with torch.cuda.device(dev):
            self.inputs = [check_state(sp.state) for sp in self.specs]
            self.outputs = [sp.out if sp.out is not None else torch.empty_like(W)
                            for sp, W in zip(self.specs, self.inputs)]
            for o, W in zip(self.outputs, self.inputs):
                if o.shape != W.shape or o.dtype != W.dtype or not o.is_contiguous():
                    raise ValueError("out must be a contiguous tensor like the state")
            self.works = [W if sp.consume_input else torch.empty_like(W)
                          for sp, W in zip(self.specs, self.inputs)]
            self.ctls = [new_ctl(dev) for _ in self.specs]
            n = len(self.specs)
            arr = (_lib.Instance * n)()
            for i, (sp, W) in enumerate(zip(self.specs, self.inputs)):
                _, nx, ny, nz = W.shape
                arr[i] = _lib.Instance(
                    W.data_ptr(), self.outputs[i].data_ptr(), self.works[i].data_ptr(),
                    self.ctls[i].data_ptr(), nx, ny, nz,
                    _lib.TF_FLAG_OPEN_BOUNDARIES if sp.handle_boundaries else 0,
                    float(sp.grid_spacing), float(sp.gamma), float(sp.C_CFL),
                    float(sp.t_final), 0.0 if sp.fixed_dt is None else float(sp.fixed_dt),
                    -1 if sp.num_steps is None else int(sp.num_steps), int(sp.lx), 0)
            self._arr = arr
            nbytes = _lib.load().tf_batch_workspace_bytes(n)
            self.workspace = torch.empty(nbytes, dtype=torch.uint8, device=dev)
            cfg = _lib.BatchConfig(int(rows), 1 if self.exact else 0, 1 if persistent else 0,
                                   int(ctas_per_sm), int(wait_limit))
            self._stream = torch.cuda.current_stream(dev)
            _lib.call("tf_batch_prepare", ctypes.cast(arr, ctypes.c_void_p), n,
                      ctypes.byref(cfg), self.workspace.data_ptr(), nbytes,
                      self._stream.cuda_stream)
            self._closed = False
        self.graph = None
        if capture_graph:
            self.capture()

    def _enqueue(self, step_base=0, steps=None):
        _lib.call("tf_batch_run", self.workspace.data_ptr(), int(step_base),
                  self.steps if steps is None else int(steps),
                  torch.cuda.current_stream(self.device).cuda_stream)

    def capture(self):
        """Record the whole run (init, first dt, the persistent step kernel,
        result copies) as one CUDA graph for cheap replays."""
        with torch.cuda.device(self.device):
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g):
                self._enqueue()
            self.graph = g
        return g

    def run(self):
        """Advance every instance; asynchronous on the current stream."""
        with torch.cuda.device(self.device):
            if self.graph is not None:
                self.graph.replay()
            else:
                self._enqueue()
        return self.outputs

    def continue_run(self, step_base, steps):
        """Further step slots for instances still running (t_final loops)."""
        with torch.cuda.device(self.device):
            self._enqueue(step_base, steps)
        return self.outputs

    def error(self) -> int:
        """Batch-level device status (synchronises)."""
        e = ctypes.c_int(0)
        _lib.call("tf_batch_error", self.workspace.data_ptr(), ctypes.byref(e),
                  torch.cuda.current_stream(self.device).cuda_stream)
        return e.value

    def summaries(self):
        """Per-instance t, iter, status (synchronises)."""
        return [ctl_summary(c) for c in self.ctls]

    def close(self):
        """Forget the C-side plan (once; the workspace stays allocated until the
        object dies, so its address cannot be reused before this)."""
        if not self._closed:
            self._closed = True
            _lib.load().tf_batch_release(ctypes.c_void_p(self.workspace.data_ptr()))

    def __del__(self):
        try:
            self.close()
        except Exception:  # interpreter shutdown
            pass


def run_batch(states, grid_spacings, gamma=5.0 / 3.0, num_steps=100, **kw):
    """Convenience: advance each state ``num_steps`` CFL steps in one batch."""
    specs = [InstanceSpec(W, dx, gamma, num_steps=num_steps) for W, dx in
             zip(states, grid_spacings)]
    b = Batch(specs, **kw)
    out = b.run()
    return out, b
