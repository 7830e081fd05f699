"""Initial states on the device.

``setup_ics`` is the reference's injection cube (scaling_jax.py:23-41) with
its return convention ``(state, grid_spacing)``; ``overpressure`` and
``shear_layer`` are the benchmark states (unit periodic cube, dx = 1/n).
All three are filled by CUDA kernels directly in device memory.
"""
from __future__ import annotations

import torch

from . import _lib


def _device(device):
    d = torch.device(device if device is not None else "cuda")
    if d.type != "cuda":
        raise ValueError("initial states are built on a CUDA device")
    return d


def setup_ics(num_cells, num_injection_cells=2, device=None):
    """scaling_jax.py:23-41: ([5, n, n, n] float32, dx = 1/(n-1))."""
    n = int(num_cells)
    dev = _device(device)
    with torch.cuda.device(dev):
        W = torch.empty((5, n, n, n), dtype=torch.float32, device=dev)
        _lib.call("tf_ics_injection_cube", W.data_ptr(), n, int(num_injection_cells),
                  torch.cuda.current_stream(dev).cuda_stream)
    return W, 1 / (n - 1)


def overpressure(num_cells, seed=0, radius=0.1, p_in=10.0, p_out=0.1, rho0=1.0, noise=0.01,
                 device=None):
    """Spherical overpressure, rho noise +-noise; returns (state, dx = 1/n)."""
    n = int(num_cells)
    dev = _device(device)
    with torch.cuda.device(dev):
        W = torch.empty((5, n, n, n), dtype=torch.float32, device=dev)
        _lib.call("tf_ics_overpressure", W.data_ptr(), n, int(seed) & (2**64 - 1),
                  float(radius), float(p_in), float(p_out), float(rho0), float(noise),
                  torch.cuda.current_stream(dev).cuda_stream)
    return W, 1.0 / n


def shear_layer(num_cells, seed=0, amplitude=0.01, device=None):
    """Shear layer with vy = amplitude*sin(4 pi x)*N(0,1); returns (state, dx = 1/n)."""
    n = int(num_cells)
    dev = _device(device)
    with torch.cuda.device(dev):
        W = torch.empty((5, n, n, n), dtype=torch.float32, device=dev)
        _lib.call("tf_ics_shear_layer", W.data_ptr(), n, int(seed) & (2**64 - 1),
                  float(amplitude), torch.cuda.current_stream(dev).cuda_stream)
    return W, 1.0 / n
