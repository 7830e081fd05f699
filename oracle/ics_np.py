"""NumPy initial states for the oracle -- TEST INFRASTRUCTURE ONLY.

``setup_ics`` restates scaling_jax.py:23-41 (the reference's injection cube).
``overpressure`` and ``shear_layer`` are the two benchmark initial states
(spherical overpressure; shear layer with a seeded vy perturbation), built on
the host with numpy's seeded generator.  They follow the same formulas as the
device builders but not the same random draws; a test hands one array to both
the oracle and the GPU path.
"""
from __future__ import annotations

import numpy as np


def setup_ics(num_cells, num_injection_cells=2, dtype=np.float32):
    """scaling_jax.py:23-41.  rho=0.125, p=0.1 background; rho=p=1 in the centre cube."""
    n = int(num_cells)
    grid_spacing = 1 / (n - 1)
    rho = np.ones((n, n, n), dtype) * dtype(0.125)
    u = np.zeros((n, n, n), dtype)
    p = np.ones((n, n, n), dtype) * dtype(0.1)
    c = n // 2
    sl = slice(c - num_injection_cells, c + num_injection_cells)
    rho[sl, sl, sl] = 1.0
    p[sl, sl, sl] = 1.0
    return np.stack([rho, u, u.copy(), u.copy(), p], axis=0), grid_spacing


def cell_centres(n, dtype=np.float64):
    """(i + 0.5) / n for i in [0, n)."""
    return (np.arange(n, dtype=np.float64) + 0.5) / n


def overpressure(n, seed=0, radius=0.1, p_in=10.0, p_out=0.1, rho0=1.0,
                 noise=0.01, dtype=np.float32):
    """Spherical overpressure: p=p_in for r<radius around (0.5,0.5,0.5), rho noise +-noise."""
    x = cell_centres(n)
    X, Y, Z = np.meshgrid(x, x, x, indexing="ij")
    r2 = (X - 0.5) ** 2 + (Y - 0.5) ** 2 + (Z - 0.5) ** 2
    rng = np.random.default_rng(seed)
    rho = rho0 * (1.0 + rng.uniform(-noise, noise, size=(n, n, n)))
    p = np.where(r2 < radius * radius, p_in, p_out)
    W = np.zeros((5, n, n, n), dtype)
    W[0] = rho
    W[4] = p
    return W, 1.0 / n


def shear_layer(n, seed=0, amplitude=0.01, dtype=np.float32):
    """Shear layer: rho=2, vx=+0.5 for |y-0.5|<0.25; rho=1, vx=-0.5 elsewhere; p=2.5;
    vy = amplitude*sin(4*pi*x)*a with a ~ N(0,1) drawn per cell from ``seed``; vz=0."""
    x = cell_centres(n)
    X, Y, _ = np.meshgrid(x, x, x, indexing="ij")
    band = np.abs(Y - 0.5) < 0.25
    rng = np.random.default_rng(seed)
    a = rng.standard_normal(size=(n, n, n))
    W = np.zeros((5, n, n, n), dtype)
    W[0] = np.where(band, 2.0, 1.0)
    W[1] = np.where(band, 0.5, -0.5)
    W[2] = amplitude * np.sin(4.0 * np.pi * X) * a
    W[4] = 2.5
    return W, 1.0 / n
