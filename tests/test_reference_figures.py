"""Field values pinned to output of the reference itself: its check images.

The reference ships no field-value tests, but its figures/check_N.png are
its own final density and pressure slices (z = N//2) after
time_integration(setup_ics(N, N//16), t_final=0.2, gamma=5/3,
handle_boundaries=True) (scaling_jax.py:75-82, 86-93, 236), rendered through
a 256-entry colormap.  tests/figure_pin.py compares a slice with such an image
at the colormap's 8-bit resolution; tests/golden/reference_figures.npz holds
the images' per-cell colours (tests/golden/make_figure_golden.py).

The oracle (CPU, float32 reference scheme) is checked here; the CUDA path in
both arithmetic modes in the gpu-marked tests.  Bars: at 32^3 and 64^3 at
least 99% of the cells have exactly the colour their value implies and all
are within one colormap entry; at 96^3 (4.4 pixels per cell, so a centre
pixel can pick up its neighbours' colour at a sharp front) 99% are within
one entry; the bin colours rise in luminance (>= 95% of successive bins).
"""
import numpy as np
import pytest

import figure_pin

GAMMA = 5.0 / 3.0
BARS = {32: (0.99, 1.0), 64: (0.99, 1.0), 96: (0.0, 0.99)}


def check(n, W, colors):
    s = W[:, :, :, n // 2]
    for panel, var in ((0, 0), (1, 4)):
        exact, within1, rising = figure_pin.agreement(s[var], colors[panel])
        print(f"N={n} {'density' if var == 0 else 'pressure'}: exact {exact:.4f} "
              f"within one entry {within1:.4f} rising {rising:.3f}")
        assert exact >= BARS[n][0] and within1 >= BARS[n][1] and rising >= 0.95, (n, var)


@pytest.mark.parametrize("n", [32, 64])
def test_oracle_matches_reference_figures(oracle_lib, n):
    from oracle import ics_np
    W, dx = ics_np.setup_ics(n, n // 16)
    out, it = oracle_lib.time_integration(W, dx, 0.2, GAMMA, True)
    check(n, out, figure_pin.load()[n])


def test_figures_distinguish_the_boundary_setting(oracle_lib):
    """The pin is selective: the same run with periodic boundaries does not
    reproduce the 32^3 image (the figures come from the open-boundary run)."""
    from oracle import ics_np
    W, dx = ics_np.setup_ics(32, 2)
    out, _ = oracle_lib.time_integration(W, dx, 0.2, GAMMA, False)
    exact, within1, _ = figure_pin.agreement(out[0, :, :, 16], figure_pin.load()[32][0])
    assert within1 < 0.97


@pytest.mark.gpu
@pytest.mark.parametrize("n", [32, 64, 96])
@pytest.mark.parametrize("exact", [True, False])
def test_cuda_path_matches_reference_figures(tg, n, exact):
    W, dx = tg.setup_ics(n, n // 16)
    Wf, _ = tg.time_integration_fn(W, dx, 0.2, GAMMA, True, False, exact=exact)
    check(n, Wf.cpu().numpy(), figure_pin.load()[n])
