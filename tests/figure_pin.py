"""Field-level comparison with the reference's check images (test helper).

tests/golden/reference_figures.npz holds the centre-pixel colour of every
cell of the reference's figures/check_N.png (density and pressure on the
plane z = N//2 after time_integration(setup_ics(N, N//16), 0.2,
handle_boundaries=True); see tests/golden/make_figure_golden.py).  The image
maps each slice, normalised to its own [min, max], through a 256-entry
colormap: a cell of normalised value g gets colormap entry int(256 g)
(clipped to 255).

Without the colormap table itself, a field is pinned like this: bin every
cell of our slice by its normalised value; give each bin the colour most of
its cells have in the image; then every cell's image colour must be the
colour of its own bin (an exact pin at 8-bit colour resolution), or of an
adjacent bin (normalisation rounding).  A different field mixes colours
within bins and fails.  The bin colours must also run through the colormap
monotonically: their luminance increases with the bin for the reference's
default colormap, which orders the image's colours independently of our data.
"""
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                      "reference_figures.npz")


def load():
    d = np.load(GOLDEN)
    return {int(n): d[f"colors_{int(n)}"] for n in d["sizes"]}


def agreement(field, colors):
    """(fraction of cells in exactly their bin's colour, fraction within one
    bin, fraction of successive bin colours that rise in luminance)."""
    f = np.asarray(field, np.float64)
    g = (f - f.min()) / (f.max() - f.min())
    k = np.minimum((g * 256).astype(int), 255)
    c = (colors[..., 0].astype(int) << 16) | (colors[..., 1].astype(int) << 8) | colors[..., 2]
    table = {}
    for b in np.unique(k):
        vals, cnt = np.unique(c[k == b], return_counts=True)
        table[int(b)] = int(vals[cnt.argmax()])
    bins_of = {}
    for b, v in table.items():
        bins_of.setdefault(v, []).append(b)
    k_img = np.full(k.shape, -10 ** 6)
    for v, bs in bins_of.items():
        k_img[c == v] = int(round(np.mean(bs)))
    d = np.abs(k_img - k)
    order = sorted(table)
    lum = np.array([0.299 * (table[b] >> 16) + 0.587 * ((table[b] >> 8) & 255)
                    + 0.114 * (table[b] & 255) for b in order])
    rising = float(np.mean(np.diff(lum) > 0)) if len(lum) > 1 else 1.0
    return float((d == 0).mean()), float((d <= 1).mean()), rising
