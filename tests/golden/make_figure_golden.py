"""Regenerate tests/golden/reference_figures.npz from the reference's figures.

The reference's only reference-produced field data are its check images
``figures/check_N.png``: matplotlib ``imshow`` of the density and the
pressure on the plane z = N//2 after ``time_integration(setup_ics(N, N//16),
t_final=0.2, gamma=5/3, handle_boundaries=True)`` (scaling_jax.py:75-82,
86-93, 236).  Each panel maps the slice, normalised to its own [min, max],
through a 256-entry colormap and upsamples it to about 421 x 421 pixels.

This script decodes the PNGs (zlib and the five PNG row filters, written
here with the standard library and numpy) and stores, per grid size, the RGB
colour at the centre pixel of every cell of both panels: uint8 arrays
``colors_N`` of shape [2, N, N, 3] (panel 0 density, panel 1 pressure; image
rows are the slice's first axis x, columns its second axis y, as imshow
shows an array).  Sizes 32, 64 and 96 are kept: their cells span 13, 6.6 and
4.4 pixels, so the centre pixel carries the cell's own colour; at 128 and
above neighbouring cells bleed into the centre pixel.

Usage: python tests/golden/make_figure_golden.py <path of the reference checkout>
"""
import os
import struct
import sys
import zlib

import numpy as np

SIZES = (32, 64, 96)


def read_png(path):
    """8-bit RGB/RGBA, non-interlaced PNG -> uint8 array [h, w, channels]."""
    f = open(path, "rb").read()
    if f[:8] != b"\x89PNG\r\n\x1a\n":
        raise ValueError(f"{path}: not a PNG")
    i, idat, w, h, bpp = 8, b"", None, None, None
    while i < len(f):
        ln = struct.unpack(">I", f[i:i + 4])[0]
        typ, data = f[i + 4:i + 8], f[i + 8:i + 8 + ln]
        if typ == b"IHDR":
            w, h, depth, ctype, _, _, interlace = struct.unpack(">IIBBBBB", data)
            if depth != 8 or ctype not in (2, 6) or interlace:
                raise ValueError(f"{path}: unsupported PNG format")
            bpp = 4 if ctype == 6 else 3
        elif typ == b"IDAT":
            idat += data
        i += 12 + ln
    raw = np.frombuffer(zlib.decompress(idat), np.uint8)
    stride = w * bpp
    out = np.zeros((h, stride), np.int32)
    prev = np.zeros(stride, np.int32)
    for r in range(h):
        base = r * (stride + 1)
        ftype = raw[base]
        line = raw[base + 1:base + 1 + stride].astype(np.int32)
        if ftype == 0:
            cur = line.copy()
        elif ftype == 2:
            cur = (line + prev) & 255
        else:
            cur = np.zeros(stride, np.int32)
            for x in range(stride):
                a = cur[x - bpp] if x >= bpp else 0
                b = prev[x]
                c = prev[x - bpp] if x >= bpp else 0
                if ftype == 1:
                    p = a
                elif ftype == 3:
                    p = (a + b) >> 1
                else:  # Paeth
                    pa, pb, pc = abs(b - c), abs(a - c), abs(a + b - 2 * c)
                    p = a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)
                cur[x] = (line[x] + p) & 255
        out[r] = cur
        prev = cur
    return out.reshape(h, w, bpp).astype(np.uint8)


def cell_colors(img, n):
    """Centre-pixel colour of every cell of the two panels: [2, n, n, 3]."""
    rgb = img[..., :3].astype(int)
    colored = (rgb.max(-1) - rgb.min(-1)) > 30  # colormap pixels; frames and text are grey
    half = img.shape[1] // 2
    panels = []
    for a, b in ((0, half), (half, img.shape[1])):
        ys, xs = np.nonzero(colored[:, a:b])
        y0, y1, x0, x1 = ys.min(), ys.max() + 1, xs.min() + a, xs.max() + 1 + a
        cy = (y0 + (np.arange(n) + 0.5) * (y1 - y0) / n).astype(int)
        cx = (x0 + (np.arange(n) + 0.5) * (x1 - x0) / n).astype(int)
        panels.append(rgb[cy][:, cx])
    return np.array(panels, dtype=np.uint8)


def main(ref_root):
    arrays = {}
    for n in SIZES:
        img = read_png(os.path.join(ref_root, "figures", f"check_{n}.png"))
        arrays[f"colors_{n}"] = cell_colors(img, n)
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_figures.npz")
    np.savez_compressed(path, sizes=np.array(SIZES), **arrays)
    print(path, {k: v.shape for k, v in arrays.items()})


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_figure_golden.py <path of the reference checkout>")
    main(sys.argv[1])
