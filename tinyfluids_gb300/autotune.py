"""Tile-shape autotuner for the fused step kernel.

The fused kernel's tile has two free parameters (``tf_tile_config``): the tile
height ``rows`` (8, 16, 32 or 34 grid rows incl. the one-cell ring; the kernel
runs rows/2 warps) and ``lx``, the number of x planes one CTA marches through.
Taller tiles waste fewer halo rows; shorter ones let two or more CTAs share an
SM and interleave their barrier phases; ``lx`` trades per-chunk warm-up work
against the number of CTAs.  The best pair depends on the grid size and is
measured, not modelled: ``tune`` times every candidate with CUDA events on the
device and keeps the fastest.  Results are cached per (GPU, grid shape,
arithmetic) in memory and in a JSON file (``$TINYFLUIDS_GB300_TUNE_CACHE`` or
``~/.cache/tinyfluids_gb300/tiles.json``).

Batches use ``size_class``: instances are grouped by their largest axis into
classes, each class is tuned once on a representative cube, and every instance
of the class uses that class's ``lx`` under the batch's common ``rows``.
"""
from __future__ import annotations

import json
import os
import threading

import torch

from . import fluid as _fluid

ROWS = (8, 16, 32)
SIZE_CLASSES = (16, 24, 32, 48, 64, 96, 128, 192, 256, 384, 512, 768, 1024)

_LOCK = threading.Lock()
_MEM: dict = {}


def cache_path() -> str:
    p = os.environ.get("TINYFLUIDS_GB300_TUNE_CACHE")
    if p:
        return p
    return os.path.join(os.path.expanduser("~"), ".cache", "tinyfluids_gb300", "tiles.json")


def _load_file():
    try:
        with open(cache_path()) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _save_file(data):
    path = cache_path()
    try:
        os.makedirs(os.path.dirname(path), exist_ok=True)
        tmp = path + f".tmp{os.getpid()}"
        with open(tmp, "w") as f:
            json.dump(data, f, indent=1, sort_keys=True)
        os.replace(tmp, path)
    except OSError:
        pass  # a read-only home is fine: the in-memory cache still works


def _key(device, shape, exact):
    name = torch.cuda.get_device_name(device).replace(" ", "_")
    return f"{name}|{shape[0]}x{shape[1]}x{shape[2]}|{'exact' if exact else 'fast'}"


def candidates(shape):
    """(rows, lx) pairs worth timing for a grid shape."""
    nx = shape[0]
    lxs = sorted({lx for lx in (16, 32, 64, 96, 128, 192, 256, 512) if lx < nx} | {nx})
    return [(r, lx) for r in ROWS for lx in lxs]


def _time_config(W, dx, tile, exact, reps, steps):
    stream = torch.cuda.current_stream(W.device)
    best = float("inf")
    out = _fluid._evolve_state(W, dx, 1e-4, 5.0 / 3.0, exact=exact, tile=tile)  # warm-up
    for _ in range(reps):
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(steps):
            out = _fluid._evolve_state(W, dx, 1e-4, 5.0 / 3.0, exact=exact, tile=tile)
        b.record(stream)
        b.synchronize()
        best = min(best, a.elapsed_time(b) / steps)
    del out
    return best


def tune(shape, exact=False, device=None, reps=3, steps=3, force=False, persist=True):
    """Time every candidate tile on a synthetic state of `shape` and return
    {"rows": r, "lx": lx, "ms": t, "table": {...}} for the fastest."""
    shape = tuple(int(s) for s in shape)
    dev = torch.device(device if device is not None else "cuda")
    key = _key(dev, shape, exact)
    with _LOCK:
        if not force:
            if key in _MEM:
                return _MEM[key]
            disk = _load_file()
            if key in disk:
                _MEM[key] = disk[key]
                return disk[key]
    from .initial_conditions import shear_layer
    n = max(shape)
    W_full, dx = shear_layer(n, seed=0, device=dev)
    W = W_full[:, :shape[0], :shape[1], :shape[2]].contiguous()
    del W_full
    table = {}
    for rows, lx in candidates(shape):
        table[f"{rows},{lx}"] = _time_config(W, dx, (rows, lx), exact, reps, steps)
    best = min(table, key=table.get)
    rows, lx = (int(v) for v in best.split(","))
    res = {"rows": rows, "lx": lx, "ms": table[best], "table": table}
    with _LOCK:
        _MEM[key] = res
        if persist:
            disk = _load_file()
            disk[key] = res
            _save_file(disk)
    return res


def tuned_tile(shape, exact=False, device=None):
    """(rows, lx) from the cache (tuning on first use)."""
    r = tune(shape, exact=exact, device=device)
    return r["rows"], r["lx"]


def size_class(n: int) -> int:
    """Smallest class size >= n (the largest class for bigger grids)."""
    for c in SIZE_CLASSES:
        if n <= c:
            return c
    return SIZE_CLASSES[-1]


def tune_batch(shapes, exact=False, device=None):
    """Tile choice for a batch: one `rows` for the launch and an `lx` per
    instance.  Each size class is tuned once on its representative cube; the
    batch takes the rows that minimise the cell-weighted sum of per-class
    times, and each class its best lx under those rows."""
    classes = {}
    for s in shapes:
        c = size_class(max(s))
        classes.setdefault(c, 0)
        classes[c] += s[0] * s[1] * s[2]
    results = {c: tune((c, c, c), exact=exact, device=device) for c in classes}
    best_rows, best_cost = None, float("inf")
    for rows in ROWS:
        cost = 0.0
        for c, cells in classes.items():
            ts = [t for k, t in results[c]["table"].items() if int(k.split(",")[0]) == rows]
            cost += cells / c ** 3 * min(ts)
        if cost < best_cost:
            best_rows, best_cost = rows, cost
    lx_by_class = {}
    for c in classes:
        items = [(t, int(k.split(",")[1])) for k, t in results[c]["table"].items()
                 if int(k.split(",")[0]) == best_rows]
        lx_by_class[c] = min(items)[1]
    lxs = [min(lx_by_class[size_class(max(s))], s[0]) for s in shapes]
    return best_rows, lxs
