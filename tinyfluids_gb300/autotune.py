"""Tile-shape autotuner for the fused step kernel.

The fused kernel has two tile layouts and, for each, two free parameters
(``tf_tile_config``).  The x-marching tile ("ldg"): the tile height ``rows``
(8, 16 or 32 grid rows incl. the one-cell ring; the kernel runs rows/2 warps)
and ``lx``, the number of x planes one CTA marches through.  The y-marching
tile ("ym"): rows/2 x rows per CTA (8 or 16 rows) and ``lx`` y planes per CTA.
Taller tiles waste fewer halo rows; shorter ones let more CTAs share an SM and
interleave their barrier phases; ``lx`` trades per-chunk warm-up work against
the number of CTAs.  The best choice depends on the grid size and is
measured, not modelled: ``tune`` times every candidate with CUDA events on the
device and keeps the fastest.  Results are cached per (GPU, grid shape,
arithmetic) in memory and in a JSON file (``$TINYFLUIDS_GB300_TUNE_CACHE`` or
``~/.cache/tinyfluids_gb300/tiles.json``).

Batches (``tune_batch``) are tuned on the batch itself: every (rows, lx
policy) candidate runs a few steps of the actual batch and the fastest wins,
because inside a full batch the best tile differs from the best tile for a
grid running alone; then the chunk length is refined per size class (the
instances of one grid size) on the batch.  The tile height stays one per
launch: in a mixed batch the largest classes carry most of the cell-updates
(88% for 96^3 and 128^3 in the batching workload of 32-128 cells per axis), so
the height they prefer is the batch's.
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
    # v2: the y-marching tile is among the candidates
    return f"v2|{name}|{shape[0]}x{shape[1]}x{shape[2]}|{'exact' if exact else 'fast'}"


def candidates(shape):
    """(rows, lx, layout) triples worth timing for a grid shape: layout "ldg"
    is the x-marching tile (lx = x planes per CTA), "ym" the y-marching tile
    (lx = y planes per CTA, 8 or 16 rows); lx 0 is the built-in chunk-length
    heuristic."""
    nx, ny = shape[0], shape[1]
    lxs = sorted({lx for lx in (2, 4, 8, 16, 32, 64, 96, 128, 192, 256, 512) if lx < nx}
                 | {nx, 0})
    lys = sorted({ly for ly in (8, 16, 32, 64, 128) if ly < ny} | {0})
    return ([(r, lx, "ldg") for r in ROWS for lx in lxs] +
            [(r, ly, "ym") for r in (8, 16) for ly in lys])


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
    for rows, lx, layout in candidates(shape):
        table[f"{rows},{lx},{layout}"] = _time_config(W, dx, (rows, lx, layout), exact, reps,
                                                      steps)
    best = min(table, key=table.get)
    rows, lx, layout = best.split(",")
    res = {"rows": int(rows), "lx": int(lx), "layout": layout, "ms": table[best],
           "table": table}
    with _LOCK:
        _MEM[key] = res
        if persist:
            disk = _load_file()
            disk[key] = res
            _save_file(disk)
    return res


def tuned_tile(shape, exact=False, device=None):
    """(rows, lx, layout) from the cache (tuning on first use)."""
    r = tune(shape, exact=exact, device=device)
    return r["rows"], r["lx"], r.get("layout", "ldg")


def size_class(n: int) -> int:
    """Smallest class size >= n (the largest class for bigger grids)."""
    for c in SIZE_CLASSES:
        if n <= c:
            return c
    return SIZE_CLASSES[-1]


def _time_batch(specs, rows, lxs, exact, dev, steps):
    """Milliseconds of a short run (`steps` steps) of the batch on copies of
    its states with per-instance chunk lengths `lxs`."""
    from dataclasses import replace
    from .batching import Batch
    trial = [replace(sp, num_steps=steps, t_final=float("inf"), fixed_dt=None, lx=lx, out=None,
                     consume_input=False)
             for sp, lx in zip(specs, lxs)]
    b = Batch(trial, rows=rows, exact=exact, autotune=False)
    b.run()
    st = torch.cuda.current_stream(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    b.run()
    e1.record(st)
    e1.synchronize()
    ms = e0.elapsed_time(e1)
    b.close()
    return ms


def tune_batch(specs, exact=False, device=None, steps=2, candidates_rows=ROWS,
               lx_policies=(0, 64, 32, 16, 8), per_class=True):
    """Tile choice for a batch: one `rows` for the launch and an `lx` per
    instance.  Inside a batch the GPU is full, so single-grid timings are a
    poor proxy; the candidates are timed on the batch itself (short runs of
    `steps` steps on copies of its states).  First every (rows, lx policy)
    pair is timed with the policy applied to all instances (policy 0: the
    whole x extent per CTA, otherwise min(nx, policy)); then, per size class
    (instances of the same grid size), each lx policy is tried for that
    class alone with the other classes fixed, and kept if the batch gets
    faster.  Returns (rows, [lx per instance]); cached per list of shapes."""
    shapes = tuple(tuple(sp.state.shape[1:]) for sp in specs)
    dev = torch.device(device if device is not None else specs[0].state.device)
    key = ("batch", torch.cuda.get_device_name(dev), shapes, bool(exact), bool(per_class))
    with _LOCK:
        if key in _MEM:
            return _MEM[key]

    def lx_of(shape, pol):
        return shape[0] if pol == 0 else min(shape[0], pol)

    best = None
    for rows in candidates_rows:
        for pol in lx_policies:
            lxs = [lx_of(s, pol) for s in shapes]
            ms = _time_batch(specs, rows, lxs, exact, dev, steps)
            if best is None or ms < best[0]:
                best = (ms, rows, lxs)
    ms_best, rows, lxs = best
    if per_class:
        classes = sorted(set(shapes), key=lambda s: -s[0] * s[1] * s[2])
        for cls in classes:
            members = [i for i, s in enumerate(shapes) if s == cls]
            tried = {lxs[members[0]]}
            for pol in lx_policies:
                lx = lx_of(cls, pol)
                if lx in tried:
                    continue
                tried.add(lx)
                cand = list(lxs)
                for i in members:
                    cand[i] = lx
                ms = _time_batch(specs, rows, cand, exact, dev, steps)
                if ms < ms_best:
                    ms_best, lxs = ms, cand
    res = (rows, lxs)
    with _LOCK:
        _MEM[key] = res
    return res
