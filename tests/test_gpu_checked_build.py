"""The checked build (TF_CHECKED=1) on the GPU: stands in for a sanitizer.

Every global load and store of the fused step is range-checked (an access
outside the state would be counted and skipped), and every stored cell
increments a per-cell write counter, so each case below shows that the step
touches no memory outside its buffers and writes every cell exactly once:
no two tiles overlap in what they store and none is missed, for ragged
shapes, both tile layouts (x- and y-marching), all tile heights, short and
long chunks, both boundary modes, both arithmetic policies, and the run loop.
"""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
GAMMA = 5.0 / 3.0

SHAPES = [(1, 1, 1), (2, 3, 5), (5, 7, 33), (33, 17, 61), (40, 31, 64), (3, 64, 29),
          (64, 15, 2), (31, 30, 32)]
# (rows, lx, loader): loader 1 = per-thread loads, 2 = TMA-staged planes
# (falls back to loads when nz % 4 != 0; the TMA path's stores are counted),
# 3 = the y-marching tile (lx = y planes per CTA)
TILES = [None, (8, 3, 1), (16, 1, 1), (16, 5, 1), (32, 2, 1), (32, 7, 1), (16, 5, 2), (32, 3, 2),
         (8, 0, 3), (8, 1, 3), (16, 2, 3)]


@pytest.fixture(scope="module")
def chk(tg):
    return tg._lib.load_checked()


def random_state(shape, seed):
    rng = np.random.default_rng(seed)
    W = np.empty((5,) + tuple(shape), np.float32)
    W[0] = rng.uniform(0.5, 2.0, shape)
    W[1:4] = rng.uniform(-1.0, 1.0, (3,) + tuple(shape))
    W[4] = rng.uniform(0.2, 3.0, shape)
    return torch.from_numpy(W).cuda()


def tile_ptr(tg, tile):
    if tile is None:
        return None, None
    tc = tg._lib.TileConfig(*tile)
    return ctypes.byref(tc), tc


def counts_after(tg, chk, W, fn):
    n = W[0].numel()
    counts = torch.zeros(n, dtype=torch.int32, device=W.device)
    assert chk.tf_debug_reset(ctypes.c_void_p(counts.data_ptr()), n) == 0
    fn()
    torch.cuda.synchronize()
    oob = chk.tf_debug_oob_count()
    assert chk.tf_debug_reset(None, 0) == 0  # no dangling counter pointer
    return counts, oob


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("hb", [False, True])
@pytest.mark.parametrize("exact", [False, True])
def test_step_in_bounds_and_each_cell_written_once(tg, chk, shape, hb, exact):
    if hb and min(shape) < 2:
        pytest.skip("open boundaries need two cells per axis")
    W = random_state(shape, 7)
    out = torch.empty_like(W)
    nx, ny, nz = shape
    flags = (1 if hb else 0) | (2 if exact else 0)
    ref = tg._evolve_state(W, 0.05, 2e-3, GAMMA, hb, exact=exact)
    for tile in TILES:
        tp, keep = tile_ptr(tg, tile)
        counts, oob = counts_after(tg, chk, W, lambda: chk.tf_evolve_state(
            ctypes.c_void_p(W.data_ptr()), ctypes.c_void_p(out.data_ptr()), nx, ny, nz, 0.05,
            2e-3, None, GAMMA, flags, tp, None))
        assert oob == 0, (shape, tile)
        assert int(counts.min()) == 1 and int(counts.max()) == 1, (shape, tile)
        assert torch.equal(out, ref), (shape, tile)  # the checks change no result


@pytest.mark.parametrize("steps", [1, 2, 5])
def test_run_loop_in_bounds(tg, chk, steps):
    W = random_state((33, 17, 61), 9)
    out, work = torch.empty_like(W), torch.empty_like(W)
    ctl = torch.zeros(16, dtype=torch.int32, device=W.device)
    counts, oob = counts_after(tg, chk, W, lambda: chk.tf_time_integration(
        ctypes.c_void_p(W.data_ptr()), ctypes.c_void_p(out.data_ptr()),
        ctypes.c_void_p(work.data_ptr()), ctypes.c_void_p(ctl.data_ptr()), 33, 17, 61, 0.05,
        float("inf"), GAMMA, 0.4, steps, 0.0, 0, None, None, None))
    assert oob == 0
    assert int(counts.min()) == steps and int(counts.max()) == steps
    assert torch.equal(out, tg.run_steps(W, 0.05, GAMMA, steps))
