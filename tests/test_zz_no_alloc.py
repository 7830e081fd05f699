"""The allocation-free run entry point, called through the C ABI.

tf_time_integration_noalloc serves callers that cannot allocate device memory
when they step a simulation (their host runtime owns the device heap, or they
run where the allocator must not be entered): its work state and control block
live in a fixed scratch array inside the library.  Its results must equal
those of the allocating entry point, tf_time_integration, on consecutive calls
(the scratch keeps the previous call's contents, so the second call checks
that nothing stale leaks through).  This file is collected last on purpose.
"""
import ctypes
import math

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
GAMMA = 5.0 / 3.0
RTOL = 2e-6  # the fast-step tolerance of tests/test_gpu_parity.py
OPEN, EXACT = 1, 2  # TF_FLAG_OPEN_BOUNDARIES, TF_FLAG_EXACT


def random_state(shape, seed):
    rng = np.random.default_rng(seed)
    W = np.empty((5,) + tuple(shape), np.float32)
    W[0] = rng.uniform(0.5, 2.0, shape)
    W[1:4] = rng.uniform(-1.0, 1.0, (3,) + tuple(shape))
    W[4] = rng.uniform(0.2, 3.0, shape)
    return torch.from_numpy(W).cuda()


def close(a, b):
    scale = b.abs().reshape(5, -1).amax(dim=1).reshape(5, 1, 1, 1) + 1e-30
    return float(((a - b).abs() / scale).max()) <= RTOL


def call_noalloc(lib, W, out, dx, t_final, max_steps, flags=0, want_iters=True,
                 shape=None):
    _, nx, ny, nz = W.shape if shape is None else (5,) + tuple(shape)
    it = ctypes.c_int(-1)
    st = lib.tf_time_integration_noalloc(
        W.data_ptr(), out.data_ptr(), nx, ny, nz, dx, t_final, GAMMA, 0.4, max_steps, 0.0,
        flags, ctypes.byref(it) if want_iters else None,
        torch.cuda.current_stream().cuda_stream)
    return st, it.value


def reference_run(tg, W, dx, t_final, steps, flags):
    hb, ex = bool(flags & OPEN), bool(flags & EXACT)
    if steps >= 0:
        return tg.run_steps(W, dx, GAMMA, steps, hb, exact=ex), steps
    ref, rit = tg.time_integration_fn(W, dx, t_final, GAMMA, hb, False, exact=ex)
    return ref, int(rit)


def test_noalloc_matches_allocating_entry_point_on_consecutive_calls(tg):
    lib = tg._lib.load()
    cases = [((24, 20, 28), 7, 0.05, math.inf, 1, 0),
             ((40, 32, 16), 4, 0.04, math.inf, 2, 0),
             ((30, 30, 30), -1, 0.05, 0.03, 3, 0),
             ((20, 18, 22), 5, 0.05, math.inf, 4, EXACT),
             ((26, 24, 20), 6, 0.05, math.inf, 5, OPEN),
             ((22, 22, 22), -1, 0.05, 0.02, 6, EXACT | OPEN)]
    for shape, steps, dx, t_final, seed, flags in cases:
        W = random_state(shape, seed)
        out = torch.empty_like(W)
        st, it = call_noalloc(lib, W, out, dx, t_final, steps, flags)
        assert st == 0, lib.tf_last_error()
        ref, rit = reference_run(tg, W, dx, t_final, steps, flags)
        assert it == rit
        assert close(out, ref)
        assert torch.equal(out, ref)  # same kernels, same op order: identical bits


def test_noalloc_t_final_without_iteration_readback(tg):
    """iters_host = NULL, the form an allocation-free caller that does not want
    to read anything back uses: the result after a stream sync equals
    time_integration's, also on a second call with another grid."""
    lib = tg._lib.load()
    for shape, seed, flags in (((28, 20, 24), 7, 0), ((18, 26, 20), 8, OPEN)):
        W = random_state(shape, seed)
        out = torch.empty_like(W)
        st, _ = call_noalloc(lib, W, out, 0.05, 0.025, -1, flags, want_iters=False)
        assert st == 0, lib.tf_last_error()
        torch.cuda.synchronize()
        ref, _ = reference_run(tg, W, 0.05, 0.025, -1, flags)
        assert torch.equal(out, ref)


def test_noalloc_reports_device_errors(tg):
    """A negative pressure gives a NaN sound speed: TF_ERR_NONFINITE from the
    t_final loop even with iters_host = NULL, and from a known step count when
    iters_host is given."""
    lib = tg._lib.load()
    W = random_state((10, 10, 10), 9)
    W[4, 4, 4, 4] = -1.0
    out = torch.empty_like(W)
    st, _ = call_noalloc(lib, W, out, 0.1, 0.5, -1, want_iters=False)
    assert st == 3, lib.tf_last_error()
    st, _ = call_noalloc(lib, W, out, 0.1, math.inf, 3, want_iters=True)
    assert st == 3, lib.tf_last_error()
    # the scratch is usable again after an error
    W2 = random_state((10, 10, 10), 10)
    st, it = call_noalloc(lib, W2, out, 0.1, math.inf, 3)
    assert st == 0 and it == 3
    assert torch.equal(out, tg.run_steps(W2, 0.1, GAMMA, 3))


def test_noalloc_rejects_overlapping_states(tg):
    """Overlapping input and output ranges are rejected before any launch."""
    lib = tg._lib.load()
    shape = (8, 8, 8)
    n5 = 5 * 8 * 8 * 8
    buf = torch.ones(2 * n5, device="cuda")
    W = buf[:n5]
    out = buf[n5 // 2:n5 // 2 + n5]  # starts inside W
    st, _ = call_noalloc(lib, W, out, 0.1, math.inf, 1, shape=shape)
    assert st == 1 and b"overlap" in lib.tf_last_error()


def test_noalloc_rejects_grids_beyond_its_scratch(tg):
    lib = tg._lib.load()
    n_max = 1 << 18
    W = torch.ones((5, 65, 64, 64), device="cuda")  # 266,240 cells > 262,144
    assert W[0].numel() > n_max
    out = torch.empty_like(W)
    st, _ = call_noalloc(lib, W, out, 0.1, math.inf, 2)
    assert st == 1
    assert b"scratch" in lib.tf_last_error()
