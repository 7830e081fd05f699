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


def call_noalloc(lib, W, out, dx, t_final, max_steps, flags=0):
    _, nx, ny, nz = W.shape
    it = ctypes.c_int(-1)
    st = lib.tf_time_integration_noalloc(
        W.data_ptr(), out.data_ptr(), nx, ny, nz, dx, t_final, GAMMA, 0.4, max_steps, 0.0,
        flags, ctypes.byref(it), torch.cuda.current_stream().cuda_stream)
    return st, it.value


def test_noalloc_matches_allocating_entry_point_on_consecutive_calls(tg):
    lib = tg._lib.load()
    cases = [((24, 20, 28), 7, 0.05, math.inf, 1), ((40, 32, 16), 4, 0.04, math.inf, 2),
             ((30, 30, 30), -1, 0.05, 0.03, 3)]
    for shape, steps, dx, t_final, seed in cases:
        W = random_state(shape, seed)
        out = torch.empty_like(W)
        st, it = call_noalloc(lib, W, out, dx, t_final, steps)
        assert st == 0, lib.tf_last_error()
        if steps >= 0:
            ref = tg.run_steps(W, dx, GAMMA, steps)
            assert it == steps
        else:
            ref, rit = tg.time_integration_fn(W, dx, t_final, GAMMA, False, False)
            assert it == int(rit)
        assert close(out, ref)
        assert torch.equal(out, ref)  # same kernels, same op order: identical bits


def test_noalloc_rejects_grids_beyond_its_scratch(tg):
    lib = tg._lib.load()
    n_max = 1 << 18
    W = torch.ones((5, 65, 64, 64), device="cuda")  # 266,240 cells > 262,144
    assert W[0].numel() > n_max
    out = torch.empty_like(W)
    st, _ = call_noalloc(lib, W, out, 0.1, math.inf, 2)
    assert st == 1
    assert b"scratch" in lib.tf_last_error()
