"""The C-ABI library: builds, loads, exports every declared symbol, and
rejects bad arguments on the host (CPU only: no compute calls)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADERS = [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))
           if f.endswith(".h")]


def declared_functions():
    names = set()
    for h in HEADERS:
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[a-z_ ]+\**\s*\**(tf_\w+)\s*\(", src, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


@pytest.fixture(scope="module")
def lib():
    from tinyfluids_gb300 import _lib, build
    build.build()
    return _lib.load()


def test_header_declares_functions():
    names = declared_functions()
    assert "tf_evolve_state" in names and "tf_time_integration" in names
    assert len(names) >= 10


def test_library_exports_every_declared_symbol(lib):
    for name in declared_functions():
        assert hasattr(lib, name), f"{name} declared in include/ but not exported"


def test_python_binding_covers_every_declared_symbol():
    from tinyfluids_gb300 import _lib
    assert set(declared_functions()) == set(_lib.SIGNATURES)


def test_abi_and_status_strings(lib):
    assert lib.tf_abi_version() == 1
    assert lib.tf_ctl_bytes() == 64
    assert lib.tf_status_string(0) == b"ok"
    assert b"argument" in lib.tf_status_string(1)


def test_host_side_argument_checks(lib):
    """Bad arguments are rejected before any CUDA call, with a message."""
    from tinyfluids_gb300 import _lib
    with pytest.raises(_lib.TinyfluidsError) as e:
        _lib.call("tf_evolve_state", None, None, 4, 4, 4, 0.1, 0.01, None, 5 / 3, 0, None, None)
    assert e.value.status == 1
    fake = ctypes.c_void_p(0x1000)
    with pytest.raises(_lib.TinyfluidsError) as e:  # aliasing output
        _lib.call("tf_evolve_state", fake, fake, 4, 4, 4, 0.1, 0.01, None, 5 / 3, 0, None, None)
    assert "alias" in str(e.value)
    other = ctypes.c_void_p(0x2000)
    with pytest.raises(_lib.TinyfluidsError):  # zero-size axis
        _lib.call("tf_evolve_state", fake, other, 0, 4, 4, 0.1, 0.01, None, 5 / 3, 0, None, None)
    with pytest.raises(_lib.TinyfluidsError):  # above the 2^40-cell limit
        _lib.call("tf_evolve_state", fake, other, 1 << 14, 1 << 14, 1 << 14, 0.1, 0.01, None,
                  5 / 3, 0, None, None)
    with pytest.raises(_lib.TinyfluidsError):  # tile grid beyond the launch limits
        tc2 = _lib.TileConfig(8, 1, 0)
        _lib.call("tf_evolve_state", fake, other, 1 << 17, 8, 8, 0.1, 0.01, None, 5 / 3, 0,
                  ctypes.byref(tc2), None)
    with pytest.raises(_lib.TinyfluidsError):  # open boundaries need 2 cells
        _lib.call("tf_evolve_state", fake, other, 1, 4, 4, 0.1, 0.01, None, 5 / 3, 1, None, None)
    with pytest.raises(_lib.TinyfluidsError):  # gamma == 1
        _lib.call("tf_evolve_state", fake, other, 4, 4, 4, 0.1, 0.01, None, 1.0, 0, None, None)
    with pytest.raises(_lib.TinyfluidsError):  # bad tile rows
        tc = _lib.TileConfig(34, 4, 0)  # not one of 8, 16, 32
        _lib.call("tf_evolve_state", fake, other, 4, 4, 4, 0.1, 0.01, None, 5 / 3, 0,
                  ctypes.byref(tc), None)
    third = ctypes.c_void_p(0x3000)
    with pytest.raises(_lib.TinyfluidsError):  # slice plane outside the grid
        _lib.call("tf_evolve_state_diag", fake, other, 4, 4, 4, 0.1, 0.01, None, 5 / 3, 0, None,
                  third, third, 4, None)
    with pytest.raises(_lib.TinyfluidsError):  # diagnostics need a totals buffer
        _lib.call("tf_diagnostics", fake, 4, 4, 4, 5 / 3, None, None, 0, None)
    with pytest.raises(_lib.TinyfluidsError):  # unbounded loop
        _lib.call("tf_time_integration", fake, other, ctypes.c_void_p(0x3000),
                  ctypes.c_void_p(0x4000), 4, 4, 4, 0.1, float("inf"), 5 / 3, 0.4, -1, 0.0, 0,
                  None, None, None)


def test_host_state_runs_check_arguments_before_any_copy(lib):
    """tf_time_integration_host: workspace size, alignment, pointer lists,
    output/input overlap and the run's own arguments are rejected before any
    CUDA call (fake addresses are never dereferenced)."""
    from tinyfluids_gb300 import _lib
    sb = (5 * 4 * 32 ** 3 + 255) // 256 * 256
    assert lib.tf_host_runs_workspace_bytes(32, 32, 32, 3) == 6 * sb + 256
    assert lib.tf_host_runs_workspace_bytes(0, 32, 32, 3) == 0
    assert lib.tf_host_runs_workspace_bytes(32, 32, 32, 0) == 0
    nbytes = 5 * 4 * 32 ** 3
    ins = (ctypes.c_void_p * 2)(0x10000000, 0x20000000)
    outs = (ctypes.c_void_p * 2)(0x30000000, 0x40000000)
    ws, wsb = ctypes.c_void_p(0x50000000), 6 * sb + 256

    def run(i=ins, o=outs, count=2, w=ws, wb=wsb, dx=0.1, tf=0.2, ms=-1, flags=0):
        with pytest.raises(_lib.TinyfluidsError) as e:
            _lib.call("tf_time_integration_host", i, o, count, 32, 32, 32, dx, tf, 5 / 3, 0.4,
                      ms, 0.0, flags, None, w, wb, None, None)
        assert e.value.status == 1, str(e.value)
        return str(e.value)

    run(count=0)
    run(i=None)
    run(w=None)
    assert "needed" in run(wb=wsb - 1)
    run(w=ctypes.c_void_p(0x50000010))  # not 256-byte aligned
    run(i=(ctypes.c_void_p * 2)(0x10000000, None))
    # state 0's output overlaps state 1's input (copied in while 0 is copied out)
    assert "overlaps" in run(o=(ctypes.c_void_p * 2)(0x20000000 + nbytes - 4, 0x40000000))
    run(dx=0.0)
    run(tf=float("inf"))  # unbounded loop
    with pytest.raises(_lib.TinyfluidsError):  # open boundaries need 2 cells per axis
        _lib.call("tf_time_integration_host", ins, outs, 2, 1, 32, 32, 0.1, 0.2, 5 / 3, 0.4,
                  -1, 0.0, 1, None, ws, wsb, None, None)


def test_host_state_api_validates_before_launch():
    import torch
    import tinyfluids_gb300 as tg
    sb = (5 * 4 * 32 ** 3 + 255) // 256 * 256
    assert tg.host_runs_workspace_bytes((5, 32, 32, 32), 3) == 6 * sb + 256
    assert tg.host_runs_workspace_bytes((32, 32, 32), 3) == 6 * sb + 256
    good = torch.zeros(5, 4, 4, 4)
    with pytest.raises(ValueError):
        tg.time_integration_host([], 0.1, 0.2, 5 / 3, False)
    with pytest.raises(TypeError):
        tg.time_integration_host([good, torch.zeros(5, 4, 4, 4, dtype=torch.float64)], 0.1, 0.2,
                                 5 / 3, False)
    with pytest.raises(ValueError):  # shapes differ
        tg.time_integration_host([good, torch.zeros(5, 4, 4, 5)], 0.1, 0.2, 5 / 3, False)
    with pytest.raises(ValueError):  # non-contiguous
        tg.time_integration_host([torch.zeros(5, 4, 4, 8)[..., ::2]], 0.1, 0.2, 5 / 3, False)
    with pytest.raises(ValueError):  # out of the wrong length
        tg.time_integration_host([good], 0.1, 0.2, 5 / 3, False, out=[good, good])
    with pytest.raises(ValueError):
        tg.time_integration_host([good], 0.1, 0.2, 5 / 3, False, num_steps=-1)
    with pytest.raises(ValueError):  # a fixed dt must be positive
        tg.time_integration_host([good], 0.1, 0.2, 5 / 3, False, dt=-1.0)


def test_product_library_is_not_the_checked_build(lib):
    assert lib.tf_debug_checked() == 0
    assert lib.tf_debug_oob_count() == -1
    assert lib.tf_debug_reset(None, 0) == 5  # TF_ERR_UNSUPPORTED


def test_python_api_validates_before_launch():
    import torch
    import tinyfluids_gb300 as tg
    with pytest.raises(TypeError):
        tg._evolve_state(torch.zeros(4, 3, 3, 3), 0.1, 0.01, 5 / 3)
    with pytest.raises(TypeError):
        tg._evolve_state(torch.zeros(5, 3, 3, 3, dtype=torch.float64), 0.1, 0.01, 5 / 3)
    with pytest.raises(ValueError):  # CPU tensors: no CPU path
        tg._evolve_state(torch.zeros(5, 3, 3, 3), 0.1, 0.01, 5 / 3)
    with pytest.raises(NotImplementedError):
        tg.time_integration.time_integration(torch.zeros(5, 3, 3, 3), 0.1, 0.2, 5 / 3, False,
                                             True)


def test_tile_choice(lib):
    """The built-in tile choice (no GPU needed: dimensions and flags only):
    the y-marching 8-row tile where it computes no more cells than the
    x-marching 16-row tile (fast arithmetic, even nz, 2^17 cells or more;
    open boundaries from 2^27 cells), else the x-marching tile (8 rows up to
    128^3 cells, 16 above); explicit tiles are taken as given."""
    import tinyfluids_gb300 as tg
    assert tg.resolved_tile((512, 512, 512), exact=False)[::2] == (8, "ym")
    assert tg.resolved_tile((768, 768, 768), exact=False)[::2] == (8, "ym")
    assert tg.resolved_tile((96, 96, 96), exact=False)[::2] == (8, "ym")
    assert tg.resolved_tile((48, 48, 48), exact=False)[::2] == (8, "ldg")
    assert tg.resolved_tile((32, 32, 32), exact=False)[::2] == (8, "ldg")
    assert tg.resolved_tile((128, 128, 128), exact=False)[::2] == (8, "ldg")
    assert tg.resolved_tile((256, 256, 256), exact=False) == (16, 32, "ldg")
    assert tg.resolved_tile((512, 512, 512), exact=True)[::2] == (16, "ldg")
    assert tg.resolved_tile((512, 512, 512), True, exact=False)[::2] == (8, "ym")
    assert tg.resolved_tile((384, 384, 384), True, exact=False)[::2] == (16, "ldg")
    assert tg.resolved_tile((512, 512, 2), True, exact=False)[::2] == (8, "ldg")
    assert tg.resolved_tile((512, 512, 511), exact=False)[::2] == (16, "ldg")
    rows, lx, lay = tg.resolved_tile((512, 512, 512), exact=False)
    assert 16 <= lx <= 64
    assert tg.resolved_tile((64, 64, 64), exact=False, tile=(8, 5, "ym")) == (8, 5, "ym")
    assert tg.resolved_tile((64, 64, 64), exact=False, tile=(32, 7)) == (32, 7, "ldg")
    with pytest.raises(tg.TinyfluidsError):
        tg.resolved_tile((64, 64, 64), exact=False, tile=(32, 0, "ym"))
