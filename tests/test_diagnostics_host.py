"""Host side of the diagnostics: the image/array writer (no GPU needed)."""
import numpy as np
import torch

from tinyfluids_gb300 import diagnostics as D


def read_pgm(path):
    with open(path, "rb") as f:
        data = f.read()
    head, rest = data.split(b"\n", 3)[:3], data.split(b"\n", 3)[3]
    assert head[0] == b"P5"
    w, h = (int(v) for v in head[1].split())
    assert int(head[2]) == 255
    return np.frombuffer(rest, dtype=np.uint8).reshape(h, w)


def test_save_slices_writes_scaled_images_and_array(tmp_path):
    nx, ny = 6, 4
    rho = np.arange(nx * ny, dtype=np.float32).reshape(nx, ny)
    p = np.full((nx, ny), 2.5, np.float32)
    paths = D.save_slices(torch.from_numpy(np.stack([rho, p])), str(tmp_path / "sub" / "check_6"))
    img = read_pgm(paths[0])
    assert img.shape == (nx, ny)  # rows = x, columns = y, like imshow(state[:, :, z])
    assert img[0, 0] == 0 and img[-1, -1] == 255
    assert np.all(np.diff(img.astype(int).ravel()) >= 0)
    assert np.all(read_pgm(paths[1]) == 0)  # constant field: no division by zero
    np.testing.assert_array_equal(np.load(paths[2]), np.stack([rho, p]))


def test_integrals_scale_by_cell_volume():
    t = torch.tensor([8.0, 1.0, -2.0, 0.0, 16.0], dtype=torch.float64)
    out = D.integrals(t, 0.5)
    assert out == {"mass": 1.0, "momentum_x": 0.125, "momentum_y": -0.25, "momentum_z": 0.0,
                   "energy": 2.0}
