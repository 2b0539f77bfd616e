"""The C restatement of the marcher: properties of nerfacc's marcher (CPU).

nerfacc pins only "samples lie inside the ROI" (NA/tests/test_ray_marching.py:26-47);
the lattice, skipping and jitter properties below follow from
NA/nerfacc/cuda/csrc/ray_marching.cu:81-192."""
import numpy as np

from oracle import march


def _rays(n, seed):
    rng = np.random.default_rng(seed)
    o = rng.random((n, 3)).astype(np.float32)
    d = rng.standard_normal((n, 3)).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return o, d.astype(np.float32)


def test_samples_inside_roi_with_full_grid():
    o, d = _rays(128, 0)
    roi = np.array([0, 0, 0, 1, 1, 1], np.float32)
    grid = np.ones((128, 128, 128), np.uint8)
    n = o.shape[0]
    packed, ri, ts, te = march.ray_marching(o, d, np.zeros(n), np.ones(n), roi, grid, 1e-2)
    mid = o[ri] + d[ri] * ((ts + te) / 2)[:, None]
    assert (mid <= 1.0 + 1e-6).all() and (mid >= -1e-6).all()
    assert packed[:, 1].sum() == ri.size and (np.diff(ri) >= 0).all()


def test_all_occupied_gives_regular_lattice():
    o = np.array([[-2.0, 0.01, 0.02]], np.float32)
    d = np.array([[1.0, 0.0, 0.0]], np.float32)
    roi = np.array([-1, -1, -1, 1, 1, 1], np.float32)
    grid = np.ones((16, 16, 16), np.uint8)
    step = 0.125
    _, ri, ts, te = march.ray_marching(o, d, np.array([1.0]), np.array([3.0]), roi, grid, step)
    # t_mid must lie inside the ROI: samples start at t=1 and stop before t_mid >= 3
    assert ri.size == 16
    np.testing.assert_allclose(ts, 1.0 + step * np.arange(16), atol=1e-6)
    np.testing.assert_allclose(te - ts, step, atol=1e-6)


def test_empty_grid_gives_no_samples():
    o, d = _rays(64, 1)
    roi = np.array([0, 0, 0, 1, 1, 1], np.float32)
    packed, ri, _, _ = march.ray_marching(o, d, np.zeros(64), np.ones(64) * 2, roi,
                                          np.zeros((32, 32, 32), np.uint8), 1e-3)
    assert ri.size == 0 and (packed[:, 1] == 0).all()


def test_skipping_keeps_samples_on_occupied_voxels():
    rng = np.random.default_rng(3)
    grid = (rng.random((32, 32, 32)) < 0.2).astype(np.uint8)
    roi = np.array([-1, -1, -1, 1, 1, 1], np.float32)
    o, d = _rays(256, 4)
    o = (o * 2 - 1).astype(np.float32)
    _, ri, ts, te = march.ray_marching(o, d, np.zeros(256), np.ones(256) * 3, roi, grid, 5e-3)
    mid = o[ri] + d[ri] * ((ts + te) / 2)[:, None]
    cell = np.clip(((mid + 1) / 2 * 32).astype(int), 0, 31)
    assert grid[cell[:, 0], cell[:, 1], cell[:, 2]].mean() > 0.99


def test_jitter_shifts_the_first_sample():
    o = np.array([[-2.0, 0.01, 0.02]], np.float32)
    d = np.array([[1.0, 0.0, 0.0]], np.float32)
    roi = np.array([-1, -1, -1, 1, 1, 1], np.float32)
    grid = np.ones((16, 16, 16), np.uint8)
    _, _, ts, _ = march.ray_marching(o, d, np.array([1.0]), np.array([3.0]), roi, grid, 0.125,
                                     jitter=np.array([0.5], np.float32))
    assert abs(ts[0] - (1.0 + 0.5 * 0.125)) < 1e-7
