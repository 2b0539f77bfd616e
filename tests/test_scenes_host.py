"""The synthetic dataset on the host: lazily built per-pixel tables and the
gather path of gen_random_patches (models/dataset_loader.py:112-145, 223-277)."""
import torch

from supernormal_gb300 import scenes


def test_cpu_patches_from_lazy_tables():
    rig = scenes.ring_cameras(3, 30, 36, radius=3.0, elevation_deg=20.0)
    ds = scenes.SyntheticDataset(scenes.sphere(0.5), rig, torch.device("cpu"))
    assert ds._tables is None                      # nothing per pixel until asked for
    g = torch.Generator().manual_seed(0)
    ro, rd, pn, vinv, nrm, mask = ds.gen_random_patches(40, generator=g)
    assert ds._tables is not None
    assert ro.shape == rd.shape == nrm.shape == (40, 3, 3, 3)
    assert vinv.shape == (40, 3, 3, 3, 3) and mask.shape == (40, 3, 3, 1) and pn.shape == (40, 3)
    # V^-1 inverts V = rows (d, camera right, camera down) of each pixel
    g = torch.Generator().manual_seed(0)
    cx = torch.randint(1, ds.W - 2, (40,), generator=g)
    cy = torch.randint(1, ds.H - 2, (40,), generator=g)
    img = torch.randint(0, ds.n_images, (40,), generator=g)
    right = ds.pose_all[img, :3, 0][:, None, None, :].expand(40, 3, 3, 3)
    down = ds.pose_all[img, :3, 1][:, None, None, :].expand(40, 3, 3, 3)
    V = torch.stack([rd, right, down], dim=-2).double()
    eye = torch.eye(3, dtype=torch.float64).expand(40, 3, 3, 3, 3)
    torch.testing.assert_close(V @ vinv.double(), eye, rtol=0, atol=1e-5)
    # unit ray directions through the sampled pixels, origin at the camera
    torch.testing.assert_close(rd.norm(dim=-1), torch.ones(40, 3, 3), rtol=0, atol=1e-6)
    torch.testing.assert_close(ro, ds.pose_all[img, :3, 3][:, None, None, :].expand(40, 3, 3, 3))
    assert torch.equal(rd[:, 1, 1], ds.rays_all[img, cy, cx])
