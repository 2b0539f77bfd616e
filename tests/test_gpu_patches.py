"""On-device patch generation (sn_gen_patches) against gathers from the
per-pixel ray and V^-1 tables (models/dataset_loader.py:112-145, 223-277)."""
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("ph,pw", [(3, 3), (5, 3)])
def test_gen_patches_matches_table_gathers(built_lib, ph, pw):
    from supernormal_gb300 import scenes

    rig = scenes.ring_cameras(5, 70, 90, radius=3.0, elevation_deg=25.0, fov_deg=40.0)
    ds = scenes.SyntheticDataset(scenes.displaced_torus(0.5, 0.2, 0.02, 20.0), rig, torch.device("cuda"))
    n = 777
    g = torch.Generator(device="cuda").manual_seed(5)
    got = ds.gen_random_patches(n, ph, pw, generator=g)
    g = torch.Generator(device="cuda").manual_seed(5)            # the same draws, gathered from tables
    cx = torch.randint(pw // 2, ds.W - 1 - pw // 2, (n,), device="cuda", generator=g)
    cy = torch.randint(ph // 2, ds.H - 1 - ph // 2, (n,), device="cuda", generator=g)
    img = torch.randint(0, ds.n_images, (n,), device="cuda", generator=g)
    px = cx[:, None, None] + torch.arange(-(pw // 2), pw // 2 + 1, device="cuda")[None, None, :]
    py = cy[:, None, None] + torch.arange(-(ph // 2), ph // 2 + 1, device="cuda")[None, :, None]
    px, py = px.expand(n, ph, pw), py.expand(n, ph, pw)
    iv = img[:, None, None].expand(n, ph, pw)
    want = (ds.pose_all[img, None, None, :3, 3].expand(n, ph, pw, 3), ds.rays_all[iv, py, px],
            ds.pose_all[img, :3, 2], ds.V_inverse_all[iv, py, px], ds.normals[iv, py, px],
            ds.masks[iv, py, px].unsqueeze(-1))
    names = ["rays_o", "rays_d", "plane_n", "vinv", "normal", "mask"]
    for name, a, b in zip(names, got, want):
        assert a.shape == b.shape, name
        if name in ("normal", "mask", "rays_o", "plane_n"):
            assert torch.equal(a, b), name                          # plain gathers / copies
        else:   # same double formulas, rounded once; reductions may order differently
            torch.testing.assert_close(a, b, rtol=1e-6, atol=1e-6, msg=name)
    # V^-1 inverts V = rows (d, right, down)
    right = ds.pose_all[img, None, None, :3, 0].expand(n, ph, pw, 3)
    down = ds.pose_all[img, None, None, :3, 1].expand(n, ph, pw, 3)
    V = torch.stack([got[1], right, down], dim=-2).double()
    eye = torch.eye(3, device="cuda", dtype=torch.float64).expand(n, ph, pw, 3, 3)
    torch.testing.assert_close(V @ got[3].double(), eye, rtol=0, atol=1e-5)
    assert ds._tables is not None            # the tables were only built for this comparison


def test_dataset_keeps_no_per_pixel_tables(built_lib):
    from supernormal_gb300 import scenes

    ds = scenes.SyntheticDataset(scenes.sphere(0.5), scenes.ring_cameras(3, 40, 50), torch.device("cuda"))
    ds.gen_random_patches(64)
    assert ds._tables is None


@pytest.mark.parametrize("which", ["sphere", "torus", "union"])
def test_scene_ground_truth_kernel_matches_torch(built_lib, which):
    """sn_scene_render_gt (one launch, double sphere tracing, central-difference
    normals) against the torch float64 path (autograd normals) on every pixel."""
    from supernormal_gb300 import scenes

    sc = {"sphere": scenes.sphere(0.45, (0.05, 0.0, -0.02)),
          "torus": scenes.displaced_torus(0.5, 0.2, 0.02, 20.0),
          "union": scenes.random_scene(3)}[which]
    assert sc.descriptor() is not None
    rig = scenes.ring_cameras(3, 48, 64, radius=3.0, elevation_deg=25.0)
    ds = scenes.SyntheticDataset(sc, rig, torch.device("cuda"))
    H, W = rig.H, rig.W
    ys, xs = torch.meshgrid(torch.arange(H, device="cuda", dtype=torch.float64),
                            torch.arange(W, device="cuda", dtype=torch.float64), indexing="ij")
    for v in range(3):
        nrm, hit = scenes.render_view_gt(sc, rig, v, xs, ys)
        m_ref = hit.reshape(H, W).float()
        m_got = ds.masks[v]
        differ = (m_ref != m_got)
        assert differ.float().mean().item() < 2e-3
        both = (m_ref > 0) & (m_got > 0)
        err = (ds.normals[v][both] - nrm.reshape(H, W, 3).float()[both]).abs().max().item()
        assert both.sum() > 100 and err < 1e-5, err
