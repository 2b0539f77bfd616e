"""The host restatement of the benchmark scene, batches and initial
parameters (oracle/scene.py, used by bench.py's CPU legs) against the
package's own construction of the same objects."""
import numpy as np
import torch

from oracle import scene as OS

ENC = dict(otype="HashGrid", n_levels=16, n_features_per_level=2, log2_hashmap_size=15,
           base_resolution=16, per_level_scale=1.447)


def test_initial_parameters_match_sdf_network(built_lib):
    from supernormal_gb300.fields import SDFNetwork

    torch.manual_seed(1234)
    net = SDFNetwork(3, 16, 64, 1, skip_in=(-1,), bias=0.5, encoding_config=ENC, input_concat=True)
    prm, geom = OS.sdf_network_init(1234, ENC)
    want = dict(table=net.encoding.params, v0=net.lin0.weight_v, g0=net.lin0.weight_g, b0=net.lin0.bias,
                v1=net.lin1.weight_v, g1=net.lin1.weight_g, b1=net.lin1.bias)
    for k, v in want.items():
        assert torch.equal(prm[k], v.detach()), k
    np.testing.assert_array_equal(geom[0], net.encoding.level_offsets())
    np.testing.assert_array_equal(geom[1], net.encoding.level_resolutions())


def test_scene_and_rig_match_package():
    from supernormal_gb300 import scenes

    sc = scenes.displaced_torus(0.5, 0.2, 0.02, 20.0)
    p = np.random.RandomState(0).uniform(-1, 1, (1000, 3))
    np.testing.assert_allclose(OS.torus_sdf(p), sc(torch.from_numpy(p)).numpy(), rtol=0, atol=1e-14)
    assert abs(OS.torus_lipschitz() - sc.lipschitz) < 1e-12
    rig = scenes.ring_cameras(5, 40, 60, radius=3.0, elevation_deg=30.0, fov_deg=40.0)
    poses, kinv = OS.ring_rig(5, 40, 60)
    np.testing.assert_allclose(poses, rig.poses[:, :3, :4].numpy(), atol=1e-12)
    np.testing.assert_allclose(kinv, np.linalg.inv(rig.intrinsics[:, :3, :3].numpy()), atol=1e-12)


def test_patches_are_consistent():
    poses, kinv = OS.ring_rig(20, 512, 612)
    rng = np.random.default_rng(0)
    ro, rd, pn, vinv, nrm, mask = OS.gen_random_patches(OS.torus_sdf, OS.torus_lipschitz(), poses, kinv,
                                                        512, 612, 64, rng)
    assert ro.shape == (64, 3, 3, 3) and vinv.shape == (64, 3, 3, 3, 3) and mask.shape == (64, 3, 3, 1)
    np.testing.assert_allclose(np.linalg.norm(rd, axis=-1), 1.0, atol=1e-6)
    # d^T V^-1 = e_0: the first row of V is the ray direction (models/dataset_loader.py:126-136)
    np.testing.assert_allclose(np.einsum("nhwi,nhwij->nhwj", rd, vinv), np.broadcast_to([1, 0, 0], rd.shape),
                               atol=1e-4)
    hit = mask[..., 0] > 0
    assert 0 < hit.sum() < hit.size
    np.testing.assert_allclose(np.linalg.norm(nrm[hit], axis=-1), 1.0, atol=1e-5)
    assert (np.abs(nrm[~hit]) == 0).all()


def test_analytic_occupancy():
    g = OS.analytic_occupancy(OS.torus_sdf, 64)
    c = (np.stack(np.meshgrid(*[np.arange(64)] * 3, indexing="ij"), -1).reshape(-1, 3) + 0.5) / 64 * 2 - 1
    sd = OS.torus_sdf(c).reshape(64, 64, 64)
    assert g[sd < -0.02].all() and not g[sd > 0.1].any()
