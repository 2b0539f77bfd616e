"""Mixed precision (FP16 table copy of FP32 masters, one-pass TF32 MLP) against
the FP32 path and the float64 oracle.

The rendered normals of a patch batch are computed three ways at the same
parameters and samples: the FP32 path, the mixed path and the float64 oracle
(at the device's own query points).  The angular deviation from the oracle is
printed and bounded: FP32 within 0.05 degrees, mixed within 2 degrees on
average (FP16 keeps 11 significant bits of each table entry)."""
import numpy as np
import pytest
import torch

from oracle import field as OF
from oracle import renderer as OR

pytestmark = pytest.mark.gpu


def _angles(a, b):
    a = a.reshape(-1, 3).astype(np.float64)
    b = b.reshape(-1, 3).astype(np.float64)
    na, nb = np.linalg.norm(a, axis=1), np.linalg.norm(b, axis=1)
    keep = (na > 1e-3) & (nb > 1e-3)
    c = (a[keep] * b[keep]).sum(1) / (na[keep] * nb[keep])
    return np.degrees(np.arccos(np.clip(c, -1, 1)))


def test_mixed_precision_field_and_render_vs_fp32_and_oracle(built_lib):
    from supernormal_gb300 import scenes
    from supernormal_gb300._lib import SN_FIELD_MLP_TF32, SN_FIELD_TABLE_FP16
    from supernormal_gb300.fields import SDFNetwork, SingleVarianceNetwork
    from supernormal_gb300.nerfacc import OccupancyGrid
    from supernormal_gb300.trainer import FusedTrainer, TrainConfig

    enc = dict(otype="HashGrid", n_levels=16, n_features_per_level=2, log2_hashmap_size=15, base_resolution=16,
               per_level_scale=1.447)
    ds = scenes.SyntheticDataset(scenes.sphere(0.5), scenes.ring_cameras(8, 96, 96, elevation_deg=15),
                                 torch.device("cuda"))
    out = {}
    g = torch.Generator(device="cuda").manual_seed(21)
    batches = [ds.gen_random_patches(128, generator=g) for _ in range(60)]
    for prec in ("fp32", "mixed"):
        torch.manual_seed(0)
        net = SDFNetwork(3, 16, 64, 1, skip_in=(-1,), bias=0.5, encoding_config=enc, input_concat=True).cuda()
        var = SingleVarianceNetwork(0.3).cuda()
        net.bindwidth = 16
        grid = OccupancyGrid(roi_aabb=[-1.0] * 3 + [1.0] * 3, resolution=32).cuda()
        grid._binary = torch.ones_like(grid._binary)
        cfg = TrainConfig(batch_size=128, step_size=1.0 / 64, occ_update_freq=0, increase_bandwidth_every=0,
                          learning_rate=2e-3, warm_up_end=5, end_iter=60, precision=prec)
        tr = FusedTrainer(net, var, cfg, occupancy_grid=grid)
        losses = [float(tr.train_step(*b)[4].item()) for b in batches]
        tr.check_status()
        assert losses[-1] < 0.7 * losses[0], (prec, losses[0], losses[-1])
        out[prec] = (net, var, grid, tr)
    # same parameters for the comparison: the FP32 run's, rendered by both paths
    net, var, grid, tr32 = out["fp32"]
    trm = out["mixed"][3]
    with torch.no_grad():
        trm.params.copy_(tr32.params)
        trm.params_half.copy_(tr32.params)
    x = (torch.rand((20000, 3), device="cuda") * 1.6 - 0.8).contiguous()
    s32 = net.sdf_raw(x)
    # the mixed trainer's field call (FP16 table copy, one-pass TF32)
    from supernormal_gb300._lib import call, stream_handle
    import ctypes as C
    trm.weight_norm_forward(stream_handle())
    sm = torch.empty_like(s32)
    d = trm._mlp()
    assert d.flags == (SN_FIELD_TABLE_FP16 | SN_FIELD_MLP_TF32)
    call("sn_field_fwd", x.shape[0], None, x, trm._table(), trm._grid_desc(), 16, C.byref(d), 1, sm,
         stream_handle())
    torch.cuda.synchronize()
    err = (sm - s32).abs().max().item()
    print(f"\nsdf |mixed - fp32| max {err:.3e} over |sdf| max {s32.abs().max().item():.3e}")
    assert err < 2e-3
    # rendered normals: FP32 path and oracle at the same samples
    from supernormal_gb300.renderer import NeuSRenderer, near_far_from_sphere

    r = NeuSRenderer(net, var)
    r.occupancy_grid = grid
    r.sampling_step_size = 1.0 / 64
    ro, rd, pn, vinv, _, _ = batches[0]
    near, far = near_far_from_sphere(ro[:, 1, 1], rd[:, 1, 1])
    o32 = r.render(ro, rd, pn, near, far, vinv, mode="eval")
    pidx, ts, te = (t.detach().cpu().numpy() for t in r.last_samples)
    prm = OF.params_from_module(net)
    geom = OF.geometry_from_module(net)
    fld = lambda q: OF.sdf_network(q, **prm, geom=geom, active_levels=16, out_cols=1)
    cpu = lambda t: t.detach().cpu().numpy()
    ref = OR.patch_forward(fld, pidx, ts, te, cpu(ro), cpu(rd), cpu(pn), cpu(vinv),
                           var.variance.detach().cpu().double(), points=cpu(r.last_points))
    a32 = _angles(cpu(o32["comp_normal"]), ref["comp_normal"].detach().numpy())
    # mixed: the same samples' field values from the FP16 / one-pass path
    pts = r.last_points
    smix = torch.empty((pts.shape[0], 1), device="cuda")
    call("sn_field_fwd", pts.shape[0], None, pts.contiguous(), trm._table(), trm._grid_desc(), 16, C.byref(d),
         1, smix, stream_handle())
    smix64 = smix.detach().cpu().double()
    refm = OR.patch_forward(lambda q: smix64[: q.shape[0]], pidx, ts, te, cpu(ro), cpu(rd), cpu(pn), cpu(vinv),
                            var.variance.detach().cpu().double(), points=cpu(pts))
    am = _angles(refm["comp_normal"].detach().numpy(), ref["comp_normal"].detach().numpy())
    print(f"rendered-normal deviation from the float64 oracle: fp32 mean {a32.mean():.2e} deg "
          f"(max {a32.max():.2e}); mixed field mean {am.mean():.2e} deg (max {am.max():.2e})")
    assert a32.mean() < 0.05
    assert am.mean() < 2.0
