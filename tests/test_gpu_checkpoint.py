"""Checkpoints in the reference's layout (exp_runner.py:297-315): the saved
dict loads into the reference's own torch.optim.Adam, whose next step equals
the fused Adam's, and a trainer resumed from it continues the original run."""
import pytest
import torch

pytestmark = pytest.mark.gpu

ENC = dict(otype="HashGrid", n_levels=16, n_features_per_level=2, log2_hashmap_size=15,
           base_resolution=16, per_level_scale=1.447)


def _setup():
    from supernormal_gb300 import scenes
    from supernormal_gb300.fields import SDFNetwork, SingleVarianceNetwork
    from supernormal_gb300.trainer import FusedTrainer, TrainConfig

    ds = scenes.SyntheticDataset(scenes.sphere(0.5), scenes.ring_cameras(6, 96, 96, elevation_deg=20),
                                 torch.device("cuda"))

    def make():
        torch.manual_seed(0)
        net = SDFNetwork(3, 1, 64, 1, skip_in=(-1,), bias=0.5, encoding_config=ENC, input_concat=True).cuda()
        var = SingleVarianceNetwork(0.3).cuda()
        cfg = TrainConfig(batch_size=128, step_size=1.0 / 96, occ_update_freq=4, occ_warmup_steps=4,
                          increase_bandwidth_every=2, end_iter=50, warm_up_end=3, seed=2)
        return FusedTrainer(net, var, cfg)

    return ds, make


def test_optimizer_state_matches_reference_adam(built_lib, tmp_path):
    from supernormal_gb300._lib import call, stream_handle

    ds, make = _setup()
    tr = make()
    g = torch.Generator(device="cuda").manual_seed(4)
    for _ in range(6):
        tr.train_step(*ds.gen_random_patches(128, generator=g))
    torch.cuda.synchronize()
    path = tmp_path / "ckpt_000006.pth"
    tr.save_checkpoint(path)
    ckpt = torch.load(path, map_location="cpu")
    assert set(ckpt) == {"sdf_network_fine", "variance_network_fine", "optimizer", "iter_step"}
    assert ckpt["iter_step"] == 6
    assert set(ckpt["sdf_network_fine"]) == {"encoding.params", "lin0.bias", "lin0.weight_g", "lin0.weight_v",
                                             "lin1.bias", "lin1.weight_g", "lin1.weight_v"}
    # the reference's optimizer over its parameter order (exp_runner.py:89-97)
    ref_params = [torch.nn.Parameter(p.detach().cpu().clone()) for p in tr._reference_params()]
    opt = torch.optim.Adam(ref_params, lr=5e-4)
    opt.load_state_dict(ckpt["optimizer"])
    lr = 3.7e-4
    for grp in opt.param_groups:
        grp["lr"] = lr
    gen = torch.Generator().manual_seed(1)
    grads = [torch.randn(p.shape, generator=gen) * 1e-2 for p in ref_params]
    for p, gr in zip(ref_params, grads):
        p.grad = gr.clone()
    opt.step()
    # the same step on the flat buffers
    with torch.no_grad():
        tr.grads.zero_()
        for name, gr in zip(tr._REFERENCE_ORDER, grads):
            tr._flat(tr.grads, name).copy_(gr.cuda())
    call("sn_adam_step", tr.n_params, tr.params, tr.grads, tr.exp_avg, tr.exp_avg_sq, None, None, None, lr, 7,
         0.9, 0.999, 1e-8, 1, stream_handle())
    torch.cuda.synchronize()
    for name, p in zip(tr._REFERENCE_ORDER, ref_params):
        got = tr._flat(tr.params, name).cpu()
        torch.testing.assert_close(got, p.detach(), rtol=1e-5, atol=1e-7, msg=name)


def test_resume_continues_the_run(built_lib, tmp_path):
    ds, make = _setup()
    tr = make()
    g = torch.Generator(device="cuda").manual_seed(4)
    batches = [ds.gen_random_patches(128, generator=g) for _ in range(8)]
    for b in batches[:6]:
        tr.train_step(*b)
    path = tmp_path / "ckpt.pth"
    tr.save_checkpoint(path)
    tr2 = make()
    tr2.load_checkpoint(path)
    tr2.net.bindwidth = tr.net.bindwidth              # the reference keeps it in the module, not the checkpoint
    tr2.grid.load_state_dict(tr.grid.state_dict())   # nor the occupancy grid
    for name in tr._REFERENCE_ORDER:
        assert torch.equal(tr._flat(tr.params, name), tr2._flat(tr2.params, name)), name
        assert torch.equal(tr._flat(tr.exp_avg, name), tr2._flat(tr2.exp_avg, name)), name
    assert int(tr2.iter_dev.item()) == int(tr.iter_dev.item()) == 6 and tr2.iter_step == 6
    l1 = tr.train_step(*batches[6]).clone()
    l2 = tr2.train_step(*batches[6]).clone()
    torch.cuda.synchronize()
    assert torch.equal(l1[1:], l2[1:])                 # the forward losses
    torch.testing.assert_close(l1, l2, rtol=1e-4, atol=1e-7)
    for name in tr._REFERENCE_ORDER:
        torch.testing.assert_close(tr._flat(tr.params, name), tr2._flat(tr2.params, name), rtol=1e-3, atol=1e-6)
