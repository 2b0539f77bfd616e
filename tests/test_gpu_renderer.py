"""GPU parity of the patch renderer and the fused training step vs the float64 oracle.

The oracle re-runs models/renderer.py's patch math and exp_runner.py's losses
on the samples our marcher/culling kept (the marcher itself is checked bit
for bit in test_gpu_nerfacc.py), with the device field's sdf values at the
device's query points (``device_valued``).  Tolerances: rendered normals 2e-4 and
weight sums 2e-5 absolute, losses 1e-4 relative, parameter gradients 2e-3
relative to each gradient's max-abs (float32 kernels with atomics vs float64)."""
import numpy as np
import pytest
import torch

from oracle import field as OF
from oracle import renderer as OR

pytestmark = pytest.mark.gpu

ENC = dict(otype="HashGrid", n_levels=16, n_features_per_level=2, log2_hashmap_size=15,
           base_resolution=16, per_level_scale=1.447)


def rel_err(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-30)


def l2_rel(a, b):
    """||a - b|| / ||b||: used for the hash-table gradient, a sum of float32
    atomics over many points (max-abs would be dominated by reordering noise)."""
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)


def grad_err(name, a, b):
    return l2_rel(a, b) if name == "table" else rel_err(a, b)


@pytest.fixture(scope="module")
def scene(built_lib):
    from supernormal_gb300 import scenes

    return scenes.SyntheticDataset(scenes.sphere(0.5), scenes.ring_cameras(6, 96, 96, elevation_deg=20),
                                   torch.device("cuda"))


def make(seed=0, d_out=16, table_scale=300.0, variance=0.25):
    from supernormal_gb300.fields import SDFNetwork, SingleVarianceNetwork

    torch.manual_seed(seed)
    net = SDFNetwork(3, d_out, 64, 1, skip_in=(-1,), bias=0.5, encoding_config=ENC, input_concat=True)
    with torch.no_grad():
        net.encoding.params.mul_(table_scale)
        net.lin0.weight_v[:, 3:].normal_(0.0, 0.05)
    net.bindwidth = 16
    return net.cuda(), SingleVarianceNetwork(variance).cuda()


def oracle_field(net):
    prm = OF.params_from_module(net)
    geom = OF.geometry_from_module(net)
    act = net.active_levels()
    return prm, (lambda x: OF.sdf_network(x, **prm, geom=geom, active_levels=act, out_cols=1))


def device_valued(fld, net, points):
    """The oracle field with the device field's float32 values at ``points`` and
    the float64 field's derivatives (straight through).  alpha's clip and the
    mask loss's clip branch on the sdf values, and inv_s amplifies a 1e-7 sdf
    difference, so the patch math is compared at the device's own values while
    the field's value parity is asserted here and its derivatives flow through
    the oracle.  ('ad' evaluates the start points, a prefix of ``points``.)"""
    dev = net.sdf(points).detach().cpu().double()
    ref = fld(torch.as_tensor(cpu(points)).double()).detach()
    assert np.abs(dev.numpy() - ref.numpy()).max() < 2e-5 * max(np.abs(ref.numpy()).max(), 1.0)

    def field(q):
        s = fld(q)
        return s + (dev[: s.shape[0]].reshape(s.shape) - s).detach()

    return field


def full_grid():
    from supernormal_gb300.nerfacc import OccupancyGrid

    g = OccupancyGrid(roi_aabb=[-1.0, -1.0, -1.0, 1.0, 1.0, 1.0], resolution=32).cuda()
    g._binary = torch.ones_like(g._binary)
    return g


def cpu(t):
    return t.detach().cpu().numpy()


@pytest.mark.parametrize("method", ["dfd", "ad"])
def test_renderer_forward_backward_matches_oracle(scene, method):
    from supernormal_gb300.renderer import NeuSRenderer, near_far_from_sphere

    net, var = make()
    r = NeuSRenderer(net, var, gradient_method=method)
    r.occupancy_grid = full_grid()
    r.sampling_step_size = 1.0 / 96
    g = torch.Generator(device="cuda").manual_seed(3)
    ro, rd, pn, vinv, nrm, mask = scene.gen_random_patches(96, generator=g)
    near, far = near_far_from_sphere(ro[:, 1, 1], rd[:, 1, 1])
    out = r.render(ro, rd, pn, near, far, vinv)
    pidx, ts, te = (cpu(t) for t in r.last_samples)
    assert pidx.size > 200
    prm, fld = oracle_field(net)
    var_ref = var.variance.detach().cpu().double().clone().requires_grad_(True)
    ref = OR.patch_forward(device_valued(fld, net, r.last_points), pidx, ts, te, cpu(ro), cpu(rd),
                           cpu(pn), cpu(vinv), var_ref, points=cpu(r.last_points),
                           gradient_method=method)
    assert np.abs(cpu(out["comp_normal"]) - cpu(ref["comp_normal"])).max() < 2e-4
    assert np.abs(cpu(out["weight_sum"]) - cpu(ref["weight_sum"])).max() < 2e-5
    assert np.abs(cpu(out["gradients"]) - cpu(ref["gradients"])).max() < 2e-3
    # losses of exp_runner.py through autograd on both sides
    L = OR.losses(out["comp_normal"].double().cpu(), out["weight_sum"].double().cpu(),
                  out["gradients"].double().cpu(), cpu(nrm), cpu(mask))
    Lr = OR.losses(ref["comp_normal"], ref["weight_sum"], ref["gradients"], cpu(nrm), cpu(mask))
    for k in ("normal", "eikonal", "mask", "total"):
        assert abs(L[k].item() - Lr[k].item()) <= 1e-4 * max(abs(Lr[k].item()), 1e-6), k
    Lg = OR.losses(out["comp_normal"], out["weight_sum"], out["gradients"],
                   torch.as_tensor(cpu(nrm)).cuda(), torch.as_tensor(cpu(mask)).cuda())
    params = [net.encoding.params, net.lin0.weight_v, net.lin0.weight_g, net.lin0.bias,
              net.lin1.weight_v, net.lin1.weight_g, net.lin1.bias, var.variance]
    grads = torch.autograd.grad(Lg["total"], params, allow_unused=True)
    names = ["table", "v0", "g0", "b0", "v1", "g1", "b1"]
    rgrads = torch.autograd.grad(Lr["total"], [prm[n] for n in names] + [var_ref], allow_unused=True)
    rg = dict(zip(names + ["variance"], rgrads))
    for n, a, b in zip(names + ["variance"], grads, rgrads):
        if b is None:
            continue
        if n in ("g0", "g1"):
            err = weight_g_err(cpu(a), b, prm["v" + n[1]], prm[n], rg["v" + n[1]])
        else:
            err = grad_err(n, cpu(a), b.numpy())
        assert err < 2e-3, (n, err)


def clip_boundary_points(ref, S, P, inv_s, band=1e-6):
    """Field points of the samples whose unclipped NeuS ratio
    q = (c0 - c1 + 1e-5) / (c0 + 1e-5) lies within ``band`` of alpha's clip
    bounds 0 and 1 (models/renderer.py:177-179), from the oracle's float64
    values.  There the float32 kernel and the float64 oracle may clip on
    different sides (q's float32 rounding error is ~1e-7), so d alpha / d q is
    passed by one and zeroed by the other; those points' sdf gradients are
    left out of a max-relative comparison.  Returns a mask over all field
    points (start points of every sample, then end points of diff samples)."""
    sdf = ref["sdf"].detach().numpy().reshape(-1, P)
    diff = np.asarray(ref["diff"])
    s0 = sdf[:S]
    s1 = np.concatenate([s0[1:], s0[-1:]], 0)
    s1[diff] = sdf[S:]
    sig = lambda z: 1.0 / (1.0 + np.exp(-z))
    c, n = sig(s0 * inv_s), sig(s1 * inv_s)
    q = (c - n + 1e-5) / (c + 1e-5)
    ii, kk = np.nonzero((np.abs(q) < band) | (np.abs(q - 1.0) < band))
    mask = np.zeros(sdf.shape, bool)
    mask[ii, kk] = True
    end_row = np.where(diff, S + np.cumsum(diff) - 1, np.minimum(np.arange(S) + 1, S - 1))
    mask[end_row[ii], kk] = True
    return mask.ravel()


class _FixedSdf:
    """sdf_network stand-in returning given values (a leaf) at the query points."""

    def __init__(self, values, ext=None):
        self.values, self.ext = values, ext

    def sdf(self, x):
        assert x.shape[0] == self.values.shape[0]
        return self.values

    def sdf_and_gradient(self, x):
        return self.values[: x.shape[0]], self.ext


@pytest.mark.parametrize("method,step,outputs,tol", [
    ("dfd", 1.0 / 96, "all", 1e-4), ("ad", 1.0 / 96, "all", 1e-4),
    ("dfd", 1.0 / 512, "weight_sum", 5e-5), ("dfd", 1.0 / 512, "all", 1e-3)])
def test_patch_adjoint_matches_oracle_on_fixed_sdf(scene, method, step, outputs, tol):
    """The fused patch kernel alone: d loss / d sdf (every start and end point),
    d / d variance and, for 'ad', d / d gradients, for a linear loss on the
    outputs, against float64 autograd of the oracle's patch math on the same
    float32 sdf values.  The fine step gives rays of several 32-sample chunks:
    a loss on the weight sums alone isolates the transmittance product and the
    weight adjoint's suffix sums (double-float in the kernel) and holds to
    5e-5; with the normal loss, the dfd differences (s1 - s0) / dt and
    (s_r - s_l) / (dx_l + dx_r) of float32 sdf values ~0.5 over steps of 2e-3
    lose ~eps * 0.5 / 2e-3 ~ 3e-5 relative in float32, in the reference's own
    float32 arithmetic as here, hence 1e-3.  Points of samples at alpha's clip
    boundary (float32 and float64 clip differently there) are left out of the
    sdf comparison; they are a small fraction of the points."""
    from supernormal_gb300.renderer import NeuSRenderer, near_far_from_sphere

    net, var = make()
    r = NeuSRenderer(net, var, gradient_method=method)
    r.occupancy_grid = full_grid()
    r.sampling_step_size = step
    g = torch.Generator(device="cuda").manual_seed(11)
    ro, rd, pn, vinv, _, _ = scene.gen_random_patches(64, generator=g)
    near, far = near_far_from_sphere(ro[:, 1, 1], rd[:, 1, 1])
    r.render(ro, rd, pn, near, far, vinv)
    pidx, ts, te = r.last_samples
    pts = r.last_points
    S, P = pidx.shape[0], 9
    assert S > 100
    if step < 0.005:
        assert torch.bincount(pidx).max().item() > 96      # several chunks per ray
    vals = net.sdf(pts).detach().clone().requires_grad_(True)
    ext = None
    if method == "ad":
        ext = (torch.randn((S * P, 3), device="cuda", generator=g) * 0.3 + torch.tensor(
            [0.0, 0.0, 1.0], device="cuda")).requires_grad_(True)
    rf = NeuSRenderer(_FixedSdf(vals, ext), var, gradient_method=method)
    out = rf.render_samples(ro, rd, pn, vinv, pidx, ts, te, method)
    gc = torch.randn(out["comp_normal"].shape, device="cuda", generator=g)
    gw = torch.randn(out["weight_sum"].shape, device="cuda", generator=g)
    gg = torch.randn(out["gradients"].shape, device="cuda", generator=g)
    if outputs == "weight_sum":
        gc.zero_()
        gg.zero_()
    L = (out["comp_normal"] * gc).sum() + (out["weight_sum"] * gw).sum() + (out["gradients"] * gg).sum()
    leaves = [vals, var.variance] + ([ext] if ext is not None else [])
    got = torch.autograd.grad(L, leaves)

    v64 = vals.detach().cpu().double().requires_grad_(True)
    var64 = var.variance.detach().cpu().double().clone().requires_grad_(True)
    e64 = None if ext is None else ext.detach().cpu().double().requires_grad_(True)
    ref = OR.patch_forward(lambda q: v64, cpu(pidx), cpu(ts), cpu(te), cpu(ro), cpu(rd), cpu(pn),
                           cpu(vinv), var64, points=cpu(pts), gradient_method=method,
                           ext_gradients=e64)
    Lr = ((ref["comp_normal"] * gc.cpu().double()).sum() + (ref["weight_sum"] * gw.cpu().double()).sum()
          + (ref["gradients"] * gg.cpu().double()).sum())
    refg = torch.autograd.grad(Lr, [v64, var64] + ([e64] if e64 is not None else []))
    inv_s = float(OR.inv_s_of(var64.detach(), torch.float64))
    edge = clip_boundary_points(ref, S, P, inv_s)
    assert edge.mean() < 0.01
    for name, a, b in zip(["sdf", "variance", "gradients"], got, refg):
        a, b = cpu(a).ravel(), b.numpy().ravel()
        if name == "sdf":
            a, b = a[~edge], b[~edge]
        assert rel_err(a, b) < tol, name


def _trainer(scene, B=128, **kw):
    from supernormal_gb300.trainer import FusedTrainer, TrainConfig

    net, var = make()
    cfg = TrainConfig(batch_size=B, step_size=1.0 / 96, occ_update_freq=0, increase_bandwidth_every=0,
                      **kw)
    tr = FusedTrainer(net, var, cfg, occupancy_grid=full_grid())
    return tr, net, var


def _check_trainer_step(tr, net, var, batch, method, min_samples, table_tol=2e-3):
    """One forward/backward of the fused step against the oracle on the kept
    samples: culling, the four losses and every parameter gradient."""
    ro, rd, pn, vinv, nrm, mask = batch
    prm, fld = oracle_field(net)
    var_ref = var.variance.detach().cpu().double().clone().requires_grad_(True)
    tr.grads.zero_()
    tr.forward_backward(ro, rd, pn, vinv, nrm, mask, tr.step_size(tr.iter_step), net.active_levels())
    torch.cuda.synchronize()
    tr.check_status()
    S = int(tr.S.item())
    assert S > min_samples
    # culling parity on the pre-cull samples
    n0 = int(tr.total0.item())
    ri0, ts0, te0 = cpu(tr.ridx0[:n0]), cpu(tr.ts0[:n0]), cpu(tr.te0[:n0])
    vis, _ = OR.cull(fld, cpu(tr.packed0), ri0, ts0, te0, cpu(tr.ro_c), cpu(tr.rd_c), var_ref.detach())
    gpu_vis = cpu(tr.vis[:n0]).astype(bool)
    assert (vis != gpu_vis).mean() < 2e-3
    pidx, ts, te = cpu(tr.ridx1[:S]), cpu(tr.ts1[:S]), cpu(tr.te1[:S])
    q1 = int(tr.q1.item())
    ref = OR.patch_forward(device_valued(fld, net, tr.xyz1[:q1]), pidx, ts, te, cpu(ro), cpu(rd),
                           cpu(pn), cpu(vinv), var_ref, points=cpu(tr.xyz1[:q1]),
                           gradient_method=method)
    Lr = OR.losses(ref["comp_normal"], ref["weight_sum"], ref["gradients"], cpu(nrm), cpu(mask))
    lo = cpu(tr.loss_out)
    for i, k in ((1, "normal"), (2, "mask"), (3, "eikonal"), (4, "total")):
        assert abs(lo[i] - Lr[k].item()) <= 1e-4 * max(abs(Lr[k].item()), 1e-6), (k, lo[i], Lr[k].item())
    names = ["table", "v0", "g0", "b0", "v1", "g1", "b1"]
    rgrads = torch.autograd.grad(Lr["total"], [prm[n] for n in names] + [var_ref])
    rg = dict(zip(names + ["variance"], rgrads))
    errs = {}
    for n, r in rg.items():
        got = cpu(tr.gviews[n])
        errs[n] = grad_err(n, got, r.numpy().reshape(got.shape))
        if n == "table":
            errs["table_levels"] = _table_level_errors(net, got, r.numpy())
        if n in ("g0", "g1"):
            errs[n] = weight_g_err(got, r, prm["v" + n[1]], prm[n], rg["v" + n[1]])
    for n in names + ["variance"]:
        assert errs[n] < table_tol if n == "table" else errs[n] < 2e-3, (n, errs)
    return errs


def weight_g_err(got, ref_g, v, g, ref_v):
    """Error of d L / d g of a weight-normed layer (w_o = g_o v_o / |v_o|)
    relative to the size of the effective-weight gradient it is a projection
    of: d L / d g_o = <d L / d w_o, v_o / |v_o|> can cancel far below
    |d L / d w_o|, and the float32 atomics sums of d L / d w are accurate to a
    fraction of |d L / d w|, not of their projection.  |d L / d w_o|^2 =
    (|v_o| / g_o)^2 |d L / d v_o|^2 + (d L / d g_o)^2 (the two are orthogonal)."""
    v, g = v.detach().double(), g.detach().double().reshape(-1)
    rv, rgg = ref_v.detach().double(), ref_g.detach().double().reshape(-1)
    nv = v.norm(dim=1)
    dw = torch.sqrt((nv / g) ** 2 * rv.pow(2).sum(1) + rgg ** 2)
    diff = np.abs(np.asarray(got, np.float64).reshape(-1) - rgg.numpy())
    return float(diff.max() / max(float(dw.max()), 1e-30))


def _table_level_errors(net, got, ref):
    """Per-level ||got - ref|| / ||ref|| of the hash-table gradient (F = 2)."""
    off = net.encoding.level_offsets() * 2
    out = []
    for l in range(len(off) - 1):
        a, b = got[off[l]:off[l + 1]].astype(np.float64), ref[off[l]:off[l + 1]]
        out.append(float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)))
    return out


@pytest.mark.parametrize("method", ["dfd", "ad"])
def test_trainer_loss_and_grads_match_oracle(scene, method):
    tr, net, var = _trainer(scene, gradient_method=method)
    g = torch.Generator(device="cuda").manual_seed(5)
    _check_trainer_step(tr, net, var, scene.gen_random_patches(128, generator=g), method, 300)


@pytest.mark.parametrize("method", ["dfd", "ad"])
def test_trainer_step_at_benchmark_shapes_matches_oracle(built_lib, method):
    """The benchmark's configuration: displaced torus seen by 612x512 views on
    an elevated ring, hash grid 16 levels x 2 features x 2^19 entries, MLP
    35 -> 64 -> 16, 128^3 occupancy grid (warm-up sweep, then updates every 8
    iterations), marching step 2/1024, FP32, here 256 patches.  After 24
    training iterations from the benchmark's initialisation, one iteration
    against the oracle on the kept samples; 'ad' takes the normals' gradients
    from SDFNetwork.gradient, so the tensor-core gradient forward and
    second-order adjoint run at these sizes too."""
    from supernormal_gb300 import scenes
    from supernormal_gb300.fields import SDFNetwork, SingleVarianceNetwork
    from supernormal_gb300.trainer import FusedTrainer, TrainConfig

    enc = dict(otype="HashGrid", n_levels=16, n_features_per_level=2, log2_hashmap_size=19,
               base_resolution=16, per_level_scale=1.447)
    rig = scenes.ring_cameras(4, 512, 612, radius=3.0, elevation_deg=30.0, fov_deg=40.0)
    ds = scenes.SyntheticDataset(scenes.displaced_torus(0.5, 0.2, 0.02, 20.0), rig, torch.device("cuda"))
    torch.manual_seed(1234)
    net = SDFNetwork(3, 16, 64, 1, skip_in=(-1,), bias=0.5, encoding_config=enc, input_concat=True).cuda()
    var = SingleVarianceNetwork(0.5).cuda()
    net.bindwidth = 16
    cfg = TrainConfig(batch_size=256, step_size=2.0 / 1024, occ_update_freq=8, occ_threshold=0.1,
                      increase_bandwidth_every=0, end_iter=5000, gradient_method=method)
    tr = FusedTrainer(net, var, cfg)
    g = torch.Generator(device="cuda").manual_seed(21)
    for _ in range(24):
        tr.train_step(*ds.gen_random_patches(256, generator=g))
    tr.check_status()
    _check_trainer_step(tr, net, var, ds.gen_random_patches(256, generator=g), method, 256 * 8)


def test_adam_matches_torch(built_lib):
    from supernormal_gb300._lib import call, stream_handle

    n = 4099
    p = torch.randn(n, device="cuda")
    g = torch.randn(n, device="cuda")
    pt = p.clone().requires_grad_(True)
    opt = torch.optim.Adam([pt], lr=1e-3)
    m = torch.zeros(n, device="cuda")
    v = torch.zeros(n, device="cuda")
    buf = torch.zeros(4 * ((n + 3) // 4), device="cuda")
    mine = buf[:n]
    mine.copy_(p)
    mb = torch.zeros_like(buf)
    vb = torch.zeros_like(buf)
    gbuf = torch.zeros_like(buf)
    for step in range(1, 4):
        gg = g * step
        pt.grad = gg.clone()
        opt.step()
        gbuf[:n] = gg
        call("sn_adam_step", n, mine, gbuf, mb, vb, None, None, None, 1e-3, step, 0.9, 0.999, 1e-8, 1,
             stream_handle())
        assert (gbuf == 0).all()
    torch.testing.assert_close(mine, pt.detach(), rtol=1e-5, atol=1e-7)


def test_training_reduces_loss(scene):
    tr, net, var = _trainer(scene, B=256, learning_rate=5e-3, warm_up_end=2, end_iter=200)
    g = torch.Generator(device="cuda").manual_seed(9)
    first = last = None
    for it in range(60):
        batch = scene.gen_random_patches(256, generator=g)
        loss = tr.train_step(*batch)
        v = float(loss[4].item())
        if it < 5:
            first = v if first is None else min(first, v)
        last = v
    tr.check_status()
    assert np.isfinite(last) and last < first


def test_render_with_no_samples_returns_zeros(scene):
    """An empty occupancy grid marches no sample: the culling callback gets
    empty tensors and the render is all zeros (the reference's torch ops
    accept the empty case too)."""
    from supernormal_gb300.renderer import NeuSRenderer, near_far_from_sphere

    net, var = make()
    r = NeuSRenderer(net, var)
    r.occupancy_grid = full_grid()
    r.occupancy_grid._binary.zero_()
    g = torch.Generator(device="cuda").manual_seed(4)
    ro, rd, pn, vinv, _, _ = scene.gen_random_patches(16, generator=g)
    near, far = near_far_from_sphere(ro[:, 1, 1], rd[:, 1, 1])
    out = r.render(ro, rd, pn, near, far, vinv, mode="eval")
    assert out["gradients"] is None
    assert torch.count_nonzero(out["comp_normal"]) == 0 and torch.count_nonzero(out["weight_sum"]) == 0


def test_render_normal_pixel_based_matches_oracle(scene):
    """NeuSRenderer.render_normal_pixel_based (models/renderer.py:278-351) on a
    view's pixel rays: normals and depths against the float64 oracle on the
    samples the marcher kept (early stop 1e-3)."""
    from supernormal_gb300 import scenes
    from supernormal_gb300.renderer import NeuSRenderer, near_far_from_sphere

    net, var = make(d_out=1)
    r = NeuSRenderer(net, var)
    r.occupancy_grid = full_grid()
    r.sampling_step_size = 1.0 / 96
    d, _ = scenes.view_rays(scene.rig, 1, torch.device("cuda"))
    rd = d[::3, ::3].reshape(-1, 3).contiguous()
    ro = scene.pose_all[1, :3, 3].expand(rd.shape).contiguous()
    near, far = near_far_from_sphere(ro, rd)
    g = torch.Generator(device="cuda").manual_seed(8)
    comp, depth = r.render_normal_pixel_based(ro, rd, near, far, generator=g)
    ridx, ts, te = (cpu(t) for t in r.last_samples)
    assert ridx.size > 500 and comp.shape == (rd.shape[0], 3) and depth.shape == (rd.shape[0], 1)
    _, fld = oracle_field(net)
    ref_c, ref_d, parts = OR.pixel_forward(fld, ridx, ts, te, cpu(ro), cpu(rd), var.variance.detach().cpu(),
                                           rd.shape[0])
    # the pieces: alpha of the same alpha_fn, weights, gradients at the midpoints
    ri_t = r.last_samples[0]
    alpha = r._center_alpha_fn(ro, rd)(r.last_samples[1], r.last_samples[2], ri_t)
    mid = (r.last_samples[1] + r.last_samples[2]) / 2.0
    grads = net.gradient(ro[ri_t] + rd[ri_t] * mid).reshape(-1, 3).detach()
    errs = {"alpha": np.abs(cpu(alpha).ravel() - parts["alpha"]).max(),
            "gradients": np.abs(cpu(grads) - parts["gradients"].numpy()).max() / np.abs(parts["gradients"].numpy()).max(),
            "normal": np.abs(cpu(comp) - ref_c.numpy()).max(), "depth": np.abs(cpu(depth) - ref_d.numpy()).max()}
    assert errs["alpha"] < 1e-5 and errs["gradients"] < 1e-5, errs
    assert errs["normal"] < 2e-4 * max(1.0, np.abs(ref_c.numpy()).max()) and errs["depth"] < 2e-4, errs
    assert (cpu(depth)[:, 0] > 0).sum() > 20
