"""GPU parity of the hash-grid field (fused encoding + MLP) against the float64 oracle.

Tolerances (float32 kernels vs float64 oracle): encoding 1e-6 relative to the
table scale; SDF values 2e-5 absolute; parameter gradients 1e-3 relative to
each gradient's max-abs (atomics reorder float32 sums)."""
import numpy as np
import pytest
import torch

from oracle import field as OF

pytestmark = pytest.mark.gpu

ENC1 = dict(otype="HashGrid", n_levels=16, n_features_per_level=2, log2_hashmap_size=15,
            base_resolution=16, per_level_scale=1.447)
ENC2 = dict(ENC1, log2_hashmap_size=19)
ENC_SHIPPED = dict(otype="HashGrid", n_levels=14, n_features_per_level=2, log2_hashmap_size=19,
                   base_resolution=32, per_level_scale=1.3195079107728942)


def make_net(enc, d_out=16, seed=0, table_scale=1.0):
    from supernormal_gb300.fields import SDFNetwork

    torch.manual_seed(seed)
    net = SDFNetwork(3, d_out, 64, 1, skip_in=(-1,), bias=0.5, encoding_config=enc, input_concat=True)
    with torch.no_grad():
        # table scaled up from the 1e-4 init so the encoding matters in the checks
        net.encoding.params.mul_(table_scale)
        net.lin0.weight_v[:, 3:].normal_(0.0, 0.3)
    return net.cuda()


def rel_err(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-30)


@pytest.mark.parametrize("enc", [ENC1, ENC2, ENC_SHIPPED])
def test_encoding_matches_oracle(built_lib, enc):
    net = make_net(enc, table_scale=1e3)
    x = (torch.rand((4096, 3), device="cuda") * 2.2 - 1.1)   # SuperNormal feeds [-1,1] (and a bit beyond)
    out = net.encoding(x).detach().cpu().numpy()
    ref = OF.encode(x.cpu(), net.encoding.params.detach().cpu(), OF.geometry_from_module(net)).numpy()
    assert rel_err(out, ref) < 1e-6


def test_encoding_active_levels_zero_tail(built_lib):
    net = make_net(ENC1, table_scale=1e3)
    x = torch.rand((512, 3), device="cuda") * 2 - 1
    out = net.encoding(x, active_levels=5).detach().cpu().numpy()
    assert (out[:, 10:] == 0).all() and np.abs(out[:, :10]).max() > 0


@pytest.mark.parametrize("enc,d_out,active", [(ENC1, 16, 16), (ENC1, 1, 7), (ENC2, 16, 3),
                                             (ENC_SHIPPED, 1, 14)])
def test_field_forward_matches_oracle(built_lib, enc, d_out, active):
    net = make_net(enc, d_out=d_out, table_scale=1e3)
    net.bindwidth = active
    x = torch.rand((3000, 3), device="cuda") * 2 - 1
    y = net(x).detach().cpu().numpy()
    prm = OF.params_from_module(net)
    ref = OF.sdf_network(x.cpu(), **prm, geom=OF.geometry_from_module(net), active_levels=active)
    np.testing.assert_allclose(y, ref.detach().numpy(), atol=2e-5)
    s = net.sdf(x).detach().cpu().numpy()
    np.testing.assert_allclose(s, ref.detach().numpy()[:, :1], atol=2e-5)


@pytest.mark.parametrize("enc,d_out,active,cols", [(ENC1, 16, 16, "all"), (ENC1, 16, 9, "sdf"),
                                                  (ENC_SHIPPED, 1, 14, "all")])
def test_field_backward_matches_oracle(built_lib, enc, d_out, active, cols):
    net = make_net(enc, d_out=d_out, table_scale=1e3)
    net.bindwidth = active
    x = (torch.rand((2000, 3), device="cuda") * 2 - 1).requires_grad_(True)
    y = net(x) if cols == "all" else net.sdf(x)
    gy = torch.randn_like(y)
    params = [net.encoding.params, net.lin0.weight_v, net.lin0.weight_g, net.lin0.bias,
              net.lin1.weight_v, net.lin1.weight_g, net.lin1.bias]
    grads = torch.autograd.grad(y, params + [x], gy)
    prm = OF.params_from_module(net)
    xr = x.detach().cpu().double().requires_grad_(True)
    ref = OF.sdf_network(xr, **prm, geom=OF.geometry_from_module(net), active_levels=active,
                         out_cols=None if cols == "all" else 1)
    names = ["table", "v0", "g0", "b0", "v1", "g1", "b1"]
    rgrads = torch.autograd.grad(ref, [prm[n] for n in names] + [xr], gy.cpu().double())
    for n, g, r in zip(names + ["x"], grads, rgrads):
        assert rel_err(g.cpu().numpy(), r.numpy()) < 1e-3, n


@pytest.mark.parametrize("enc,d_out,active,count,flags", [(ENC1, 1, 16, None, 0), (ENC_SHIPPED, 1, 9, 1700, 0),
                                                          (ENC2, 1, 16, 0, 0), (ENC1, 16, 12, 2100, 0),
                                                          (ENC1, 1, 16, 2300, 3)])
def test_encoding_cache_gives_the_recomputed_backward(built_lib, enc, d_out, active, count, flags):
    """sn_field_fwd with an encoding cache writes the encoding of its points
    (level-major) and nothing else; sn_field_bwd reading it gives the
    recomputing backward's gradients (atomics order aside)."""
    import ctypes as C

    from supernormal_gb300._lib import call, stream_handle

    net = make_net(enc, d_out=d_out, table_scale=1e3)
    n, L = 2500, net.encoding.n_levels
    x = torch.rand((n, 3), device="cuda") * 2 - 1
    cnt = None if count is None else torch.tensor([count], dtype=torch.int32, device="cuda")
    m = n if count is None else count
    w0, b0, w1, b1 = (t.detach().contiguous() for t in net.mlp_tensors())
    table32 = net.encoding.params.detach()
    table = table32.half().contiguous() if flags & 1 else table32
    cache = torch.full((L * 2 * n,), float("nan"), device="cuda")
    cached, plain = net._mlp_desc(w0, b0, w1, b1), net._mlp_desc(w0, b0, w1, b1)
    cached.flags = plain.flags = flags
    cached.enc_cache = cache.data_ptr()
    gd, st = C.byref(net.encoding.desc), stream_handle()
    out_c, out_p = torch.zeros((n, d_out), device="cuda"), torch.zeros((n, d_out), device="cuda")
    call("sn_field_fwd", n, cnt, x, table, gd, active, C.byref(cached), d_out, out_c, st)
    call("sn_field_fwd", n, cnt, x, table, gd, active, C.byref(plain), d_out, out_p, st)
    assert torch.equal(out_c, out_p)
    c3 = cache.view(L, n, 2)
    assert torch.isnan(c3[active:]).all() and torch.isnan(c3[:, m:]).all()   # nothing else written
    if m:
        ref = net.encoding(x, active_levels=active).detach()
        if flags & 1:   # FP16 table: the oracle encoding of the rounded table
            ref = torch.from_numpy(OF.encode(x.cpu(), table.float().cpu(), OF.geometry_from_module(net)).numpy())
            ref[:, 2 * active:] = 0
            ref = ref.cuda().float()
        got = c3[:active, :m].permute(1, 0, 2).reshape(m, 2 * active)
        assert rel_err(got.cpu(), ref[:m, :2 * active].cpu()) < 1e-6
    go = torch.randn((n, d_out), device="cuda")
    cache_fwd = cache.clone()

    def bwd(desc, with_x):
        gs = [torch.zeros_like(table32), torch.zeros_like(w0), torch.zeros_like(b0), torch.zeros_like(w1),
              torch.zeros_like(b1), torch.zeros_like(x) if with_x else None]
        call("sn_field_bwd", n, cnt, x, go, d_out, table, gd, active, C.byref(desc), *gs, st)
        return [t for t in gs if t is not None]

    # with and without grad_x (the table gradient alone is the training call)
    for with_x in (True, False):
        cache.copy_(cache_fwd)
        for u, v in zip(bwd(cached, with_x), bwd(plain, with_x)):
            assert torch.isfinite(u).all()
            scale = max(float(v.abs().max()), 1e-30)
            assert float((u - v).abs().max()) <= 1e-5 * scale, with_x


@pytest.mark.parametrize("spread", [1e-3, 3e-2])
def test_field_backward_clustered_points(built_lib, spread):
    """Warps of 32 neighbouring points (as a patch's samples are): coarse levels
    put a whole warp in one cell, which takes the shuffle-reduced scatter."""
    net = make_net(ENC1, d_out=16, table_scale=1e3)
    net.bindwidth = 16
    g = torch.Generator(device="cuda").manual_seed(5)
    centres = torch.rand((70, 1, 3), device="cuda", generator=g) * 1.6 - 0.8
    x = (centres + spread * torch.randn((70, 32, 3), device="cuda", generator=g)).reshape(-1, 3)
    x = x[:2221].contiguous().requires_grad_(True)       # ragged last warp
    y = net(x)
    gy = torch.randn_like(y)
    params = [net.encoding.params, net.lin0.weight_v, net.lin0.weight_g, net.lin0.bias,
              net.lin1.weight_v, net.lin1.weight_g, net.lin1.bias]
    grads = torch.autograd.grad(y, params + [x], gy)
    prm = OF.params_from_module(net)
    xr = x.detach().cpu().double().requires_grad_(True)
    ref = OF.sdf_network(xr, **prm, geom=OF.geometry_from_module(net), active_levels=16)
    names = ["table", "v0", "g0", "b0", "v1", "g1", "b1"]
    rgrads = torch.autograd.grad(ref, [prm[n] for n in names] + [xr], gy.cpu().double())
    for n, gd, r in zip(names + ["x"], grads, rgrads):
        assert rel_err(gd.cpu().numpy(), r.numpy()) < 1e-3, n


@pytest.mark.parametrize("enc,active", [(ENC1, 16), (ENC_SHIPPED, 9)])
def test_gradient_and_second_order_adjoint_match_oracle(built_lib, enc, active):
    net = make_net(enc, d_out=16, table_scale=1e3)
    net.bindwidth = active
    x = torch.rand((1500, 3), device="cuda") * 2 - 1
    sdf, grad = net.sdf_and_gradient(x)
    prm = OF.params_from_module(net)
    xr = x.cpu().double().requires_grad_(True)
    s_ref = OF.sdf_network(xr, **prm, geom=OF.geometry_from_module(net), active_levels=active, out_cols=1)
    (g_ref,) = torch.autograd.grad(s_ref.sum(), xr, create_graph=True)
    np.testing.assert_allclose(sdf.detach().cpu().numpy(), s_ref.detach().numpy(), atol=2e-5)
    assert rel_err(grad.detach().cpu().numpy(), g_ref.detach().numpy()) < 1e-4
    gg = torch.randn_like(grad)
    gs = torch.randn_like(sdf)
    params = [net.encoding.params, net.lin0.weight_v, net.lin0.weight_g, net.lin0.bias,
              net.lin1.weight_v, net.lin1.weight_g, net.lin1.bias]
    grads = torch.autograd.grad((grad * gg).sum() + (sdf * gs).sum(), params, allow_unused=True)
    names = ["table", "v0", "g0", "b0", "v1", "g1", "b1"]
    obj = (g_ref * gg.cpu().double()).sum() + (s_ref * gs.cpu().double()).sum()
    rgrads = torch.autograd.grad(obj, [prm[n] for n in names], allow_unused=True)
    for n, g, r in zip(names, grads, rgrads):
        g = np.zeros(prm[n].shape) if g is None else g.cpu().numpy()
        r = np.zeros(prm[n].shape) if r is None else r.numpy()
        err = (np.linalg.norm(g - r) / max(np.linalg.norm(r), 1e-30)) if n == "table" else rel_err(g, r)
        assert err < 2e-3, (n, err)


def test_second_order_adjoint_vs_central_differences(built_lib):
    """Config-4 style check: d/dtheta of L = <gamma, grad_x sdf> against float64
    central differences (h = 1e-4) of the oracle on 512 random parameters."""
    enc = dict(ENC1, log2_hashmap_size=17)
    net = make_net(enc, d_out=16, table_scale=1e3)
    net.bindwidth = 16
    x = torch.rand((64 * 9, 3), device="cuda") * 2 - 1
    gamma = torch.randn((x.shape[0], 3), device="cuda")
    _, grad = net.sdf_and_gradient(x)
    names = ["table", "v0", "g0", "b0", "v1", "g1", "b1"]
    params = [net.encoding.params, net.lin0.weight_v, net.lin0.weight_g, net.lin0.bias,
              net.lin1.weight_v, net.lin1.weight_g, net.lin1.bias]
    grads = torch.autograd.grad((grad * gamma).sum(), params, allow_unused=True)
    prm = {k: v.detach() for k, v in OF.params_from_module(net).items()}
    geom = OF.geometry_from_module(net)
    xr = x.cpu().double()
    gam = gamma.cpu().double()
    cache = {}

    def objective(p):
        xx = xr.clone().requires_grad_(True)
        s = OF.sdf_network(xx, **p, geom=geom, active_levels=16, out_cols=1, cache=cache)
        (gx,) = torch.autograd.grad(s.sum(), xx)
        return float((gx * gam).sum())

    rng = np.random.default_rng(0)
    # parameters that matter: table entries touched by the points + all MLP weights
    touched = np.unique(np.concatenate([OF.corner_indices(x.cpu().numpy(), l, *geom)[2].ravel()
                                        for l in range(16)]))
    picks = []
    for _ in range(512):
        n = names[rng.integers(0, 6)] if rng.random() < 0.5 else "table"
        if n == "table":
            e = int(rng.choice(touched))
            picks.append((n, 2 * e + int(rng.integers(0, 2))))
        else:
            picks.append((n, int(rng.integers(0, prm[n].numel()))))
    h = 1e-4
    errs = []
    for n, i in picks:
        p_plus = dict(prm)
        p_minus = dict(prm)
        t = prm[n].clone().reshape(-1)
        t[i] += h
        p_plus[n] = t.reshape(prm[n].shape)
        t2 = prm[n].clone().reshape(-1)
        t2[i] -= h
        p_minus[n] = t2.reshape(prm[n].shape)
        fd = (objective(p_plus) - objective(p_minus)) / (2 * h)
        g = grads[names.index(n)]
        got = 0.0 if g is None else float(g.reshape(-1)[i])
        errs.append((abs(got - fd), abs(fd)))
    errs = np.array(errs)
    scale = max(errs[:, 1].max(), 1e-12)
    assert (errs[:, 0] <= 2e-3 * scale + 1e-3 * errs[:, 1]).all(), errs[:, 0].max() / scale


def test_gradient_matches_reference_fixture(built_lib):
    from pathlib import Path

    d = np.load(Path(__file__).parent / "golden" / "reference_field.npz")
    from supernormal_gb300.fields import SDFNetwork

    L, F, T, base, s = d["enc"]
    enc = dict(otype="HashGrid", n_levels=int(L), n_features_per_level=int(F),
               log2_hashmap_size=int(T), base_resolution=int(base), per_level_scale=float(s))
    net = SDFNetwork(3, 16, 64, 1, skip_in=(-1,), bias=0.5, encoding_config=enc, input_concat=True)
    net.load_state_dict({k[6:]: torch.from_numpy(d[k]).float() for k in d.files if k.startswith("param/")})
    net.bindwidth = int(d["bindwidth"])
    net = net.cuda()
    x = torch.from_numpy(d["x"]).float().cuda()
    g = net.gradient(x)
    assert rel_err(g.detach().cpu().numpy(), d["gradient"]) < 1e-4
    names = [str(n) for n in d["param_names"]]
    params = dict(net.named_parameters())
    grads = torch.autograd.grad((g * torch.from_numpy(d["g_grad"]).float().cuda()).sum(),
                                [params[n] for n in names], allow_unused=True)
    for n, gr in zip(names, grads):
        ref = d[f"grad2/{n}"]
        got = np.zeros_like(ref) if gr is None else gr.cpu().numpy()
        if np.abs(ref).max() == 0:
            assert np.abs(got).max() == 0, n
            continue
        err = (np.linalg.norm(got - ref) / np.linalg.norm(ref)) if n == "encoding.params" else rel_err(got, ref)
        assert err < 2e-3, (n, err)


def test_weightnorm_matches_torch(built_lib):
    from supernormal_gb300.fields import _WeightNorm

    v = torch.randn((64, 35), device="cuda", requires_grad=True)
    g = torch.rand((64, 1), device="cuda", requires_grad=True)
    w = _WeightNorm.apply(v, g)
    wr = g * v / v.norm(dim=1, keepdim=True)
    torch.testing.assert_close(w, wr, rtol=1e-6, atol=1e-6)
    gw = torch.randn_like(w)
    gv, gg = torch.autograd.grad(w, [v, g], gw)
    gvr, ggr = torch.autograd.grad(wr, [v, g], gw)
    torch.testing.assert_close(gv, gvr, rtol=1e-5, atol=1e-5)
    torch.testing.assert_close(gg, ggr, rtol=1e-5, atol=1e-5)


def test_state_dict_keys_match_reference(built_lib):
    net = make_net(ENC_SHIPPED, d_out=1)
    keys = set(net.state_dict().keys())
    assert keys == {"encoding.params", "lin0.bias", "lin0.weight_g", "lin0.weight_v",
                    "lin1.bias", "lin1.weight_g", "lin1.weight_v"}
    assert net.encoding.params.numel() == int(OF.grid_geometry(14, 2, 19, 32, 1.3195079107728942)[0][-1]) * 2


@pytest.mark.parametrize("d_out,active", [(1, 16), (16, 11)])
def test_bf16_first_layer_forward(built_lib, d_out, active):
    """SN_FIELD_MLP_BF16 (forward only): the first layer's inputs and W0 are
    rounded to BF16 (round to nearest even) and their products accumulated in
    FP32 on the tensor cores.  Checked against that arithmetic emulated in
    float64 from the same rounded operands; the backward entry points reject
    the flag."""
    import ctypes as C

    from supernormal_gb300._lib import SN_ERR_UNSUPPORTED, SN_FIELD_MLP_BF16, SupernormalError, call, stream_handle

    net = make_net(ENC1, d_out=d_out, table_scale=1e3)
    n = 3000
    x = torch.rand((n, 3), device="cuda") * 2 - 1
    w0, b0, w1, b1 = (t.detach().contiguous() for t in net.mlp_tensors())
    desc = net._mlp_desc(w0, b0, w1, b1)
    desc.flags = SN_FIELD_MLP_BF16
    gd, st = C.byref(net.encoding.desc), stream_handle()
    table = net.encoding.params.detach()
    out = torch.zeros((n, d_out), device="cuda")
    call("sn_field_fwd", n, None, x, table, gd, active, C.byref(desc), d_out, out, st)
    enc = net.encoding(x, active_levels=active).detach()
    inp = torch.cat([x, enc], 1).to(torch.bfloat16).double()
    h = inp @ w0.to(torch.bfloat16).double().t() + b0.double()
    ref = torch.nn.functional.softplus(h, beta=100.0, threshold=20.0) @ w1.double().t() + b1.double()
    err = (out.double() - ref).abs().max().item()
    assert err < 2e-5 * max(1.0, ref.abs().max().item()), err
    # the rounding is visible: BF16 differs from the FP32-accurate forward
    plain = net._mlp_desc(w0, b0, w1, b1)
    out32 = torch.zeros_like(out)
    call("sn_field_fwd", n, None, x, table, gd, active, C.byref(plain), d_out, out32, st)
    assert (out - out32).abs().max().item() > 1e-5
    go = torch.ones_like(out)
    with pytest.raises(SupernormalError) as e:
        call("sn_field_bwd", n, None, x, go, d_out, table, gd, active, C.byref(desc), torch.zeros_like(table),
             None, None, None, None, None, st)
    assert e.value.status == SN_ERR_UNSUPPORTED


@pytest.mark.parametrize("count", [700, 0])
def test_gradient_kernels_bounded_by_device_count(built_lib, count):
    """sn_field_grad_fwd / sn_field_grad_bwd with a device count below the
    capacity (a graph-captured step's live points): outputs past the count are
    not written, and the parameter gradients are those of the first `count`
    points alone (atomics order aside); a count of 0 writes and adds nothing."""
    import ctypes as C

    from supernormal_gb300._lib import call, stream_handle

    net = make_net(ENC1, d_out=16, table_scale=1e3)
    cap, active = 1500, 16
    x = torch.rand((cap, 3), device="cuda") * 2 - 1
    w0, b0, w1, b1 = (t.detach().contiguous() for t in net.mlp_tensors())
    desc = net._mlp_desc(w0, b0, w1, b1)
    gd, st = C.byref(net.encoding.desc), stream_handle()
    table = net.encoding.params.detach()
    cnt = torch.tensor([count], dtype=torch.int32, device="cuda")
    sdf = torch.full((cap,), float("nan"), device="cuda")
    grad = torch.full((cap, 3), float("nan"), device="cuda")
    call("sn_field_grad_fwd", cap, cnt, x, table, gd, active, C.byref(desc), sdf, grad, st)
    sdf_n = torch.empty((max(count, 1),), device="cuda")
    grad_n = torch.empty((max(count, 1), 3), device="cuda")
    if count:
        call("sn_field_grad_fwd", count, None, x[:count].contiguous(), table, gd, active, C.byref(desc),
             sdf_n, grad_n, st)
    torch.cuda.synchronize()
    assert torch.isnan(sdf[count:]).all() and torch.isnan(grad[count:]).all()
    if count:
        assert torch.equal(sdf[:count], sdf_n) and torch.equal(grad[:count], grad_n)
    gamma = torch.randn((cap, 3), device="cuda")
    rho = torch.randn((cap,), device="cuda")

    def bwd(n, counter):
        gs = [torch.zeros_like(table), torch.zeros_like(w0), torch.zeros_like(b0), torch.zeros_like(w1),
              torch.zeros_like(b1)]
        call("sn_field_grad_bwd", n, counter, x[:n].contiguous(), gamma[:n].contiguous(), rho[:n].contiguous(),
             table, gd, active, C.byref(desc), *gs, st)
        return gs

    got = bwd(cap, cnt)
    torch.cuda.synchronize()
    if count == 0:
        assert all(float(t.abs().max()) == 0.0 for t in got)
        return
    want = bwd(count, None)
    torch.cuda.synchronize()
    for u, v in zip(got, want):
        scale = max(float(v.abs().max()), 1e-30)
        assert float((u - v).abs().max()) <= 1e-5 * scale


def test_field_batch_skips_empty_segments(built_lib):
    """sn_field_fwd_batch with a zero-point segment between two others: the
    others' outputs are their own sn_field_fwd launches' bit for bit."""
    import ctypes as C

    from supernormal_gb300._lib import FieldSegment, call, stream_handle

    nets = [make_net(ENC1, d_out=1, seed=s, table_scale=1e3) for s in (0, 1, 2)]
    ns = [1300, 0, 517]
    xs = [torch.rand((max(n, 1), 3), device="cuda") * 2 - 1 for n in ns]
    st = stream_handle()
    keep, segs, outs, want = [], (FieldSegment * 3)(), [], []
    for k, (net, n, x) in enumerate(zip(nets, ns, xs)):
        w0, b0, w1, b1 = (t.detach().contiguous() for t in net.mlp_tensors())
        d = net._mlp_desc(w0, b0, w1, b1)
        keep.append((w0, b0, w1, b1, d))
        out = torch.full((max(n, 1), 1), float("nan"), device="cuda")
        outs.append(out)
        segs[k] = FieldSegment(n, x.data_ptr(), net.encoding.params.data_ptr(), C.pointer(net.encoding.desc),
                               16, C.pointer(d), out.data_ptr())
        ref = torch.zeros((max(n, 1), 1), device="cuda")
        if n:
            call("sn_field_fwd", n, None, x, net.encoding.params.detach(), C.byref(net.encoding.desc), 16,
                 C.byref(d), 1, ref, st)
        want.append(ref)
    call("sn_field_fwd_batch", 3, segs, 1, st)
    torch.cuda.synchronize()
    assert torch.equal(outs[0], want[0]) and torch.equal(outs[2], want[2])
    assert torch.isnan(outs[1]).all()


def test_bounded_wait_reports_timeout_and_the_context_survives(built_lib):
    """The failure path of the tensor-core field kernels, without a GPU fault:
    a bounded mbarrier wait on a barrier that nothing arrives at gives up,
    SN_STATUS_TIMEOUT reaches the status word, and the context keeps working.
    The time per poll bounds how long the kernels' own limit lets a stuck MMA
    wait before they report it."""
    import ctypes as C

    from supernormal_gb300._lib import SN_STATUS_TIMEOUT, call, lib, stream_handle

    st = stream_handle()
    polls = 1 << 12
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    call("sn_selftest_bounded_wait", polls, status, st)
    e1.record()
    torch.cuda.synchronize()
    assert int(status.item()) & SN_STATUS_TIMEOUT
    ms = e0.elapsed_time(e1)
    limit = int(lib().sn_bounded_wait_polls())
    print(f"bounded wait: {polls} polls in {ms:.3f} ms; the kernels' limit of {limit} polls ~ {ms * limit / polls / 1e3:.2f} s")
    assert ms * limit / polls < 3_000.0        # the kernels give up within a few seconds
    # the context is intact: a field forward afterwards gives the oracle's values
    net = make_net(ENC1, d_out=1, table_scale=1e3)
    x = torch.rand((777, 3), device="cuda") * 2 - 1
    w0, b0, w1, b1 = (t.detach().contiguous() for t in net.mlp_tensors())
    d = net._mlp_desc(w0, b0, w1, b1)
    out = torch.zeros((777, 1), device="cuda")
    call("sn_field_fwd", 777, None, x, net.encoding.params.detach(), C.byref(net.encoding.desc), 16, C.byref(d), 1,
         out, st)
    prm = OF.params_from_module(net)
    ref = OF.sdf_network(x.cpu().double(), **prm, geom=OF.geometry_from_module(net), active_levels=16, out_cols=1)
    assert np.abs(out.cpu().numpy() - ref.detach().numpy()).max() < 2e-5
