"""The oracle against fixtures produced by the reference's own Python (CPU).

tests/golden/make_golden.py ran models/fields.py and models/renderer.py (with
tiny-cuda-nn / nerfacc replaced by oracle restatements) and stored inputs,
outputs, losses and gradients.  Here the standalone oracle reproduces them,
which pins oracle.field's MLP / weight-norm / bandwidth handling / gradient()
and oracle.renderer's patch math and losses to the reference code.  The
reference casts the encoding to float32 (models/fields.py:26,78), hence the
1e-6-level tolerances."""
from pathlib import Path

import numpy as np
import torch

from oracle import field as OF
from oracle import nerfacc_ref as NR
from oracle import renderer as OR

G = Path(__file__).parent / "golden"


def _params(d):
    t = lambda k: torch.from_numpy(d[f"param/{k}"]).double().requires_grad_(True)
    return dict(table=t("encoding.params"), v0=t("lin0.weight_v"), g0=t("lin0.weight_g"),
                b0=t("lin0.bias"), v1=t("lin1.weight_v"), g1=t("lin1.weight_g"), b1=t("lin1.bias"))


NAME = {"encoding.params": "table", "lin0.weight_v": "v0", "lin0.weight_g": "g0", "lin0.bias": "b0",
        "lin1.weight_v": "v1", "lin1.weight_g": "g1", "lin1.bias": "b1"}


def _geom(d):
    L, F, T, base, s = d["enc"]
    return OF.grid_geometry(int(L), int(F), int(T), int(base), float(s))


def rel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-30)


def test_field_forward_and_grads_match_reference_code():
    d = np.load(G / "reference_field.npz")
    prm = _params(d)
    geom = _geom(d)
    x = torch.from_numpy(d["x"]).double()
    y = OF.sdf_network(x, **prm, geom=geom, active_levels=int(d["bindwidth"]))
    assert rel(y.detach().numpy(), d["y"]) < 2e-6
    grads = torch.autograd.grad((y * torch.from_numpy(d["g_out"])).sum(), list(prm.values()))
    for n, g in zip(prm, grads):
        key = [k for k, v in NAME.items() if v == n][0]
        assert rel(g.numpy(), d[f"grad/{key}"]) < 2e-6, n


def test_field_gradient_and_second_order_match_reference_code():
    d = np.load(G / "reference_field.npz")
    prm = _params(d)
    geom = _geom(d)
    x = torch.from_numpy(d["x"]).double().requires_grad_(True)
    s = OF.sdf_network(x, **prm, geom=geom, active_levels=int(d["bindwidth"]), out_cols=1)
    (gx,) = torch.autograd.grad(s.sum(), x, create_graph=True)
    assert rel(gx.detach().numpy(), d["gradient"][:, 0, :]) < 2e-6
    g2 = torch.autograd.grad((gx * torch.from_numpy(d["g_grad"][:, 0, :])).sum(), list(prm.values()),
                             allow_unused=True)
    for n, g in zip(prm, g2):
        key = [k for k, v in NAME.items() if v == n][0]
        ref = d[f"grad2/{key}"]
        got = np.zeros_like(ref) if g is None else g.numpy()
        assert rel(got, ref) < 2e-6 or np.abs(ref).max() == 0, n


def test_culling_matches_reference_code():
    d = np.load(G / "reference_render.npz")
    prm = _params(d)
    geom = _geom(d)
    fld = lambda x: OF.sdf_network(x, **prm, geom=geom, active_levels=int(d["bindwidth"]), out_cols=1)
    ro_c, rd_c = d["rays_o"][:, 1, 1], d["rays_d"][:, 1, 1]
    alpha = OR.center_alpha(fld, d["pre_ray_indices"], d["pre_t_starts"], d["pre_t_ends"], ro_c, rd_c,
                            torch.tensor(float(d["variance"]))).detach().numpy()
    assert rel(alpha, d["cull_alpha"]) < 1e-6
    vis = NR.visibility(alpha, d["pre_packed"], 1e-8)
    np.testing.assert_array_equal(vis, d["visibility"])


def test_patch_render_losses_and_grads_match_reference_code():
    d = np.load(G / "reference_render.npz")
    prm = _params(d)
    geom = _geom(d)
    var = torch.tensor(float(d["variance"]), dtype=torch.float64, requires_grad=True)
    fld = lambda x: OF.sdf_network(x, **prm, geom=geom, active_levels=int(d["bindwidth"]), out_cols=1)
    out = OR.patch_forward(fld, d["patch_indices"], d["t_starts"], d["t_ends"], d["rays_o"], d["rays_d"],
                           d["plane_n"], d["vinv"], var)
    assert rel(out["comp_normal"].detach().numpy(), d["comp_normal"]) < 2e-6
    assert rel(out["weight_sum"].detach().numpy(), d["weight_sum"]) < 2e-6
    assert rel(out["gradients"].detach().numpy(), d["gradients"]) < 2e-6
    L = OR.losses(out["comp_normal"], out["weight_sum"], out["gradients"], d["normal"], d["mask"])
    got = np.array([L["normal"].item(), L["eikonal"].item(), L["mask"].item(), L["total"].item()])
    assert rel(got, d["losses"]) < 2e-6
    names = list(prm) + ["variance"]
    grads = torch.autograd.grad(L["total"], list(prm.values()) + [var])
    inv = {v: k for k, v in NAME.items()}
    for n, g in zip(names, grads):
        key = "variance" if n == "variance" else inv[n]
        assert rel(g.numpy(), d[f"grad/{key}"]) < 2e-5, n


def test_patch_math_on_reference_sdf_values():
    """The oracle's patch math alone, fed the sdf values the reference's own
    SDFNetwork call produced at the patch points: same outputs, and the same
    d loss / d sdf at every start and end point."""
    d = np.load(G / "reference_render.npz")
    var = torch.tensor(float(d["variance"]), dtype=torch.float64, requires_grad=True)
    sdf = torch.from_numpy(d["patch_sdf"]).requires_grad_(True)
    out = OR.patch_forward(lambda q: sdf, d["patch_indices"], d["t_starts"], d["t_ends"], d["rays_o"],
                           d["rays_d"], d["plane_n"], d["vinv"], var)
    assert rel(out["comp_normal"].detach().numpy(), d["comp_normal"]) < 1e-12
    assert rel(out["weight_sum"].detach().numpy(), d["weight_sum"]) < 1e-12
    L = OR.losses(out["comp_normal"], out["weight_sum"], out["gradients"], d["normal"], d["mask"])
    dsdf, dvar = torch.autograd.grad(L["total"], [sdf, var])
    assert rel(dsdf.numpy(), d["patch_dsdf"]) < 1e-10
    assert rel(dvar.numpy(), d["grad/variance"]) < 1e-10
