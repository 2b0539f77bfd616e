"""Generate golden fixtures by running the reference's own Python on CPU.

Runs SuperNormal's models/fields.py (SDFNetwork, SingleVarianceNetwork) and
models/renderer.py (NeuSRenderer.render) unmodified, from the reference tree,
with the third-party pieces that are absent here replaced by stubs:
  * tinycudann.Encoding -> oracle.field's hash-grid restatement (tiny-cuda-nn
    commit 2ec562e853e6f482b5d09168705205f46358fb39 is not available);
  * nerfacc (ray_marching, OccupancyGrid, render_weight_from_alpha_patch_based,
    accumulate_along_rays_patch_based) -> oracle.march / oracle.nerfacc_ref
    restatements (CPU), themselves pinned by nerfacc's known-answer vectors;
  * icecream, mcubes -> no-ops (not on the path).
The losses are exp_runner.py:169-203 written out (exp_runner.py itself needs
pyhocon / open3d / trimesh, which are absent).

Writes tests/golden/reference_render.npz and tests/golden/reference_field.npz.
Usage:  python tests/golden/make_golden.py  [SuperNormal tree; default $SUPERNORMAL_REFERENCE, else "reference" beside the repository]
"""
from __future__ import annotations

import os
import sys
import types
from pathlib import Path

import numpy as np
import torch
import torch.nn as nn

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))

from oracle import field as OF          # noqa: E402
from oracle import march as OM          # noqa: E402
from oracle import nerfacc_ref as NR    # noqa: E402

ENC = dict(otype="HashGrid", n_levels=6, n_features_per_level=2, log2_hashmap_size=10,
           base_resolution=8, per_level_scale=1.5)


# ---------------------------------------------------------------------------
# stubs for the absent third-party modules
# ---------------------------------------------------------------------------
class StubEncoding(nn.Module):
    """tcnn.Encoding stand-in: the oracle's hash grid (float64 math)."""

    def __init__(self, n_input_dims, encoding_config, seed=1337, dtype=None):
        super().__init__()
        c = encoding_config
        self.geom = OF.grid_geometry(c["n_levels"], c["n_features_per_level"], c["log2_hashmap_size"],
                                     c["base_resolution"], c["per_level_scale"])
        self.n_output_dims = c["n_levels"] * c["n_features_per_level"]
        g = torch.Generator().manual_seed(seed)
        n = int(self.geom[0][-1]) * c["n_features_per_level"]
        self.params = nn.Parameter((torch.rand(n, generator=g, dtype=torch.float64) * 2 - 1) * 0.3)

    def forward(self, x):
        return OF.encode(x, self.params, self.geom)


def install_stubs():
    tcnn = types.ModuleType("tinycudann")
    tcnn.Encoding = StubEncoding
    ic = types.ModuleType("icecream")
    ic.ic = lambda *a, **k: None
    mc = types.ModuleType("mcubes")
    mc.marching_cubes = lambda *a, **k: (np.zeros((0, 3)), np.zeros((0, 3), np.int64))
    sys.modules.update({"tinycudann": tcnn, "icecream": ic, "mcubes": mc,
                        "nerfacc": make_nerfacc_stub()})


RECORD = {}


def make_nerfacc_stub():
    from enum import Enum

    m = types.ModuleType("nerfacc")

    class ContractionType(Enum):
        AABB = 0

    class OccupancyGrid(nn.Module):
        def __init__(self, roi_aabb, resolution=128, contraction_type=ContractionType.AABB):
            super().__init__()
            self.roi_aabb = torch.as_tensor(roi_aabb, dtype=torch.float32)
            self.binary = torch.ones((resolution,) * 3, dtype=torch.bool)
            self.contraction_type = contraction_type

        def to(self, *a, **k):
            return self

    def ray_marching(rays_o, rays_d, t_min=None, t_max=None, grid=None, alpha_fn=None,
                     early_stop_eps=1e-4, alpha_thre=0.0, render_step_size=1e-3, stratified=False,
                     cone_angle=0.0, **kw):
        jitter = RECORD["jitter"] if stratified else None
        packed, ri, ts, te = OM.ray_marching(rays_o.detach().float().numpy(), rays_d.detach().float().numpy(),
                                             t_min.detach().float().numpy(), t_max.detach().float().numpy(),
                                             grid.roi_aabb.numpy(), grid.binary.numpy(), render_step_size,
                                             jitter=jitter)
        ri_t, ts_t, te_t = torch.from_numpy(ri), torch.from_numpy(ts)[:, None], torch.from_numpy(te)[:, None]
        RECORD["pre_cull"] = (packed, ri, ts, te)
        alphas = alpha_fn(ts_t, te_t, ri_t)
        RECORD["cull_alpha"] = alphas.detach().double().numpy().ravel()
        vis = NR.visibility(RECORD["cull_alpha"], packed, early_stop_eps, alpha_thre)
        RECORD["vis"] = vis
        v = torch.from_numpy(vis)
        return ri_t[v], ts_t[v], te_t[v]

    def render_weight_from_alpha_patch_based(alphas, ray_indices, n_rays=None):
        S, P, _ = alphas.shape
        packed = NR.pack_info(ray_indices.numpy(), n_rays)
        a = alphas.reshape(S, P)
        parts = []
        for b, c in packed:
            if c == 0:
                continue
            seg = a[b:b + c]
            T = torch.cumprod(torch.cat([torch.ones_like(seg[:1]), 1.0 - seg[:-1]], 0), 0)
            parts.append(seg * T)
        return torch.cat(parts, 0).reshape(S, P, 1)

    def accumulate_along_rays_patch_based(weights, ray_indices, values=None, n_patches=None):
        src = weights if values is None else weights * values
        out = torch.zeros((n_patches, src.shape[1], src.shape[2]), dtype=src.dtype)
        return out.index_add(0, ray_indices, src)

    m.ContractionType = ContractionType
    m.OccupancyGrid = OccupancyGrid
    m.ray_marching = ray_marching
    m.render_weight_from_alpha_patch_based = render_weight_from_alpha_patch_based
    m.accumulate_along_rays_patch_based = accumulate_along_rays_patch_based
    m.render_weight_from_alpha = None
    m.accumulate_along_rays = None
    return m


def exp_runner_losses(render_out, true_normal, mask):
    """exp_runner.py:169-203 with loss_type l2 and unit weights."""
    import torch.nn.functional as F

    mask = (mask > 0.5).to(true_normal.dtype)
    mask_sum = mask.sum() + 1e-5
    normal_error = (render_out["comp_normal"] - true_normal) * mask
    normal_loss = F.mse_loss(normal_error, torch.zeros_like(normal_error), reduction="sum") / mask_sum
    gn = torch.linalg.norm(render_out["gradients"], ord=2, dim=-1)
    eikonal_loss = F.mse_loss(gn, torch.ones_like(gn), reduction="mean")
    mask_loss = F.binary_cross_entropy(render_out["weight_sum"].clip(1e-5, 1.0 - 1e-5), mask)
    return normal_loss, eikonal_loss, mask_loss, normal_loss + mask_loss + eikonal_loss


def main(ref_root: str):
    sys.path.insert(0, ref_root)
    install_stubs()
    torch.set_default_dtype(torch.float64)
    from models.fields import SDFNetwork, SingleVarianceNetwork   # the reference modules
    from models.renderer import NeuSRenderer

    from supernormal_gb300 import scenes

    torch.manual_seed(0)
    net = SDFNetwork(d_in=3, d_out=16, d_hidden=64, n_layers=1, skip_in=[-1], bias=0.5,
                     geometric_init=True, weight_norm=True, encoding_config=ENC, input_concat=True)
    with torch.no_grad():
        net.lin0.weight_v[:, 3:].normal_(0.0, 0.05)
    var = SingleVarianceNetwork(0.25)
    for _ in range(ENC["n_levels"]):
        net.increase_bandwidth()
    state = {k: v.detach().double().numpy().copy() for k, v in net.state_dict().items()}

    # ---- field fixture: forward / sdf / gradient and parameter gradients ----
    gx = torch.Generator().manual_seed(1)
    x = (torch.rand((257, 3), generator=gx) * 2 - 1)
    g_out = torch.randn((257, 16), generator=gx)
    y = net(x)
    params = dict(net.named_parameters())
    names = sorted(params)
    grads = torch.autograd.grad((y * g_out).sum(), [params[n] for n in names])
    xg = x.clone().requires_grad_(True)
    grad_x = net.gradient(xg)                                   # (N, 1, 3), create_graph=True
    g_grad = torch.randn(grad_x.shape, generator=gx)
    ggrads = torch.autograd.grad((grad_x * g_grad).sum(), [params[n] for n in names], allow_unused=True)
    ggrads = [torch.zeros_like(params[n]) if g is None else g for n, g in zip(names, ggrads)]
    np.savez_compressed(
        HERE / "reference_field.npz", x=x.numpy(), g_out=g_out.numpy(), y=y.detach().numpy(),
        sdf=net.sdf(x).detach().numpy(), gradient=grad_x.detach().numpy(), g_grad=g_grad.numpy(),
        param_names=np.array(names), bindwidth=net.bindwidth,
        **{f"param/{k}": v for k, v in state.items()},
        **{f"grad/{n}": g.numpy() for n, g in zip(names, grads)},
        **{f"grad2/{n}": g.numpy() for n, g in zip(names, ggrads)},
        enc=np.array([ENC[k] for k in ("n_levels", "n_features_per_level", "log2_hashmap_size",
                                       "base_resolution")] + [ENC["per_level_scale"]]))

    # ---- render fixture: NeuSRenderer.render + exp_runner losses ----
    # models/renderer.py reshapes the whole SDFNetwork output to one column per
    # sample (:109-117, :162), so it runs only with d_out = 1, the shipped config
    torch.manual_seed(0)
    net = SDFNetwork(d_in=3, d_out=1, d_hidden=64, n_layers=1, skip_in=[-1], bias=0.5,
                     geometric_init=True, weight_norm=True, encoding_config=ENC, input_concat=True)
    with torch.no_grad():
        net.lin0.weight_v[:, 3:].normal_(0.0, 0.05)
    for _ in range(ENC["n_levels"]):
        net.increase_bandwidth()
    state = {k: v.detach().double().numpy().copy() for k, v in net.state_dict().items()}
    var = SingleVarianceNetwork(0.6)   # inv_s = e^6: sharp enough that culling drops samples
    rig = scenes.ring_cameras(4, 40, 40, radius=3.0, elevation_deg=20.0, fov_deg=40.0)
    gp = torch.Generator().manual_seed(2)
    ro, rd, pn, vinv, nrm, mask = scenes.sample_patches(scenes.sphere(0.45), rig, 24, generator=gp)
    B = ro.shape[0]
    ro_c, rd_c = ro[:, 1, 1], rd[:, 1, 1]
    a = (rd_c.double() ** 2).sum(-1)
    b = 2.0 * (ro_c.double() * rd_c.double()).sum(-1)
    c = (ro_c.double() ** 2).sum(-1) - 1.0
    mid = 0.5 * (-b) / a
    near = (mid - torch.sqrt(b ** 2 - 4 * a * c) / (2 * a)).float()
    far = (mid + torch.sqrt(b ** 2 - 4 * a * c) / (2 * a)).float()
    RECORD["jitter"] = torch.rand(B, generator=gp).float().numpy()
    r = NeuSRenderer(net, var, "dfd")
    r.sampling_step_size = 1.0 / 40
    # the last SDFNetwork call of render() evaluates every patch point at once
    # (models/renderer.py:160): keep its points, values and, below, dL/dsdf
    calls = []
    hook = net.register_forward_hook(lambda m, inp, outp: calls.append((inp[0].detach(), outp)))
    out = r.render(ro.double(), rd.double(), pn.double(), near.double(), far.double(), vinv.double())
    hook.remove()
    patch_x, patch_sdf = calls[-1]
    nl, el, ml, total = exp_runner_losses(out, nrm.double(), mask.double())
    all_params = dict(net.named_parameters())
    all_params["variance"] = var.variance
    pn_names = sorted(all_params)
    *rgrads, patch_dsdf = torch.autograd.grad(total, [all_params[n] for n in pn_names] + [patch_sdf])
    packed0, ri0, ts0, te0 = RECORD["pre_cull"]
    vis = RECORD["vis"]
    np.savez_compressed(
        HERE / "reference_render.npz",
        rays_o=ro.numpy(), rays_d=rd.numpy(), plane_n=pn.numpy(), vinv=vinv.numpy(),
        normal=nrm.numpy(), mask=mask.numpy(), near=near.numpy(), far=far.numpy(),
        jitter=RECORD["jitter"], step_size=r.sampling_step_size, variance=var.variance.item(),
        bindwidth=net.bindwidth, pre_packed=packed0, pre_ray_indices=ri0, pre_t_starts=ts0,
        pre_t_ends=te0, cull_alpha=RECORD["cull_alpha"], visibility=vis,
        patch_indices=ri0[vis], t_starts=ts0[vis], t_ends=te0[vis],
        comp_normal=out["comp_normal"].detach().numpy(), weight_sum=out["weight_sum"].detach().numpy(),
        gradients=out["gradients"].detach().numpy(),
        patch_points=patch_x.numpy(), patch_sdf=patch_sdf.detach().numpy(),
        patch_dsdf=patch_dsdf.numpy(),
        losses=np.array([nl.item(), el.item(), ml.item(), total.item()]),
        enc=np.array([ENC[k] for k in ("n_levels", "n_features_per_level", "log2_hashmap_size",
                                       "base_resolution")] + [ENC["per_level_scale"]]),
        param_names=np.array(pn_names), **{f"param/{k}": v for k, v in state.items()},
        **{f"grad/{n}": g.numpy() for n, g in zip(pn_names, rgrads)})
    print("wrote", HERE / "reference_field.npz", "and", HERE / "reference_render.npz")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.environ.get("SUPERNORMAL_REFERENCE", str(Path(__file__).resolve().parents[3] / "reference")))
