"""Reconstruction quality of a trained field against its analytic scene.

The measures of the mixed-precision report: mean angular error of rendered
normals against the ground-truth normal maps (mask pixels), IoU of the
rendered mask (weight sum > 0.5, as the mask loss' target binarisation) with
the ground-truth mask, and Chamfer distance / F-score at 0.01 between the
SDF's zero level set (zero crossings on a regular grid, the input mesh
extraction would triangulate, models/renderer.py:9-34) and points on the
analytic surface.
"""
from __future__ import annotations

import torch

from . import scenes
from .renderer import NeuSRenderer, near_far_from_sphere


@torch.no_grad()
def render_view(renderer: NeuSRenderer, ds: scenes.SyntheticDataset, view: int, chunk: int = 4096):
    """Rendered normals (H, W, 3) and weight sums (H, W) of a dataset view
    (H and W multiples of 3; the image is tiled into 3x3 patches)."""
    H, W = ds.H, ds.W
    ph, pw = H // 3, W // 3
    blk = lambda t: t[: 3 * ph, : 3 * pw].reshape(ph, 3, pw, 3, *t.shape[2:]).transpose(1, 2).reshape(
        ph * pw, 3, 3, *t.shape[2:]).contiguous()
    d, vi = scenes.view_rays(ds.rig, view, ds.device)
    rays_d = blk(d)
    vinv = blk(vi)
    pose = ds.pose_all[view]
    rays_o = pose[:3, 3].expand(rays_d.shape).contiguous()
    plane_n = pose[:3, 2].expand(rays_d.shape[0], 3).contiguous()
    normals = torch.zeros_like(rays_d)
    wsum = torch.zeros(rays_d.shape[:3] + (1,), device=rays_d.device)
    for a in range(0, rays_d.shape[0], chunk):
        b = min(a + chunk, rays_d.shape[0])
        near, far = near_far_from_sphere(rays_o[a:b, 1, 1].contiguous(), rays_d[a:b, 1, 1].contiguous())
        r = renderer.render(rays_o[a:b], rays_d[a:b], plane_n[a:b], near, far, vinv[a:b], mode="eval")
        normals[a:b] = r["comp_normal"]
        wsum[a:b] = r["weight_sum"]
    unblk = lambda t: t.reshape(ph, pw, 3, 3, *t.shape[3:]).transpose(1, 2).reshape(3 * ph, 3 * pw, *t.shape[3:])
    return unblk(normals), unblk(wsum)[..., 0]


def angular_error_deg(pred: torch.Tensor, gt: torch.Tensor, mask: torch.Tensor) -> float:
    """Mean angle (degrees) between normalised predicted and true normals on mask pixels."""
    p = torch.nn.functional.normalize(pred.reshape(-1, 3).double(), dim=-1)
    g = torch.nn.functional.normalize(gt.reshape(-1, 3).double(), dim=-1)
    m = mask.reshape(-1) > 0.5
    if int(m.sum()) == 0:
        return float("nan")
    cos = (p[m] * g[m]).sum(-1).clamp(-1.0, 1.0)
    return float(torch.rad2deg(torch.acos(cos)).mean())


def mask_iou(weight_sum: torch.Tensor, gt_mask: torch.Tensor, thr: float = 0.5) -> float:
    a = weight_sum.reshape(-1) > thr
    b = gt_mask.reshape(-1) > 0.5
    union = int((a | b).sum())
    return float(int((a & b).sum()) / union) if union else float("nan")


@torch.no_grad()
def sdf_grid(net, res: int = 128, bound: float = 1.0, chunk: int = 1 << 21) -> torch.Tensor:
    """SDF (res, res, res) on a regular grid over [-bound, bound]^3 (z, y, x order)."""
    dev = next(net.parameters()).device
    lin = torch.linspace(-bound, bound, res, device=dev)
    zz, yy, xx = torch.meshgrid(lin, lin, lin, indexing="ij")
    pts = torch.stack([xx, yy, zz], dim=-1).reshape(-1, 3).contiguous()
    out = torch.empty(pts.shape[0], device=dev)
    for a in range(0, pts.shape[0], chunk):
        out[a:a + chunk] = net.sdf_raw(pts[a:a + chunk].contiguous()).reshape(-1)
    return out.reshape(res, res, res)


def zero_crossings(grid: torch.Tensor, bound: float = 1.0) -> torch.Tensor:
    """Points where the SDF changes sign along grid edges (linear interpolation)."""
    res = grid.shape[0]
    h = 2.0 * bound / (res - 1)
    pts = []
    for axis in range(3):
        a = grid.narrow(axis, 0, res - 1)
        b = grid.narrow(axis, 1, res - 1)
        cross = (a * b) < 0
        idx = cross.nonzero()
        if idx.numel() == 0:
            continue
        va, vb = a[cross], b[cross]
        t = va / (va - vb)
        zyx = idx.double()
        zyx[:, axis] += t.double()
        pts.append(torch.stack([zyx[:, 2], zyx[:, 1], zyx[:, 0]], dim=-1) * h - bound)
    return torch.cat(pts) if pts else torch.zeros((0, 3), dtype=torch.float64, device=grid.device)


def surface_points(scene: scenes.SDFScene, n: int, device, seed: int = 0, iters: int = 12) -> torch.Tensor:
    """n points on the analytic surface: random points projected by Newton
    steps x <- x - f(x) grad f / |grad f|^2, kept where |f| < 1e-6."""
    g = torch.Generator(device=device).manual_seed(seed)
    x = (torch.rand((4 * n, 3), generator=g, device=device, dtype=torch.float64) * 2 - 1) * 0.9
    for _ in range(iters):
        with torch.enable_grad():
            q = x.detach().requires_grad_(True)
            f = scene(q)
            (gr,) = torch.autograd.grad(f.sum(), q)
        x = (x - (f.detach() / (gr * gr).sum(-1).clamp_min(1e-12))[:, None] * gr).detach()
    keep = scene(x).abs() < 1e-6
    return x[keep][:n]


def chamfer_fscore(a: torch.Tensor, b: torch.Tensor, tau: float = 0.01, chunk: int = 2048) -> dict:
    """Symmetric Chamfer (mean of the two mean nearest distances) and F-score at tau."""
    def nn(p, q):
        out = torch.empty(p.shape[0], dtype=torch.float64, device=p.device)
        for s in range(0, p.shape[0], chunk):
            out[s:s + chunk] = torch.cdist(p[s:s + chunk].double(), q.double()).min(dim=1).values
        return out
    if a.shape[0] == 0 or b.shape[0] == 0:
        return {"chamfer": float("nan"), "fscore": 0.0, "precision": 0.0, "recall": 0.0}
    da, db = nn(a, b), nn(b, a)
    prec = float((da < tau).double().mean())
    rec = float((db < tau).double().mean())
    f = 2 * prec * rec / (prec + rec) if prec + rec > 0 else 0.0
    return {"chamfer": 0.5 * (float(da.mean()) + float(db.mean())), "fscore": f, "precision": prec, "recall": rec}


@torch.no_grad()
def evaluate(net, var, grid, ds: scenes.SyntheticDataset, scene: scenes.SDFScene, step_size: float,
             views=None, grid_res: int = 128, n_surface: int = 20000) -> dict:
    """Angular error, mask IoU and Chamfer / F@0.01 of a trained field."""
    r = NeuSRenderer(net, var)
    r.occupancy_grid = grid
    r.sampling_step_size = step_size
    views = range(ds.n_images) if views is None else views
    ang, iou = [], []
    for v in views:
        nrm, ws = render_view(r, ds, v)
        H3, W3 = nrm.shape[0], nrm.shape[1]
        ang.append(angular_error_deg(nrm, ds.normals[v, :H3, :W3], ds.masks[v, :H3, :W3]))
        iou.append(mask_iou(ws, ds.masks[v, :H3, :W3]))
    zc = zero_crossings(sdf_grid(net, grid_res))
    gt = surface_points(scene, n_surface, zc.device)
    cf = chamfer_fscore(zc, gt, 0.01)
    return {"normal_angular_error_deg": sum(ang) / len(ang), "mask_iou": sum(iou) / len(iou),
            "chamfer": cf["chamfer"], "fscore@0.01": cf["fscore"], "surface_points": int(zc.shape[0])}
