"""ORACLE (test infrastructure only): restatement of the patch renderer and losses.

Follows models/renderer.py:80-122 (culling alpha), :142-267 (patch expansion,
NeuS alpha, patch weights, dfd normals, accumulation) and exp_runner.py:169-203
(losses) with torch CPU tensors, float64 for the parity checks (``dtype``
float32 for a timed host baseline), so autograd gives the reference
gradients.  The field is passed in as a callable (N,3) -> (N,1).
"""
from __future__ import annotations

import numpy as np
import torch
import torch.nn.functional as F

from . import nerfacc_ref


def inv_s_of(variance, dtype=torch.float64):
    return torch.exp(variance.to(dtype) * 10.0).clip(1e-6, 1e6)


def neus_alpha(s0, s1, inv_s):
    """models/renderer.py:171-179."""
    prev_cdf = torch.sigmoid(s0 * inv_s)
    next_cdf = torch.sigmoid(s1 * inv_s)
    p = prev_cdf - next_cdf
    c = prev_cdf
    return ((p + 1e-5) / (c + 1e-5)).clip(0.0, 1.0)


def diff_mask_of(ts, te):
    """t_end != next t_start over the flattened list (last compares with itself)."""
    ts = np.asarray(ts, np.float32).reshape(-1)
    te = np.asarray(te, np.float32).reshape(-1)
    nxt = np.concatenate([ts[1:], ts[-1:]])
    return (te - nxt) != 0


def _f32_points(o, d, t):
    """o + d * t as the reference forms it on the device: float32 product, then
    float32 sum (two roundings)."""
    return (np.asarray(o, np.float32) + (np.asarray(d, np.float32) * np.asarray(t, np.float32)).astype(np.float32)
            ).astype(np.float32)


def center_alpha(field, ridx, ts, te, rays_o_c, rays_d_c, variance, dtype=torch.float64, f32_points=False):
    """alpha_fn_patch_center (models/renderer.py:80-122).  f32_points: the
    query points in the reference's float32 arithmetic (so hash cells match a
    float32 pipeline exactly); else in ``dtype``."""
    ridx = np.asarray(ridx)
    o = torch.as_tensor(np.asarray(rays_o_c, np.float32)[ridx]).to(dtype)
    d = torch.as_tensor(np.asarray(rays_d_c, np.float32)[ridx]).to(dtype)
    tsd = torch.as_tensor(np.asarray(ts, np.float32)).to(dtype).reshape(-1, 1)
    ted = torch.as_tensor(np.asarray(te, np.float32)).to(dtype).reshape(-1, 1)
    diff = torch.as_tensor(diff_mask_of(ts, te))
    if f32_points:
        o32, d32 = np.asarray(rays_o_c, np.float32)[ridx], np.asarray(rays_d_c, np.float32)[ridx]
        ps = torch.as_tensor(_f32_points(o32, d32, np.asarray(ts, np.float32).reshape(-1, 1))).to(dtype)
        pe = torch.as_tensor(_f32_points(o32, d32, np.asarray(te, np.float32).reshape(-1, 1))).to(dtype)
    else:
        ps, pe = o + d * tsd, o + d * ted
    sdf = field(torch.cat([ps, pe[diff]], 0))
    n = ps.shape[0]
    s0 = sdf[:n]
    s1 = torch.cat([s0[1:], s0[-1:]], 0).clone()
    s1[diff] = sdf[n:]
    return neus_alpha(s0, s1, inv_s_of(variance, dtype)).reshape(-1)


def cull(field, packed, ridx, ts, te, rays_o_c, rays_d_c, variance, early_stop_eps=1e-8,
         dtype=torch.float64):
    """Visibility culling inside nerfacc.ray_marching (NA/nerfacc/ray_marching.py:193-220)."""
    with torch.no_grad():
        alpha = center_alpha(field, ridx, ts, te, rays_o_c, rays_d_c, variance, dtype).numpy()
    vis = nerfacc_ref.visibility(alpha, packed, early_stop_eps)
    return vis, alpha


def patch_forward(field, patch_idx, ts, te, rays_o_all, rays_d_all, plane_n, vinv, variance,
                  points=None, gradient_method="dfd", ext_gradients=None, dtype=torch.float64):
    """models/renderer.py:142-267 for gradient_method='dfd' (float64 unless
    ``dtype`` says otherwise).

    patch_idx/ts/te are the culled centre samples; rays_* are (B, H, W, 3).
    ``points`` (optional, ((S + E) * H * W, 3) float32) are the field query
    points as a float32 pipeline formed them (the reference computes them in
    float32); the field is then evaluated exactly there, so hash-grid cell
    choices match and only arithmetic precision differs."""
    pidx = torch.as_tensor(np.asarray(patch_idx, np.int64))
    ro = torch.as_tensor(np.asarray(rays_o_all, np.float32)).to(dtype)
    rd = torch.as_tensor(np.asarray(rays_d_all, np.float32)).to(dtype)
    pn = torch.as_tensor(np.asarray(plane_n, np.float32)).to(dtype)
    vi = torch.as_tensor(np.asarray(vinv, np.float32)).to(dtype)
    B, H, W, _ = ro.shape
    S = pidx.shape[0]
    tsc = torch.as_tensor(np.asarray(ts, np.float32)).to(dtype).reshape(S, 1, 1, 1)
    tec = torch.as_tensor(np.asarray(te, np.float32)).to(dtype).reshape(S, 1, 1, 1)
    dc = rd[:, H // 2, W // 2]
    dot_c = (dc * pn).sum(-1, keepdim=True)[pidx][:, None, None, :]
    dot_p = (rd * pn[:, None, None, :]).sum(-1, keepdim=True)[pidx]
    t_s = tsc * dot_c / dot_p
    t_e = tec * dot_c / dot_p
    diff = torch.as_tensor(diff_mask_of(ts, te))
    ps = ro[pidx] + rd[pidx] * t_s
    pe = ro[pidx] + rd[pidx] * t_e
    pts = torch.cat([ps, pe[diff]], 0)
    q = pts.reshape(-1, 3) if points is None else torch.as_tensor(np.asarray(points, np.float32)).to(dtype)
    assert q.shape[0] == pts.reshape(-1, 3).shape[0], "points do not match the sample layout"
    sdf = field(q).reshape(*pts.shape[:-1], 1)
    s0 = sdf[:S]
    s1 = torch.cat([s0[1:], s0[-1:]], 0)
    s1 = torch.where(diff[:, None, None, None], torch.zeros_like(s1), s1)
    s1 = s1.clone()
    s1[diff] = sdf[S:]
    inv_s = inv_s_of(variance, dtype)
    alpha = neus_alpha(s0, s1, inv_s)                                 # (S, H, W, 1)
    # patch weights: w = alpha * prod_{j<i}(1 - alpha_j) within each patch
    a = alpha.reshape(S, H * W)
    packed = nerfacc_ref.pack_info(np.asarray(patch_idx), n_rays=B)
    w_parts = []
    for b, c in packed:
        if c == 0:
            continue
        seg = a[b:b + c]
        T = torch.cumprod(torch.cat([torch.ones_like(seg[:1]), 1.0 - seg[:-1]], 0), 0)
        w_parts.append(seg * T)
    weights = torch.cat(w_parts, 0).reshape(S, H, W, 1)
    # dfd gradients (models/renderer.py:187-223)
    dist_x = torch.linalg.vector_norm(ps[:, :, 1:, :] - ps[:, :, :-1, :], dim=-1, keepdim=True).detach()
    dist_y = torch.linalg.vector_norm(ps[:, 1:, :, :] - ps[:, :-1, :, :], dim=-1, keepdim=True).detach()
    df_dt = (s1 - s0) / (t_e - t_s)
    df_dx = (s0[:, :, 2:] - s0[:, :, :-2]) / (dist_x[:, :, :-1] + dist_x[:, :, 1:])
    df_dy = (s0[:, 2:, :] - s0[:, :-2, :]) / (dist_y[:, 1:, :] + dist_y[:, :-1, :])
    dx_l = (s0[:, :, 1:2] - s0[:, :, 0:1]) / dist_x[:, :, 0:1]
    dx_r = (s0[:, :, -1:] - s0[:, :, -2:-1]) / dist_x[:, :, -1:]
    dy_t = (s0[:, 1:2, :] - s0[:, 0:1, :]) / dist_y[:, 0:1, :]
    dy_b = (s0[:, -1:, :] - s0[:, -2:-1, :]) / dist_y[:, -1:, :]
    df_dx = torch.cat([dx_l, df_dx, dx_r], dim=2)
    df_dy = torch.cat([dy_t, df_dy, dy_b], dim=1)
    proj = torch.cat([df_dt, df_dx, df_dy], dim=-1)
    gradients = (vi[pidx] @ proj[..., None])[..., 0]                  # (S, H, W, 3)
    if gradient_method == "ad" and ext_gradients is not None:
        # given start-point gradients (S * H * W, 3): isolates the patch math
        gradients = ext_gradients.reshape(S, H, W, 3)
    elif gradient_method == "ad":
        # SDFNetwork.gradient at the start points (models/renderer.py:225-226,
        # models/fields.py:107-119: autograd with create_graph)
        xs = q[: S * H * W].detach().clone().requires_grad_(True)
        s_ad = field(xs)
        (g_ad,) = torch.autograd.grad(s_ad.sum(), xs, create_graph=True)
        gradients = g_ad.reshape(S, H, W, 3)
    # accumulation (models/renderer.py:263-267)
    wsum = torch.zeros((B, H * W, 1), dtype=dtype).index_add(0, pidx, weights.reshape(S, H * W, 1))
    comp = torch.zeros((B, H * W, 3), dtype=dtype).index_add(
        0, pidx, (weights * gradients).reshape(S, H * W, 3))
    return dict(alpha=alpha, weights=weights, gradients=gradients,
                weight_sum=wsum.reshape(B, H, W, 1), comp_normal=comp.reshape(B, H, W, 3),
                sdf=sdf, t_s=t_s, t_e=t_e, diff=diff)


def losses(comp_normal, weight_sum, gradients, gt_normal, gt_mask, loss_type="l2",
           normal_weight=1.0, eikonal_weight=1.0, mask_weight=1.0):
    """exp_runner.py:169-203 (mask binarised when mask_weight > 0)."""
    like = comp_normal
    as_t = lambda a: (a if isinstance(a, torch.Tensor) else torch.as_tensor(np.asarray(a, np.float32))
                      ).to(device=like.device, dtype=like.dtype)
    gt_normal = as_t(gt_normal)
    mask = as_t(gt_mask)
    mask = (mask > 0.5).to(like.dtype) if mask_weight > 0.0 else torch.ones_like(mask)
    mask_sum = mask.sum() + 1e-5
    err = (comp_normal - gt_normal) * mask
    if loss_type == "l1":
        normal_loss = F.l1_loss(err, torch.zeros_like(err), reduction="sum") / mask_sum
    else:
        normal_loss = F.mse_loss(err, torch.zeros_like(err), reduction="sum") / mask_sum
    gn = torch.linalg.norm(gradients, ord=2, dim=-1)
    eikonal = F.mse_loss(gn, torch.ones_like(gn), reduction="mean")
    mask_loss = F.binary_cross_entropy(weight_sum.clip(1e-5, 1.0 - 1e-5), mask)
    total = normal_weight * normal_loss + mask_weight * mask_loss + eikonal_weight * eikonal
    return dict(normal=normal_loss, eikonal=eikonal, mask=mask_loss, total=total)


def pixel_forward(field, ridx, ts, te, rays_o, rays_d, variance, n_rays):
    """NeuSRenderer.render_normal_pixel_based after marching and culling
    (models/renderer.py:338-351), float64: alpha of alpha_fn on the kept
    samples, per-ray weights (NA/nerfacc/vol_rendering.py:624-678), the SDF
    gradient (autograd) at the sample midpoints, accumulated normals and
    depths.  Returns (comp_normal (n_rays, 3), comp_depth (n_rays, 1))."""
    ridx = np.asarray(ridx, np.int64)
    with torch.no_grad():
        alpha = center_alpha(field, ridx, ts, te, rays_o, rays_d, variance, f32_points=True).numpy()
    packed = nerfacc_ref.pack_info(ridx, n_rays)
    w = nerfacc_ref.weights_fwd(alpha, packed)
    # midpoints and positions in the reference's float32 arithmetic (:342-345)
    mid32 = ((np.asarray(ts, np.float32).reshape(-1, 1) + np.asarray(te, np.float32).reshape(-1, 1))
             .astype(np.float32) / np.float32(2.0)).astype(np.float32)
    mid = torch.as_tensor(mid32).double()
    x32 = _f32_points(np.asarray(rays_o, np.float32)[ridx], np.asarray(rays_d, np.float32)[ridx], mid32)
    x = torch.as_tensor(x32).double().requires_grad_(True)
    (g,) = torch.autograd.grad(field(x).sum(), x)
    wt = torch.as_tensor(w).reshape(-1, 1)
    idx = torch.as_tensor(ridx)
    comp = torch.zeros((n_rays, 3), dtype=torch.float64).index_add(0, idx, wt * g)
    depth = torch.zeros((n_rays, 1), dtype=torch.float64).index_add(0, idx, wt * mid)
    return comp, depth, {"alpha": alpha, "weights": w, "gradients": g.detach()}
