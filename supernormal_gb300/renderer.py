"""Patch-based NeuS renderer on the fused kernels: drop-in for models/renderer.py.

``NeuSRenderer.render`` keeps the reference inputs and outputs
(models/renderer.py:63-276): centre-ray marching with SDF-alpha culling,
patch expansion through the marching plane, one field evaluation for all
patch pixels, then NeuS alpha, patch weights, dfd normals and accumulation
in one fused kernel whose backward is hand-written.  The returned tensors
are autograd-connected, so the caller's losses (exp_runner.py:191-203)
back-propagate through the custom kernels.
"""
from __future__ import annotations


import torch
from torch import Tensor

from ._lib import call, stream_handle
from .nerfacc import (ContractionType, OccupancyGrid, _pack_counts, accumulate_along_rays, ray_marching,
                      render_weight_from_alpha)

__all__ = ["NeuSRenderer", "near_far_from_sphere"]


def near_far_from_sphere(rays_o: Tensor, rays_d: Tensor):
    """Unit-sphere chord (models/dataset_loader.py:279-297)."""
    a = torch.sum(rays_d ** 2, dim=-1, keepdim=True)
    b = 2.0 * torch.sum(rays_o * rays_d, dim=-1, keepdim=True)
    c = torch.sum(rays_o ** 2, dim=-1, keepdim=True) - 1.0
    mid = 0.5 * (-b) / a
    near = mid - torch.sqrt(b ** 2 - 4 * a * c) / (2 * a)
    far = mid + torch.sqrt(b ** 2 - 4 * a * c) / (2 * a)
    return near[..., 0], far[..., 0]


class PatchGeometry:
    """No-grad per-step geometry shared by the forward and backward kernels."""

    def __init__(self, H, W, packed, S, end_packed, E, t_pix_s, t_pix_e, rays_o, rays_d, vinv):
        self.H, self.W, self.P = H, W, H * W
        self.packed, self.S, self.end_packed, self.E = packed, S, end_packed, E
        self.t_pix_s, self.t_pix_e = t_pix_s, t_pix_e
        self.rays_o, self.rays_d, self.vinv = rays_o, rays_d, vinv
        self.n_patches = packed.shape[0]


class _PatchRenderFn(torch.autograd.Function):
    """Fused NeuS alpha + patch weights + gradients + accumulation; ``ext``
    (optional, (S, P, 3)) gives the gradients ('ad'), else dfd is used."""

    @staticmethod
    def forward(ctx, sdf: Tensor, variance: Tensor, ext, geo: PatchGeometry):
        dev = sdf.device
        B, P, S = geo.n_patches, geo.P, geo.S
        ctx.sdf_shape = sdf.shape
        ctx.ext_shape = None if ext is None else ext.shape
        sdf = sdf.contiguous().float().reshape(-1)
        var = variance.detach().reshape(1).contiguous().float()
        ext = None if ext is None else ext.detach().contiguous().float()
        comp = torch.empty((B, P, 3), device=dev)
        wsum = torch.empty((B, P), device=dev)
        grads = torch.empty((S, P, 3), device=dev) if ext is None else ext.reshape(S, P, 3).clone()
        call("sn_patch_render_fwd", B, geo.H, geo.W, geo.packed, None, S, geo.end_packed, sdf,
             geo.t_pix_s, geo.t_pix_e, geo.rays_o, geo.rays_d, geo.vinv, var, None, None,
             grads if ext is None else None, comp, wsum, ext, stream_handle())
        ctx.save_for_backward(sdf, var, ext if ext is not None else torch.empty(0, device=dev))
        ctx.has_ext = ext is not None
        ctx.geo = geo
        return comp, wsum, grads

    @staticmethod
    def backward(ctx, g_comp, g_wsum, g_grads):
        sdf, var, ext = ctx.saved_tensors
        ext = ext if ctx.has_ext else None
        geo = ctx.geo
        dev = sdf.device
        B, P, S = geo.n_patches, geo.P, geo.S
        g_comp = torch.zeros((B, P, 3), device=dev) if g_comp is None else g_comp.contiguous().float()
        g_wsum = torch.zeros((B, P), device=dev) if g_wsum is None else g_wsum.contiguous().float()
        g_grads = None if g_grads is None else g_grads.contiguous().float()
        d_sdf = torch.empty_like(sdf)
        d_ext = torch.empty((S, P, 3), device=dev) if ext is not None else None
        partials = torch.zeros((B, 4), device=dev)
        carry = torch.empty((B, P), device=dev)
        st = stream_handle()
        call("sn_patch_render_bwd", B, geo.H, geo.W, geo.packed, None, S, geo.end_packed, sdf,
             geo.t_pix_s, geo.t_pix_e, geo.rays_o, geo.rays_d, geo.vinv, var, g_comp, g_wsum,
             g_grads, d_sdf, partials, carry, ext, d_ext, st)
        call("sn_patch_carry_fixup", B, P, geo.packed, None, S, geo.end_packed, carry, d_sdf, st)
        d_var = torch.zeros((1,), device=dev)
        call("sn_patch_finalize", B, P, partials, None, S, var, None, 0.0, 0.0, 0.0, None, d_var, st)
        if d_ext is not None:
            d_ext = d_ext.reshape(ctx.ext_shape)
        return d_sdf.reshape(ctx.sdf_shape), d_var.reshape(()), d_ext, None


class NeuSRenderer:
    def __init__(self, sdf_network, deviation_network, gradient_method="dfd"):
        self.sdf_network = sdf_network
        self.deviation_network = deviation_network
        self.scene_aabb = torch.as_tensor([-1., -1., -1., 1., 1., 1.], dtype=torch.float32)
        self.contraction_type = ContractionType.AABB
        self.occupancy_grid = OccupancyGrid(roi_aabb=self.scene_aabb, resolution=128,
                                            contraction_type=self.contraction_type).to("cuda")
        self.sampling_step_size = 0.01
        self.gradient_method = gradient_method

    def occ_eval_fn(self, x):
        sdf = self.sdf_network.sdf(x)
        return torch.sigmoid(-sdf * 80)

    def _variance(self) -> Tensor:
        return self.deviation_network.variance

    def _center_alpha_fn(self, rays_o_c: Tensor, rays_d_c: Tensor):
        net = self.sdf_network

        def alpha_fn(t_starts, t_ends, ray_indices):
            n = t_starts.shape[0]
            dev = t_starts.device
            if n == 0:
                return torch.empty((0, 1), device=dev)
            st = stream_handle()
            ts = t_starts.reshape(-1).contiguous()
            te = t_ends.reshape(-1).contiguous()
            diff = torch.empty((n,), dtype=torch.int32, device=dev)
            call("sn_end_diff", n, None, ts, te, diff, st)
            end_packed, n_ends = _pack_counts(diff)
            xyz = torch.empty((2 * n, 3), device=dev)
            q = torch.empty((1,), dtype=torch.int32, device=dev)
            call("sn_center_points", n, None, ray_indices.contiguous(), ts, te, rays_o_c, rays_d_c,
                 end_packed, n_ends, xyz, q, st)
            sdf = net.sdf_raw(xyz, q)
            alpha = torch.empty((n, 1), device=dev)
            var = self._variance().detach().reshape(1).contiguous().float()
            call("sn_center_alpha", n, None, sdf, 1, end_packed, var, alpha, st)
            return alpha

        return alpha_fn

    def render(self, rays_o_patch_all, rays_d_patch_all, marching_plane_normal, near, far,
               V_inverse_patch_all, val_gradient_method="dfd", mode="train", generator=None):
        patch_H, patch_W = rays_o_patch_all.shape[1], rays_o_patch_all.shape[2]
        num_patch = rays_o_patch_all.shape[0]
        P = patch_H * patch_W
        dev = rays_o_patch_all.device
        ro = rays_o_patch_all.contiguous().float()
        rd = rays_d_patch_all.contiguous().float()
        ro_c = ro[:, patch_H // 2, patch_W // 2].contiguous()
        rd_c = rd[:, patch_H // 2, patch_W // 2].contiguous()
        gradient_method = self.gradient_method if mode == "train" else val_gradient_method
        if gradient_method not in ("dfd", "ad"):
            raise NotImplementedError(f"gradient_method {gradient_method!r}: the fused renderer "
                                      "implements 'dfd' (the shipped configuration) and 'ad'")
        with torch.no_grad():
            patch_indices, t_s, t_e = ray_marching(
                ro_c, rd_c, t_min=near, t_max=far, grid=self.occupancy_grid,
                render_step_size=self.sampling_step_size, stratified=True, cone_angle=0.0,
                early_stop_eps=1e-8, alpha_fn=self._center_alpha_fn(ro_c, rd_c), generator=generator)
        self.last_samples = (patch_indices, t_s, t_e)
        return self.render_samples(ro, rd, marching_plane_normal, V_inverse_patch_all, patch_indices,
                                   t_s, t_e, gradient_method)

    @torch.no_grad()
    def render_normal_pixel_based(self, rays_o: Tensor, rays_d: Tensor, near: Tensor, far: Tensor,
                                  generator=None):
        """Per-pixel normal and depth rendering for validation
        (models/renderer.py:278-351): rays (N, 3) marched with stratified
        jitter and culled at early_stop_eps = 1e-3 with the NeuS alpha of the
        same alpha_fn, weights per ray, normals from SDFNetwork.gradient at
        the sample midpoints, then accumulated.  Returns (comp_normal (N, 3),
        comp_depth (N, 1))."""
        ro = rays_o.contiguous().float()
        rd = rays_d.contiguous().float()
        n_rays = ro.shape[0]
        alpha_fn = self._center_alpha_fn(ro, rd)
        ray_indices, t_starts, t_ends = ray_marching(
            ro, rd, t_min=near.reshape(-1), t_max=far.reshape(-1), grid=self.occupancy_grid,
            render_step_size=self.sampling_step_size, stratified=True, cone_angle=0.0, alpha_thre=0.0,
            early_stop_eps=1e-3, alpha_fn=alpha_fn, generator=generator)
        self.last_samples = (ray_indices, t_starts, t_ends)
        if ray_indices.numel() == 0:
            return torch.zeros((n_rays, 3), device=ro.device), torch.zeros((n_rays, 1), device=ro.device)
        alpha = alpha_fn(t_starts, t_ends, ray_indices)
        midpoints = (t_starts + t_ends) / 2.0
        positions = ro[ray_indices] + rd[ray_indices] * midpoints
        gradients = self.sdf_network.gradient(positions).reshape(-1, 3).detach()
        weights = render_weight_from_alpha(alpha, ray_indices=ray_indices, n_rays=n_rays)
        comp_normal = accumulate_along_rays(weights, ray_indices, values=gradients, n_rays=n_rays)
        comp_depth = accumulate_along_rays(weights, ray_indices, values=midpoints, n_rays=n_rays)
        return comp_normal, comp_depth

    def extract_geometry(self, bound_min, bound_max, resolution, threshold=0.0):
        """Mesh of the SDF's zero level set (models/renderer.py:353-358): the
        lattice of -sdf from the fused field and the device marching cubes;
        (vertices float64 (V, 3), triangles int64 (T, 3)) numpy arrays."""
        from .mesh import marching_cubes, sdf_lattice

        u = sdf_lattice(self.sdf_network, bound_min, bound_max, resolution)
        v, t = marching_cubes(u, threshold, bound_min, bound_max)
        return v.double().cpu().numpy(), t.long().cpu().numpy()

    def render_samples(self, rays_o_patch_all, rays_d_patch_all, marching_plane_normal,
                       V_inverse_patch_all, patch_indices, t_s, t_e, gradient_method="dfd"):
        """The part of render() after marching and culling (models/renderer.py:142-276),
        for given culled centre samples (patch_indices, t_starts, t_ends).
        'ad' takes the gradients from SDFNetwork.gradient at the start points
        (models/renderer.py:225-226) with the second-order adjoint."""
        patch_H, patch_W = rays_o_patch_all.shape[1], rays_o_patch_all.shape[2]
        num_patch = rays_o_patch_all.shape[0]
        P = patch_H * patch_W
        dev = rays_o_patch_all.device
        ro = rays_o_patch_all.contiguous().float()
        rd = rays_d_patch_all.contiguous().float()
        patch_indices = patch_indices.contiguous().long()
        S = patch_indices.shape[0]
        samples_per_ray = S / num_patch
        inv_s = self.deviation_network(torch.zeros([1, 3], device=dev))[:, :1].clip(1e-6, 1e6)
        if S == 0:
            z = torch.zeros([num_patch, patch_H, patch_W, 3], device=dev)
            return {"s_val": 1 / inv_s, "weight_sum": torch.zeros([num_patch, patch_H, patch_W, 1],
                                                                   device=dev),
                    "gradients": None, "comp_normal": z, "samples_per_ray": 0.0}
        st = stream_handle()
        ts = t_s.reshape(-1).contiguous()
        te = t_e.reshape(-1).contiguous()
        with torch.no_grad():
            diff = torch.empty((S,), dtype=torch.int32, device=dev)
            call("sn_end_diff", S, None, ts, te, diff, st)
            end_packed, n_ends = _pack_counts(diff)
            E = int(n_ends.item())
            xyz = torch.empty(((S + E) * P, 3), device=dev)
            tps = torch.empty((S, P), device=dev)
            tpe = torch.empty((S, P), device=dev)
            call("sn_patch_points", S, None, patch_H, patch_W, patch_indices, ts, te, ro, rd,
                 marching_plane_normal.contiguous().float(), end_packed, n_ends, xyz, tps, tpe, None,
                 st)
            counts = torch.empty((num_patch,), dtype=torch.int32, device=dev)
            call("sn_count_indices", S, patch_indices, num_patch, counts, st)
            packed, _ = _pack_counts(counts)
        self.last_points = xyz
        geo = PatchGeometry(patch_H, patch_W, packed, S, end_packed, E, tps, tpe, ro, rd,
                            V_inverse_patch_all.contiguous().float())
        sdf = self.sdf_network.sdf(xyz)
        ext = None
        if gradient_method == "ad":
            _, ext = self.sdf_network.sdf_and_gradient(xyz[: S * P])
        comp, wsum, grads = _PatchRenderFn.apply(sdf, self._variance(), ext, geo)
        return {
            "s_val": 1 / inv_s,
            "weight_sum": wsum.reshape(num_patch, patch_H, patch_W, 1),
            "gradients": grads.reshape(S, patch_H, patch_W, 3),
            "comp_normal": comp.reshape(num_patch, patch_H, patch_W, 3),
            "samples_per_ray": samples_per_ray,
        }
