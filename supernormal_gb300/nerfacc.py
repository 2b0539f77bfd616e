"""nerfacc-compatible operators used by SuperNormal's renderer, on sm_103a kernels.

Drop-in for the names ``models/renderer.py`` imports from nerfacc 0.3.5
(``ContractionType, OccupancyGrid, ray_marching,
render_weight_from_alpha_patch_based, accumulate_along_rays_patch_based,
render_weight_from_alpha, accumulate_along_rays``) plus the helpers they are
built from (``pack_info, unpack_info, render_visibility,
render_transmittance_from_alpha, query_grid, contract_inv``).  Signatures,
argument meanings, output shapes/dtypes and error behaviour follow
``NA/nerfacc/*.py`` (NA = third_parties/nerfacc-0.3.5/nerfacc-0.3.5).
Every computation runs in the CUDA library; CPU tensors raise
``NotImplementedError`` exactly as nerfacc does.
"""
from __future__ import annotations

from enum import Enum
from typing import Callable, List, Optional, Tuple, Union

import torch
import torch.nn as nn
from torch import Tensor

from ._lib import SN_STATUS_CAPACITY, SN_STATUS_MARCH_LIMIT, call, stream_handle

__all__ = [
    "ContractionType", "Grid", "OccupancyGrid", "ray_marching", "render_visibility",
    "render_weight_from_alpha", "render_weight_from_alpha_patch_based",
    "render_transmittance_from_alpha", "accumulate_along_rays",
    "accumulate_along_rays_patch_based", "pack_info", "unpack_info", "query_grid",
    "contract_inv", "ray_aabb_intersect",
]


class ContractionType(Enum):
    """Space contraction of a grid (NA/nerfacc/contraction.py:12-68)."""

    AABB = 0
    UN_BOUNDED_TANH = 1
    UN_BOUNDED_SPHERE = 2

    def to_cpp_version(self) -> int:
        return self.value


def _need_cuda(t: Tensor) -> None:
    if not t.is_cuda:
        raise NotImplementedError("Only support cuda inputs.")


def _ws(nbytes: int, device) -> Tensor:
    return torch.empty(max(int(nbytes), 16), dtype=torch.uint8, device=device)


def _pack_counts(counts: Tensor) -> Tuple[Tensor, Tensor]:
    """counts (n,) int32 -> packed_info (n, 2) int32 and device total (1,) int32."""
    n = counts.numel()
    dev = counts.device
    packed = torch.empty((n, 2), dtype=torch.int32, device=dev)
    total = torch.zeros((1,), dtype=torch.int32, device=dev)
    ws = _ws(int(call("sn_scan_workspace_bytes", n)), dev)
    call("sn_pack_counts", n, counts, packed, total, ws, stream_handle())
    return packed, total


# ---------------------------------------------------------------------------
# packing (NA/nerfacc/pack.py)
# ---------------------------------------------------------------------------
@torch.no_grad()
def pack_info(ray_indices: Tensor, n_rays: int = None) -> Tensor:
    """packed_info (n_rays, 2) int32 from sorted ray_indices (NA/nerfacc/pack.py:46-77)."""
    assert ray_indices.dim() == 1, "ray_indices must be a 1D tensor with shape (n_samples)."
    _need_cuda(ray_indices)
    ray_indices = ray_indices.contiguous().long()
    if n_rays is None:
        n_rays = int(ray_indices.max()) + 1 if ray_indices.numel() > 0 else 0
    counts = torch.empty((n_rays,), dtype=torch.int32, device=ray_indices.device)
    call("sn_count_indices", ray_indices.numel(), ray_indices, n_rays, counts, stream_handle())
    packed, _ = _pack_counts(counts)
    return packed


@torch.no_grad()
def unpack_info(packed_info: Tensor, n_samples: int) -> Tensor:
    """ray_indices (n_samples,) int64 from packed_info (NA/nerfacc/pack.py:80-117)."""
    assert packed_info.dim() == 2 and packed_info.shape[-1] == 2, \
        "packed_info must be a 2D tensor with shape (n_rays, 2)."
    _need_cuda(packed_info)
    packed_info = packed_info.contiguous().int()
    out = torch.empty((n_samples,), dtype=torch.int64, device=packed_info.device)
    call("sn_unpack_info", packed_info.shape[0], packed_info, n_samples, out, stream_handle())
    return out


# ---------------------------------------------------------------------------
# grids (NA/nerfacc/grid.py, contraction.py)
# ---------------------------------------------------------------------------
@torch.no_grad()
def contract_inv(x: Tensor, roi: Tensor, type: ContractionType = ContractionType.AABB) -> Tensor:
    """[0,1]^3 -> world (NA/nerfacc/contraction.py:86-102): the cell-point kernel
    on a 1x1x1 grid whose only cell spans [0,1]^3."""
    _need_cuda(x)
    x = x.contiguous().float()
    out = torch.empty_like(x)
    cells = torch.zeros((x.shape[0],), dtype=torch.int64, device=x.device)
    call("sn_occ_points", x.shape[0], cells, x, 1, 1, 1, roi.contiguous().float(), type.value, out,
         stream_handle())
    return out


@torch.no_grad()
def query_grid(samples: Tensor, grid_roi: Tensor, grid_values: Tensor,
               grid_type: ContractionType) -> Tensor:
    """Grid values at samples (NA/nerfacc/grid.py:19-47); boolean grids only."""
    assert samples.dim() == 2 and samples.size(-1) == 3
    assert grid_roi.dim() == 1 and grid_roi.size(0) == 6
    assert grid_values.dim() == 3
    assert isinstance(grid_type, ContractionType)
    _need_cuda(samples)
    if grid_values.dtype != torch.bool:
        raise NotImplementedError("query_grid: only boolean grids are supported")
    out = torch.empty((samples.shape[0],), dtype=torch.bool, device=samples.device)
    rx, ry, rz = grid_values.shape
    call("sn_grid_query", samples.shape[0], samples.contiguous().float(), grid_roi.contiguous().float(),
         grid_values.contiguous().view(torch.uint8), rx, ry, rz, grid_type.value,
         out.view(torch.uint8), stream_handle())
    return out


class Grid(nn.Module):
    """Abstract grid: roi_aabb, binary, contraction_type (NA/nerfacc/grid.py:50-110)."""

    def __init__(self, *args, **kwargs):
        super().__init__()
        self.register_buffer("_dummy", torch.empty(0), persistent=False)

    @property
    def device(self) -> torch.device:
        return self._dummy.device

    @property
    def roi_aabb(self) -> Tensor:
        if hasattr(self, "_roi_aabb"):
            return getattr(self, "_roi_aabb")
        raise NotImplementedError("please set an attribute named _roi_aabb")

    @property
    def binary(self) -> Tensor:
        if hasattr(self, "_binary"):
            return getattr(self, "_binary")
        raise NotImplementedError("please set an attribute named _binary")

    @property
    def contraction_type(self) -> ContractionType:
        if hasattr(self, "_contraction_type"):
            return getattr(self, "_contraction_type")
        raise NotImplementedError("please set an attribute named _contraction_type")


class OccupancyGrid(Grid):
    """EMA occupancy grid (NA/nerfacc/grid.py:113-294) with the same buffers
    (``_roi_aabb``, ``_binary``, ``resolution``, ``occs`` persistent;
    ``grid_coords``/``grid_indices`` not) and update rule; cell sampling,
    query-point construction, the EMA max and the mean-threshold
    binarisation run as device kernels."""

    NUM_DIM: int = 3

    def __init__(self, roi_aabb: Union[List[int], Tensor],
                 resolution: Union[int, List[int], Tensor] = 128,
                 contraction_type: ContractionType = ContractionType.AABB) -> None:
        super().__init__()
        if isinstance(resolution, int):
            resolution = [resolution] * self.NUM_DIM
        if isinstance(resolution, (list, tuple)):
            resolution = torch.tensor(resolution, dtype=torch.int32)
        assert isinstance(resolution, Tensor), f"Invalid type: {type(resolution)}"
        assert resolution.shape == (self.NUM_DIM,), f"Invalid shape: {resolution.shape}"
        if isinstance(roi_aabb, (list, tuple)):
            roi_aabb = torch.tensor(roi_aabb, dtype=torch.float32)
        assert isinstance(roi_aabb, Tensor), f"Invalid type: {type(roi_aabb)}"
        assert roi_aabb.shape == torch.Size([self.NUM_DIM * 2]), f"Invalid shape: {roi_aabb.shape}"
        self.num_cells = int(resolution.prod().item())
        self.register_buffer("_roi_aabb", roi_aabb)
        self.register_buffer("_binary", torch.zeros(resolution.tolist(), dtype=torch.bool))
        self._contraction_type = contraction_type
        self.register_buffer("resolution", resolution)
        self.register_buffer("occs", torch.zeros(self.num_cells))
        res = resolution.tolist()
        coords = torch.stack(torch.meshgrid([torch.arange(r, dtype=torch.long) for r in res],
                                            indexing="ij"), dim=-1).reshape(self.num_cells, 3)
        self.register_buffer("grid_coords", coords, persistent=False)
        self.register_buffer("grid_indices", torch.arange(self.num_cells), persistent=False)

    @torch.no_grad()
    def _get_all_cells(self) -> Tensor:
        return self.grid_indices

    @torch.no_grad()
    def _sample_uniform_and_occupied_cells(self, n: int) -> Tensor:
        uniform = torch.randint(self.num_cells, (n,), device=self.device)
        occupied = torch.nonzero(self._binary.flatten())[:, 0]
        if n < len(occupied):
            occupied = occupied[torch.randint(len(occupied), (n,), device=self.device)]
        return torch.cat([uniform, occupied], dim=0)

    @torch.no_grad()
    def _update(self, step: int, occ_eval_fn: Callable, occ_thre: float = 0.01,
                ema_decay: float = 0.95, warmup_steps: int = 256) -> None:
        _need_cuda(self.occs)
        if step < warmup_steps:
            cells = None
        else:
            cells = self._sample_uniform_and_occupied_cells(self.num_cells // 4).contiguous()
        n = self.num_cells if cells is None else cells.numel()
        jitter = torch.rand((n, 3), device=self.device)
        self._update_cells(cells, jitter, occ_eval_fn, occ_thre, ema_decay)

    @torch.no_grad()
    def _update_cells(self, cells: Optional[Tensor], jitter: Tensor, occ_eval_fn: Callable,
                      occ_thre: float, ema_decay: float) -> None:
        """The body of ``_update`` for given cells (None = every cell) and
        jitter (n, 3) in [0, 1): query points, occupancy, EMA, binarisation."""
        _need_cuda(self.occs)
        if self._contraction_type == ContractionType.UN_BOUNDED_SPHERE:
            raise NotImplementedError("UN_BOUNDED_SPHERE occupancy updates are not on SuperNormal's path")
        n = self.num_cells if cells is None else cells.numel()
        rx, ry, rz = (int(r) for r in self.resolution.tolist())
        jitter = jitter.contiguous().float()
        x = torch.empty((n, 3), device=self.device)
        st = stream_handle()
        call("sn_occ_points", n, cells, jitter, rx, ry, rz, self._roi_aabb.contiguous().float(),
             self._contraction_type.value, x, st)
        occ = occ_eval_fn(x).squeeze(-1).contiguous().float()
        vals = torch.empty((n,), device=self.device) if cells is not None else None
        call("sn_occ_ema_update", n, cells, occ, float(ema_decay), self.occs, vals, st)
        ws = _ws(int(call("sn_occ_binarize_workspace_bytes", self.num_cells)), self.device)
        binary = torch.empty_like(self._binary)
        call("sn_occ_binarize", self.num_cells, self.occs, float(occ_thre), binary.view(torch.uint8),
             None, ws, st)
        self._binary = binary

    @torch.no_grad()
    def every_n_step(self, step: int, occ_eval_fn: Callable, occ_thre: float = 1e-2,
                     ema_decay: float = 0.95, warmup_steps: int = 256, n: int = 16) -> None:
        if not self.training:
            raise RuntimeError(
                "You should only call this function only during training. "
                "Please call _update() directly if you want to update the "
                "field during inference.")
        if step % n == 0 and self.training:
            self._update(step=step, occ_eval_fn=occ_eval_fn, occ_thre=occ_thre,
                         ema_decay=ema_decay, warmup_steps=warmup_steps)

    @torch.no_grad()
    def query_occ(self, samples: Tensor) -> Tensor:
        return query_grid(samples, self._roi_aabb, self.binary, self.contraction_type)


@torch.no_grad()
def ray_aabb_intersect(rays_o: Tensor, rays_d: Tensor, aabb: Tensor) -> Tuple[Tensor, Tensor]:
    """Slab test (NA/nerfacc/intersection.py); off SuperNormal's path (it passes
    explicit t_min/t_max), provided for API completeness with tensor ops."""
    inv = 1.0 / rays_d
    t0 = (aabb[:3] - rays_o) * inv
    t1 = (aabb[3:] - rays_o) * inv
    tmin = torch.minimum(t0, t1).amax(-1).clamp_min(0.0)
    tmax = torch.maximum(t0, t1).amin(-1)
    miss = tmax <= tmin
    tmin = torch.where(miss, torch.full_like(tmin, 1e10), tmin)
    tmax = torch.where(miss, torch.full_like(tmax, 1e10), tmax)
    return tmin, tmax


# ---------------------------------------------------------------------------
# marching (NA/nerfacc/ray_marching.py)
# ---------------------------------------------------------------------------
def _grid_args(grid: Optional[Grid], device):
    if grid is not None:
        roi = grid.roi_aabb.contiguous().float()
        binary = grid.binary.contiguous()
        ctype = grid.contraction_type.value
    else:
        roi = torch.tensor([-1e10, -1e10, -1e10, 1e10, 1e10, 1e10], dtype=torch.float32, device=device)
        binary = torch.ones([1, 1, 1], dtype=torch.bool, device=device)
        ctype = ContractionType.AABB.value
    if binary.dtype != torch.bool:
        raise TypeError("grid.binary must be a torch.bool tensor")
    rx, ry, rz = binary.shape
    return roi, binary.view(torch.uint8), rx, ry, rz, ctype


def _check_status(status: Tensor) -> None:
    v = int(status.item())
    if v & SN_STATUS_MARCH_LIMIT:
        raise RuntimeError("ray_marching: a ray exceeded the marching iteration limit "
                           "(step size too small for its [t_min, t_max] range)")
    if v & SN_STATUS_CAPACITY:
        raise RuntimeError("ray_marching: sample buffer capacity exceeded")


def march_packed(rays_o: Tensor, rays_d: Tensor, t_min: Tensor, t_max: Tensor,
                 grid: Optional[Grid], render_step_size: float, cone_angle: float = 0.0,
                 jitter: Optional[Tensor] = None):
    """Marcher core: returns packed_info, ray_indices, t_starts (N,1), t_ends (N,1)."""
    dev = rays_o.device
    n = rays_o.shape[0]
    roi, binary, rx, ry, rz, ctype = _grid_args(grid, dev)
    st = stream_handle()
    status = torch.zeros((1,), dtype=torch.int32, device=dev)
    counts = torch.empty((n,), dtype=torch.int32, device=dev)
    args = (rays_o, rays_d, t_min, t_max, jitter, roi, binary, rx, ry, rz, ctype,
            float(render_step_size), float(cone_angle), 0)
    call("sn_march_count", n, *args, counts, status, st)
    packed, total = _pack_counts(counts)
    n_samples = int(total.item())
    _check_status(status)
    ray_indices = torch.empty((n_samples,), dtype=torch.int64, device=dev)
    t_starts = torch.empty((n_samples, 1), dtype=torch.float32, device=dev)
    t_ends = torch.empty((n_samples, 1), dtype=torch.float32, device=dev)
    call("sn_march_fill", n, *args, packed, n_samples, ray_indices, t_starts, t_ends, status, st)
    return packed, ray_indices, t_starts, t_ends


@torch.no_grad()
def ray_marching(rays_o: Tensor, rays_d: Tensor, t_min: Optional[Tensor] = None,
                 t_max: Optional[Tensor] = None, scene_aabb: Optional[Tensor] = None,
                 grid: Optional[Grid] = None, sigma_fn: Optional[Callable] = None,
                 alpha_fn: Optional[Callable] = None, early_stop_eps: float = 1e-4,
                 alpha_thre: float = 0.0, near_plane: Optional[float] = None,
                 far_plane: Optional[float] = None, render_step_size: float = 1e-3,
                 stratified: bool = False, cone_angle: float = 0.0,
                 generator: Optional[torch.Generator] = None
                 ) -> Tuple[Tensor, Tensor, Tensor]:
    """Ray marching with occupancy-grid skipping and visibility culling
    (NA/nerfacc/ray_marching.py:13-222): returns ray_indices (N,) int64,
    t_starts (N, 1), t_ends (N, 1).  ``generator`` (an addition) draws the
    stratified jitter, so that a render can be reproduced."""
    _need_cuda(rays_o)
    if alpha_fn is not None and sigma_fn is not None:
        raise ValueError("Only one of `alpha_fn` and `sigma_fn` should be provided.")
    if t_min is None or t_max is None:
        if scene_aabb is not None:
            t_min, t_max = ray_aabb_intersect(rays_o, rays_d, scene_aabb)
        else:
            t_min = torch.zeros_like(rays_o[..., 0])
            t_max = torch.ones_like(rays_o[..., 0]) * 1e10
    if near_plane is not None:
        t_min = torch.clamp(t_min, min=near_plane)
    if far_plane is not None:
        t_max = torch.clamp(t_max, max=far_plane)
    rays_o = rays_o.contiguous().float()
    rays_d = rays_d.contiguous().float()
    t_min = t_min.contiguous().float()
    t_max = t_max.contiguous().float()
    jitter = (torch.rand(t_min.shape, dtype=t_min.dtype, device=t_min.device, generator=generator)
              if stratified else None)
    packed, ray_indices, t_starts, t_ends = march_packed(
        rays_o, rays_d, t_min, t_max, grid, render_step_size, cone_angle, jitter)
    if sigma_fn is not None or alpha_fn is not None:
        if sigma_fn is not None:
            sigmas = sigma_fn(t_starts, t_ends, ray_indices)
            assert sigmas.shape == t_starts.shape, \
                "sigmas must have shape of (N, 1)! Got {}".format(sigmas.shape)
            alphas = 1.0 - torch.exp(-sigmas * (t_ends - t_starts))
        else:
            alphas = alpha_fn(t_starts, t_ends, ray_indices)
            assert alphas.shape == t_starts.shape, \
                "alphas must have shape of (N, 1)! Got {}".format(alphas.shape)
        ray_indices, t_starts, t_ends = _cull(packed, ray_indices, t_starts, t_ends,
                                              alphas.contiguous().float(), early_stop_eps, alpha_thre)
    return ray_indices, t_starts, t_ends


def _cull(packed, ray_indices, t_starts, t_ends, alphas, early_stop_eps, alpha_thre):
    dev = alphas.device
    n_rays = packed.shape[0]
    st = stream_handle()
    vis = torch.empty((alphas.shape[0],), dtype=torch.uint8, device=dev)
    counts = torch.empty((n_rays,), dtype=torch.int32, device=dev)
    call("sn_visibility_from_alpha", n_rays, packed, alphas, float(early_stop_eps),
         float(alpha_thre), vis, counts, st)
    packed_out, total = _pack_counts(counts)
    n = int(total.item())
    ri = torch.empty((n,), dtype=torch.int64, device=dev)
    ts = torch.empty((n, 1), dtype=torch.float32, device=dev)
    te = torch.empty((n, 1), dtype=torch.float32, device=dev)
    call("sn_compact_samples", n_rays, packed, vis, packed_out, ray_indices, t_starts, t_ends,
         ri, ts, te, st)
    return ri, ts, te


# ---------------------------------------------------------------------------
# volume rendering (NA/nerfacc/vol_rendering.py)
# ---------------------------------------------------------------------------
@torch.no_grad()
def render_visibility(alphas: Tensor, *, ray_indices: Optional[Tensor] = None,
                      packed_info: Optional[Tensor] = None, n_rays: Optional[int] = None,
                      early_stop_eps: float = 1e-4, alpha_thre: float = 0.0) -> Tensor:
    """Visible samples: T >= early_stop_eps and alpha >= alpha_thre
    (NA/nerfacc/vol_rendering.py:680-748).  Returns bool (n_samples,)."""
    assert ray_indices is not None or packed_info is not None, \
        "Either ray_indices or packed_info should be provided."
    _need_cuda(alphas)
    if packed_info is None:
        packed_info = pack_info(ray_indices, n_rays=n_rays)
    packed_info = packed_info.contiguous().int()
    alphas = alphas.contiguous().float()
    vis = torch.empty((alphas.shape[0],), dtype=torch.bool, device=alphas.device)
    call("sn_visibility_from_alpha", packed_info.shape[0], packed_info, alphas,
         float(early_stop_eps), float(alpha_thre), vis.view(torch.uint8), None, stream_handle())
    return vis


@torch.no_grad()
def render_transmittance_from_alpha(alphas: Tensor, *, packed_info: Optional[Tensor] = None,
                                    ray_indices: Optional[Tensor] = None,
                                    n_rays: Optional[int] = None) -> Tensor:
    """Exclusive transmittance (NA/nerfacc/vol_rendering.py:406-460), forward only
    (SuperNormal uses it only under no_grad, through render_visibility)."""
    assert ray_indices is not None or packed_info is not None, \
        "Either ray_indices or packed_info should be provided."
    _need_cuda(alphas)
    if packed_info is None:
        packed_info = pack_info(ray_indices, n_rays=n_rays)
    packed_info = packed_info.contiguous().int()
    alphas = alphas.contiguous().float()
    out = torch.empty_like(alphas)
    call("sn_transmittance_from_alpha", packed_info.shape[0], 1, packed_info, alphas, out,
         stream_handle())
    return out


class _WeightFromAlpha(torch.autograd.Function):
    """w = alpha * T per (ray, pixel lane); backward is the reference's formula
    (NA/nerfacc/cuda/csrc/render_weight.cu:87-118, :298-340)."""

    @staticmethod
    def forward(ctx, packed_info: Tensor, alphas: Tensor, patch_size: int):
        packed_info = packed_info.contiguous().int()
        alphas = alphas.contiguous().float()
        weights = torch.empty_like(alphas)
        call("sn_weight_from_alpha_fwd", packed_info.shape[0], patch_size, packed_info, alphas,
             weights, stream_handle())
        ctx.patch_size = patch_size
        if ctx.needs_input_grad[1]:
            ctx.save_for_backward(packed_info, alphas, weights)
        return weights

    @staticmethod
    def backward(ctx, grad_weights: Tensor):
        packed_info, alphas, weights = ctx.saved_tensors
        grad_weights = grad_weights.contiguous().float()
        grad_alphas = torch.empty_like(alphas)
        call("sn_weight_from_alpha_bwd", packed_info.shape[0], ctx.patch_size, packed_info, alphas,
             weights, grad_weights, grad_alphas, stream_handle())
        return None, grad_alphas, None


def render_weight_from_alpha(alphas: Tensor, *, packed_info: Optional[Tensor] = None,
                             ray_indices: Optional[Tensor] = None,
                             n_rays: Optional[int] = None) -> Tensor:
    """Weights w_i = alpha_i prod_{j<i}(1 - alpha_j) (NA/nerfacc/vol_rendering.py:624-678)."""
    assert ray_indices is not None or packed_info is not None, \
        "Either ray_indices or packed_info should be provided."
    _need_cuda(alphas)
    if packed_info is None:
        packed_info = pack_info(ray_indices, n_rays=n_rays)
    return _WeightFromAlpha.apply(packed_info, alphas, 1)


def render_weight_from_alpha_patch_based(alphas: Tensor, ray_indices: Tensor, *,
                                         n_rays: Optional[int] = None) -> Tensor:
    """Patch weights for alphas (n_samples, patch_size, 1) grouped by patch index
    (NA/nerfacc/vol_rendering.py:533-576)."""
    _need_cuda(alphas)
    packed_info = pack_info(ray_indices, n_rays=n_rays)
    return _WeightFromAlpha.apply(packed_info, alphas, alphas.shape[1])


class _Accumulate(torch.autograd.Function):
    @staticmethod
    def forward(ctx, weights: Tensor, values: Optional[Tensor], ray_indices: Tensor, n_rays: int,
                patch_size: int, dim: int):
        weights = weights.contiguous().float()
        ray_indices = ray_indices.contiguous().long()
        vals = values.contiguous().float() if values is not None else None
        out = torch.empty((n_rays, patch_size, dim), dtype=torch.float32, device=weights.device)
        call("sn_accumulate_fwd", ray_indices.numel(), patch_size, dim, ray_indices, weights, vals,
             n_rays, out, stream_handle())
        ctx.save_for_backward(weights, vals if vals is not None else torch.empty(0), ray_indices)
        ctx.has_values = vals is not None
        ctx.shape = (patch_size, dim)
        return out

    @staticmethod
    def backward(ctx, grad_out: Tensor):
        weights, vals, ray_indices = ctx.saved_tensors
        vals = vals if ctx.has_values else None
        P, D = ctx.shape
        grad_out = grad_out.contiguous().float()
        gw = torch.empty_like(weights) if ctx.needs_input_grad[0] else None
        gv = torch.empty_like(vals) if (vals is not None and ctx.needs_input_grad[1]) else None
        call("sn_accumulate_bwd", ray_indices.numel(), P, D, ray_indices, weights, vals, grad_out,
             gw, gv, stream_handle())
        return gw, gv, None, None, None, None


def accumulate_along_rays(weights: Tensor, ray_indices: Tensor, values: Optional[Tensor] = None,
                          n_rays: Optional[int] = None) -> Tensor:
    """sum of weights * values per ray (NA/nerfacc/vol_rendering.py:132-197) -> (n_rays, D)."""
    assert ray_indices.dim() == 1 and weights.dim() == 2
    _need_cuda(weights)
    if values is not None:
        assert values.dim() == 2 and values.shape[0] == weights.shape[0], \
            "Invalid shapes: {} vs {}".format(values.shape, weights.shape)
        dim = values.shape[-1]
    else:
        dim = 1
    if ray_indices.numel() == 0:
        assert n_rays is not None
        return torch.zeros((n_rays, dim), device=weights.device)
    if n_rays is None:
        n_rays = int(ray_indices.max()) + 1
    out = _Accumulate.apply(weights.reshape(-1, 1, 1),
                            values.reshape(values.shape[0], 1, dim) if values is not None else None,
                            ray_indices, n_rays, 1, dim)
    return out.reshape(n_rays, dim)


def accumulate_along_rays_patch_based(weights: Tensor, ray_indices: Tensor,
                                      values: Optional[Tensor] = None,
                                      n_patches: Optional[int] = None) -> Tensor:
    """Per-pixel sums over a patch's samples (NA/nerfacc/vol_rendering.py:269-335)
    -> (n_patches, patch_size, D)."""
    assert ray_indices.dim() == 1 and weights.dim() == 3
    _need_cuda(weights)
    if values is not None:
        assert values.dim() == 3 and values.shape[0] == weights.shape[0], \
            "Invalid shapes: {} vs {}".format(values.shape, weights.shape)
        dim = values.shape[-1]
    else:
        dim = weights.shape[-1]
    if ray_indices.numel() == 0:
        assert n_patches is not None
        return torch.zeros((n_patches, weights.shape[1], dim), device=weights.device)
    if n_patches is None:
        n_patches = int(ray_indices.max()) + 1
    return _Accumulate.apply(weights, values, ray_indices, n_patches, weights.shape[1], dim)
