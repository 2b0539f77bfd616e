"""Fused SuperNormal training step: one iteration of Runner.train() on device.

Reproduces exp_runner.py:147-210 for the 'dfd' gradient method: occupancy
update every n steps, centre-ray marching with stratified jitter, SDF-alpha
culling, patch expansion, one field evaluation for every patch pixel, NeuS
alpha + patch weights + dfd normals + accumulation + losses + adjoint in one
kernel, the field backward, weight-norm adjoints, the warm-up/cosine learning
rate and Adam.  Every size that depends on the data (samples marched,
samples kept, extra end points, field points) lives in device memory, all
buffers have fixed capacity, and kernels bound their work by those device
counts, so a step issues no host synchronisation and can be captured in a
CUDA graph.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass
from typing import Optional

import torch
from torch import Tensor

from ._lib import (SN_FIELD_MLP_TF32, SN_FIELD_TABLE_FP16, SN_STATUS_CAPACITY, SN_STATUS_MARCH_LIMIT,
                   SN_STATUS_TIMEOUT, call, lib, stream_handle)
from .fields import SDFNetwork, SingleVarianceNetwork

__all__ = ["TrainConfig", "FusedTrainer"]


@dataclass
class TrainConfig:
    batch_size: int = 2048
    patch_h: int = 3
    patch_w: int = 3
    step_size: float = 2.0 / 1024.0       # fixed marching step (config: <=1024 samples per chord)
    start_step_size: Optional[float] = None   # log schedule (exp_runner.py:81-83,149) when set
    end_step_size: Optional[float] = None
    end_iter: int = 5000
    learning_rate: float = 5e-4
    learning_rate_alpha: float = 0.05
    warm_up_end: int = 50
    increase_bandwidth_every: int = 300
    occ_update_freq: int = 8
    occ_threshold: float = 0.1
    occ_ema_decay: float = 0.95
    occ_warmup_steps: int = 256
    occ_sigmoid_k: float = 80.0
    early_stop_eps: float = 1e-8
    loss_type: str = "l2"
    gradient_method: str = "dfd"            # 'dfd' (shipped) or 'ad' (second-order adjoint)
    precision: str = "fp32"                 # 'fp32' or 'mixed' (FP16 table copy, one-pass TF32 MLP)
    encoding_cache: bool = True             # field forward keeps the encoding for the backward
    normal_weight: float = 1.0
    eikonal_weight: float = 1.0
    mask_weight: float = 1.0
    seed: int = 0


def _align4(n: int) -> int:
    return (n + 3) // 4 * 4


class FusedTrainer:
    """Owns flat parameter / gradient / Adam buffers and fixed-capacity step buffers.

    The network's parameters become views into one flat buffer (their
    ``.data`` and ``.grad`` are re-pointed), so the modules, their
    state_dicts and this trainer always agree."""

    def __init__(self, sdf_network: SDFNetwork, deviation_network: SingleVarianceNetwork,
                 cfg: TrainConfig, occupancy_grid=None, device="cuda"):
        self.net, self.dev_net, self.cfg = sdf_network, deviation_network, cfg
        self.device = torch.device(device)
        if not sdf_network._supported:
            raise NotImplementedError("FusedTrainer needs the fused-field SDFNetwork shape")
        if cfg.patch_h < 3 or cfg.patch_w < 3 or cfg.patch_h * cfg.patch_w > 32:
            raise ValueError("patch must be at least 3x3 and at most 32 pixels")
        dev = self.device
        self.P = cfg.patch_h * cfg.patch_w
        self.B = cfg.batch_size
        # ---- flat parameters (table first: float2 aligned) ----
        named = [("table", sdf_network.encoding.params)]
        for l in (0, 1):
            lin = getattr(sdf_network, f"lin{l}")
            named += [(f"v{l}", lin.weight_v), (f"g{l}", lin.weight_g), (f"b{l}", lin.bias)]
        named.append(("variance", deviation_network.variance))
        offs, o = {}, 0
        for name, p in named:
            offs[name] = (o, p.numel(), tuple(p.shape))
            o += _align4(p.numel())
        self.n_params = o
        self.params = torch.zeros(o, device=dev)
        self.grads = torch.zeros(o, device=dev)
        self.exp_avg = torch.zeros(o, device=dev)
        self.exp_avg_sq = torch.zeros(o, device=dev)
        self.views, self.gviews = {}, {}
        with torch.no_grad():
            for name, p in named:
                a, n, shape = offs[name]
                self.params[a:a + n].copy_(p.detach().reshape(-1).to(dev))
                v = self.params[a:a + n].view(shape)
                gv = self.grads[a:a + n].view(shape)
                p.data = v
                p.grad = gv
                self.views[name], self.gviews[name] = v, gv
        self.offsets = offs
        if cfg.precision not in ("fp32", "mixed"):
            raise ValueError(f"precision {cfg.precision!r}: 'fp32' or 'mixed'")
        if cfg.precision == "mixed" and cfg.gradient_method != "dfd":
            raise NotImplementedError("mixed precision is built for the dfd gradient path")
        # mixed: the field kernels read an FP16 copy of the table, refreshed by
        # every Adam step from the FP32 master weights (gradients stay FP32)
        self.params_half = None
        if cfg.precision == "mixed":
            self.params_half = self.params.to(torch.float16)
        self.table_numel = offs["table"][1]
        self.H = sdf_network.d_hidden
        self.dout = sdf_network.d_out
        self.din = sdf_network.lin0.in_features
        self.w0 = torch.empty((self.H, self.din), device=dev)
        self.w1 = torch.empty((self.dout, self.H), device=dev)
        self.n0 = torch.empty((self.H,), device=dev)
        self.n1 = torch.empty((self.dout,), device=dev)
        self.dw0 = torch.zeros_like(self.w0)
        self.dw1 = torch.zeros_like(self.w1)
        # ---- occupancy grid ----
        from .nerfacc import OccupancyGrid
        self.grid = occupancy_grid if occupancy_grid is not None else OccupancyGrid(
            roi_aabb=[-1.0, -1.0, -1.0, 1.0, 1.0, 1.0], resolution=128).to(dev)
        self.res = tuple(int(r) for r in self.grid.resolution.tolist())
        self.n_cells = self.res[0] * self.res[1] * self.res[2]
        self.occ_cells = torch.empty((2 * (self.n_cells // 4),), dtype=torch.int64, device=dev)
        self.occ_count = torch.zeros((1,), dtype=torch.int32, device=dev)
        self.occ_xyz = torch.empty((self.n_cells, 3), device=dev)
        self.occ_sdf = torch.empty((self.n_cells, 1), device=dev)
        self.occ_vals = torch.empty((2 * (self.n_cells // 4),), device=dev)
        self.occ_ws = torch.empty(int(call("sn_occ_sample_workspace_bytes", self.n_cells)),
                                  dtype=torch.uint8, device=dev)
        self.bin_ws = torch.empty(int(call("sn_occ_binarize_workspace_bytes", self.n_cells)),
                                  dtype=torch.uint8, device=dev)
        # ---- device scalars ----
        self.iter_dev = torch.zeros((1,), dtype=torch.int32, device=dev)
        self.dt_dev = torch.zeros((1,), device=dev)   # marching step of the step-size schedule
        self.lr_dev = torch.zeros((1,), device=dev)
        self.adam_step_dev = torch.zeros((1,), dtype=torch.int32, device=dev)
        self.status = torch.zeros((1,), dtype=torch.int32, device=dev)
        self.loss_out = torch.zeros((5,), device=dev)
        self.mask_sum = torch.zeros((1,), device=dev)
        self.iter_step = 0
        self.profile = False        # when True, CUDA events mark the stages of each step
        self.marks: list = []       # [(tag, torch.cuda.Event)] of the steps run while profiling
        self.q_hist: list = []      # device copies of the training field-point count per step
        self._capturing = False
        self._alloc_step_buffers(self._max_step_size_for_capacity())

    def _mark(self, tag: str) -> None:
        if self.profile:
            # under graph capture the event becomes a node of the graph
            ev = torch.cuda.Event(enable_timing=True, external=self._capturing)
            ev.record(torch.cuda.current_stream())
            self.marks.append((tag, ev))

    # ------------------------------------------------------------------
    def _max_step_size_for_capacity(self) -> float:
        c = self.cfg
        if c.start_step_size is not None:
            return min(c.start_step_size, c.end_step_size or c.start_step_size)
        return c.step_size

    def _alloc_step_buffers(self, min_step: float) -> None:
        dev, B, P = self.device, self.B, self.P
        # a unit-sphere chord is at most 2 long: bound on samples per centre ray
        self.max_steps = int(math.ceil(2.0 / min_step)) + 3
        C0 = B * self.max_steps
        self.C0 = C0
        i32 = dict(dtype=torch.int32, device=dev)
        self.near = torch.empty((B,), device=dev)
        self.far = torch.empty((B,), device=dev)
        self.ro_c = torch.empty((B, 3), device=dev)
        self.rd_c = torch.empty((B, 3), device=dev)
        self.jitter = torch.empty((B,), device=dev)
        self.counts0 = torch.empty((B,), **i32)
        self.packed0 = torch.empty((B, 2), **i32)
        self.total0 = torch.zeros((1,), **i32)
        self.ridx0 = torch.empty((C0,), dtype=torch.int64, device=dev)
        self.ts0 = torch.empty((C0,), device=dev)
        self.te0 = torch.empty((C0,), device=dev)
        self.ridx_pad = torch.empty((C0,), dtype=torch.int64, device=dev)
        self.ts_pad = torch.empty((C0,), device=dev)
        self.te_pad = torch.empty((C0,), device=dev)
        self.diff = torch.empty((C0,), **i32)
        self.endp = torch.empty((C0, 2), **i32)
        self.n_ends = torch.zeros((1,), **i32)
        self.q0 = torch.zeros((1,), **i32)
        self.xyz0 = torch.empty((2 * C0, 3), device=dev)
        self.sdf0 = torch.empty((2 * C0, 1), device=dev)
        self.alpha0 = torch.empty((C0,), device=dev)
        self.vis = torch.empty((C0,), dtype=torch.uint8, device=dev)
        self.counts1 = torch.empty((B,), **i32)
        self.packed1 = torch.empty((B, 2), **i32)
        self.S = torch.zeros((1,), **i32)
        self.ridx1 = torch.empty((C0,), dtype=torch.int64, device=dev)
        self.ts1 = torch.empty((C0,), device=dev)
        self.te1 = torch.empty((C0,), device=dev)
        self.endp1 = torch.empty((C0, 2), **i32)
        self.n_ends1 = torch.zeros((1,), **i32)
        self.q1 = torch.zeros((1,), **i32)
        self.xyz1 = torch.empty((2 * C0 * P, 3), device=dev)
        self.tps = torch.empty((C0, P), device=dev)
        self.tpe = torch.empty((C0, P), device=dev)
        self.sdf1 = torch.empty((2 * C0 * P, 1), device=dev)
        self.d_sdf = torch.empty((2 * C0 * P, 1), device=dev)
        # encoding of the training points, level-major (n_levels x 2 x capacity floats)
        self.enc_cache = (torch.empty((self.net.encoding.n_levels * 2 * 2 * C0 * P,), device=dev)
                          if self.cfg.encoding_cache else None)
        self.partials = torch.zeros((B, 4), device=dev)
        self.carry = torch.empty((B, P), device=dev)
        if self.cfg.gradient_method == "ad":
            self.sp_count = torch.zeros((1,), **i32)
            self.ext_g = torch.empty((C0 * P, 3), device=dev)
            self.d_ext = torch.empty((C0 * P, 3), device=dev)
        self.mask_bin = torch.empty((B, P), device=dev)
        ws_n = max(B, C0)
        self.scan_ws = torch.empty(int(call("sn_scan_workspace_bytes", ws_n)), dtype=torch.uint8,
                                   device=dev)

    # ------------------------------------------------------------------
    def _grid_desc(self):
        return C.byref(self.net.encoding.desc)

    def _table(self) -> Tensor:
        """The table the field kernels read: FP32 master or its FP16 copy."""
        if self.params_half is not None:
            return self.params_half[: self.table_numel]
        return self.views["table"]

    def _mlp(self):
        d = self.net._mlp_desc(self.w0, self.views["b0"], self.w1, self.views["b1"])
        d.status = self.status.data_ptr()
        if self.params_half is not None:
            d.flags = SN_FIELD_TABLE_FP16 | SN_FIELD_MLP_TF32
        return d

    def step_size(self, it: int) -> float:
        c = self.cfg
        if c.start_step_size is None:
            return c.step_size
        slop = (math.log10(c.start_step_size) - math.log10(c.end_step_size)) / c.end_iter
        return 10 ** (math.log10(c.start_step_size) - slop * it)

    def step_key(self, it: int):
        """What a captured iteration depends on besides its device state: the
        fixed step size, or None when the step follows the log schedule (the
        marcher then reads the step that sn_step_size_schedule writes on the
        device from the device iteration counter)."""
        return None if self.cfg.start_step_size is not None else self.cfg.step_size

    @torch.no_grad()
    def weight_norm_forward(self, st) -> None:
        v = self.views
        call("sn_weightnorm_fwd", self.H, self.din, v["v0"], v["g0"], self.w0, self.n0, st)
        call("sn_weightnorm_fwd", self.dout, self.H, v["v1"], v["g1"], self.w1, self.n1, st)

    @torch.no_grad()
    def occupancy_update(self, it: int) -> None:
        """OccupancyGrid.every_n_step body (NA/nerfacc/grid.py:196-239), on device."""
        c, st = self.cfg, stream_handle()
        g = self.grid
        roi = g._roi_aabb.contiguous().float()
        active = self.net.active_levels()
        self._mark("occ_begin")
        self.weight_norm_forward(st)
        seed = (c.seed * 1000003 + 17) & 0xFFFFFFFF
        if it < c.occ_warmup_steps:
            cells, cap, count = None, self.n_cells, None
        else:
            n_u = self.n_cells // 4
            call("sn_occ_sample_cells", self.n_cells, g._binary.view(torch.uint8), n_u, seed,
                 self.iter_dev, self.occ_cells, self.occ_count, self.occ_ws, st)
            cells, cap, count = self.occ_cells, 2 * n_u, self.occ_count
        call("sn_occ_points_n", cap, count, cells, seed ^ 0x9E37, self.iter_dev, *self.res, roi,
             g._contraction_type.value, self.occ_xyz, st)
        call("sn_field_fwd", cap, count, self.occ_xyz, self._table(), self._grid_desc(), active,
             C.byref(self._mlp()), 1, self.occ_sdf, st)
        call("sn_occ_ema_sdf", cap, count, cells, self.occ_sdf, float(c.occ_sigmoid_k),
             float(c.occ_ema_decay), g.occs, self.occ_vals, st)
        call("sn_occ_binarize", self.n_cells, g.occs, float(c.occ_threshold),
             g._binary.view(torch.uint8), None, self.bin_ws, st)
        self._mark("occ_end")

    @torch.no_grad()
    def train_step(self, rays_o: Tensor, rays_d: Tensor, plane_n: Tensor, vinv: Tensor,
                   normal: Tensor, mask: Tensor) -> Tensor:
        """One iteration on a batch from gen_random_patches; returns the
        device loss vector {d/d variance, normal, mask BCE, eikonal, total}."""
        c, st = self.cfg, stream_handle()
        it = self.iter_step
        if c.occ_update_freq > 0 and it % c.occ_update_freq == 0:
            self.occupancy_update(it)
        if c.increase_bandwidth_every > 0 and it % c.increase_bandwidth_every == 0:
            self.net.increase_bandwidth()
        self.run_step(rays_o, rays_d, plane_n, vinv, normal, mask, self.step_key(it),
                      self.net.active_levels())
        self.iter_step += 1
        return self.loss_out

    @torch.no_grad()
    def run_step(self, rays_o, rays_d, plane_n, vinv, normal, mask, dt, active: int) -> None:
        """The capturable part of an iteration (fixed bandwidth; dt fixed, or
        None for the device-side step-size schedule)."""
        self.forward_backward(rays_o, rays_d, plane_n, vinv, normal, mask, dt, active)
        self.optimizer_step()

    @torch.no_grad()
    def optimizer_step(self) -> None:
        """Learning-rate schedule and Adam over the flat parameters (zeroes grads)."""
        c, st = self.cfg, stream_handle()
        call("sn_lr_schedule", self.iter_dev, self.lr_dev, self.adam_step_dev, float(c.learning_rate),
             int(c.warm_up_end), int(c.end_iter), float(c.learning_rate_alpha), st)
        self._mark("adam_begin")
        call("sn_adam_step", self.n_params, self.params, self.grads, self.exp_avg, self.exp_avg_sq,
             self.params_half, self.lr_dev, self.adam_step_dev, 0.0, 1, 0.9, 0.999, 1e-8, 1, st)
        self._mark("adam_end")

    @torch.no_grad()
    def forward_backward(self, rays_o, rays_d, plane_n, vinv, normal, mask, dt,
                         active: int) -> None:
        """Loss and gradients (accumulated into the flat gradient buffer).
        dt: the marching step, or None to take it from the configured log
        schedule at the device iteration counter."""
        c, st = self.cfg, stream_handle()
        B, P, H, W, C0 = self.B, self.P, c.patch_h, c.patch_w, self.C0
        assert rays_o.shape[0] == B and rays_o.is_contiguous() and rays_d.is_contiguous()
        v = self.views
        roi = self.grid._roi_aabb
        binary = self.grid._binary.view(torch.uint8)
        rx, ry, rz = self.res
        ctype = self.grid._contraction_type.value
        gd = self._grid_desc()
        kc = (H // 2) * W + W // 2
        seed = (c.seed * 7919 + 1) & 0xFFFFFFFF
        self._mark("step_begin")
        self.weight_norm_forward(st)
        mlp = C.byref(self._mlp())
        mlp_pts = self._mlp()      # training points: the forward fills the encoding cache
        if self.enc_cache is not None:
            mlp_pts.enc_cache = self.enc_cache.data_ptr()
        mlp_pts = C.byref(mlp_pts)
        # --- inputs: mask binarisation, near/far and jitter of the centre rays ---
        call("sn_mask_prep", B * P, mask, self.mask_bin, self.mask_sum, st)
        call("sn_near_far_sphere", B, _center_ptr(rays_o, kc), _center_ptr(rays_d, kc), 3 * P,
             self.near, self.far, self.jitter, seed, self.iter_dev, self.ro_c, self.rd_c, st)
        # --- marching over the centre rays: one pass into per-ray slots, scan, pack ---
        dt_dev = None
        if dt is None:
            call("sn_step_size_schedule", self.iter_dev, float(c.start_step_size), float(c.end_step_size),
                 int(c.end_iter), self.dt_dev, st)
            dt_dev, dt = self.dt_dev, c.start_step_size
        call("sn_march_padded", B, self.ro_c, self.rd_c, self.near, self.far, self.jitter, roi, binary,
             rx, ry, rz, ctype, float(dt), dt_dev, 0.0, 0, self.max_steps, self.counts0, self.ridx_pad,
             self.ts_pad, self.te_pad, self.status, st)
        call("sn_pack_counts", B, self.counts0, self.packed0, self.total0, self.scan_ws, st)
        call("sn_compact_padded", B, self.max_steps, self.packed0, self.ridx_pad, self.ts_pad,
             self.te_pad, self.ridx0, self.ts0, self.te0, st)
        self._mark("march_end")
        # --- culling: field at centre samples, NeuS alpha, visibility, compaction ---
        call("sn_end_diff", C0, self.total0, self.ts0, self.te0, self.diff, st)
        call("sn_pack_counts_n", C0, self.total0, self.diff, self.endp, self.n_ends, self.scan_ws, st)
        call("sn_center_points", C0, self.total0, self.ridx0, self.ts0, self.te0, self.ro_c,
             self.rd_c, self.endp, self.n_ends, self.xyz0, self.q0, st)
        call("sn_field_fwd", 2 * C0, self.q0, self.xyz0, self._table(), gd, active, mlp, 1, self.sdf0, st)
        call("sn_center_alpha", C0, self.total0, self.sdf0, 1, self.endp, v["variance"], self.alpha0, st)
        call("sn_visibility_from_alpha", B, self.packed0, self.alpha0, float(c.early_stop_eps), 0.0,
             self.vis, self.counts1, st)
        call("sn_pack_counts", B, self.counts1, self.packed1, self.S, self.scan_ws, st)
        call("sn_compact_samples", B, self.packed0, self.vis, self.packed1, self.ridx0, self.ts0,
             self.te0, self.ridx1, self.ts1, self.te1, st)
        self._mark("cull_end")
        # --- training points: expansion through the marching plane ---
        call("sn_end_diff", C0, self.S, self.ts1, self.te1, self.diff, st)
        call("sn_pack_counts_n", C0, self.S, self.diff, self.endp1, self.n_ends1, self.scan_ws, st)
        call("sn_patch_points", C0, self.S, H, W, self.ridx1, self.ts1, self.te1, rays_o, rays_d,
             plane_n, self.endp1, self.n_ends1, self.xyz1, self.tps, self.tpe, self.q1, st)
        cap1 = 2 * C0 * P
        self._mark("field_fwd_begin")
        call("sn_field_fwd", cap1, self.q1, self.xyz1, self._table(), gd, active, mlp_pts, 1, self.sdf1, st)
        self._mark("field_fwd_end")
        if self.profile and not self._capturing:
            self.q_hist.append(self.q1.clone())   # field points of this step (device copy)
        ad = c.gradient_method == "ad"
        if ad:  # gradients = d sdf / dx at the start points (models/renderer.py:225-226)
            call("sn_scale_count", self.S, P, 0, self.sp_count, st)
            call("sn_field_grad_fwd", C0 * P, self.sp_count, self.xyz1, v["table"], gd, active, mlp,
                 None, self.ext_g, st)
        # --- render + loss + adjoint ---
        call("sn_patch_render_train", B, H, W, self.packed1, self.S, C0, self.endp1, self.sdf1,
             self.tps, self.tpe, rays_o, rays_d, vinv, v["variance"], normal, self.mask_bin,
             self.mask_sum, 1 if c.loss_type == "l1" else 0, float(c.normal_weight),
             float(c.eikonal_weight), float(c.mask_weight), self.d_sdf, self.partials, self.carry,
             self.ext_g if ad else None, self.d_ext if ad else None, st)
        call("sn_patch_carry_fixup", B, P, self.packed1, self.S, C0, self.endp1, self.carry,
             self.d_sdf, st)
        call("sn_patch_finalize", B, P, self.partials, self.S, C0, v["variance"], self.mask_sum,
             float(c.normal_weight), float(c.eikonal_weight), float(c.mask_weight), self.loss_out,
             self.gviews["variance"], st)
        self._mark("render_end")
        # --- field backward and weight-norm adjoints ---
        g = self.gviews
        self.dw0.zero_()
        self.dw1.zero_()
        self._mark("field_bwd_begin")
        call("sn_field_bwd", cap1, self.q1, self.xyz1, self.d_sdf, 1, self._table(), gd, active, mlp_pts,
             g["table"], self.dw0, g["b0"], self.dw1, g["b1"], None, st)
        if ad:  # second-order adjoint of the gradients
            call("sn_field_grad_bwd", C0 * P, self.sp_count, self.xyz1, self.d_ext, None, v["table"],
                 gd, active, mlp, g["table"], self.dw0, g["b0"], self.dw1, g["b1"], st)
        self._mark("field_bwd_end")
        call("sn_weightnorm_bwd", self.H, self.din, v["v0"], v["g0"], self.n0, self.dw0, g["v0"],
             g["g0"], st)
        call("sn_weightnorm_bwd", self.dout, self.H, v["v1"], v["g1"], self.n1, self.dw1, g["v1"],
             g["g1"], st)

    def set_precision(self, precision: str) -> None:
        """Switch between the FP32 field ('fp32') and the FP16 table copy with
        one-pass TF32 MLP products ('mixed'); the copy is formed from the FP32
        master weights (captured iterations must be re-captured)."""
        if precision not in ("fp32", "mixed"):
            raise ValueError(f"precision {precision!r}: 'fp32' or 'mixed'")
        if precision == self.cfg.precision:
            return
        if precision == "mixed" and self.cfg.gradient_method != "dfd":
            raise NotImplementedError("mixed precision is built for the dfd gradient path")
        self.cfg.precision = precision
        self.params_half = self.params.to(torch.float16) if precision == "mixed" else None

    # ---- checkpoints in the reference's layout (exp_runner.py:298-315) ----
    # The reference's optimizer is torch.optim.Adam over
    # list(sdf_network.parameters()) + list(deviation_network.parameters())
    # (exp_runner.py:89-97): the hash table, then per layer the parameters
    # weight_norm leaves (bias, weight_g, weight_v), then the variance.
    _REFERENCE_ORDER = ("table", "b0", "g0", "v0", "b1", "g1", "v1", "variance")

    def _reference_params(self):
        views = dict(self.views)
        return [views[k] for k in self._REFERENCE_ORDER]

    def _flat(self, buf: Tensor, name: str) -> Tensor:
        a, n, shape = self.offsets[name]
        return buf[a:a + n].view(shape)

    @torch.no_grad()
    def optimizer_state_dict(self) -> dict:
        """The torch.optim.Adam state_dict the reference would save: per
        parameter (in the reference's order) step, exp_avg, exp_avg_sq taken
        from the flat Adam buffers, and the current learning rate."""
        params = [p.detach().clone() for p in self._reference_params()]
        opt = torch.optim.Adam(params, lr=float(self.cfg.learning_rate), betas=(0.9, 0.999), eps=1e-8)
        steps = int(self.iter_dev.item())
        if steps > 0:
            for name, p in zip(self._REFERENCE_ORDER, params):
                opt.state[p] = {"step": torch.tensor(float(steps)),
                                "exp_avg": self._flat(self.exp_avg, name).clone(),
                                "exp_avg_sq": self._flat(self.exp_avg_sq, name).clone()}
        sd = opt.state_dict()
        sd["param_groups"][0]["lr"] = float(self.lr_dev.item()) if steps > 0 else float(self.cfg.learning_rate)
        return sd

    @torch.no_grad()
    def load_optimizer_state_dict(self, sd: dict) -> None:
        """Loads a torch.optim.Adam state_dict of the reference's optimizer
        (validated by torch itself) into the flat Adam buffers; the step
        count becomes the device iteration counter."""
        params = [p.detach().clone() for p in self._reference_params()]
        opt = torch.optim.Adam(params, lr=float(self.cfg.learning_rate))
        opt.load_state_dict(sd)
        steps = set()
        for name, p in zip(self._REFERENCE_ORDER, params):
            st = opt.state.get(p)
            if not st:
                self._flat(self.exp_avg, name).zero_()
                self._flat(self.exp_avg_sq, name).zero_()
                continue
            self._flat(self.exp_avg, name).copy_(st["exp_avg"])
            self._flat(self.exp_avg_sq, name).copy_(st["exp_avg_sq"])
            steps.add(int(float(st["step"])))
        if len(steps) > 1:
            raise ValueError(f"parameters have different Adam step counts {sorted(steps)}")
        k = steps.pop() if steps else 0
        self.iter_dev.fill_(k)

    def state_dict(self) -> dict:
        """Checkpoint with the reference's keys (exp_runner.py:305-310)."""
        return {"sdf_network_fine": self.net.state_dict(),
                "variance_network_fine": self.dev_net.state_dict(),
                "optimizer": self.optimizer_state_dict(),
                "iter_step": self.iter_step}

    @torch.no_grad()
    def load_state_dict(self, ckpt: dict) -> None:
        """Resumes from a checkpoint of the reference's layout
        (exp_runner.py:297-303); the parameters are copied into the flat
        buffers the kernels use (the module tensors stay views of them)."""
        self.net.load_state_dict(ckpt["sdf_network_fine"])
        self.dev_net.load_state_dict(ckpt["variance_network_fine"])
        self.load_optimizer_state_dict(ckpt["optimizer"])
        self.iter_step = int(ckpt["iter_step"])
        if self.params_half is not None:
            self.params_half.copy_(self.params)

    def save_checkpoint(self, path) -> None:
        torch.save(self.state_dict(), path)

    def load_checkpoint(self, path) -> None:
        self.load_state_dict(torch.load(path, map_location=self.device))

    def check_status(self) -> None:
        v = int(self.status.item())
        if v & SN_STATUS_MARCH_LIMIT:
            raise RuntimeError("marching iteration limit hit")
        if v & SN_STATUS_CAPACITY:
            raise RuntimeError("sample capacity exceeded")
        if v & SN_STATUS_TIMEOUT:
            raise RuntimeError("a tensor-core field kernel timed out waiting for its MMAs")


def _center_ptr(t: Tensor, kc: int) -> int:
    """Address of pixel kc of patch 0 in a (B, H, W, 3) tensor."""
    return t.data_ptr() + kc * 3 * t.element_size()


class HostPrefetcher:
    """Feeds a FusedTrainer from batches in pinned host memory.

    Two device slots: while step i runs on the current stream, batch i+1 is
    copied host -> device on a side stream, so the copies of every step stay
    inside the loop but overlap the previous step's kernels.  The side stream
    waits until the step that last read a slot has run before refilling it,
    and each step waits for its own batch's copies.

        pf = HostPrefetcher(trainer, host_batches[0])
        pf.put(host_batches[0])
        for i in range(n):
            loss = pf.step(host_batches[i + 1] if i + 1 < n else None)
    """

    def __init__(self, trainer: FusedTrainer, example: tuple, graph: "GraphStep | None" = None):
        dev = trainer.device
        self.tr = trainer
        self.graph = graph            # steps as CUDA-graph replays (the batch is copied into its inputs)
        self.slots = [tuple(torch.empty(t.shape, dtype=t.dtype, device=dev) for t in example) for _ in range(2)]
        self.copy_stream = torch.cuda.Stream(device=dev)
        self.ready = [torch.cuda.Event(), torch.cuda.Event()]
        self.free = [torch.cuda.Event(), torch.cuda.Event()]
        self.used = [False, False]   # a step has read the slot (its free event is recorded)
        self.next_slot = 0
        self.queue: list[int] = []   # slots holding (or receiving) put() batches, oldest first

    def put(self, host_batch: tuple) -> None:
        """Start copying a pinned host batch into the next slot (at most two batches ahead)."""
        if len(self.queue) == 2:
            raise RuntimeError("HostPrefetcher.put: both slots hold batches no step has consumed")
        slot = self.next_slot
        self.next_slot ^= 1
        start = torch.cuda.Event()
        start.record(torch.cuda.current_stream(self.tr.device))   # the copy follows its caller's point
        self.copy_stream.wait_event(start)
        if self.used[slot]:
            self.copy_stream.wait_event(self.free[slot])          # the step that read the slot has run
        with torch.cuda.stream(self.copy_stream):
            for dst, src in zip(self.slots[slot], host_batch):
                dst.copy_(src, non_blocking=True)
        self.ready[slot].record(self.copy_stream)
        self.queue.append(slot)

    def step(self, next_host_batch: tuple | None = None) -> Tensor:
        """One training step on the oldest put() batch; starts copying next_host_batch."""
        if not self.queue:
            raise RuntimeError("HostPrefetcher.step: no batch was put()")
        slot = self.queue.pop(0)
        main = torch.cuda.current_stream(self.tr.device)
        main.wait_event(self.ready[slot])
        if next_host_batch is not None:
            self.put(next_host_batch)
        if self.graph is not None:
            loss = self.graph.step(self.slots[slot])
        else:
            loss = self.tr.train_step(*self.slots[slot])
        self.free[slot].record(main)
        self.used[slot] = True
        return loss


class GraphStep:
    """A training iteration of a FusedTrainer as CUDA-graph replays.

    ``run_step`` (fixed step size and active levels) is captured over static
    input buffers; the post-warm-up occupancy update is captured too.  Both
    are re-captured when the step size or the bandwidth changes, and after
    the trainer's storages were reallocated (``invalidate``).  During the
    occupancy warm-up the update runs eagerly.

    ``profile=True`` captures the trainer's stage events into the graphs
    (event-record nodes) plus a copy of the step's field-point count into
    pinned memory, in three graph copies replayed in turn: a copy's events
    are read when it comes round again, after waiting for its previous
    replay while the two later steps are still queued, so profiling adds no
    gap between replays.  ``stage_marks`` then holds, per replayed step, the
    marks as (tag, ms from the first mark), ``points`` the field points,
    ``samples`` the marched and kept centre samples, and ``launches`` counts
    the library kernels replayed."""

    def __init__(self, trainer: FusedTrainer, profile: bool = False):
        self.tr = trainer
        c, dev = trainer.cfg, trainer.device
        B, H, W = trainer.B, c.patch_h, c.patch_w
        self.inputs = (torch.empty((B, H, W, 3), device=dev), torch.empty((B, H, W, 3), device=dev),
                       torch.empty((B, 3), device=dev), torch.empty((B, H, W, 3, 3), device=dev),
                       torch.empty((B, H, W, 3), device=dev), torch.empty((B, H, W, 1), device=dev))
        self.profile = profile
        self.n_copies = 3 if profile else 1
        self.stage_marks: list = []
        self.points: list = []
        self.samples: list = []    # per replayed step: (marched centre samples, kept samples)
        self.launches = 0
        self.captures = 0          # graphs captured so far (iteration copies and occupancy update)
        self.invalidate()

    def invalidate(self) -> None:
        self._steps = [None] * self.n_copies
        self._step_key = None
        self._next = 0
        self._occ = None

    def _capture(self, fn, snap_points: bool = False) -> dict:
        tr = self.tr
        torch.cuda.synchronize()
        self.flush()
        rec = {"graph": torch.cuda.CUDAGraph(), "pending": False,
               "q_host": torch.zeros((3,), dtype=torch.int32).pin_memory() if snap_points else None}
        prof = tr.profile
        tr.marks.clear()
        tr.profile, tr._capturing = self.profile, True
        n0 = lib().sn_kernel_launches()
        try:
            with torch.cuda.graph(rec["graph"]):
                fn()
                if snap_points and self.profile:
                    rec["q_host"][0:1].copy_(tr.q1, non_blocking=True)
                    rec["q_host"][1:2].copy_(tr.total0, non_blocking=True)
                    rec["q_host"][2:3].copy_(tr.S, non_blocking=True)
        finally:
            tr.profile, tr._capturing = prof, False
        rec["launches"] = lib().sn_kernel_launches() - n0
        self.captures += 1
        rec["marks"] = list(tr.marks)
        tr.marks.clear()
        return rec

    def _replay(self, rec: dict) -> None:
        self._harvest(rec)
        rec["graph"].replay()
        rec["pending"] = True
        self.launches += rec["launches"]

    def _harvest(self, rec) -> None:
        """Read a finished replay's marks (waits for that replay only)."""
        if rec is None or not rec["pending"]:
            return
        rec["pending"] = False
        if not self.profile or not rec["marks"]:
            return
        marks = rec["marks"]
        marks[-1][1].synchronize()
        t0 = marks[0][1]
        self.stage_marks.append([(tag, t0.elapsed_time(ev)) for tag, ev in marks])
        if rec["q_host"] is not None:
            q = rec["q_host"].tolist()
            self.points.append(q[0])
            self.samples.append((q[1], q[2]))

    def flush(self) -> None:
        """Wait for every replay and read the marks of those not read yet."""
        torch.cuda.synchronize()
        for rec in self._steps + [self._occ]:
            self._harvest(rec)

    def prepare(self) -> None:
        """Capture, ahead of the first replays, the graphs the coming
        iterations need at the current step size and bandwidth (the step
        copies and, past the occupancy warm-up, the occupancy update)."""
        tr, c = self.tr, self.tr.cfg
        it = tr.iter_step
        key = (tr.step_key(it), tr.net.active_levels())
        if key != self._step_key:
            self.flush()
            self._steps = [None] * self.n_copies
            self._step_key = key
            self._next = 0
        for k in range(self.n_copies):
            if self._steps[k] is None:
                self._steps[k] = self._capture(lambda: tr.run_step(*self.inputs, key[0], key[1]),
                                               snap_points=True)
        if c.occ_update_freq > 0 and it >= c.occ_warmup_steps and self._occ is None:
            self._occ = self._capture(lambda: tr.occupancy_update(c.occ_warmup_steps))

    def step(self, batch=None) -> Tensor:
        """One iteration; ``batch`` (6 tensors as from gen_random_patches) is
        copied into the static inputs, or the caller filled ``inputs``."""
        tr, c = self.tr, self.tr.cfg
        if tr.profile:
            raise RuntimeError("GraphStep replaces the trainer's eager stage events (profile=True here)")
        it = tr.iter_step
        if c.occ_update_freq > 0 and it % c.occ_update_freq == 0:
            if it < c.occ_warmup_steps:
                tr.occupancy_update(it)
            else:
                if self._occ is None:
                    self._occ = self._capture(lambda: tr.occupancy_update(c.occ_warmup_steps))
                self._replay(self._occ)
        if c.increase_bandwidth_every > 0 and it % c.increase_bandwidth_every == 0:
            tr.net.increase_bandwidth()
        if batch is not None:
            for dst, src in zip(self.inputs, batch):
                dst.copy_(src, non_blocking=True)
        key = (tr.step_key(it), tr.net.active_levels())
        if key != self._step_key:
            self.flush()
            self._steps = [None] * self.n_copies
            self._step_key = key
            self._next = 0
        k = self._next
        self._next = (k + 1) % self.n_copies
        if self._steps[k] is None:
            self._steps[k] = self._capture(lambda: tr.run_step(*self.inputs, key[0], key[1]), snap_points=True)
        self._replay(self._steps[k])
        tr.iter_step += 1
        return tr.loss_out
