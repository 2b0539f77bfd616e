"""SDF field modules: drop-in for models/fields.py on the sm_103a kernels.

``SDFNetwork`` keeps the reference constructor (models/fields.py:8-70), its
geometric initialisation (same torch RNG call sequence), its state_dict keys
(``encoding.params``, ``lin{l}.bias``, ``lin{l}.weight_g``,
``lin{l}.weight_v``), ``bindwidth`` / ``increase_bandwidth`` and the
``forward / sdf / gradient`` methods.  The hash-grid encoding (the
``tcnn.Encoding`` of models/fields.py:26) and the MLP run fused in one
kernel with a hand-written backward; the MLP shape the kernels cover is the
one SuperNormal ships: one hidden layer of 64 with input concatenation.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional

import numpy as np
import torch
import torch.nn as nn
from torch import Tensor

from ._lib import SN_STATUS_TIMEOUT, GridDesc, MlpDesc, call, lib, stream_handle

__all__ = ["HashGridEncoding", "WeightNormLinear", "SDFNetwork", "SingleVarianceNetwork",
           "grid_desc"]


def grid_desc(n_levels: int, n_features_per_level: int, log2_hashmap_size: int,
              base_resolution: int, per_level_scale: float) -> GridDesc:
    """tcnn GridEncoding level geometry (offsets, resolutions, scales)."""
    d = GridDesc()
    call("sn_grid_desc_init", C.byref(d), int(n_levels), int(n_features_per_level),
         int(log2_hashmap_size), int(base_resolution), float(per_level_scale))
    return d


def _need_cuda(t: Tensor) -> None:
    if not t.is_cuda:
        raise NotImplementedError("supernormal_gb300 fields run on CUDA tensors only")


class HashGridEncoding(nn.Module):
    """Multi-resolution hash encoding with tcnn's parameter layout; parameter
    ``params`` is the flat table (offsets[L] * F floats), initialised
    uniform(-1e-4, 1e-4) like tcnn's GridEncoding."""

    def __init__(self, n_input_dims: int, encoding_config: dict, seed: int = 1337,
                 dtype=torch.float32):
        super().__init__()
        otype = encoding_config.get("otype", "HashGrid")
        if otype not in ("HashGrid", "Grid") or encoding_config.get("type", "Hash") != "Hash":
            raise NotImplementedError(f"encoding otype {otype!r} is not supported (HashGrid only)")
        if n_input_dims != 3:
            raise NotImplementedError("only 3-D inputs are supported")
        if encoding_config.get("interpolation", "Linear") != "Linear":
            raise NotImplementedError("only linear interpolation is supported")
        self.n_input_dims = n_input_dims
        self.n_levels = int(encoding_config.get("n_levels", 16))
        self.n_features_per_level = int(encoding_config.get("n_features_per_level", 2))
        self.log2_hashmap_size = int(encoding_config.get("log2_hashmap_size", 19))
        self.base_resolution = int(encoding_config.get("base_resolution", 16))
        self.per_level_scale = float(encoding_config.get("per_level_scale", 2.0))
        self.desc = grid_desc(self.n_levels, self.n_features_per_level, self.log2_hashmap_size,
                              self.base_resolution, self.per_level_scale)
        self.n_output_dims = self.n_levels * self.n_features_per_level
        n_params = int(self.desc.offsets[self.n_levels]) * self.n_features_per_level
        gen = torch.Generator().manual_seed(int(seed))
        init = (torch.rand(n_params, generator=gen, dtype=torch.float64) * 2.0 - 1.0) * 1e-4
        self.params = nn.Parameter(init.to(dtype))

    @property
    def n_params(self) -> int:
        return self.params.numel()

    def level_offsets(self) -> np.ndarray:
        return np.array(self.desc.offsets[: self.n_levels + 1], dtype=np.int64)

    def level_resolutions(self) -> np.ndarray:
        return np.array(self.desc.resolutions[: self.n_levels], dtype=np.int64)

    def level_scales(self) -> np.ndarray:
        return np.array(self.desc.scales[: self.n_levels], dtype=np.float32)

    def forward(self, x: Tensor, active_levels: Optional[int] = None) -> Tensor:
        _need_cuda(x)
        act = self.n_levels if active_levels is None else int(active_levels)
        return _HashGridFn.apply(x, self.params, self, act)


class _HashGridFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x: Tensor, table: Tensor, enc: HashGridEncoding, active: int):
        x = x.contiguous().float()
        out = torch.empty((x.shape[0], enc.n_output_dims), device=x.device, dtype=torch.float32)
        call("sn_hashgrid_fwd", x.shape[0], x, table, C.byref(enc.desc), active, out, stream_handle())
        ctx.save_for_backward(x)
        ctx.enc, ctx.active, ctx.n_table = enc, active, table.numel()
        return out

    @staticmethod
    def backward(ctx, grad_out: Tensor):
        (x,) = ctx.saved_tensors
        gt = None
        if ctx.needs_input_grad[1]:
            gt = torch.zeros(ctx.n_table, device=x.device, dtype=torch.float32)
            call("sn_hashgrid_bwd", x.shape[0], x, grad_out.contiguous().float(),
                 C.byref(ctx.enc.desc), ctx.active, gt, stream_handle())
        if ctx.needs_input_grad[0]:
            raise NotImplementedError("d(encoding)/dx alone is not exposed; use SDFNetwork.gradient")
        return None, gt, None, None


class _WeightNorm(torch.autograd.Function):
    """w = g * v / ||v|| per output row (torch.nn.utils.weight_norm, dim=0)."""

    @staticmethod
    def forward(ctx, v: Tensor, g: Tensor):
        v = v.contiguous().float()
        g = g.contiguous().float()
        rows, cols = v.shape
        w = torch.empty_like(v)
        norms = torch.empty((rows,), device=v.device, dtype=torch.float32)
        call("sn_weightnorm_fwd", rows, cols, v, g, w, norms, stream_handle())
        ctx.save_for_backward(v, g, norms)
        return w

    @staticmethod
    def backward(ctx, gw: Tensor):
        v, g, norms = ctx.saved_tensors
        rows, cols = v.shape
        gv = torch.empty_like(v)
        gg = torch.empty((rows,), device=v.device, dtype=torch.float32)
        call("sn_weightnorm_bwd", rows, cols, v, g, norms, gw.contiguous().float(), gv, gg,
             stream_handle())
        return gv, gg.reshape(g.shape)


class WeightNormLinear(nn.Module):
    """Linear layer with the parameters torch's weight_norm registers
    (``weight_g`` (out, 1), ``weight_v`` (out, in), ``bias``)."""

    def __init__(self, lin: nn.Linear, weight_norm: bool = True):
        super().__init__()
        self.use_wn = weight_norm
        w = lin.weight.detach().clone()
        if weight_norm:
            self.weight_g = nn.Parameter(torch.linalg.vector_norm(w, dim=1, keepdim=True))
            self.weight_v = nn.Parameter(w)
        else:
            self.weight = nn.Parameter(w)
        self.bias = nn.Parameter(lin.bias.detach().clone())
        self.in_features, self.out_features = lin.in_features, lin.out_features

    def effective_weight(self) -> Tensor:
        if not self.use_wn:
            return self.weight
        if self.weight_v.is_cuda:
            return _WeightNorm.apply(self.weight_v, self.weight_g)
        return self.weight_g * self.weight_v / torch.linalg.vector_norm(self.weight_v, dim=1,
                                                                       keepdim=True)


class _FieldFn(torch.autograd.Function):
    """Fused encoding + MLP; backward recomputes activations (no stored hidden state)."""

    @staticmethod
    def forward(ctx, x, table, w0, b0, w1, b1, net: "SDFNetwork", out_cols: int):
        x = x.contiguous().float()
        active = net.active_levels()
        desc = net._mlp_desc(w0, b0, w1, b1)
        out = torch.empty((x.shape[0], out_cols), device=x.device, dtype=torch.float32)
        call("sn_field_fwd", x.shape[0], None, x, table, C.byref(net.encoding.desc), active,
             C.byref(desc), out_cols, out, stream_handle())
        ctx.save_for_backward(x, table, w0, b0, w1, b1)
        ctx.net, ctx.out_cols, ctx.active = net, out_cols, active
        return out

    @staticmethod
    def backward(ctx, grad_out):
        x, table, w0, b0, w1, b1 = ctx.saved_tensors
        net = ctx.net
        dev = x.device
        need = ctx.needs_input_grad
        g_table = torch.zeros_like(table) if need[1] else None
        g_w0 = torch.zeros_like(w0) if need[2] else None
        g_b0 = torch.zeros_like(b0) if need[3] else None
        g_w1 = torch.zeros_like(w1) if need[4] else None
        g_b1 = torch.zeros_like(b1) if need[5] else None
        g_x = torch.empty_like(x) if need[0] else None
        desc = net._mlp_desc(w0, b0, w1, b1)
        call("sn_field_bwd", x.shape[0], None, x, grad_out.contiguous().float(), ctx.out_cols, table,
             C.byref(net.encoding.desc), ctx.active, C.byref(desc), g_table, g_w0, g_b0, g_w1, g_b1,
             g_x, stream_handle())
        return g_x, g_table, g_w0, g_b0, g_w1, g_b1, None, None


class _FieldGradFn(torch.autograd.Function):
    """(sdf, d sdf/dx) in one kernel; backward is the hand-written second-order
    adjoint (the double backward of models/fields.py:107-119 with create_graph)."""

    @staticmethod
    def forward(ctx, x, table, w0, b0, w1, b1, net: "SDFNetwork"):
        x = x.contiguous().float()
        active = net.active_levels()
        desc = net._mlp_desc(w0, b0, w1, b1)
        sdf = torch.empty((x.shape[0], 1), device=x.device, dtype=torch.float32)
        grad = torch.empty((x.shape[0], 3), device=x.device, dtype=torch.float32)
        call("sn_field_grad_fwd", x.shape[0], None, x, table, C.byref(net.encoding.desc), active,
             C.byref(desc), sdf, grad, stream_handle())
        ctx.save_for_backward(x, table, w0, b0, w1, b1)
        ctx.net, ctx.active = net, active
        return sdf, grad

    @staticmethod
    def backward(ctx, g_sdf, g_grad):
        x, table, w0, b0, w1, b1 = ctx.saved_tensors
        if ctx.needs_input_grad[0]:
            raise NotImplementedError("d^2 sdf / dx^2 (the Hessian) is not implemented")
        need = ctx.needs_input_grad
        g_table = torch.zeros_like(table) if need[1] else None
        g_w0 = torch.zeros_like(w0) if need[2] else None
        g_b0 = torch.zeros_like(b0) if need[3] else None
        g_w1 = torch.zeros_like(w1) if need[4] else None
        g_b1 = torch.zeros_like(b1) if need[5] else None
        g_grad = torch.zeros((x.shape[0], 3), device=x.device) if g_grad is None else g_grad.contiguous().float()
        g_sdf = None if g_sdf is None else g_sdf.contiguous().float().reshape(-1)
        desc = ctx.net._mlp_desc(w0, b0, w1, b1)
        call("sn_field_grad_bwd", x.shape[0], None, x, g_grad, g_sdf, table,
             C.byref(ctx.net.encoding.desc), ctx.active, C.byref(desc), g_table, g_w0, g_b0, g_w1,
             g_b1, stream_handle())
        return None, g_table, g_w0, g_b0, g_w1, g_b1, None


class SDFNetwork(nn.Module):
    """SDF MLP over a hash-grid encoding (models/fields.py:7-130)."""

    def __init__(self, d_in, d_out, d_hidden, n_layers, skip_in=(4,), bias=0.5,
                 geometric_init=True, weight_norm=True, inside_outside=False,
                 encoding_config=None, input_concat=False):
        super().__init__()
        self.input_concat = input_concat
        dims = [d_in] + [d_hidden for _ in range(n_layers)] + [d_out]
        if encoding_config is None:
            raise NotImplementedError("SDFNetwork needs an encoding_config (models/fields.py:37)")
        self.encoding = HashGridEncoding(d_in, encoding_config)
        dims[0] = self.encoding.n_output_dims
        if input_concat:
            dims[0] += d_in
        self.num_layers = len(dims)
        self.skip_in = skip_in
        self.bindwidth = 0
        self.enc_dim = self.encoding.n_output_dims
        self.d_in, self.d_out, self.d_hidden = d_in, d_out, d_hidden
        for l in range(0, self.num_layers - 1):
            out_dim = dims[l + 1] - dims[0] if l + 1 in self.skip_in else dims[l + 1]
            lin = nn.Linear(dims[l], out_dim)
            if geometric_init:
                if l == self.num_layers - 2:
                    if not inside_outside:
                        torch.nn.init.normal_(lin.weight, mean=np.sqrt(np.pi) / np.sqrt(dims[l]), std=0.0001)
                        torch.nn.init.constant_(lin.bias, -bias)
                    else:
                        torch.nn.init.normal_(lin.weight, mean=-np.sqrt(np.pi) / np.sqrt(dims[l]), std=0.0001)
                        torch.nn.init.constant_(lin.bias, bias)
                elif l == 0:
                    torch.nn.init.constant_(lin.bias, 0.0)
                    torch.nn.init.constant_(lin.weight[:, 3:], 0.0)
                    torch.nn.init.normal_(lin.weight[:, :3], 0.0, np.sqrt(2) / np.sqrt(out_dim))
                elif l in self.skip_in:
                    torch.nn.init.constant_(lin.bias, 0.0)
                    torch.nn.init.normal_(lin.weight, 0.0, np.sqrt(2) / np.sqrt(out_dim))
                    torch.nn.init.constant_(lin.weight[:, -(dims[0] - 3):], 0.0)
                else:
                    torch.nn.init.constant_(lin.bias, 0.0)
                    torch.nn.init.normal_(lin.weight, 0.0, np.sqrt(2) / np.sqrt(out_dim))
            setattr(self, "lin" + str(l), WeightNormLinear(lin, weight_norm))
        self.beta, self.threshold = 100.0, 20.0
        # device status word of the tensor-core field kernels (not in the state_dict)
        self.register_buffer("_kernel_status", torch.zeros(1, dtype=torch.int32), persistent=False)
        self._supported = (n_layers == 1 and d_hidden == 64 and input_concat and d_in == 3
                           and self.encoding.n_features_per_level == 2
                           and self.encoding.n_levels <= 16 and 1 <= d_out <= 16)

    def _check(self, x: Tensor) -> None:
        _need_cuda(x)
        if not self._supported:
            raise NotImplementedError(
                "the fused field kernels cover SDFNetwork(d_in=3, d_hidden=64, n_layers=1, "
                "input_concat=True, d_out<=16) over a HashGrid with 2 features and <=16 levels")

    def increase_bandwidth(self):
        self.bindwidth += 1

    def active_levels(self) -> int:
        # enc_mask[bindwidth*2:] = 0 with 2 features per level (models/fields.py:81-83)
        return max(0, min(self.bindwidth, self.encoding.n_levels))

    def _mlp_desc(self, w0, b0, w1, b1) -> MlpDesc:
        d = MlpDesc()
        d.d_in = w0.shape[1]
        d.d_hidden = w0.shape[0]
        d.d_out = w1.shape[0]
        d.beta = self.beta
        d.threshold = self.threshold
        d.w0, d.b0, d.w1, d.b1 = w0.data_ptr(), b0.data_ptr(), w1.data_ptr(), b1.data_ptr()
        d.status = self._kernel_status.data_ptr()
        return d

    def check_status(self) -> None:
        """Raise if a field kernel reported a failed bounded wait (host sync)."""
        if int(self._kernel_status.item()) & SN_STATUS_TIMEOUT:
            raise RuntimeError("a tensor-core field kernel timed out waiting for its MMAs")

    def mlp_tensors(self):
        return (self.lin0.effective_weight(), self.lin0.bias, self.lin1.effective_weight(),
                self.lin1.bias)

    def _field(self, x: Tensor, out_cols: int) -> Tensor:
        self._check(x)
        w0, b0, w1, b1 = self.mlp_tensors()
        return _FieldFn.apply(x, self.encoding.params, w0.contiguous(), b0.contiguous(),
                              w1.contiguous(), b1.contiguous(), self, out_cols)

    def forward(self, inputs: Tensor) -> Tensor:
        return self._field(inputs, self.d_out)

    def sdf(self, x: Tensor) -> Tensor:
        return self._field(x, 1)

    @torch.no_grad()
    def sdf_raw(self, x: Tensor, count: Optional[Tensor] = None) -> Tensor:
        """No-grad sdf (n, 1) of a capacity buffer x; count (device int32) bounds
        the rows evaluated, so no host synchronisation is needed."""
        self._check(x)
        w0, b0, w1, b1 = (t.detach().contiguous() for t in self.mlp_tensors())
        desc = self._mlp_desc(w0, b0, w1, b1)
        out = torch.empty((x.shape[0], 1), device=x.device, dtype=torch.float32)
        call("sn_field_fwd", x.shape[0], count, x.contiguous(), self.encoding.params.detach(),
             C.byref(self.encoding.desc), self.active_levels(), C.byref(desc), 1, out,
             stream_handle())
        return out

    def sdf_hidden_appearance(self, x: Tensor) -> Tensor:
        return self.forward(x)

    def sdf_and_gradient(self, x: Tensor):
        """(sdf (N, 1), d sdf / d x (N, 3)), both differentiable w.r.t. the parameters."""
        self._check(x)
        w0, b0, w1, b1 = self.mlp_tensors()
        return _FieldGradFn.apply(x.detach(), self.encoding.params, w0.contiguous(), b0.contiguous(),
                                  w1.contiguous(), b1.contiguous(), self)

    @torch.enable_grad()
    def gradient(self, x: Tensor) -> Tensor:
        """d sdf / d x, (N, 1, 3) (models/fields.py:107-119).  As with the
        reference's create_graph=True, the result is differentiable w.r.t. the
        parameters (second-order adjoint in sn_field_grad_bwd); like the
        reference, x is marked requires_grad."""
        x.requires_grad_(True)
        _, g = self.sdf_and_gradient(x)
        return g.unsqueeze(1)


class SingleVarianceNetwork(nn.Module):
    """inv_s = exp(10 * variance) (models/fields.py:133-139)."""

    def __init__(self, init_val):
        super().__init__()
        self.register_parameter("variance", nn.Parameter(torch.tensor(init_val)))

    def forward(self, x):
        return torch.ones([len(x), 1], device=self.variance.device) * torch.exp(self.variance * 10.0)
