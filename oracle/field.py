"""ORACLE (test infrastructure only): float64 restatement of the SDF field.

Hash-grid encoding per the Instant-NGP paper (Mueller et al., SIGGRAPH 2022)
with tiny-cuda-nn's conventions that SuperNormal relies on
(models/fields.py:26,78; config/diligent.conf:80-87):
  level scale s_l = 2^(l log2 b) N_min - 1, resolution ceil(s_l) + 1,
  pos = fma(s_l, x, 0.5) in float32 (cell choice), trilinear weights,
  dense index when res^3 fits the level (taken modulo the level size in
  uint32, so negative inputs wrap), else the XOR prime hash
  (1, 2654435761, 805459861) modulo the level size; levels concatenated
  entry-major with F features per entry.
The cell indices are computed in numpy uint32 exactly as the device does;
interpolation, the MLP (models/fields.py:76-99: concat [x, enc], Linear ->
Softplus(beta=100) -> Linear, weight-normed) and all gradients (torch
autograd, including the second order for SDFNetwork.gradient) are float64.
"""
from __future__ import annotations

import math

import numpy as np
import torch

P1, P2 = np.uint32(2654435761), np.uint32(805459861)


def grid_geometry(n_levels, n_features, log2_hashmap_size, base_resolution, per_level_scale):
    """tcnn GridEncoding level table: (offsets[L+1], resolutions[L], scales[L] float32)."""
    log2_pls = np.float32(np.log2(np.float64(np.float32(per_level_scale))))
    offsets, res, scales = [0], [], []
    for l in range(n_levels):
        scale = np.float32(np.exp2(np.float64(l) * np.float64(log2_pls)) * np.float64(base_resolution)
                           - 1.0)
        r = int(math.ceil(float(scale))) + 1
        dense = r ** 3
        params = min(dense, 0xFFFFFFFF // 2)
        params = (params + 7) // 8 * 8
        params = min(params, 1 << log2_hashmap_size)
        offsets.append(offsets[-1] + params)
        res.append(r)
        scales.append(scale)
    return np.array(offsets, np.int64), np.array(res, np.int64), np.array(scales, np.float32)


def corner_indices(x32: np.ndarray, level: int, offsets, res, scales):
    """Cells (N,3) int, frac (N,3) float32 and absolute entry index (N,8) int64 of a level."""
    s = np.float32(scales[level])
    pos = (x32.astype(np.float64) * np.float64(s) + 0.5).astype(np.float32)   # == fmaf(s, x, 0.5)
    cell = np.floor(pos)
    frac = (pos - cell).astype(np.float32)
    cell_u = cell.astype(np.int64).astype(np.uint32)        # (uint32)(int)floor(pos)
    r = np.uint32(res[level])
    size = int(offsets[level + 1] - offsets[level])
    dense = int(res[level]) ** 3 <= size
    idx = np.zeros((x32.shape[0], 8), dtype=np.int64)
    with np.errstate(over="ignore"):
        for k in range(8):
            q = [cell_u[:, d] + np.uint32((k >> d) & 1) for d in range(3)]
            if dense:
                v = q[0] + q[1] * r + q[2] * (r * r)
            else:
                v = q[0] ^ (q[1] * P1) ^ (q[2] * P2)
            idx[:, k] = offsets[level] + (v.astype(np.int64) % size)
    return cell, frac, idx


def encode(x: torch.Tensor, table: torch.Tensor, geom, n_features=2, active_levels=None,
           cache: dict | None = None, dtype=torch.float64):
    """(N, L*F) encoding in ``dtype`` (float64 for the parity checks; float32
    for a timed host baseline), differentiable w.r.t. table and x.  ``cache``
    (optional dict) keeps the per-level cell data of a fixed x across calls."""
    offsets, res, scales = geom
    L = len(res)
    active = L if active_levels is None else active_levels
    x32 = x.detach().cpu().numpy().astype(np.float32) if cache is None or not cache else None
    xd = x.to(dtype)
    outs = []
    for l in range(L):
        if l >= active:
            outs.append(torch.zeros((x.shape[0], n_features), dtype=dtype))
            continue
        if cache is not None and l in cache:
            cell, frac32, idx = cache[l]
        else:
            if x32 is None:
                x32 = x.detach().cpu().numpy().astype(np.float32)
            cell, frac32, idx = corner_indices(x32, l, offsets, res, scales)
            if cache is not None:
                cache[l] = (cell, frac32, idx)
        # value: the float32 fraction tcnn forms (pos rounded to float32 before
        # floor/subtract); derivative: d frac / dx = scale
        xs = xd * float(scales[l])
        frac = torch.from_numpy(frac32).to(dtype) + (xs - xs.detach())
        feat = table.to(dtype).reshape(-1, n_features)[torch.from_numpy(idx)]      # (N, 8, F)
        acc = 0.0
        for k in range(8):
            w = 1.0
            for d in range(3):
                w = w * (frac[:, d] if (k >> d) & 1 else 1.0 - frac[:, d])
            acc = acc + w[:, None] * feat[:, k, :]
        outs.append(acc)
    return torch.cat(outs, dim=1)


def weight_norm(v: torch.Tensor, g: torch.Tensor) -> torch.Tensor:
    return g.reshape(-1, 1) * v / torch.linalg.vector_norm(v, dim=1, keepdim=True)


def softplus(h, beta=100.0, threshold=20.0):
    return torch.where(h * beta > threshold, h, torch.log1p(torch.exp(h * beta)) / beta)


def sdf_network(x, table, v0, g0, b0, v1, g1, b1, geom, active_levels=None, out_cols=None,
                cache=None, dtype=torch.float64):
    """SDFNetwork.forward with n_layers=1, input_concat=True (in ``dtype``)."""
    enc = encode(x, table, geom, active_levels=active_levels, cache=cache, dtype=dtype)
    inp = torch.cat([x.to(dtype), enc], dim=1)
    h = inp @ weight_norm(v0.to(dtype), g0.to(dtype)).T + b0.to(dtype)
    a = softplus(h)
    y = a @ weight_norm(v1.to(dtype), g1.to(dtype)).T + b1.to(dtype)
    return y if out_cols is None else y[:, :out_cols]


def params_from_module(net):
    """float64 CPU leaf copies of an SDFNetwork's parameters (requires_grad)."""
    t = lambda p: p.detach().double().cpu().clone().requires_grad_(True)
    return dict(table=t(net.encoding.params), v0=t(net.lin0.weight_v), g0=t(net.lin0.weight_g),
                b0=t(net.lin0.bias), v1=t(net.lin1.weight_v), g1=t(net.lin1.weight_g),
                b1=t(net.lin1.bias))


def geometry_from_module(net):
    """The level table the device kernels use (its float32 scales come from the
    library's descriptor; grid_geometry restates them independently)."""
    e = net.encoding
    return (e.level_offsets(), e.level_resolutions(), e.level_scales())
