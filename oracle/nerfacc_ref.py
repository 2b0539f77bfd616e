"""ORACLE (test infrastructure only): numpy restatements of nerfacc's rendering ops.

Each function follows the reference file it names
(NA = third_parties/nerfacc-0.3.5/nerfacc-0.3.5).  Loops are sequential in the
reference kernels' order, float64 unless the caller passes float32 and asks
for it (``dtype``).
"""
from __future__ import annotations

import numpy as np


def pack_info(ray_indices, n_rays=None):
    """NA/nerfacc/pack.py:46-77: counts per ray, exclusive cumsum -> (n_rays, 2) int32."""
    ray_indices = np.asarray(ray_indices, dtype=np.int64)
    if n_rays is None:
        n_rays = int(ray_indices.max()) + 1 if ray_indices.size else 0
    counts = np.bincount(ray_indices, minlength=n_rays).astype(np.int32)[:n_rays]
    offs = np.cumsum(counts) - counts
    return np.stack([offs, counts], axis=1).astype(np.int32)


def unpack_info(packed_info, n_samples):
    """NA/nerfacc/cuda/csrc/pack.cu:7-27."""
    out = np.zeros(n_samples, dtype=np.int64)
    for r, (b, c) in enumerate(np.asarray(packed_info)):
        out[b:b + c] = r
    return out


def transmittance(alphas, packed_info, patch_size=1, dtype=np.float64):
    """Exclusive product of (1 - alpha) per ray (and pixel lane)."""
    a = np.asarray(alphas, dtype=dtype).reshape(-1, patch_size)
    T = np.zeros_like(a)
    for b, c in np.asarray(packed_info):
        t = np.ones(patch_size, dtype=dtype)
        for j in range(b, b + c):
            T[j] = t
            t = t * (dtype(1.0) - a[j])
    return T


def visibility(alphas, packed_info, early_stop_eps=1e-4, alpha_thre=0.0, dtype=np.float64):
    """NA/nerfacc/vol_rendering.py:680-748 (T >= eps, alpha >= thre when thre > 0).
    dtype=np.float32 forms T with float32 roundings in sample order."""
    a = np.asarray(alphas, dtype=dtype).reshape(-1)
    T = transmittance(a, packed_info, 1, dtype).reshape(-1)
    vis = T >= dtype(early_stop_eps)
    if alpha_thre > 0:
        vis &= a >= dtype(alpha_thre)
    return vis


def weights_fwd(alphas, packed_info, patch_size=1, dtype=np.float64):
    """NA/nerfacc/cuda/csrc/render_weight.cu:87-118 (patch) / :154-183 (ray)."""
    a = np.asarray(alphas, dtype=dtype).reshape(-1, patch_size)
    return (a * transmittance(a, packed_info, patch_size, dtype)).reshape(np.shape(alphas))


def weights_bwd(alphas, weights, grad_weights, packed_info, patch_size=1, dtype=np.float64):
    """NA/nerfacc/cuda/csrc/render_weight.cu:298-340:
    grad_a_j = (g_j T_j - sum_{i>=j} g_i w_i) / max(1 - a_j, 1e-10)."""
    a = np.asarray(alphas, dtype=dtype).reshape(-1, patch_size)
    w = np.asarray(weights, dtype=dtype).reshape(-1, patch_size)
    g = np.asarray(grad_weights, dtype=dtype).reshape(-1, patch_size)
    out = np.zeros_like(a)
    for b, c in np.asarray(packed_info):
        acc = (g[b:b + c] * w[b:b + c]).sum(axis=0)
        t = np.ones(patch_size, dtype=dtype)
        for j in range(b, b + c):
            out[j] = (g[j] * t - acc) / np.maximum(dtype(1.0) - a[j], dtype(1e-10))
            acc = acc - g[j] * w[j]
            t = t * (dtype(1.0) - a[j])
    return out.reshape(np.shape(alphas))


def accumulate(weights, ray_indices, values=None, n_rays=None):
    """NA/nerfacc/vol_rendering.py:269-335: out[r, k, :] = sum w * v over the ray's samples."""
    w = np.asarray(weights, dtype=np.float64)
    if w.ndim == 2:
        w = w[:, None, :]
    src = w if values is None else w * np.asarray(values, dtype=np.float64).reshape(
        w.shape[0], w.shape[1], -1)
    if n_rays is None:
        n_rays = int(np.max(ray_indices)) + 1
    out = np.zeros((n_rays,) + src.shape[1:], dtype=np.float64)
    np.add.at(out, np.asarray(ray_indices), src)
    return out
