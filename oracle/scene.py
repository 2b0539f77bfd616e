"""ORACLE (test infrastructure only): the benchmark scene and training batches on host cores.

A numpy / torch-CPU restatement, for the timed host baselines of bench.py,
of what the package builds on the device for the benchmark workload:

* the displaced torus SDF and the pinhole ring rig of the synthetic data
  (the stand-in for the DiLiGenT-MV captures the reference trains on);
* ``gen_random_patches`` (models/dataset_loader.py:223-277): random views and
  patch centres, per-pixel rays R normalize(K^-1 [x, y, 1]) from the camera
  centre, the marching-plane normal (the camera z axis) and
  V^-1 = inv([d; right; down]) per pixel (:112-137), with the ground-truth
  normal and mask of each sampled pixel found by sphere tracing;
* ``SDFNetwork.__init__``'s parameters (models/fields.py:39-70 geometric
  initialisation, same torch RNG call sequence) and the flat hash table
  initialised uniform(-1e-4, 1e-4) from its own seeded generator;
* the occupancy grid of the analytic scene: a cell is occupied when
  sigmoid(-80 sdf(centre)) exceeds min(mean, threshold), the update rule of
  NA/nerfacc/grid.py:229-237 applied to the true surface.
"""
from __future__ import annotations

import math

import numpy as np
import torch

from . import field as OF


def torus_sdf(p, R=0.5, r=0.2, amp=0.02, freq=20.0):
    """Torus around z with a radial displacement amp sin(f theta) sin(f phi) (float64)."""
    p = np.asarray(p, np.float64)
    rxy = np.sqrt(p[..., 0] ** 2 + p[..., 1] ** 2)
    ring = rxy - R
    d = np.sqrt(ring ** 2 + p[..., 2] ** 2) - r
    if amp:
        d = d - amp * np.sin(freq * np.arctan2(p[..., 1], p[..., 0])) * np.sin(freq * np.arctan2(p[..., 2], ring))
    return d


def torus_lipschitz(R=0.5, r=0.2, amp=0.02, freq=20.0):
    return 1.0 + abs(amp) * freq * (1.0 / max(R - r, 1e-3) + 1.0 / r)


def ring_rig(n_views, H, W, radius=3.0, elevation_deg=30.0, fov_deg=40.0):
    """Camera-to-world poses (n, 3, 4) and K^-1 (n, 3, 3) of a ring looking at
    the origin (OpenCV axes: x right, y down, z forward)."""
    f = 0.5 * W / math.tan(0.5 * math.radians(fov_deg))
    el = math.radians(elevation_deg)
    K = np.array([[f, 0.0, 0.5 * (W - 1)], [0.0, f, 0.5 * (H - 1)], [0.0, 0.0, 1.0]])
    kinv = np.linalg.inv(K)
    poses = []
    for i in range(n_views):
        az = 2.0 * math.pi * i / n_views
        eye = np.array([radius * math.cos(el) * math.cos(az), radius * math.cos(el) * math.sin(az),
                        radius * math.sin(el)])
        z = -eye / np.linalg.norm(eye)
        x = np.cross(z, [0.0, 0.0, 1.0])
        x /= np.linalg.norm(x)
        y = np.cross(z, x)
        poses.append(np.stack([x, y, z, eye], axis=1))
    return np.stack(poses), np.repeat(kinv[None], n_views, axis=0)


def near_far(o, d):
    """Unit-sphere chord (models/dataset_loader.py:279-297)."""
    a = (d * d).sum(-1)
    b = 2.0 * (o * d).sum(-1)
    c = (o * o).sum(-1) - 1.0
    disc = np.sqrt(np.maximum(b * b - 4 * a * c, 0.0))
    mid = -0.5 * b / a
    return mid - disc / (2 * a), mid + disc / (2 * a)


def sphere_trace(sdf, lip, o, d, iters=400, eps=1e-6):
    near, far = near_far(o, d)
    t = near.copy()
    alive = np.ones(t.shape, bool)
    hit = np.zeros(t.shape, bool)
    for _ in range(iters):
        s = sdf(o + d * t[..., None])
        newly = alive & (np.abs(s) < eps)
        hit |= newly
        alive &= ~newly
        t = np.where(alive, t + s / lip * 0.9, t)
        alive &= t < far
        if not alive.any():
            break
    return t, hit


def gen_random_patches(sdf, lip, poses, kinv, H, W, n, rng, ph=3, pw=3):
    """(rays_o, rays_d, plane_n, V^-1, normal, mask) float32 for n random
    patches (models/dataset_loader.py:223-277)."""
    cx = rng.integers(pw // 2, W - 1 - pw // 2, n)
    cy = rng.integers(ph // 2, H - 1 - ph // 2, n)
    img = rng.integers(0, poses.shape[0], n)
    ox, oy = np.meshgrid(np.arange(-(pw // 2), pw // 2 + 1), np.arange(-(ph // 2), ph // 2 + 1))
    px = cx[:, None, None] + ox[None]
    py = cy[:, None, None] + oy[None]
    pix = np.stack([px, py, np.ones_like(px)], -1).astype(np.float64)
    v = np.einsum("nij,nhwj->nhwi", kinv[img], pix)
    v /= np.linalg.norm(v, axis=-1, keepdims=True)
    R = poses[img, :, :3]
    d = np.einsum("nij,nhwj->nhwi", R, v)
    o = np.broadcast_to(poses[img, None, None, :, 3], d.shape)
    t, hit = sphere_trace(sdf, lip, o, d)
    pts = o + d * t[..., None]
    h = 1e-6
    grad = np.stack([(sdf(pts + h * e) - sdf(pts - h * e)) / (2 * h) for e in np.eye(3)], -1)
    normal = grad / np.maximum(np.linalg.norm(grad, axis=-1, keepdims=True), 1e-12) * hit[..., None]
    right = np.broadcast_to(R[:, None, None, :, 0], d.shape)
    down = np.broadcast_to(R[:, None, None, :, 1], d.shape)
    vinv = np.linalg.inv(np.stack([d, right, down], axis=-2))
    f32 = lambda a: np.ascontiguousarray(a, dtype=np.float32)
    return (f32(o), f32(d), f32(R[:, :, 2]), f32(vinv), f32(normal), f32(hit[..., None]))


def sdf_network_init(seed, enc, d_out=16, d_hidden=64, bias=0.5, table_seed=1337):
    """Parameters of SDFNetwork(3, d_out, d_hidden, 1, skip_in=(-1,), bias,
    geometric_init=True, weight_norm=True, input_concat=True) after
    torch.manual_seed(seed): the nn.Linear draws and the geometric
    initialisation of models/fields.py:39-65 in the same order, weight norm
    g = ||v|| per row (torch.nn.utils.weight_norm at construction), and the
    hash table uniform(-1e-4, 1e-4) from a generator seeded with table_seed.
    Returns (params dict of float32 leaves, level geometry)."""
    geom = OF.grid_geometry(enc["n_levels"], enc["n_features_per_level"], enc["log2_hashmap_size"],
                            enc["base_resolution"], enc["per_level_scale"])
    n_table = int(geom[0][-1]) * enc["n_features_per_level"]
    gen = torch.Generator().manual_seed(table_seed)
    table = ((torch.rand(n_table, generator=gen, dtype=torch.float64) * 2.0 - 1.0) * 1e-4).float()
    torch.manual_seed(seed)
    d0 = 3 + enc["n_levels"] * enc["n_features_per_level"]
    lin0 = torch.nn.Linear(d0, d_hidden)
    torch.nn.init.constant_(lin0.bias, 0.0)
    torch.nn.init.constant_(lin0.weight[:, 3:], 0.0)
    torch.nn.init.normal_(lin0.weight[:, :3], 0.0, np.sqrt(2) / np.sqrt(d_hidden))
    lin1 = torch.nn.Linear(d_hidden, d_out)
    torch.nn.init.normal_(lin1.weight, mean=np.sqrt(np.pi) / np.sqrt(d_hidden), std=0.0001)
    torch.nn.init.constant_(lin1.bias, -bias)
    p = lambda t: t.detach().clone()
    vn = lambda w: torch.linalg.vector_norm(w.detach(), dim=1, keepdim=True)
    prm = dict(table=table, v0=p(lin0.weight), g0=vn(lin0.weight), b0=p(lin0.bias),
               v1=p(lin1.weight), g1=vn(lin1.weight), b1=p(lin1.bias))
    return prm, geom


def analytic_occupancy(sdf, res=128, threshold=0.1, k=80.0):
    """Binary occupancy grid (res^3, "ij" cell order) of the true surface."""
    c = (np.stack(np.meshgrid(*[np.arange(res)] * 3, indexing="ij"), -1).reshape(-1, 3) + 0.5) / res * 2 - 1
    occ = 1.0 / (1.0 + np.exp(np.clip(sdf(c) * k, -60.0, 60.0)))
    return (occ > min(occ.mean(), threshold)).reshape(res, res, res).astype(np.uint8)
