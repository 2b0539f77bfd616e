"""Mesh extraction: drop-in for extract_fields / extract_geometry (models/renderer.py:9-34).

The reference queries the SDF on a res^3 lattice over [bound_min, bound_max]
in 64^3 blocks and triangulates the field with PyMCubes on the host.  Here
the lattice points are formed on the device slab by slab
(``sn_lattice_points``), evaluated there, and triangulated by the device
marching cubes (``sn_marching_cubes``): an indexed mesh whose vertices sit
at the linear-interpolation crossings of the lattice edges whose ends lie on
either side of the threshold.  Vertices come back in world coordinates,
``vertex / (res - 1) * (bound_max - bound_min) + bound_min`` as the
reference scales PyMCubes' index-space vertices.
"""
from __future__ import annotations

from typing import Callable

import numpy as np
import torch
from torch import Tensor

from ._lib import call, stream_handle

__all__ = ["extract_fields", "extract_geometry", "marching_cubes", "sdf_lattice"]


def _bounds(b) -> np.ndarray:
    if isinstance(b, Tensor):
        b = b.detach().cpu().numpy()
    return np.ascontiguousarray(np.asarray(b, dtype=np.float64).reshape(3))


def _res3(resolution):
    if isinstance(resolution, int):
        return (resolution,) * 3
    r = tuple(int(v) for v in resolution)
    assert len(r) == 3
    return r


@torch.no_grad()
def extract_fields(bound_min, bound_max, resolution, query_func: Callable[[Tensor], Tensor],
                   device="cuda", slab_points: int = 1 << 21) -> Tensor:
    """u[i, j, k] = query_func(lattice point (i, j, k)) as a (res, res, res)
    float32 device tensor (models/renderer.py:9-24; X first, Z fastest)."""
    nx, ny, nz = _res3(resolution)
    lo, hi = _bounds(bound_min), _bounds(bound_max)
    u = torch.empty((nx, ny, nz), device=device)
    per_slab = max(1, slab_points // (ny * nz))
    x = torch.empty((min(per_slab, nx) * ny * nz, 3), device=device)
    st = stream_handle()
    for i0 in range(0, nx, per_slab):
        ni = min(per_slab, nx - i0)
        pts = x[: ni * ny * nz]
        call("sn_lattice_points", i0, ni, nx, ny, nz, lo.ctypes.data, hi.ctypes.data, pts, st)
        u[i0:i0 + ni] = query_func(pts).reshape(ni, ny, nz)
    return u


@torch.no_grad()
def sdf_lattice(sdf_network, bound_min, bound_max, resolution, negate: bool = True,
                slab_points: int = 1 << 21) -> Tensor:
    """The lattice of -sdf (the reference's query_func, models/renderer.py:353-358)
    from the fused field kernel, without autograd."""
    dev = next(sdf_network.parameters()).device

    def q(pts):
        s = sdf_network.sdf_raw(pts)
        if negate:
            out = torch.empty_like(s)
            call("sn_negate", s.numel(), s, out, stream_handle())
            return out
        return s

    return extract_fields(bound_min, bound_max, resolution, q, device=dev, slab_points=slab_points)


@torch.no_grad()
def marching_cubes(u: Tensor, threshold: float, bound_min, bound_max):
    """Device marching cubes of the lattice values u (nx, ny, nz): returns
    (vertices (V, 3) float32 world coordinates, triangles (T, 3) int32) on
    u's device."""
    u = u.contiguous().float()
    nx, ny, nz = u.shape
    lo, hi = _bounds(bound_min), _bounds(bound_max)
    dev = u.device
    ws = torch.empty(int(call("sn_marching_cubes_workspace_bytes", nx, ny, nz)), dtype=torch.uint8, device=dev)
    counts = torch.zeros((2,), dtype=torch.int32, device=dev)
    st = stream_handle()
    call("sn_marching_cubes", u, nx, ny, nz, float(threshold), lo.ctypes.data, hi.ctypes.data, 0, 0, None, None,
         counts, ws, st)
    n_v, n_t = (int(v) for v in counts.tolist())
    verts = torch.empty((n_v, 3), device=dev)
    tris = torch.empty((n_t, 3), dtype=torch.int32, device=dev)
    call("sn_marching_cubes", u, nx, ny, nz, float(threshold), lo.ctypes.data, hi.ctypes.data, n_v, n_t, verts,
         tris, counts, ws, st)
    return verts, tris


def extract_geometry(bound_min, bound_max, resolution, threshold, query_func, device="cuda"):
    """models/renderer.py:27-34: (vertices (V, 3) float64, triangles (T, 3)
    int64) as numpy arrays, like PyMCubes' output after the reference's scaling."""
    u = extract_fields(bound_min, bound_max, resolution, query_func, device=device)
    v, t = marching_cubes(u, threshold, bound_min, bound_max)
    return v.double().cpu().numpy(), t.long().cpu().numpy()
