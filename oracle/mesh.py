"""ORACLE (test infrastructure only): mesh extraction restated on the host.

* ``extract_fields`` restates models/renderer.py:9-24: the query function on
  a res^3 lattice over [bound_min, bound_max] (torch.linspace per axis,
  'ij' meshgrid in 64^3 blocks), X first and Z fastest.
* ``edge_crossings`` is the vertex set every marching-cubes variant (PyMCubes,
  which the reference calls in models/renderer.py:27-34, included) produces:
  one vertex per lattice edge whose ends lie on either side of the threshold,
  at the linear-interpolation crossing, scaled to world coordinates as
  models/renderer.py:30-33 does.  PyMCubes itself is not installed here, so
  the triangles are checked by their properties (closed, consistently
  oriented, Euler characteristic) rather than against its table.
"""
from __future__ import annotations

import numpy as np
import torch


def extract_fields(bound_min, bound_max, resolution, query_func, block=64):
    X = torch.linspace(float(bound_min[0]), float(bound_max[0]), resolution).split(block)
    Y = torch.linspace(float(bound_min[1]), float(bound_max[1]), resolution).split(block)
    Z = torch.linspace(float(bound_min[2]), float(bound_max[2]), resolution).split(block)
    u = np.zeros([resolution] * 3, dtype=np.float32)
    for xi, xs in enumerate(X):
        for yi, ys in enumerate(Y):
            for zi, zs in enumerate(Z):
                xx, yy, zz = torch.meshgrid(xs, ys, zs, indexing="ij")
                pts = torch.cat([xx.reshape(-1, 1), yy.reshape(-1, 1), zz.reshape(-1, 1)], dim=-1)
                val = query_func(pts).reshape(len(xs), len(ys), len(zs)).detach().cpu().numpy()
                u[xi * block: xi * block + len(xs), yi * block: yi * block + len(ys),
                  zi * block: zi * block + len(zs)] = val
    return u


def edge_crossings(u, threshold, bound_min, bound_max):
    """(V, 3) float64 world positions of every threshold crossing on a lattice edge."""
    u = np.asarray(u, np.float64)
    res = np.array(u.shape)
    lo = np.asarray(bound_min, np.float64)
    step = (np.asarray(bound_max, np.float64) - lo) / (res - 1)
    inside = u > threshold
    out = []
    for axis in range(3):
        a = [slice(None)] * 3
        b = [slice(None)] * 3
        a[axis] = slice(0, -1)
        b[axis] = slice(1, None)
        flip = inside[tuple(a)] != inside[tuple(b)]
        idx = np.argwhere(flip).astype(np.float64)
        u0, u1 = u[tuple(a)][flip], u[tuple(b)][flip]
        idx[:, axis] += (threshold - u0) / (u1 - u0)
        out.append(idx * step + lo)
    return np.concatenate(out) if out else np.zeros((0, 3))
