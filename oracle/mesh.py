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


# ---------------------------------------------------------------------------
# The device marching cubes restated on the host (the triangle rule of
# supernormal_gb300/csrc/mesh.cu: per-face pairing that cuts off each inside
# corner, segments oriented from the boundary's entry into the inside to the
# next exit, loops fanned from a vertex none of whose diagonals lies on a cube
# face).  It numbers vertices the same way (flagged lattice edges in (axis,
# i, j, k) order), so the device's triangle arrays can be compared exactly.
def _edge_of(c0, axis):
    if axis == 0:
        return (c0 >> 1) & 3
    if axis == 1:
        return 4 + ((c0 & 1) | (((c0 >> 2) & 1) << 1))
    return 8 + (c0 & 3)


def _edge_faces(e):
    axis, o = e >> 2, e & 3
    x0, x1 = (1 if axis == 0 else 0), (1 if axis == 2 else 2)
    return (1 << (2 * x0 + (o & 1))) | (1 << (2 * x1 + ((o >> 1) & 1)))


def mc_table():
    table = []
    for cs in range(256):
        nxt = [-1] * 12
        for a in range(3):
            b, c = (a + 1) % 3, (a + 2) % 3
            for s in range(2):
                bc = [(0, 0), (1, 0), (1, 1), (0, 1)]
                q = [(s << a) | (bc[i if s else (4 - i) % 4][0] << b) | (bc[i if s else (4 - i) % 4][1] << c)
                     for i in range(4)]
                cr = []
                for i in range(4):
                    p, r = q[i], q[(i + 1) % 4]
                    if ((cs >> p) & 1) != ((cs >> r) & 1):
                        cr.append((_edge_of(min(p, r), {1: 0, 2: 1, 4: 2}[p ^ r]), bool((cs >> r) & 1)))
                for i, (e, entry) in enumerate(cr):
                    if entry:
                        for j in range(1, len(cr)):
                            k = (i + j) % len(cr)
                            if not cr[k][1]:
                                nxt[e] = cr[k][0]
                                break
        seen, tris = [False] * 12, []
        for e0 in range(12):
            if nxt[e0] < 0 or seen[e0]:
                continue
            loop, e = [], e0
            while not seen[e]:
                seen[e] = True
                loop.append(e)
                e = nxt[e]
            n = len(loop)
            ap = next(c for c in range(n) if all(j in (c, (c + 1) % n, (c - 1) % n)
                                                 or not (_edge_faces(loop[c]) & _edge_faces(loop[j]))
                                                 for j in range(n)))
            tris += [(loop[ap], loop[(ap + i) % n], loop[(ap + i + 1) % n]) for i in range(1, n - 1)]
        table.append(tris)
    return table


def marching_cubes(u, threshold, bound_min, bound_max):
    """(vertices (V, 3) float64, triangles (T, 3) int64) as the device builds them."""
    u = np.asarray(u, np.float32)
    nx, ny, nz = u.shape
    inside = u > np.float32(threshold)
    lo = np.asarray(bound_min, np.float64)
    step = ((np.asarray(bound_max, np.float64) - lo) / (np.array(u.shape) - 1)).astype(np.float32)
    ids = np.full((3, nx, ny, nz), -1, np.int64)
    verts, nv = [], 0
    for axis in range(3):
        a = [slice(None)] * 3
        b = [slice(None)] * 3
        a[axis], b[axis] = slice(0, -1), slice(1, None)
        flip = np.zeros(u.shape, bool)
        flip[tuple(a)] = inside[tuple(a)] != inside[tuple(b)]
        idx = np.argwhere(flip)
        ids[axis][flip] = nv + np.arange(len(idx))
        nv += len(idx)
        u0 = u[tuple(idx.T)]
        shifted = idx.copy()
        shifted[:, axis] += 1
        u1 = u[tuple(shifted.T)]
        t = ((np.float32(threshold) - u0) / (u1 - u0)).astype(np.float32)
        pos = idx.astype(np.float32)
        pos[:, axis] = (pos[:, axis] + t).astype(np.float32)
        verts.append(pos.astype(np.float64) * step + lo)
    table = mc_table()
    cs = np.zeros((nx - 1, ny - 1, nz - 1), np.int64)
    for c in range(8):
        cs |= inside[(c & 1):nx - 1 + (c & 1), ((c >> 1) & 1):ny - 1 + ((c >> 1) & 1),
                     ((c >> 2) & 1):nz - 1 + ((c >> 2) & 1)].astype(np.int64) << c
    tris = []
    for (i, j, k) in np.argwhere(cs > 0):
        for tri in table[cs[i, j, k]]:
            row = []
            for e in tri:
                axis, o = e >> 2, e & 3
                b0, b1 = o & 1, (o >> 1) & 1
                di = 0 if axis == 0 else b0
                dj = 0 if axis == 1 else (b0 if axis == 0 else b1)
                dk = 0 if axis == 2 else b1
                row.append(ids[axis, i + di, j + dj, k + dk])
            tris.append(row)
    v = np.concatenate(verts) if verts else np.zeros((0, 3))
    return v, np.asarray(tris, np.int64).reshape(-1, 3)
