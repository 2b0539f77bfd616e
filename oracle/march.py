"""ORACLE (test infrastructure only): ctypes wrapper of oracle/march.c."""
from __future__ import annotations

import ctypes as C

import numpy as np

from .build import build

_lib = None


def _load():
    global _lib
    if _lib is None:
        L = C.CDLL(str(build()))
        P = C.c_void_p
        common = [C.c_int64, P, P, P, P, P, P, P, C.c_int, C.c_int, C.c_int, C.c_float, C.c_float,
                  C.c_int64]
        L.oracle_march_count.argtypes = common + [P]
        L.oracle_march_count.restype = C.c_int
        L.oracle_march_fill.argtypes = common + [P, P, P, P]
        L.oracle_march_fill.restype = C.c_int
        L.oracle_occ_points.argtypes = [C.c_int64, P, P, C.c_int, C.c_int, C.c_int, P, P]
        L.oracle_occ_points.restype = None
        L.oracle_unit_to_roi.argtypes = [C.c_int64, P, P, P]
        L.oracle_unit_to_roi.restype = None
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data


def ray_marching(rays_o, rays_d, t_min, t_max, roi, binary, step_size, jitter=None,
                 cone_angle=0.0, max_iters=1 << 24):
    """float32 marcher (NA/nerfacc/cuda/csrc/ray_marching.cu:81-289 semantics).

    Returns packed_info (n,2) int32, ray_indices int64, t_starts, t_ends (float32)."""
    f32 = lambda a: np.ascontiguousarray(a, dtype=np.float32)
    rays_o, rays_d, t_min, t_max, roi = map(f32, (rays_o, rays_d, t_min, t_max, roi))
    jitter = None if jitter is None else f32(jitter)
    bits = np.ascontiguousarray(binary, dtype=np.uint8)
    rx, ry, rz = bits.shape
    n = rays_o.shape[0]
    L = _load()
    counts = np.zeros(n, dtype=np.int32)
    args = (n, _p(rays_o), _p(rays_d), _p(t_min), _p(t_max), _p(jitter), _p(roi), _p(bits), rx, ry,
            rz, float(step_size), float(cone_angle), int(max_iters))
    if L.oracle_march_count(*args, _p(counts)) != 0:
        raise RuntimeError("oracle marcher: iteration limit")
    total = int(counts.sum())
    ridx = np.zeros(total, dtype=np.int64)
    ts = np.zeros(total, dtype=np.float32)
    te = np.zeros(total, dtype=np.float32)
    if L.oracle_march_fill(*args, _p(counts), _p(ridx), _p(ts), _p(te)) != 0:
        raise RuntimeError("oracle marcher: iteration limit")
    offs = np.concatenate([[0], np.cumsum(counts)[:-1]]).astype(np.int32)
    packed = np.stack([offs, counts], axis=1).astype(np.int32)
    return packed, ridx, ts, te


def occ_points(cells, jitter, resolution, roi):
    """Occupancy query points of grid cells (NA/nerfacc/grid.py:210-225, AABB):
    float32 (n, 3); cells None = every cell in order."""
    jitter = np.ascontiguousarray(jitter, dtype=np.float32)
    n = jitter.shape[0]
    cells = None if cells is None else np.ascontiguousarray(cells, dtype=np.int64)
    roi = np.ascontiguousarray(roi, dtype=np.float32)
    rx, ry, rz = (int(r) for r in resolution)
    out = np.zeros((n, 3), dtype=np.float32)
    _load().oracle_occ_points(n, _p(cells), _p(jitter), rx, ry, rz, _p(roi), _p(out))
    return out


def unit_to_roi(u, roi):
    """[0,1]^3 -> roi (helpers_contraction.h:23-28, AABB contract_inv), float32."""
    u = np.ascontiguousarray(u, dtype=np.float32).reshape(-1, 3)
    roi = np.ascontiguousarray(roi, dtype=np.float32)
    out = np.zeros_like(u)
    _load().oracle_unit_to_roi(u.shape[0], _p(u), _p(roi), _p(out))
    return out
