"""ORACLE (test infrastructure only): the occupancy-grid update of nerfacc 0.3.5.

Restates ``OccupancyGrid._update`` (NA/nerfacc/grid.py:196-239, NA =
third_parties/nerfacc-0.3.5/nerfacc-0.3.5) and the renderer's
``occ_eval_fn`` (models/renderer.py:56-60) in numpy float32, in the
reference's operation order.  The random draws (uniform cells, the selector
among occupied cells, the jitter) are inputs, so a caller can replay the
reference's own draws.

Repeated cells.  After the warm-up the sampled cells may repeat (uniform
draws collide with each other and with the occupied draws).  The reference
writes ``occs[indices] = max(occs[indices] * decay, occ)`` with an index_put
that stores an unspecified one of a repeated cell's candidates (on the CPU
the last, on CUDA any).  ``ema_update`` returns the candidate sets and the
largest candidate, which is what the GPU path stores.
"""
from __future__ import annotations

import numpy as np

from . import march as _march


def occupied_cells(binary):
    """``torch.nonzero(self._binary.flatten())[:, 0]`` (grid.py:187): flat indices, ascending."""
    return np.flatnonzero(np.asarray(binary).reshape(-1)).astype(np.int64)


def sample_cells(binary, n, uniform, selector=None):
    """grid.py:181-194: ``n`` uniform cells (given draws) followed by the
    occupied cells, or ``n`` of them chosen by ``selector`` when there are
    more than ``n``."""
    occ = occupied_cells(binary)
    uniform = np.asarray(uniform, dtype=np.int64)
    assert uniform.shape == (n,)
    if n < len(occ):
        assert selector is not None and len(selector) == n
        occ = occ[np.asarray(selector, dtype=np.int64)]
    return np.concatenate([uniform, occ])


def query_points(cells, jitter, resolution, roi):
    """grid.py:210-225 for the AABB contraction (float32, C restatement)."""
    return _march.occ_points(cells, jitter, resolution, roi)


def occ_from_sdf(sdf, k=80.0):
    """models/renderer.py:56-60: sigmoid(-sdf * 80), as 1 / (1 + exp(sdf * 80)) in float32."""
    s = np.asarray(sdf, dtype=np.float32)
    with np.errstate(over="ignore"):
        e = np.exp((s * np.float32(k)).astype(np.float32)).astype(np.float32)
    return (np.float32(1.0) / (np.float32(1.0) + e)).astype(np.float32)


def ema_update(occs, cells, occ, decay=0.95):
    """grid.py:229-230.  Returns (new occs with a repeated cell at its largest
    candidate, {cell: candidate values} for the repeated cells)."""
    occs = np.asarray(occs, dtype=np.float32)
    occ = np.asarray(occ, dtype=np.float32)
    if cells is None:
        cells = np.arange(occs.size, dtype=np.int64)
    cells = np.asarray(cells, dtype=np.int64)
    cand = np.maximum((occs[cells] * np.float32(decay)).astype(np.float32), occ)
    new = occs.copy()
    new[cells] = 0.0
    np.maximum.at(new, cells, cand)
    uniq, counts = np.unique(cells, return_counts=True)
    repeated = {}
    for c in uniq[counts > 1]:
        repeated[int(c)] = cand[cells == c]
    return new, repeated


def binarize(occs, occ_thre):
    """grid.py:235-237: occs > clamp(mean(occs), max=occ_thre).  The mean is
    formed in float64 and rounded once (torch reduces in float32 in an order
    of its own, so cells within a few ulp of the threshold may differ)."""
    occs = np.asarray(occs, dtype=np.float32)
    thr = np.float32(min(np.float32(occs.astype(np.float64).mean()), np.float32(occ_thre)))
    return occs > thr, thr


def update(occs, cells, jitter, occ_eval, resolution, roi, occ_thre=0.01, decay=0.95):
    """One ``_update`` (grid.py:196-239) with given cells (None = warm-up, all
    cells) and jitter; ``occ_eval`` maps (n, 3) float32 points to occupancy."""
    x = query_points(cells, jitter, resolution, roi)
    occ = np.asarray(occ_eval(x), dtype=np.float32).reshape(-1)
    new, repeated = ema_update(occs, cells, occ, decay)
    binary, thr = binarize(new, occ_thre)
    return {"x": x, "occ": occ, "occs": new, "binary": binary.reshape(tuple(resolution)),
            "threshold": thr, "repeated": repeated}
