"""Generate the occupancy-update fixture by running nerfacc's own grid.py on CPU.

Loads NA/nerfacc/grid.py and NA/nerfacc/contraction.py (NA =
third_parties/nerfacc-0.3.5/nerfacc-0.3.5) unmodified from the SuperNormal
tree, with the compiled extension ``nerfacc.cuda`` replaced by a stub whose
``contract_inv`` is the oracle's AABB restatement (the only op of
``OccupancyGrid._update`` that calls the extension), and runs
``OccupancyGrid._update`` three times on a 16^3 grid:

  * step 0 (warm-up: every cell);
  * step 300 (uniform + occupied cells: repeated cells occur) after cells
    that the field no longer occupies were given high occupancy, so the
    decay of a sampled cell shows;
  * step 600 with more occupied cells than uniform draws (the selector path).

``torch.randint`` and ``torch.rand_like`` inside grid.py are recorded (the
module's ``torch`` name is a recording proxy), so the test can replay the
reference's own draws.  One CPU thread: the CPU index_put then stores a
repeated cell's last candidate.

Writes tests/golden/reference_occupancy.npz.
Usage:  python tests/golden/make_occupancy.py  [SuperNormal tree; default $SUPERNORMAL_REFERENCE, else "reference" beside the repository]
"""
from __future__ import annotations

import importlib.util
import os
import sys
import types
from pathlib import Path

import numpy as np
import torch

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))

from oracle import march as OM  # noqa: E402

REC: dict = {}


class RecordingTorch:
    """``torch`` as grid.py sees it: randint / rand_like outputs are recorded."""

    def __getattr__(self, name):
        return getattr(torch, name)

    def randint(self, *a, **k):
        r = torch.randint(*a, **k)
        REC.setdefault("randint", []).append(r.clone())
        return r

    def rand_like(self, *a, **k):
        r = torch.rand_like(*a, **k)
        REC["jitter"] = r.clone()
        return r


def load_reference_grid(ref_root: Path):
    na = ref_root / "third_parties" / "nerfacc-0.3.5" / "nerfacc-0.3.5" / "nerfacc"
    pkg = types.ModuleType("nerfacc")
    pkg.__path__ = [str(na)]
    cuda = types.ModuleType("nerfacc.cuda")
    cuda.ContractionTypeGetter = lambda v: v

    def contract_inv(x, roi, ctype):
        assert ctype == 0, "only the AABB contraction is restated"
        REC["x_unit"] = x.clone()
        return torch.from_numpy(OM.unit_to_roi(x.numpy(), roi.numpy()))

    cuda.contract_inv = contract_inv
    sys.modules.update({"nerfacc": pkg, "nerfacc.cuda": cuda})
    mods = {}
    for name in ("contraction", "grid"):
        spec = importlib.util.spec_from_file_location(f"nerfacc.{name}", na / f"{name}.py")
        m = importlib.util.module_from_spec(spec)
        sys.modules[f"nerfacc.{name}"] = m
        spec.loader.exec_module(m)
        mods[name] = m
    mods["grid"].torch = RecordingTorch()
    return mods["grid"]


def main(ref_root: str):
    torch.set_num_threads(1)
    grid_mod = load_reference_grid(Path(ref_root))
    torch.manual_seed(0)
    grid = grid_mod.OccupancyGrid(roi_aabb=[-1.0, -1.0, -1.0, 1.0, 1.0, 1.0], resolution=16)
    grid.train()

    def sdf_a(x):   # displaced sphere
        r = torch.linalg.vector_norm(x, dim=-1)
        return r - 0.5 + 0.05 * torch.sin(7.0 * x[..., 0]) * torch.sin(5.0 * x[..., 1])

    def make_eval(sdf):
        def occ_eval_fn(x):   # models/renderer.py:56-60 with an analytic sdf
            REC["x"] = x.clone()
            occ = torch.sigmoid(-sdf(x)[..., None] * 80)
            REC["occ"] = occ.clone()
            return occ
        return occ_eval_fn

    out = {}
    steps = []

    def run(tag, step, sdf, occ_thre):
        REC.clear()
        before_occs = grid.occs.clone()
        before_bin = grid._binary.clone()
        grid._update(step=step, occ_eval_fn=make_eval(sdf), occ_thre=occ_thre, ema_decay=0.95,
                     warmup_steps=256)
        draws = REC.get("randint", [])
        cells = np.arange(grid.num_cells) if step < 256 else torch.cat(
            [draws[0], _occupied(before_bin, draws)]).numpy()
        out.update({f"{tag}/step": step, f"{tag}/occ_thre": occ_thre,
                    f"{tag}/occs_before": before_occs.numpy(),
                    f"{tag}/binary_before": before_bin.numpy(),
                    f"{tag}/uniform": draws[0].numpy() if draws else np.zeros(0, np.int64),
                    f"{tag}/selector": draws[1].numpy() if len(draws) > 1 else np.zeros(0, np.int64),
                    f"{tag}/cells": cells, f"{tag}/jitter": REC["jitter"].numpy(),
                    f"{tag}/x_unit": REC["x_unit"].numpy(), f"{tag}/x": REC["x"].numpy(),
                    f"{tag}/occ": REC["occ"].numpy().reshape(-1),
                    f"{tag}/occs_after": grid.occs.numpy().copy(),
                    f"{tag}/binary_after": grid._binary.numpy().copy()})
        steps.append(tag)

    def _occupied(binary, draws):
        occ = torch.nonzero(binary.flatten())[:, 0]
        return occ[draws[1]] if len(draws) > 1 else occ

    run("warmup", 0, sdf_a, 0.1)
    # cells outside the surface that once were occupied: the sampled ones must decay
    with torch.no_grad():
        far = torch.nonzero(grid.occs < 1e-3)[:, 0]
        g = torch.Generator().manual_seed(5)
        planted = far[torch.randperm(far.numel(), generator=g)[:400]]
        grid.occs[planted] = 0.9
    out["planted"] = planted.numpy()
    run("sampled", 300, sdf_a, 0.1)
    # more occupied cells than uniform draws: the selector branch
    with torch.no_grad():
        g = torch.Generator().manual_seed(6)
        grid._binary = (torch.rand(grid._binary.shape, generator=g) < 0.4)
    run("selected", 600, sdf_a, 0.1)
    out["steps"] = np.array(steps)
    out["resolution"] = np.array([16, 16, 16])
    out["roi"] = np.array([-1, -1, -1, 1, 1, 1], np.float32)
    np.savez_compressed(HERE / "reference_occupancy.npz", **out)
    print("wrote", HERE / "reference_occupancy.npz")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.environ.get("SUPERNORMAL_REFERENCE", str(Path(__file__).resolve().parents[3] / "reference")))
