"""The occupancy-update oracle against nerfacc's own grid.py, run on CPU.

The fixture (tests/golden/make_occupancy.py) ran ``OccupancyGrid._update``
of NA/nerfacc/grid.py unmodified for a warm-up step, a sampled step with
repeated cells and planted stale occupancy, and a step that takes the
occupied-cell selector.  Bars: sampling, query points, EMA and
binarisation bit-exact; a repeated cell's stored value is one of its
candidates (the reference's index_put keeps an unspecified one), and the
oracle's choice is the largest."""
from pathlib import Path

import numpy as np
import pytest
import torch

from oracle import occupancy as OO

FIX = np.load(Path(__file__).parent / "golden" / "reference_occupancy.npz")
STEPS = [str(s) for s in FIX["steps"]]


@pytest.mark.parametrize("tag", STEPS)
def test_sampling_and_points(tag):
    f = lambda k: FIX[f"{tag}/{k}"]
    res, roi = FIX["resolution"], FIX["roi"]
    if int(f("step")) >= 256:
        n = int(np.prod(res)) // 4
        sel = f("selector") if f("selector").size else None
        cells = OO.sample_cells(f("binary_before"), n, f("uniform"), sel)
        np.testing.assert_array_equal(cells, f("cells"))
    else:
        cells = None
        np.testing.assert_array_equal(f("cells"), np.arange(int(np.prod(res))))
    x = OO.query_points(cells, f("jitter"), res, roi)
    np.testing.assert_array_equal(x, f("x"))


@pytest.mark.parametrize("tag", STEPS)
def test_ema_and_binarize(tag):
    f = lambda k: FIX[f"{tag}/{k}"]
    cells = None if int(f("step")) < 256 else f("cells")
    new, repeated = OO.ema_update(f("occs_before"), cells, f("occ"), 0.95)
    ref = f("occs_after")
    rep = np.array(sorted(repeated), dtype=np.int64)
    mask = np.ones(ref.size, bool)
    mask[rep] = False
    np.testing.assert_array_equal(new[mask], ref[mask])
    for c, cand in repeated.items():
        assert ref[c] in cand, (tag, c)              # the reference stored one candidate
        assert new[c] == cand.max()                  # the oracle (and GPU) keeps the largest
    if tag == "sampled":
        assert len(repeated) > 0
    binary, thr = OO.binarize(ref, float(f("occ_thre")))
    near = np.abs(ref - thr) <= 4 * np.spacing(np.float32(thr))
    b_ref = f("binary_after").reshape(-1)
    np.testing.assert_array_equal(binary.reshape(-1)[~near], b_ref[~near])


def test_planted_cells_decay():
    """Cells that held occupancy the field no longer has decay by 0.95 when sampled."""
    f = lambda k: FIX[f"sampled/{k}"]
    planted = FIX["planted"]
    hit = np.intersect1d(planted, f("cells"))
    assert hit.size > 10
    before, after = f("occs_before")[hit], f("occs_after")[hit]
    occ_max = np.array([f("occ")[f("cells") == c].max() for c in hit])
    np.testing.assert_array_equal(after, np.maximum((before * np.float32(0.95)).astype(np.float32), occ_max))
    assert (after < before).all()


def test_occ_from_sdf_matches_torch_sigmoid():
    g = torch.Generator().manual_seed(0)
    sdf = (torch.rand(4096, generator=g) - 0.5) * 0.4
    ref = torch.sigmoid(-sdf * 80).numpy()
    got = OO.occ_from_sdf(sdf.numpy())
    np.testing.assert_allclose(got, ref, rtol=4e-7, atol=0)   # host exp implementations: a few ulp
