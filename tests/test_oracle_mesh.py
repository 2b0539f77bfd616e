"""The host restatement of the device marching cubes (oracle/mesh.py): its
vertices are the lattice-edge crossings, and its triangles form closed,
consistently oriented surfaces on fields with every ambiguous face case."""
import numpy as np
import pytest

from oracle import mesh as OMS


def _check(v, t):
    e = np.concatenate([t[:, [0, 1]], t[:, [1, 2]], t[:, [2, 0]]])
    assert len({tuple(x) for x in e.tolist()}) == len(e)
    _, cnt = np.unique(np.sort(e, axis=1), axis=0, return_counts=True)
    assert (cnt == 2).all()
    return len(v) - len(cnt) + len(t)


def test_table_cases():
    tab = OMS.mc_table()
    assert len(tab[0]) == 0 and len(tab[255]) == 0 and len(tab[1]) == 1 and len(tab[15]) == 2
    assert max(len(t) for t in tab) <= 5
    # complementary cases cover the same edges
    for c in range(256):
        a = sorted({e for tri in tab[c] for e in tri})
        b = sorted({e for tri in tab[255 - c] for e in tri})
        assert a == b


@pytest.mark.parametrize("seed", [0, 1])
def test_random_fields_are_closed(seed):
    rng = np.random.default_rng(seed)
    u = rng.uniform(-1, 1, (14, 12, 10)).astype(np.float32)
    u[0], u[-1], u[:, 0], u[:, -1], u[:, :, 0], u[:, :, -1] = -1, -1, -1, -1, -1, -1
    v, t = OMS.marching_cubes(u, 0.0, (0, 0, 0), (13, 11, 9))
    ref = OMS.edge_crossings(u, 0.0, (0, 0, 0), (13, 11, 9))
    assert len(v) == len(ref) and len(t) > 100
    np.testing.assert_allclose(v[np.lexsort(v.T)], ref[np.lexsort(ref.T)], atol=1e-5)
    _check(v, t)


def test_sphere_euler():
    g = np.linspace(-1, 1, 24)
    x, y, z = np.meshgrid(g, g, g, indexing="ij")
    v, t = OMS.marching_cubes((0.6 - np.sqrt(x * x + y * y + z * z)).astype(np.float32), 0.0, (-1,) * 3, (1,) * 3)
    assert _check(v, t) == 2
