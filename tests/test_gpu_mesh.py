"""Device mesh extraction (models/renderer.py:9-34, 353-358): lattice values
against the oracle's extract_fields, vertices against the lattice-edge
crossings every marching-cubes variant produces, and the triangles by their
properties: closed, consistently oriented, outward, Euler characteristic."""
import numpy as np
import pytest
import torch

from oracle import mesh as OMS

pytestmark = pytest.mark.gpu


def _mc(u, thr=0.0, lo=(-1.0, -1.0, -1.0), hi=(1.0, 1.0, 1.0)):
    from supernormal_gb300.mesh import marching_cubes

    v, t = marching_cubes(torch.as_tensor(u, device="cuda"), thr, lo, hi)
    return v.double().cpu().numpy(), t.long().cpu().numpy()


def _topology(v, t, closed=True):
    e = np.concatenate([t[:, [0, 1]], t[:, [1, 2]], t[:, [2, 0]]])
    directed = {tuple(x) for x in e.tolist()}
    assert len(directed) == len(e), "a directed edge appears twice: inconsistent orientation"
    und = np.sort(e, axis=1)
    _, cnt = np.unique(und, axis=0, return_counts=True)
    if closed:
        assert (cnt == 2).all(), "open or non-manifold edges"
    else:                                  # cut by the lattice's box: boundary edges once
        assert (cnt <= 2).all(), "non-manifold edges"
    return len(v) - len(cnt) + len(t)     # Euler characteristic


def _lattice(f, res, lo=-1.0, hi=1.0):
    g = np.linspace(lo, hi, res)
    x, y, z = np.meshgrid(g, g, g, indexing="ij")
    return f(x, y, z).astype(np.float32)


def test_sphere_mesh():
    u = _lattice(lambda x, y, z: 0.5 - np.sqrt(x * x + y * y + z * z), 48)   # -sdf of a sphere
    v, t = _mc(u)
    ref = OMS.edge_crossings(u, 0.0, (-1, -1, -1), (1, 1, 1))
    assert len(v) == len(ref)
    np.testing.assert_allclose(v[np.lexsort(v.T)], ref[np.lexsort(ref.T)], atol=2e-6)
    assert _topology(v, t) == 2
    c = v[t].mean(1)
    n = np.cross(v[t[:, 1]] - v[t[:, 0]], v[t[:, 2]] - v[t[:, 0]])
    assert ((n * c).sum(1) > 0).all()                                    # normals point outward
    assert np.abs(np.linalg.norm(v, axis=1) - 0.5).max() < 0.01


def test_torus_mesh_genus_one():
    def f(x, y, z):
        q = np.sqrt(x * x + y * y) - 0.5
        return 0.2 - np.sqrt(q * q + z * z)
    v, t = _mc(_lattice(f, 64))
    assert _topology(v, t) == 0


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_random_field_is_watertight(seed):
    """Random values (every ambiguous face configuration occurs) inside a
    border that is outside: closed, consistently oriented surfaces."""
    rng = np.random.default_rng(seed)
    u = rng.uniform(-1, 1, (24, 20, 18)).astype(np.float32)
    u[0], u[-1], u[:, 0], u[:, -1], u[:, :, 0], u[:, :, -1] = -1, -1, -1, -1, -1, -1
    v, t = _mc(u, 0.0, (0, 0, 0), (23, 19, 17))
    ref = OMS.edge_crossings(u, 0.0, (0, 0, 0), (23, 19, 17))
    assert len(v) == len(ref) and len(t) > 100
    np.testing.assert_allclose(v[np.lexsort(v.T)], ref[np.lexsort(ref.T)], atol=2e-5)
    _topology(v, t)
    # the host restatement numbers vertices the same way: identical triangles
    hv, ht = OMS.marching_cubes(u, 0.0, (0, 0, 0), (23, 19, 17))
    np.testing.assert_array_equal(t, ht)
    np.testing.assert_allclose(v, hv, atol=2e-5)


def test_empty_and_capacity():
    from supernormal_gb300._lib import call, stream_handle

    u = torch.full((8, 8, 8), -1.0, device="cuda")
    v, t = _mc(u.cpu().numpy())
    assert v.shape == (0, 3) and t.shape == (0, 3)
    # outputs are written only up to the given capacity; the counts are exact
    uu = torch.as_tensor(_lattice(lambda x, y, z: 0.5 - np.sqrt(x * x + y * y + z * z), 16), device="cuda")
    ws = torch.empty(int(call("sn_marching_cubes_workspace_bytes", 16, 16, 16)), dtype=torch.uint8, device="cuda")
    counts = torch.zeros(2, dtype=torch.int32, device="cuda")
    verts = torch.full((10, 3), 7.0, device="cuda")
    tris = torch.full((5, 3), -7, dtype=torch.int32, device="cuda")
    lo = np.array([-1.0, -1.0, -1.0])
    hi = np.array([1.0, 1.0, 1.0])
    call("sn_marching_cubes", uu, 16, 16, 16, 0.0, lo.ctypes.data, hi.ctypes.data, 10, 5, verts, tris, counts, ws,
         stream_handle())
    n_v, n_t = counts.tolist()
    assert n_v > 10 and n_t > 5 and (tris >= 0).all()


def test_sdf_network_extract_geometry_matches_oracle_lattice(built_lib):
    """NeuSRenderer.extract_geometry: the -sdf lattice of the fused field
    against the oracle's extract_fields with the float64 field, then a mesh
    whose vertices are the crossings of that lattice."""
    from oracle import field as OF
    from supernormal_gb300.fields import SDFNetwork, SingleVarianceNetwork
    from supernormal_gb300.mesh import sdf_lattice
    from supernormal_gb300.renderer import NeuSRenderer

    enc = dict(otype="HashGrid", n_levels=16, n_features_per_level=2, log2_hashmap_size=15,
               base_resolution=16, per_level_scale=1.447)
    torch.manual_seed(0)
    net = SDFNetwork(3, 1, 64, 1, skip_in=(-1,), bias=0.5, encoding_config=enc, input_concat=True)
    with torch.no_grad():
        net.encoding.params.mul_(300.0)
        net.lin0.weight_v[:, 3:].normal_(0.0, 0.05)
    net.bindwidth = 16
    net = net.cuda()
    lo, hi = torch.tensor([-1.0, -1.0, -1.0]), torch.tensor([1.0, 1.0, 1.0])
    u = sdf_lattice(net, lo, hi, 40).cpu().numpy()
    prm = OF.params_from_module(net)
    geom = OF.geometry_from_module(net)
    ref = OMS.extract_fields(lo, hi, 40, lambda p: -OF.sdf_network(p, **prm, geom=geom, active_levels=16,
                                                                    out_cols=1))
    assert np.abs(u - ref).max() < 2e-5 * max(1.0, np.abs(ref).max())
    r = NeuSRenderer(net, SingleVarianceNetwork(0.3).cuda())
    v, t = r.extract_geometry(lo, hi, 40)
    assert v.dtype == np.float64 and t.dtype == np.int64 and len(t) > 100
    crossing = OMS.edge_crossings(u, 0.0, lo.numpy(), hi.numpy())
    assert len(v) == len(crossing)
    _topology(v, t, closed=False)         # this field's zero set reaches the box
    hv, ht = OMS.marching_cubes(u, 0.0, lo.numpy(), hi.numpy())
    np.testing.assert_array_equal(t, ht)
