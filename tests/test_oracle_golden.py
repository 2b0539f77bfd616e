"""The oracle against nerfacc's own known-answer vectors (CPU)."""
import json
from pathlib import Path

import numpy as np

from oracle import nerfacc_ref as R

KAT = json.loads((Path(__file__).parent / "golden" / "nerfacc_kat.json").read_text())


def test_visibility_kat():
    for c in KAT["visibility"]:
        packed = R.pack_info(c["ray_indices"], c["n_rays"])
        vis = R.visibility(c["alphas"], packed, c["early_stop_eps"], c["alpha_thre"])
        assert vis.tolist() == c["expect"], c["cite"]


def test_transmittance_kat():
    for c in KAT["transmittance"]:
        packed = R.pack_info(c["ray_indices"], c["n_rays"])
        T = R.transmittance(c["alphas"], packed).reshape(-1)
        np.testing.assert_allclose(T, c["expect"], atol=1e-12, err_msg=c["cite"])


def test_weights_kat():
    for c in KAT["weights"]:
        packed = R.pack_info(c["ray_indices"], c["n_rays"])
        w = R.weights_fwd(c["alphas"], packed)
        np.testing.assert_allclose(w, c["expect"], atol=c["atol"], err_msg=c["cite"])


def test_weights_from_density_grads_kat():
    for c in KAT["weights_from_density_grads"]:
        packed = np.array(c["packed_info"], dtype=np.int32)
        sig = np.array(c["sigmas"])
        alpha = 1.0 - np.exp(-sig * c["delta"])
        w = R.weights_fwd(alpha, packed)
        np.testing.assert_allclose(w, c["weights"], atol=c["atol"], err_msg=c["cite"])
        ga = R.weights_bwd(alpha, w, np.ones_like(w), packed)
        gs = ga * (1.0 - alpha) * c["delta"]
        np.testing.assert_allclose(gs, c["sigmas_grad_of_sum"], atol=c["atol"], err_msg=c["cite"])
        assert (R.pack_info(c["ray_indices"], c["n_rays"]) == packed).all()


def test_accumulate_kat():
    rng = np.random.default_rng(0)
    for c in KAT["accumulate"]:
        w = np.array(c["weights"])[:, None]
        v = rng.random((len(c["weights"]), c["values_dim"]))
        out = R.accumulate(w, c["ray_indices"], v[:, None, :], c["n_rays"])[:, 0, :]
        np.testing.assert_allclose(out[0], w[0] * v[0])
        assert (out[1] == 0).all()
        np.testing.assert_allclose(out[2], (w[1:] * v[1:]).sum(0))


def test_pack_roundtrip_kat():
    for c in KAT["pack"]:
        ri = R.unpack_info(c["packed_info"], c["n_samples"])
        assert ri.tolist() == c["ray_indices"]
        assert R.pack_info(ri, len(c["packed_info"])).tolist() == c["packed_info"]


def test_patch_weights_reduce_to_per_ray():
    """A patch of P lanes is P independent rays with the same packing."""
    rng = np.random.default_rng(1)
    ri = np.sort(rng.integers(0, 7, 40))
    packed = R.pack_info(ri, 7)
    a = rng.random((40, 9))
    w = R.weights_fwd(a, packed, patch_size=9)
    for k in range(9):
        np.testing.assert_allclose(w[:, k], R.weights_fwd(a[:, k], packed))
    g = rng.standard_normal((40, 9))
    ga = R.weights_bwd(a, w, g, packed, patch_size=9)
    for k in range(9):
        np.testing.assert_allclose(ga[:, k], R.weights_bwd(a[:, k], w[:, k], g[:, k], packed))
