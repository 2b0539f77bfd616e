"""GPU parity of the nerfacc-compatible operators (CUDA path vs oracle / reference kernels).

Bars: integer outputs (ray indices, packed info, visibility) bit-exact; the
marcher's t values bit-exact (same float32 op order as the reference);
weights forward bit-exact vs the reference kernel and within 1e-6 of the
float64 oracle; weight adjoint bit-exact vs the reference kernel."""
import json
from pathlib import Path

import numpy as np
import pytest
import torch

from oracle import march as omarch
from oracle import nerfacc_ref as R

pytestmark = pytest.mark.gpu
KAT = json.loads((Path(__file__).parent / "golden" / "nerfacc_kat.json").read_text())


@pytest.fixture(scope="module")
def nf(built_lib):
    from supernormal_gb300 import nerfacc

    return nerfacc


@pytest.fixture(scope="module")
def ref():
    from oracle import refkernels

    r = refkernels.load()
    if isinstance(r, Exception):
        pytest.skip(f"reference checker kernels unavailable: {r}")
    return r


def T(x, dtype=torch.float32):
    return torch.as_tensor(np.asarray(x), dtype=dtype, device="cuda")


def test_kat_visibility_transmittance_weights(nf):
    for c in KAT["visibility"]:
        ri = T(c["ray_indices"], torch.int64)
        vis = nf.render_visibility(T(c["alphas"])[:, None], ray_indices=ri, n_rays=c["n_rays"],
                                   early_stop_eps=c["early_stop_eps"], alpha_thre=c["alpha_thre"])
        assert vis.cpu().tolist() == c["expect"], c["cite"]
    for c in KAT["transmittance"]:
        ri = T(c["ray_indices"], torch.int64)
        Tt = nf.render_transmittance_from_alpha(T(c["alphas"])[:, None], ray_indices=ri,
                                                n_rays=c["n_rays"])
        np.testing.assert_allclose(Tt.cpu().numpy().ravel(), c["expect"], atol=1e-6, err_msg=c["cite"])
    for c in KAT["weights"]:
        ri = T(c["ray_indices"], torch.int64)
        w = nf.render_weight_from_alpha(T(c["alphas"])[:, None], ray_indices=ri, n_rays=c["n_rays"])
        np.testing.assert_allclose(w.cpu().numpy().ravel(), c["expect"], atol=c["atol"], err_msg=c["cite"])


def test_kat_density_grads(nf):
    for c in KAT["weights_from_density_grads"]:
        sig = T(c["sigmas"])[:, None].requires_grad_(True)
        alphas = 1.0 - torch.exp(-sig * c["delta"])
        for kw in ({"ray_indices": T(c["ray_indices"], torch.int64), "n_rays": c["n_rays"]},
                   {"packed_info": T(c["packed_info"], torch.int32)}):
            w = nf.render_weight_from_alpha(alphas, **kw)
            (g,) = torch.autograd.grad(w.sum(), sig, retain_graph=True)
            np.testing.assert_allclose(w.detach().cpu().numpy().ravel(), c["weights"], atol=c["atol"])
            np.testing.assert_allclose(g.cpu().numpy().ravel(), c["sigmas_grad_of_sum"], atol=c["atol"])


def test_kat_accumulate_and_pack(nf):
    c = KAT["accumulate"][0]
    ri = T(c["ray_indices"], torch.int64)
    w = T(c["weights"])[:, None]
    v = torch.rand((5, c["values_dim"]), device="cuda")
    out = nf.accumulate_along_rays(w, ri, values=v, n_rays=3)
    assert out.shape == (3, 2)
    torch.testing.assert_close(out[0], w[0] * v[0])
    assert (out[1] == 0).all()
    torch.testing.assert_close(out[2], (w[1:] * v[1:]).sum(0))
    p = KAT["pack"][0]
    packed = T(p["packed_info"], torch.int32)
    ri2 = nf.unpack_info(packed, p["n_samples"])
    assert ri2.cpu().tolist() == p["ray_indices"]
    assert nf.pack_info(ri2, n_rays=3).cpu().tolist() == p["packed_info"]


@pytest.mark.parametrize("P,n_patches", [(9, 1), (9, 300), (1, 1000), (25, 64)])
def test_patch_weights_vs_oracle(nf, P, n_patches):
    g = torch.Generator(device="cuda").manual_seed(P + n_patches)
    counts = torch.randint(0, 40, (n_patches,), device="cuda", generator=g)
    counts[0] = 0  # an empty patch
    ri = torch.repeat_interleave(torch.arange(n_patches, device="cuda"), counts)
    a = torch.rand((ri.numel(), P, 1), device="cuda", generator=g) ** 3
    a = a.requires_grad_(True)
    w = nf.render_weight_from_alpha_patch_based(a, ri, n_rays=n_patches)
    gw = torch.randn_like(w)
    (ga,) = torch.autograd.grad(w, a, gw)
    packed = R.pack_info(ri.cpu().numpy(), n_patches)
    an = a.detach().cpu().numpy().reshape(-1, P)
    w_ref = R.weights_fwd(an, packed, P)
    np.testing.assert_allclose(w.detach().cpu().numpy().reshape(-1, P), w_ref, atol=1e-6)
    wn = w.detach().cpu().numpy().reshape(-1, P)
    gn = gw.cpu().numpy().reshape(-1, P)
    ga_ref = R.weights_bwd(an, wn, gn, packed, P)
    # The reference adjoint (g*T - sum_{i>=j} g_i w_i) / (1 - alpha) is formed in
    # float32: its rounding error is ~eps32 * (|g T| + sum |g_i w_i|) / (1 - alpha).
    scale = np.zeros_like(an)
    for b, c in packed:
        if c:
            scale[b:b + c] = np.abs(gn[b:b + c] * wn[b:b + c]).sum(0)
    tol = 1e-5 + 1e-4 * np.abs(ga_ref) + 8 * 1.2e-7 * (scale + np.abs(gn)) / np.maximum(1 - an, 1e-10)
    assert (np.abs(ga.cpu().numpy().reshape(-1, P) - ga_ref) <= tol).all()


def test_patch_weights_bit_exact_vs_reference_kernel(nf, ref):
    g = torch.Generator(device="cuda").manual_seed(7)
    n_patches, P = 512, 9
    counts = torch.randint(0, 80, (n_patches,), device="cuda", generator=g)
    ri = torch.repeat_interleave(torch.arange(n_patches, device="cuda"), counts)
    a = (torch.rand((ri.numel(), P, 1), device="cuda", generator=g) ** 4).contiguous()
    packed = nf.pack_info(ri, n_rays=n_patches)
    w_ref = ref.patch_weight_fwd(packed, a)
    a_req = a.clone().requires_grad_(True)
    w = nf.render_weight_from_alpha_patch_based(a_req, ri, n_rays=n_patches)
    assert torch.equal(w.detach(), w_ref)
    gw = torch.randn_like(w).contiguous()
    (ga,) = torch.autograd.grad(w, a_req, gw)
    ga_ref = ref.patch_weight_bwd(packed, a, w_ref, gw)
    assert torch.equal(ga, ga_ref)


def _march_case(seed, n=2048, res=(128, 128, 128), occ=0.3):
    rng = np.random.default_rng(seed)
    ang = rng.random((n, 2)) * np.array([2 * np.pi, np.pi])
    eye = np.stack([np.sin(ang[:, 1]) * np.cos(ang[:, 0]), np.sin(ang[:, 1]) * np.sin(ang[:, 0]),
                    np.cos(ang[:, 1])], 1) * 3.0
    tgt = (rng.random((n, 3)) - 0.5) * 1.2
    d = tgt - eye
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    o = eye.astype(np.float32)
    d = d.astype(np.float32)
    b = 2 * (o * d).sum(1)
    c = (o * o).sum(1) - 1
    disc = np.maximum(b * b - 4 * c, 0)
    near = ((-b - np.sqrt(disc)) / 2).astype(np.float32)
    far = ((-b + np.sqrt(disc)) / 2).astype(np.float32)
    # a blobby occupancy pattern (sphere shell + noise) on the 128^3 grid
    g = np.stack(np.meshgrid(*[np.linspace(-1, 1, r) for r in res], indexing="ij"), -1)
    rad = np.linalg.norm(g, axis=-1)
    grid = ((np.abs(rad - 0.5) < 0.08) | (rng.random(res) < occ * 0.02)).astype(np.uint8)
    jitter = rng.random(n).astype(np.float32)
    return o, d, near, far, grid, jitter


@pytest.mark.parametrize("step", [2.0 / 1024, 1e-2, 3.7e-3])
def test_marcher_bit_exact_vs_oracle(nf, step):
    o, d, near, far, grid, jitter = _march_case(int(step * 1e6))
    roi = np.array([-1, -1, -1, 1, 1, 1], np.float32)
    packed_r, ri_r, ts_r, te_r = omarch.ray_marching(o, d, near, far, roi, grid, step, jitter=jitter)
    packed, ri, ts, te = nf.march_packed(T(o), T(d), T(near), T(far), _grid(nf, grid), step, 0.0,
                                         jitter=T(jitter))
    assert torch.equal(packed.cpu(), torch.from_numpy(packed_r))
    assert torch.equal(ri.cpu(), torch.from_numpy(ri_r))
    assert np.array_equal(ts.cpu().numpy().ravel().view(np.uint32), ts_r.view(np.uint32))
    assert np.array_equal(te.cpu().numpy().ravel().view(np.uint32), te_r.view(np.uint32))
    assert ri_r.size > 1000


def test_marcher_bit_exact_vs_reference_kernel(nf, ref):
    o, d, near, far, grid, jitter = _march_case(11)
    step = 2.0 / 1024
    t_min = T(near) + T(jitter) * step   # the reference applies jitter in torch before the kernel
    roi = T([-1, -1, -1, 1, 1, 1])
    g = _grid(nf, grid)
    packed_r, ri_r, ts_r, te_r = ref.ray_marching(T(o), T(d), t_min.contiguous(), T(far), roi,
                                                  g.binary.contiguous(), step)
    packed, ri, ts, te = nf.march_packed(T(o), T(d), T(near), T(far), g, step, 0.0, jitter=T(jitter))
    assert torch.equal(packed, packed_r)
    assert torch.equal(ri, ri_r)
    assert torch.equal(ts, ts_r) and torch.equal(te, te_r)


def test_padded_single_pass_marcher_matches(nf):
    from supernormal_gb300._lib import call, stream_handle

    o, d, near, far, grid, jitter = _march_case(21)
    step = 2.0 / 1024
    g = _grid(nf, grid)
    packed, ri, ts, te = nf.march_packed(T(o), T(d), T(near), T(far), g, step, 0.0, jitter=T(jitter))
    n = o.shape[0]
    stride = int(np.ceil(2.0 / step)) + 3
    st = stream_handle()
    counts = torch.empty(n, dtype=torch.int32, device="cuda")
    rp = torch.empty(n * stride, dtype=torch.int64, device="cuda")
    tsp = torch.empty(n * stride, device="cuda")
    tep = torch.empty(n * stride, device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    roi, binary, rx, ry, rz, ct = nf._grid_args(g, "cuda")
    # the step size from device memory (the scalar argument is then ignored)
    step_dev = torch.tensor([step], dtype=torch.float32, device="cuda")
    call("sn_march_padded", n, T(o), T(d), T(near), T(far), T(jitter), roi, binary, rx, ry, rz, ct, 123.0,
         step_dev, 0.0, 0, stride, counts, rp, tsp, tep, status, st)
    packed2, total = nf._pack_counts(counts)
    m = int(total.item())
    ri2 = torch.empty(m, dtype=torch.int64, device="cuda")
    ts2 = torch.empty(m, device="cuda")
    te2 = torch.empty(m, device="cuda")
    call("sn_compact_padded", n, stride, packed2, rp, tsp, tep, ri2, ts2, te2, st)
    assert int(status.item()) == 0
    assert torch.equal(packed2, packed) and torch.equal(ri2, ri)
    assert torch.equal(ts2, ts.ravel()) and torch.equal(te2, te.ravel())


def test_marcher_edge_cases(nf):
    # no rays; rays that miss the sphere (NaN near/far) give no samples; empty grid
    g = _grid(nf, np.ones((8, 8, 8), np.uint8))
    packed, ri, ts, te = nf.march_packed(T(np.zeros((0, 3))), T(np.zeros((0, 3))), T([]), T([]), g,
                                         0.01)
    assert ri.numel() == 0 and packed.shape == (0, 2)
    o = T([[0.0, 0.0, 5.0]])
    d = T([[1.0, 0.0, 0.0]])
    packed, ri, _, _ = nf.march_packed(o, d, T([float("nan")]), T([float("nan")]), g, 0.01)
    assert ri.numel() == 0
    with pytest.raises(Exception):
        nf.march_packed(o, d, T([0.0]), T([1.0]), g, 0.0)


def test_ray_marching_api_culling_matches_oracle(nf):
    o, d, near, far, grid, _ = _march_case(5, n=512)
    g = _grid(nf, grid)
    step = 5e-3

    def alpha_fn(t_starts, t_ends, ray_indices):
        mid = (t_starts + t_ends) / 2
        p = T(o)[ray_indices] + T(d)[ray_indices] * mid
        return torch.sigmoid((0.5 - p.norm(dim=-1, keepdim=True)) * 40.0)

    ri, ts, te = nf.ray_marching(T(o), T(d), t_min=T(near), t_max=T(far), grid=g,
                                 render_step_size=step, alpha_fn=alpha_fn, early_stop_eps=1e-3)
    packed_r, ri_r, ts_r, te_r = omarch.ray_marching(o, d, near, far, np.array([-1, -1, -1, 1, 1, 1],
                                                                                 np.float32), grid, step)
    a = alpha_fn(T(ts_r)[:, None], T(te_r)[:, None], T(ri_r, torch.int64)).cpu().numpy().ravel()
    vis = R.visibility(a.astype(np.float32), packed_r, 1e-3, dtype=np.float32)
    np.testing.assert_array_equal(ri.cpu().numpy(), ri_r[vis])
    np.testing.assert_array_equal(ts.cpu().numpy().ravel(), ts_r[vis])
    np.testing.assert_array_equal(te.cpu().numpy().ravel(), te_r[vis])


def test_occupancy_grid_every_n_step_properties(nf):
    """every_n_step end to end with torch's own draws (the bit-exact replay of the
    reference's draws is tests/test_gpu_occupancy.py)."""
    grid = nf.OccupancyGrid(roi_aabb=[-1.0, -1.0, -1.0, 1.0, 1.0, 1.0], resolution=32).cuda()
    occ_fn = lambda x: torch.sigmoid((0.5 - x.norm(dim=-1, keepdim=True)) * 80.0)
    torch.manual_seed(0)
    grid.every_n_step(0, occ_fn, occ_thre=0.1, n=8)
    occs = grid.occs.cpu().numpy()
    # cell centres up to jitter: occupancy is ~1 well inside r=0.5, ~0 well outside
    c = (np.stack(np.meshgrid(*[np.arange(32)] * 3, indexing="ij"), -1).reshape(-1, 3) + 0.5) / 32 * 2 - 1
    r = np.linalg.norm(c, axis=1)
    assert (occs[r < 0.4] > 0.99).all() and (occs[r > 0.6] < 0.01).all()
    thr = min(occs.mean(), 0.1)
    np.testing.assert_array_equal(grid.binary.cpu().numpy().ravel(), occs > thr)
    # second update (warm-up): EMA max with decay
    prev = occs.copy()
    grid.every_n_step(8, occ_fn, occ_thre=0.1, n=8)
    new = grid.occs.cpu().numpy()
    assert (new >= prev * 0.95 - 1e-7).all()
    # post-warm-up sampling path
    grid._update(300, occ_fn, occ_thre=0.1)
    assert torch.isfinite(grid.occs).all()
    with pytest.raises(RuntimeError):
        grid.eval()
        grid.every_n_step(0, occ_fn)


def _grid(nf, binary):
    res = list(binary.shape)
    g = nf.OccupancyGrid(roi_aabb=[-1.0, -1.0, -1.0, 1.0, 1.0, 1.0], resolution=res).cuda()
    g._binary = torch.as_tensor(binary.astype(bool), device="cuda")
    return g


@pytest.mark.parametrize("cap,live", [(0, 0), (5000, 0), (5000, 4096), (5000, 5000), (3 * 4096 + 7, 4097),
                                      (1 << 21, 190_000)])
def test_pack_counts_bounded_by_device_count(nf, cap, live):
    """sn_pack_counts_n: the packed prefix and total of the live entries,
    bit for bit as sn_pack_counts over those entries alone, and nothing
    written past the count (garbage past it is ignored)."""
    from supernormal_gb300._lib import call, stream_handle

    g = torch.Generator(device="cuda").manual_seed(cap + live)
    counts = torch.randint(0, 7, (cap,), dtype=torch.int32, device="cuda", generator=g)
    if cap > live:
        counts[live:] = 1 << 20                        # never read
    ws = torch.empty(int(call("sn_scan_workspace_bytes", max(cap, 1))), dtype=torch.uint8, device="cuda")
    packed = torch.full((max(cap, 1), 2), -5, dtype=torch.int32, device="cuda")
    total = torch.full((1,), -1, dtype=torch.int32, device="cuda")
    n_dev = torch.tensor([live], dtype=torch.int32, device="cuda")
    call("sn_pack_counts_n", cap, n_dev, counts, packed, total, ws, stream_handle())
    want_p = torch.full((max(live, 1), 2), -5, dtype=torch.int32, device="cuda")
    want_t = torch.zeros((1,), dtype=torch.int32, device="cuda")
    if live:
        call("sn_pack_counts", live, counts[:live].contiguous(), want_p, want_t, ws, stream_handle())
    torch.cuda.synchronize()
    assert int(total.item()) == int(want_t.item())
    if live:
        assert torch.equal(packed[:live], want_p[:live])
    if cap > live:
        assert (packed[live:cap] == -5).all()


def test_marcher_limits_report_status_without_faulting(nf):
    """Failure detection through the device status word, with no GPU fault:
    a marching iteration limit below what the rays need sets
    SN_STATUS_MARCH_LIMIT (each ray stops where the limit struck, the call
    itself succeeds); per-ray slots shorter than a ray's samples set
    SN_STATUS_CAPACITY and keep the samples that fit, which equal the
    unbounded marcher's first samples; a status word is only ever OR-ed."""
    from supernormal_gb300._lib import SN_STATUS_CAPACITY, SN_STATUS_MARCH_LIMIT, call, stream_handle

    o, d, near, far, grid, jitter = _march_case(21)
    step = 2.0 / 1024
    g = _grid(nf, grid)
    n = o.shape[0]
    st = stream_handle()
    roi, binary, rx, ry, rz, ct = nf._grid_args(g, "cuda")
    args = (T(o), T(d), T(near), T(far), T(jitter), roi, binary, rx, ry, rz, ct, step)
    full = torch.empty(n, dtype=torch.int32, device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    call("sn_march_count", n, *args, 0.0, 0, full, status, st)
    assert int(status.item()) == 0 and int(full.max().item()) > 8
    # iteration limit
    limited = torch.empty_like(full)
    call("sn_march_count", n, *args, 0.0, 4, limited, status, st)
    assert int(status.item()) & SN_STATUS_MARCH_LIMIT
    assert bool((limited <= full).all()) and bool((limited < full).any())
    # slot capacity: slots of 8 samples
    stride = 8
    counts = torch.empty_like(full)
    rp = torch.full((n * stride,), -1, dtype=torch.int64, device="cuda")
    tsp = torch.empty(n * stride, device="cuda")
    tep = torch.empty(n * stride, device="cuda")
    status2 = torch.full((1,), 0x100, dtype=torch.int32, device="cuda")     # an unrelated bit, kept
    call("sn_march_padded", n, *args, None, 0.0, 0, stride, counts, rp, tsp, tep, status2, st)
    s2 = int(status2.item())
    assert s2 & SN_STATUS_CAPACITY and s2 & 0x100
    packed, ri, ts, te = nf.march_packed(T(o), T(d), T(near), T(far), g, step, 0.0, jitter=T(jitter))
    pk = packed.cpu().numpy()
    rpv, tsv = rp.view(n, stride).cpu().numpy(), tsp.view(n, stride).cpu().numpy()
    tsr = ts.ravel().cpu().numpy()
    for r in range(n):
        b, c = pk[r]
        k = min(c, stride)
        assert (rpv[r, :k] == r).all()
        assert np.array_equal(tsv[r, :k], tsr[b:b + k])
