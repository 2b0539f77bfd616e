"""Tensor-core (tcgen05, 3xTF32) MLP pieces against float64 torch.

3xTF32 keeps products to ~2^-21 relative; over K <= 64 fp32-accumulated terms
the result is within 2e-6 of the largest output (float32 itself is ~1e-7)."""
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,k", [(1, 35), (128, 35), (1000, 35), (4099, 8), (777, 64), (300, 3)])
def test_linear_tc_matches_float64(built_lib, n, k):
    from supernormal_gb300._lib import call, stream_handle

    g = torch.Generator(device="cuda").manual_seed(n * 131 + k)
    x = torch.randn((n, k), device="cuda", generator=g)
    w = torch.randn((64, k), device="cuda", generator=g) * 0.3
    b = torch.randn((64,), device="cuda", generator=g)
    y = torch.full((n, 64), float("nan"), device="cuda")
    status = torch.zeros((1,), dtype=torch.int32, device="cuda")
    call("sn_linear_tc", n, k, x, w, b, y, status, stream_handle())
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    ref = x.double() @ w.double().T + b.double()
    err = (y.double() - ref).abs().max().item() / ref.abs().max().item()
    assert err < 2e-6, err
    # no bias, a second call on the same buffers
    call("sn_linear_tc", n, k, x, w, None, y, status, stream_handle())
    torch.cuda.synchronize()
    ref = x.double() @ w.double().T
    assert (y.double() - ref).abs().max().item() / ref.abs().max().item() < 2e-6
