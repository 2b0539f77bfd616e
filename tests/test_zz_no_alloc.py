"""sn_pack_counts_static (no allocation, static device scratch) against
sn_pack_counts (caller workspace), through the C ABI, two calls in a row.

Collected last so it also runs after every other test in the same process."""
import pytest
import torch

pytestmark = pytest.mark.gpu


def _pack(lib_call, name, counts, ws=None):
    from supernormal_gb300._lib import stream_handle

    n = counts.numel()
    packed = torch.full((n, 2), -7, dtype=torch.int32, device="cuda")
    total = torch.full((1,), -7, dtype=torch.int32, device="cuda")
    args = [n, counts, packed, total] + ([ws] if name == "sn_pack_counts" else []) + [stream_handle()]
    lib_call(name, *args)
    return packed, total


@pytest.mark.parametrize("n", [0, 1, 4095, 4097, 1_000_003, 16_777_216])
def test_pack_counts_static_matches_workspace_version(built_lib, n):
    from supernormal_gb300._lib import call

    g = torch.Generator(device="cuda").manual_seed(n + 1)
    counts = torch.randint(0, 40, (n,), dtype=torch.int32, device="cuda", generator=g)
    ws = torch.empty(max(int(call("sn_scan_workspace_bytes", n)), 16), dtype=torch.uint8, device="cuda")
    ref_packed, ref_total = _pack(call, "sn_pack_counts", counts, ws)
    for _ in range(2):          # the static scratch is reused across calls
        packed, total = _pack(call, "sn_pack_counts_static", counts)
        torch.cuda.synchronize()
        assert torch.equal(packed, ref_packed)
        assert torch.equal(total, ref_total)
    if n:
        assert int(total.item()) == int(counts.long().sum().item())


def test_pack_counts_static_rejects_sizes_past_its_limit(built_lib):
    from supernormal_gb300._lib import call, lib, stream_handle

    n = 16_777_216 + 1
    with pytest.raises(RuntimeError, match="static scratch limit"):
        call("sn_pack_counts_static", n, None, None, None, stream_handle())
    assert b"16777216" in lib().sn_last_error()
