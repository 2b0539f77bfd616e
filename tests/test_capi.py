"""C ABI: the library loads, exports every symbol the header declares, and the
Python binding agrees with the header's parameter lists.  No compute calls."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
HEADER = ROOT / "include" / "supernormal_gb300.h"


def _declarations():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    decls = {}
    for m in re.finditer(r"(?:^|\n)\s*(?:const\s+)?(?:int|size_t|uint32_t|uint64_t|char\s*\*)\s*\*?\s*(sn_\w+)\s*\(([^;]*?)\)\s*;",
                         text):
        name, params = m.group(1), m.group(2).strip()
        n = 0 if params in ("", "void") else len([p for p in params.split(",") if p.strip()])
        decls[name] = n
    return decls


def test_header_parses():
    d = _declarations()
    assert len(d) >= 40
    assert "sn_march_count" in d and "sn_field_bwd" in d


def test_every_declared_symbol_is_exported(built_lib):
    for name in _declarations():
        assert hasattr(built_lib, name), f"{name} declared in the header but not exported"


def test_binding_matches_header():
    from supernormal_gb300._lib import SIGNATURES

    d = _declarations()
    assert set(d) == set(SIGNATURES), set(d) ^ set(SIGNATURES)
    for name, n in d.items():
        assert len(SIGNATURES[name][1]) == n, f"{name}: header has {n} params, binding {len(SIGNATURES[name][1])}"


def test_version_and_error_string(built_lib):
    from supernormal_gb300 import _lib

    assert b"sm_103a" in built_lib.sn_version()
    # argument validation happens on the host before any CUDA call
    with pytest.raises(_lib.SupernormalError) as ei:
        _lib.call("sn_march_count", 4, None, None, None, None, None, None, None, 8, 8, 8, 0,
                  0.0, 0.0, 0, None, None, None)
    assert "step_size" in str(ei.value)
    assert ei.value.status == _lib.SN_ERR_INVALID


def test_grid_desc_matches_oracle_geometry(built_lib):
    from oracle.field import grid_geometry
    from supernormal_gb300.fields import grid_desc

    for cfg in [(16, 2, 15, 16, 1.447), (16, 2, 19, 16, 1.447), (14, 2, 19, 32, 1.3195079107728942)]:
        d = grid_desc(*cfg)
        offs, res, scales = grid_geometry(*cfg)
        L = cfg[0]
        assert list(d.offsets[: L + 1]) == offs.tolist()
        assert list(d.resolutions[:L]) == res.tolist()
        np.testing.assert_array_equal(np.array(d.scales[:L], dtype=np.float32), scales)


def test_unsupported_field_shape_is_rejected(built_lib):
    from supernormal_gb300 import _lib
    from supernormal_gb300.fields import grid_desc

    d = grid_desc(16, 4, 15, 16, 1.447)  # 4 features per level: not covered
    m = _lib.MlpDesc(3 + 64, 64, 1, 100.0, 20.0, 1, 1, 1, 1)
    with pytest.raises(_lib.SupernormalError):
        _lib.call("sn_field_fwd", 8, None, 1, 1, C.byref(d), 16, C.byref(m), 1, 1, None)
