"""ctypes binding of the C ABI declared in include/supernormal_gb300.h.

The library is the product path: there is no CPU or PyTorch fallback.
``lib()`` raises if the shared object is missing (run ``__graft_entry__.build()``
or ``python supernormal_gb300/build.py``), and every call raises
``SupernormalError`` when the C entry point returns a non-zero status.
"""
from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "lib" / "libsngb300.so"

SN_OK = 0
SN_ERR_INVALID = 1
SN_ERR_CAPACITY = 2
SN_ERR_CUDA = 3
SN_ERR_LIMIT = 4
SN_ERR_UNSUPPORTED = 5
SN_STATUS_MARCH_LIMIT = 1
SN_STATUS_CAPACITY = 2
SN_STATUS_TIMEOUT = 4
SN_FIELD_TABLE_FP16 = 1
SN_FIELD_MLP_TF32 = 2
SN_FIELD_MLP_BF16 = 4
SN_MAX_LEVELS = 32


class SupernormalError(RuntimeError):
    def __init__(self, fn: str, status: int, msg: str):
        super().__init__(f"{fn} failed (status {status}): {msg}")
        self.status = status


class GridDesc(C.Structure):
    _fields_ = [
        ("n_levels", C.c_int32),
        ("n_features", C.c_int32),
        ("offsets", C.c_uint32 * (SN_MAX_LEVELS + 1)),
        ("resolutions", C.c_uint32 * SN_MAX_LEVELS),
        ("scales", C.c_float * SN_MAX_LEVELS),
    ]


class MlpDesc(C.Structure):
    _fields_ = [
        ("d_in", C.c_int32),
        ("d_hidden", C.c_int32),
        ("d_out", C.c_int32),
        ("beta", C.c_float),
        ("threshold", C.c_float),
        ("w0", C.c_void_p),
        ("b0", C.c_void_p),
        ("w1", C.c_void_p),
        ("b1", C.c_void_p),
        ("status", C.c_void_p),
        ("flags", C.c_uint32),
        ("enc_cache", C.c_void_p),
    ]


SN_SCENE_MAX_PRIMS = 4
SN_PRIM_SPHERE, SN_PRIM_TORUS, SN_PRIM_BOX = 0, 1, 2


class Prim(C.Structure):
    _fields_ = [("kind", C.c_int32), ("reserved", C.c_int32), ("center", C.c_double * 3),
                ("size", C.c_double * 3), ("amp", C.c_double), ("freq", C.c_double)]


class SceneDesc(C.Structure):
    _fields_ = [("n_prims", C.c_int32), ("reserved", C.c_int32), ("prims", Prim * SN_SCENE_MAX_PRIMS),
                ("disp_amp", C.c_double), ("disp_freq", C.c_double), ("lipschitz", C.c_double)]


SN_FIELD_MAX_SEGMENTS = 4


class FieldSegment(C.Structure):
    _fields_ = [("n", C.c_int64), ("x", C.c_void_p), ("table", C.c_void_p), ("grid", C.POINTER(GridDesc)),
                ("active_levels", C.c_int32), ("mlp", C.POINTER(MlpDesc)), ("out", C.c_void_p)]


_P, _I64, _I, _F, _SZ = C.c_void_p, C.c_int64, C.c_int, C.c_float, C.c_size_t
_GD, _MD, _SD = C.POINTER(GridDesc), C.POINTER(MlpDesc), C.POINTER(SceneDesc)

# name -> (restype, argtypes); mirrors include/supernormal_gb300.h
SIGNATURES: dict[str, tuple] = {
    "sn_version": (C.c_char_p, []),
    "sn_last_error": (C.c_char_p, []),
    "sn_kernel_launches": (C.c_uint64, []),
    "sn_scan_workspace_bytes": (_SZ, [_I64]),
    "sn_pack_counts": (_I, [_I64, _P, _P, _P, _P, _P]),
    "sn_pack_counts_static": (_I, [_I64, _P, _P, _P, _P]),
    "sn_pack_counts_n": (_I, [_I64, _P, _P, _P, _P, _P, _P]),
    "sn_count_indices": (_I, [_I64, _P, _I64, _P, _P]),
    "sn_unpack_info": (_I, [_I64, _P, _I64, _P, _P]),
    "sn_march_count": (_I, [_I64, _P, _P, _P, _P, _P, _P, _P, _I, _I, _I, _I, _F, _F, _I64, _P, _P, _P]),
    "sn_march_fill": (_I, [_I64, _P, _P, _P, _P, _P, _P, _P, _I, _I, _I, _I, _F, _F, _I64, _P, _I64,
                           _P, _P, _P, _P, _P]),
    "sn_march_padded": (_I, [_I64, _P, _P, _P, _P, _P, _P, _P, _I, _I, _I, _I, _F, _P, _F, _I64, _I64,
                             _P, _P, _P, _P, _P, _P]),
    "sn_compact_padded": (_I, [_I64, _I64, _P, _P, _P, _P, _P, _P, _P, _P]),
    "sn_grid_query": (_I, [_I64, _P, _P, _P, _I, _I, _I, _I, _P, _P]),
    "sn_occ_points": (_I, [_I64, _P, _P, _I, _I, _I, _P, _I, _P, _P]),
    "sn_occ_ema_update": (_I, [_I64, _P, _P, _F, _P, _P, _P]),
    "sn_occ_binarize_workspace_bytes": (_SZ, [_I64]),
    "sn_occ_binarize": (_I, [_I64, _P, _F, _P, _P, _P, _P]),
    "sn_occ_points_n": (_I, [_I64, _P, _P, C.c_uint64, _P, _I, _I, _I, _P, _I, _P, _P]),
    "sn_occ_ema_sdf": (_I, [_I64, _P, _P, _P, _F, _F, _P, _P, _P]),
    "sn_occ_sample_workspace_bytes": (_SZ, [_I64]),
    "sn_occ_sample_cells": (_I, [_I64, _P, _I64, C.c_uint64, _P, _P, _P, _P, _P]),
    "sn_near_far_sphere": (_I, [_I64, _P, _P, _I64, _P, _P, _P, C.c_uint64, _P, _P, _P, _P]),
    "sn_transmittance_from_alpha": (_I, [_I64, _I, _P, _P, _P, _P]),
    "sn_visibility_from_alpha": (_I, [_I64, _P, _P, _F, _F, _P, _P, _P]),
    "sn_weight_from_alpha_fwd": (_I, [_I64, _I, _P, _P, _P, _P]),
    "sn_weight_from_alpha_bwd": (_I, [_I64, _I, _P, _P, _P, _P, _P, _P]),
    "sn_accumulate_fwd": (_I, [_I64, _I, _I, _P, _P, _P, _I64, _P, _P]),
    "sn_accumulate_bwd": (_I, [_I64, _I, _I, _P, _P, _P, _P, _P, _P, _P]),
    "sn_grid_desc_init": (_I, [_GD, _I, _I, _I, _I, _F]),
    "sn_hashgrid_fwd": (_I, [_I64, _P, _P, _GD, _I, _P, _P]),
    "sn_hashgrid_bwd": (_I, [_I64, _P, _P, _GD, _I, _P, _P]),
    "sn_field_fwd": (_I, [_I64, _P, _P, _P, _GD, _I, _MD, _I, _P, _P]),
    "sn_field_fwd_batch": (_I, [_I, C.POINTER(FieldSegment), _I, _P]),
    "sn_field_bwd": (_I, [_I64, _P, _P, _P, _I, _P, _GD, _I, _MD, _P, _P, _P, _P, _P, _P, _P]),
    "sn_field_grad_fwd": (_I, [_I64, _P, _P, _P, _GD, _I, _MD, _P, _P, _P]),
    "sn_field_grad_bwd": (_I, [_I64, _P, _P, _P, _P, _P, _GD, _I, _MD, _P, _P, _P, _P, _P, _P]),
    "sn_selftest_bounded_wait": (_I, [C.c_uint32, _P, _P]),
    "sn_bounded_wait_polls": (C.c_uint32, []),
    "sn_weightnorm_fwd": (_I, [_I, _I, _P, _P, _P, _P, _P]),
    "sn_weightnorm_bwd": (_I, [_I, _I, _P, _P, _P, _P, _P, _P, _P]),
    "sn_end_diff": (_I, [_I64, _P, _P, _P, _P, _P]),
    "sn_center_points": (_I, [_I64, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P]),
    "sn_center_alpha": (_I, [_I64, _P, _P, _I, _P, _P, _P, _P]),
    "sn_compact_samples": (_I, [_I64, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P]),
    "sn_patch_points": (_I, [_I64, _P, _I, _I, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P]),
    "sn_patch_render_fwd": (_I, [_I64, _I, _I, _P, _P, _I64, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P,
                                 _P, _P, _P, _P, _P]),
    "sn_patch_render_bwd": (_I, [_I64, _I, _I, _P, _P, _I64, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P,
                                 _P, _P, _P, _P, _P, _P, _P]),
    "sn_patch_render_train": (_I, [_I64, _I, _I, _P, _P, _I64, _P, _P, _P, _P, _P, _P, _P, _P, _P,
                                   _P, _P, _I, _F, _F, _F, _P, _P, _P, _P, _P, _P]),
    "sn_patch_carry_fixup": (_I, [_I64, _I, _P, _P, _I64, _P, _P, _P, _P]),
    "sn_patch_finalize": (_I, [_I64, _I, _P, _P, _I64, _P, _P, _F, _F, _F, _P, _P, _P]),
    "sn_scale_count": (_I, [_P, C.c_int32, C.c_int32, _P, _P]),
    "sn_gen_patches": (_I, [_I64, _I, _I, _P, _P, _P, _I, _I, _I, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P]),
    "sn_mask_prep": (_I, [_I64, _P, _P, _P, _P]),
    "sn_scene_render_gt": (_I, [_SD, _I, _I, _I, _P, _P, _I, C.c_double, _P, _P, _P]),
    "sn_scene_sdf": (_I, [_SD, _I64, _P, _P, _P]),
    "sn_lattice_points": (_I, [_I64, _I64, _I, _I, _I, _P, _P, _P, _P]),
    "sn_negate": (_I, [_I64, _P, _P, _P]),
    "sn_marching_cubes_workspace_bytes": (_SZ, [_I, _I, _I]),
    "sn_marching_cubes": (_I, [_P, _I, _I, _I, _F, _P, _P, _I64, _I64, _P, _P, _P, _P, _P]),
    "sn_lr_schedule": (_I, [_P, _P, _P, _F, _I, _I, _F, _P]),
    "sn_step_size_schedule": (_I, [_P, C.c_double, C.c_double, _I, _P, _P]),
    "sn_adam_step": (_I, [_I64, _P, _P, _P, _P, _P, _P, _P, _F, _I, _F, _F, _F, _I, _P]),
}

_lock = threading.Lock()
_lib = None


def lib_path() -> Path:
    return LIB_PATH


def lib():
    """Load (once) and return the ctypes library with typed entry points."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not LIB_PATH.exists():
            raise RuntimeError(
                f"supernormal_gb300 CUDA library not built ({LIB_PATH} missing); "
                "run `python -c 'import __graft_entry__ as g; g.build()'`")
        L = C.CDLL(str(LIB_PATH))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
        return _lib


def last_error() -> str:
    return (lib().sn_last_error() or b"").decode(errors="replace")


def ptr(x) -> int | None:
    """Device (or host) address of a tensor, None for None, ints pass through."""
    if x is None:
        return None
    if isinstance(x, int):
        return x
    return x.data_ptr()


def call(name: str, *args) -> int:
    """Call an entry point; tensors become pointers; raise on a failing status."""
    fn = getattr(lib(), name)
    conv = []
    for a, t in zip(args, fn.argtypes):
        if t is C.c_void_p:
            conv.append(ptr(a))
        else:
            conv.append(a)
    if len(conv) != len(fn.argtypes):
        raise TypeError(f"{name} takes {len(fn.argtypes)} arguments, got {len(args)}")
    st = fn(*conv)
    if fn.restype is C.c_int and st != SN_OK:
        raise SupernormalError(name, st, last_error())
    return st


def stream_handle(stream=None) -> int:
    import torch

    s = stream if stream is not None else torch.cuda.current_stream()
    return s.cuda_stream
