"""ORACLE (test infrastructure only): launch the reference's own CUDA kernels
(oracle/_ref cubins) on the GPU, as the checker in tests/ and as the timed
reference-kernel baseline of bench.py.

The cubins are nerfacc 0.3.5's ray_marching.cu / render_weight.cu / contraction.cu compiled
from source for sm_103a by oracle/build_ref.py.  They are loaded with the
CUDA driver API into the current (torch) context and launched with the
reference's own launch shapes (ray_marching.cu:227-228,
render_weight.cu:519-527).
"""
from __future__ import annotations

import ctypes as C
import json
import math
from pathlib import Path

import torch

REF = Path(__file__).resolve().parent / "_ref"


class Int3(C.Structure):
    _fields_ = [("x", C.c_int), ("y", C.c_int), ("z", C.c_int)]


class RefKernels:
    def __init__(self):
        man = REF / "manifest.json"
        if not man.exists():
            raise FileNotFoundError("reference checker kernels not built (oracle/build_ref.py)")
        self.manifest = json.loads(man.read_text())
        self.cu = C.CDLL("libcuda.so.1")
        torch.zeros(1, device="cuda")  # make torch's primary context current
        self.funcs = {}
        for stem, info in self.manifest["kernels"].items():
            mod = C.c_void_p()
            self._chk(self.cu.cuModuleLoad(C.byref(mod), str(REF / info["cubin"]).encode()),
                      "cuModuleLoad")
            for kname, sym in info["symbols"].items():
                f = C.c_void_p()
                self._chk(self.cu.cuModuleGetFunction(C.byref(f), mod, sym.encode()),
                          f"cuModuleGetFunction({kname})")
                self.funcs[kname] = f

    @staticmethod
    def _chk(rc, what):
        if rc != 0:
            raise RuntimeError(f"{what} failed with CUresult {rc}")

    def _launch(self, name, grid, block, args):
        arr = (C.c_void_p * len(args))(*[C.cast(C.pointer(a), C.c_void_p) for a in args])
        st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
        self._chk(self.cu.cuLaunchKernel(self.funcs[name], C.c_uint(grid[0]), C.c_uint(grid[1]),
                                         C.c_uint(grid[2]), C.c_uint(block[0]), C.c_uint(block[1]),
                                         C.c_uint(block[2]), C.c_uint(0), st, arr, None),
                  f"cuLaunchKernel({name})")

    def ray_marching(self, rays_o, rays_d, t_min, t_max, roi, grid_binary, step_size, cone_angle=0.0):
        """Both rounds of ray_marching_kernel with the reference host logic
        (NA/nerfacc/cuda/csrc/ray_marching.cu:194-289)."""
        n = rays_o.shape[0]
        dev = rays_o.device
        rx, ry, rz = grid_binary.shape
        num_steps = torch.empty(n, dtype=torch.int32, device=dev)
        vp = lambda t: C.c_void_p(t.data_ptr() if t is not None else 0)
        common = [C.c_uint32(n), vp(rays_o), vp(rays_d), vp(t_min), vp(t_max), vp(roi),
                  Int3(rx, ry, rz), vp(grid_binary), C.c_int(0), C.c_float(step_size),
                  C.c_float(cone_angle)]
        blocks = (n - 1) // 256 + 1
        self._launch("ray_marching_kernel", (blocks, 1, 1), (256, 1, 1),
                     common + [C.c_void_p(0), vp(num_steps), C.c_void_p(0), C.c_void_p(0), C.c_void_p(0)])
        cum = num_steps.cumsum(0, dtype=torch.int32)
        packed = torch.stack([cum - num_steps, num_steps], 1).contiguous()
        total = int(cum[-1].item()) if n else 0
        ts = torch.empty((total, 1), device=dev)
        te = torch.empty((total, 1), device=dev)
        ri = torch.empty((total,), dtype=torch.int64, device=dev)
        self._launch("ray_marching_kernel", (blocks, 1, 1), (256, 1, 1),
                     common + [vp(packed), C.c_void_p(0), vp(ri), vp(ts), vp(te)])
        return packed, ri, ts, te

    def _patch_shape(self, n_patches, P):
        ty = 2 ** math.ceil(math.log2(P))
        tx = 256 // ty
        return ((n_patches + tx - 1) // tx, (P + ty - 1) // ty, 1), (tx, ty, 1)

    def patch_weight_fwd(self, packed, alphas):
        n_patches, P = packed.shape[0], alphas.shape[1]
        w = torch.empty_like(alphas)
        g, b = self._patch_shape(n_patches, P)
        vp = lambda t: C.c_void_p(t.data_ptr())
        self._launch("weight_from_alpha_patch_based_forward_kernel", g, b,
                     [C.c_uint32(n_patches), C.c_uint32(P), vp(packed), vp(alphas), vp(w)])
        return w

    def patch_weight_bwd(self, packed, alphas, weights, grad_weights):
        n_patches, P = packed.shape[0], alphas.shape[1]
        ga = torch.empty_like(alphas)
        g, b = self._patch_shape(n_patches, P)
        vp = lambda t: C.c_void_p(t.data_ptr())
        self._launch("weight_from_alpha_patch_based_backward_kernel", g, b,
                     [C.c_uint32(n_patches), C.c_uint32(P), vp(packed), vp(alphas), vp(weights),
                      vp(grad_weights), vp(ga)])
        return ga

    def contract_inv(self, x_unit, roi, ctype=0):
        """contract_inv_kernel (NA/nerfacc/cuda/csrc/contraction.cu:36-61,89-113)."""
        n = x_unit.shape[0]
        out = torch.empty_like(x_unit)
        vp = lambda t: C.c_void_p(t.data_ptr())
        self._launch("contract_inv_kernel", ((n + 255) // 256, 1, 1), (256, 1, 1),
                     [C.c_uint32(n), vp(x_unit), vp(roi), C.c_int(ctype), vp(out)])
        return out


def load():
    try:
        return RefKernels()
    except (FileNotFoundError, OSError) as e:
        return e
