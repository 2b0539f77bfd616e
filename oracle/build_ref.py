"""ORACLE (test infrastructure only): build the reference's own CUDA kernels as a checker.

Compiles nerfacc 0.3.5's ``ray_marching.cu``, ``render_weight.cu`` and ``contraction.cu`` from the
read-only SuperNormal tree (third_parties/nerfacc-0.3.5/nerfacc-0.3.5/nerfacc/cuda/csrc)
to sm_103a cubins in ``oracle/_ref/``, and records the exported kernel symbol
names (read with ``nm`` from host objects of the same sources) in
``oracle/_ref/manifest.json``.  Nothing is copied from the reference tree:
the compiler reads the sources where they lie.  The cubins are loaded with the
CUDA driver API by oracle/refkernels.py to compare our kernels with the
reference ones on the GPU.  Needs the reference tree, so it runs only where
that tree is mounted; elsewhere the prebuilt files are used as they are.
"""
from __future__ import annotations

import json
import os
import subprocess
import sys
import sysconfig
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
# the SuperNormal tree: $SUPERNORMAL_REFERENCE, else a "reference" directory beside the repository
REF_ROOT = Path(os.environ.get("SUPERNORMAL_REFERENCE", HERE.parent.parent / "reference"))
CSRC = REF_ROOT / "third_parties" / "nerfacc-0.3.5" / "nerfacc-0.3.5" / "nerfacc" / "cuda" / "csrc"
SOURCES = ["ray_marching.cu", "render_weight.cu", "contraction.cu"]
KERNELS = {
    "ray_marching.cu": ["ray_marching_kernel"],
    "render_weight.cu": ["weight_from_alpha_patch_based_forward_kernel",
                         "weight_from_alpha_patch_based_backward_kernel"],
    "contraction.cu": ["contract_inv_kernel"],
}


def _includes() -> list[str]:
    import torch.utils.cpp_extension as ce

    inc = []
    for p in ce.include_paths():
        inc += ["-I", p]
    inc += ["-I", sysconfig.get_paths()["include"]]
    return inc


FLAGS = ["-std=c++17", "-O3", "-D__CUDA_NO_HALF_OPERATORS__", "-D__CUDA_NO_HALF_CONVERSIONS__",
         "-D__CUDA_NO_BFLOAT16_CONVERSIONS__", "-D__CUDA_NO_HALF2_OPERATORS__",
         "-DTORCH_EXTENSION_NAME=nerfacc_ref", "-diag-suppress", "177,550"]


def available() -> bool:
    return all((CSRC / s).exists() for s in SOURCES)


def build(force: bool = False) -> bool:
    """Build the cubins + manifest; returns False when the reference tree is absent."""
    if not available():
        return False
    OUT.mkdir(exist_ok=True)
    manifest_path = OUT / "manifest.json"
    if manifest_path.exists() and not force and all((OUT / (Path(s).stem + ".cubin")).exists()
                                                    for s in SOURCES):
        return True
    nvcc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    inc = _includes()
    manifest = {"arch": "sm_103a", "kernels": {}}
    procs = []
    for s in SOURCES:
        stem = Path(s).stem
        cubin = OUT / f"{stem}.cubin"
        obj = OUT / f"{stem}.host.o"
        procs.append((s, subprocess.Popen(
            [nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-cubin", *FLAGS, *inc,
             str(CSRC / s), "-o", str(cubin)], stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
        procs.append((s, subprocess.Popen(
            [nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-c", "-Xcompiler", "-fPIC", *FLAGS,
             *inc, str(CSRC / s), "-o", str(obj)], stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    for s, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            raise RuntimeError(f"building reference {s} failed:\n{out.decode(errors='replace')}")
    for s in SOURCES:
        stem = Path(s).stem
        obj = OUT / f"{stem}.host.o"
        syms = subprocess.run(["nm", str(obj)], capture_output=True, text=True, check=True).stdout
        names = {}
        for kname in KERNELS[s]:
            hits = [ln.split()[-1] for ln in syms.splitlines()
                    if ln.split() and ln.split()[-1].startswith(f"_Z{len(kname)}{kname}")]
            if not hits:
                raise RuntimeError(f"symbol of {kname} not found in {obj.name}")
            names[kname] = sorted(set(hits))[0]
        manifest["kernels"][stem] = {"cubin": f"{stem}.cubin", "symbols": names}
        obj.unlink()
    manifest_path.write_text(json.dumps(manifest, indent=1))
    return True


if __name__ == "__main__":
    ok = build(force="--force" in sys.argv)
    print("reference kernels built" if ok else "reference tree not present; nothing built")
