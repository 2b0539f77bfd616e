"""supernormal_gb300: SuperNormal's training hot path as sm_103a CUDA kernels.

Modules:
  nerfacc   — nerfacc-compatible marching / grid / rendering operators
  fields    — SDFNetwork / SingleVarianceNetwork on the fused hash-grid field
  renderer  — patch-based NeuSRenderer (drop-in for models/renderer.py)
  trainer   — fused, host-sync-free training step (Runner.train iteration)
  scenes    — analytic synthetic scenes with ground-truth normals and masks
  build     — in-tree nvcc build of the CUDA library
"""
__version__ = "0.1.0"


def lib_version() -> str:
    from ._lib import lib

    return lib().sn_version().decode()
