"""ORACLE — test infrastructure, not part of the product.

CPU restatements of the reference algorithms on SuperNormal's training hot
path, used only by tests/, ``__graft_entry__.smoke()`` and bench.py's CPU
baseline leg as the checker:

* ``oracle.march``       — C restatement of nerfacc's marcher (bit-exact float32)
* ``oracle.nerfacc_ref`` — numpy restatements of packing, transmittance,
  visibility, (patch) weights and their adjoint, accumulation
* ``oracle.field``       — float64 torch restatement of the hash-grid encoding
  (Instant-NGP / tiny-cuda-nn conventions) and SDFNetwork's MLP
* ``oracle.renderer``    — float64 torch restatement of NeuSRenderer.render's
  patch math and the training losses (models/renderer.py, exp_runner.py)

Parity status: the nerfacc pieces are pinned by the golden vectors of
nerfacc's own tests (NA/tests/test_rendering.py, test_pack.py) and, on the
GPU, by the reference's own kernels built from source (oracle/build_ref.py);
the renderer / field math is pinned by fixtures generated by running the
reference Python (models/renderer.py, models/fields.py) with tiny-cuda-nn
replaced by ``oracle.field``'s encoding (tests/golden/make_golden.py).  The
hash-grid encoding itself is pinned only against its published algorithm:
tiny-cuda-nn (commit 2ec562e853e6f482b5d09168705205f46358fb39) is not
available here.
"""
