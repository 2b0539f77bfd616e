// NeuS device helpers shared by the culling and the patch-render kernels.
#pragma once

#include "common.cuh"

namespace sn {

// SingleVarianceNetwork: inv_s = exp(variance * 10), clipped to [1e-6, 1e6]
// (models/fields.py:133-139, models/renderer.py:171).
__device__ __forceinline__ float inv_s_from(const float* variance) {
  const float v = expf(__fmul_rn(*variance, 10.0f));
  return fminf(fmaxf(v, 1e-6f), 1e6f);
}

// alpha = clip((sigmoid(s0*inv_s) - sigmoid(s1*inv_s) + 1e-5) / (sigmoid(s0*inv_s) + 1e-5), 0, 1)
// (models/renderer.py:171-179), optionally returning the two cdfs and the
// unclipped ratio for the adjoint.
__device__ __forceinline__ float neus_alpha(float s0, float s1, float inv_s, float* c_out,
                                            float* n_out, float* q_out) {
  const float c = sigmoidf_(__fmul_rn(s0, inv_s));
  const float nn = sigmoidf_(__fmul_rn(s1, inv_s));
  const float p = __fsub_rn(c, nn);
  const float q = __fdiv_rn(__fadd_rn(p, 1e-5f), __fadd_rn(c, 1e-5f));
  if (c_out) *c_out = c;
  if (n_out) *n_out = nn;
  if (q_out) *q_out = q;
  return fminf(fmaxf(q, 0.0f), 1.0f);
}

}  // namespace sn
