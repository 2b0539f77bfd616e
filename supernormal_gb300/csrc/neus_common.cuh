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

// Double-float (hi + lo) arithmetic for the transmittance product and the
// adjoint's suffix sums over long rays.
// sum_{i >= j} g_i w_i is formed as total - prefix, which in float32 loses
// everything below eps * |total| exactly where the suffix is small (behind the
// surface); carrying the rounding errors (Knuth's TwoSum) keeps it to
// ~eps * |suffix|.  Explicit rounding intrinsics: no contraction, no
// reassociation.
struct ff {
  float hi, lo;
};
__device__ __forceinline__ ff two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bp = __fsub_rn(s, a);
  const float ap = __fsub_rn(s, bp);
  return ff{s, __fadd_rn(__fsub_rn(a, ap), __fsub_rn(b, bp))};
}
__device__ __forceinline__ ff ff_add(ff x, ff y) {
  const ff s = two_sum(x.hi, y.hi);
  const float e = __fadd_rn(s.lo, __fadd_rn(x.lo, y.lo));
  const float h = __fadd_rn(s.hi, e);
  return ff{h, __fsub_rn(e, __fsub_rn(h, s.hi))};
}
__device__ __forceinline__ ff ff_add_f(ff x, float y) { return ff_add(x, ff{y, 0.0f}); }
__device__ __forceinline__ ff ff_neg(ff x) { return ff{-x.hi, -x.lo}; }
__device__ __forceinline__ float ff_val(ff x) { return __fadd_rn(x.hi, x.lo); }
// a * b exactly as a double-float (one FMA for the rounding error).
__device__ __forceinline__ ff two_prod(float a, float b) {
  const float p = __fmul_rn(a, b);
  return ff{p, __fmaf_rn(a, b, -p)};
}
// (x.hi + x.lo)(y.hi + y.lo) to double-float precision (the lo * lo term dropped).
__device__ __forceinline__ ff ff_mul(ff x, ff y) {
  const ff p = two_prod(x.hi, y.hi);
  const float e = __fmaf_rn(x.hi, y.lo, __fmaf_rn(x.lo, y.hi, p.lo));
  const float h = __fadd_rn(p.hi, e);
  return ff{h, __fsub_rn(e, __fsub_rn(h, p.hi))};
}
__device__ __forceinline__ ff shfl_ff(ff v, int src) {
  return ff{__shfl_sync(0xffffffffu, v.hi, src), __shfl_sync(0xffffffffu, v.lo, src)};
}
__device__ __forceinline__ ff shfl_up_ff(ff v, int d) {
  return ff{__shfl_up_sync(0xffffffffu, v.hi, d), __shfl_up_sync(0xffffffffu, v.lo, d)};
}
__device__ __forceinline__ ff warp_sum_ff(ff v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
    v = ff_add(v, ff{__shfl_xor_sync(0xffffffffu, v.hi, o), __shfl_xor_sync(0xffffffffu, v.lo, o)});
  return v;
}

}  // namespace sn
