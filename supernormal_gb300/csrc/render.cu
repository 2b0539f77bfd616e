// Volume-rendering primitives behind nerfacc's weight / visibility /
// accumulation ops, for per-ray (patch_size = 1) and patch-based samples.
//
// Sample layout follows the reference: a ray (or patch) owns the contiguous
// samples [base, base+steps) of packed_info, and each sample carries
// patch_size pixel lanes stored as alphas[(base+j)*patch_size + k]
// (NA/nerfacc/cuda/csrc/render_weight.cu:87-118).  One thread walks one
// (ray, lane) sequence front to back, so products and sums are formed in the
// reference's order; the backward pass writes the reference's contractions
// (fma) explicitly so results match its kernels bit for bit.
#include "common.cuh"

namespace sn {

__global__ void weight_fwd_kernel(int64_t n_rays, int P, const int32_t* __restrict__ packed,
                                  const float* __restrict__ alphas, float* __restrict__ weights,
                                  float* __restrict__ trans) {
  const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (tid >= n_rays * P) return;
  const int64_t r = tid / P;
  const int k = (int)(tid - r * P);
  const int64_t base = packed[2 * r];
  const int steps = packed[2 * r + 1];
  const float* a = alphas + base * P + k;
  float T = 1.0f;
  for (int j = 0; j < steps; ++j) {
    const float al = a[(int64_t)j * P];
    if (trans) trans[(base + j) * P + k] = T;
    if (weights) weights[(base + j) * P + k] = __fmul_rn(al, T);
    T = __fmul_rn(T, __fsub_rn(1.0f, al));
  }
}

__global__ void weight_bwd_kernel(int64_t n_rays, int P, const int32_t* __restrict__ packed,
                                  const float* __restrict__ alphas, const float* __restrict__ weights,
                                  const float* __restrict__ gw, float* __restrict__ ga) {
  const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (tid >= n_rays * P) return;
  const int64_t r = tid / P;
  const int k = (int)(tid - r * P);
  const int64_t base = packed[2 * r];
  const int steps = packed[2 * r + 1];
  const int64_t o = base * P + k;
  // reference: accum += g*w (contracted to fma by nvcc)
  float accum = 0.0f;
  for (int j = 0; j < steps; ++j) {
    const int64_t s = o + (int64_t)j * P;
    accum = __fmaf_rn(gw[s], weights[s], accum);
  }
  float T = 1.0f;
  for (int j = 0; j < steps; ++j) {
    const int64_t s = o + (int64_t)j * P;
    const float al = alphas[s], g = gw[s];
    // (g*T - accum) / fmaxf(1 - alpha, 1e-10)  with g*T - accum -> fma(g, T, -accum)
    ga[s] = __fdiv_rn(__fmaf_rn(g, T, -accum), fmaxf(__fsub_rn(1.0f, al), 1e-10f));
    accum = __fmaf_rn(-g, weights[s], accum);
    T = __fmul_rn(T, __fsub_rn(1.0f, al));
  }
}

// One warp per ray: transmittance before each sample as a warp product scan of
// (1 - alpha) with a carry between 32-sample chunks (the reference's CUB
// scan is tree-ordered as well); visible = T >= eps (and alpha >= thre).
__global__ void __launch_bounds__(256) visibility_kernel(int64_t n_rays, const int32_t* __restrict__ packed,
                                                         const float* __restrict__ alphas, float eps,
                                                         float thre, uint8_t* __restrict__ vis,
                                                         int32_t* __restrict__ counts) {
  const int64_t r = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (r >= n_rays) return;  // whole warp
  const int64_t base = packed[2 * r];
  const int steps = packed[2 * r + 1];
  float carry = 1.0f;
  int c = 0;
  for (int j0 = 0; j0 < steps; j0 += 32) {
    const int j = j0 + lane;
    const bool ok = j < steps;
    const float al = ok ? alphas[base + j] : 0.0f;
    float incl = ok ? __fsub_rn(1.0f, al) : 1.0f;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const float y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl = __fmul_rn(y, incl);
    }
    float excl = __shfl_up_sync(0xffffffffu, incl, 1);
    if (lane == 0) excl = 1.0f;
    const float T = __fmul_rn(carry, excl);
    carry = __fmul_rn(carry, __shfl_sync(0xffffffffu, incl, 31));
    bool v = ok && T >= eps;
    if (thre > 0.0f) v = v && (al >= thre);
    if (ok) vis[base + j] = v ? 1 : 0;
    c += __popc(__ballot_sync(0xffffffffu, v));
  }
  if (counts && lane == 0) counts[r] = c;
}

// out[idx[s], k, d] += w[s,k] * v[s,k,d]
__global__ void accumulate_fwd_kernel(int64_t n, int P, int D, const int64_t* __restrict__ idx,
                                      const float* __restrict__ w, const float* __restrict__ v,
                                      int64_t n_rays, float* __restrict__ out) {
  const int64_t total = n * P;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t s = t / P;
    const int k = (int)(t - s * P);
    const int64_t r = idx[s];
    if (r < 0 || r >= n_rays) continue;
    const float ww = w[t];
    float* o = out + (r * P + k) * D;
    if (v) {
      const float* vv = v + t * D;
      for (int d = 0; d < D; ++d) atomicAdd(o + d, __fmul_rn(ww, vv[d]));
    } else {
      atomicAdd(o, ww);
    }
  }
}

__global__ void accumulate_bwd_kernel(int64_t n, int P, int D, const int64_t* __restrict__ idx,
                                      const float* __restrict__ w, const float* __restrict__ v,
                                      const float* __restrict__ g, float* __restrict__ gw,
                                      float* __restrict__ gv) {
  const int64_t total = n * P;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t s = t / P;
    const int k = (int)(t - s * P);
    const int64_t r = idx[s];
    const float* go = g + (r * P + k) * D;
    if (v) {
      const float* vv = v + t * D;
      float acc = 0.0f;
      for (int d = 0; d < D; ++d) {
        const float gd = go[d];
        acc = __fadd_rn(acc, __fmul_rn(gd, vv[d]));
        if (gv) gv[t * D + d] = __fmul_rn(gd, w[t]);
      }
      if (gw) gw[t] = acc;
    } else {
      if (gw) gw[t] = go[0];
    }
  }
}

}  // namespace sn

using namespace sn;

extern "C" {

int sn_transmittance_from_alpha(int64_t n_rays, int patch_size, const int32_t* packed_info,
                                const float* alphas, float* transmittance, void* stream) {
  SN_REQUIRE(n_rays >= 0 && patch_size >= 1, "transmittance: bad sizes");
  if (n_rays == 0) return SN_OK;
  const int64_t n = n_rays * patch_size;
  weight_fwd_kernel<<<div_up(n, 128), 128, 0, as_stream(stream)>>>(
      n_rays, patch_size, packed_info, alphas, nullptr, transmittance);
  return check_launch("transmittance_from_alpha");
}

int sn_visibility_from_alpha(int64_t n_rays, const int32_t* packed_info, const float* alphas,
                             float early_stop_eps, float alpha_thre, uint8_t* visibility,
                             int32_t* vis_counts, void* stream) {
  SN_REQUIRE(n_rays >= 0, "visibility: n_rays < 0");
  if (n_rays == 0) return SN_OK;
  visibility_kernel<<<div_up(n_rays * 32, 256), 256, 0, as_stream(stream)>>>(
      n_rays, packed_info, alphas, early_stop_eps, alpha_thre, visibility, vis_counts);
  return check_launch("visibility_from_alpha");
}

int sn_weight_from_alpha_fwd(int64_t n_rays, int patch_size, const int32_t* packed_info,
                             const float* alphas, float* weights, void* stream) {
  SN_REQUIRE(n_rays >= 0 && patch_size >= 1, "weight_fwd: bad sizes");
  if (n_rays == 0) return SN_OK;
  const int64_t n = n_rays * patch_size;
  weight_fwd_kernel<<<div_up(n, 128), 128, 0, as_stream(stream)>>>(n_rays, patch_size, packed_info,
                                                                   alphas, weights, nullptr);
  return check_launch("weight_from_alpha_fwd");
}

int sn_weight_from_alpha_bwd(int64_t n_rays, int patch_size, const int32_t* packed_info,
                             const float* alphas, const float* weights, const float* grad_weights,
                             float* grad_alphas, void* stream) {
  SN_REQUIRE(n_rays >= 0 && patch_size >= 1, "weight_bwd: bad sizes");
  if (n_rays == 0) return SN_OK;
  const int64_t n = n_rays * patch_size;
  weight_bwd_kernel<<<div_up(n, 128), 128, 0, as_stream(stream)>>>(
      n_rays, patch_size, packed_info, alphas, weights, grad_weights, grad_alphas);
  return check_launch("weight_from_alpha_bwd");
}

int sn_accumulate_fwd(int64_t n_samples, int patch_size, int dim, const int64_t* ray_indices,
                      const float* weights, const float* values, int64_t n_rays, float* out,
                      void* stream) {
  SN_REQUIRE(n_samples >= 0 && n_rays >= 0 && patch_size >= 1 && dim >= 1, "accumulate: bad sizes");
  SN_REQUIRE(values != nullptr || dim == 1, "accumulate: dim must be 1 without values");
  cudaStream_t st = as_stream(stream);
  if (n_rays > 0 &&
      cudaMemsetAsync(out, 0, (size_t)n_rays * patch_size * dim * sizeof(float), st) != cudaSuccess) {
    set_error("accumulate: memset failed");
    return SN_ERR_CUDA;
  }
  if (n_samples == 0) return SN_OK;
  accumulate_fwd_kernel<<<stride_grid(n_samples * patch_size, 256, 8), 256, 0, st>>>(
      n_samples, patch_size, dim, ray_indices, weights, values, n_rays, out);
  return check_launch("accumulate_fwd");
}

int sn_accumulate_bwd(int64_t n_samples, int patch_size, int dim, const int64_t* ray_indices,
                      const float* weights, const float* values, const float* grad_out,
                      float* grad_weights, float* grad_values, void* stream) {
  SN_REQUIRE(n_samples >= 0 && patch_size >= 1 && dim >= 1, "accumulate_bwd: bad sizes");
  if (n_samples == 0) return SN_OK;
  accumulate_bwd_kernel<<<stride_grid(n_samples * patch_size, 256, 8), 256, 0, as_stream(stream)>>>(
      n_samples, patch_size, dim, ray_indices, weights, values, grad_out, grad_weights, grad_values);
  return check_launch("accumulate_bwd");
}

}  // extern "C"
