// Renderer glue of SuperNormal's patch-based NeuS training step
// (models/renderer.py:63-276) as device kernels:
//   * end-point bookkeeping: diff_mask = t_end != next t_start over the
//     flattened sample list (models/renderer.py:88-93, :151-154) and the
//     slot of every extra end evaluation;
//   * query-point builders for patch-centre samples (alpha_fn,
//     :80-98) and for all pixels of a patch via the marching plane
//     (t_pix = t_c * (d_c . n) / (d_pix . n), :146-159);
//   * NeuS SDF->alpha for the culling pass (:100-117);
//   * compaction of visible samples (NA/nerfacc/ray_marching.py:208-220);
//   * unit-sphere near/far with stratified jitter, mask binarisation.
// The fused per-patch render / loss / adjoint lives in patch.cu.
//
// Field query points are laid out as [S*P start points][E*P end points]:
// start (i, k) at i*P + k and the end of diff sample i at (S + slot_i)*P + k,
// which is the order the reference concatenates positions_all.
#include "neus_common.cuh"

#include <string.h>

namespace sn {

// diff[i] = t_ends[i] != t_starts[i+1] (last sample compares with itself)
// for i < min(*count, cap); entries past the count are not written.
__global__ void end_diff_kernel(int64_t cap, const int32_t* __restrict__ count,
                                const float* __restrict__ ts, const float* __restrict__ te,
                                int32_t* __restrict__ diff) {
  const int64_t n = count ? min((int64_t)*count, cap) : cap;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float nxt = (i + 1 < n) ? ts[i + 1] : ts[i];
    diff[i] = (__fsub_rn(te[i], nxt) != 0.0f) ? 1 : 0;
  }
}

// Centre-ray query points: starts then ends of diff samples.
__global__ void center_points_kernel(int64_t cap, const int32_t* __restrict__ count,
                                     const int64_t* __restrict__ ridx, const float* __restrict__ ts,
                                     const float* __restrict__ te, const float* __restrict__ ro,
                                     const float* __restrict__ rd, const int32_t* __restrict__ endp,
                                     const int32_t* __restrict__ n_ends, float* __restrict__ xyz,
                                     int32_t* __restrict__ q_out) {
  const int64_t n = count ? min((int64_t)*count, cap) : cap;
  if (blockIdx.x == 0 && threadIdx.x == 0 && q_out) q_out[0] = (int32_t)(n + *n_ends);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = ridx[i];
    const int2 ep = reinterpret_cast<const int2*>(endp)[i];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const float o = ro[3 * r + d], dd = rd[3 * r + d];
      xyz[3 * i + d] = __fadd_rn(o, __fmul_rn(dd, ts[i]));
      if (ep.y) xyz[3 * (n + ep.x) + d] = __fadd_rn(o, __fmul_rn(dd, te[i]));
    }
  }
}

// Culling alpha at centre samples: sdf_next = end value if diff, else the next start.
__global__ void center_alpha_kernel(int64_t cap, const int32_t* __restrict__ count,
                                    const float* __restrict__ sdf, int sdf_stride,
                                    const int32_t* __restrict__ endp,
                                    const float* __restrict__ variance,
                                    float* __restrict__ alpha) {
  const int64_t n = count ? min((int64_t)*count, cap) : cap;
  const float inv_s = inv_s_from(variance);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int2 ep = reinterpret_cast<const int2*>(endp)[i];
    const float s0 = sdf[i * sdf_stride];
    const float s1 = ep.y ? sdf[(n + ep.x) * sdf_stride] : (i + 1 < n ? sdf[(i + 1) * sdf_stride] : s0);
    alpha[i] = neus_alpha(s0, s1, inv_s, nullptr, nullptr, nullptr);
  }
}

// Keep visible samples, preserving order: one warp per ray, a ballot per
// 32-sample chunk gives each visible sample its output slot.
__global__ void __launch_bounds__(256) compact_kernel(
    int64_t n_rays, const int32_t* __restrict__ pin, const uint8_t* __restrict__ vis,
    const int32_t* __restrict__ pout, const int64_t* __restrict__ ridx, const float* __restrict__ ts,
    const float* __restrict__ te, int64_t* __restrict__ ridx_o, float* __restrict__ ts_o,
    float* __restrict__ te_o) {
  const int64_t r = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (r >= n_rays) return;  // whole warp
  const int64_t bi = pin[2 * r], bo = pout[2 * r];
  const int steps = pin[2 * r + 1];
  int c = 0;
  for (int j0 = 0; j0 < steps; j0 += 32) {
    const int j = j0 + lane;
    const bool v = j < steps && vis[bi + j];
    const unsigned m = __ballot_sync(0xffffffffu, v);
    if (v) {
      const int64_t o = bo + c + __popc(m & ((1u << lane) - 1u));
      ridx_o[o] = ridx[bi + j];
      ts_o[o] = ts[bi + j];
      te_o[o] = te[bi + j];
    }
    c += __popc(m);
  }
}

// Patch pixel expansion through the marching plane and query points.
__global__ void patch_points_kernel(int64_t cap, const int32_t* __restrict__ count, int P, int kc,
                                    const int64_t* __restrict__ pidx, const float* __restrict__ ts,
                                    const float* __restrict__ te, const float* __restrict__ ro,
                                    const float* __restrict__ rd, const float* __restrict__ pn,
                                    const int32_t* __restrict__ endp,
                                    const int32_t* __restrict__ n_ends, float* __restrict__ xyz,
                                    float* __restrict__ tps, float* __restrict__ tpe,
                                    int32_t* __restrict__ q_out) {
  const int64_t n = count ? min((int64_t)*count, cap) : cap;
  if (blockIdx.x == 0 && threadIdx.x == 0 && q_out) q_out[0] = (int32_t)((n + *n_ends) * P);
  const int64_t total = n * P;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = t / P;
    const int k = (int)(t - i * P);
    const int64_t b = pidx[i];
    const float* nrm = pn + 3 * b;
    const float* dc = rd + (b * P + kc) * 3;
    const float* dp = rd + (b * P + k) * 3;
    const float* op = ro + (b * P + k) * 3;
    float dotc = __fmul_rn(dc[0], nrm[0]);
    dotc = __fadd_rn(dotc, __fmul_rn(dc[1], nrm[1]));
    dotc = __fadd_rn(dotc, __fmul_rn(dc[2], nrm[2]));
    float dotp = __fmul_rn(dp[0], nrm[0]);
    dotp = __fadd_rn(dotp, __fmul_rn(dp[1], nrm[1]));
    dotp = __fadd_rn(dotp, __fmul_rn(dp[2], nrm[2]));
    const float t0 = __fdiv_rn(__fmul_rn(ts[i], dotc), dotp);
    const float t1 = __fdiv_rn(__fmul_rn(te[i], dotc), dotp);
    tps[t] = t0;
    tpe[t] = t1;
    const int2 ep = reinterpret_cast<const int2*>(endp)[i];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      xyz[3 * t + d] = __fadd_rn(op[d], __fmul_rn(dp[d], t0));
      if (ep.y) xyz[3 * ((n + ep.x) * P + k) + d] = __fadd_rn(op[d], __fmul_rn(dp[d], t1));
    }
  }
}

// near/far of the unit-sphere chord for rays read with a stride
// (models/dataset_loader.py:279-297; NaN when the ray misses the sphere, so
// the marcher emits no samples for it), plus optional stratified jitter
// u in [0, 1) from the counter-based generator.
__global__ void near_far_kernel(int64_t n, const float* __restrict__ ro, const float* __restrict__ rd,
                                int64_t stride, float* __restrict__ near, float* __restrict__ far,
                                float* __restrict__ jitter, uint64_t seed,
                                const int32_t* __restrict__ stream_dev, float* __restrict__ o_out,
                                float* __restrict__ d_out) {
  const uint64_t sid = stream_dev ? (uint64_t)(uint32_t)*stream_dev : 0ull;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float* o = ro + i * stride;
    const float* d = rd + i * stride;
    if (o_out) {
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        o_out[3 * i + k] = o[k];
        d_out[3 * i + k] = d[k];
      }
    }
    const float a = __fadd_rn(__fadd_rn(__fmul_rn(d[0], d[0]), __fmul_rn(d[1], d[1])), __fmul_rn(d[2], d[2]));
    const float od = __fadd_rn(__fadd_rn(__fmul_rn(o[0], d[0]), __fmul_rn(o[1], d[1])), __fmul_rn(o[2], d[2]));
    const float b = __fmul_rn(2.0f, od);
    const float oo = __fadd_rn(__fadd_rn(__fmul_rn(o[0], o[0]), __fmul_rn(o[1], o[1])), __fmul_rn(o[2], o[2]));
    const float c = __fsub_rn(oo, 1.0f);
    const float mid = __fdiv_rn(__fmul_rn(0.5f, -b), a);
    const float h = __fdiv_rn(sqrtf(__fsub_rn(__fmul_rn(b, b), __fmul_rn(__fmul_rn(4.0f, a), c))),
                              __fmul_rn(2.0f, a));
    near[i] = __fsub_rn(mid, h);
    far[i] = __fadd_rn(mid, h);
    if (jitter) jitter[i] = uniform01(seed, sid, (uint64_t)i);
  }
}

__global__ void scale_count_kernel(const int32_t* __restrict__ in, int32_t mul, int32_t add,
                                   int32_t* __restrict__ out) {
  *out = *in * mul + add;
}

// mask := (mask > 0.5) as float, out = sum(mask) + 1e-5 (exp_runner.py:169-175).
// One block (no second pass); the sum of 0/1 values is exact in float below
// 2^24 elements, so the block size does not change it.
constexpr int kMaskThreads = 1024;
__global__ void __launch_bounds__(kMaskThreads)
mask_prep_kernel(int64_t n, const float* __restrict__ mask_in, float* __restrict__ mask_out,
                 float* __restrict__ mask_sum) {
  __shared__ float red[kMaskThreads / 32];
  float s = 0.0f;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
    const float m = mask_in[i] > 0.5f ? 1.0f : 0.0f;
    mask_out[i] = m;
    s += m;
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    float t = 0.0f;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
    *mask_sum = t + 1e-5f;
  }
}

// One thread per patch pixel: world ray direction R normalize(K^-1 [x, y, 1]),
// V = rows (d, camera right, camera down) and V^-1 by the adjugate, in double
// and rounded once (models/dataset_loader.py:112-137), plus the ground-truth
// gathers and per-patch origin / plane normal (models/dataset_loader.py:223-277).
__global__ void gen_patches_kernel(int64_t n_patches, int ph, int pw, const int32_t* __restrict__ cx,
                                   const int32_t* __restrict__ cy, const int32_t* __restrict__ img, int H,
                                   int W, const double* __restrict__ kinv, const double* __restrict__ pose,
                                   const float* __restrict__ normals, const float* __restrict__ masks,
                                   float* __restrict__ rays_o, float* __restrict__ rays_d,
                                   float* __restrict__ plane_n, float* __restrict__ vinv,
                                   float* __restrict__ normal_out, float* __restrict__ mask_out) {
  const int P = ph * pw;
  const int64_t n = n_patches * P;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = i / P;
    const int r = (int)(i - b * P), yy = r / pw, xx = r - yy * pw;
    const int v = img[b];
    const int px = cx[b] + xx - pw / 2, py = cy[b] + yy - ph / 2;
    const double* K = kinv + 9 * v;
    const double* T = pose + 12 * v;   // rows of [R | t]
    double q[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) q[k] = K[3 * k] * px + K[3 * k + 1] * py + K[3 * k + 2];
    const double inv_norm = 1.0 / sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2]);
    double rw[3][3];   // rows d, right, down
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      rw[0][k] = (T[4 * k] * q[0] + T[4 * k + 1] * q[1] + T[4 * k + 2] * q[2]) * inv_norm;
      rw[1][k] = T[4 * k];
      rw[2][k] = T[4 * k + 1];
    }
    double c[3][3];    // c[j] = r(j+1) x r(j+2): column j of the adjugate
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const double* a = rw[(j + 1) % 3];
      const double* e = rw[(j + 2) % 3];
      c[j][0] = a[1] * e[2] - a[2] * e[1];
      c[j][1] = a[2] * e[0] - a[0] * e[2];
      c[j][2] = a[0] * e[1] - a[1] * e[0];
    }
    const double det = rw[0][0] * c[0][0] + rw[0][1] * c[0][1] + rw[0][2] * c[0][2];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      rays_d[3 * i + k] = (float)rw[0][k];
      rays_o[3 * i + k] = (float)T[4 * k + 3];
#pragma unroll
      for (int j = 0; j < 3; ++j) vinv[9 * i + 3 * k + j] = (float)(c[j][k] / det);
    }
    const int64_t pix = ((int64_t)v * H + py) * W + px;
    if (normals) {
#pragma unroll
      for (int k = 0; k < 3; ++k) normal_out[3 * i + k] = normals[3 * pix + k];
    }
    if (masks) mask_out[i] = masks[pix];
    if (r == 0) {
#pragma unroll
      for (int k = 0; k < 3; ++k) plane_n[3 * b + k] = (float)T[4 * k + 2];
    }
  }
}

}  // namespace sn

using namespace sn;

extern "C" {

int sn_end_diff(int64_t cap, const int32_t* count, const float* t_starts, const float* t_ends,
                int32_t* diff, void* stream) {
  SN_REQUIRE(cap >= 0, "end_diff: cap < 0");
  if (cap == 0) return SN_OK;
  end_diff_kernel<<<stride_grid(cap, 256, 8), 256, 0, as_stream(stream)>>>(cap, count, t_starts,
                                                                           t_ends, diff);
  return check_launch("end_diff");
}

int sn_center_points(int64_t cap, const int32_t* count, const int64_t* ray_indices,
                     const float* t_starts, const float* t_ends, const float* rays_o,
                     const float* rays_d, const int32_t* end_packed, const int32_t* n_ends,
                     float* xyz, int32_t* n_points, void* stream) {
  SN_REQUIRE(cap >= 0, "center_points: cap < 0");
  if (cap == 0) {  // no samples: no points
    if (n_points && cudaMemsetAsync(n_points, 0, sizeof(int32_t), as_stream(stream)) != cudaSuccess) {
      set_error("center_points: memset failed");
      return SN_ERR_CUDA;
    }
    return SN_OK;
  }
  SN_REQUIRE(n_ends != nullptr && end_packed != nullptr, "center_points: null end info");
  center_points_kernel<<<stride_grid(cap > 0 ? cap : 1, 256, 8), 256, 0, as_stream(stream)>>>(
      cap, count, ray_indices, t_starts, t_ends, rays_o, rays_d, end_packed, n_ends, xyz, n_points);
  return check_launch("center_points");
}

int sn_center_alpha(int64_t cap, const int32_t* count, const float* sdf, int sdf_stride,
                    const int32_t* end_packed, const float* variance, float* alpha, void* stream) {
  SN_REQUIRE(cap >= 0 && sdf_stride >= 1, "center_alpha: bad sizes");
  if (cap == 0) return SN_OK;
  center_alpha_kernel<<<stride_grid(cap, 256, 8), 256, 0, as_stream(stream)>>>(
      cap, count, sdf, sdf_stride, end_packed, variance, alpha);
  return check_launch("center_alpha");
}

int sn_compact_samples(int64_t n_rays, const int32_t* packed_in, const uint8_t* visibility,
                       const int32_t* packed_out, const int64_t* ray_indices,
                       const float* t_starts, const float* t_ends, int64_t* ray_indices_out,
                       float* t_starts_out, float* t_ends_out, void* stream) {
  SN_REQUIRE(n_rays >= 0, "compact: n_rays < 0");
  if (n_rays == 0) return SN_OK;
  compact_kernel<<<div_up(n_rays * 32, 256), 256, 0, as_stream(stream)>>>(
      n_rays, packed_in, visibility, packed_out, ray_indices, t_starts, t_ends, ray_indices_out,
      t_starts_out, t_ends_out);
  return check_launch("compact_samples");
}

int sn_patch_points(int64_t cap, const int32_t* count, int patch_h, int patch_w,
                    const int64_t* patch_indices, const float* t_starts, const float* t_ends,
                    const float* rays_o, const float* rays_d, const float* plane_normal,
                    const int32_t* end_packed, const int32_t* n_ends, float* xyz,
                    float* t_pix_starts, float* t_pix_ends, int32_t* n_points, void* stream) {
  SN_REQUIRE(cap >= 0 && patch_h >= 1 && patch_w >= 1, "patch_points: bad sizes");
  SN_REQUIRE(n_ends != nullptr && end_packed != nullptr, "patch_points: null end info");
  const int P = patch_h * patch_w;
  const int kc = (patch_h / 2) * patch_w + patch_w / 2;
  patch_points_kernel<<<stride_grid((cap > 0 ? cap : 1) * P, 256, 8), 256, 0, as_stream(stream)>>>(
      cap, count, P, kc, patch_indices, t_starts, t_ends, rays_o, rays_d, plane_normal, end_packed,
      n_ends, xyz, t_pix_starts, t_pix_ends, n_points);
  return check_launch("patch_points");
}

int sn_near_far_sphere(int64_t n, const float* rays_o, const float* rays_d, int64_t stride,
                       float* near, float* far, float* jitter, uint64_t seed,
                       const int32_t* stream_counter, float* rays_o_out, float* rays_d_out,
                       void* stream) {
  SN_REQUIRE(n >= 0 && stride >= 3, "near_far_sphere: bad sizes");
  SN_REQUIRE(rays_o && rays_d && near && far, "near_far_sphere: null buffer");
  SN_REQUIRE((rays_o_out == nullptr) == (rays_d_out == nullptr),
             "near_far_sphere: give both ray copies or neither");
  if (n == 0) return SN_OK;
  near_far_kernel<<<stride_grid(n, 256, 8), 256, 0, as_stream(stream)>>>(
      n, rays_o, rays_d, stride, near, far, jitter, seed, stream_counter, rays_o_out, rays_d_out);
  return check_launch("near_far_sphere");
}

int sn_gen_patches(int64_t n_patches, int patch_h, int patch_w, const int32_t* cx, const int32_t* cy,
                   const int32_t* img, int n_views, int H, int W, const double* kinv, const double* pose,
                   const float* normals, const float* masks, float* rays_o, float* rays_d, float* plane_n,
                   float* vinv, float* normal_out, float* mask_out, void* stream) {
  SN_REQUIRE(n_patches >= 0 && patch_h >= 1 && patch_w >= 1 && n_views >= 1 && H >= patch_h && W >= patch_w,
             "gen_patches: bad sizes");
  SN_REQUIRE(cx && cy && img && kinv && pose && rays_o && rays_d && plane_n && vinv, "gen_patches: null buffer");
  SN_REQUIRE(!normals || normal_out, "gen_patches: normals given without normal_out");
  SN_REQUIRE(!masks || mask_out, "gen_patches: masks given without mask_out");
  if (n_patches == 0) return SN_OK;
  gen_patches_kernel<<<stride_grid(n_patches * patch_h * patch_w, 256, 8), 256, 0, as_stream(stream)>>>(
      n_patches, patch_h, patch_w, cx, cy, img, H, W, kinv, pose, normals, masks, rays_o, rays_d, plane_n, vinv,
      normal_out, mask_out);
  return check_launch("gen_patches");
}

int sn_scale_count(const int32_t* in, int32_t mul, int32_t add, int32_t* out, void* stream) {
  SN_REQUIRE(in && out, "scale_count: null buffer");
  scale_count_kernel<<<1, 1, 0, as_stream(stream)>>>(in, mul, add, out);
  return check_launch("scale_count");
}

int sn_mask_prep(int64_t n, const float* mask_in, float* mask_out, float* mask_sum, void* stream) {
  SN_REQUIRE(n >= 0, "mask_prep: n < 0");
  mask_prep_kernel<<<1, kMaskThreads, 0, as_stream(stream)>>>(n, mask_in, mask_out, mask_sum);
  return check_launch("mask_prep");
}

}  // extern "C"
