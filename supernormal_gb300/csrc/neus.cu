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
//   * one fused per-patch kernel: NeuS alpha (:164-179), patch weights
//     w = alpha*T (:180 -> NA/nerfacc/cuda/csrc/render_weight.cu:87-118),
//     dfd normals (:187-223), accumulation of normals and mask (:263-267),
//     and, in training mode, the normal / eikonal / mask losses of
//     exp_runner.py:191-203 and the whole adjoint back to the SDF values.
//
// Field query points are laid out as [S*P start points][E*P end points]:
// start (i, k) at i*P + k and the end of diff sample i at (S + slot_i)*P + k,
// which is the order the reference concatenates positions_all.
#include "common.cuh"

namespace sn {

// diff[i] = t_ends[i] != t_starts[i+1] (last sample compares with itself);
// entries in [count, cap) are set to 0.
__global__ void end_diff_kernel(int64_t cap, const int32_t* __restrict__ count,
                                const float* __restrict__ ts, const float* __restrict__ te,
                                int32_t* __restrict__ diff) {
  const int64_t n = count ? min((int64_t)*count, cap) : cap;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < cap;
       i += (int64_t)gridDim.x * blockDim.x) {
    if (i >= n) {
      diff[i] = 0;  // entries past the live count take part in capacity-sized scans
      continue;
    }
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

__device__ __forceinline__ float inv_s_from(const float* variance) {
  // SingleVarianceNetwork: exp(variance * 10), clipped to [1e-6, 1e6]
  const float v = expf(__fmul_rn(*variance, 10.0f));
  return fminf(fmaxf(v, 1e-6f), 1e6f);
}

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

// Keep visible samples, preserving order (one thread per ray).
__global__ void compact_kernel(int64_t n_rays, const int32_t* __restrict__ pin,
                               const uint8_t* __restrict__ vis, const int32_t* __restrict__ pout,
                               const int64_t* __restrict__ ridx, const float* __restrict__ ts,
                               const float* __restrict__ te, int64_t* __restrict__ ridx_o,
                               float* __restrict__ ts_o, float* __restrict__ te_o) {
  const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= n_rays) return;
  const int64_t bi = pin[2 * r], bo = pout[2 * r];
  const int steps = pin[2 * r + 1];
  int c = 0;
  for (int j = 0; j < steps; ++j) {
    if (vis[bi + j]) {
      ridx_o[bo + c] = ridx[bi + j];
      ts_o[bo + c] = ts[bi + j];
      te_o[bo + c] = te[bi + j];
      ++c;
    }
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

// ---------------------------------------------------------------------------
// fused per-patch render / loss / adjoint
// ---------------------------------------------------------------------------
enum PatchMode { kFwd = 0, kBwd = 1, kTrain = 2 };

struct PatchArgs {
  int64_t n_patches;
  int H, W, P;
  const int32_t* packed;    // (n_patches, 2) over compacted samples
  const int32_t* s_count;   // device S (nullable: s_cap)
  int64_t s_cap;
  const int32_t* endp;      // (S, 2) {slot, diff}
  const float* sdf;         // field outputs, layout [S*P starts][E*P ends]
  const float* tps;         // (S, P)
  const float* tpe;         // (S, P)
  const float* ro;          // (n_patches, P, 3)
  const float* rd;          // (n_patches, P, 3)
  const float* vinv;        // (n_patches, P, 3, 3)
  const float* variance;    // device scalar
  // forward outputs (nullable)
  float* alpha;
  float* weights;
  float* grads;             // (S, P, 3)
  float* comp_normal;       // (n_patches, P, 3)
  float* weight_sum;        // (n_patches, P)
  // backward inputs
  const float* g_comp;      // (n_patches, P, 3)
  const float* g_wsum;      // (n_patches, P)
  const float* g_grads;     // (S, P, 3) nullable
  // training inputs
  const float* gt_normal;   // (n_patches, P, 3)
  const float* gt_mask;     // (n_patches, P) already binarised
  const float* mask_sum;    // device scalar: sum(mask) + 1e-5
  int loss_l1;
  float w_normal, w_eik, w_mask;
  // backward outputs
  float* d_sdf;             // same layout as sdf; every live entry is written once
  float* partials;          // (n_patches, 4): d_inv_s, normal, bce, eikonal
  float* carry;             // (n_patches, P): end adjoint owed to the next patch's first start
  // 'ad' gradient method: gradients come from the field (d sdf / dx at the
  // start points, models/renderer.py:225-226) instead of dfd
  const float* ext_grads;   // (S, P, 3) nullable
  float* d_grads;           // (S, P, 3): dL / d gradients when ext_grads is given
};

struct Lane {
  int k, r, c;
  unsigned mask;
  float o[3], d[3];
  float V[9];
};

struct SampleState {
  float s0, s1;   // sdf at start / end
  float ts, te;   // pixel-ray t
  float alpha, q, cdf0, cdf1;
  float g[3];     // dfd gradient
  float proj[3];  // df_dt, df_dx, df_dy
  float dt;       // te - ts
  float dxl, dxr, dyu, dyd;  // neighbour distances (0 where absent)
  int diff, slot;
};

__device__ __forceinline__ float dist3(const float a[3], const float b[3]) {
  const float x = __fsub_rn(a[0], b[0]), y = __fsub_rn(a[1], b[1]), z = __fsub_rn(a[2], b[2]);
  return sqrtf(__fadd_rn(__fadd_rn(__fmul_rn(x, x), __fmul_rn(y, y)), __fmul_rn(z, z)));
}

// Forward quantities of sample i at this lane (all P lanes of the patch call it).
__device__ __forceinline__ void sample_fwd(const PatchArgs& a, const Lane& L, int64_t i,
                                           int64_t S, float inv_s, SampleState& st) {
  const int P = a.P, W = a.W, H = a.H;
  const int2 ep = reinterpret_cast<const int2*>(a.endp)[i];
  st.diff = ep.y;
  st.slot = ep.x;
  st.s0 = a.sdf[i * P + L.k];
  if (ep.y)
    st.s1 = a.sdf[(S + ep.x) * P + L.k];
  else
    st.s1 = (i + 1 < S) ? a.sdf[(i + 1) * P + L.k] : st.s0;
  st.ts = a.tps[i * P + L.k];
  st.te = a.tpe[i * P + L.k];
  st.alpha = neus_alpha(st.s0, st.s1, inv_s, &st.cdf0, &st.cdf1, &st.q);
  if (a.ext_grads) {
#pragma unroll
    for (int e = 0; e < 3; ++e) st.g[e] = a.ext_grads[(i * P + L.k) * 3 + e];
    st.dt = __fsub_rn(st.te, st.ts);
    st.dxl = st.dxr = st.dyu = st.dyd = 0.0f;
    return;
  }

  float pos[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) pos[d] = __fadd_rn(L.o[d], __fmul_rn(L.d[d], st.ts));
  // neighbour values
  const int kl = L.c > 0 ? L.k - 1 : L.k, kr = L.c < W - 1 ? L.k + 1 : L.k;
  const int ku = L.r > 0 ? L.k - W : L.k, kd = L.r < H - 1 ? L.k + W : L.k;
  const float sl = __shfl_sync(L.mask, st.s0, kl), sr = __shfl_sync(L.mask, st.s0, kr);
  const float su = __shfl_sync(L.mask, st.s0, ku), sd = __shfl_sync(L.mask, st.s0, kd);
  float pl[3], pr[3], pu[3], pd[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    pl[d] = __shfl_sync(L.mask, pos[d], kl);
    pr[d] = __shfl_sync(L.mask, pos[d], kr);
    pu[d] = __shfl_sync(L.mask, pos[d], ku);
    pd[d] = __shfl_sync(L.mask, pos[d], kd);
  }
  st.dxl = L.c > 0 ? dist3(pos, pl) : 0.0f;
  st.dxr = L.c < W - 1 ? dist3(pr, pos) : 0.0f;
  st.dyu = L.r > 0 ? dist3(pos, pu) : 0.0f;
  st.dyd = L.r < H - 1 ? dist3(pd, pos) : 0.0f;
  st.dt = __fsub_rn(st.te, st.ts);
  st.proj[0] = __fdiv_rn(__fsub_rn(st.s1, st.s0), st.dt);
  if (L.c == 0)
    st.proj[1] = __fdiv_rn(__fsub_rn(sr, st.s0), st.dxr);
  else if (L.c == W - 1)
    st.proj[1] = __fdiv_rn(__fsub_rn(st.s0, sl), st.dxl);
  else
    st.proj[1] = __fdiv_rn(__fsub_rn(sr, sl), __fadd_rn(st.dxl, st.dxr));
  if (L.r == 0)
    st.proj[2] = __fdiv_rn(__fsub_rn(sd, st.s0), st.dyd);
  else if (L.r == H - 1)
    st.proj[2] = __fdiv_rn(__fsub_rn(st.s0, su), st.dyu);
  else
    st.proj[2] = __fdiv_rn(__fsub_rn(sd, su), __fadd_rn(st.dyu, st.dyd));
#pragma unroll
  for (int e = 0; e < 3; ++e) {
    float v = __fmul_rn(L.V[3 * e + 0], st.proj[0]);
    v = __fadd_rn(v, __fmul_rn(L.V[3 * e + 1], st.proj[1]));
    v = __fadd_rn(v, __fmul_rn(L.V[3 * e + 2], st.proj[2]));
    st.g[e] = v;
  }
}

// Sum of v over the P active lanes (every lane gets the total, in lane order).
__device__ __forceinline__ float lane_sum(unsigned mask, int P, float v) {
  float t = 0.0f;
  for (int s = 0; s < P; ++s) t += __shfl_sync(mask, v, s);
  return t;
}

template <int MODE>
__global__ void __launch_bounds__(128) patch_render_kernel(PatchArgs a) {
  const int lane = threadIdx.x & 31;
  const int64_t p = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  if (p >= a.n_patches) return;
  const int P = a.P;
  if (lane >= P) return;
  Lane L;
  L.k = lane;
  L.r = lane / a.W;
  L.c = lane - L.r * a.W;
  L.mask = (P == 32) ? 0xffffffffu : ((1u << P) - 1u);
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    L.o[d] = a.ro[(p * P + L.k) * 3 + d];
    L.d[d] = a.rd[(p * P + L.k) * 3 + d];
  }
#pragma unroll
  for (int e = 0; e < 9; ++e) L.V[e] = a.vinv[(p * P + L.k) * 9 + e];

  const int64_t S = a.s_count ? min((int64_t)*a.s_count, a.s_cap) : a.s_cap;
  const int64_t base = a.packed[2 * p];
  const int steps = a.packed[2 * p + 1];
  const float inv_s = inv_s_from(a.variance);
  if (MODE != kFwd) a.carry[p * P + L.k] = 0.0f;

  // ---- forward pass ----
  float T = 1.0f, comp[3] = {0.0f, 0.0f, 0.0f}, wsum = 0.0f, eik = 0.0f;
  if (MODE != kBwd) {
    for (int j = 0; j < steps; ++j) {
      const int64_t i = base + j;
      SampleState st;
      sample_fwd(a, L, i, S, inv_s, st);
      const float w = __fmul_rn(st.alpha, T);
      T = __fmul_rn(T, __fsub_rn(1.0f, st.alpha));
      wsum = __fadd_rn(wsum, w);
#pragma unroll
      for (int e = 0; e < 3; ++e) comp[e] = __fadd_rn(comp[e], __fmul_rn(w, st.g[e]));
      if (MODE == kFwd) {
        if (a.alpha) a.alpha[i * P + L.k] = st.alpha;
        if (a.weights) a.weights[i * P + L.k] = w;
        if (a.grads) {
#pragma unroll
          for (int e = 0; e < 3; ++e) a.grads[(i * P + L.k) * 3 + e] = st.g[e];
        }
      } else {
        const float nr = sqrtf(st.g[0] * st.g[0] + st.g[1] * st.g[1] + st.g[2] * st.g[2]);
        eik += (nr - 1.0f) * (nr - 1.0f);
      }
    }
    if (MODE == kFwd) {
#pragma unroll
      for (int e = 0; e < 3; ++e) a.comp_normal[(p * P + L.k) * 3 + e] = comp[e];
      a.weight_sum[p * P + L.k] = wsum;
      return;
    }
  }

  // ---- output gradients ----
  float gc[3], gws;
  float gradscale_eik = 0.0f;
  if (MODE == kTrain) {
    const float m = a.gt_mask[p * P + L.k];
    const float msum = *a.mask_sum;
    float nl = 0.0f;
#pragma unroll
    for (int e = 0; e < 3; ++e) {
      const float err = __fmul_rn(__fsub_rn(comp[e], a.gt_normal[(p * P + L.k) * 3 + e]), m);
      if (a.loss_l1) {
        nl += fabsf(err);
        const float sg = err > 0.0f ? 1.0f : (err < 0.0f ? -1.0f : 0.0f);
        gc[e] = a.w_normal * sg * m / msum;
      } else {
        nl += err * err;
        gc[e] = a.w_normal * 2.0f * err * m / msum;
      }
    }
    const float npix = (float)(a.n_patches * P);
    const float cl = fminf(fmaxf(wsum, 1e-5f), 1.0f - 1e-5f);
    const float lg = fmaxf(logf(cl), -100.0f), lg1 = fmaxf(logf(1.0f - cl), -100.0f);
    const float bce = -(m * lg + (1.0f - m) * lg1);
    const bool pass = wsum >= 1e-5f && wsum <= 1.0f - 1e-5f;
    gws = pass ? a.w_mask * (cl - m) / fmaxf((1.0f - cl) * cl, 1e-12f) / npix : 0.0f;
    gradscale_eik = a.w_eik * 2.0f / (float)(S * P);
    const float nl_p = lane_sum(L.mask, P, nl), bce_p = lane_sum(L.mask, P, bce),
                eik_p = lane_sum(L.mask, P, eik);
    if (L.k == 0) {
      a.partials[4 * p + 1] = nl_p;
      a.partials[4 * p + 2] = bce_p;
      a.partials[4 * p + 3] = eik_p;
    }
  } else {
#pragma unroll
    for (int e = 0; e < 3; ++e) gc[e] = a.g_comp[(p * P + L.k) * 3 + e];
    gws = a.g_wsum[p * P + L.k];
  }

  // ---- backward: accum = sum_j g_w_j w_j (reference order) ----
  float accum = 0.0f;
  T = 1.0f;
  for (int j = 0; j < steps; ++j) {
    SampleState st;
    sample_fwd(a, L, base + j, S, inv_s, st);
    const float w = __fmul_rn(st.alpha, T);
    T = __fmul_rn(T, __fsub_rn(1.0f, st.alpha));
    const float gw = gc[0] * st.g[0] + gc[1] * st.g[1] + gc[2] * st.g[2] + gws;
    accum = __fmaf_rn(gw, w, accum);
  }
  T = 1.0f;
  float d_inv = 0.0f, carry = 0.0f;
  const int W = a.W, H = a.H;
  for (int j = 0; j < steps; ++j) {
    const int64_t i = base + j;
    SampleState st;
    sample_fwd(a, L, i, S, inv_s, st);
    const float w = __fmul_rn(st.alpha, T);
    const float gw = gc[0] * st.g[0] + gc[1] * st.g[1] + gc[2] * st.g[2] + gws;
    // patch weight adjoint (NA/nerfacc/cuda/csrc/render_weight.cu:325-337)
    const float dalpha = __fdiv_rn(__fmaf_rn(gw, T, -accum), fmaxf(__fsub_rn(1.0f, st.alpha), 1e-10f));
    accum = __fmaf_rn(-gw, w, accum);
    T = __fmul_rn(T, __fsub_rn(1.0f, st.alpha));
    // alpha = clip(q) -> sigmoid terms
    const float dq = (st.q >= 0.0f && st.q <= 1.0f) ? dalpha : 0.0f;
    const float ce = st.cdf0 + 1e-5f;
    const float dp = dq / ce;
    const float dc = dp - dq * (st.cdf0 - st.cdf1 + 1e-5f) / (ce * ce);
    const float dn = -dp;
    const float dx0 = dc * st.cdf0 * (1.0f - st.cdf0);
    const float dx1 = dn * st.cdf1 * (1.0f - st.cdf1);
    float ds0 = dx0 * inv_s, ds1 = dx1 * inv_s;
    d_inv += dx0 * st.s0 + dx1 * st.s1;
    // gradient adjoint: accumulation + eikonal (+ caller's)
    float dg[3];
#pragma unroll
    for (int e = 0; e < 3; ++e) dg[e] = gc[e] * w;
    if (MODE == kTrain) {
      const float nr = sqrtf(st.g[0] * st.g[0] + st.g[1] * st.g[1] + st.g[2] * st.g[2]);
      if (nr > 0.0f) {
        const float k = gradscale_eik * (nr - 1.0f) / nr;
#pragma unroll
        for (int e = 0; e < 3; ++e) dg[e] += k * st.g[e];
      }
    } else if (a.g_grads) {
#pragma unroll
      for (int e = 0; e < 3; ++e) dg[e] += a.g_grads[(i * P + L.k) * 3 + e];
    }
    if (a.ext_grads) {
      // 'ad': the gradients are field outputs; their adjoint goes to the field
#pragma unroll
      for (int e = 0; e < 3; ++e) a.d_grads[(i * P + L.k) * 3 + e] = dg[e];
    } else {
    float dpj[3];
#pragma unroll
    for (int b = 0; b < 3; ++b) dpj[b] = L.V[b] * dg[0] + L.V[3 + b] * dg[1] + L.V[6 + b] * dg[2];
    // df_dt
    const float gt = dpj[0] / st.dt;
    ds1 += gt;
    ds0 -= gt;
    // df_dx / df_dy: contributions to self, left/right, up/down
    float to_l = 0.0f, to_r = 0.0f, to_u = 0.0f, to_d = 0.0f;
    if (L.c == 0) {
      const float g = dpj[1] / st.dxr;
      to_r += g;
      ds0 -= g;
    } else if (L.c == W - 1) {
      const float g = dpj[1] / st.dxl;
      ds0 += g;
      to_l -= g;
    } else {
      const float g = dpj[1] / (st.dxl + st.dxr);
      to_r += g;
      to_l -= g;
    }
    if (L.r == 0) {
      const float g = dpj[2] / st.dyd;
      to_d += g;
      ds0 -= g;
    } else if (L.r == H - 1) {
      const float g = dpj[2] / st.dyu;
      ds0 += g;
      to_u -= g;
    } else {
      const float g = dpj[2] / (st.dyu + st.dyd);
      to_d += g;
      to_u -= g;
    }
    const int kl = L.c > 0 ? L.k - 1 : L.k, kr = L.c < W - 1 ? L.k + 1 : L.k;
    const int ku = L.r > 0 ? L.k - W : L.k, kd = L.r < H - 1 ? L.k + W : L.k;
    const float from_l = __shfl_sync(L.mask, to_r, kl);  // left neighbour's "to right"
    const float from_r = __shfl_sync(L.mask, to_l, kr);
    const float from_u = __shfl_sync(L.mask, to_d, ku);
    const float from_d = __shfl_sync(L.mask, to_u, kd);
    if (L.c > 0) ds0 += from_l;
    if (L.c < W - 1) ds0 += from_r;
    if (L.r > 0) ds0 += from_u;
    if (L.r < H - 1) ds0 += from_d;
    }
    ds0 += carry;
    carry = 0.0f;
    // route the end adjoint
    if (st.diff) {
      a.d_sdf[(S + st.slot) * P + L.k] = ds1;
    } else if (i + 1 >= S) {
      ds0 += ds1;  // last sample compares with itself
    } else if (j + 1 < steps) {
      carry = ds1;  // next start of this patch
    } else {
      a.carry[p * P + L.k] = ds1;  // first start of a later patch: added by the fixup kernel
    }
    a.d_sdf[i * P + L.k] = ds0;
  }
  const float d_inv_p = lane_sum(L.mask, P, d_inv);
  if (L.k == 0) a.partials[4 * p + 0] = d_inv_p;
}

// Adds each patch's carried end adjoint to the start of the sample after its
// last one (only when that end was not evaluated separately).
__global__ void carry_fixup_kernel(int64_t n_patches, int P, const int32_t* __restrict__ packed,
                                   const int32_t* __restrict__ s_count, int64_t s_cap,
                                   const int32_t* __restrict__ endp,
                                   const float* __restrict__ carry, float* __restrict__ d_sdf) {
  const int64_t S = s_count ? min((int64_t)*s_count, s_cap) : s_cap;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n_patches * P;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p = t / P;
    const int k = (int)(t - p * P);
    const int steps = packed[2 * p + 1];
    if (steps == 0) continue;
    const int64_t last = (int64_t)packed[2 * p] + steps - 1;
    if (last + 1 >= S || endp[2 * last + 1]) continue;
    d_sdf[(last + 1) * P + k] += carry[t];
  }
}

// Sums per-patch partials: out[0] = d loss / d variance contribution
// (d_inv_s * d inv_s / d variance), out[1..3] = normal, bce, eikonal sums,
// out[4] = total training loss.
__global__ void __launch_bounds__(256)
patch_finalize_kernel(int64_t n_patches, int P, const float* __restrict__ partials,
                      const int32_t* __restrict__ s_count, int64_t s_cap,
                      const float* __restrict__ variance, const float* __restrict__ mask_sum,
                      float w_normal, float w_eik, float w_mask, float* __restrict__ out,
                      float* __restrict__ grad_variance) {
  __shared__ double red[4][8];
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  for (int64_t p = threadIdx.x; p < n_patches; p += blockDim.x)
#pragma unroll
    for (int q = 0; q < 4; ++q) acc[q] += (double)partials[4 * p + q];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    double v = acc[q];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) red[q][threadIdx.x >> 5] = v;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double s[4] = {0, 0, 0, 0};
    for (int q = 0; q < 4; ++q)
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s[q] += red[q][w];
    const float ev = expf(__fmul_rn(*variance, 10.0f));
    const bool pass = ev >= 1e-6f && ev <= 1e6f;
    const float dvar = pass ? (float)s[0] * ev * 10.0f : 0.0f;
    if (grad_variance) *grad_variance += dvar;
    if (out) {
      const int64_t S = s_count ? min((int64_t)*s_count, s_cap) : s_cap;
      const float nl = mask_sum ? (float)s[1] / *mask_sum : 0.0f;
      const float bce = (float)(s[2] / (double)(n_patches * P));
      const float eik = S > 0 ? (float)(s[3] / (double)(S * P)) : 0.0f;
      out[0] = dvar;
      out[1] = nl;
      out[2] = bce;
      out[3] = eik;
      out[4] = w_normal * nl + w_mask * bce + w_eik * eik;
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
__global__ void __launch_bounds__(256)
mask_prep_kernel(int64_t n, const float* __restrict__ mask_in, float* __restrict__ mask_out,
                 float* __restrict__ mask_sum) {
  __shared__ float red[8];
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
  compact_kernel<<<div_up(n_rays, 128), 128, 0, as_stream(stream)>>>(
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

static int patch_common(PatchArgs& a, int64_t n_patches, int patch_h, int patch_w,
                        const int32_t* packed, const int32_t* s_count, int64_t s_cap,
                        const int32_t* end_packed, const float* sdf, const float* tps,
                        const float* tpe, const float* rays_o, const float* rays_d,
                        const float* vinv, const float* variance) {
  memset(&a, 0, sizeof(a));
  SN_REQUIRE(n_patches >= 0 && s_cap >= 0, "patch_render: negative size");
  SN_REQUIRE(patch_h >= 3 && patch_w >= 3 && patch_h * patch_w <= 32,
             "patch_render: patch must be at least 3x3 and at most 32 pixels (got %dx%d)", patch_h,
             patch_w);
  SN_REQUIRE(packed && end_packed && sdf && tps && tpe && rays_o && rays_d && vinv && variance,
             "patch_render: null input");
  a.n_patches = n_patches;
  a.H = patch_h;
  a.W = patch_w;
  a.P = patch_h * patch_w;
  a.packed = packed;
  a.s_count = s_count;
  a.s_cap = s_cap;
  a.endp = end_packed;
  a.sdf = sdf;
  a.tps = tps;
  a.tpe = tpe;
  a.ro = rays_o;
  a.rd = rays_d;
  a.vinv = vinv;
  a.variance = variance;
  return SN_OK;
}

int sn_patch_render_fwd(int64_t n_patches, int patch_h, int patch_w, const int32_t* packed_info,
                        const int32_t* s_count, int64_t s_cap, const int32_t* end_packed,
                        const float* sdf, const float* t_pix_starts, const float* t_pix_ends,
                        const float* rays_o, const float* rays_d, const float* v_inverse,
                        const float* variance, float* alpha, float* weights, float* gradients,
                        float* comp_normal, float* weight_sum, const float* ext_gradients,
                        void* stream) {
  PatchArgs a;
  SN_TRY(patch_common(a, n_patches, patch_h, patch_w, packed_info, s_count, s_cap, end_packed, sdf,
                      t_pix_starts, t_pix_ends, rays_o, rays_d, v_inverse, variance));
  SN_REQUIRE(comp_normal && weight_sum, "patch_render_fwd: null output");
  a.ext_grads = ext_gradients;
  a.alpha = alpha;
  a.weights = weights;
  a.grads = gradients;
  a.comp_normal = comp_normal;
  a.weight_sum = weight_sum;
  if (n_patches == 0) return SN_OK;
  patch_render_kernel<kFwd><<<div_up(n_patches * 32, 128), 128, 0, as_stream(stream)>>>(a);
  return check_launch("patch_render_fwd");
}

int sn_patch_render_bwd(int64_t n_patches, int patch_h, int patch_w, const int32_t* packed_info,
                        const int32_t* s_count, int64_t s_cap, const int32_t* end_packed,
                        const float* sdf, const float* t_pix_starts, const float* t_pix_ends,
                        const float* rays_o, const float* rays_d, const float* v_inverse,
                        const float* variance, const float* grad_comp_normal,
                        const float* grad_weight_sum, const float* grad_gradients, float* d_sdf,
                        float* partials, float* carry, const float* ext_gradients,
                        float* d_gradients, void* stream) {
  PatchArgs a;
  SN_TRY(patch_common(a, n_patches, patch_h, patch_w, packed_info, s_count, s_cap, end_packed, sdf,
                      t_pix_starts, t_pix_ends, rays_o, rays_d, v_inverse, variance));
  SN_REQUIRE(grad_comp_normal && grad_weight_sum && d_sdf && partials && carry,
             "patch_render_bwd: null buffer");
  SN_REQUIRE(ext_gradients == nullptr || d_gradients != nullptr,
             "patch_render_bwd: d_gradients required with ext_gradients");
  a.ext_grads = ext_gradients;
  a.d_grads = d_gradients;
  a.carry = carry;
  a.g_comp = grad_comp_normal;
  a.g_wsum = grad_weight_sum;
  a.g_grads = grad_gradients;
  a.d_sdf = d_sdf;
  a.partials = partials;
  if (n_patches == 0) return SN_OK;
  patch_render_kernel<kBwd><<<div_up(n_patches * 32, 128), 128, 0, as_stream(stream)>>>(a);
  return check_launch("patch_render_bwd");
}

int sn_patch_render_train(int64_t n_patches, int patch_h, int patch_w, const int32_t* packed_info,
                          const int32_t* s_count, int64_t s_cap, const int32_t* end_packed,
                          const float* sdf, const float* t_pix_starts, const float* t_pix_ends,
                          const float* rays_o, const float* rays_d, const float* v_inverse,
                          const float* variance, const float* gt_normal, const float* gt_mask,
                          const float* mask_sum, int loss_l1, float w_normal, float w_eikonal,
                          float w_mask, float* d_sdf, float* partials, float* carry,
                          const float* ext_gradients, float* d_gradients, void* stream) {
  PatchArgs a;
  SN_TRY(patch_common(a, n_patches, patch_h, patch_w, packed_info, s_count, s_cap, end_packed, sdf,
                      t_pix_starts, t_pix_ends, rays_o, rays_d, v_inverse, variance));
  SN_REQUIRE(gt_normal && gt_mask && mask_sum && d_sdf && partials && carry,
             "patch_render_train: null buffer");
  SN_REQUIRE(ext_gradients == nullptr || d_gradients != nullptr,
             "patch_render_train: d_gradients required with ext_gradients");
  a.ext_grads = ext_gradients;
  a.d_grads = d_gradients;
  a.carry = carry;
  a.gt_normal = gt_normal;
  a.gt_mask = gt_mask;
  a.mask_sum = mask_sum;
  a.loss_l1 = loss_l1;
  a.w_normal = w_normal;
  a.w_eik = w_eikonal;
  a.w_mask = w_mask;
  a.d_sdf = d_sdf;
  a.partials = partials;
  if (n_patches == 0) return SN_OK;
  patch_render_kernel<kTrain><<<div_up(n_patches * 32, 128), 128, 0, as_stream(stream)>>>(a);
  return check_launch("patch_render_train");
}

int sn_patch_carry_fixup(int64_t n_patches, int patch_size, const int32_t* packed_info,
                         const int32_t* s_count, int64_t s_cap, const int32_t* end_packed,
                         const float* carry, float* d_sdf, void* stream) {
  SN_REQUIRE(n_patches >= 0 && patch_size >= 1, "patch_carry_fixup: bad sizes");
  if (n_patches == 0) return SN_OK;
  carry_fixup_kernel<<<stride_grid(n_patches * patch_size, 256, 8), 256, 0, as_stream(stream)>>>(
      n_patches, patch_size, packed_info, s_count, s_cap, end_packed, carry, d_sdf);
  return check_launch("patch_carry_fixup");
}

int sn_patch_finalize(int64_t n_patches, int patch_size, const float* partials,
                      const int32_t* s_count, int64_t s_cap, const float* variance,
                      const float* mask_sum, float w_normal, float w_eikonal, float w_mask,
                      float* out, float* grad_variance, void* stream) {
  SN_REQUIRE(n_patches >= 0 && patch_size >= 1, "patch_finalize: bad sizes");
  SN_REQUIRE(partials && variance, "patch_finalize: null buffer");
  patch_finalize_kernel<<<1, 256, 0, as_stream(stream)>>>(n_patches, patch_size, partials, s_count,
                                                          s_cap, variance, mask_sum, w_normal,
                                                          w_eikonal, w_mask, out, grad_variance);
  return check_launch("patch_finalize");
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

int sn_scale_count(const int32_t* in, int32_t mul, int32_t add, int32_t* out, void* stream) {
  SN_REQUIRE(in && out, "scale_count: null buffer");
  scale_count_kernel<<<1, 1, 0, as_stream(stream)>>>(in, mul, add, out);
  return check_launch("scale_count");
}

int sn_mask_prep(int64_t n, const float* mask_in, float* mask_out, float* mask_sum, void* stream) {
  SN_REQUIRE(n >= 0, "mask_prep: n < 0");
  mask_prep_kernel<<<1, 256, 0, as_stream(stream)>>>(n, mask_in, mask_out, mask_sum);
  return check_launch("mask_prep");
}

}  // extern "C"
