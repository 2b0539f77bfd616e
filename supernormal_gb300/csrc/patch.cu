// Fused patch render of SuperNormal's training step (models/renderer.py:164-267):
// NeuS alpha, patch weights w = alpha * T (NA/nerfacc/cuda/csrc/render_weight.cu:87-118),
// dfd normals (models/renderer.py:187-223) or given 'ad' gradients, accumulation of
// normals and mask, and, in training mode, the losses of exp_runner.py:191-203 with
// the whole adjoint back to the field outputs.
//
// Layout: one block per patch, one warp per pixel of the patch, and the lanes of a
// warp take 32 consecutive samples of that pixel ray at a time.  Per-sample work
// (alpha, dfd, adjoints) is parallel across lanes; the transmittance product and
// the adjoint's suffix sums are warp scans with a carry between 32-sample chunks;
// dfd neighbours (same sample, adjacent pixels) are exchanged through shared
// memory.  Field-point layout: start (i, k) at i*P + k, the end of diff sample i
// at (S + slot_i)*P + k.
#include "neus_common.cuh"

#include <string.h>

namespace sn {

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
  float* alpha;             // forward outputs (nullable)
  float* weights;
  float* grads;             // (S, P, 3)
  float* comp_normal;       // (n_patches, P, 3)
  float* weight_sum;        // (n_patches, P)
  const float* g_comp;      // backward inputs
  const float* g_wsum;
  const float* g_grads;     // (S, P, 3) nullable
  const float* gt_normal;   // training inputs
  const float* gt_mask;
  const float* mask_sum;
  int loss_l1;
  float w_normal, w_eik, w_mask;
  float* d_sdf;             // backward outputs
  float* partials;          // (n_patches, 4): d_inv_s, normal, bce, eikonal
  float* carry;             // (n_patches, P)
  const float* ext_grads;   // 'ad': (S, P, 3) gradients from the field, nullable
  float* d_grads;           // 'ad': dL / d gradients
};

struct PixelRay {
  int k, r, c;
  float o[3], d[3], V[9];
};

struct Sample {
  float s0, s1, ts, te, dt, alpha, q, cdf0, cdf1;
  float g[3];
  float dxl, dxr, dyu, dyd;
  int diff, slot;
};

constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ float dist3(const float* a, const float* b) {
  const float x = __fsub_rn(a[0], b[0]), y = __fsub_rn(a[1], b[1]), z = __fsub_rn(a[2], b[2]);
  return sqrtf(__fadd_rn(__fadd_rn(__fmul_rn(x, x), __fmul_rn(y, y)), __fmul_rn(z, z)));
}

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
  return v;
}

// Per-sample quantities that need no neighbour; stages s0 and the start point in
// shared memory for the dfd of the other pixels.
__device__ __forceinline__ void load_sample(const PatchArgs& a, const PixelRay& R, int64_t i,
                                            int64_t S, float inv_s, bool ok, int lane,
                                            float* sm_s0, float* sm_pos, Sample& s) {
  const int P = a.P, k = R.k;
  if (ok) {
    const int2 ep = reinterpret_cast<const int2*>(a.endp)[i];
    s.diff = ep.y;
    s.slot = ep.x;
    s.s0 = a.sdf[i * P + k];
    s.s1 = ep.y ? a.sdf[(S + ep.x) * P + k] : (i + 1 < S ? a.sdf[(i + 1) * P + k] : s.s0);
    s.ts = a.tps[i * P + k];
    s.te = a.tpe[i * P + k];
  } else {
    s.diff = 0;
    s.slot = 0;
    s.s0 = s.s1 = 0.0f;
    s.ts = 0.0f;
    s.te = 1.0f;
  }
  s.dt = __fsub_rn(s.te, s.ts);
  s.alpha = neus_alpha(s.s0, s.s1, inv_s, &s.cdf0, &s.cdf1, &s.q);
  if (!ok) s.alpha = 0.0f;
  sm_s0[lane * P + k] = s.s0;
#pragma unroll
  for (int d = 0; d < 3; ++d) sm_pos[(lane * P + k) * 3 + d] = __fadd_rn(R.o[d], __fmul_rn(R.d[d], s.ts));
}

// dfd gradient (models/renderer.py:187-223) from the staged neighbours.
__device__ __forceinline__ void dfd_grad(const PatchArgs& a, const PixelRay& R, int lane,
                                         const float* sm_s0, const float* sm_pos, Sample& s) {
  const int P = a.P, W = a.W, H = a.H, k = R.k;
  const int kl = R.c > 0 ? k - 1 : k, kr = R.c < W - 1 ? k + 1 : k;
  const int ku = R.r > 0 ? k - W : k, kd = R.r < H - 1 ? k + W : k;
  const float* pos = sm_pos + (lane * P + k) * 3;
  const float sl = sm_s0[lane * P + kl], sr = sm_s0[lane * P + kr];
  const float su = sm_s0[lane * P + ku], sd = sm_s0[lane * P + kd];
  s.dxl = R.c > 0 ? dist3(pos, sm_pos + (lane * P + kl) * 3) : 0.0f;
  s.dxr = R.c < W - 1 ? dist3(sm_pos + (lane * P + kr) * 3, pos) : 0.0f;
  s.dyu = R.r > 0 ? dist3(pos, sm_pos + (lane * P + ku) * 3) : 0.0f;
  s.dyd = R.r < H - 1 ? dist3(sm_pos + (lane * P + kd) * 3, pos) : 0.0f;
  float proj[3];
  proj[0] = __fdiv_rn(__fsub_rn(s.s1, s.s0), s.dt);
  if (R.c == 0)
    proj[1] = __fdiv_rn(__fsub_rn(sr, s.s0), s.dxr);
  else if (R.c == W - 1)
    proj[1] = __fdiv_rn(__fsub_rn(s.s0, sl), s.dxl);
  else
    proj[1] = __fdiv_rn(__fsub_rn(sr, sl), __fadd_rn(s.dxl, s.dxr));
  if (R.r == 0)
    proj[2] = __fdiv_rn(__fsub_rn(sd, s.s0), s.dyd);
  else if (R.r == H - 1)
    proj[2] = __fdiv_rn(__fsub_rn(s.s0, su), s.dyu);
  else
    proj[2] = __fdiv_rn(__fsub_rn(sd, su), __fadd_rn(s.dyu, s.dyd));
#pragma unroll
  for (int e = 0; e < 3; ++e) {
    float v = __fmul_rn(R.V[3 * e + 0], proj[0]);
    v = __fadd_rn(v, __fmul_rn(R.V[3 * e + 1], proj[1]));
    v = __fadd_rn(v, __fmul_rn(R.V[3 * e + 2], proj[2]));
    s.g[e] = v;
  }
}

// One chunk's sample state: load, stage, neighbours, gradient.  Two block barriers.
__device__ __forceinline__ void chunk_sample(const PatchArgs& a, const PixelRay& R, int64_t i,
                                             int64_t S, float inv_s, bool ok, int lane,
                                             float* sm_s0, float* sm_pos, Sample& s) {
  load_sample(a, R, i, S, inv_s, ok, lane, sm_s0, sm_pos, s);
  __syncthreads();
  if (a.ext_grads) {
#pragma unroll
    for (int e = 0; e < 3; ++e) s.g[e] = ok ? a.ext_grads[(i * a.P + R.k) * 3 + e] : 0.0f;
    s.dxl = s.dxr = s.dyu = s.dyd = 0.0f;
  } else {
    dfd_grad(a, R, lane, sm_s0, sm_pos, s);
    if (!ok) s.g[0] = s.g[1] = s.g[2] = 0.0f;
  }
  __syncthreads();
}

// Transmittance T_j = prod_{i<j} (1 - alpha_i) along the pixel ray: the
// exclusive product over the lanes of 1 - alpha (formed exactly as a
// double-float), times the running carry of the earlier chunks (which
// advances).  Double-float throughout, so T keeps ~2^-44 relative accuracy
// over a thousand samples where a float32 running product drifts by ~j ulp.
__device__ __forceinline__ ff transmittance(float alpha, bool ok, ff& carry, int lane) {
  ff incl = ok ? two_sum(1.0f, -alpha) : ff{1.0f, 0.0f};
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const ff y = shfl_up_ff(incl, o);
    if (lane >= o) incl = ff_mul(y, incl);
  }
  ff excl = shfl_up_ff(incl, 1);
  if (lane == 0) excl = ff{1.0f, 0.0f};
  const ff T = ff_mul(carry, excl);
  carry = ff_mul(carry, shfl_ff(incl, 31));
  return T;
}

// d loss / d w_j of one sample: the rendered-normal gradient along the
// sample's gradient plus the weight-sum gradient (one expression for every
// pass, so the passes see the same rounded values).
__device__ __forceinline__ float weight_grad(const float gc[3], float gws, const float g[3]) {
  return __fadd_rn(__fmaf_rn(gc[2], g[2], __fmaf_rn(gc[1], g[1], __fmul_rn(gc[0], g[0]))), gws);
}

// 3x3 patches (288 threads): at least three blocks per SM (72 registers);
// unbounded, the kernel takes 96 registers and only two blocks fit.
template <int MODE, int MAXT>
__global__ void __launch_bounds__(MAXT, MAXT == 288 ? 3 : 1) patch_block_kernel(PatchArgs a) {
  extern __shared__ float sm[];
  const int P = a.P;
  float* sm_s0 = sm;             // [32][P]
  float* sm_pos = sm + 32 * P;   // [32][P][3]
  float* sm_x = sm + 128 * P;    // [32][P][4] dfd adjoint exchange
  __shared__ float red[32][4];
  const int k = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t p = blockIdx.x;
  PixelRay R;
  R.k = k;
  R.r = k / a.W;
  R.c = k - R.r * a.W;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    R.o[d] = a.ro[(p * P + k) * 3 + d];
    R.d[d] = a.rd[(p * P + k) * 3 + d];
  }
#pragma unroll
  for (int e = 0; e < 9; ++e) R.V[e] = a.vinv[(p * P + k) * 9 + e];
  const int64_t S = a.s_count ? min((int64_t)*a.s_count, a.s_cap) : a.s_cap;
  const int64_t base = a.packed[2 * p];
  const int steps = a.packed[2 * p + 1];
  const float inv_s = inv_s_from(a.variance);
  if (MODE != kFwd && lane == 0) a.carry[p * P + k] = 0.0f;

  // ---------------- forward ----------------
  ff Tc{1.0f, 0.0f};
  float cp0 = 0.0f, cp1 = 0.0f, cp2 = 0.0f, ws = 0.0f, eik = 0.0f;
  if (MODE != kBwd) {
    for (int j0 = 0; j0 < steps; j0 += 32) {
      const int j = j0 + lane;
      const bool ok = j < steps && base + j < S;  // S clamps a packed table past capacity
      const int64_t i = base + j;
      Sample s;
      chunk_sample(a, R, i, S, inv_s, ok, lane, sm_s0, sm_pos, s);
      const ff Tf = transmittance(s.alpha, ok, Tc, lane);
      const float w = ok ? __fmul_rn(s.alpha, ff_val(Tf)) : 0.0f;
      ws = __fadd_rn(ws, w);
      cp0 = __fadd_rn(cp0, __fmul_rn(w, s.g[0]));
      cp1 = __fadd_rn(cp1, __fmul_rn(w, s.g[1]));
      cp2 = __fadd_rn(cp2, __fmul_rn(w, s.g[2]));
      if (MODE == kFwd && ok) {
        if (a.alpha) a.alpha[i * P + k] = s.alpha;
        if (a.weights) a.weights[i * P + k] = w;
        if (a.grads) {
#pragma unroll
          for (int e = 0; e < 3; ++e) a.grads[(i * P + k) * 3 + e] = s.g[e];
        }
      }
      if (MODE == kTrain && ok) {
        const float nr = sqrtf(s.g[0] * s.g[0] + s.g[1] * s.g[1] + s.g[2] * s.g[2]);
        eik += (nr - 1.0f) * (nr - 1.0f);
      }
    }
    ws = warp_sum(ws);
    cp0 = warp_sum(cp0);
    cp1 = warp_sum(cp1);
    cp2 = warp_sum(cp2);
    if (MODE == kFwd) {
      if (lane == 0) {
        a.comp_normal[(p * P + k) * 3 + 0] = cp0;
        a.comp_normal[(p * P + k) * 3 + 1] = cp1;
        a.comp_normal[(p * P + k) * 3 + 2] = cp2;
        a.weight_sum[p * P + k] = ws;
      }
      return;
    }
  }

  // ---------------- output gradients ----------------
  float gc[3], gws, eik_scale = 0.0f;
  if (MODE == kTrain) {
    const float m = a.gt_mask[p * P + k];
    const float msum = *a.mask_sum;
    const float cp[3] = {cp0, cp1, cp2};
    float nl = 0.0f;
#pragma unroll
    for (int e = 0; e < 3; ++e) {
      const float err = __fmul_rn(__fsub_rn(cp[e], a.gt_normal[(p * P + k) * 3 + e]), m);
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
    const float cl = fminf(fmaxf(ws, 1e-5f), 1.0f - 1e-5f);
    const float bce = -(m * fmaxf(logf(cl), -100.0f) + (1.0f - m) * fmaxf(logf(1.0f - cl), -100.0f));
    const bool pass = ws >= 1e-5f && ws <= 1.0f - 1e-5f;
    gws = pass ? a.w_mask * (cl - m) / fmaxf((1.0f - cl) * cl, 1e-12f) / npix : 0.0f;
    eik_scale = a.w_eik * 2.0f / (float)(S * P);
    eik = warp_sum(eik);
    if (lane == 0) {
      red[k][1] = nl;
      red[k][2] = bce;
      red[k][3] = eik;
    }
  } else {
#pragma unroll
    for (int e = 0; e < 3; ++e) gc[e] = a.g_comp[(p * P + k) * 3 + e];
    gws = a.g_wsum[p * P + k];
  }

  // ---------------- adjoint: total = sum_j g_w_j w_j (double-float) ----------------
  ff total{0.0f, 0.0f};
  Tc = ff{1.0f, 0.0f};
  for (int j0 = 0; j0 < steps; j0 += 32) {
    const int j = j0 + lane;
    const bool ok = j < steps && base + j < S;  // S clamps a packed table past capacity
    Sample s;
    chunk_sample(a, R, base + j, S, inv_s, ok, lane, sm_s0, sm_pos, s);
    const ff Tf = transmittance(s.alpha, ok, Tc, lane);
    const float gw = ok ? weight_grad(gc, gws, s.g) : 0.0f;
    if (ok) total = ff_add(total, ff_mul(ff{gw, 0.0f}, ff_mul(Tf, ff{s.alpha, 0.0f})));
  }
  total = warp_sum_ff(total);

  // ---------------- adjoint per sample ----------------
  const int W = a.W, H = a.H;
  const int kl = R.c > 0 ? k - 1 : k, kr = R.c < W - 1 ? k + 1 : k;
  const int ku = R.r > 0 ? k - W : k, kd = R.r < H - 1 ? k + W : k;
  float d_inv = 0.0f, carry_in = 0.0f;
  ff prefix{0.0f, 0.0f};
  Tc = ff{1.0f, 0.0f};
  for (int j0 = 0; j0 < steps; j0 += 32) {
    const int j = j0 + lane;
    const bool ok = j < steps && base + j < S;  // S clamps a packed table past capacity
    const int64_t i = base + j;
    Sample s;
    chunk_sample(a, R, i, S, inv_s, ok, lane, sm_s0, sm_pos, s);
    const ff Tf = transmittance(s.alpha, ok, Tc, lane);
    const float T = ff_val(Tf);
    const float w = ok ? __fmul_rn(s.alpha, T) : 0.0f;
    const float gw = ok ? weight_grad(gc, gws, s.g) : 0.0f;
    // accum_j = sum_{i >= j} g_i w_i (NA/nerfacc/cuda/csrc/render_weight.cu:325-337)
    // = total - (sum of earlier chunks + this chunk's exclusive scan), in
    // double-float so the suffix behind the surface keeps its digits.  The
    // terms g_i alpha_i T_i are double-float products too: with T carried as
    // prod (1 - alpha) from exact differences, T_j - sum_{i >= j} alpha_i T_i
    // telescopes to the transmittance past the ray's end, so the numerator
    // g_j T_j - accum_j keeps its digits when that remainder is small (an
    // opaque ray), where float32 terms would leave rounding noise of order
    // eps * g_j T_j.
    ff incl = ok ? ff_mul(ff{gw, 0.0f}, ff_mul(Tf, ff{s.alpha, 0.0f})) : ff{0.0f, 0.0f};
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const ff y = shfl_up_ff(incl, o);
      if (lane >= o) incl = ff_add(y, incl);
    }
    ff excl = shfl_up_ff(incl, 1);
    if (lane == 0) excl = ff{0.0f, 0.0f};
    const ff accum = ff_add(total, ff_neg(ff_add(prefix, excl)));
    prefix = ff_add(prefix, shfl_ff(incl, 31));
    const float num = ff_val(ff_add(ff_mul(ff{gw, 0.0f}, Tf), ff_neg(accum)));
    const float dalpha = __fdiv_rn(num, fmaxf(__fsub_rn(1.0f, s.alpha), 1e-10f));
    // alpha = clip(q): sigmoid terms
    const float dq = (ok && s.q >= 0.0f && s.q <= 1.0f) ? dalpha : 0.0f;
    const float ce = s.cdf0 + 1e-5f;
    const float dp = dq / ce;
    const float dc = dp - dq * (s.cdf0 - s.cdf1 + 1e-5f) / (ce * ce);
    const float dn = -dp;
    const float dx0 = dc * s.cdf0 * (1.0f - s.cdf0);
    const float dx1 = dn * s.cdf1 * (1.0f - s.cdf1);
    float ds0 = dx0 * inv_s, ds1 = dx1 * inv_s;
    d_inv += dx0 * s.s0 + dx1 * s.s1;
    // gradient adjoint: accumulation + eikonal (+ caller's)
    float dg[3];
#pragma unroll
    for (int e = 0; e < 3; ++e) dg[e] = gc[e] * w;
    if (MODE == kTrain) {
      const float nr = sqrtf(s.g[0] * s.g[0] + s.g[1] * s.g[1] + s.g[2] * s.g[2]);
      if (ok && nr > 0.0f) {
        const float kk = eik_scale * (nr - 1.0f) / nr;
#pragma unroll
        for (int e = 0; e < 3; ++e) dg[e] += kk * s.g[e];
      }
    } else if (a.g_grads && ok) {
#pragma unroll
      for (int e = 0; e < 3; ++e) dg[e] += a.g_grads[(i * P + k) * 3 + e];
    }
    if (a.ext_grads) {
      if (ok) {
#pragma unroll
        for (int e = 0; e < 3; ++e) a.d_grads[(i * P + k) * 3 + e] = dg[e];
      }
    } else {
      float dpj[3];
#pragma unroll
      for (int b = 0; b < 3; ++b) dpj[b] = R.V[b] * dg[0] + R.V[3 + b] * dg[1] + R.V[6 + b] * dg[2];
      const float gt = ok ? dpj[0] / s.dt : 0.0f;
      ds1 += gt;
      ds0 -= gt;
      float to_l = 0.0f, to_r = 0.0f, to_u = 0.0f, to_d = 0.0f;
      if (ok) {
        if (R.c == 0) {
          const float g = dpj[1] / s.dxr;
          to_r += g;
          ds0 -= g;
        } else if (R.c == W - 1) {
          const float g = dpj[1] / s.dxl;
          ds0 += g;
          to_l -= g;
        } else {
          const float g = dpj[1] / (s.dxl + s.dxr);
          to_r += g;
          to_l -= g;
        }
        if (R.r == 0) {
          const float g = dpj[2] / s.dyd;
          to_d += g;
          ds0 -= g;
        } else if (R.r == H - 1) {
          const float g = dpj[2] / s.dyu;
          ds0 += g;
          to_u -= g;
        } else {
          const float g = dpj[2] / (s.dyu + s.dyd);
          to_d += g;
          to_u -= g;
        }
      }
      float* x = sm_x + (lane * P + k) * 4;
      x[0] = to_l;
      x[1] = to_r;
      x[2] = to_u;
      x[3] = to_d;
      __syncthreads();
      if (R.c > 0) ds0 += sm_x[(lane * P + kl) * 4 + 1];      // left neighbour's "to right"
      if (R.c < W - 1) ds0 += sm_x[(lane * P + kr) * 4 + 0];  // right neighbour's "to left"
      if (R.r > 0) ds0 += sm_x[(lane * P + ku) * 4 + 3];      // upper neighbour's "to down"
      if (R.r < H - 1) ds0 += sm_x[(lane * P + kd) * 4 + 2];  // lower neighbour's "to up"
      __syncthreads();
    }
    // route the end adjoint: its own end point, the next start of this ray, or
    // (after the patch's last sample) the next patch's first start via `carry`
    const bool to_next = ok && !s.diff && (j + 1 < steps);
    const float routed = to_next ? ds1 : 0.0f;
    float prev = __shfl_up_sync(kFull, routed, 1);
    if (lane == 0) prev = carry_in;
    carry_in = __shfl_sync(kFull, routed, 31);
    if (ok) {
      ds0 += prev;
      if (s.diff) {
        a.d_sdf[(S + s.slot) * P + k] = ds1;
      } else if (j + 1 == steps) {
        if (i + 1 < S)
          a.carry[p * P + k] = ds1;
        else
          ds0 += ds1;  // the last sample compares with itself
      }
      a.d_sdf[i * P + k] = ds0;
    }
  }
  d_inv = warp_sum(d_inv);
  if (lane == 0) red[k][0] = d_inv;
  __syncthreads();
  if (threadIdx.x == 0) {
    float acc[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    for (int q = 0; q < P; ++q) {
      acc[0] += red[q][0];
      if (MODE == kTrain) {
        acc[1] += red[q][1];
        acc[2] += red[q][2];
        acc[3] += red[q][3];
      }
    }
    a.partials[4 * p + 0] = acc[0];
    if (MODE == kTrain) {
      a.partials[4 * p + 1] = acc[1];
      a.partials[4 * p + 2] = acc[2];
      a.partials[4 * p + 3] = acc[3];
    }
  }
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

// Sums per-patch partials: grad_variance += d loss/d variance and
// out = {d/d variance, normal, bce, eikonal, total} (exp_runner.py:191-203).
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
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
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

static int patch_common(PatchArgs& a, int64_t n_patches, int patch_h, int patch_w,
                        const int32_t* packed, const int32_t* s_count, int64_t s_cap,
                        const int32_t* end_packed, const float* sdf, const float* tps,
                        const float* tpe, const float* rays_o, const float* rays_d,
                        const float* vinv, const float* variance) {
  memset(&a, 0, sizeof(a));
  SN_REQUIRE(n_patches >= 0 && s_cap >= 0, "patch_render: negative size");
  SN_REQUIRE(n_patches < (int64_t)1 << 31, "patch_render: too many patches");
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

template <int MODE>
static int launch_patch(const PatchArgs& a, cudaStream_t st, const char* what) {
  if (a.n_patches == 0) return SN_OK;
  const size_t smem = (size_t)256 * a.P * sizeof(float);
  const unsigned threads = 32 * a.P;
  // register budget follows the block size: 3x3 patches get up to 224 registers
  if (a.P <= 9)
    patch_block_kernel<MODE, 288><<<(unsigned)a.n_patches, threads, smem, st>>>(a);
  else if (a.P <= 16)
    patch_block_kernel<MODE, 512><<<(unsigned)a.n_patches, threads, smem, st>>>(a);
  else
    patch_block_kernel<MODE, 1024><<<(unsigned)a.n_patches, threads, smem, st>>>(a);
  return check_launch(what);
}

}  // namespace sn

using namespace sn;

extern "C" {

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
  return launch_patch<kFwd>(a, as_stream(stream), "patch_render_fwd");
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
  return launch_patch<kBwd>(a, as_stream(stream), "patch_render_bwd");
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
  return launch_patch<kTrain>(a, as_stream(stream), "patch_render_train");
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

}  // extern "C"
