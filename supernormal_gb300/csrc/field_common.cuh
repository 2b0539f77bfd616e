// Definitions shared by the standalone encoding kernels (field.cu) and the
// tensor-core field kernels (field_tc.cu): hash-grid
// level geometry in tiny-cuda-nn's conventions (see field.cu), the 8-corner
// lookup of one level, and the argument block of the fused field kernels.
#pragma once

#include "common.cuh"

namespace sn {

constexpr int kH = 64;                    // hidden width (fixed, models/fields.py conf d_hidden)
constexpr int kMaxL = 16;                 // levels handled by the fused kernels
constexpr int kF = 2;                     // features per level (SuperNormal hard-codes 2)
constexpr int kDinMax = 3 + kMaxL * kF;   // 35
constexpr int kDinPad = 36;               // row stride of W0 in shared memory
constexpr int kDoutMax = 16;

struct GridDev {
  int L;
  uint32_t offset[kMaxL];
  uint32_t res[kMaxL];
  uint32_t size[kMaxL];     // entries in the level (tcnn hashmap_size)
  uint32_t magic[kMaxL];    // Granlund-Montgomery reciprocal of size
  uint8_t sh1[kMaxL], sh2[kMaxL];
  uint8_t dense[kMaxL];
  uint8_t pow2[kMaxL];      // size is a power of two (every hashed level): mod is a mask
  float scale[kMaxL];
};

// n mod d for uint32 n and invariant d (Granlund & Montgomery 1994, fig. 4.1).
__device__ __forceinline__ uint32_t fast_mod(uint32_t n, uint32_t d, uint32_t m, int s1, int s2) {
  const uint32_t t = __umulhi(m, n);
  const uint32_t q = (t + ((n - t) >> s1)) >> s2;
  return n - q * d;
}

struct LevelCorners {
  uint32_t idx[8];
  float w[8];
  float frac[3];
  uint32_t cell[3];  // integer cell coordinates (the 8 indices are a function of these)
};

// The 8 corners of x's cell at level l: entry indices and trilinear weights.
// Per-dimension terms are formed once (index of corner (dx,dy,dz) = a sum of
// the dense strides or an XOR of the prime products, weight = (wx * wy) * wz),
// which gives exactly the values of the corner-by-corner formula.
__device__ __forceinline__ void level_corners(const GridDev& g, int l, const float x[3],
                                              LevelCorners& c) {
  const float s = g.scale[l];
  float w0[3], w1[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const float p = __fmaf_rn(s, x[d], 0.5f);
    const float f = floorf(p);
    c.cell[d] = (uint32_t)(int)f;
    c.frac[d] = __fsub_rn(p, f);
    w1[d] = c.frac[d];
    w0[d] = __fsub_rn(1.0f, c.frac[d]);
  }
  const bool dense = g.dense[l] != 0;
  const uint32_t my = dense ? g.res[l] : 2654435761u;
  const uint32_t mz = dense ? g.res[l] * g.res[l] : 805459861u;
  const uint32_t tx[2] = {c.cell[0], c.cell[0] + 1u};
  const uint32_t ty[2] = {c.cell[1] * my, (c.cell[1] + 1u) * my};
  const uint32_t tz[2] = {c.cell[2] * mz, (c.cell[2] + 1u) * mz};
  float wxy[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) wxy[k] = __fmul_rn((k & 1) ? w1[0] : w0[0], (k & 2) ? w1[1] : w0[1]);
  const uint32_t off = g.offset[l], size = g.size[l];
  const bool pow2 = g.pow2[l] != 0;
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    const int dx = k & 1, dy = (k >> 1) & 1, dz = (k >> 2) & 1;
    const uint32_t index = dense ? tx[dx] + ty[dy] + tz[dz] : tx[dx] ^ ty[dy] ^ tz[dz];
    c.idx[k] = off + (pow2 ? (index & (size - 1u)) : fast_mod(index, size, g.magic[l], g.sh1[l], g.sh2[l]));
    c.w[k] = __fmul_rn(wxy[k & 3], dz ? w1[2] : w0[2]);
  }
}

// Entry index of the corner with integer coordinates (qx, qy, qz) at level l
// (the same arithmetic as level_corners).
__device__ __forceinline__ uint32_t corner_index(const GridDev& g, int l, uint32_t qx, uint32_t qy,
                                                 uint32_t qz) {
  const bool dense = g.dense[l] != 0;
  const uint32_t my = dense ? g.res[l] : 2654435761u;
  const uint32_t mz = dense ? g.res[l] * g.res[l] : 805459861u;
  const uint32_t index = dense ? qx + qy * my + qz * mz : qx ^ (qy * my) ^ (qz * mz);
  const uint32_t size = g.size[l];
  return g.offset[l] + (g.pow2[l] ? (index & (size - 1u)) : fast_mod(index, size, g.magic[l], g.sh1[l], g.sh2[l]));
}

// True on every lane when all 32 lanes of the warp are in the same cell.  Must
// be reached by all 32 lanes; the three shuffles are issued unconditionally
// (a short-circuit && around them would leave some lanes out of a full-mask
// shuffle and deadlock the warp).
__device__ __forceinline__ bool warp_same_cell(const LevelCorners& c) {
  const uint32_t c0 = __shfl_sync(0xffffffffu, c.cell[0], 0);
  const uint32_t c1 = __shfl_sync(0xffffffffu, c.cell[1], 0);
  const uint32_t c2 = __shfl_sync(0xffffffffu, c.cell[2], 0);
  const bool same = (c.cell[0] == c0) & (c.cell[1] == c1) & (c.cell[2] == c2);
  return __all_sync(0xffffffffu, same);
}

// d w_k / d x_d for linear interpolation (scale * +-1 * product of the other two factors).
__device__ __forceinline__ float corner_dw(const LevelCorners& c, int k, int d, float s) {
  float w = 1.0f;
#pragma unroll
  for (int e = 0; e < 3; ++e) {
    if (e == d) continue;
    const bool hi = (k >> e) & 1;
    w *= hi ? c.frac[e] : 1.0f - c.frac[e];
  }
  return ((k >> d) & 1) ? s * w : -s * w;
}

__device__ __forceinline__ void encode_level(const float* __restrict__ table, const GridDev& g,
                                             int l, const float x[3], float& e0, float& e1) {
  LevelCorners c;
  level_corners(g, l, x, c);
  const float2* t2 = reinterpret_cast<const float2*>(table);
  float2 v[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) v[k] = __ldg(t2 + c.idx[k]);
  float a = 0.0f, b = 0.0f;
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    a = __fmaf_rn(c.w[k], v[k].x, a);
    b = __fmaf_rn(c.w[k], v[k].y, b);
  }
  e0 = a;
  e1 = b;
}

struct FieldArgs {
  int64_t cap;
  const int32_t* count;   // optional device count (n = min(*count, cap))
  const float* x;
  const float* table;
  GridDev g;
  int active;             // active levels
  int din;                // 3 + L*F
  int dout;               // rows of W1
  int out_cols;           // outputs computed / gradients read (<= dout)
  float beta, thresh;
  const float* w0;        // (64, din)
  const float* b0;        // (64)
  const float* w1;        // (dout, 64)
  const float* b1;        // (dout)
  float* out;             // (n, out_cols)
  const float* grad_out;  // (n, out_cols)
  float* grad_table;
  float* grad_w0;
  float* grad_b0;
  float* grad_w1;
  float* grad_b1;
  float* grad_x;          // (n, 3) optional
  int32_t* status;        // optional: SN_STATUS_TIMEOUT is OR-ed here
  bool pair16;            // grad_table is 16-byte aligned: entry pairs may be added as float4
  bool table_half;        // table holds FP16 pairs (SN_FIELD_TABLE_FP16)
  bool one_pass;          // single-pass TF32 MLP products (SN_FIELD_MLP_TF32)
  bool bf16;              // forward: single-pass BF16 first layer (SN_FIELD_MLP_BF16)
  float2* enc_out;        // forward: level l of point p written at enc_out[l * cap + p]
  const float2* enc_in;   // backward: the encoding read from there instead of gathered
};

// Table entry (F = 2 features) as float2, from an FP32 or FP16 table.
__device__ __forceinline__ float2 load_entry(const FieldArgs& a, uint32_t idx) {
  if (a.table_half) return __half22float2(__ldg(reinterpret_cast<const __half2*>(a.table) + idx));
  return __ldg(reinterpret_cast<const float2*>(a.table) + idx);
}

// Encoding of one level from either table type.
__device__ __forceinline__ void encode_level_a(const FieldArgs& a, int l, const float x[3], float& e0,
                                               float& e1) {
  LevelCorners c;
  level_corners(a.g, l, x, c);
  float2 v[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) v[k] = load_entry(a, c.idx[k]);
  float s0 = 0.0f, s1 = 0.0f;
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    s0 = __fmaf_rn(c.w[k], v[k].x, s0);
    s1 = __fmaf_rn(c.w[k], v[k].y, s1);
  }
  e0 = s0;
  e1 = s1;
}

__device__ __forceinline__ int64_t effective_n(const FieldArgs& a) {
  if (!a.count) return a.cap;
  const int64_t c = *a.count;
  return c < a.cap ? c : a.cap;
}

// Tensor-core launchers (field_tc.cu).
int field_fwd_tc(const FieldArgs& a, cudaStream_t st);
int field_fwd_tc_segments(const FieldArgs* segs, int n_seg, cudaStream_t st);
int field_bwd_tc(const FieldArgs& a, cudaStream_t st);
int bounded_wait_selftest(int32_t* status, uint32_t polls, cudaStream_t st);
uint32_t bounded_wait_limit();
int field_grad_fwd_tc(const FieldArgs& a, float* sdf, float* grad, cudaStream_t st);
int field_grad_bwd_tc(const FieldArgs& a, const float* gamma, const float* rho, cudaStream_t st);

// Host helpers (field.cu).
int make_grid_dev(const sn_grid_desc* d, GridDev& g);
int fill_field_args(FieldArgs& a, int64_t n, const int32_t* count, const float* x, const float* table,
                    const sn_grid_desc* grid, int active_levels, const sn_mlp_desc* mlp, int out_cols);

}  // namespace sn
