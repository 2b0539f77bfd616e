// Tensor-core (tcgen05) fused SDF field: hash-grid encoding + SDFNetwork MLP
// (models/fields.py:76-99) forward and backward, fp32-accurate (3xTF32).
//
// A CTA owns 128-point tiles (persistent over tiles) with 16 warps: warp w
// serves TMEM lane quadrant q = w % 4 (points 32q..32q+31 of the tile) as
// member g = w / 4 of that quadrant's group of four.  The four members split
// the per-point work -- hash-grid levels (interleaved, see level_of), hidden units --
// and write their parts of each point's row straight into the point's TMEM
// lane, where the tensor core reads it as the A operand.  One thread issues
// the MMAs; everyone else waits on an mbarrier (bounded).
//
// MLP input order inside the kernels (K = 40): encoding features first
// (level l, feature f -> column 2l + f), then x (columns 32..34), then zeros;
// W0 is permuted to match when it is staged, and the weight gradient is
// permuted back when it is flushed.
//
// Forward:  H = IN W0^T (TMEM), act = softplus(H + b0), out = W1 act + b1.
// Backward: recompute H, dH = (W1^T g) * softplus'(H + b0),
//           dIN = dH W0 (TMEM) -> table-gradient scatter (+ dL/dx),
//           dW0 += dH^T IN over the CTA's points (TMEM, A = [dH_hi; dH_lo]
//           stacked as 128 rows so two MMAs per K step give all four
//           hi/lo products), db0 from a row of ones in IN^T,
//           dW1, db1 by warp reductions.
#include "field_common.cuh"
#include "tc.cuh"

#include <cuda_bf16.h>

#include <string.h>

namespace sn {
namespace {

constexpr int kTile = 128;
constexpr int kK1 = 40;        // MLP input width inside the kernels (35 used)
constexpr int kN2 = 48;        // dIN columns (N of the second MMA; 35 used)
constexpr int kXCol = 32;      // first column of x in the permuted input
constexpr int kOnesRow = 35;   // row of ones in IN^T (gives db0)
constexpr uint32_t kCols = 256;      // forward: up to two CTAs per SM
constexpr uint32_t kBwdCols = 512;   // backward: one CTA per SM
// IN^T and [dH_hi; dH_lo] (K = the tile's points, written one point per
// thread): core matrices 144 bytes apart along K so a warp's 32 stores of one
// row fall in 32 banks.
constexpr uint32_t kLboP = 144, kSboP = (kTile / 4) * kLboP;

// The three 3xTF32 passes (hi.hi, lo.hi, hi.lo) of a GEMM are issued by
// threads of different warps into separate TMEM accumulators (no ordering
// between the issuing threads is needed) and summed by the readers; one
// mbarrier counts one commit per issuing thread.
//
// Forward TMEM columns (256): H part 0 [0,64), parts 1+2 [64,128); input
// rows hi [128,168), lo [168,208).
constexpr uint32_t kFwdColH0 = 0, kFwdColH1 = 64, kFwdColInHi = 128, kFwdColInLo = 128 + kK1;
// Backward TMEM columns (512): H parts / dIN parts at [0,64), [64,128),
// [128,192); input rows then dH (hi, lo) share [192,320); dW0 accumulates in
// [320,368).
__host__ __device__ constexpr uint32_t col_part(int p) { return 64u * (uint32_t)p; }
constexpr uint32_t kColInHi = 192, kColInLo = 192 + kK1;
constexpr uint32_t kColDhHi = 192, kColDhLo = 256, kColDw0 = 320;

// K steps of D (+)= A[TMEM columns from a] B[shared memory, descriptor b]^T.
__device__ __forceinline__ void mma_chain(uint32_t d, uint32_t a, uint64_t b, int ksteps, uint32_t idesc,
                                          bool fresh) {
  for (int ks = 0; ks < ksteps; ++ks)
    tc::mma_ts(d, a + 8u * ks, b + 16u * ks, idesc, (fresh && ks == 0) ? 0u : 1u);
}

// With M members per quadrant group, member g handles levels g, g+M, g+2M, ...
// (coarse and fine levels mixed, which balances the scatter's shuffle and
// atomic work); with eight members (the backward kernels) levels g and 15 - g,
// which measured 1.3 % faster than g and g + 8 in the backward (the members
// scattering levels 1-4, whose same-cell groups cost the most, then also hold
// the cheapest fine levels).  Member g's 32/M features sit in permuted input
// columns (32/M)g .. (32/M)g + 32/M - 1.
template <int M>
__device__ __forceinline__ int level_of(int g, int i) {
  if constexpr (M == 8) return i == 0 ? g : 15 - g;
  return g + M * i;
}

// Permuted input column -> column of W0 (or -1 for a zero column).
template <int M>
__device__ __forceinline__ int w0_col(int c, int L) {
  constexpr int kFpm = kXCol / M;  // features per member
  if (c < kXCol) {
    const int l = level_of<M>(c / kFpm, (c % kFpm) >> 1);
    return l < L ? 3 + 2 * l + (c & 1) : -1;
  }
  if (c < kXCol + 3) return c - kXCol;
  return -1;
}

// Table-gradient contributions of the warp's 32 points at one level.
//  * Lanes sharing a cell are summed first: the cell of the first remaining
//    lane is matched exactly (three coordinates), and if it holds at least
//    kMinGroupLanes lanes their float2 contributions to the 8 corners are
//    summed by a reduce-scatter over the warp (corner bit 2 follows lane bit
//    4, bit 1 lane bit 3, bit 0 lane bit 2) and added by one float2 atomic per
//    corner, issued together by lanes 0, 4, ..., 28; up to kMaxCellGroups cells.
//  * The lanes left add their own 8 corners; an x-adjacent corner pair that
//    occupies one aligned pair of entries goes out as one 16-byte atomic.
// Measured on the bench workload's backward (two rounds each): groups of
// >= 8 lanes, at most 2 per level, beat >= 4 lanes / 4 groups by 2 %, and
// smaller groups or more of them were slower (their shuffles cost more than
// the L2 requests they save).
constexpr int kMaxCellGroups = 2;
constexpr int kMinGroupLanes = 8;

__device__ __forceinline__ void scatter_level(const GridDev& gd, int l, const LevelCorners& c, float d0,
                                              float d1, bool live, bool pair16, float2* gt2, int lane) {
  constexpr unsigned kAll = 0xffffffffu;
  unsigned rest = __ballot_sync(kAll, live);
  for (int it = 0; it < kMaxCellGroups && rest != 0u; ++it) {
    const int ld = __ffs(rest) - 1;
    const uint32_t c0 = __shfl_sync(kAll, c.cell[0], ld);
    const uint32_t c1 = __shfl_sync(kAll, c.cell[1], ld);
    const uint32_t c2 = __shfl_sync(kAll, c.cell[2], ld);
    const bool in = ((rest >> lane) & 1u) & (c.cell[0] == c0) & (c.cell[1] == c1) & (c.cell[2] == c2);
    const unsigned gm = __ballot_sync(kAll, in);
    if (__popc(gm) < kMinGroupLanes) break;  // the same decision on every lane
    const float e0 = in ? d0 : 0.0f, e1 = in ? d1 : 0.0f;
    float v[16];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      v[2 * k] = c.w[k] * e0;
      v[2 * k + 1] = c.w[k] * e1;
    }
    float a8[8], a4[4], a2[2];
    bool up = lane & 16;
#pragma unroll
    for (int i = 0; i < 8; ++i) a8[i] = (up ? v[i + 8] : v[i]) + __shfl_xor_sync(kAll, up ? v[i] : v[i + 8], 16);
    up = lane & 8;
#pragma unroll
    for (int i = 0; i < 4; ++i) a4[i] = (up ? a8[i + 4] : a8[i]) + __shfl_xor_sync(kAll, up ? a8[i] : a8[i + 4], 8);
    up = lane & 4;
#pragma unroll
    for (int i = 0; i < 2; ++i) a2[i] = (up ? a4[i + 2] : a4[i]) + __shfl_xor_sync(kAll, up ? a4[i] : a4[i + 2], 4);
#pragma unroll
    for (int sft = 2; sft > 0; sft >>= 1) {
      a2[0] += __shfl_xor_sync(kAll, a2[0], sft);
      a2[1] += __shfl_xor_sync(kAll, a2[1], sft);
    }
    const int k = lane >> 2;  // corner summed into lanes 4k..4k+3
    if ((lane & 3) == 0)
      atomicAdd(gt2 + corner_index(gd, l, c0 + (k & 1), c1 + ((k >> 1) & 1), c2 + (k >> 2)),
                make_float2(a2[0], a2[1]));
    rest &= ~gm;
  }
  if ((rest >> lane) & 1u) {
#pragma unroll
    for (int m = 0; m < 4; ++m) {  // corners 2m (dx = 0) and 2m + 1 (dx = 1)
      const uint32_t i0 = c.idx[2 * m], i1 = c.idx[2 * m + 1];
      const float2 v0 = make_float2(c.w[2 * m] * d0, c.w[2 * m] * d1);
      const float2 v1 = make_float2(c.w[2 * m + 1] * d0, c.w[2 * m + 1] * d1);
      if (pair16 && i1 == (i0 ^ 1u)) {
        const float4 q = (i0 & 1u) ? make_float4(v1.x, v1.y, v0.x, v0.y) : make_float4(v0.x, v0.y, v1.x, v1.y);
        atomicAdd(reinterpret_cast<float4*>(gt2 + (i0 & ~1u)), q);
      } else {
        atomicAdd(gt2 + i0, v0);
        atomicAdd(gt2 + i1, v1);
      }
    }
  }
}

// W0 (64, din) -> B1 (N = 64 hidden, K = 40 inputs, K-major) hi/lo, and, when
// b2 is given, W0^T -> B2 (N = 48 inputs, K = 64 hidden, K-major) hi/lo.
template <int M>
__device__ void stage_w0(const FieldArgs& a, uint8_t* b1_hi, uint8_t* b1_lo, uint8_t* b2_hi,
                         uint8_t* b2_lo) {
  for (int e = threadIdx.x; e < kH * kN2; e += blockDim.x) {
    const int j = e / kN2, c = e - j * kN2;
    const int src = c < kK1 ? w0_col<M>(c, a.g.L) : -1;
    const float v = src >= 0 ? a.w0[j * a.din + src] : 0.0f;
    uint32_t hi, lo;
    tc::tf32_split(v, hi, lo);
    if (c < kK1) {
      const uint32_t o1 = tc::kmajor_offset(j, c, kK1);
      *reinterpret_cast<uint32_t*>(b1_hi + o1) = hi;
      *reinterpret_cast<uint32_t*>(b1_lo + o1) = lo;
    }
    if (b2_hi) {
      const uint32_t o2 = tc::kmajor_offset(c, j, kH);
      *reinterpret_cast<uint32_t*>(b2_hi + o2) = hi;
      *reinterpret_cast<uint32_t*>(b2_lo + o2) = lo;
    }
  }
}

// BF16 first-layer operands: K padded to 48, core matrices of 8 rows x 8
// elements (16 bytes), K-adjacent core matrices contiguous (LBO 128 bytes),
// 8-row groups kBf16Sbo bytes apart.
constexpr int kK1b = 48;
constexpr uint32_t kBf16Sbo = (kK1b / 8) * 128u;

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);  // .x (lower K) in the low half
  return *reinterpret_cast<const uint32_t*>(&v);
}

// W0 (64, din) -> B (N = 64 hidden, K = 48 permuted inputs, K-major), BF16.
template <int M>
__device__ void stage_w0_bf16(const FieldArgs& a, uint8_t* b) {
  for (int e = threadIdx.x; e < kH * kK1b; e += blockDim.x) {
    const int j = e / kK1b, c = e - j * kK1b;
    const int src = c < kK1 ? w0_col<M>(c, a.g.L) : -1;
    const float v = src >= 0 ? a.w0[j * a.din + src] : 0.0f;
    const uint32_t off = (uint32_t)(j >> 3) * kBf16Sbo + (uint32_t)(c >> 3) * 128u + (uint32_t)(j & 7) * 16u +
                         (uint32_t)(c & 7) * 2u;
    *reinterpret_cast<__nv_bfloat16*>(b + off) = __float2bfloat16_rn(v);
  }
}

__device__ __forceinline__ void load_point(const FieldArgs& a, int64_t p, int64_t n, float x[3]) {
  if (p < n) {
    x[0] = a.x[3 * p];
    x[1] = a.x[3 * p + 1];
    x[2] = a.x[3 * p + 2];
  } else {
    x[0] = x[1] = x[2] = 0.0f;
  }
}
template <int OC>
__device__ __forceinline__ void load_grad(const FieldArgs& a, int64_t p, int64_t n, float go[OC]) {
#pragma unroll
  for (int o = 0; o < OC; ++o) go[o] = (p < n && o < a.out_cols) ? a.grad_out[p * a.out_cols + o] : 0.0f;
}

// Member g's levels of point p from the encoding cache (zeros past n or the
// active levels, as encode_group gives).  Read once, so streamed past L2.
template <int M>
__device__ __forceinline__ void load_enc(const FieldArgs& a, int g, int64_t p, int64_t n,
                                         float e[2 * (16 / M)]) {
#pragma unroll
  for (int i = 0; i < 16 / M; ++i) {
    const int l = level_of<M>(g, i);
    float2 v = make_float2(0.0f, 0.0f);
    if (p < n && l < a.active) v = __ldcs(a.enc_in + (int64_t)l * a.cap + p);
    e[2 * i] = v.x;
    e[2 * i + 1] = v.y;
  }
}

// Encoding of member g's levels of point x: e[2i + f] for level level_of(g, i).
// PAIRED: two levels at a time, all 16 corner gathers issued before any is
// used (about two L2 round trips per phase instead of four; the backward,
// which has the registers for it).  Otherwise one level at a time.
template <bool PAIRED, int M = 4>
__device__ __forceinline__ void encode_group(const FieldArgs& a, int g, bool live, const float x[3],
                                             float e[2 * (16 / M)]) {
  constexpr int kLpm = 16 / M;  // levels per member
  if constexpr (!PAIRED) {
#pragma unroll
    for (int i = 0; i < kLpm; ++i) {
      const int l = level_of<M>(g, i);
      float e0 = 0.0f, e1 = 0.0f;
      if (live && l < a.active) encode_level_a(a, l, x, e0, e1);
      e[2 * i] = e0;
      e[2 * i + 1] = e1;
    }
  } else {
#pragma unroll
  for (int i0 = 0; i0 < kLpm; i0 += 2) {
    const int la = level_of<M>(g, i0), lb = level_of<M>(g, i0 + 1);
    const bool ua = la < a.active, ub = lb < a.active;  // uniform across the CTA
    LevelCorners ca, cb;
    float2 va[8], vb[8];
    if (ua) {
      level_corners(a.g, la, x, ca);
#pragma unroll
      for (int k = 0; k < 8; ++k) va[k] = load_entry(a, ca.idx[k]);
    }
    if (ub) {
      level_corners(a.g, lb, x, cb);
#pragma unroll
      for (int k = 0; k < 8; ++k) vb[k] = load_entry(a, cb.idx[k]);
    }
    float a0 = 0.0f, a1 = 0.0f, b0 = 0.0f, b1 = 0.0f;
    if (ua) {
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        a0 = __fmaf_rn(ca.w[k], va[k].x, a0);
        a1 = __fmaf_rn(ca.w[k], va[k].y, a1);
      }
    }
    if (ub) {
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        b0 = __fmaf_rn(cb.w[k], vb[k].x, b0);
        b1 = __fmaf_rn(cb.w[k], vb[k].y, b1);
      }
    }
    e[2 * i0] = live ? a0 : 0.0f;
    e[2 * i0 + 1] = live ? a1 : 0.0f;
    e[2 * i0 + 2] = live ? b0 : 0.0f;
    e[2 * i0 + 3] = live ? b1 : 0.0f;
  }
  }
}

// Sums 8 per-lane values over the warp by a reduce-scatter (9 shuffles):
// lanes 4m .. 4m+3 end with the sum of value m.
__device__ __forceinline__ float warp_reduce_scatter8(const float v[8], int lane) {
  constexpr unsigned kAll = 0xffffffffu;
  float a4[4], a2[2];
  bool up = lane & 16;
#pragma unroll
  for (int i = 0; i < 4; ++i) a4[i] = (up ? v[i + 4] : v[i]) + __shfl_xor_sync(kAll, up ? v[i] : v[i + 4], 16);
  up = lane & 8;
#pragma unroll
  for (int i = 0; i < 2; ++i) a2[i] = (up ? a4[i + 2] : a4[i]) + __shfl_xor_sync(kAll, up ? a4[i] : a4[i + 2], 8);
  up = lane & 4;
  float a1 = (up ? a2[1] : a2[0]) + __shfl_xor_sync(kAll, up ? a2[0] : a2[1], 4);
  a1 += __shfl_xor_sync(kAll, a1, 2);
  a1 += __shfl_xor_sync(kAll, a1, 1);
  return a1;
}

// Sums 16 per-lane values over the warp by a reduce-scatter (16 shuffles):
// lanes 2m and 2m+1 end with the sum of value m.
__device__ __forceinline__ float warp_reduce_scatter16(const float v[16], int lane) {
  constexpr unsigned kAll = 0xffffffffu;
  float a8[8], a4[4], a2[2];
  bool up = lane & 16;
#pragma unroll
  for (int i = 0; i < 8; ++i) a8[i] = (up ? v[i + 8] : v[i]) + __shfl_xor_sync(kAll, up ? v[i] : v[i + 8], 16);
  up = lane & 8;
#pragma unroll
  for (int i = 0; i < 4; ++i) a4[i] = (up ? a8[i + 4] : a8[i]) + __shfl_xor_sync(kAll, up ? a8[i] : a8[i + 4], 8);
  up = lane & 4;
#pragma unroll
  for (int i = 0; i < 2; ++i) a2[i] = (up ? a4[i + 2] : a4[i]) + __shfl_xor_sync(kAll, up ? a4[i] : a4[i + 2], 4);
  up = lane & 2;
  float a1 = (up ? a2[1] : a2[0]) + __shfl_xor_sync(kAll, up ? a2[0] : a2[1], 2);
  a1 += __shfl_xor_sync(kAll, a1, 1);
  return a1;
}

__device__ __forceinline__ void st_split8(uint32_t ta_hi, uint32_t ta_lo, const float v[8]) {
  uint32_t hi[8], lo[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) tc::tf32_split(v[i], hi[i], lo[i]);
  tc::tmem_st8(ta_hi, hi);
  tc::tmem_st8(ta_lo, lo);
}

__device__ __forceinline__ void st_split4(uint32_t ta_hi, uint32_t ta_lo, const float v[4]) {
  uint32_t hi[4], lo[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) tc::tf32_split(v[i], hi[i], lo[i]);
  tc::tmem_st4(ta_hi, hi);
  tc::tmem_st4(ta_lo, lo);
}
// Stores N (4, 8 or 16) values, split into TF32 hi/lo, at columns c_hi / c_lo.
template <int N>
__device__ __forceinline__ void st_split(uint32_t ta_hi, uint32_t ta_lo, const float* v) {
  if (N == 4) {
    st_split4(ta_hi, ta_lo, v);
  } else {
#pragma unroll
    for (int i = 0; i < N; i += 8) st_split8(ta_hi + i, ta_lo + i, v + i);
  }
}

// ---------------------------------------------------------------------------
// forward
// ---------------------------------------------------------------------------
// M members per TMEM lane quadrant: 128 M threads; member g owns levels
// level_of<M>(g, i), input columns (32/M)g .. and hidden units (64/M)g ...
// M = 4: 512 threads, two CTAs per SM; M = 8: 1024 threads, one CTA per SM.
constexpr int kFwdMembers = 4;

template <int M>
struct FwdSmem {
  static constexpr uint32_t b1_hi = 0, b1_lo = 10240, w1 = 20480, b0 = 24576, b1 = 24832,
                            part = 24896, bar = part + M * kTile * kDoutMax * 4, slot = bar + 8,
                            end = slot + 8;
  // M = 4: more than 228/3 KB, so at most two CTAs (2 x 256 TMEM columns) per SM
  static constexpr size_t bytes = M == 4 ? 80 * 1024 : end;
};
static_assert(FwdSmem<4>::end <= FwdSmem<4>::bytes, "forward shared memory map");

template <int N>
__device__ __forceinline__ void tmem_ld_n(uint32_t ta, float* v) {
  if constexpr (N == 16) tc::tmem_ld16(ta, v);
  else if constexpr (N == 8) tc::tmem_ld8(ta, v);
  else tc::tmem_ld4(ta, v);
}

// Segments of one forward launch: point sets that each have their own table,
// level geometry and MLP (several objects' queries in one persistent launch).
constexpr int kMaxSegments = 4;
struct FieldSegments {
  int n;
  FieldArgs seg[kMaxSegments];
};

// ONE: a single output column (the sdf; every training call), else up to kDoutMax.
// Each CTA works through the segments in order: it stages segment s's
// weights, processes its share of s's tiles (persistent, strided by the
// grid), then moves on; one launch of one segment is the ordinary forward.
template <bool ONE, int M>
__global__ void __launch_bounds__(128 * M, M == 4 ? 2 : 1)
field_fwd_tc_kernel(const __grid_constant__ FieldSegments segs) {
  constexpr int kOc = ONE ? 1 : kDoutMax;
  constexpr int kNt = 128 * M;      // threads
  constexpr int kLpm = 16 / M;      // levels per member
  constexpr int kFpm = 2 * kLpm;    // input features per member
  constexpr int kHpm = kH / M;      // hidden units per member
  using Sm = FwdSmem<M>;
  extern __shared__ __align__(1024) uint8_t sm[];
  float* s_w1 = reinterpret_cast<float*>(sm + Sm::w1);
  float* s_b0 = reinterpret_cast<float*>(sm + Sm::b0);
  float* s_b1 = reinterpret_cast<float*>(sm + Sm::b1);
  float* s_part = reinterpret_cast<float*>(sm + Sm::part);
  uint64_t* bar = reinterpret_cast<uint64_t*>(sm + Sm::bar);
  uint32_t* slot = reinterpret_cast<uint32_t*>(sm + Sm::slot);
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  const int q = warp & 3, g = warp >> 2;
  const int pt = 32 * q + lane;  // point within the tile == TMEM lane

  if (warp == 0) {
    tc::tmem_alloc(slot, kCols);
    tc::tmem_relinquish();
  }
  if (t == 0) tc::mbar_init(bar, 2);  // one commit each from threads 0 and 32
  const uint32_t lb = (uint32_t)(32 * q);
  const uint32_t s_b1_hi = tc::smem_u32(sm + Sm::b1_hi), s_b1_lo = tc::smem_u32(sm + Sm::b1_lo);
  uint32_t phase = 0;
  bool ok = true;
  uint32_t tbase = 0;

  for (int si = 0; si < segs.n && ok; ++si) {
    const FieldArgs& a = segs.seg[si];
    const int oc = a.out_cols;
    const float inv_beta = 1.0f / a.beta;
    if (si > 0) __syncthreads();     // the previous segment's last tile is done with the weights
    if (a.bf16) {
      if constexpr (M == 4) stage_w0_bf16<M>(a, sm + Sm::b1_hi);
    } else {
      stage_w0<M>(a, sm + Sm::b1_hi, sm + Sm::b1_lo, nullptr, nullptr);
    }
    for (int e = t; e < kDoutMax * kH; e += kNt) s_w1[e] = e / kH < oc ? a.w1[e] : 0.0f;
    if (t < kH) s_b0[t] = a.b0[t];
    if (t < kDoutMax) s_b1[t] = t < oc ? a.b1[t] : 0.0f;
    tc::fence_proxy_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    tbase = *slot;

    const int64_t n = effective_n(a);
    const int64_t n_tiles = (n + kTile - 1) / kTile;
    // this point's coordinates one tile ahead: the stream read overlaps a tile
    float xn[3] = {0.0f, 0.0f, 0.0f};
    load_point(a, (int64_t)blockIdx.x * kTile + pt, n, xn);
    for (int64_t tile = blockIdx.x; tile < n_tiles; tile += gridDim.x) {
      const int64_t p = tile * kTile + pt;
      const bool live = p < n;
      const float x[3] = {xn[0], xn[1], xn[2]};
      load_point(a, (tile + gridDim.x) * kTile + pt, n, xn);
      {
        float e[kFpm];
        encode_group<(M == 8), M>(a, g, live, x, e);
        if (a.enc_out && live) {
#pragma unroll
          for (int i = 0; i < kLpm; ++i) {
            const int l = level_of<M>(g, i);
            if (l < a.active) __stcs(a.enc_out + (int64_t)l * a.cap + p, make_float2(e[2 * i], e[2 * i + 1]));
          }
        }
        if (a.bf16) {
          // BF16 pairs: member g's 8 features in columns 4g .. 4g + 3, x (and
          // the zero padding up to K = 48) in columns 16 .. 23
          if constexpr (M == 4) {
            uint32_t pk[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) pk[i] = pack_bf16(e[2 * i], e[2 * i + 1]);
            tc::tmem_st4(tc::taddr(tbase, lb, kFwdColInHi + 4 * g), pk);
            if (g == 0) {
              const uint32_t xp[8] = {pack_bf16(x[0], x[1]), pack_bf16(x[2], 0.0f), 0u, 0u, 0u, 0u, 0u, 0u};
              tc::tmem_st8(tc::taddr(tbase, lb, kFwdColInHi + kXCol / 2), xp);
            }
          }
        } else {
          st_split<kFpm>(tc::taddr(tbase, lb, kFwdColInHi + kFpm * g), tc::taddr(tbase, lb, kFwdColInLo + kFpm * g), e);
          if (g == 0) {
            const float xv[8] = {x[0], x[1], x[2], 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
            st_split8(tc::taddr(tbase, lb, kFwdColInHi + kXCol), tc::taddr(tbase, lb, kFwdColInLo + kXCol), xv);
          }
        }
      }
      tc::tmem_wait_st();
      tc::fence_before_sync();
      __syncthreads();
      if (t == 0 || t == 32) {  // H = IN W0^T, M=128, N=64, K=40 (BF16: K=48, three K=16 steps)
        tc::fence_after_sync();
        if (a.bf16) {
          if (t == 0) {
            const uint64_t wb = tc::smem_desc(s_b1_hi, 128u, kBf16Sbo);
            for (int ks = 0; ks < kK1b / 16; ++ks)
              tc::mma_ts_f16(tc::taddr(tbase, 0, kFwdColH0), tc::taddr(tbase, 0, kFwdColInHi + 8u * ks),
                             wb + (uint64_t)((256u * ks) >> 4), tc::idesc_bf16(kTile, kH), ks > 0 ? 1u : 0u);
          }
        } else {
          const uint32_t idesc = tc::idesc_tf32(kTile, kH);
          const uint32_t sbo = (kK1 / 4) * 128u;
          const uint64_t w_hi = tc::smem_desc(s_b1_hi, 128u, sbo), w_lo = tc::smem_desc(s_b1_lo, 128u, sbo);
          if (t == 0) {
            mma_chain(tc::taddr(tbase, 0, kFwdColH0), tc::taddr(tbase, 0, kFwdColInHi), w_hi, kK1 / 8, idesc, true);
          } else if (!a.one_pass) {
            mma_chain(tc::taddr(tbase, 0, kFwdColH1), tc::taddr(tbase, 0, kFwdColInLo), w_hi, kK1 / 8, idesc, true);
            mma_chain(tc::taddr(tbase, 0, kFwdColH1), tc::taddr(tbase, 0, kFwdColInHi), w_lo, kK1 / 8, idesc, false);
          }
        }
        tc::mma_commit(bar);
      }
      const bool got = tc::mbar_wait_bounded(bar, phase);
      phase ^= 1u;
      if (!__syncthreads_and(got)) {
        ok = false;
        break;
      }
      tc::fence_after_sync();
      // hidden units kHpm g .. kHpm g + kHpm - 1 of this point -> partial outputs
      float h[kHpm];
      tmem_ld_n<kHpm>(tc::taddr(tbase, lb, kFwdColH0 + kHpm * g), h);
      if (!a.one_pass && !a.bf16) {
        float h1[kHpm];
        tmem_ld_n<kHpm>(tc::taddr(tbase, lb, kFwdColH1 + kHpm * g), h1);
        tc::tmem_wait_ld();
#pragma unroll
        for (int i = 0; i < kHpm; ++i) h[i] += h1[i];
      }
      tc::tmem_wait_ld();
      float part[kOc];
#pragma unroll
      for (int o = 0; o < kOc; ++o) part[o] = 0.0f;
#pragma unroll
      for (int i = 0; i < kHpm; ++i) {
        const int j = kHpm * g + i;
        float act, sg_unused;
        softplus_fwd_grad_fast(h[i] + s_b0[j], a.beta, inv_beta, a.thresh, act, sg_unused);
#pragma unroll
        for (int o = 0; o < kOc; ++o)
          if (o < oc) part[o] = fmaf(s_w1[o * kH + j], act, part[o]);
      }
#pragma unroll
      for (int o = 0; o < kOc; ++o)
        if (o < oc) s_part[(g * kTile + pt) * kDoutMax + o] = part[o];
      tc::fence_before_sync();
      __syncthreads();
      if (g == 0 && live) {
        for (int o = 0; o < oc; ++o) {
          float sum = s_b1[o];
#pragma unroll
          for (int m = 0; m < M; ++m) sum += s_part[(m * kTile + pt) * kDoutMax + o];
          a.out[p * oc + o] = sum;
        }
      }
      __syncthreads();
    }
  }
  if (!ok) {
    if (t == 0) {
      for (int si = 0; si < segs.n; ++si)
        if (segs.seg[si].status) atomicOr(segs.seg[si].status, SN_STATUS_TIMEOUT);
    }
    (void)tc::mbar_wait_bounded(bar, phase ^ 1u);
    __syncthreads();
  }
  tc::fence_after_sync();
  if (warp == 0) tc::tmem_dealloc(*slot, kCols);
}

// ---------------------------------------------------------------------------
// backward
// ---------------------------------------------------------------------------
struct BwdSmem {
  static constexpr uint32_t b1_hi = 0, b1_lo = 10240, b2_hi = 20480, b2_lo = 32768, a3 = 45056,
                            b3_hi = a3 + 16 * kSboP, b3_lo = b3_hi + 6 * kSboP, w1 = b3_lo + 6 * kSboP,
                            b0 = w1 + kDoutMax * kH * 4, dx = b0 + kH * 4, bar = dx + 8 * kTile * 3 * 4,
                            bar3 = bar + 8, slot = bar3 + 8, dw1 = slot + 8, db1 = dw1 + kDoutMax * kH * 4,
                            end = db1 + kDoutMax * 4;
};
constexpr size_t kBwdSmemBytes = BwdSmem::end;
static_assert(BwdSmem::end <= 227 * 1024, "backward shared memory map");

__device__ __forceinline__ void st_smem_u32(uint8_t* base, uint32_t off, uint32_t v) {
  *reinterpret_cast<uint32_t*>(base + off) = v;
}

// Part p of the second MMA, dIN = dH W0 (M=128, N=48, K=64): p = 0 dH_hi W_hi,
// 1 dH_lo W_hi, 2 dH_hi W_lo, each into its own accumulator.
__device__ __forceinline__ void issue_mma2_part(uint32_t tbase, const uint8_t* sm, int part) {
  const uint32_t sbo2 = (kH / 4) * 128u;
  const uint64_t w = tc::smem_desc(tc::smem_u32(sm + (part == 2 ? BwdSmem::b2_lo : BwdSmem::b2_hi)), 128u, sbo2);
  mma_chain(tc::taddr(tbase, 0, col_part(part)), tc::taddr(tbase, 0, part == 1 ? kColDhLo : kColDhHi), w, kH / 8,
            tc::idesc_tf32(kTile, kN2), true);
}

// Part p of the first MMA, H = IN W0^T (M=128, N=64, K=40).
__device__ __forceinline__ void issue_mma1_part(uint32_t tbase, uint32_t s_b1_hi, uint32_t s_b1_lo, int part) {
  const uint32_t sbo = (kK1 / 4) * 128u;
  const uint64_t w = tc::smem_desc(part == 2 ? s_b1_lo : s_b1_hi, 128u, sbo);
  mma_chain(tc::taddr(tbase, 0, col_part(part)), tc::taddr(tbase, 0, part == 1 ? kColInLo : kColInHi), w, kK1 / 8,
            tc::idesc_tf32(kTile, kH), true);
}

// Third MMA: dW0 += [dH_hi; dH_lo]^T-rows x IN^T (M=128, N=48, K=128 points),
// accumulated in TMEM over all of the CTA's tiles.
__device__ __forceinline__ void issue_mma3(uint32_t tbase, const uint8_t* sm, bool first_tile, bool one_pass) {
  const uint32_t s_a3 = tc::smem_u32(sm + BwdSmem::a3);
  const uint32_t s_b3_hi = tc::smem_u32(sm + BwdSmem::b3_hi), s_b3_lo = tc::smem_u32(sm + BwdSmem::b3_lo);
  const uint32_t idesc = tc::idesc_tf32(kTile, kN2);
  const uint32_t d3 = tc::taddr(tbase, 0, kColDw0);
  const uint64_t da = tc::smem_desc(s_a3, kLboP, kSboP), dbh = tc::smem_desc(s_b3_hi, kLboP, kSboP),
                 dbl = tc::smem_desc(s_b3_lo, kLboP, kSboP);
  for (int ks = 0; ks < kTile / 8; ++ks) {
    const uint64_t k0 = (2u * kLboP * ks) >> 4;
    tc::mma_ss(d3, da + k0, dbh + k0, idesc, (first_tile && ks == 0) ? 0u : 1u);
    if (!one_pass) tc::mma_ss(d3, da + k0, dbl + k0, idesc, 1);
  }
}

// N (4, 8 or 16) columns from col of this warp's lanes, summed over the
// three accumulator parts (part 0 alone for one-pass products).
template <int N>
__device__ __forceinline__ void ld_parts(uint32_t tbase, uint32_t lb, uint32_t col, bool one_pass, float* v) {
#pragma unroll
  for (int p = 0; p < 3; ++p) {
    if (p > 0 && one_pass) break;
    float u[N];
    const uint32_t ta = tc::taddr(tbase, lb, col_part(p) + col);
    if (N == 16) {
      tc::tmem_ld16(ta, u);
    } else if (N == 8) {
      tc::tmem_ld8(ta, u);
    } else {
      tc::tmem_ld4(ta, u);
    }
    tc::tmem_wait_ld();
#pragma unroll
    for (int i = 0; i < N; ++i) v[i] = p == 0 ? u[i] : v[i] + u[i];
  }
}

// M members per TMEM lane quadrant: 128 M threads, each member owning 16/M
// levels, 32/M input columns and 64/M hidden units of its 32 points.
constexpr int kBwdMembers = 8;

template <bool ONE, int M>
__global__ void __launch_bounds__(128 * M, 1) field_bwd_tc_kernel(FieldArgs a) {
  constexpr int kOc = ONE ? 1 : kDoutMax;
  constexpr int kNt = 128 * M;      // threads
  constexpr int kLpm = 16 / M;      // levels per member
  constexpr int kFpm = 2 * kLpm;    // input features per member
  constexpr int kHpm = kH / M;      // hidden units per member
  extern __shared__ __align__(1024) uint8_t sm[];
  float* s_w1 = reinterpret_cast<float*>(sm + BwdSmem::w1);
  float* s_b0 = reinterpret_cast<float*>(sm + BwdSmem::b0);
  float* s_dx = reinterpret_cast<float*>(sm + BwdSmem::dx);
  uint8_t* a3 = sm + BwdSmem::a3;
  uint8_t* b3_hi = sm + BwdSmem::b3_hi;
  uint8_t* b3_lo = sm + BwdSmem::b3_lo;
  uint64_t* bar = reinterpret_cast<uint64_t*>(sm + BwdSmem::bar);    // first and second MMAs
  uint64_t* bar3 = reinterpret_cast<uint64_t*>(sm + BwdSmem::bar3);  // weight-gradient MMAs
  uint32_t* slot = reinterpret_cast<uint32_t*>(sm + BwdSmem::slot);
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  const int q = warp & 3, g = warp >> 2;
  const int pt = 32 * q + lane;
  const int oc = a.out_cols;
  const float inv_beta = 1.0f / a.beta;
  const bool want_table = a.grad_table != nullptr;
  const bool want_x = a.grad_x != nullptr;

  stage_w0<M>(a, sm + BwdSmem::b1_hi, sm + BwdSmem::b1_lo, sm + BwdSmem::b2_hi, sm + BwdSmem::b2_lo);
  for (int e = t; e < kDoutMax * kH; e += kNt) s_w1[e] = e / kH < oc ? a.w1[e] : 0.0f;
  if (t < kH) s_b0[t] = a.b0[t];
  float* s_dw1 = reinterpret_cast<float*>(sm + BwdSmem::dw1);
  float* s_db1 = reinterpret_cast<float*>(sm + BwdSmem::db1);
  for (int e = t; e < kDoutMax * kH; e += kNt) s_dw1[e] = 0.0f;
  if (t < kDoutMax) s_db1[t] = 0.0f;
  // constant rows of IN^T: ones (hi) at kOnesRow, zeros above it
  for (int e = t; e < (kN2 - kOnesRow) * kTile; e += kNt) {
    const int r = kOnesRow + e / kTile, c = e % kTile;
    const uint32_t off = tc::kmajor_offset_strided(r, c, kLboP, kSboP);
    st_smem_u32(b3_hi, off, r == kOnesRow ? __float_as_uint(1.0f) : 0u);
    st_smem_u32(b3_lo, off, 0u);
  }
  if (warp == 0) {
    tc::tmem_alloc(slot, kBwdCols);
    tc::tmem_relinquish();
  }
  if (t == 0) {
    tc::mbar_init(bar, 3);   // one commit from each of the three pass threads
    tc::mbar_init(bar3, 1);
  }
  tc::fence_proxy_async_smem();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tbase = *slot;
  const uint32_t lb = (uint32_t)(32 * q);
  const uint32_t s_b1_hi = tc::smem_u32(sm + BwdSmem::b1_hi), s_b1_lo = tc::smem_u32(sm + BwdSmem::b1_lo);
  uint32_t phase = 0, phase3 = 0;
  bool ok = true, first = true, pending3 = false;

  const int64_t n = effective_n(a);
  const int64_t n_tiles = (n + kTile - 1) / kTile;
  // this point's coordinates and output gradient one tile ahead
  // (and, with the encoding cache, its member levels)
  const bool cached = a.enc_in != nullptr;
  float xn[3] = {0.0f, 0.0f, 0.0f}, gon[kOc], en[kFpm];
  load_point(a, (int64_t)blockIdx.x * kTile + pt, n, xn);
  load_grad<kOc>(a, (int64_t)blockIdx.x * kTile + pt, n, gon);
  if (cached) load_enc<M>(a, g, (int64_t)blockIdx.x * kTile + pt, n, en);
  for (int64_t tile = blockIdx.x; tile < n_tiles; tile += gridDim.x) {
    const int64_t p = tile * kTile + pt;
    const bool live = p < n;
    const float x[3] = {xn[0], xn[1], xn[2]};
    float go[kOc];
#pragma unroll
    for (int o = 0; o < kOc; ++o) go[o] = gon[o];
    float e[kFpm];
    if (cached) {
#pragma unroll
      for (int i = 0; i < kFpm; ++i) e[i] = en[i];
      load_enc<M>(a, g, (tile + gridDim.x) * kTile + pt, n, en);
    }
    load_point(a, (tile + gridDim.x) * kTile + pt, n, xn);
    load_grad<kOc>(a, (tile + gridDim.x) * kTile + pt, n, gon);
    // ---- input rows: TMEM (A of the first MMA) and IN^T (B of the third) ----
    bool ok3 = true;
    {
      if (!cached) encode_group<(M == 4), M>(a, g, live, x, e);
      st_split<kFpm>(tc::taddr(tbase, lb, kColInHi + kFpm * g), tc::taddr(tbase, lb, kColInLo + kFpm * g), e);
      // the previous tile's weight-gradient MMAs still read IN^T and dH^T:
      // wait for them only now, so they overlap its scatter and these gathers
      if (pending3) {
        ok3 = tc::mbar_wait_bounded(bar3, phase3);
        if (ok3) {
          phase3 ^= 1u;
          pending3 = false;
        }
      }
#pragma unroll
      for (int i = 0; i < kFpm; ++i) {
        uint32_t hi, lo;
        tc::tf32_split(e[i], hi, lo);
        const uint32_t off = tc::kmajor_offset_strided(kFpm * g + i, pt, kLboP, kSboP);
        st_smem_u32(b3_hi, off, hi);
        st_smem_u32(b3_lo, off, lo);
      }
      if (g == 0) {
        const float xv[8] = {x[0], x[1], x[2], 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
        st_split8(tc::taddr(tbase, lb, kColInHi + kXCol), tc::taddr(tbase, lb, kColInLo + kXCol), xv);
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          uint32_t hi, lo;
          tc::tf32_split(x[d], hi, lo);
          const uint32_t off = tc::kmajor_offset_strided(kXCol + d, pt, kLboP, kSboP);
          st_smem_u32(b3_hi, off, hi);
          st_smem_u32(b3_lo, off, lo);
        }
      }
    }
    tc::tmem_wait_st();
    tc::fence_proxy_async_smem();
    tc::fence_before_sync();
    if (!__syncthreads_and(ok3)) {
      ok = false;
      break;
    }
    if (t == 0 || t == 32 || t == 64) {
      const int part = t >> 5;
      tc::fence_after_sync();
      if (part == 0 || !a.one_pass) issue_mma1_part(tbase, s_b1_hi, s_b1_lo, part);
      tc::mma_commit(bar);
    }
    bool got = tc::mbar_wait_bounded(bar, phase);
    phase ^= 1u;
    if (!__syncthreads_and(got)) {
      ok = false;
      break;
    }
    tc::fence_after_sync();
    // ---- dH for this member's hidden units kHpm g .. kHpm g + kHpm - 1 ----
    {
      float h[kHpm];
      ld_parts<kHpm>(tbase, lb, kHpm * g, a.one_pass, h);
      float dh[kHpm], act[kHpm];
#pragma unroll
      for (int i = 0; i < kHpm; ++i) {
        const int j = kHpm * g + i;
        const float pre = h[i] + s_b0[j];
        float sg;
        softplus_fwd_grad_fast(pre, a.beta, inv_beta, a.thresh, act[i], sg);
        float da = 0.0f;
#pragma unroll
        for (int o = 0; o < kOc; ++o)
          if (o < oc) da = fmaf(go[o], s_w1[o * kH + j], da);
        dh[i] = live ? da * sg : 0.0f;
      }
      // dW1[o][j] += sum over the warp's points of g_o * act_j
#pragma unroll
      for (int o = 0; o < kOc; ++o) {
        if (o < oc) {
          float v[kHpm];
#pragma unroll
          for (int i = 0; i < kHpm; ++i) v[i] = live ? go[o] * act[i] : 0.0f;
          if (kHpm == 16) {
            const float r = warp_reduce_scatter16(v, lane);
            if ((lane & 1) == 0) atomicAdd(s_dw1 + o * kH + kHpm * g + (lane >> 1), r);
          } else {
            const float r = warp_reduce_scatter8(v, lane);
            if ((lane & 3) == 0) atomicAdd(s_dw1 + o * kH + kHpm * g + (lane >> 2), r);
          }
        }
      }
      if (g == 0) {
#pragma unroll
        for (int o = 0; o < kOc; ++o) {
          if (o < oc) {
            float v = go[o];
#pragma unroll
            for (int s = 16; s > 0; s >>= 1) v += __shfl_xor_sync(0xffffffffu, v, s);
            if (lane == 0) atomicAdd(s_db1 + o, v);
          }
        }
      }
      st_split<kHpm>(tc::taddr(tbase, lb, kColDhHi + kHpm * g), tc::taddr(tbase, lb, kColDhLo + kHpm * g), dh);
#pragma unroll
      for (int i = 0; i < kHpm; ++i) {
        uint32_t hi, lo;
        tc::tf32_split(dh[i], hi, lo);
        st_smem_u32(a3, tc::kmajor_offset_strided(kHpm * g + i, pt, kLboP, kSboP), hi);
        st_smem_u32(a3, tc::kmajor_offset_strided(kH + kHpm * g + i, pt, kLboP, kSboP), lo);
      }
    }
    tc::tmem_wait_st();
    tc::fence_proxy_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    // dIN (needed next): its three parts from three threads of different warps
    if (t == 0 || t == 32 || t == 64) {
      const int part = t >> 5;
      tc::fence_after_sync();
      if (part == 0 || !a.one_pass) issue_mma2_part(tbase, sm, part);
      tc::mma_commit(bar);
    }
    got = tc::mbar_wait_bounded(bar, phase);
    phase ^= 1u;
    if (!__syncthreads_and(got)) {
      ok = false;
      break;
    }
    tc::fence_after_sync();
    // the weight-gradient MMAs only now: issued beside dIN they were queued
    // ahead of it in the tensor pipe and delayed it; they run during the
    // scatter and are waited for before the next tile rewrites their operands
    if (t == 96) {
      issue_mma3(tbase, sm, first, a.one_pass);
      tc::mma_commit(bar3);
    }
    first = false;
    pending3 = true;
    // ---- dIN: table-gradient scatter for this member's levels, dL/dx ----
    {
      float din[kFpm];
      ld_parts<kFpm>(tbase, lb, kFpm * g, a.one_pass, din);
      float dxl[8];
      if (g == 0) ld_parts<8>(tbase, lb, kXCol, a.one_pass, dxl);
      float dx[3] = {0.0f, 0.0f, 0.0f};
      if (g == 0) {
        dx[0] = dxl[0];
        dx[1] = dxl[1];
        dx[2] = dxl[2];
      }
      float2* gt2 = reinterpret_cast<float2*>(a.grad_table);
#pragma unroll
      for (int i = 0; i < kLpm; ++i) {
        const int l = level_of<M>(g, i);
        if (l < a.active) {
          LevelCorners c;
          level_corners(a.g, l, x, c);
          const float d0 = live ? din[2 * i] : 0.0f, d1 = live ? din[2 * i + 1] : 0.0f;
          if (want_table) scatter_level(a.g, l, c, d0, d1, live, a.pair16, gt2, lane);
          if (want_x && live) {
#pragma unroll
            for (int k = 0; k < 8; ++k) {
              const float2 v = load_entry(a, c.idx[k]);
              const float gv = d0 * v.x + d1 * v.y;
#pragma unroll
              for (int d = 0; d < 3; ++d) dx[d] = fmaf(gv, corner_dw(c, k, d, a.g.scale[l]), dx[d]);
            }
          }
        }
      }
      if (want_x) {
#pragma unroll
        for (int d = 0; d < 3; ++d) s_dx[(g * kTile + pt) * 3 + d] = dx[d];
      }
    }
    // (the next tile's first barrier orders these TMEM reads before its MMAs)
    if (want_x) {
      __syncthreads();
      if (g == 0 && live) {
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          float s = 0.0f;
#pragma unroll
          for (int m = 0; m < M; ++m) s += s_dx[(m * kTile + pt) * 3 + d];
          a.grad_x[3 * p + d] = s;
        }
      }
      __syncthreads();
    }
  }
  if (!ok) (void)tc::mbar_wait_bounded(bar, phase ^ 1u);  // drain a timed-out first/second MMA
  if (pending3) ok = tc::mbar_wait_bounded(bar3, phase3) && ok;
  ok = __syncthreads_and(ok);
  if (!ok && t == 0 && a.status) atomicOr(a.status, SN_STATUS_TIMEOUT);
  tc::fence_after_sync();
  if (ok && !first) {
    // dW0 / db0: lanes 0..63 hold the dH_hi rows, 64..127 the dH_lo rows
    if (g == 0) {
      const int j = pt & (kH - 1);
#pragma unroll
      for (int c0 = 0; c0 < kN2; c0 += 16) {
        float v[16];
        tc::tmem_ld16(tc::taddr(tbase, lb, kColDw0 + c0), v);
        tc::tmem_wait_ld();
#pragma unroll
        for (int i = 0; i < 16; ++i) {
          const int c = c0 + i;
          if (c == kOnesRow) {
            if (a.grad_b0) atomicAdd(a.grad_b0 + j, v[i]);
          } else if (c < kK1 && a.grad_w0) {
            const int col = w0_col<M>(c, a.g.L);
            if (col >= 0 && v[i] != 0.0f) atomicAdd(a.grad_w0 + j * a.din + col, v[i]);
          }
        }
      }
    }
    // dW1 / db1 (block sums in shared memory)
    if (a.grad_w1)
      for (int e = t; e < oc * kH; e += kNt)
        if (s_dw1[e] != 0.0f) atomicAdd(a.grad_w1 + e, s_dw1[e]);
    if (a.grad_b1 && t < oc && s_db1[t] != 0.0f) atomicAdd(a.grad_b1 + t, s_db1[t]);
  }
  __syncthreads();
  tc::fence_after_sync();
  if (warp == 0) tc::tmem_dealloc(tbase, kBwdCols);
}


// ---------------------------------------------------------------------------
// second-order adjoint of d sdf / d x (SDFNetwork.gradient with create_graph)
// ---------------------------------------------------------------------------
// With IN = [e, x] and Z = [eta, gamma] in the permuted input order (eta = E
// gamma, E = d e / d x), h = IN W0^T + b0 and the sdf row w1 of W1:
//   H = IN W0^T, MU = Z W0^T                                  (first MMAs)
//   u = w1 softplus'(h), delta = MU w1 softplus''(h) + rho w1 softplus'(h)
//   DE = delta W0, VV = u W0 (encoding columns)               (second MMAs)
//   dT_{c,f} += DE_{l,f} w_c + VV_{l,f} (gamma . d w_c / d x)  (scatter)
//   dW0 += delta^T IN + u^T Z over the CTA's points           (third MMAs)
//   db0 += delta (row of ones in IN^T, zero in Z^T),
//   dw1 += MU softplus'(h) + rho softplus(h), db1 += rho.
// The third MMAs run in two halves through the same shared-memory operands
// (delta with IN^T, then u with Z^T), each waited for before its operands
// are overwritten.
//
// TMEM columns (512): H [0,64), later DE [0,32); MU [64,128), later VV
// [64,96); IN rows hi/lo [128,208) and Z rows hi/lo [208,288), and after the
// first MMAs delta hi/lo [128,256) and u hi/lo [256,384) (A of the second
// MMAs); dW0 accumulates in [384,432).
constexpr uint32_t kGColH = 0, kGColMu = 64, kGColInHi = 128, kGColInLo = 128 + kK1, kGColZHi = 208,
                   kGColZLo = 208 + kK1, kGColDHi = 128, kGColDLo = 192, kGColUHi = 256, kGColULo = 320,
                   kGColDw0 = 384;
constexpr int kGradMembers = 8;

struct GradSmem {
  static constexpr uint32_t b1_hi = 0, b1_lo = 10240, b2_hi = 20480, b2_lo = 32768, a3 = 45056,
                            b3_hi = a3 + 16 * kSboP, b3_lo = b3_hi + 6 * kSboP, w1 = b3_lo + 6 * kSboP,
                            b0 = w1 + kH * 4, dw1 = b0 + kH * 4, db1 = dw1 + kH * 4, bar = db1 + 16,
                            bar3 = bar + 8, slot = bar3 + 8, end = slot + 8;
};
constexpr size_t kGradSmemBytes = GradSmem::end;
static_assert(GradSmem::end <= 227 * 1024, "second-order shared memory map");

// Table-gradient contributions of the warp's points at one level with given
// per-corner values v[k] (the same lane grouping and atomics as scatter_level).
__device__ __forceinline__ void scatter_level_values(const GridDev& gd, int l, const LevelCorners& c,
                                                     const float2 v[8], bool live, bool pair16, float2* gt2,
                                                     int lane) {
  constexpr unsigned kAll = 0xffffffffu;
  unsigned rest = __ballot_sync(kAll, live);
  for (int it = 0; it < kMaxCellGroups && rest != 0u; ++it) {
    const int ld = __ffs(rest) - 1;
    const uint32_t c0 = __shfl_sync(kAll, c.cell[0], ld);
    const uint32_t c1 = __shfl_sync(kAll, c.cell[1], ld);
    const uint32_t c2 = __shfl_sync(kAll, c.cell[2], ld);
    const bool in = ((rest >> lane) & 1u) & (c.cell[0] == c0) & (c.cell[1] == c1) & (c.cell[2] == c2);
    const unsigned gm = __ballot_sync(kAll, in);
    if (__popc(gm) < kMinGroupLanes) break;  // the same decision on every lane
    float s[16];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      s[2 * k] = in ? v[k].x : 0.0f;
      s[2 * k + 1] = in ? v[k].y : 0.0f;
    }
    float a8[8], a4[4], a2[2];
    bool up = lane & 16;
#pragma unroll
    for (int i = 0; i < 8; ++i) a8[i] = (up ? s[i + 8] : s[i]) + __shfl_xor_sync(kAll, up ? s[i] : s[i + 8], 16);
    up = lane & 8;
#pragma unroll
    for (int i = 0; i < 4; ++i) a4[i] = (up ? a8[i + 4] : a8[i]) + __shfl_xor_sync(kAll, up ? a8[i] : a8[i + 4], 8);
    up = lane & 4;
#pragma unroll
    for (int i = 0; i < 2; ++i) a2[i] = (up ? a4[i + 2] : a4[i]) + __shfl_xor_sync(kAll, up ? a4[i] : a4[i + 2], 4);
#pragma unroll
    for (int sft = 2; sft > 0; sft >>= 1) {
      a2[0] += __shfl_xor_sync(kAll, a2[0], sft);
      a2[1] += __shfl_xor_sync(kAll, a2[1], sft);
    }
    const int k = lane >> 2;  // corner summed into lanes 4k..4k+3
    if ((lane & 3) == 0)
      atomicAdd(gt2 + corner_index(gd, l, c0 + (k & 1), c1 + ((k >> 1) & 1), c2 + (k >> 2)),
                make_float2(a2[0], a2[1]));
    rest &= ~gm;
  }
  if ((rest >> lane) & 1u) {
#pragma unroll
    for (int m = 0; m < 4; ++m) {
      const uint32_t i0 = c.idx[2 * m], i1 = c.idx[2 * m + 1];
      const float2 v0 = v[2 * m], v1 = v[2 * m + 1];
      if (pair16 && i1 == (i0 ^ 1u)) {
        const float4 q = (i0 & 1u) ? make_float4(v1.x, v1.y, v0.x, v0.y) : make_float4(v0.x, v0.y, v1.x, v1.y);
        atomicAdd(reinterpret_cast<float4*>(gt2 + (i0 & ~1u)), q);
      } else {
        atomicAdd(gt2 + i0, v0);
        atomicAdd(gt2 + i1, v1);
      }
    }
  }
}

// gamma . d w_k / d x for the 8 corners (trilinear weight derivatives).
__device__ __forceinline__ void corner_dir_derivs(const LevelCorners& c, float s, const float gam[3], float wg[8]) {
#pragma unroll
  for (int k = 0; k < 8; ++k)
    wg[k] = gam[0] * corner_dw(c, k, 0, s) + gam[1] * corner_dw(c, k, 1, s) + gam[2] * corner_dw(c, k, 2, s);
}

// Member g's levels of point x: encoding e and eta = E gamma.
template <int M>
__device__ __forceinline__ void encode_eta_group(const FieldArgs& a, int g, bool live, const float x[3],
                                                 const float gam[3], float e[2 * (16 / M)],
                                                 float eta[2 * (16 / M)]) {
  constexpr int kLpm = 16 / M;
#pragma unroll
  for (int i = 0; i < kLpm; ++i) {
    const int l = level_of<M>(g, i);
    float e0 = 0.0f, e1 = 0.0f, h0 = 0.0f, h1 = 0.0f;
    if (live && l < a.active) {
      LevelCorners c;
      level_corners(a.g, l, x, c);
      float2 tv[8];
#pragma unroll
      for (int k = 0; k < 8; ++k) tv[k] = load_entry(a, c.idx[k]);
      float wg[8];
      corner_dir_derivs(c, a.g.scale[l], gam, wg);
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        e0 = __fmaf_rn(c.w[k], tv[k].x, e0);
        e1 = __fmaf_rn(c.w[k], tv[k].y, e1);
        h0 = fmaf(wg[k], tv[k].x, h0);
        h1 = fmaf(wg[k], tv[k].y, h1);
      }
    }
    e[2 * i] = e0;
    e[2 * i + 1] = e1;
    eta[2 * i] = h0;
    eta[2 * i + 1] = h1;
  }
}

// A = [rows hi; rows lo] of a3 (M = 128, K = the tile's points) times B = the
// staged transposed inputs (N = 48) hi and lo, accumulated into dW0.
__device__ __forceinline__ void issue_grad_mma3(uint32_t tbase, const uint8_t* sm, bool fresh, bool one_pass) {
  const uint32_t idesc = tc::idesc_tf32(kTile, kN2);
  const uint32_t d3 = tc::taddr(tbase, 0, kGColDw0);
  const uint64_t da = tc::smem_desc(tc::smem_u32(sm + GradSmem::a3), kLboP, kSboP),
                 dbh = tc::smem_desc(tc::smem_u32(sm + GradSmem::b3_hi), kLboP, kSboP),
                 dbl = tc::smem_desc(tc::smem_u32(sm + GradSmem::b3_lo), kLboP, kSboP);
  for (int ks = 0; ks < kTile / 8; ++ks) {
    const uint64_t k0 = (2u * kLboP * ks) >> 4;
    tc::mma_ss(d3, da + k0, dbh + k0, idesc, (fresh && ks == 0) ? 0u : 1u);
    if (!one_pass) tc::mma_ss(d3, da + k0, dbl + k0, idesc, 1);
  }
}

// 3xTF32 D = A W^T with A in TMEM (hi at a_hi, lo at a_lo), W staged hi/lo.
__device__ __forceinline__ void mma_3x(uint32_t d, uint32_t a_hi, uint32_t a_lo, uint64_t w_hi, uint64_t w_lo,
                                       int ksteps, uint32_t idesc) {
  mma_chain(d, a_hi, w_hi, ksteps, idesc, true);
  mma_chain(d, a_lo, w_hi, ksteps, idesc, false);
  mma_chain(d, a_hi, w_lo, ksteps, idesc, false);
}

// Writes v (hi/lo) as row `row` (hi) and row + kH (lo) of a3, column pt.
__device__ __forceinline__ void st_a3(uint8_t* a3, int row, int pt, float v) {
  uint32_t hi, lo;
  tc::tf32_split(v, hi, lo);
  st_smem_u32(a3, tc::kmajor_offset_strided(row, pt, kLboP, kSboP), hi);
  st_smem_u32(a3, tc::kmajor_offset_strided(kH + row, pt, kLboP, kSboP), lo);
}
// Writes v (hi/lo) as row `row` of the transposed inputs, column pt.
__device__ __forceinline__ void st_b3(uint8_t* b3_hi, uint8_t* b3_lo, int row, int pt, float v) {
  uint32_t hi, lo;
  tc::tf32_split(v, hi, lo);
  const uint32_t off = tc::kmajor_offset_strided(row, pt, kLboP, kSboP);
  st_smem_u32(b3_hi, off, hi);
  st_smem_u32(b3_lo, off, lo);
}

template <int M>
__global__ void __launch_bounds__(128 * M, 1)
field_grad_bwd_tc_kernel(FieldArgs a, const float* __restrict__ gamma, const float* __restrict__ rho_in) {
  constexpr int kNt = 128 * M;
  constexpr int kLpm = 16 / M;
  constexpr int kFpm = 2 * kLpm;
  constexpr int kHpm = kH / M;
  static_assert(kHpm == 8 && kFpm == 4, "eight members per quadrant");
  extern __shared__ __align__(1024) uint8_t sm[];
  float* s_w1 = reinterpret_cast<float*>(sm + GradSmem::w1);
  float* s_b0 = reinterpret_cast<float*>(sm + GradSmem::b0);
  float* s_dw1 = reinterpret_cast<float*>(sm + GradSmem::dw1);
  float* s_db1 = reinterpret_cast<float*>(sm + GradSmem::db1);
  uint8_t* a3 = sm + GradSmem::a3;
  uint8_t* b3_hi = sm + GradSmem::b3_hi;
  uint8_t* b3_lo = sm + GradSmem::b3_lo;
  uint64_t* bar = reinterpret_cast<uint64_t*>(sm + GradSmem::bar);
  uint64_t* bar3 = reinterpret_cast<uint64_t*>(sm + GradSmem::bar3);
  uint32_t* slot = reinterpret_cast<uint32_t*>(sm + GradSmem::slot);
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  const int q = warp & 3, g = warp >> 2;
  const int pt = 32 * q + lane;
  const bool want_table = a.grad_table != nullptr;

  stage_w0<M>(a, sm + GradSmem::b1_hi, sm + GradSmem::b1_lo, sm + GradSmem::b2_hi, sm + GradSmem::b2_lo);
  if (t < kH) {
    s_w1[t] = a.w1[t];  // the sdf row of W1
    s_b0[t] = a.b0[t];
    s_dw1[t] = 0.0f;
  }
  if (t == 0) s_db1[0] = 0.0f;
  // constant rows of the transposed inputs: zeros above the ones row (row
  // kOnesRow is written per tile: one for IN^T, zero for Z^T)
  for (int e = t; e < (kN2 - kOnesRow - 1) * kTile; e += kNt) {
    const int r = kOnesRow + 1 + e / kTile, c = e % kTile;
    const uint32_t off = tc::kmajor_offset_strided(r, c, kLboP, kSboP);
    st_smem_u32(b3_hi, off, 0u);
    st_smem_u32(b3_lo, off, 0u);
  }
  if (warp == 0) {
    tc::tmem_alloc(slot, kBwdCols);
    tc::tmem_relinquish();
  }
  if (t == 0) {
    tc::mbar_init(bar, 1);
    tc::mbar_init(bar3, 1);
  }
  tc::fence_proxy_async_smem();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tbase = *slot;
  const uint32_t lb = (uint32_t)(32 * q);
  const uint32_t idesc1 = tc::idesc_tf32(kTile, kH), idesc2 = tc::idesc_tf32(kTile, 32);
  const uint32_t sbo1 = (kK1 / 4) * 128u, sbo2 = (kH / 4) * 128u;
  const uint64_t w1_hi = tc::smem_desc(tc::smem_u32(sm + GradSmem::b1_hi), 128u, sbo1),
                 w1_lo = tc::smem_desc(tc::smem_u32(sm + GradSmem::b1_lo), 128u, sbo1),
                 w2_hi = tc::smem_desc(tc::smem_u32(sm + GradSmem::b2_hi), 128u, sbo2),
                 w2_lo = tc::smem_desc(tc::smem_u32(sm + GradSmem::b2_lo), 128u, sbo2);
  const float inv_beta = 1.0f / a.beta;
  uint32_t phase = 0, phase3 = 0;
  bool ok = true, first = true, pending3 = false;

  const int64_t n = effective_n(a);
  const int64_t n_tiles = (n + kTile - 1) / kTile;
  float xn[3], gn[3], rn = 0.0f;
  auto load_next = [&](int64_t p) {
    load_point(a, p, n, xn);
    const bool in = p < n;
#pragma unroll
    for (int d = 0; d < 3; ++d) gn[d] = in ? gamma[3 * p + d] : 0.0f;
    rn = (in && rho_in) ? rho_in[p] : 0.0f;
  };
  load_next((int64_t)blockIdx.x * kTile + pt);
  for (int64_t tile = blockIdx.x; tile < n_tiles; tile += gridDim.x) {
    const int64_t p = tile * kTile + pt;
    const bool live = p < n;
    const float x[3] = {xn[0], xn[1], xn[2]};
    const float gam[3] = {gn[0], gn[1], gn[2]};
    const float rho = rn;
    load_next((tile + gridDim.x) * kTile + pt);
    // ---- IN and Z rows (TMEM, A of the first MMAs), IN^T (B of the third) ----
    float eta[kFpm];
    bool ok3 = true;
    {
      float e[kFpm];
      encode_eta_group<M>(a, g, live, x, gam, e, eta);
      st_split<kFpm>(tc::taddr(tbase, lb, kGColInHi + kFpm * g), tc::taddr(tbase, lb, kGColInLo + kFpm * g), e);
      st_split<kFpm>(tc::taddr(tbase, lb, kGColZHi + kFpm * g), tc::taddr(tbase, lb, kGColZLo + kFpm * g), eta);
      if (g == 0) {
        const float xv[8] = {x[0], x[1], x[2], 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
        const float gv[8] = {gam[0], gam[1], gam[2], 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
        st_split8(tc::taddr(tbase, lb, kGColInHi + kXCol), tc::taddr(tbase, lb, kGColInLo + kXCol), xv);
        st_split8(tc::taddr(tbase, lb, kGColZHi + kXCol), tc::taddr(tbase, lb, kGColZLo + kXCol), gv);
      }
      // the previous tile's u^T Z MMAs still read a3 and the transposed inputs
      if (pending3) {
        ok3 = tc::mbar_wait_bounded(bar3, phase3);
        if (ok3) {
          phase3 ^= 1u;
          pending3 = false;
        }
      }
#pragma unroll
      for (int i = 0; i < kFpm; ++i) st_b3(b3_hi, b3_lo, kFpm * g + i, pt, e[i]);
      if (g == 0) {
#pragma unroll
        for (int d = 0; d < 3; ++d) st_b3(b3_hi, b3_lo, kXCol + d, pt, x[d]);
        const uint32_t off = tc::kmajor_offset_strided(kOnesRow, pt, kLboP, kSboP);
        st_smem_u32(b3_hi, off, __float_as_uint(1.0f));
        st_smem_u32(b3_lo, off, 0u);
      }
    }
    tc::tmem_wait_st();
    tc::fence_proxy_async_smem();
    tc::fence_before_sync();
    if (!__syncthreads_and(ok3)) {
      ok = false;
      break;
    }
    if (t == 0) {  // H = IN W0^T, MU = Z W0^T (M=128, N=64, K=40)
      tc::fence_after_sync();
      mma_3x(tc::taddr(tbase, 0, kGColH), tc::taddr(tbase, 0, kGColInHi), tc::taddr(tbase, 0, kGColInLo), w1_hi,
             w1_lo, kK1 / 8, idesc1);
      mma_3x(tc::taddr(tbase, 0, kGColMu), tc::taddr(tbase, 0, kGColZHi), tc::taddr(tbase, 0, kGColZLo), w1_hi,
             w1_lo, kK1 / 8, idesc1);
      tc::mma_commit(bar);
    }
    bool got = tc::mbar_wait_bounded(bar, phase);
    phase ^= 1u;
    if (!__syncthreads_and(got)) {
      ok = false;
      break;
    }
    tc::fence_after_sync();
    // ---- u, delta, dw1 for this member's hidden units 8g .. 8g + 7 ----
    float u[kHpm];
    {
      float h[kHpm], mu[kHpm];
      tc::tmem_ld8(tc::taddr(tbase, lb, kGColH + kHpm * g), h);
      tc::tmem_ld8(tc::taddr(tbase, lb, kGColMu + kHpm * g), mu);
      tc::tmem_wait_ld();
      float dl[kHpm], v[kHpm];
#pragma unroll
      for (int i = 0; i < kHpm; ++i) {
        const int j = kHpm * g + i;
        const float pre = h[i] + s_b0[j];
        float act, s1;
        softplus_fwd_grad_fast(pre, a.beta, inv_beta, a.thresh, act, s1);
        const float s2 = pre * a.beta > a.thresh ? 0.0f : a.beta * s1 * (1.0f - s1);
        const float w1 = s_w1[j];
        u[i] = live ? w1 * s1 : 0.0f;
        dl[i] = live ? fmaf(mu[i] * w1, s2, rho * w1 * s1) : 0.0f;
        v[i] = live ? fmaf(mu[i], s1, rho * act) : 0.0f;
      }
      const float r = warp_reduce_scatter8(v, lane);
      if ((lane & 3) == 0) atomicAdd(s_dw1 + kHpm * g + (lane >> 2), r);
      if (g == 0) {
        float rs = live ? rho : 0.0f;
#pragma unroll
        for (int s = 16; s > 0; s >>= 1) rs += __shfl_xor_sync(0xffffffffu, rs, s);
        if (lane == 0) atomicAdd(s_db1, rs);
      }
      st_split8(tc::taddr(tbase, lb, kGColDHi + kHpm * g), tc::taddr(tbase, lb, kGColDLo + kHpm * g), dl);
      st_split8(tc::taddr(tbase, lb, kGColUHi + kHpm * g), tc::taddr(tbase, lb, kGColULo + kHpm * g), u);
#pragma unroll
      for (int i = 0; i < kHpm; ++i) st_a3(a3, kHpm * g + i, pt, dl[i]);
    }
    tc::tmem_wait_st();
    tc::fence_proxy_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    if (t == 0) {  // DE = delta W0, VV = u W0 (M=128, N=32 encoding columns, K=64)
      tc::fence_after_sync();
      mma_3x(tc::taddr(tbase, 0, kGColH), tc::taddr(tbase, 0, kGColDHi), tc::taddr(tbase, 0, kGColDLo), w2_hi,
             w2_lo, kH / 8, idesc2);
      mma_3x(tc::taddr(tbase, 0, kGColMu), tc::taddr(tbase, 0, kGColUHi), tc::taddr(tbase, 0, kGColULo), w2_hi,
             w2_lo, kH / 8, idesc2);
      tc::mma_commit(bar);
    }
    got = tc::mbar_wait_bounded(bar, phase);
    phase ^= 1u;
    if (!__syncthreads_and(got)) {
      ok = false;
      break;
    }
    tc::fence_after_sync();
    if (t == 32) {  // dW0 += delta^T IN (db0 from the ones row), behind the second MMAs
      issue_grad_mma3(tbase, sm, first, false);
      tc::mma_commit(bar3);
    }
    first = false;
    pending3 = true;
    // ---- table gradient for this member's levels ----
    if (want_table) {
      float de[kFpm], vv[kFpm];
      tc::tmem_ld4(tc::taddr(tbase, lb, kGColH + kFpm * g), de);
      tc::tmem_ld4(tc::taddr(tbase, lb, kGColMu + kFpm * g), vv);
      tc::tmem_wait_ld();
      float2* gt2 = reinterpret_cast<float2*>(a.grad_table);
#pragma unroll
      for (int i = 0; i < kLpm; ++i) {
        const int l = level_of<M>(g, i);
        if (l < a.active) {
          LevelCorners c;
          level_corners(a.g, l, x, c);
          float wg[8];
          corner_dir_derivs(c, a.g.scale[l], gam, wg);
          float2 v[8];
#pragma unroll
          for (int k = 0; k < 8; ++k)
            v[k] = live ? make_float2(fmaf(de[2 * i], c.w[k], vv[2 * i] * wg[k]),
                                      fmaf(de[2 * i + 1], c.w[k], vv[2 * i + 1] * wg[k]))
                        : make_float2(0.0f, 0.0f);
          scatter_level_values(a.g, l, c, v, live, a.pair16, gt2, lane);
        }
      }
    }
    // ---- dW0 += u^T Z: wait for delta^T IN, then reuse its operands ----
    ok3 = tc::mbar_wait_bounded(bar3, phase3);
    if (ok3) {
      phase3 ^= 1u;
      pending3 = false;
    }
    if (ok3) {
#pragma unroll
      for (int i = 0; i < kHpm; ++i) st_a3(a3, kHpm * g + i, pt, u[i]);
#pragma unroll
      for (int i = 0; i < kFpm; ++i) st_b3(b3_hi, b3_lo, kFpm * g + i, pt, eta[i]);
      if (g == 0) {
#pragma unroll
        for (int d = 0; d < 3; ++d) st_b3(b3_hi, b3_lo, kXCol + d, pt, gam[d]);
        const uint32_t off = tc::kmajor_offset_strided(kOnesRow, pt, kLboP, kSboP);
        st_smem_u32(b3_hi, off, 0u);
        st_smem_u32(b3_lo, off, 0u);
      }
    }
    tc::fence_proxy_async_smem();
    tc::fence_before_sync();
    if (!__syncthreads_and(ok3)) {
      ok = false;
      break;
    }
    if (t == 32) {
      tc::fence_after_sync();
      issue_grad_mma3(tbase, sm, false, false);
      tc::mma_commit(bar3);
    }
    pending3 = true;
  }
  if (!ok) (void)tc::mbar_wait_bounded(bar, phase ^ 1u);  // drain a timed-out first/second MMA
  if (pending3) ok = tc::mbar_wait_bounded(bar3, phase3) && ok;
  ok = __syncthreads_and(ok);
  if (!ok && t == 0 && a.status) atomicOr(a.status, SN_STATUS_TIMEOUT);
  tc::fence_after_sync();
  if (ok && !first) {
    // dW0 / db0: lanes 0..63 hold the hi rows, 64..127 the lo rows
    if (g == 0) {
      const int j = pt & (kH - 1);
#pragma unroll
      for (int c0 = 0; c0 < kN2; c0 += 16) {
        float v[16];
        tc::tmem_ld16(tc::taddr(tbase, lb, kGColDw0 + c0), v);
        tc::tmem_wait_ld();
#pragma unroll
        for (int i = 0; i < 16; ++i) {
          const int c = c0 + i;
          if (c == kOnesRow) {
            if (a.grad_b0) atomicAdd(a.grad_b0 + j, v[i]);
          } else if (c < kK1 && a.grad_w0) {
            const int col = w0_col<M>(c, a.g.L);
            if (col >= 0 && v[i] != 0.0f) atomicAdd(a.grad_w0 + j * a.din + col, v[i]);
          }
        }
      }
    }
    if (a.grad_w1 && t < kH && s_dw1[t] != 0.0f) atomicAdd(a.grad_w1 + t, s_dw1[t]);
    if (a.grad_b1 && t == 0 && s_db1[0] != 0.0f) atomicAdd(a.grad_b1, s_db1[0]);
  }
  __syncthreads();
  tc::fence_after_sync();
  if (warp == 0) tc::tmem_dealloc(tbase, kBwdCols);
}

// ---------------------------------------------------------------------------
// d sdf / d x (SDFNetwork.gradient): sdf and grad = W0x^T u + E^T (W0e^T u)
// ---------------------------------------------------------------------------
// H = IN W0^T (first MMA), u = w1 softplus'(H + b0), sdf = w1 . softplus + b1,
// V = u W0 (second MMA, all 48 input columns), and per point
// grad = V_x + sum over levels and corners of (V_{l,0} T_{c,0} + V_{l,1} T_{c,1}) d w_c / d x.
// TMEM columns (256, two CTAs per SM): H [0,64); IN rows hi/lo [64,144), after
// the first MMA u hi/lo [64,192) (A of the second); V [192,240).
constexpr uint32_t kFColH = 0, kFColInHi = 64, kFColInLo = 64 + kK1, kFColUHi = 64, kFColULo = 128,
                   kFColV = 192;
constexpr int kGradFwdMembers = 4;

template <int M>
struct GradFwdSmem {
  static constexpr uint32_t b1_hi = 0, b1_lo = 10240, b2_hi = 20480, b2_lo = 32768, w1 = 45056, b0 = w1 + kH * 4,
                            part = b0 + kH * 4, bar = part + M * kTile * 16, slot = bar + 8, end = slot + 8;
  // more than 228/3 KB, so at most two CTAs (2 x 256 TMEM columns) per SM
  static constexpr size_t bytes = 80 * 1024;
};
static_assert(GradFwdSmem<kGradFwdMembers>::end <= GradFwdSmem<kGradFwdMembers>::bytes, "gradient shared memory map");

template <int M>
__global__ void __launch_bounds__(128 * M, 2)
field_grad_fwd_tc_kernel(FieldArgs a, float* __restrict__ out_sdf, float* __restrict__ out_grad) {
  constexpr int kLpm = 16 / M;
  constexpr int kFpm = 2 * kLpm;
  constexpr int kHpm = kH / M;
  static_assert(kFpm == 8 && kHpm == 16, "four members per quadrant");
  using Sm = GradFwdSmem<M>;
  extern __shared__ __align__(1024) uint8_t sm[];
  float* s_w1 = reinterpret_cast<float*>(sm + Sm::w1);
  float* s_b0 = reinterpret_cast<float*>(sm + Sm::b0);
  float4* s_part = reinterpret_cast<float4*>(sm + Sm::part);
  uint64_t* bar = reinterpret_cast<uint64_t*>(sm + Sm::bar);
  uint32_t* slot = reinterpret_cast<uint32_t*>(sm + Sm::slot);
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  const int q = warp & 3, g = warp >> 2;
  const int pt = 32 * q + lane;

  stage_w0<M>(a, sm + Sm::b1_hi, sm + Sm::b1_lo, sm + Sm::b2_hi, sm + Sm::b2_lo);
  if (t < kH) {
    s_w1[t] = a.w1[t];  // the sdf row of W1
    s_b0[t] = a.b0[t];
  }
  const float b1v = a.b1[0];
  if (warp == 0) {
    tc::tmem_alloc(slot, kCols);
    tc::tmem_relinquish();
  }
  if (t == 0) tc::mbar_init(bar, 1);
  tc::fence_proxy_async_smem();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tbase = *slot;
  const uint32_t lb = (uint32_t)(32 * q);
  const uint32_t idesc1 = tc::idesc_tf32(kTile, kH), idesc2 = tc::idesc_tf32(kTile, kN2);
  const uint32_t sbo1 = (kK1 / 4) * 128u, sbo2 = (kH / 4) * 128u;
  const uint64_t w1_hi = tc::smem_desc(tc::smem_u32(sm + Sm::b1_hi), 128u, sbo1),
                 w1_lo = tc::smem_desc(tc::smem_u32(sm + Sm::b1_lo), 128u, sbo1),
                 w2_hi = tc::smem_desc(tc::smem_u32(sm + Sm::b2_hi), 128u, sbo2),
                 w2_lo = tc::smem_desc(tc::smem_u32(sm + Sm::b2_lo), 128u, sbo2);
  const float inv_beta = 1.0f / a.beta;
  uint32_t phase = 0;
  bool ok = true;

  const int64_t n = effective_n(a);
  const int64_t n_tiles = (n + kTile - 1) / kTile;
  float xn[3];
  load_point(a, (int64_t)blockIdx.x * kTile + pt, n, xn);
  for (int64_t tile = blockIdx.x; tile < n_tiles; tile += gridDim.x) {
    const int64_t p = tile * kTile + pt;
    const bool live = p < n;
    const float x[3] = {xn[0], xn[1], xn[2]};
    load_point(a, (tile + gridDim.x) * kTile + pt, n, xn);
    {
      float e[kFpm];
      encode_group<false, M>(a, g, live, x, e);
      st_split<kFpm>(tc::taddr(tbase, lb, kFColInHi + kFpm * g), tc::taddr(tbase, lb, kFColInLo + kFpm * g), e);
      if (g == 0) {
        const float xv[8] = {x[0], x[1], x[2], 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
        st_split8(tc::taddr(tbase, lb, kFColInHi + kXCol), tc::taddr(tbase, lb, kFColInLo + kXCol), xv);
      }
    }
    tc::tmem_wait_st();
    tc::fence_before_sync();
    __syncthreads();
    if (t == 0) {  // H = IN W0^T (M=128, N=64, K=40)
      tc::fence_after_sync();
      mma_3x(tc::taddr(tbase, 0, kFColH), tc::taddr(tbase, 0, kFColInHi), tc::taddr(tbase, 0, kFColInLo), w1_hi,
             w1_lo, kK1 / 8, idesc1);
      tc::mma_commit(bar);
    }
    bool got = tc::mbar_wait_bounded(bar, phase);
    phase ^= 1u;
    if (!__syncthreads_and(got)) {
      ok = false;
      break;
    }
    tc::fence_after_sync();
    // u and the sdf partial for hidden units kHpm g .. kHpm g + kHpm - 1
    float sdf_part = 0.0f;
    {
      float h[kHpm], u[kHpm];
      tc::tmem_ld16(tc::taddr(tbase, lb, kFColH + kHpm * g), h);
      tc::tmem_wait_ld();
#pragma unroll
      for (int i = 0; i < kHpm; ++i) {
        const int j = kHpm * g + i;
        float act, s1;
        softplus_fwd_grad_fast(h[i] + s_b0[j], a.beta, inv_beta, a.thresh, act, s1);
        u[i] = s_w1[j] * s1;
        sdf_part = fmaf(s_w1[j], act, sdf_part);
      }
      st_split<kHpm>(tc::taddr(tbase, lb, kFColUHi + kHpm * g), tc::taddr(tbase, lb, kFColULo + kHpm * g), u);
    }
    tc::tmem_wait_st();
    tc::fence_before_sync();
    __syncthreads();
    if (t == 0) {  // V = u W0 (M=128, N=48, K=64)
      tc::fence_after_sync();
      mma_3x(tc::taddr(tbase, 0, kFColV), tc::taddr(tbase, 0, kFColUHi), tc::taddr(tbase, 0, kFColULo), w2_hi,
             w2_lo, kH / 8, idesc2);
      tc::mma_commit(bar);
    }
    got = tc::mbar_wait_bounded(bar, phase);
    phase ^= 1u;
    if (!__syncthreads_and(got)) {
      ok = false;
      break;
    }
    tc::fence_after_sync();
    // gradient partial: this member's levels (+ the linear x part for member 0)
    {
      float v[kFpm], vx[8];
      tc::tmem_ld8(tc::taddr(tbase, lb, kFColV + kFpm * g), v);
      tc::tmem_ld8(tc::taddr(tbase, lb, kFColV + kXCol), vx);
      tc::tmem_wait_ld();
      float gx[3] = {0.0f, 0.0f, 0.0f};
      if (g == 0) {
        gx[0] = vx[0];
        gx[1] = vx[1];
        gx[2] = vx[2];
      }
      if (live) {
#pragma unroll
        for (int i = 0; i < kLpm; ++i) {
          const int l = level_of<M>(g, i);
          if (l < a.active) {
            LevelCorners c;
            level_corners(a.g, l, x, c);
            float2 tv[8];
#pragma unroll
            for (int k = 0; k < 8; ++k) tv[k] = load_entry(a, c.idx[k]);
            const float s = a.g.scale[l];
#pragma unroll
            for (int k = 0; k < 8; ++k) {
              const float gk = v[2 * i] * tv[k].x + v[2 * i + 1] * tv[k].y;
#pragma unroll
              for (int d = 0; d < 3; ++d) gx[d] = fmaf(gk, corner_dw(c, k, d, s), gx[d]);
            }
          }
        }
      }
      s_part[g * kTile + pt] = make_float4(sdf_part, gx[0], gx[1], gx[2]);
    }
    __syncthreads();
    // (the next tile writes s_part only after two more barriers)
    if (g == 0 && live) {
      float4 s = s_part[pt];
#pragma unroll
      for (int m = 1; m < M; ++m) {
        const float4 o = s_part[m * kTile + pt];
        s.x += o.x;
        s.y += o.y;
        s.z += o.z;
        s.w += o.w;
      }
      if (out_sdf) out_sdf[p] = s.x + b1v;
      out_grad[3 * p + 0] = s.y;
      out_grad[3 * p + 1] = s.z;
      out_grad[3 * p + 2] = s.w;
    }
  }
  if (!ok) {
    if (t == 0 && a.status) atomicOr(a.status, SN_STATUS_TIMEOUT);
    (void)tc::mbar_wait_bounded(bar, phase ^ 1u);
  }
  __syncthreads();
  tc::fence_after_sync();
  if (warp == 0) tc::tmem_dealloc(tbase, kCols);
}

// The bounded mbarrier wait of the tensor-core kernels, on an mbarrier that
// nothing arrives at, for `polls` polls (0: the kernels' own limit): the wait
// gives up and the timeout is reported through the status word, as a kernel
// whose MMAs never completed reports it.  The kernel then returns normally.
__global__ void bounded_wait_selftest_kernel(int32_t* status, uint32_t polls) {
  __shared__ uint64_t bar;
  if (threadIdx.x == 0) tc::mbar_init(&bar, 1);
  __syncthreads();
  const bool got = tc::mbar_wait_polls(&bar, 0, polls ? polls : tc::kWaitLimit);
  if (!got && threadIdx.x == 0) atomicOr(status, SN_STATUS_TIMEOUT);
}

}  // namespace

int bounded_wait_selftest(int32_t* status, uint32_t polls, cudaStream_t st) {
  bounded_wait_selftest_kernel<<<1, 32, 0, st>>>(status, polls);
  return check_launch("bounded_wait_selftest");
}
uint32_t bounded_wait_limit() { return tc::kWaitLimit; }

// Launchers used by sn_field_fwd / sn_field_bwd (field.cu).
int field_fwd_tc_segments(const FieldArgs* segs, int n_seg, cudaStream_t st) {
  constexpr int M = kFwdMembers;
  constexpr size_t smem = FwdSmem<M>::bytes;
  SN_REQUIRE(n_seg >= 1 && n_seg <= kMaxSegments, "field_fwd: %d segments (1..%d)", n_seg, kMaxSegments);
  const bool one = segs[0].out_cols == 1;
  FieldSegments fs;
  memset(&fs, 0, sizeof(fs));
  fs.n = n_seg;
  int64_t max_tiles = 0;
  for (int i = 0; i < n_seg; ++i) {
    SN_REQUIRE((segs[i].out_cols == 1) == one, "field_fwd: segments mix one and several output columns");
    fs.seg[i] = segs[i];
    const int64_t tiles = (segs[i].cap + kTile - 1) / kTile;
    if (tiles > max_tiles) max_tiles = tiles;
  }
  const void* fn = one ? reinterpret_cast<const void*>(field_fwd_tc_kernel<true, M>)
                       : reinterpret_cast<const void*>(field_fwd_tc_kernel<false, M>);
  SN_TRY(ensure_smem_limit(fn, smem, "field_fwd"));
  const int64_t cap = (M == 4 ? 2LL : 1LL) * num_sms();
  const unsigned grid = (unsigned)(max_tiles < cap ? (max_tiles > 0 ? max_tiles : 1) : cap);
  if (one)
    field_fwd_tc_kernel<true, M><<<grid, 128 * M, smem, st>>>(fs);
  else
    field_fwd_tc_kernel<false, M><<<grid, 128 * M, smem, st>>>(fs);
  return check_launch("field_fwd");
}

int field_fwd_tc(const FieldArgs& a, cudaStream_t st) { return field_fwd_tc_segments(&a, 1, st); }

int field_grad_fwd_tc(const FieldArgs& a, float* sdf, float* grad, cudaStream_t st) {
  constexpr int M = kGradFwdMembers;
  constexpr size_t smem = GradFwdSmem<M>::bytes;
  const void* fn = reinterpret_cast<const void*>(field_grad_fwd_tc_kernel<M>);
  SN_TRY(ensure_smem_limit(fn, smem, "field_grad_fwd"));
  const int64_t n_tiles = (a.cap + kTile - 1) / kTile;
  const int64_t cap = 2LL * num_sms();
  const unsigned grid = (unsigned)(n_tiles < cap ? n_tiles : cap);
  field_grad_fwd_tc_kernel<M><<<grid, 128 * M, smem, st>>>(a, sdf, grad);
  return check_launch("field_grad_fwd");
}

int field_grad_bwd_tc(const FieldArgs& a, const float* gamma, const float* rho, cudaStream_t st) {
  constexpr int M = kGradMembers;
  const void* fn = reinterpret_cast<const void*>(field_grad_bwd_tc_kernel<M>);
  SN_TRY(ensure_smem_limit(fn, kGradSmemBytes, "field_grad_bwd"));
  const int64_t n_tiles = (a.cap + kTile - 1) / kTile;
  const int64_t cap = num_sms();
  const unsigned grid = (unsigned)(n_tiles < cap ? n_tiles : cap);
  field_grad_bwd_tc_kernel<M><<<grid, 128 * M, kGradSmemBytes, st>>>(a, gamma, rho);
  return check_launch("field_grad_bwd");
}

int field_bwd_tc(const FieldArgs& a, cudaStream_t st) {
  constexpr int M = kBwdMembers;
  const void* fn = a.out_cols == 1 ? reinterpret_cast<const void*>(field_bwd_tc_kernel<true, M>)
                                   : reinterpret_cast<const void*>(field_bwd_tc_kernel<false, M>);
  SN_TRY(ensure_smem_limit(fn, kBwdSmemBytes, "field_bwd"));
  const int64_t n_tiles = (a.cap + kTile - 1) / kTile;
  const int64_t cap = num_sms();
  const unsigned grid = (unsigned)(n_tiles < cap ? n_tiles : cap);
  if (a.out_cols == 1)
    field_bwd_tc_kernel<true, M><<<grid, 128 * M, kBwdSmemBytes, st>>>(a);
  else
    field_bwd_tc_kernel<false, M><<<grid, 128 * M, kBwdSmemBytes, st>>>(a);
  return check_launch("field_bwd");
}

}  // namespace sn
