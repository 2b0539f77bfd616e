// SDF field: multi-resolution hash-grid encoding + one-hidden-layer MLP.
//
// Encoding: Instant-NGP multiresolution hash encoding (Mueller et al. 2022)
// with tiny-cuda-nn's conventions as used by SuperNormal's
// `tcnn.Encoding(3, {otype: HashGrid, ...})` (models/fields.py:26,78):
//   scale_l = 2^(l*log2(per_level_scale)) * base_resolution - 1
//   resolution_l = ceil(scale_l) + 1
//   pos = fma(scale_l, x, 0.5); cell = floor(pos); frac = pos - cell
//   dense index (cell_x + cell_y*res + cell_z*res^2) when res^3 fits the
//   level, else the XOR prime hash (1, 2654435761, 805459861); both taken
//   modulo the level size in uint32 arithmetic (so SuperNormal's [-1,1]
//   inputs wrap exactly as they do there), trilinear weights over the 8
//   corners in corner order 0..7.
// Table layout: entry-major, F features contiguous per entry, levels
// concatenated at offsets[l] (the tcnn `params` layout).
//
// MLP: SDFNetwork with n_layers = 1 and input_concat
// (models/fields.py:76-99): in = [x, enc], h = W0 in + b0,
// a = softplus_beta(h), y = W1 a + b1, with W0/W1 the weight-normed
// matrices.  Levels at or beyond `active_levels` are the encoding features
// SuperNormal masks to zero (bandwidth, models/fields.py:81-83); their
// gather and gradient are skipped, which is exact because the mask
// multiplies them by zero.
#include "field_common.cuh"

#include <math.h>
#include <string.h>

namespace sn {

// --- standalone encoding (tcnn.Encoding forward / backward) -----------------
__global__ void hashgrid_fwd_kernel(int64_t n, const float* __restrict__ x,
                                    const float* __restrict__ table, GridDev g, int active,
                                    float* __restrict__ out) {
  const int64_t total = n * g.L;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p = t / g.L;
    const int l = (int)(t - p * g.L);
    float e0 = 0.0f, e1 = 0.0f;
    if (l < active) {
      const float xp[3] = {x[3 * p], x[3 * p + 1], x[3 * p + 2]};
      encode_level(table, g, l, xp, e0, e1);
    }
    reinterpret_cast<float2*>(out)[t] = make_float2(e0, e1);
  }
}

__global__ void hashgrid_bwd_kernel(int64_t n, const float* __restrict__ x,
                                    const float* __restrict__ gout, GridDev g, int active,
                                    float* __restrict__ gtable) {
  const int64_t total = n * g.L;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p = t / g.L;
    const int l = (int)(t - p * g.L);
    if (l >= active) continue;
    const float xp[3] = {x[3 * p], x[3 * p + 1], x[3 * p + 2]};
    const float2 go = reinterpret_cast<const float2*>(gout)[t];
    LevelCorners c;
    level_corners(g, l, xp, c);
    float2* gt2 = reinterpret_cast<float2*>(gtable);
#pragma unroll
    for (int k = 0; k < 8; ++k) atomicAdd(gt2 + c.idx[k], make_float2(c.w[k] * go.x, c.w[k] * go.y));
  }
}

// --- weight normalisation (torch.nn.utils.weight_norm, dim=0) ----------------
__global__ void weightnorm_fwd_kernel(int rows, int cols, const float* __restrict__ v,
                                      const float* __restrict__ gain, float* __restrict__ w,
                                      float* __restrict__ norms) {
  const int r = blockIdx.x;
  if (r >= rows) return;
  float s = 0.0f;
  for (int c = threadIdx.x; c < cols; c += 32) s = fmaf(v[r * cols + c], v[r * cols + c], s);
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  const float nrm = sqrtf(s);
  const float k = gain[r] / nrm;
  for (int c = threadIdx.x; c < cols; c += 32) w[r * cols + c] = v[r * cols + c] * k;
  if (threadIdx.x == 0 && norms) norms[r] = nrm;
}

__global__ void weightnorm_bwd_kernel(int rows, int cols, const float* __restrict__ v,
                                      const float* __restrict__ gain,
                                      const float* __restrict__ norms,
                                      const float* __restrict__ gw, float* __restrict__ gv,
                                      float* __restrict__ gg) {
  const int r = blockIdx.x;
  if (r >= rows) return;
  float s = 0.0f;
  for (int c = threadIdx.x; c < cols; c += 32) s = fmaf(gw[r * cols + c], v[r * cols + c], s);
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  const float nrm = norms[r];
  const float dg = s / nrm;
  const float k = gain[r] / nrm;
  const float m = dg / nrm;
  for (int c = threadIdx.x; c < cols; c += 32)
    gv[r * cols + c] = k * (gw[r * cols + c] - v[r * cols + c] * m);
  if (threadIdx.x == 0) gg[r] = dg;
}

int make_grid_dev(const sn_grid_desc* d, GridDev& g) {
  SN_REQUIRE(d != nullptr, "grid descriptor is null");
  SN_REQUIRE(d->n_features == kF, "only %d features per level are supported (got %d)", kF,
             d->n_features);
  if (d->n_levels < 1 || d->n_levels > kMaxL) {
    set_error("1..%d levels supported (got %d)", kMaxL, d->n_levels);
    return SN_ERR_UNSUPPORTED;
  }
  memset(&g, 0, sizeof(g));
  g.L = d->n_levels;
  for (int l = 0; l < g.L; ++l) {
    const uint32_t size = d->offsets[l + 1] - d->offsets[l];
    SN_REQUIRE(size > 0, "empty level %d", l);
    g.offset[l] = d->offsets[l];
    g.res[l] = d->resolutions[l];
    g.size[l] = size;
    g.scale[l] = d->scales[l];
    const uint64_t r = d->resolutions[l];
    g.dense[l] = (r * r * r <= (uint64_t)size) ? 1 : 0;
    g.pow2[l] = (size & (size - 1)) == 0 ? 1 : 0;
    int lg = 0;
    while (((uint64_t)1 << lg) < size) ++lg;
    const uint64_t m = (((uint64_t)1 << 32) * (((uint64_t)1 << lg) - size)) / size + 1;
    g.magic[l] = (uint32_t)m;
    g.sh1[l] = lg < 1 ? lg : 1;
    g.sh2[l] = lg > 1 ? lg - 1 : 0;
  }
  return SN_OK;
}

int fill_field_args(FieldArgs& a, int64_t n, const int32_t* count, const float* x,
                           const float* table, const sn_grid_desc* grid, int active_levels,
                           const sn_mlp_desc* mlp, int out_cols) {
  memset(&a, 0, sizeof(a));
  SN_REQUIRE(n >= 0, "field: n < 0");
  SN_REQUIRE(mlp != nullptr, "field: mlp descriptor is null");
  SN_TRY(make_grid_dev(grid, a.g));
  if (mlp->d_hidden != kH) {
    set_error("field: hidden width %d unsupported (kernels are built for %d)", mlp->d_hidden, kH);
    return SN_ERR_UNSUPPORTED;
  }
  SN_REQUIRE(mlp->d_in == 3 + grid->n_levels * grid->n_features,
             "field: d_in %d != 3 + levels*features", mlp->d_in);
  if (mlp->d_out < 1 || mlp->d_out > kDoutMax) {
    set_error("field: d_out %d outside 1..%d", mlp->d_out, kDoutMax);
    return SN_ERR_UNSUPPORTED;
  }
  SN_REQUIRE(out_cols >= 1 && out_cols <= mlp->d_out, "field: out_cols %d outside 1..d_out", out_cols);
  SN_REQUIRE(x && table && mlp->w0 && mlp->b0 && mlp->w1 && mlp->b1, "field: null buffer");
  a.cap = n;
  a.count = count;
  a.x = x;
  a.table = table;
  a.active = active_levels < 0 ? 0 : (active_levels > a.g.L ? a.g.L : active_levels);
  a.din = mlp->d_in;
  a.dout = mlp->d_out;
  a.out_cols = out_cols;
  a.beta = mlp->beta;
  a.thresh = mlp->threshold;
  a.w0 = mlp->w0;
  a.b0 = mlp->b0;
  a.w1 = mlp->w1;
  a.b1 = mlp->b1;
  a.status = mlp->status;
  a.table_half = (mlp->flags & SN_FIELD_TABLE_FP16) != 0;
  a.one_pass = (mlp->flags & SN_FIELD_MLP_TF32) != 0;
  a.bf16 = (mlp->flags & SN_FIELD_MLP_BF16) != 0;
  return SN_OK;
}

}  // namespace sn

using namespace sn;

extern "C" {

int sn_grid_desc_init(sn_grid_desc* d, int n_levels, int n_features, int log2_hashmap_size,
                      int base_resolution, float per_level_scale) {
  SN_REQUIRE(d != nullptr, "grid_desc_init: null descriptor");
  SN_REQUIRE(n_levels >= 1 && n_levels <= SN_MAX_LEVELS, "grid_desc_init: n_levels outside 1..%d",
             SN_MAX_LEVELS);
  SN_REQUIRE(n_features >= 1, "grid_desc_init: n_features < 1");
  SN_REQUIRE(log2_hashmap_size >= 1 && log2_hashmap_size <= 30, "grid_desc_init: bad log2 size");
  SN_REQUIRE(base_resolution >= 1, "grid_desc_init: base_resolution < 1");
  SN_REQUIRE(per_level_scale >= 1.0f, "grid_desc_init: per_level_scale < 1");
  memset(d, 0, sizeof(*d));
  d->n_levels = n_levels;
  d->n_features = n_features;
  // float32 level constants, each rounded once from a double evaluation so
  // every host (x86 or Arm libm) produces the same bits
  const float log2_pls = (float)log2((double)per_level_scale);
  uint32_t offset = 0;
  for (int l = 0; l < n_levels; ++l) {
    const float scale =
        (float)(exp2((double)l * (double)log2_pls) * (double)base_resolution - 1.0);
    const uint32_t res = (uint32_t)ceilf(scale) + 1u;
    const uint32_t max_params = 0xffffffffu / 2;
    const double dense = pow((double)res, 3.0);
    uint32_t params = dense > (double)max_params ? max_params : res * res * res;
    params = (params + 7u) / 8u * 8u;
    const uint32_t hsize = 1u << log2_hashmap_size;
    if (params > hsize) params = hsize;
    d->scales[l] = scale;
    d->resolutions[l] = res;
    d->offsets[l] = offset;
    offset += params;
  }
  d->offsets[n_levels] = offset;
  return SN_OK;
}

int sn_hashgrid_fwd(int64_t n, const float* x, const float* table, const sn_grid_desc* grid,
                    int active_levels, float* out, void* stream) {
  GridDev g;
  SN_TRY(make_grid_dev(grid, g));
  SN_REQUIRE(n >= 0, "hashgrid_fwd: n < 0");
  if (n == 0) return SN_OK;
  const int act = active_levels < 0 ? 0 : (active_levels > g.L ? g.L : active_levels);
  hashgrid_fwd_kernel<<<stride_grid(n * g.L, 256, 8), 256, 0, as_stream(stream)>>>(n, x, table, g,
                                                                                  act, out);
  return check_launch("hashgrid_fwd");
}

int sn_hashgrid_bwd(int64_t n, const float* x, const float* grad_out, const sn_grid_desc* grid,
                    int active_levels, float* grad_table, void* stream) {
  GridDev g;
  SN_TRY(make_grid_dev(grid, g));
  SN_REQUIRE(n >= 0, "hashgrid_bwd: n < 0");
  if (n == 0) return SN_OK;
  const int act = active_levels < 0 ? 0 : (active_levels > g.L ? g.L : active_levels);
  hashgrid_bwd_kernel<<<stride_grid(n * g.L, 256, 8), 256, 0, as_stream(stream)>>>(
      n, x, grad_out, g, act, grad_table);
  return check_launch("hashgrid_bwd");
}

int sn_field_fwd(int64_t n, const int32_t* count, const float* x, const float* table,
                 const sn_grid_desc* grid, int active_levels, const sn_mlp_desc* mlp, int out_cols,
                 float* out, void* stream) {
  FieldArgs a;
  SN_TRY(fill_field_args(a, n, count, x, table, grid, active_levels, mlp, out_cols));
  SN_REQUIRE(out != nullptr, "field_fwd: out is null");
  a.out = out;
  if (mlp->enc_cache) {
    SN_REQUIRE((reinterpret_cast<uintptr_t>(mlp->enc_cache) & 7u) == 0, "field_fwd: enc_cache not 8-byte aligned");
    a.enc_out = reinterpret_cast<float2*>(mlp->enc_cache);
  }
  if (n == 0) return SN_OK;
  return field_fwd_tc(a, as_stream(stream));
}

int sn_field_fwd_batch(int n_segments, const sn_field_segment* segments, int out_cols, void* stream) {
  SN_REQUIRE(segments != nullptr, "field_fwd_batch: null segments");
  SN_REQUIRE(n_segments >= 1 && n_segments <= SN_FIELD_MAX_SEGMENTS, "field_fwd_batch: %d segments (1..%d)",
             n_segments, SN_FIELD_MAX_SEGMENTS);
  FieldArgs args[SN_FIELD_MAX_SEGMENTS];
  int live = 0;
  for (int i = 0; i < n_segments; ++i) {
    const sn_field_segment& sg = segments[i];
    SN_REQUIRE(sg.out != nullptr, "field_fwd_batch: segment %d has no output", i);
    SN_TRY(fill_field_args(args[live], sg.n, nullptr, sg.x, reinterpret_cast<const float*>(sg.table), sg.grid,
                           sg.active_levels, sg.mlp, out_cols));
    SN_REQUIRE(sg.mlp->enc_cache == nullptr, "field_fwd_batch: segment %d asks for an encoding cache", i);
    args[live].out = sg.out;
    if (sg.n > 0) ++live;
  }
  if (live == 0) return SN_OK;
  return field_fwd_tc_segments(args, live, as_stream(stream));
}

int sn_field_bwd(int64_t n, const int32_t* count, const float* x, const float* grad_out,
                 int out_cols, const float* table, const sn_grid_desc* grid, int active_levels,
                 const sn_mlp_desc* mlp, float* grad_table, float* grad_w0, float* grad_b0,
                 float* grad_w1, float* grad_b1, float* grad_x, void* stream) {
  FieldArgs a;
  SN_TRY(fill_field_args(a, n, count, x, table, grid, active_levels, mlp, out_cols));
  if (a.bf16) {
    set_error("field_bwd: SN_FIELD_MLP_BF16 is supported by sn_field_fwd only");
    return SN_ERR_UNSUPPORTED;
  }
  SN_REQUIRE(grad_out != nullptr, "field_bwd: grad_out is null");
  a.grad_out = grad_out;
  a.grad_table = grad_table;
  a.grad_w0 = grad_w0;
  a.grad_b0 = grad_b0;
  a.grad_w1 = grad_w1;
  a.grad_b1 = grad_b1;
  a.grad_x = grad_x;
  a.pair16 = (reinterpret_cast<uintptr_t>(grad_table) & 15u) == 0;
  if (mlp->enc_cache) {
    SN_REQUIRE((reinterpret_cast<uintptr_t>(mlp->enc_cache) & 7u) == 0, "field_bwd: enc_cache not 8-byte aligned");
    a.enc_in = reinterpret_cast<const float2*>(mlp->enc_cache);
  }
  if (n == 0) return SN_OK;
  return field_bwd_tc(a, as_stream(stream));
}

int sn_field_grad_fwd(int64_t n, const int32_t* count, const float* x, const float* table,
                      const sn_grid_desc* grid, int active_levels, const sn_mlp_desc* mlp,
                      float* sdf, float* grad, void* stream) {
  FieldArgs a;
  SN_TRY(fill_field_args(a, n, count, x, table, grid, active_levels, mlp, 1));
  if (a.table_half || a.one_pass || a.bf16) {
    set_error("field_grad: SN_FIELD_* precision flags are supported by the fused field forward/backward only");
    return SN_ERR_UNSUPPORTED;
  }
  SN_REQUIRE(grad != nullptr, "field_grad_fwd: grad is null");
  if (n == 0) return SN_OK;
  return field_grad_fwd_tc(a, sdf, grad, as_stream(stream));
}

int sn_field_grad_bwd(int64_t n, const int32_t* count, const float* x, const float* grad_grad,
                      const float* grad_sdf, const float* table, const sn_grid_desc* grid,
                      int active_levels, const sn_mlp_desc* mlp, float* grad_table, float* grad_w0,
                      float* grad_b0, float* grad_w1, float* grad_b1, void* stream) {
  FieldArgs a;
  SN_TRY(fill_field_args(a, n, count, x, table, grid, active_levels, mlp, 1));
  if (a.table_half || a.one_pass || a.bf16) {
    set_error("field_grad: SN_FIELD_* precision flags are supported by the fused field forward/backward only");
    return SN_ERR_UNSUPPORTED;
  }
  SN_REQUIRE(grad_grad != nullptr, "field_grad_bwd: grad_grad is null");
  a.grad_table = grad_table;
  a.grad_w0 = grad_w0;
  a.grad_b0 = grad_b0;
  a.grad_w1 = grad_w1;
  a.grad_b1 = grad_b1;
  a.pair16 = (reinterpret_cast<uintptr_t>(grad_table) & 15u) == 0;
  if (n == 0) return SN_OK;
  return field_grad_bwd_tc(a, grad_grad, grad_sdf, as_stream(stream));
}

int sn_weightnorm_fwd(int rows, int cols, const float* v, const float* g, float* w, float* norms,
                      void* stream) {
  SN_REQUIRE(rows > 0 && cols > 0, "weightnorm_fwd: bad shape");
  weightnorm_fwd_kernel<<<rows, 32, 0, as_stream(stream)>>>(rows, cols, v, g, w, norms);
  return check_launch("weightnorm_fwd");
}

int sn_weightnorm_bwd(int rows, int cols, const float* v, const float* g, const float* norms,
                      const float* grad_w, float* grad_v, float* grad_g, void* stream) {
  SN_REQUIRE(rows > 0 && cols > 0, "weightnorm_bwd: bad shape");
  weightnorm_bwd_kernel<<<rows, 32, 0, as_stream(stream)>>>(rows, cols, v, g, norms, grad_w, grad_v,
                                                            grad_g);
  return check_launch("weightnorm_bwd");
}

int sn_selftest_bounded_wait(uint32_t polls, int32_t* status, void* stream) {
  SN_REQUIRE(status != nullptr, "selftest_bounded_wait: status is null");
  return bounded_wait_selftest(status, polls, as_stream(stream));
}

uint32_t sn_bounded_wait_polls(void) { return bounded_wait_limit(); }

}  // extern "C"
