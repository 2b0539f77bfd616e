/*
 * supernormal_gb300 — C ABI of the GB300 (sm_103a) kernels behind the
 * SuperNormal training hot path: occupancy-grid ray marching, the
 * multi-resolution hash-grid SDF field, NeuS SDF->alpha, patch-based
 * render weights and ray accumulation.
 *
 * Conventions (every entry point):
 *   - plain C types only: device pointers, element counts, scalars;
 *   - `stream` is a cudaStream_t passed as void* (NULL = legacy stream);
 *   - outputs go to caller-allocated device buffers (nothing is allocated
 *     inside the library except where an entry point says so);
 *   - the return value is an SN_* status; on failure sn_last_error() holds
 *     a message (thread-local).  Launches are asynchronous: device-side
 *     conditions (iteration limits, capacity overflow) are reported through
 *     the optional `status` device word an entry point takes.
 *
 * Reference paths below are relative to the SuperNormal repository;
 * "NA/" abbreviates third_parties/nerfacc-0.3.5/nerfacc-0.3.5/.
 */
#ifndef SUPERNORMAL_GB300_H
#define SUPERNORMAL_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define SN_OK 0
#define SN_ERR_INVALID 1     /* bad argument (shape, size, null pointer)      */
#define SN_ERR_CAPACITY 2    /* output capacity smaller than required         */
#define SN_ERR_CUDA 3        /* CUDA launch / runtime error                   */
#define SN_ERR_LIMIT 4       /* a device loop hit its iteration limit         */
#define SN_ERR_UNSUPPORTED 5 /* configuration outside what the kernels cover  */

/* device status word bits (OR-ed by kernels into an int32 device word) */
#define SN_STATUS_MARCH_LIMIT 1   /* a ray exceeded the marching iteration cap */
#define SN_STATUS_CAPACITY 2      /* a sample buffer overflowed its capacity   */
#define SN_STATUS_TIMEOUT 4       /* a tensor-core kernel's bounded wait ran out */

/* contraction types; same values as nerfacc's ContractionType
 * (NA/nerfacc/cuda/csrc/include/helpers_contraction.h:9-14) */
#define SN_CONTRACTION_AABB 0
#define SN_CONTRACTION_UN_BOUNDED_TANH 1
#define SN_CONTRACTION_UN_BOUNDED_SPHERE 2

/* ---- library ------------------------------------------------------------ */
/* Version string of the library build. */
const char* sn_version(void);
/* Message of the last failing call on this host thread ("" if none). */
const char* sn_last_error(void);
/* Number of kernels this library has launched in the process (all threads). */
uint64_t sn_kernel_launches(void);

/* ---- packing (NA/nerfacc/pack.py) ---------------------------------------- */
/* Bytes of device workspace sn_pack_counts needs for n entries. */
size_t sn_scan_workspace_bytes(int64_t n);
/* packed_info[i] = {exclusive prefix sum of counts, counts[i]}; *total = sum.
 * Replaces the cumsum/stack in NA/nerfacc/cuda/csrc/ray_marching.cu:257-258
 * and NA/nerfacc/pack.py:73-75, without a host synchronisation. */
int sn_pack_counts(int64_t n, const int32_t* counts, int32_t* packed_info,
                   int32_t* total, void* workspace, void* stream);
/* sn_pack_counts over the first min(*count, cap) entries of a capacity-sized
 * array (count: device int32): the same packed_info and total there, nothing
 * read or written past the count, so a fixed-capacity (graph-captured) step
 * scans only its live entries. */
int sn_pack_counts_n(int64_t cap, const int32_t* count, const int32_t* counts,
                     int32_t* packed_info, int32_t* total, void* workspace,
                     void* stream);
/* sn_pack_counts that allocates nothing and takes no workspace: the tile sums
 * of the multi-tile scan live in a static device array.  No reference
 * counterpart (the reference's cumsum allocates through torch); it serves
 * callers that hold only borrowed device pointers and have no device
 * allocator of their own (a C or FFI binding handed tensors by its framework).
 * Limit: n <= 16,777,216 entries (larger n -> SN_ERR_INVALID with a message).
 * The first call on each device looks up the scratch address with that device
 * current; make it before any stream capture.  The address is kept for the
 * life of the process: after cudaDeviceReset on a device, do not call this
 * entry point on that device again.  The scratch is one per device: calls
 * that overlap on a device (other streams or threads) race. */
int sn_pack_counts_static(int64_t n, const int32_t* counts, int32_t* packed_info,
                          int32_t* total, void* stream);
/* counts[r] = number of samples with ray_indices == r (counts zeroed here).
 * Replaces the scatter_add_ in NA/nerfacc/pack.py:70-72. */
int sn_count_indices(int64_t n_samples, const int64_t* ray_indices,
                     int64_t n_rays, int32_t* counts, void* stream);
/* ray_indices of each sample from packed_info.
 * Replaces unpack_info_kernel (NA/nerfacc/cuda/csrc/pack.cu:7-27). */
int sn_unpack_info(int64_t n_rays, const int32_t* packed_info,
                   int64_t n_samples, int64_t* ray_indices, void* stream);

/* ---- ray marching (NA/nerfacc/cuda/csrc/ray_marching.cu) ----------------- */
/* Count pass of the marcher: num_steps[i] = samples on ray i.
 * Replaces the first launch of ray_marching_kernel
 * (NA/nerfacc/cuda/csrc/ray_marching.cu:81-192, host :194-255).
 * jitter (nullable, n_rays) adds jitter[i]*step_size to t_min[i] exactly as
 * NA/nerfacc/ray_marching.py:157-158 does; grid_binary is (rx,ry,rz) uint8
 * (torch.bool) and roi is 6 floats on the device. status (nullable) gets
 * SN_STATUS_MARCH_LIMIT if a ray exceeds max_iters loop iterations
 * (max_iters <= 0 selects 1<<24). */
int sn_march_count(int64_t n_rays, const float* rays_o, const float* rays_d,
                   const float* t_min, const float* t_max, const float* jitter,
                   const float* roi, const uint8_t* grid_binary, int rx, int ry,
                   int rz, int contraction_type, float step_size,
                   float cone_angle, int64_t max_iters, int32_t* num_steps,
                   int32_t* status, void* stream);
/* Fill pass: writes ray_indices / t_starts / t_ends at packed_info offsets.
 * Replaces the second launch of ray_marching_kernel
 * (NA/nerfacc/cuda/csrc/ray_marching.cu:263-286).  Samples beyond
 * `capacity` are dropped and flag SN_STATUS_CAPACITY. */
int sn_march_fill(int64_t n_rays, const float* rays_o, const float* rays_d,
                  const float* t_min, const float* t_max, const float* jitter,
                  const float* roi, const uint8_t* grid_binary, int rx, int ry,
                  int rz, int contraction_type, float step_size,
                  float cone_angle, int64_t max_iters,
                  const int32_t* packed_info, int64_t capacity,
                  int64_t* ray_indices, float* t_starts, float* t_ends,
                  int32_t* status, void* stream);
/* Single-pass marcher: ray i writes its samples to slots
 * [i*slot_stride, i*slot_stride + num_steps[i]) (num_steps written too;
 * SN_STATUS_CAPACITY if a ray has more than slot_stride samples).  Same
 * samples as count + fill; used with sn_pack_counts + sn_compact_padded.
 * step_size_dev (nullable) holds the step size in device memory and then
 * replaces step_size, so a captured launch follows a step-size schedule
 * (sn_step_size_schedule). */
int sn_march_padded(int64_t n_rays, const float* rays_o, const float* rays_d,
                    const float* t_min, const float* t_max, const float* jitter,
                    const float* roi, const uint8_t* grid_binary, int rx, int ry,
                    int rz, int contraction_type, float step_size,
                    const float* step_size_dev, float cone_angle,
                    int64_t max_iters, int64_t slot_stride, int32_t* num_steps,
                    int64_t* ray_indices, float* t_starts, float* t_ends,
                    int32_t* status, void* stream);
/* Copies padded per-ray samples to their packed_info offsets. */
int sn_compact_padded(int64_t n_rays, int64_t slot_stride,
                      const int32_t* packed_info, const int64_t* ray_indices_in,
                      const float* t_starts_in, const float* t_ends_in,
                      int64_t* ray_indices_out, float* t_starts_out,
                      float* t_ends_out, void* stream);
/* out[i] = grid_binary at samples[i] (0 outside the AABB roi).
 * Replaces query_occ_kernel (NA/nerfacc/cuda/csrc/ray_marching.cu:295-358). */
int sn_grid_query(int64_t n, const float* samples, const float* roi,
                  const uint8_t* grid_binary, int rx, int ry, int rz,
                  int contraction_type, uint8_t* out, void* stream);

/* ---- occupancy grid (NA/nerfacc/grid.py:196-239) -------------------------- */
/* World-space query points of grid cells:
 * x = contract_inv((coords(cell) + jitter) / res) (NA/nerfacc/grid.py:210-225).
 * cells (nullable => cell i for point i), jitter (n,3) in [0,1). */
int sn_occ_points(int64_t n, const int64_t* cells, const float* jitter,
                  int rx, int ry, int rz, const float* roi,
                  int contraction_type, float* x_out, void* stream);
/* occs[c] = max(occs[c]*ema_decay, occ[i]) for c = cells[i]
 * (NA/nerfacc/grid.py:229-230).  cells == NULL: cell i for i < n, updated
 * in place.  Sampled cells may repeat: every candidate is formed from the
 * cell's value before the update, and a repeated cell ends at the largest
 * candidate, max(occs[c]*ema_decay, max_i occ[i]) (the reference's index_put
 * stores an unspecified one of them); workspace holds n floats and is
 * required when cells != NULL. */
int sn_occ_ema_update(int64_t n, const int64_t* cells, const float* occ,
                      float ema_decay, float* occs, float* workspace,
                      void* stream);
size_t sn_occ_binarize_workspace_bytes(int64_t n_cells);
/* binary[c] = occs[c] > min(mean(occs), occ_thre) (NA/nerfacc/grid.py:235-237);
 * mean_out (nullable, device) receives the mean. */
int sn_occ_binarize(int64_t n_cells, const float* occs, float occ_thre,
                    uint8_t* binary, float* mean_out, void* workspace,
                    void* stream);
/* Device-count forms used by the fused training step (no host sync):
 * query points of cells[i] (nullable => cell i) for i < *count with jitter
 * drawn in-kernel from (seed, *stream_counter). */
int sn_occ_points_n(int64_t cap, const int32_t* count, const int64_t* cells,
                    uint64_t seed, const int32_t* stream_counter, int rx,
                    int ry, int rz, const float* roi, int contraction_type,
                    float* x_out, void* stream);
/* occs[c] = max(occs[c]*ema_decay, sigmoid(-sigmoid_k * sdf[i])) for
 * i < min(*count, cap): the renderer's occ_eval_fn (models/renderer.py:56-60)
 * fused with the EMA, repeated cells resolved as in sn_occ_ema_update
 * (workspace: cap floats, required when cells != NULL). */
int sn_occ_ema_sdf(int64_t cap, const int32_t* count, const int64_t* cells,
                   const float* sdf, float sigmoid_k, float ema_decay,
                   float* occs, float* workspace, void* stream);
size_t sn_occ_sample_workspace_bytes(int64_t n_cells);
/* Post-warm-up cell sampling (NA/nerfacc/grid.py:168-182): n_uniform
 * uniform cells followed by min(n_occupied, n_uniform) occupied cells (all,
 * or a uniform draw); *count = total (cells needs 2*n_uniform entries). */
int sn_occ_sample_cells(int64_t n_cells, const uint8_t* binary,
                        int64_t n_uniform, uint64_t seed,
                        const int32_t* stream_counter, int64_t* cells,
                        int32_t* count, void* workspace, void* stream);

/* ---- volume rendering (NA/nerfacc/vol_rendering.py) ----------------------- */
/* Exclusive transmittance T_i = prod_{j<i}(1 - alpha_j) per ray segment of
 * packed_info, with patch_size pixel lanes per sample (1 = per-ray).
 * Replaces transmittance_from_alpha_forward_cub / _naive
 * (NA/nerfacc/cuda/csrc/render_transmittance_cub.cu:111-134). */
int sn_transmittance_from_alpha(int64_t n_rays, int patch_size,
                                const int32_t* packed_info,
                                const float* alphas, float* transmittance,
                                void* stream);
/* visibility[s] = T_s >= early_stop_eps && (alpha_thre <= 0 || alpha_s >= alpha_thre)
 * and vis_counts[r] (nullable) = visible samples of ray r.
 * Replaces render_visibility (NA/nerfacc/vol_rendering.py:680-748). */
int sn_visibility_from_alpha(int64_t n_rays, const int32_t* packed_info,
                             const float* alphas, float early_stop_eps,
                             float alpha_thre, uint8_t* visibility,
                             int32_t* vis_counts, void* stream);
/* Weights w = alpha * T per (ray, pixel lane); patch_size = 1 gives the
 * per-ray variant.  Replaces weight_from_alpha_patch_based_forward_kernel
 * (NA/nerfacc/cuda/csrc/render_weight.cu:87-118, host :502-543) and
 * weight_from_alpha_forward_kernel (:154-183). */
int sn_weight_from_alpha_fwd(int64_t n_rays, int patch_size,
                             const int32_t* packed_info, const float* alphas,
                             float* weights, void* stream);
/* grad_alpha_j = (g_j T_j - sum_{i>=j} g_i w_i) / max(1 - alpha_j, 1e-10).
 * Replaces weight_from_alpha_patch_based_backward_kernel
 * (NA/nerfacc/cuda/csrc/render_weight.cu:298-340, host :583-626). */
int sn_weight_from_alpha_bwd(int64_t n_rays, int patch_size,
                             const int32_t* packed_info, const float* alphas,
                             const float* weights, const float* grad_weights,
                             float* grad_alphas, void* stream);
/* out[ray_indices[s], k, :] += weights[s,k] * values[s,k,:] (values NULL =>
 * dim 1, value 1).  out is zero-filled here.  Replaces the scatter_add_ of
 * accumulate_along_rays(_patch_based) (NA/nerfacc/vol_rendering.py:132-335). */
int sn_accumulate_fwd(int64_t n_samples, int patch_size, int dim,
                      const int64_t* ray_indices, const float* weights,
                      const float* values, int64_t n_rays, float* out,
                      void* stream);
/* Adjoint of sn_accumulate_fwd: grad_weights[s,k] = sum_d g[r,k,d] v[s,k,d],
 * grad_values[s,k,d] = g[r,k,d] w[s,k] (either output nullable). */
int sn_accumulate_bwd(int64_t n_samples, int patch_size, int dim,
                      const int64_t* ray_indices, const float* weights,
                      const float* values, const float* grad_out,
                      float* grad_weights, float* grad_values, void* stream);

/* ---- SDF field (models/fields.py SDFNetwork + tcnn HashGrid) --------------- */
#define SN_MAX_LEVELS 32

/* Hash-grid geometry in tiny-cuda-nn's layout (entry-major, n_features per
 * entry, levels concatenated).  Filled by sn_grid_desc_init. */
typedef struct sn_grid_desc {
  int32_t n_levels;
  int32_t n_features;
  uint32_t offsets[SN_MAX_LEVELS + 1]; /* first entry of each level; [L] = total */
  uint32_t resolutions[SN_MAX_LEVELS];
  float scales[SN_MAX_LEVELS];
} sn_grid_desc;

/* One-hidden-layer MLP with effective (post weight-norm) weights, row-major
 * like torch.nn.Linear.weight: w0 (d_hidden, d_in), w1 (d_out, d_hidden). */
typedef struct sn_mlp_desc {
  int32_t d_in;      /* 3 + n_levels * n_features (input_concat) */
  int32_t d_hidden;  /* 64 */
  int32_t d_out;     /* 1..16 */
  float beta;        /* Softplus beta (100) */
  float threshold;   /* Softplus threshold (20) */
  const float* w0;
  const float* b0;
  const float* w1;
  const float* b1;
  int32_t* status;   /* nullable device word: SN_STATUS_TIMEOUT is OR-ed here */
  uint32_t flags;    /* SN_FIELD_* precision options of the fused field kernels */
  float* enc_cache;  /* nullable: encoding cache of the fused field kernels (below) */
} sn_mlp_desc;

/* sn_mlp_desc.flags (fused field forward / backward only):
 * SN_FIELD_TABLE_FP16 -- the `table` pointer addresses the hash table as FP16
 *   pairs (an FP16 copy of FP32 master weights; gradients stay FP32);
 * SN_FIELD_MLP_TF32 -- the MLP's tensor-core products in one TF32 pass
 *   instead of the FP32-accurate three;
 * SN_FIELD_MLP_BF16 -- sn_field_fwd only: the first layer's products in one
 *   BF16 pass (inputs and W0 rounded to BF16, FP32 accumulation); the
 *   backward and gradient entry points reject it. */
#define SN_FIELD_TABLE_FP16 1u
#define SN_FIELD_MLP_TF32 2u
#define SN_FIELD_MLP_BF16 4u

/* sn_mlp_desc.enc_cache (no reference counterpart; the reference's autograd
 * keeps tcnn's encoding output alive between forward and backward in the
 * same way): n_levels * 2 floats per point of capacity n, 8-byte aligned,
 * level l of point p at enc_cache[2 * (l * n + p)].  sn_field_fwd writes the levels
 * below active_levels of its points there; sn_field_bwd reads them instead of
 * gathering the table again.  The backward must see the same n, count, x,
 * table and active_levels as the forward that filled the cache; results are
 * identical to the recomputing backward.  sn_field_grad_fwd/bwd ignore it. */

/* Level offsets, resolutions and scales of tcnn's GridEncoding for
 * {otype: HashGrid, n_levels, n_features_per_level, log2_hashmap_size,
 *  base_resolution, per_level_scale} (models/fields.py:26, config/*.conf). */
int sn_grid_desc_init(sn_grid_desc* desc, int n_levels, int n_features,
                      int log2_hashmap_size, int base_resolution,
                      float per_level_scale);
/* Encoding forward: out (n, L*F); levels >= active_levels give zeros.
 * Replaces tcnn.Encoding.forward (models/fields.py:78) plus the bandwidth
 * mask (:81-83). */
int sn_hashgrid_fwd(int64_t n, const float* x, const float* table,
                    const sn_grid_desc* grid, int active_levels, float* out,
                    void* stream);
/* Encoding backward: grad_table += d out / d table ^T grad_out (atomics). */
int sn_hashgrid_bwd(int64_t n, const float* x, const float* grad_out,
                    const sn_grid_desc* grid, int active_levels,
                    float* grad_table, void* stream);
/* Fused field forward: out (n, out_cols) = first out_cols outputs of
 * SDFNetwork.forward (models/fields.py:76-99).  count (nullable, device)
 * bounds n at run time (n is then a capacity). */
int sn_field_fwd(int64_t n, const int32_t* count, const float* x,
                 const float* table, const sn_grid_desc* grid,
                 int active_levels, const sn_mlp_desc* mlp, int out_cols,
                 float* out, void* stream);
/* Several objects' field forwards in one launch: segment i evaluates its n
 * points x (n, 3) with its own table, level geometry, active levels and MLP
 * into out (n, out_cols), as sn_field_fwd would (same kernels, same values;
 * no device count, no encoding cache).  The persistent CTAs stage each
 * segment's weights in turn.  No reference counterpart: it batches the
 * SDF-grid queries (models/renderer.py:9-24) of several served objects. */
#define SN_FIELD_MAX_SEGMENTS 4
typedef struct {
  int64_t n;
  const float* x;
  const void* table;          /* FP32, or FP16 pairs with SN_FIELD_TABLE_FP16 in mlp->flags */
  const sn_grid_desc* grid;
  int32_t active_levels;
  const sn_mlp_desc* mlp;
  float* out;
} sn_field_segment;
int sn_field_fwd_batch(int n_segments, const sn_field_segment* segments,
                       int out_cols, void* stream);
/* Fused field backward with recomputation: accumulates (+=) the gradients of
 * sum(grad_out * out) into grad_table / grad_w0 / grad_b0 / grad_w1 /
 * grad_b1 and writes grad_x (each nullable).  Replaces the autograd backward
 * through the torch MLP and tcnn's encoding backward. */
int sn_field_bwd(int64_t n, const int32_t* count, const float* x,
                 const float* grad_out, int out_cols, const float* table,
                 const sn_grid_desc* grid, int active_levels,
                 const sn_mlp_desc* mlp, float* grad_table, float* grad_w0,
                 float* grad_b0, float* grad_w1, float* grad_b1,
                 float* grad_x, void* stream);
/* Self-test of the failure path of the tensor-core field kernels (no
 * reference counterpart): one thread block waits, with the bounded mbarrier
 * wait those kernels use, on an mbarrier that nothing arrives at, for `polls`
 * polls (0: the kernels' own limit, sn_bounded_wait_polls()).  The wait gives
 * up, SN_STATUS_TIMEOUT is OR-ed into *status (device word) and the kernel
 * returns; the context stays usable.  This is the report a field kernel makes
 * when its MMAs never complete. */
int sn_selftest_bounded_wait(uint32_t polls, int32_t* status, void* stream);
uint32_t sn_bounded_wait_polls(void);
/* sdf (nullable, n) and grad = d sdf / d x (n, 3) in one pass: replaces
 * SDFNetwork.gradient's autograd.grad (models/fields.py:107-119). */
int sn_field_grad_fwd(int64_t n, const int32_t* count, const float* x,
                      const float* table, const sn_grid_desc* grid,
                      int active_levels, const sn_mlp_desc* mlp, float* sdf,
                      float* grad, void* stream);
/* Hand-written adjoint of (sdf, grad) = field_grad_fwd(x): given
 * grad_grad = dL/dgrad (n, 3) and grad_sdf = dL/dsdf (nullable, n),
 * accumulates (+=) the parameter gradients including the second-order terms
 * through the MLP Jacobian and the trilinear weight derivatives (the double
 * backward that create_graph=True gives the reference; models/fields.py:113-119).
 * grad_w1 / grad_b1 receive row 0 / entry 0 (the sdf output). */
int sn_field_grad_bwd(int64_t n, const int32_t* count, const float* x,
                      const float* grad_grad, const float* grad_sdf,
                      const float* table, const sn_grid_desc* grid,
                      int active_levels, const sn_mlp_desc* mlp,
                      float* grad_table, float* grad_w0, float* grad_b0,
                      float* grad_w1, float* grad_b1, void* stream);
/* torch.nn.utils.weight_norm (dim=0): w = g * v / ||v||_row (models/fields.py:66-67). */
int sn_weightnorm_fwd(int rows, int cols, const float* v, const float* g,
                      float* w, float* norms, void* stream);
int sn_weightnorm_bwd(int rows, int cols, const float* v, const float* g,
                      const float* norms, const float* grad_w, float* grad_v,
                      float* grad_g, void* stream);

/* ---- renderer glue (models/renderer.py:63-276) ----------------------------- */
/* diff[i] = t_ends[i] != t_starts[i+1] over the flattened samples (the last
 * sample compares with its own start): models/renderer.py:88-93, :151-154.
 * count (nullable, device) bounds cap at run time; entries past the count
 * are not written (sn_pack_counts_n scans only below the count). */
int sn_end_diff(int64_t cap, const int32_t* count, const float* t_starts,
                const float* t_ends, int32_t* diff, void* stream);
/* Query points of patch-centre samples for the culling alpha_fn
 * (models/renderer.py:80-98): xyz[i] = o + d*t_start, and for diff samples
 * xyz[n + slot] = o + d*t_end (end_packed = sn_pack_counts of diff).
 * n_points (device) receives n + n_ends. */
int sn_center_points(int64_t cap, const int32_t* count,
                     const int64_t* ray_indices, const float* t_starts,
                     const float* t_ends, const float* rays_o,
                     const float* rays_d, const int32_t* end_packed,
                     const int32_t* n_ends, float* xyz, int32_t* n_points,
                     void* stream);
/* NeuS alpha at centre samples from the field output (column 0 of a
 * row-major (points, sdf_stride) array): models/renderer.py:100-117. */
int sn_center_alpha(int64_t cap, const int32_t* count, const float* sdf,
                    int sdf_stride, const int32_t* end_packed,
                    const float* variance, float* alpha, void* stream);
/* Order-preserving compaction of visible samples (the boolean indexing of
 * NA/nerfacc/ray_marching.py:216-220); packed_out = sn_pack_counts of the
 * per-ray visible counts. */
int sn_compact_samples(int64_t n_rays, const int32_t* packed_in,
                       const uint8_t* visibility, const int32_t* packed_out,
                       const int64_t* ray_indices, const float* t_starts,
                       const float* t_ends, int64_t* ray_indices_out,
                       float* t_starts_out, float* t_ends_out, void* stream);
/* Patch expansion through the marching plane (models/renderer.py:146-159):
 * t_pix = t_c * (d_c . n) / (d_pix . n) for every pixel, start points at
 * xyz[i*P + k] and end points of diff samples at xyz[(S + slot)*P + k].
 * n_points (device) receives (S + n_ends) * P. */
int sn_patch_points(int64_t cap, const int32_t* count, int patch_h,
                    int patch_w, const int64_t* patch_indices,
                    const float* t_starts, const float* t_ends,
                    const float* rays_o, const float* rays_d,
                    const float* plane_normal, const int32_t* end_packed,
                    const int32_t* n_ends, float* xyz, float* t_pix_starts,
                    float* t_pix_ends, int32_t* n_points, void* stream);
/* Fused patch render forward: NeuS alpha (models/renderer.py:164-179),
 * patch weights (:180), dfd gradients (:187-223) and accumulation of
 * normals and mask (:263-267).  One warp per patch, one lane per pixel.
 * alpha / weights / gradients (nullable) are per sample; comp_normal
 * (n_patches, P, 3) and weight_sum (n_patches, P) per patch pixel.
 * ext_gradients (nullable, (S, P, 3)) replaces the dfd gradients by given
 * ones: the 'ad' method, gradients = SDFNetwork.gradient at the start points
 * (models/renderer.py:225-226). */
int sn_patch_render_fwd(int64_t n_patches, int patch_h, int patch_w,
                        const int32_t* packed_info, const int32_t* s_count,
                        int64_t s_cap, const int32_t* end_packed,
                        const float* sdf, const float* t_pix_starts,
                        const float* t_pix_ends, const float* rays_o,
                        const float* rays_d, const float* v_inverse,
                        const float* variance, float* alpha, float* weights,
                        float* gradients, float* comp_normal,
                        float* weight_sum, const float* ext_gradients,
                        void* stream);
/* Adjoint of sn_patch_render_fwd: d_sdf (field-point layout; every live
 * entry written) and per-patch partials[4p] = d loss / d inv_s.  carry
 * (n_patches, P) receives the end adjoint a patch owes the next sample when
 * that sample starts a later patch; sn_patch_carry_fixup adds it.  With
 * ext_gradients, d_gradients (S, P, 3) receives dL / d gradients. */
int sn_patch_render_bwd(int64_t n_patches, int patch_h, int patch_w,
                        const int32_t* packed_info, const int32_t* s_count,
                        int64_t s_cap, const int32_t* end_packed,
                        const float* sdf, const float* t_pix_starts,
                        const float* t_pix_ends, const float* rays_o,
                        const float* rays_d, const float* v_inverse,
                        const float* variance, const float* grad_comp_normal,
                        const float* grad_weight_sum,
                        const float* grad_gradients, float* d_sdf,
                        float* partials, float* carry,
                        const float* ext_gradients, float* d_gradients,
                        void* stream);
/* Training form: forward, the losses of exp_runner.py:191-203 (normal L2 or
 * L1 over sum(mask), eikonal mean, mask BCE) and the adjoint in one pass.
 * partials[4p..4p+3] = d/d inv_s, normal-loss sum, BCE sum, eikonal sum. */
int sn_patch_render_train(int64_t n_patches, int patch_h, int patch_w,
                          const int32_t* packed_info, const int32_t* s_count,
                          int64_t s_cap, const int32_t* end_packed,
                          const float* sdf, const float* t_pix_starts,
                          const float* t_pix_ends, const float* rays_o,
                          const float* rays_d, const float* v_inverse,
                          const float* variance, const float* gt_normal,
                          const float* gt_mask, const float* mask_sum,
                          int loss_l1, float w_normal, float w_eikonal,
                          float w_mask, float* d_sdf, float* partials,
                          float* carry, const float* ext_gradients,
                          float* d_gradients, void* stream);
/* d_sdf[start after the last sample of patch p] += carry[p] where that
 * sample's end was not evaluated separately (run after the render adjoint). */
int sn_patch_carry_fixup(int64_t n_patches, int patch_size,
                         const int32_t* packed_info, const int32_t* s_count,
                         int64_t s_cap, const int32_t* end_packed,
                         const float* carry, float* d_sdf, void* stream);
/* Reduces per-patch partials: grad_variance (nullable) += d loss/d variance;
 * out (nullable, 5 floats) = {d/d variance, normal, bce, eikonal, total}. */
int sn_patch_finalize(int64_t n_patches, int patch_size, const float* partials,
                      const int32_t* s_count, int64_t s_cap,
                      const float* variance, const float* mask_sum,
                      float w_normal, float w_eikonal, float w_mask,
                      float* out, float* grad_variance, void* stream);
/* near/far of the unit-sphere chord (models/dataset_loader.py:279-297) for
 * rays read every `stride` floats (NaN when the ray misses: no samples),
 * jitter (nullable) in [0,1) drawn from (seed, *stream_counter), and
 * optional contiguous (n, 3) copies of the rays read. */
int sn_near_far_sphere(int64_t n, const float* rays_o, const float* rays_d,
                       int64_t stride, float* near, float* far, float* jitter,
                       uint64_t seed, const int32_t* stream_counter,
                       float* rays_o_out, float* rays_d_out, void* stream);
/* Training patches on the device (models/dataset_loader.py:223-277) with the
 * rays and V^-1 formed per pixel instead of read from per-view (H, W, 3) and
 * (H, W, 3, 3) tables (:112-145): for patch b of view img[b] centred at
 * (cx[b], cy[b]), pixel (x, y) gets d = R normalize(K^-1 [x, y, 1]), origin t
 * and V^-1 with V = rows (d, R[:,0], R[:,1]); plane_n[b] = R[:,2].  kinv
 * (n_views, 3, 3) and pose (n_views, 3, 4) = [R | t] are double; normals
 * (n_views, H, W, 3) and masks (n_views, H, W) are gathered when given.
 * Outputs: rays_o / rays_d / normal_out (n, ph, pw, 3), vinv (n, ph, pw, 3, 3),
 * mask_out (n, ph, pw), plane_n (n, 3).  Centres must keep the patch inside
 * the view. */
int sn_gen_patches(int64_t n_patches, int patch_h, int patch_w,
                   const int32_t* cx, const int32_t* cy, const int32_t* img,
                   int n_views, int H, int W, const double* kinv,
                   const double* pose, const float* normals, const float* masks,
                   float* rays_o, float* rays_d, float* plane_n, float* vinv,
                   float* normal_out, float* mask_out, void* stream);
/* *out = *in * mul + add on the device (counts derived without a host sync). */
int sn_scale_count(const int32_t* in, int32_t mul, int32_t add, int32_t* out,
                   void* stream);
/* mask_out = (mask_in > 0.5), *mask_sum = sum(mask_out) + 1e-5
 * (exp_runner.py:169-175). */
int sn_mask_prep(int64_t n, const float* mask_in, float* mask_out,
                 float* mask_sum, void* stream);

/* ---- synthetic analytic scenes (benchmark and test data) ------------------- */
/* No reference counterpart: the reference trains on captured normal maps
 * (models/dataset_loader.py); the benchmarks here render multi-view normal
 * maps and masks of analytic SDF scenes instead.  A scene is the union (min)
 * of up to SN_SCENE_MAX_PRIMS primitives minus a displacement
 * disp_amp * sin(f x) sin(f y) sin(f z); a torus lies around z with ring
 * radius size[0], tube radius size[1] and a radial displacement
 * amp * sin(freq theta) sin(freq phi); a box has half extents size[];
 * lipschitz bounds the SDF's slope (sphere-tracing step sdf / lipschitz * 0.9). */
#define SN_SCENE_MAX_PRIMS 4
enum { SN_PRIM_SPHERE = 0, SN_PRIM_TORUS = 1, SN_PRIM_BOX = 2 };
typedef struct {
  int32_t kind;
  int32_t reserved;
  double center[3];
  double size[3];
  double amp, freq;
} sn_prim;
typedef struct {
  int32_t n_prims;
  int32_t reserved;
  sn_prim prims[SN_SCENE_MAX_PRIMS];
  double disp_amp, disp_freq;
  double lipschitz;
} sn_scene_desc;
/* Ground-truth normal maps and masks of n_views pinhole views: pixel (x, y)
 * of view v looks along R_v normalize(K_v^-1 [x, y, 1]) from t_v (kinv
 * (n_views, 3, 3) and pose (n_views, 3, 4) = [R | t], double), is clipped to
 * the unit sphere and sphere-traced in double (at most max_iters steps, hit
 * when |sdf| < eps); normals (n_views, H, W, 3) get the unit SDF gradient at
 * the hit (zero on a miss), masks (n_views, H, W) 1 or 0. */
int sn_scene_render_gt(const sn_scene_desc* scene, int n_views, int H, int W,
                       const double* kinv, const double* pose, int max_iters,
                       double eps, float* normals, float* masks, void* stream);
/* out[i] = the scene's SDF at x[i] (n, 3) (evaluated in double). */
int sn_scene_sdf(const sn_scene_desc* scene, int64_t n, const float* x,
                 float* out, void* stream);

/* ---- mesh extraction (models/renderer.py:9-34, 353-358) ------------------ */
/* Lattice points of slab [i0, i0 + n_i) of an nx x ny x nz lattice over
 * [bound_min, bound_max] (double, 3 each): x_out[((i - i0) ny + j) nz + k] =
 * bound_min + (i, j, k) (bound_max - bound_min) / (n - 1).  Replaces the
 * torch.linspace / meshgrid blocks of extract_fields (models/renderer.py:9-24). */
int sn_lattice_points(int64_t i0, int64_t n_i, int nx, int ny, int nz,
                      const double* bound_min, const double* bound_max,
                      float* x_out, void* stream);
/* out[i] = -in[i] (the query_func of NeuSRenderer.extract_geometry is -sdf). */
int sn_negate(int64_t n, const float* in, float* out, void* stream);
size_t sn_marching_cubes_workspace_bytes(int nx, int ny, int nz);
/* Marching cubes of values (nx, ny, nz; k fastest) at threshold (inside:
 * value > threshold); replaces mcubes.marching_cubes in extract_geometry
 * (models/renderer.py:27-34).  One vertex per lattice edge whose ends lie on
 * either side, at the linear-interpolation crossing, in world coordinates
 * bound_min + index (bound_max - bound_min) / (n - 1); triangles index the
 * vertices, right-hand normals pointing from the inside out, each cube face
 * pairing its crossings so that inside corners are cut off (no cracks).
 * counts[0] = vertices, counts[1] = triangles (device); at most vert_cap /
 * tri_cap are written, so a first call with zero capacities sizes the
 * outputs.  Needs 3 nx ny nz < 2^31. */
int sn_marching_cubes(const float* values, int nx, int ny, int nz,
                      float threshold, const double* bound_min,
                      const double* bound_max, int64_t vert_cap,
                      int64_t tri_cap, float* vertices, int32_t* triangles,
                      int32_t* counts, void* workspace, void* stream);

/* ---- optimiser (exp_runner.py:97, 205-210, 270-279) ------------------------ */
/* Reads iteration k from *iter, writes lr(k) of the warm-up + cosine schedule
 * and adam_step = k + 1, then stores k + 1 in *iter. */
int sn_lr_schedule(int32_t* iter, float* lr, int32_t* adam_step, float base_lr,
                   int warm_up_end, int end_iter, float alpha, void* stream);
/* Marching step of iteration *iter on the log schedule of exp_runner.py:81-83,
 * 149 (renderer.sampling_step_size = 10 ** (log10(start) - slop * iter), slop =
 * (log10(start) - log10(end)) / end_iter), formed in double and rounded once
 * to float into *step; *iter is read, not changed. */
int sn_step_size_schedule(const int32_t* iter, double start_step, double end_step,
                          int end_iter, float* step, void* stream);
/* torch.optim.Adam step over a flat buffer (16-byte aligned).  lr_dev /
 * step_dev (nullable) override lr / step; zero_grad clears grad after use;
 * param_half (nullable) receives an fp16 copy of the updated parameters. */
int sn_adam_step(int64_t n, float* param, float* grad, float* exp_avg,
                 float* exp_avg_sq, void* param_half, const float* lr_dev,
                 const int32_t* step_dev, float lr, int step, float beta1,
                 float beta2, float eps, int zero_grad, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* SUPERNORMAL_GB300_H */
