/*
 * ORACLE (test infrastructure only; never linked into the product path).
 *
 * Plain-C, single-threaded restatement of nerfacc 0.3.5's occupancy-grid
 * marcher, used to check the CUDA marcher bit for bit:
 *   third_parties/nerfacc-0.3.5/nerfacc-0.3.5/nerfacc/cuda/csrc/ray_marching.cu
 *     :9-14   calc_dt, :16-25 grid_idx_at, :27-45 grid_occupied_at,
 *     :47-57  distance_to_next_voxel, :59-75 advance_to_next_voxel,
 *     :81-192 ray_marching_kernel (count and fill rounds)
 *   .../include/helpers_contraction.h:16-21 roi_to_unit (AABB contraction)
 *   .../include/helpers_math.h:177-180 make_int3(float3) truncation,
 *     :1471-1475 sign = copysignf(1, x).
 * float32 arithmetic in the reference's evaluation order; nvcc contracts
 * `origin + t_mid * dir` into an FMA, written here as fmaf.  Build with
 * -ffp-contract=off so the host compiler adds no contractions of its own.
 * Only the AABB contraction (SuperNormal's) is restated.
 */
#include <math.h>
#include <stdint.h>

static float calc_dt(float t, float cone, float dt_min, float dt_max) {
  float v = t * cone;
  v = v < dt_min ? dt_min : v;  /* clamp(t*cone, dt_min, dt_max) */
  v = v > dt_max ? dt_max : v;
  return v;
}

static int occupied_at(const float p[3], const float lo[3], const float hi[3], const int res[3],
                       const uint8_t* bits) {
  if (p[0] < lo[0] || p[0] > hi[0] || p[1] < lo[1] || p[1] > hi[1] || p[2] < lo[2] ||
      p[2] > hi[2])
    return 0;
  int ix[3];
  for (int d = 0; d < 3; ++d) {
    float u = (p[d] - lo[d]) / (hi[d] - lo[d]);
    int v = (int)(u * (float)res[d]);
    if (v < 0) v = 0;
    if (v > res[d] - 1) v = res[d] - 1;
    ix[d] = v;
  }
  return bits[ix[0] * (res[1] * res[2]) + ix[1] * res[2] + ix[2]] != 0;
}

static float advance_voxel(float t, float dt_min, const float p[3], const float dir[3],
                           const float inv[3], const float lo[3], const float hi[3],
                           const int res[3], float far) {
  float tx[3];
  for (int d = 0; d < 3; ++d) {
    float ext = hi[d] - lo[d];
    float r = (float)res[d];
    float xu = ((p[d] - lo[d]) / ext) * r;
    float f = floorf((xu + 0.5f) + copysignf(0.5f, dir[d]));
    tx[d] = (((f - xu) * inv[d]) / r) * ext;
  }
  float dist = fminf(fminf(tx[0], tx[1]), tx[2]);
  dist = fmaxf(dist, 0.0f);
  float target = fminf(t + dist, far);
  float s = t;
  do {
    s = s + dt_min;
  } while (s < target);
  return s;
}

/* Marches one ray; writes up to `room` samples when out arrays are given.
 * Returns the number of samples, or -1 when max_iters is exceeded. */
static int64_t march_ray(const float o[3], const float d[3], float near, float far, float step,
                         float cone, const float lo[3], const float hi[3], const int res[3],
                         const uint8_t* bits, int64_t max_iters, float* ts, float* te) {
  float inv[3] = {1.0f / d[0], 1.0f / d[1], 1.0f / d[2]};
  const float dt_min = step, dt_max = 1e10f;
  int64_t j = 0, iters = 0;
  float t0 = near;
  float dt = calc_dt(t0, cone, dt_min, dt_max);
  float t1 = t0 + dt;
  float tm = (t0 + t1) * 0.5f;
  while (tm < far) {
    if (++iters > max_iters) return -1;
    float p[3];
    for (int k = 0; k < 3; ++k) p[k] = fmaf(tm, d[k], o[k]);
    if (occupied_at(p, lo, hi, res, bits)) {
      if (ts) {
        ts[j] = t0;
        te[j] = t1;
      }
      ++j;
      t0 = t1;
      t1 = t0 + calc_dt(t0, cone, dt_min, dt_max);
      tm = (t0 + t1) * 0.5f;
    } else {
      tm = advance_voxel(tm, dt_min, p, d, inv, lo, hi, res, far);
      dt = calc_dt(tm, cone, dt_min, dt_max);
      t0 = tm - dt * 0.5f;
      t1 = tm + dt * 0.5f;
    }
  }
  return j;
}

/* Count round: num_steps[i]; returns 0, or -1 on an iteration-limit hit. */
int oracle_march_count(int64_t n_rays, const float* rays_o, const float* rays_d, const float* t_min,
                       const float* t_max, const float* jitter, const float* roi,
                       const uint8_t* bits, int rx, int ry, int rz, float step, float cone,
                       int64_t max_iters, int32_t* num_steps) {
  const float lo[3] = {roi[0], roi[1], roi[2]}, hi[3] = {roi[3], roi[4], roi[5]};
  const int res[3] = {rx, ry, rz};
  for (int64_t i = 0; i < n_rays; ++i) {
    float near = t_min[i];
    if (jitter) near = near + jitter[i] * step;
    int64_t c = march_ray(rays_o + 3 * i, rays_d + 3 * i, near, t_max[i], step, cone, lo, hi, res,
                          bits, max_iters, 0, 0);
    if (c < 0) return -1;
    num_steps[i] = (int32_t)c;
  }
  return 0;
}

/* Fill round at exclusive-prefix offsets of num_steps. */
int oracle_march_fill(int64_t n_rays, const float* rays_o, const float* rays_d, const float* t_min,
                      const float* t_max, const float* jitter, const float* roi, const uint8_t* bits,
                      int rx, int ry, int rz, float step, float cone, int64_t max_iters,
                      const int32_t* num_steps, int64_t* ray_indices, float* t_starts,
                      float* t_ends) {
  const float lo[3] = {roi[0], roi[1], roi[2]}, hi[3] = {roi[3], roi[4], roi[5]};
  const int res[3] = {rx, ry, rz};
  int64_t base = 0;
  for (int64_t i = 0; i < n_rays; ++i) {
    float near = t_min[i];
    if (jitter) near = near + jitter[i] * step;
    int64_t c = march_ray(rays_o + 3 * i, rays_d + 3 * i, near, t_max[i], step, cone, lo, hi, res,
                          bits, max_iters, t_starts + base, t_ends + base);
    if (c < 0) return -1;
    for (int64_t j = 0; j < c; ++j) ray_indices[base + j] = i;
    base += num_steps[i];
  }
  return 0;
}

/* Occupancy-grid query points (NA/nerfacc/grid.py:210-225).  grid_coords is
 * the "ij" meshgrid of the resolution (grid.py:296-312), so cell
 * c = (x * ry + y) * rz + z; u = (coords + jitter) / resolution in float32
 * (an exact int -> float conversion, then one addition and one division),
 * then unit_to_roi, u * (hi - lo) + lo
 * (NA/nerfacc/cuda/csrc/include/helpers_contraction.h:23-28), whose multiply
 * and add nvcc contracts into one FMA.  cells == NULL: cell i.  AABB only. */
void oracle_occ_points(int64_t n, const int64_t* cells, const float* jitter, int rx, int ry,
                       int rz, const float* roi, float* x) {
  const float res[3] = {(float)rx, (float)ry, (float)rz};
  for (int64_t i = 0; i < n; ++i) {
    const int64_t c = cells ? cells[i] : i;
    const int64_t co[3] = {c / ((int64_t)ry * rz), (c / rz) % ry, c % rz};
    for (int d = 0; d < 3; ++d) {
      const float u = ((float)co[d] + jitter[3 * i + d]) / res[d];
      x[3 * i + d] = fmaf(u, roi[3 + d] - roi[d], roi[d]);
    }
  }
}

/* unit_to_roi alone (helpers_contraction.h:23-28): x = fma(u, hi - lo, lo). */
void oracle_unit_to_roi(int64_t n, const float* u, const float* roi, float* x) {
  for (int64_t i = 0; i < n; ++i)
    for (int d = 0; d < 3; ++d) x[3 * i + d] = fmaf(u[3 * i + d], roi[3 + d] - roi[d], roi[d]);
}
