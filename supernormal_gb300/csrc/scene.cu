// Ground truth of the synthetic analytic scenes on the device.
//
// The training data of the benchmarks are multi-view normal maps and masks
// of analytic SDF scenes (sphere, displaced torus, box, and unions of them
// with a displacement), standing in for the DiLiGenT-MV captures the
// reference trains on (models/dataset_loader.py).  One thread per pixel:
// the ray of pixel (x, y) of view v is R_v * normalize(K_v^-1 [x, y, 1])
// from the camera centre (models/dataset_loader.py:223-277 conventions),
// clipped to the unit sphere, sphere-traced in double precision with a
// Lipschitz-bounded step, and the world normal at the hit is the normalised
// central-difference gradient of the SDF (step 1e-6, double).  A miss gives
// a zero normal and mask 0.
#include "common.cuh"

namespace sn {

__device__ double prim_sdf(const sn_prim& pr, const double p[3]) {
  const double q0 = p[0] - (double)pr.center[0], q1 = p[1] - (double)pr.center[1],
               q2 = p[2] - (double)pr.center[2];
  if (pr.kind == SN_PRIM_SPHERE) return sqrt(q0 * q0 + q1 * q1 + q2 * q2) - (double)pr.size[0];
  if (pr.kind == SN_PRIM_TORUS) {
    // torus around z: ring radius R = size[0], tube radius r = size[1], with a
    // radial displacement amp * sin(f theta) * sin(f phi)
    const double rxy = sqrt(q0 * q0 + q1 * q1);
    const double ring = rxy - (double)pr.size[0];
    double d = sqrt(ring * ring + q2 * q2) - (double)pr.size[1];
    if (pr.amp != 0.0f) {
      const double th = atan2(q1, q0), ph = atan2(q2, ring);
      d -= (double)pr.amp * sin((double)pr.freq * th) * sin((double)pr.freq * ph);
    }
    return d;
  }
  // box with half extents size[]
  const double a0 = fabs(q0) - (double)pr.size[0], a1 = fabs(q1) - (double)pr.size[1],
               a2 = fabs(q2) - (double)pr.size[2];
  const double o0 = fmax(a0, 0.0), o1 = fmax(a1, 0.0), o2 = fmax(a2, 0.0);
  return sqrt(o0 * o0 + o1 * o1 + o2 * o2) + fmin(fmax(a0, fmax(a1, a2)), 0.0);
}

__device__ double scene_sdf(const sn_scene_desc& s, const double p[3]) {
  double d = prim_sdf(s.prims[0], p);
  for (int k = 1; k < s.n_prims; ++k) d = fmin(d, prim_sdf(s.prims[k], p));
  if (s.disp_amp != 0.0f) {
    const double f = (double)s.disp_freq;
    d -= (double)s.disp_amp * sin(f * p[0]) * sin(f * p[1]) * sin(f * p[2]);
  }
  return d;
}

__global__ void scene_gt_kernel(sn_scene_desc s, int64_t n_pix, int H, int W,
                                const double* __restrict__ kinv, const double* __restrict__ pose,
                                int max_iters, double eps, float* __restrict__ normals,
                                float* __restrict__ masks) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n_pix;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t v = i / ((int64_t)H * W);
    const int rem = (int)(i - v * (int64_t)H * W);
    const int y = rem / W, x = rem - y * W;
    const double* Ki = kinv + 9 * v;
    const double* Pv = pose + 12 * v;
    double c[3], d[3], o[3];
    for (int r = 0; r < 3; ++r) c[r] = Ki[3 * r + 0] * x + Ki[3 * r + 1] * y + Ki[3 * r + 2];
    const double cn = sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
    for (int r = 0; r < 3; ++r) c[r] /= cn;
    for (int r = 0; r < 3; ++r) {
      d[r] = Pv[4 * r + 0] * c[0] + Pv[4 * r + 1] * c[1] + Pv[4 * r + 2] * c[2];
      o[r] = Pv[4 * r + 3];
    }
    // unit-sphere chord (models/dataset_loader.py:279-297 near_far_from_sphere)
    const double a = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
    const double b = 2.0 * (o[0] * d[0] + o[1] * d[1] + o[2] * d[2]);
    const double cc = o[0] * o[0] + o[1] * o[1] + o[2] * o[2] - 1.0;
    const double disc = sqrt(fmax(b * b - 4.0 * a * cc, 0.0));
    const double mid = -0.5 * b / a;
    double t = mid - disc / (2.0 * a);
    const double far = mid + disc / (2.0 * a);
    const double lip = (double)s.lipschitz;
    bool hit = false;
    for (int it = 0; it < max_iters && t < far; ++it) {
      const double p[3] = {o[0] + d[0] * t, o[1] + d[1] * t, o[2] + d[2] * t};
      const double sd = scene_sdf(s, p);
      if (fabs(sd) < eps) {
        hit = true;
        break;
      }
      t += sd / lip * 0.9;
    }
    float nrm[3] = {0.0f, 0.0f, 0.0f};
    if (hit) {
      const double p[3] = {o[0] + d[0] * t, o[1] + d[1] * t, o[2] + d[2] * t};
      const double h = 1e-6;
      double g[3];
      for (int k = 0; k < 3; ++k) {
        double pp[3] = {p[0], p[1], p[2]}, pm[3] = {p[0], p[1], p[2]};
        pp[k] += h;
        pm[k] -= h;
        g[k] = (scene_sdf(s, pp) - scene_sdf(s, pm)) / (2.0 * h);
      }
      const double gn = fmax(sqrt(g[0] * g[0] + g[1] * g[1] + g[2] * g[2]), 1e-12);
      for (int k = 0; k < 3; ++k) nrm[k] = (float)(g[k] / gn);
    }
    for (int k = 0; k < 3; ++k) normals[3 * i + k] = nrm[k];
    masks[i] = hit ? 1.0f : 0.0f;
  }
}

__global__ void scene_sdf_kernel(sn_scene_desc s, int64_t n, const float* __restrict__ x,
                                 float* __restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double p[3] = {(double)x[3 * i], (double)x[3 * i + 1], (double)x[3 * i + 2]};
    out[i] = (float)scene_sdf(s, p);
  }
}

static int check_scene(const sn_scene_desc* s) {
  SN_REQUIRE(s != nullptr, "scene: null descriptor");
  SN_REQUIRE(s->n_prims >= 1 && s->n_prims <= SN_SCENE_MAX_PRIMS, "scene: %d primitives (1..%d)",
             s->n_prims, SN_SCENE_MAX_PRIMS);
  for (int k = 0; k < s->n_prims; ++k)
    SN_REQUIRE(s->prims[k].kind >= SN_PRIM_SPHERE && s->prims[k].kind <= SN_PRIM_BOX,
               "scene: primitive %d has unknown kind %d", k, s->prims[k].kind);
  SN_REQUIRE(s->lipschitz > 0.0f, "scene: lipschitz bound must be > 0");
  return SN_OK;
}

}  // namespace sn

using namespace sn;

extern "C" {

int sn_scene_render_gt(const sn_scene_desc* scene, int n_views, int H, int W, const double* kinv,
                       const double* pose, int max_iters, double eps, float* normals, float* masks,
                       void* stream) {
  SN_TRY(check_scene(scene));
  SN_REQUIRE(n_views >= 0 && H > 0 && W > 0 && max_iters > 0 && eps > 0.0, "scene_render_gt: bad sizes");
  SN_REQUIRE(kinv && pose && normals && masks, "scene_render_gt: null buffer");
  const int64_t n = (int64_t)n_views * H * W;
  if (n == 0) return SN_OK;
  scene_gt_kernel<<<stride_grid(n, 128, 16), 128, 0, as_stream(stream)>>>(*scene, n, H, W, kinv, pose,
                                                                          max_iters, eps, normals, masks);
  return check_launch("scene_render_gt");
}

int sn_scene_sdf(const sn_scene_desc* scene, int64_t n, const float* x, float* out, void* stream) {
  SN_TRY(check_scene(scene));
  SN_REQUIRE(n >= 0, "scene_sdf: n < 0");
  SN_REQUIRE(n == 0 || (x && out), "scene_sdf: null buffer");
  if (n == 0) return SN_OK;
  scene_sdf_kernel<<<stride_grid(n, 256, 8), 256, 0, as_stream(stream)>>>(*scene, n, x, out);
  return check_launch("scene_sdf");
}

}  // extern "C"
