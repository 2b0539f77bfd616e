// Mesh extraction on the device: SDF lattice query points and marching cubes.
//
// The reference extracts a mesh from the SDF on a res^3 lattice over the
// bounding box (models/renderer.py:9-34, extract_fields + extract_geometry,
// called from exp_runner.py for validation meshes and the Chamfer / F-score
// evaluation) with PyMCubes on the host.  Here the lattice points are formed
// per slab on the device, the field kernels evaluate them, and marching
// cubes runs as four passes over the lattice:
//   1. edge flags: a lattice edge carries a vertex when its two ends lie on
//      different sides of the threshold (inside: value > threshold);
//   2. exclusive scan of the flags -> vertex ids (shared by the cubes that
//      meet at the edge, so the mesh is indexed and watertight);
//   3. per cube: triangle count of its corner configuration, exclusive scan
//      -> triangle offsets;
//   4. vertices at the linear-interpolation crossing of each flagged edge,
//      and each cube's triangles as vertex ids.
//
// The triangle table is generated at compile time (make_mc_table) rather than
// transcribed: on every cube face the sign changes are paired so that each
// inside corner is cut off on its own (the same pairing from both cubes that
// share the face, so no cracks), the face segments are oriented from the
// crossing where the face boundary (counter-clockwise around the outward
// normal) enters the inside to the next crossing where it leaves, the
// segments chain into closed loops, and each loop is fanned into triangles
// from a vertex none of whose diagonals lies on a cube face; the right-hand
// normals then point from the inside to the outside.
#include "common.cuh"
#include "scan.cuh"

namespace sn {
namespace {

// Corner c of a cube is (dx, dy, dz) = (c & 1, c >> 1 & 1, c >> 2 & 1).
// Edge e = axis * 4 + the two other corner bits of its lower corner.
constexpr int kMcMaxTri = 5;

struct McTable {
  uint8_t ntri[256];
  int8_t edge[256][3 * kMcMaxTri];
  uint8_t max_tri;
};

constexpr int mc_edge_of(int c0, int axis) {
  return axis == 0 ? ((c0 >> 1) & 3) : axis == 1 ? (4 + ((c0 & 1) | (((c0 >> 2) & 1) << 1))) : (8 + (c0 & 3));
}

// Faces of the cube edge e as a 6-bit mask (bit 2 * axis + side).
constexpr int mc_edge_faces(int e) {
  const int axis = e >> 2, o = e & 3;
  const int x0 = axis == 0 ? 1 : 0, x1 = axis == 2 ? 1 : 2;  // the other two axes, low first
  return (1 << (2 * x0 + (o & 1))) | (1 << (2 * x1 + ((o >> 1) & 1)));
}

constexpr McTable make_mc_table() {
  McTable t{};
  t.max_tri = 0;
  for (int cs = 0; cs < 256; ++cs) {
    int next[12] = {-1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1};
    for (int a = 0; a < 3; ++a) {
      const int b = (a + 1) % 3, c = (a + 2) % 3;  // e_b x e_c = e_a
      for (int s = 0; s < 2; ++s) {
        // corners counter-clockwise around the outward normal (+e_a if s, else -e_a)
        int q[4] = {0, 0, 0, 0};
        const int bc[4][2] = {{0, 0}, {1, 0}, {1, 1}, {0, 1}};
        for (int i = 0; i < 4; ++i) {
          const int k = s ? i : (4 - i) % 4;
          q[i] = (s << a) | (bc[k][0] << b) | (bc[k][1] << c);
        }
        int cross_edge[4] = {0, 0, 0, 0};
        bool cross_entry[4] = {false, false, false, false};
        int nc = 0;
        for (int i = 0; i < 4; ++i) {
          const int p = q[i], r = q[(i + 1) % 4];
          const bool ip = (cs >> p) & 1, ir = (cs >> r) & 1;
          if (ip != ir) {
            const int lo = p < r ? p : r;
            const int axis = (p ^ r) == 1 ? 0 : (p ^ r) == 2 ? 1 : 2;
            cross_edge[nc] = mc_edge_of(lo, axis);
            cross_entry[nc] = ir;   // the boundary walk enters the inside here
            ++nc;
          }
        }
        for (int i = 0; i < nc; ++i) {
          if (!cross_entry[i]) continue;
          for (int j = 1; j < nc; ++j) {
            const int k = (i + j) % nc;
            if (!cross_entry[k]) {
              next[cross_edge[i]] = cross_edge[k];
              break;
            }
          }
        }
      }
    }
    bool seen[12] = {false, false, false, false, false, false, false, false, false, false, false, false};
    int nt = 0;
    for (int e0 = 0; e0 < 12; ++e0) {
      if (next[e0] < 0 || seen[e0]) continue;
      int loop[12] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
      int n = 0;
      for (int e = e0; !seen[e]; e = next[e]) {
        seen[e] = true;
        loop[n++] = e;
      }
      // fan apex: a vertex none of whose diagonals lies on a cube face, so no
      // diagonal can coincide with one of the neighbouring cube's (such a pair
      // would make the edge shared by four triangles); every loop has one
      int ap = 0;
      for (int c = 0; c < n; ++c) {
        bool good = true;
        for (int j = 0; j < n; ++j)
          if (j != c && j != (c + 1) % n && j != (c + n - 1) % n &&
              (mc_edge_faces(loop[c]) & mc_edge_faces(loop[j])) != 0)
            good = false;
        if (good) {
          ap = c;
          break;
        }
      }
      for (int i = 1; i + 1 < n; ++i) {
        t.edge[cs][3 * nt + 0] = (int8_t)loop[ap];
        t.edge[cs][3 * nt + 1] = (int8_t)loop[(ap + i) % n];
        t.edge[cs][3 * nt + 2] = (int8_t)loop[(ap + i + 1) % n];
        ++nt;
      }
    }
    t.ntri[cs] = (uint8_t)nt;
    if (nt > t.max_tri) t.max_tri = (uint8_t)nt;
  }
  return t;
}

constexpr McTable kMcHost = make_mc_table();
static_assert(kMcHost.max_tri <= kMcMaxTri, "marching-cubes table: too many triangles in a case");
static_assert(kMcHost.ntri[0] == 0 && kMcHost.ntri[255] == 0, "marching-cubes table: empty and full cubes");
static_assert(kMcHost.ntri[1] == 1 && kMcHost.ntri[3] == 2 && kMcHost.ntri[15] == 2,
              "marching-cubes table: corner, edge and face cases");
__constant__ McTable kMc = make_mc_table();

struct Lattice {
  int nx, ny, nz;
  int64_t n;        // nx * ny * nz
  float thr;
};

__device__ __forceinline__ int64_t lat(const Lattice& L, int64_t i, int64_t j, int64_t k) {
  return (i * L.ny + j) * L.nz + k;
}

// Flag of edge e = axis * n + lattice index of its lower end.
__device__ __forceinline__ int edge_flag(const Lattice& L, const float* u, int64_t e) {
  const int axis = (int)(e / L.n);
  const int64_t p = e - axis * L.n;
  const int64_t k = p % L.nz, j = (p / L.nz) % L.ny, i = p / ((int64_t)L.ny * L.nz);
  if ((axis == 0 && i + 1 >= L.nx) || (axis == 1 && j + 1 >= L.ny) || (axis == 2 && k + 1 >= L.nz)) return 0;
  const int64_t q = p + (axis == 0 ? (int64_t)L.ny * L.nz : axis == 1 ? (int64_t)L.nz : 1);
  return (u[p] > L.thr) != (u[q] > L.thr) ? 1 : 0;
}

__device__ __forceinline__ int cube_case(const Lattice& L, const float* u, int64_t i, int64_t j, int64_t k) {
  int cs = 0;
#pragma unroll
  for (int c = 0; c < 8; ++c)
    cs |= (u[lat(L, i + (c & 1), j + ((c >> 1) & 1), k + ((c >> 2) & 1))] > L.thr ? 1 : 0) << c;
  return cs;
}

// Per-tile sums of a generated int32 sequence (edge flags or triangle counts).
template <int KIND>  // 0: edge flags (3 n entries), 1: triangle counts per cube
__device__ __forceinline__ int mc_value(const Lattice& L, const float* u, int64_t idx) {
  if (KIND == 0) return edge_flag(L, u, idx);
  const int64_t cz = L.nz - 1, cy = L.ny - 1;
  const int64_t k = idx % cz, j = (idx / cz) % cy, i = idx / (cy * cz);
  return kMc.ntri[cube_case(L, u, i, j, k)];
}

template <int KIND>
__global__ void __launch_bounds__(kScanThreads)
mc_tile_reduce(Lattice L, const float* __restrict__ u, int64_t total, int32_t* __restrict__ tile_sums) {
  const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
  int s = 0;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i)
    if (base + i < total) s += mc_value<KIND>(L, u, base + i);
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  __shared__ int ws[32];
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    int t = ws[threadIdx.x];
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if (threadIdx.x == 0) tile_sums[blockIdx.x] = t;
  }
}

// Emits, per tile: the vertices of flagged edges (KIND 0) or the triangles
// of each cube (KIND 1) at the scanned offsets.  Triangles look up the
// vertex ids of their edges in vid (the scan of the edge flags, written by
// the KIND 0 pass).
template <int KIND>
__global__ void __launch_bounds__(kScanThreads)
mc_tile_emit(Lattice L, const float* __restrict__ u, int64_t total, const int32_t* __restrict__ tile_off,
             int32_t* __restrict__ vid, float3 origin, float3 spacing, float* __restrict__ verts,
             int32_t* __restrict__ tris, int64_t cap) {
  const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
  int v[kScanItems], f[kScanItems];
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) f[i] = v[i] = base + i < total ? mc_value<KIND>(L, u, base + i) : 0;
  block_exclusive_scan(v);
  const int off = tile_off[blockIdx.x];
#pragma unroll
  for (int it = 0; it < kScanItems; ++it) {
    const int64_t idx = base + it;
    if (idx >= total) break;
    const int id = v[it] + off;
    if (KIND == 0) {
      if (vid) vid[idx] = id;
      if (!f[it] || !verts || id >= cap) continue;
      const int axis = (int)(idx / L.n);
      const int64_t p = idx - axis * L.n;
      const int64_t k = p % L.nz, j = (p / L.nz) % L.ny, i = p / ((int64_t)L.ny * L.nz);
      const int64_t q = p + (axis == 0 ? (int64_t)L.ny * L.nz : axis == 1 ? (int64_t)L.nz : 1);
      const float u0 = u[p], u1 = u[q];
      const float t = (L.thr - u0) / (u1 - u0);
      float pos[3] = {(float)i, (float)j, (float)k};
      pos[axis] += t;
      verts[3 * (int64_t)id + 0] = fmaf(pos[0], spacing.x, origin.x);
      verts[3 * (int64_t)id + 1] = fmaf(pos[1], spacing.y, origin.y);
      verts[3 * (int64_t)id + 2] = fmaf(pos[2], spacing.z, origin.z);
    } else {
      if (!f[it]) continue;
      const int64_t cz = L.nz - 1, cy = L.ny - 1;
      const int64_t k = idx % cz, j = (idx / cz) % cy, i = idx / (cy * cz);
      const int cs = cube_case(L, u, i, j, k);
      for (int tri = 0; tri < f[it]; ++tri) {
        if (id + tri >= cap) break;
#pragma unroll
        for (int m = 0; m < 3; ++m) {
          const int e = kMc.edge[cs][3 * tri + m];
          const int axis = e >> 2, o = e & 3;
          const int b0 = o & 1, b1 = (o >> 1) & 1;  // the two other corner bits, low axis first
          const int64_t di = axis == 0 ? 0 : b0, dj = axis == 1 ? 0 : (axis == 0 ? b0 : b1),
                        dk = axis == 2 ? 0 : b1;
          tris[3 * (int64_t)(id + tri) + m] = vid[axis * L.n + lat(L, i + di, j + dj, k + dk)];
        }
      }
    }
  }
}

__global__ void lattice_points_kernel(int64_t i0, int64_t n_pts, int ny, int nz, double3 lo, double3 step,
                                      float* __restrict__ x) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n_pts;
       p += (int64_t)gridDim.x * blockDim.x) {
    const int64_t k = p % nz, j = (p / nz) % ny, i = i0 + p / ((int64_t)ny * nz);
    x[3 * p + 0] = (float)(lo.x + step.x * (double)i);
    x[3 * p + 1] = (float)(lo.y + step.y * (double)j);
    x[3 * p + 2] = (float)(lo.z + step.z * (double)k);
  }
}

__global__ void negate_kernel(int64_t n, const float* __restrict__ in, float* __restrict__ out) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x)
    out[p] = -in[p];
}

int64_t n_tiles_of(int64_t total) { return (total + kScanTile - 1) / kScanTile; }

}  // namespace
}  // namespace sn

using namespace sn;

extern "C" {

int sn_lattice_points(int64_t i0, int64_t n_i, int nx, int ny, int nz, const double* bound_min,
                      const double* bound_max, float* x_out, void* stream) {
  SN_REQUIRE(nx >= 2 && ny >= 2 && nz >= 2, "lattice_points: resolution must be >= 2 per axis");
  SN_REQUIRE(i0 >= 0 && n_i >= 0 && i0 + n_i <= nx, "lattice_points: slab [%lld, %lld) outside [0, %d)",
             (long long)i0, (long long)(i0 + n_i), nx);
  SN_REQUIRE(bound_min && bound_max && (n_i == 0 || x_out), "lattice_points: null buffer");
  const int64_t n = n_i * ny * nz;
  if (n == 0) return SN_OK;
  const double3 lo = make_double3(bound_min[0], bound_min[1], bound_min[2]);
  const double3 st = make_double3((bound_max[0] - bound_min[0]) / (nx - 1), (bound_max[1] - bound_min[1]) / (ny - 1),
                                  (bound_max[2] - bound_min[2]) / (nz - 1));
  lattice_points_kernel<<<stride_grid(n, 256, 8), 256, 0, as_stream(stream)>>>(i0, n, ny, nz, lo, st, x_out);
  return check_launch("lattice_points");
}

int sn_negate(int64_t n, const float* in, float* out, void* stream) {
  SN_REQUIRE(n >= 0 && (n == 0 || (in && out)), "negate: bad arguments");
  if (n == 0) return SN_OK;
  negate_kernel<<<stride_grid(n, 256, 8), 256, 0, as_stream(stream)>>>(n, in, out);
  return check_launch("negate");
}

size_t sn_marching_cubes_workspace_bytes(int nx, int ny, int nz) {
  if (nx < 2 || ny < 2 || nz < 2) return 0;
  const int64_t n = (int64_t)nx * ny * nz;
  const int64_t cubes = (int64_t)(nx - 1) * (ny - 1) * (nz - 1);
  size_t b = (size_t)(3 * n) * sizeof(int32_t);                              // vertex id per edge
  b += (size_t)(n_tiles_of(3 * n) + n_tiles_of(cubes) + 4) * sizeof(int32_t);  // tile sums + totals
  return (b + 255) & ~(size_t)255;
}

int sn_marching_cubes(const float* values, int nx, int ny, int nz, float threshold, const double* bound_min,
                      const double* bound_max, int64_t vert_cap, int64_t tri_cap, float* vertices,
                      int32_t* triangles, int32_t* counts, void* workspace, void* stream) {
  SN_REQUIRE(nx >= 2 && ny >= 2 && nz >= 2, "marching_cubes: resolution must be >= 2 per axis");
  const int64_t n = (int64_t)nx * ny * nz;
  SN_REQUIRE(3 * n < ((int64_t)1 << 31), "marching_cubes: %lld lattice edges exceed int32 ids", (long long)(3 * n));
  SN_REQUIRE(values && counts && workspace && bound_min && bound_max, "marching_cubes: null buffer");
  SN_REQUIRE(vert_cap >= 0 && tri_cap >= 0 && (vert_cap == 0 || vertices) && (tri_cap == 0 || triangles),
             "marching_cubes: output capacity without a buffer");
  cudaStream_t st = as_stream(stream);
  Lattice L{nx, ny, nz, n, threshold};
  const int64_t cubes = (int64_t)(nx - 1) * (ny - 1) * (nz - 1);
  int32_t* vid = reinterpret_cast<int32_t*>(workspace);
  int32_t* tiles_e = vid + 3 * n;
  const int64_t te = n_tiles_of(3 * n), tc = n_tiles_of(cubes);
  int32_t* tiles_c = tiles_e + te;
  const float3 origin = make_float3((float)bound_min[0], (float)bound_min[1], (float)bound_min[2]);
  const float3 spacing = make_float3((float)((bound_max[0] - bound_min[0]) / (nx - 1)),
                                     (float)((bound_max[1] - bound_min[1]) / (ny - 1)),
                                     (float)((bound_max[2] - bound_min[2]) / (nz - 1)));
  mc_tile_reduce<0><<<(unsigned)te, kScanThreads, 0, st>>>(L, values, 3 * n, tiles_e);
  scan_tile_offsets<<<1, kScanThreads, 0, st>>>(tiles_e, te, counts);
  mc_tile_emit<0><<<(unsigned)te, kScanThreads, 0, st>>>(L, values, 3 * n, tiles_e, vid, origin, spacing,
                                                         vertices, nullptr, vert_cap);
  mc_tile_reduce<1><<<(unsigned)tc, kScanThreads, 0, st>>>(L, values, cubes, tiles_c);
  scan_tile_offsets<<<1, kScanThreads, 0, st>>>(tiles_c, tc, counts + 1);
  mc_tile_emit<1><<<(unsigned)tc, kScanThreads, 0, st>>>(L, values, cubes, tiles_c, vid, origin, spacing,
                                                         nullptr, triangles, tri_cap);
  return check_launch("marching_cubes", 6);
}

}  // extern "C"
