// Occupancy-grid ray marching, sample packing and grid queries.
//
// The marcher restates nerfacc's fixed-step marcher with empty-space
// skipping (NA/nerfacc/cuda/csrc/ray_marching.cu:9-192,
// NA/nerfacc/cuda/csrc/include/helpers_contraction.h:16-114) so that, for
// the same rays, t_min, step size and grid, the emitted samples are
// bit-identical: every floating-point operation below is written with an
// explicit rounding intrinsic in the order the reference evaluates it.
// nvcc contracts the reference's `origin + t_mid * dir` into one FMA
// (default -fmad=true); all other products there are exact scalings by 0.5
// or are not followed by an addition, so they are plain roundings.
#include "common.cuh"
#include "scan.cuh"

#include <string.h>

#include <mutex>

namespace sn {

static thread_local char g_err[512];
static unsigned long long g_launches = 0;

void count_launches(int k) { __atomic_fetch_add(&g_launches, (unsigned long long)k, __ATOMIC_RELAXED); }

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

int num_sms() {
  static int cached = 0;
  if (cached == 0) {
    int dev = 0, v = 0;
    if (cudaGetDevice(&dev) == cudaSuccess &&
        cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess && v > 0)
      cached = v;
    else
      cached = 132;
  }
  return cached;
}

// Scans each tile, adds the tile offset and writes packed_info = {offset, count}.
__global__ void __launch_bounds__(kScanThreads)
scan_tile_apply(const int32_t* __restrict__ in, int64_t n, const int32_t* __restrict__ tile_offsets,
                int32_t* __restrict__ packed, int32_t* __restrict__ total,
                const int32_t* __restrict__ live = nullptr) {
  if (live) n = min(n, (int64_t)*live);   // entries at or past *live are neither read nor written
  if ((int64_t)blockIdx.x * kScanTile >= n) {
    if (!tile_offsets && threadIdx.x == 0 && total) *total = 0;
    return;
  }
  const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
  int v[kScanItems], c[kScanItems];
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) c[i] = v[i] = (base + i < n) ? in[base + i] : 0;
  int tot = block_exclusive_scan(v);
  const int off = tile_offsets ? tile_offsets[blockIdx.x] : 0;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) {
    if (base + i < n) {
      int2 pk = make_int2(v[i] + off, c[i]);
      reinterpret_cast<int2*>(packed)[base + i] = pk;
    }
  }
  if (!tile_offsets && threadIdx.x == 0 && total) *total = tot;
}

int pack_counts(int64_t n, const int32_t* counts, int32_t* packed, int32_t* total, void* ws,
                cudaStream_t st, const int32_t* live = nullptr) {
  if (n == 0) {
    if (total) {
      if (cudaMemsetAsync(total, 0, sizeof(int32_t), st) != cudaSuccess) {
        set_error("pack_counts: memset failed");
        return SN_ERR_CUDA;
      }
    }
    return SN_OK;
  }
  const int64_t n_tiles = (n + kScanTile - 1) / kScanTile;
  if (n_tiles == 1) {
    scan_tile_apply<<<1, kScanThreads, 0, st>>>(counts, n, nullptr, packed, total, live);
    return check_launch("pack_counts");
  }
  SN_REQUIRE(ws != nullptr, "pack_counts: workspace required for n=%lld", (long long)n);
  int32_t* tiles = reinterpret_cast<int32_t*>(ws);
  scan_tile_reduce<<<(unsigned)n_tiles, kScanThreads, 0, st>>>(counts, n, tiles, live);
  scan_tile_offsets<<<1, kScanThreads, 0, st>>>(tiles, n_tiles, total, live, n);
  scan_tile_apply<<<(unsigned)n_tiles, kScanThreads, 0, st>>>(counts, n, tiles, packed, nullptr, live);
  return check_launch("pack_counts", 3);
}

struct SmemLimit {
  int dev;
  const void* fn;
  size_t bytes;
};
static std::mutex g_smem_mu;
static SmemLimit g_smem_set[64];
static int g_smem_n = 0;

int ensure_smem_limit(const void* fn, size_t bytes, const char* what) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    set_error("%s: cudaGetDevice failed: %s", what, cudaGetErrorString(e));
    return SN_ERR_CUDA;
  }
  std::lock_guard<std::mutex> lock(g_smem_mu);
  for (int i = 0; i < g_smem_n; ++i)
    if (g_smem_set[i].dev == dev && g_smem_set[i].fn == fn && g_smem_set[i].bytes >= bytes) return SN_OK;
  e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e != cudaSuccess) {
    set_error("%s: cannot set the shared memory limit to %zu bytes: %s", what, bytes, cudaGetErrorString(e));
    return SN_ERR_CUDA;
  }
  if (g_smem_n < 64) g_smem_set[g_smem_n++] = SmemLimit{dev, fn, bytes};
  return SN_OK;
}

// Static scratch of sn_pack_counts_static: tile sums of up to kPackStaticMaxTiles
// tiles.  Its device address is looked up once per device (with that device
// current) and cached for the life of the process.  cudaDeviceReset destroys
// the module that holds the array, and a later call would write through the
// stale address, so a process that resets a device must not call the entry
// point on that device again.
constexpr int64_t kPackStaticMaxTiles = 4096;
constexpr int64_t kPackStaticMaxEntries = kPackStaticMaxTiles * kScanTile;
static __device__ __align__(256) int32_t g_pack_scratch[kPackStaticMaxTiles];
constexpr int kPackScratchDevices = 64;
static std::mutex g_pack_scratch_mu;
static int32_t* g_pack_scratch_ptr[kPackScratchDevices];

int pack_scratch_for_current_device(int32_t** out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    set_error("pack_counts_static: cudaGetDevice failed: %s", cudaGetErrorString(e));
    return SN_ERR_CUDA;
  }
  SN_REQUIRE(dev >= 0 && dev < kPackScratchDevices, "pack_counts_static: device %d out of range", dev);
  std::lock_guard<std::mutex> lock(g_pack_scratch_mu);
  if (!g_pack_scratch_ptr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_pack_scratch);
    if (e != cudaSuccess || p == nullptr) {
      set_error("pack_counts_static: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
      return SN_ERR_CUDA;
    }
    g_pack_scratch_ptr[dev] = static_cast<int32_t*>(p);
  }
  *out = g_pack_scratch_ptr[dev];
  return SN_OK;
}

// ---------------------------------------------------------------------------
// counts / unpack
// ---------------------------------------------------------------------------
__global__ void count_indices_kernel(int64_t n, const int64_t* __restrict__ idx, int64_t n_rays,
                                     int32_t* __restrict__ counts) {
  // warp-uniform loop so the whole warp takes part in every ballot/match
  const int lane = threadIdx.x & 31;
  const int64_t warp0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) - lane;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t b = warp0; b < n; b += stride) {
    const int64_t s = b + lane;
    const int64_t r = s < n ? idx[s] : -1;
    const bool ok = r >= 0 && r < n_rays;
    const unsigned m = __ballot_sync(0xffffffffu, ok);
    if (ok) {
      // samples of one ray are usually adjacent: one atomic per distinct key
      const unsigned peers = __match_any_sync(m, r);
      if (lane == __ffs(peers) - 1) atomicAdd(&counts[r], __popc(peers));
    }
  }
}

__global__ void unpack_info_kernel(int64_t n_rays, const int32_t* __restrict__ packed,
                                   int64_t n_samples, int64_t* __restrict__ out) {
  // one warp per ray: lanes write the ray's samples cooperatively
  const int lane = threadIdx.x & 31;
  for (int64_t r = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; r < n_rays;
       r += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    const int base = packed[2 * r], cnt = packed[2 * r + 1];
    for (int j = lane; j < cnt; j += 32) {
      int64_t s = (int64_t)base + j;
      if (s < n_samples) out[s] = r;
    }
  }
}

// ---------------------------------------------------------------------------
// marcher
// ---------------------------------------------------------------------------
struct GridView {
  const float* roi;  // device, 6 floats: {min xyz, max xyz}
  float lo[3], hi[3];
  int res[3];
  const uint8_t* bits;
  int ctype;
  float ext[3], rext[3], rres[3];  // extent; exact reciprocals of extent and resolution, or 0
};

// 1/v when v is a normal power of two (then x * (1/v) rounds exactly as x / v,
// both being the correctly rounded value of the same real number), else 0.
__device__ __forceinline__ float pow2_recip(float v) {
  const uint32_t b = __float_as_uint(v);
  const uint32_t e = (b >> 23) & 0xFFu;
  const bool p2 = (b & 0x807FFFFFu) == 0u && e >= 1u && e <= 253u;
  return p2 ? __uint_as_float((254u - e) << 23) : 0.0f;
}
// x / v, as a multiplication when r = pow2_recip(v) is nonzero (same bits).
__device__ __forceinline__ float div_by(float x, float v, float r) {
  return r != 0.0f ? __fmul_rn(x, r) : __fdiv_rn(x, v);
}

__device__ __forceinline__ void load_roi(GridView& g) {
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    g.lo[d] = g.roi[d];
    g.hi[d] = g.roi[3 + d];
    g.ext[d] = __fsub_rn(g.hi[d], g.lo[d]);
    g.rext[d] = pow2_recip(g.ext[d]);
    g.rres[d] = pow2_recip((float)g.res[d]);
  }
}

// roi -> [0,1]^3 and the two unbounded contractions
// (NA/nerfacc/cuda/csrc/include/helpers_contraction.h:16-114).
__device__ __forceinline__ void contract(const GridView& g, const float p[3], float u[3]) {
#pragma unroll
  for (int d = 0; d < 3; ++d) u[d] = div_by(__fsub_rn(p[d], g.lo[d]), g.ext[d], g.rext[d]);
  if (g.ctype == SN_CONTRACTION_UN_BOUNDED_TANH) {
#pragma unroll
    for (int d = 0; d < 3; ++d) u[d] = __fmaf_rn(tanhf(__fsub_rn(u[d], 0.5f)), 0.5f, 0.5f);
  } else if (g.ctype == SN_CONTRACTION_UN_BOUNDED_SPHERE) {
#pragma unroll
    for (int d = 0; d < 3; ++d) u[d] = __fmaf_rn(u[d], 2.0f, -1.0f);
    float nsq = __fmaf_rn(u[2], u[2], __fmaf_rn(u[1], u[1], __fmul_rn(u[0], u[0])));
    float nrm = sqrtf(nsq);
    if (nrm > 1.0f) {
      float k = __fsub_rn(2.0f, __fdiv_rn(1.0f, nrm));
#pragma unroll
      for (int d = 0; d < 3; ++d) u[d] = __fmul_rn(k, __fdiv_rn(u[d], nrm));
    }
#pragma unroll
    for (int d = 0; d < 3; ++d) u[d] = __fmaf_rn(u[d], 0.25f, 0.5f);
  }
}

// grid_occupied_at + grid_idx_at (NA/nerfacc/cuda/csrc/ray_marching.cu:16-45):
// AABB rejection, contraction, truncating int conversion, clamp, x-major index.
__device__ __forceinline__ bool occupied_at(const GridView& g, const float p[3]) {
  if (g.ctype == SN_CONTRACTION_AABB &&
      (p[0] < g.lo[0] || p[0] > g.hi[0] || p[1] < g.lo[1] || p[1] > g.hi[1] ||
       p[2] < g.lo[2] || p[2] > g.hi[2]))
    return false;
  float u[3];
  contract(g, p, u);
  int ix[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    int v = (int)__fmul_rn(u[d], (float)g.res[d]);
    v = v < 0 ? 0 : v;
    v = v > g.res[d] - 1 ? g.res[d] - 1 : v;
    ix[d] = v;
  }
  const int idx = ix[0] * (g.res[1] * g.res[2]) + ix[1] * g.res[2] + ix[2];
  return g.bits[idx] != 0;
}

// distance_to_next_voxel + advance_to_next_voxel
// (NA/nerfacc/cuda/csrc/ray_marching.cu:47-75): DDA target, then stepping in
// dt_min increments (at least one) so samples stay on the marching lattice.
__device__ __forceinline__ float advance_voxel(const GridView& g, float t, float dt_min,
                                               const float p[3], const float dir[3],
                                               const float inv[3], float far) {
  float tx[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const float ext = g.ext[d];
    const float res = (float)g.res[d];
    const float xu = __fmul_rn(div_by(__fsub_rn(p[d], g.lo[d]), ext, g.rext[d]), res);
    const float f = floorf(__fadd_rn(__fadd_rn(xu, 0.5f), copysignf(0.5f, dir[d])));
    tx[d] = __fmul_rn(div_by(__fmul_rn(__fsub_rn(f, xu), inv[d]), res, g.rres[d]), ext);
  }
  float dist = fminf(fminf(tx[0], tx[1]), tx[2]);
  dist = fmaxf(dist, 0.0f);
  float target = fminf(__fadd_rn(t, dist), far);
  float s = t;
  do {
    s = __fadd_rn(s, dt_min);
  } while (s < target);
  return s;
}

__device__ __forceinline__ float calc_dt(float t, float cone, float dt_min, float dt_max) {
  return fminf(fmaxf(__fmul_rn(t, cone), dt_min), dt_max);
}

struct MarchArgs {
  int64_t n_rays;
  const float* rays_o;
  const float* rays_d;
  const float* t_min;
  const float* t_max;
  const float* jitter;
  GridView grid;
  float step;
  const float* step_dev;  // nullable: the step size in device memory (overrides step)
  float cone;
  int64_t max_iters;
  const int32_t* packed;
  int64_t capacity;
  int32_t* num_steps;
  int64_t* ray_indices;
  float* t_starts;
  float* t_ends;
  int32_t* status;
};

// Warp-per-ray marcher with speculative occupied runs.  The reference marcher
// (NA/nerfacc/cuda/csrc/ray_marching.cu:135-185) walks one ray sequentially:
//   while t_mid < far: if occupied(origin + t_mid*dir): emit [t0, t1], t0 = t1,
//   t1 = t0 + dt, t_mid = (t0 + t1)/2; else t_mid = DDA skip, t0/t1 = t_mid -/+ dt/2.
// Here the same samples come out bit for bit.  From a state (t0, t1), lane l forms the state
// after l consecutive occupied steps with exactly the sequential additions
// (t0' = t1, t1' = t0' + dt, at most 31 of them), all 32 lanes look up the grid
// at their t_mid in one round trip, and a ballot finds the first lane that is
// empty or past `far`.  Lanes before it are samples; that lane's state is the
// sequential marcher's state at the same point, from which it takes the DDA
// skip (or the marcher stops), and the warp restarts from the broadcast state.
// Modes: count only (num_steps), fill at packed_info offsets, or fill into
// fixed slots ray*slot_stride (padded; num_steps written too).
// CONE false: cone_angle == 0, where calc_dt(t) = clamp(t * 0, dt_min, dt_max)
// is dt_min for every t, so each speculative step is one addition.
// Lanes that speculate on consecutive DDA skips through empty space.  Lane l
// forms l skips one after another, so a round costs a chain of kSkipLanes - 1
// skips plus one grid round trip; on the bench workload's trained grid 8
// lanes beat 12, 16, 24 and 32 (0.097 / 0.098 / 0.100 / 0.111 / 0.118 ms per
// marching stage, two rounds each, identical samples).
constexpr int kSkipLanes = 8;

template <int MODE, bool CONE>  // MODE: 0 count, 1 fill packed, 2 fill padded
__global__ void __launch_bounds__(128) march_warp_kernel(MarchArgs a, int64_t slot_stride) {
  const auto step_dt = [&](float t, float cone, float lo, float hi) {
    return CONE ? calc_dt(t, cone, lo, hi) : lo;
  };
  const int lane = threadIdx.x & 31;
  const int64_t ray = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  if (ray >= a.n_rays) return;  // whole warp exits together
  GridView g = a.grid;
  load_roi(g);
  float o[3], d[3], inv[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    o[k] = a.rays_o[3 * ray + k];
    d[k] = a.rays_d[3 * ray + k];
    inv[k] = __fdiv_rn(1.0f, d[k]);
  }
  const float step = a.step_dev ? *a.step_dev : a.step;
  float near = a.t_min[ray];
  const float far = a.t_max[ray];
  if (a.jitter) near = __fadd_rn(near, __fmul_rn(a.jitter[ray], step));
  int64_t base = 0, room = 0;
  if (MODE == 1) {
    base = a.packed[2 * ray];
    room = a.packed[2 * ray + 1];
  } else if (MODE == 2) {
    base = ray * slot_stride;
    room = slot_stride;
  }
  const float dt_min = step, dt_max = 1e10f;
  int64_t j = 0, iters = 0;
  float t0 = near;
  float dt = step_dt(t0, a.cone, dt_min, dt_max);
  float t1 = __fadd_rn(t0, dt);
  // t_mid of the current state: (t0 + t1) / 2 after an occupied step, but the
  // skip's own result after a DDA skip (the sequential loop tests that value)
  float tm0 = __fmul_rn(__fadd_rn(t0, t1), 0.5f);
  bool overflow = false, limit = false;
  while (true) {
    // state after `lane` occupied steps, as the sequential additions form it:
    // l1 = s_lane, l0 = s_(lane-1) (t0 for lane 0) with s_0 = t1 and
    // s_(k+1) = fl(s_k + dt).  With a constant dt, s_k is guessed in closed
    // form (t1 + k delta, one rounding) and every lane checks its own step
    // against the sequential rule; all steps agreeing makes every guess the
    // sequential value (induction from s_0).  Otherwise (a binade crossing
    // that rounds, a tie, cone > 0) the additions are replayed one by one.
    float l0 = t0, l1 = t1;
    bool exact = false;
    if (!CONE) {
      const float delta = __fsub_rn(__fadd_rn(t1, dt_min), t1);
      if (lane > 0) {
        l0 = __fmaf_rn((float)(lane - 1), delta, t1);
        l1 = __fmaf_rn((float)lane, delta, t1);
      }
      exact = __all_sync(0xffffffffu, lane == 0 || __fadd_rn(l0, dt_min) == l1);
      if (!exact) {
        l0 = t0;
        l1 = t1;
      }
    }
    if (!exact) {
      for (int s = 0; s < lane; ++s) {
        l0 = l1;
        l1 = __fadd_rn(l0, step_dt(l0, a.cone, dt_min, dt_max));
      }
    }
    const float tm = lane == 0 ? tm0 : __fmul_rn(__fadd_rn(l0, l1), 0.5f);
    float p[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) p[k] = __fmaf_rn(tm, d[k], o[k]);
    const bool inside = tm < far;
    const bool occ = inside && occupied_at(g, p);
    const unsigned empty = __ballot_sync(0xffffffffu, !occ);
    const int m = empty ? __ffs(empty) - 1 : 32;  // occupied run length
    if (lane < m && MODE != 0) {
      const int64_t jj = j + lane;
      if (jj < room && base + jj < a.capacity) {
        a.t_starts[base + jj] = l0;
        a.t_ends[base + jj] = l1;
        a.ray_indices[base + jj] = ray;
      } else {
        overflow = true;
      }
    }
    j += m;
    iters += m + 1;
    if (m == 32) {  // the whole warp was occupied: continue after lane 31
      t0 = __shfl_sync(0xffffffffu, l1, 31);
      t1 = __fadd_rn(t0, step_dt(t0, a.cone, dt_min, dt_max));
      tm0 = __fmul_rn(__fadd_rn(t0, t1), 0.5f);
    } else {
      // lane m holds the sequential state at the first non-occupied position
      const bool done = !__shfl_sync(0xffffffffu, inside, m);
      if (done) break;
      float ntm = 0.0f, n0 = 0.0f, n1 = 0.0f;
      if (lane == m) {
        if (g.ctype == SN_CONTRACTION_AABB) {
          ntm = advance_voxel(g, tm, dt_min, p, d, inv, far);
          const float ndt = step_dt(ntm, a.cone, dt_min, dt_max);
          n0 = __fsub_rn(ntm, __fmul_rn(ndt, 0.5f));
          n1 = __fadd_rn(ntm, __fmul_rn(ndt, 0.5f));
        } else {
          n0 = l1;
          n1 = __fadd_rn(n0, step_dt(n0, a.cone, dt_min, dt_max));
          ntm = __fmul_rn(__fadd_rn(n0, n1), 0.5f);
        }
      }
      t0 = __shfl_sync(0xffffffffu, n0, m);
      t1 = __shfl_sync(0xffffffffu, n1, m);
      ntm = __shfl_sync(0xffffffffu, ntm, m);
      tm0 = ntm;
      if (!(ntm < far)) break;
      // the sequential loop re-tests occupancy at ntm from state (t0, t1):
      // the next speculation round starts there (its lane 0 is that test)
      if (m == 0 && g.ctype == SN_CONTRACTION_AABB) {
        // Empty space (the round's first position was empty): speculate on
        // the skips instead.  Lane l takes l further DDA skips from ntm, each
        // from the position the previous one reached, as the sequential loop
        // would if every one of them were empty; all lanes then test their
        // positions in one round trip.  The first lane that is occupied, or
        // past far, is where the sequential loop stops skipping, so every
        // state formed here is the sequential one.
        bool finished = false;
        float base_tm = ntm;
        while (true) {
          float tm_l = base_tm;
          for (int s = 1; s < kSkipLanes; ++s) {
            if (lane >= s && tm_l < far) {
              float q[3];
#pragma unroll
              for (int k = 0; k < 3; ++k) q[k] = __fmaf_rn(tm_l, d[k], o[k]);
              tm_l = advance_voxel(g, tm_l, dt_min, q, d, inv, far);
            }
          }
          const bool in = lane < kSkipLanes && tm_l < far;
          bool oc = false;
          if (in) {
            float q[3];
#pragma unroll
            for (int k = 0; k < 3; ++k) q[k] = __fmaf_rn(tm_l, d[k], o[k]);
            oc = occupied_at(g, q);
          }
          const unsigned stop = __ballot_sync(0xffffffffu, lane < kSkipLanes && (oc || !in));
          if (stop) {
            const int k = __ffs(stop) - 1;
            const float tk = __shfl_sync(0xffffffffu, tm_l, k);
            iters += k;
            if (!(tk < far)) {
              finished = true;
            } else {
              const float ndt = step_dt(tk, a.cone, dt_min, dt_max);
              t0 = __fsub_rn(tk, __fmul_rn(ndt, 0.5f));
              t1 = __fadd_rn(tk, __fmul_rn(ndt, 0.5f));
              tm0 = tk;   // occupied: the next round's lane 0 emits there
            }
            break;
          }
          // all kSkipLanes positions empty and before far: skip on from the last
          const float tl = __shfl_sync(0xffffffffu, tm_l, kSkipLanes - 1);
          float q[3];
#pragma unroll
          for (int k = 0; k < 3; ++k) q[k] = __fmaf_rn(tl, d[k], o[k]);
          base_tm = advance_voxel(g, tl, dt_min, q, d, inv, far);
          iters += kSkipLanes;
          if (!(base_tm < far)) {
            finished = true;
            break;
          }
          if (iters > a.max_iters) break;
        }
        if (finished) break;
      }
    }
    if (iters > a.max_iters) {
      limit = true;
      break;
    }
  }
  if (lane == 0) {
    if (MODE != 1) a.num_steps[ray] = (int32_t)j;
    if (limit) atomicOr(a.status, SN_STATUS_MARCH_LIMIT);
  }
  if (MODE != 0 && __any_sync(0xffffffffu, overflow) && lane == 0) atomicOr(a.status, SN_STATUS_CAPACITY);
}

// Copy padded per-ray samples (ray*stride + j, j < count) to packed offsets.
__global__ void compact_padded_kernel(int64_t n_rays, int64_t stride, const int32_t* __restrict__ packed,
                                      const int64_t* __restrict__ ri_in, const float* __restrict__ ts_in,
                                      const float* __restrict__ te_in, int64_t* __restrict__ ri_out,
                                      float* __restrict__ ts_out, float* __restrict__ te_out) {
  const int lane = threadIdx.x & 31;
  for (int64_t r = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; r < n_rays;
       r += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    const int64_t b = packed[2 * r];
    const int c = packed[2 * r + 1];
    for (int j = lane; j < c; j += 32) {
      ri_out[b + j] = ri_in[r * stride + j];
      ts_out[b + j] = ts_in[r * stride + j];
      te_out[b + j] = te_in[r * stride + j];
    }
  }
}

__global__ void grid_query_kernel(int64_t n, const float* __restrict__ x, GridView g,
                                  uint8_t* __restrict__ out) {
  load_roi(g);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    float p[3] = {x[3 * i], x[3 * i + 1], x[3 * i + 2]};
    out[i] = occupied_at(g, p) ? 1 : 0;
  }
}

// ---------------------------------------------------------------------------
// occupancy grid maintenance
// ---------------------------------------------------------------------------
// contract_inv for the three contraction types
// (NA/nerfacc/cuda/csrc/include/helpers_contraction.h:23-129).
__device__ __forceinline__ void contract_inv(const float lo[3], const float hi[3], int ctype,
                                             float u[3]) {
  if (ctype == SN_CONTRACTION_UN_BOUNDED_TANH) {
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      float v = atanhf(__fmaf_rn(u[d], 2.0f, -1.0f));
      v = fminf(fmaxf(v, -1e10f), 1e10f);
      u[d] = __fadd_rn(v, 0.5f);
    }
  } else if (ctype == SN_CONTRACTION_UN_BOUNDED_SPHERE) {
#pragma unroll
    for (int d = 0; d < 3; ++d) u[d] = __fmul_rn(__fsub_rn(u[d], 0.5f), 4.0f);
    float nsq = __fmaf_rn(u[2], u[2], __fmaf_rn(u[1], u[1], __fmul_rn(u[0], u[0])));
    float nrm = sqrtf(nsq);
    if (nrm > 1.0f) {
      float den = fmaxf(__fsub_rn(__fmul_rn(2.0f, nrm), __fmul_rn(1.0f, nsq)), 1e-10f);
#pragma unroll
      for (int d = 0; d < 3; ++d) u[d] = __fdiv_rn(u[d], den);
    }
#pragma unroll
    for (int d = 0; d < 3; ++d) u[d] = __fmaf_rn(u[d], 0.5f, 0.5f);
  }
#pragma unroll
  for (int d = 0; d < 3; ++d) u[d] = __fmaf_rn(u[d], __fsub_rn(hi[d], lo[d]), lo[d]);
}

__global__ void occ_points_kernel(int64_t n, const int64_t* __restrict__ cells,
                                  const float* __restrict__ jitter, int rx, int ry, int rz,
                                  const float* __restrict__ roi, int ctype, float* __restrict__ x) {
  float lo[3], hi[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    lo[d] = roi[d];
    hi[d] = roi[3 + d];
  }
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = cells ? cells[i] : i;
    const int64_t cz = c % rz, cy = (c / rz) % ry, cx = c / ((int64_t)ry * rz);
    float u[3];
    u[0] = __fdiv_rn(__fadd_rn((float)cx, jitter[3 * i + 0]), (float)rx);
    u[1] = __fdiv_rn(__fadd_rn((float)cy, jitter[3 * i + 1]), (float)ry);
    u[2] = __fdiv_rn(__fadd_rn((float)cz, jitter[3 * i + 2]), (float)rz);
    contract_inv(lo, hi, ctype, u);
    x[3 * i + 0] = u[0];
    x[3 * i + 1] = u[1];
    x[3 * i + 2] = u[2];
  }
}

constexpr int kReduceThreads = 512;

__global__ void __launch_bounds__(kReduceThreads)
occ_partial_sum(int64_t n, const float* __restrict__ occs, double* __restrict__ partial) {
  double s = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    s += (double)occs[i];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  __shared__ double ws[kReduceThreads / 32];
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    double t = threadIdx.x < kReduceThreads / 32 ? ws[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if (threadIdx.x == 0) partial[blockIdx.x] = t;
  }
}

__global__ void __launch_bounds__(kReduceThreads)
occ_threshold_kernel(int64_t n, const float* __restrict__ occs, const double* __restrict__ partial,
                     int n_partial, float thre, uint8_t* __restrict__ binary, float* mean_out) {
  __shared__ float s_thr;
  if (threadIdx.x < 32) {
    double t = 0.0;
    for (int k = threadIdx.x; k < n_partial; k += 32) t += partial[k];
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if (threadIdx.x == 0) {
      const float mean = (float)(t / (double)n);
      s_thr = fminf(mean, thre);
      if (mean_out && blockIdx.x == 0) *mean_out = mean;
    }
  }
  __syncthreads();
  const float thr = s_thr;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    binary[i] = occs[i] > thr ? 1 : 0;
}

// ---- device-side occupancy update (no host synchronisation) ----------------
// Query points of cells[i] (or cell i) with in-kernel jitter for i < *count.
__global__ void occ_points_n_kernel(int64_t cap, const int32_t* __restrict__ count,
                                    const int64_t* __restrict__ cells, uint64_t seed,
                                    const int32_t* __restrict__ stream_dev, int rx, int ry, int rz,
                                    const float* __restrict__ roi, int ctype, float* __restrict__ x) {
  const int64_t n = count ? min((int64_t)*count, cap) : cap;
  const uint64_t sid = stream_dev ? (uint64_t)(uint32_t)*stream_dev : 0ull;
  float lo[3], hi[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    lo[d] = roi[d];
    hi[d] = roi[3 + d];
  }
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = cells ? cells[i] : i;
    const int64_t cz = c % rz, cy = (c / rz) % ry, cx = c / ((int64_t)ry * rz);
    float u[3];
    u[0] = __fdiv_rn(__fadd_rn((float)cx, uniform01(seed, sid, 3 * (uint64_t)i + 0)), (float)rx);
    u[1] = __fdiv_rn(__fadd_rn((float)cy, uniform01(seed, sid, 3 * (uint64_t)i + 1)), (float)ry);
    u[2] = __fdiv_rn(__fadd_rn((float)cz, uniform01(seed, sid, 3 * (uint64_t)i + 2)), (float)rz);
    contract_inv(lo, hi, ctype, u);
    x[3 * i + 0] = u[0];
    x[3 * i + 1] = u[1];
    x[3 * i + 2] = u[2];
  }
}

// EMA update of the occupancy values (NA/nerfacc/grid.py:229-230:
// occs[indices] = max(occs[indices] * decay, occ)).  With cells == nullptr
// every cell appears once (the warm-up sweep) and one pass updates it in
// place.  Sampled cells may repeat, and every candidate must be formed from
// the cell's value before the update, so the sampled form takes three passes:
//   (1) vals[i] = max(occs[c] * decay, occ_i)       (reads occs only)
//   (2) occs[c] = vals[i]                            (a repeated cell keeps any one)
//   (3) atomicMax(occs[c], vals[i])                  (... then the largest)
// A repeated cell ends at max(old * decay, max_i occ_i): one of the values
// the reference's unordered index_put can store, and the one the scatter-max
// it names as intended gives.  occs >= 0 (an EMA of sigmoid values), so the
// float order equals the int order of the bit patterns.
__device__ __forceinline__ float occ_from_sdf(float sdf, float k) {
  // torch.sigmoid(-sdf * k) (models/renderer.py:56-60): 1 / (1 + exp(sdf * k))
  return 1.0f / (1.0f + expf(__fmul_rn(sdf, k)));
}

template <bool kFromSdf>
__global__ void occ_ema_value_kernel(int64_t cap, const int32_t* __restrict__ count,
                                     const int64_t* __restrict__ cells, const float* __restrict__ in,
                                     float k, float decay, float* __restrict__ occs,
                                     float* __restrict__ vals) {
  const int64_t n = count ? min((int64_t)*count, cap) : cap;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = cells ? cells[i] : i;
    const float occ = kFromSdf ? occ_from_sdf(in[i], k) : in[i];
    const float v = fmaxf(__fmul_rn(occs[c], decay), occ);
    if (cells)
      vals[i] = v;
    else
      occs[c] = v;
  }
}

__global__ void occ_ema_store_kernel(int64_t cap, const int32_t* __restrict__ count,
                                     const int64_t* __restrict__ cells, const float* __restrict__ vals,
                                     float* __restrict__ occs) {
  const int64_t n = count ? min((int64_t)*count, cap) : cap;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    occs[cells[i]] = vals[i];
}

__global__ void occ_ema_max_kernel(int64_t cap, const int32_t* __restrict__ count,
                                   const int64_t* __restrict__ cells, const float* __restrict__ vals,
                                   float* __restrict__ occs) {
  const int64_t n = count ? min((int64_t)*count, cap) : cap;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    atomicMax(reinterpret_cast<int*>(occs) + cells[i], __float_as_int(fmaxf(vals[i], 0.0f)));
}

// Launches the one-pass (all cells) or three-pass (sampled cells) update.
template <bool kFromSdf>
static int occ_ema_launch(int64_t cap, const int32_t* count, const int64_t* cells, const float* in,
                          float k, float decay, float* occs, float* vals, cudaStream_t st,
                          const char* what) {
  const unsigned g = stride_grid(cap, 256, 8);
  occ_ema_value_kernel<kFromSdf><<<g, 256, 0, st>>>(cap, count, cells, in, k, decay, occs, vals);
  if (!cells) return check_launch(what);
  occ_ema_store_kernel<<<g, 256, 0, st>>>(cap, count, cells, vals, occs);
  occ_ema_max_kernel<<<g, 256, 0, st>>>(cap, count, cells, vals, occs);
  return check_launch(what, 3);
}

__global__ void __launch_bounds__(kScanThreads)
u8_tile_count(const uint8_t* __restrict__ bits, int64_t n, int32_t* __restrict__ tile_sums) {
  const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
  int s = 0;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i)
    if (base + i < n) s += bits[base + i] ? 1 : 0;
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

__global__ void __launch_bounds__(kScanThreads)
u8_tile_compact(const uint8_t* __restrict__ bits, int64_t n, const int32_t* __restrict__ tile_off,
                int32_t* __restrict__ list) {
  const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
  int v[kScanItems], f[kScanItems];
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) f[i] = v[i] = (base + i < n && bits[base + i]) ? 1 : 0;
  block_exclusive_scan(v);
  const int off = tile_off[blockIdx.x];
#pragma unroll
  for (int i = 0; i < kScanItems; ++i)
    if (f[i]) list[off + v[i]] = (int32_t)(base + i);
}

// cells[0, n_uniform) uniform over the grid; then min(n_occ, n_uniform)
// occupied cells (all of them, or a uniform draw when there are more),
// as NA/nerfacc/grid.py:168-182 does; *count = total.
__global__ void occ_select_kernel(int64_t n_cells, int64_t n_uniform, const int32_t* __restrict__ list,
                                  const int32_t* __restrict__ n_occ_dev, uint64_t seed,
                                  const int32_t* __restrict__ stream_dev, int64_t* __restrict__ cells,
                                  int32_t* __restrict__ count) {
  const int64_t n_occ = *n_occ_dev;
  const uint64_t sid = stream_dev ? (uint64_t)(uint32_t)*stream_dev : 0ull;
  const int64_t n_take = n_occ < n_uniform ? n_occ : n_uniform;
  if (blockIdx.x == 0 && threadIdx.x == 0) *count = (int32_t)(n_uniform + n_take);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n_uniform;
       i += (int64_t)gridDim.x * blockDim.x) {
    cells[i] = (int64_t)(uniform_u32(seed, sid ^ 0x5151u, (uint64_t)i) % (uint64_t)n_cells);
    if (i < n_take) {
      const int64_t j = n_occ > n_uniform
                            ? (int64_t)(uniform_u32(seed, sid ^ 0xA3A3u, (uint64_t)i) % (uint64_t)n_occ)
                            : i;
      cells[n_uniform + i] = list[j];
    }
  }
}

static int make_grid(GridView& g, const float* roi, const uint8_t* bits, int rx, int ry, int rz,
                     int ctype) {
  SN_REQUIRE(roi != nullptr, "roi is null");
  g.roi = roi;
  SN_REQUIRE(rx > 0 && ry > 0 && rz > 0, "grid resolution must be positive (%d,%d,%d)", rx, ry, rz);
  SN_REQUIRE(ctype >= 0 && ctype <= 2, "unknown contraction type %d", ctype);
  SN_REQUIRE(bits != nullptr, "grid_binary is null");
  g.res[0] = rx;
  g.res[1] = ry;
  g.res[2] = rz;
  g.bits = bits;
  g.ctype = ctype;
  return SN_OK;
}

}  // namespace sn

using namespace sn;

extern "C" {

const char* sn_version(void) { return "supernormal_gb300 0.1.0 (sm_103a)"; }

const char* sn_last_error(void) { return sn::g_err; }

uint64_t sn_kernel_launches(void) { return __atomic_load_n(&sn::g_launches, __ATOMIC_RELAXED); }

size_t sn_scan_workspace_bytes(int64_t n) {
  const int64_t n_tiles = (n + sn::kScanTile - 1) / sn::kScanTile;
  size_t b = (size_t)(n_tiles > 0 ? n_tiles : 1) * sizeof(int32_t);
  return (b + 255) & ~(size_t)255;
}

int sn_pack_counts(int64_t n, const int32_t* counts, int32_t* packed_info, int32_t* total,
                   void* workspace, void* stream) {
  SN_REQUIRE(n >= 0, "pack_counts: n < 0");
  SN_REQUIRE(n <= ((int64_t)1 << 31) - 1, "pack_counts: n too large");
  SN_REQUIRE(n == 0 || (counts && packed_info), "pack_counts: null buffer");
  return sn::pack_counts(n, counts, packed_info, total, workspace, as_stream(stream));
}

// sn_pack_counts without a caller workspace: the multi-tile scan's tile sums
// live in a file-scope device array, so the call allocates nothing.  Limit:
// kPackStaticMaxTiles tiles of kScanTile entries (16,777,216 entries, 16 KiB of
// scratch).  Nothing in the scratch has to start at zero (every tile sum is
// written by scan_tile_reduce before scan_tile_offsets reads it).  The scratch
// is one per device, so calls that overlap on the device (other streams or
// host threads) race on it.
int sn_pack_counts_n(int64_t cap, const int32_t* count, const int32_t* counts, int32_t* packed_info,
                     int32_t* total, void* workspace, void* stream) {
  SN_REQUIRE(cap >= 0, "pack_counts_n: cap < 0");
  SN_REQUIRE(cap <= ((int64_t)1 << 31) - 1, "pack_counts_n: cap too large");
  SN_REQUIRE(count != nullptr, "pack_counts_n: a device count is required");
  SN_REQUIRE(cap == 0 || (counts && packed_info), "pack_counts_n: null buffer");
  return sn::pack_counts(cap, counts, packed_info, total, workspace, as_stream(stream), count);
}

int sn_pack_counts_static(int64_t n, const int32_t* counts, int32_t* packed_info, int32_t* total,
                          void* stream) {
  SN_REQUIRE(n >= 0, "pack_counts_static: n < 0");
  SN_REQUIRE(n <= sn::kPackStaticMaxEntries,
             "pack_counts_static: n = %lld exceeds the static scratch limit of %lld entries",
             (long long)n, (long long)sn::kPackStaticMaxEntries);
  SN_REQUIRE(n == 0 || (counts && packed_info), "pack_counts_static: null buffer");
  int32_t* scratch = nullptr;
  SN_TRY(sn::pack_scratch_for_current_device(&scratch));
  return sn::pack_counts(n, counts, packed_info, total, scratch, as_stream(stream));
}

int sn_count_indices(int64_t n_samples, const int64_t* ray_indices, int64_t n_rays, int32_t* counts,
                     void* stream) {
  SN_REQUIRE(n_samples >= 0 && n_rays >= 0, "count_indices: negative size");
  cudaStream_t st = as_stream(stream);
  if (n_rays > 0 && cudaMemsetAsync(counts, 0, (size_t)n_rays * sizeof(int32_t), st) != cudaSuccess) {
    set_error("count_indices: memset failed");
    return SN_ERR_CUDA;
  }
  if (n_samples == 0) return SN_OK;
  count_indices_kernel<<<stride_grid(n_samples, 256, 8), 256, 0, st>>>(n_samples, ray_indices,
                                                                       n_rays, counts);
  return check_launch("count_indices");
}

int sn_unpack_info(int64_t n_rays, const int32_t* packed_info, int64_t n_samples,
                   int64_t* ray_indices, void* stream) {
  SN_REQUIRE(n_rays >= 0 && n_samples >= 0, "unpack_info: negative size");
  if (n_rays == 0 || n_samples == 0) return SN_OK;
  unpack_info_kernel<<<stride_grid(n_rays * 32, 256, 8), 256, 0, as_stream(stream)>>>(
      n_rays, packed_info, n_samples, ray_indices);
  return check_launch("unpack_info");
}

static int march_common(MarchArgs& a, int64_t n_rays, const float* rays_o, const float* rays_d,
                        const float* t_min, const float* t_max, const float* jitter,
                        const float* roi, const uint8_t* grid_binary, int rx, int ry, int rz,
                        int ctype, float step, float cone, int64_t max_iters, int32_t* status) {
  SN_REQUIRE(n_rays >= 0, "march: n_rays < 0");
  SN_REQUIRE(step > 0.0f && step < 1e30f, "march: step_size must be positive and finite (got %g)",
             (double)step);
  SN_REQUIRE(cone >= 0.0f && cone < 1e30f, "march: cone_angle must be >= 0 (got %g)", (double)cone);
  SN_REQUIRE(status != nullptr, "march: a device status word is required");
  SN_REQUIRE(roi != nullptr, "march: roi is null");
  memset(&a, 0, sizeof(a));
  SN_TRY(make_grid(a.grid, roi, grid_binary, rx, ry, rz, ctype));
  a.n_rays = n_rays;
  a.rays_o = rays_o;
  a.rays_d = rays_d;
  a.t_min = t_min;
  a.t_max = t_max;
  a.jitter = jitter;
  a.step = step;
  a.cone = cone;
  a.max_iters = max_iters > 0 ? max_iters : ((int64_t)1 << 24);
  a.status = status;
  return SN_OK;
}


int sn_march_count(int64_t n_rays, const float* rays_o, const float* rays_d, const float* t_min,
                   const float* t_max, const float* jitter, const float* roi,
                   const uint8_t* grid_binary, int rx, int ry, int rz, int contraction_type,
                   float step_size, float cone_angle, int64_t max_iters, int32_t* num_steps,
                   int32_t* status, void* stream) {
  MarchArgs a;
  SN_TRY(march_common(a, n_rays, rays_o, rays_d, t_min, t_max, jitter, roi, grid_binary, rx, ry, rz,
                      contraction_type, step_size, cone_angle, max_iters, status));
  if (n_rays == 0) return SN_OK;
  a.num_steps = num_steps;
  if (a.cone == 0.0f)
    march_warp_kernel<0, false><<<div_up(n_rays * 32, 128), 128, 0, as_stream(stream)>>>(a, 0);
  else
    march_warp_kernel<0, true><<<div_up(n_rays * 32, 128), 128, 0, as_stream(stream)>>>(a, 0);
  return check_launch("march_count");
}

int sn_march_padded(int64_t n_rays, const float* rays_o, const float* rays_d, const float* t_min,
                    const float* t_max, const float* jitter, const float* roi,
                    const uint8_t* grid_binary, int rx, int ry, int rz, int contraction_type,
                    float step_size, const float* step_size_dev, float cone_angle,
                    int64_t max_iters, int64_t slot_stride, int32_t* num_steps,
                    int64_t* ray_indices, float* t_starts, float* t_ends, int32_t* status,
                    void* stream) {
  MarchArgs a;
  SN_TRY(march_common(a, n_rays, rays_o, rays_d, t_min, t_max, jitter, roi, grid_binary, rx, ry, rz,
                      contraction_type, step_size, cone_angle, max_iters, status));
  SN_REQUIRE(slot_stride > 0, "march_padded: slot_stride must be positive");
  a.step_dev = step_size_dev;
  SN_REQUIRE(num_steps && ray_indices && t_starts && t_ends, "march_padded: null output");
  if (n_rays == 0) return SN_OK;
  a.num_steps = num_steps;
  a.capacity = n_rays * slot_stride;
  a.ray_indices = ray_indices;
  a.t_starts = t_starts;
  a.t_ends = t_ends;
  if (a.cone == 0.0f)
    march_warp_kernel<2, false><<<div_up(n_rays * 32, 128), 128, 0, as_stream(stream)>>>(a, slot_stride);
  else
    march_warp_kernel<2, true><<<div_up(n_rays * 32, 128), 128, 0, as_stream(stream)>>>(a, slot_stride);
  return check_launch("march_padded");
}

int sn_compact_padded(int64_t n_rays, int64_t slot_stride, const int32_t* packed_info,
                      const int64_t* ray_indices_in, const float* t_starts_in,
                      const float* t_ends_in, int64_t* ray_indices_out, float* t_starts_out,
                      float* t_ends_out, void* stream) {
  SN_REQUIRE(n_rays >= 0 && slot_stride > 0, "compact_padded: bad sizes");
  if (n_rays == 0) return SN_OK;
  compact_padded_kernel<<<stride_grid(n_rays * 32, 256, 8), 256, 0, as_stream(stream)>>>(
      n_rays, slot_stride, packed_info, ray_indices_in, t_starts_in, t_ends_in, ray_indices_out,
      t_starts_out, t_ends_out);
  return check_launch("compact_padded");
}

int sn_march_fill(int64_t n_rays, const float* rays_o, const float* rays_d, const float* t_min,
                  const float* t_max, const float* jitter, const float* roi,
                  const uint8_t* grid_binary, int rx, int ry, int rz, int contraction_type,
                  float step_size, float cone_angle, int64_t max_iters,
                  const int32_t* packed_info, int64_t capacity, int64_t* ray_indices,
                  float* t_starts, float* t_ends, int32_t* status, void* stream) {
  MarchArgs a;
  SN_TRY(march_common(a, n_rays, rays_o, rays_d, t_min, t_max, jitter, roi, grid_binary, rx, ry, rz,
                      contraction_type, step_size, cone_angle, max_iters, status));
  SN_REQUIRE(capacity >= 0, "march_fill: capacity < 0");
  if (n_rays == 0) return SN_OK;
  SN_REQUIRE(packed_info != nullptr, "march_fill: packed_info is null");
  a.packed = packed_info;
  a.capacity = capacity;
  a.ray_indices = ray_indices;
  a.t_starts = t_starts;
  a.t_ends = t_ends;
  if (a.cone == 0.0f)
    march_warp_kernel<1, false><<<div_up(n_rays * 32, 128), 128, 0, as_stream(stream)>>>(a, 0);
  else
    march_warp_kernel<1, true><<<div_up(n_rays * 32, 128), 128, 0, as_stream(stream)>>>(a, 0);
  return check_launch("march_fill");
}

int sn_grid_query(int64_t n, const float* samples, const float* roi, const uint8_t* grid_binary,
                  int rx, int ry, int rz, int contraction_type, uint8_t* out, void* stream) {
  SN_REQUIRE(n >= 0, "grid_query: n < 0");
  GridView g;
  memset(&g, 0, sizeof(g));
  SN_TRY(make_grid(g, roi, grid_binary, rx, ry, rz, contraction_type));
  if (n == 0) return SN_OK;
  grid_query_kernel<<<stride_grid(n, 256, 8), 256, 0, as_stream(stream)>>>(n, samples, g, out);
  return check_launch("grid_query");
}

int sn_occ_points(int64_t n, const int64_t* cells, const float* jitter, int rx, int ry, int rz,
                  const float* roi, int contraction_type, float* x_out, void* stream) {
  SN_REQUIRE(n >= 0, "occ_points: n < 0");
  SN_REQUIRE(rx > 0 && ry > 0 && rz > 0, "occ_points: bad resolution");
  SN_REQUIRE(contraction_type >= 0 && contraction_type <= 2, "occ_points: bad contraction");
  SN_REQUIRE(roi && jitter && x_out, "occ_points: null buffer");
  if (n == 0) return SN_OK;
  occ_points_kernel<<<stride_grid(n, 256, 8), 256, 0, as_stream(stream)>>>(
      n, cells, jitter, rx, ry, rz, roi, contraction_type, x_out);
  return check_launch("occ_points");
}

int sn_occ_ema_update(int64_t n, const int64_t* cells, const float* occ, float ema_decay,
                      float* occs, float* workspace, void* stream) {
  SN_REQUIRE(n >= 0, "occ_ema_update: n < 0");
  SN_REQUIRE(ema_decay >= 0.0f, "occ_ema_update: ema_decay < 0");
  SN_REQUIRE(occ && occs, "occ_ema_update: null buffer");
  SN_REQUIRE(!cells || workspace, "occ_ema_update: sampled cells need a workspace of n floats");
  if (n == 0) return SN_OK;
  return occ_ema_launch<false>(n, nullptr, cells, occ, 0.0f, ema_decay, occs, workspace,
                               as_stream(stream), "occ_ema_update");
}

size_t sn_occ_binarize_workspace_bytes(int64_t n_cells) {
  (void)n_cells;
  return (size_t)(4 * 1024) * sizeof(double);
}

int sn_occ_binarize(int64_t n_cells, const float* occs, float occ_thre, uint8_t* binary,
                    float* mean_out, void* workspace, void* stream) {
  SN_REQUIRE(n_cells > 0, "occ_binarize: n_cells must be > 0");
  SN_REQUIRE(workspace != nullptr, "occ_binarize: workspace required");
  cudaStream_t st = as_stream(stream);
  int nb = (int)stride_grid(n_cells, kReduceThreads, 4);
  if (nb > 4096) nb = 4096;
  double* partial = reinterpret_cast<double*>(workspace);
  occ_partial_sum<<<nb, kReduceThreads, 0, st>>>(n_cells, occs, partial);
  occ_threshold_kernel<<<stride_grid(n_cells, kReduceThreads, 4), kReduceThreads, 0, st>>>(
      n_cells, occs, partial, nb, occ_thre, binary, mean_out);
  return check_launch("occ_binarize", 2);
}

}  // extern "C"

extern "C" {

int sn_occ_points_n(int64_t cap, const int32_t* count, const int64_t* cells, uint64_t seed,
                    const int32_t* stream_counter, int rx, int ry, int rz, const float* roi,
                    int contraction_type, float* x_out, void* stream) {
  SN_REQUIRE(cap >= 0, "occ_points_n: cap < 0");
  SN_REQUIRE(rx > 0 && ry > 0 && rz > 0, "occ_points_n: bad resolution");
  SN_REQUIRE(contraction_type >= 0 && contraction_type <= 2, "occ_points_n: bad contraction");
  SN_REQUIRE(roi && x_out, "occ_points_n: null buffer");
  if (cap == 0) return SN_OK;
  occ_points_n_kernel<<<stride_grid(cap, 256, 8), 256, 0, as_stream(stream)>>>(
      cap, count, cells, seed, stream_counter, rx, ry, rz, roi, contraction_type, x_out);
  return check_launch("occ_points_n");
}

int sn_occ_ema_sdf(int64_t cap, const int32_t* count, const int64_t* cells, const float* sdf,
                   float sigmoid_k, float ema_decay, float* occs, float* workspace, void* stream) {
  SN_REQUIRE(cap >= 0, "occ_ema_sdf: cap < 0");
  SN_REQUIRE(sdf && occs, "occ_ema_sdf: null buffer");
  SN_REQUIRE(!cells || workspace, "occ_ema_sdf: sampled cells need a workspace of cap floats");
  if (cap == 0) return SN_OK;
  return occ_ema_launch<true>(cap, count, cells, sdf, sigmoid_k, ema_decay, occs, workspace,
                              as_stream(stream), "occ_ema_sdf");
}

size_t sn_occ_sample_workspace_bytes(int64_t n_cells) {
  const int64_t n_tiles = (n_cells + sn::kScanTile - 1) / sn::kScanTile;
  size_t b = (size_t)(n_tiles + 1) * sizeof(int32_t) + 256;   // tile offsets + total
  b += (size_t)n_cells * sizeof(int32_t);                      // occupied list
  return (b + 255) & ~(size_t)255;
}

int sn_occ_sample_cells(int64_t n_cells, const uint8_t* binary, int64_t n_uniform, uint64_t seed,
                        const int32_t* stream_counter, int64_t* cells, int32_t* count,
                        void* workspace, void* stream) {
  SN_REQUIRE(n_cells > 0 && n_uniform >= 0, "occ_sample_cells: bad sizes");
  SN_REQUIRE(binary && cells && count && workspace, "occ_sample_cells: null buffer");
  cudaStream_t st = as_stream(stream);
  const int64_t n_tiles = (n_cells + kScanTile - 1) / kScanTile;
  int32_t* tiles = reinterpret_cast<int32_t*>(workspace);
  int32_t* n_occ = tiles + n_tiles;
  int32_t* list = reinterpret_cast<int32_t*>(
      (reinterpret_cast<uintptr_t>(tiles + n_tiles + 1) + 255) & ~(uintptr_t)255);
  u8_tile_count<<<(unsigned)n_tiles, kScanThreads, 0, st>>>(binary, n_cells, tiles);
  scan_tile_offsets<<<1, kScanThreads, 0, st>>>(tiles, n_tiles, n_occ);
  u8_tile_compact<<<(unsigned)n_tiles, kScanThreads, 0, st>>>(binary, n_cells, tiles, list);
  occ_select_kernel<<<stride_grid(n_uniform > 0 ? n_uniform : 1, 256, 8), 256, 0, st>>>(
      n_cells, n_uniform, list, n_occ, seed, stream_counter, cells, count);
  return check_launch("occ_sample_cells", 4);
}

}  // extern "C"
