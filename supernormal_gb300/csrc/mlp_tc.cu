// Tensor-core (tcgen05) pieces of the SDF network's MLP.
//
// sn_linear_tc: y = x W^T + b for the first layer of SDFNetwork
// (models/fields.py:90-99: in = [x, enc] -> Linear(din, 64)), fp32-accurate
// through 3xTF32 on the tensor cores.  One CTA of 128 threads per 128-row
// tile (persistent over tiles); thread t owns row t: it splits its row into
// TF32 hi/lo parts and stores them into its own TMEM lane (A operand), one
// thread issues the MMAs against W (hi/lo) held in shared memory in the
// canonical K-major layout, and every thread reads its row of D back from
// TMEM.  Nothing is staged through shared memory per row.
#include "common.cuh"
#include "tc.cuh"

namespace sn {

constexpr int kTcRows = 128;   // rows per tile (M)
constexpr int kTcN = 64;       // output features (hidden width)
constexpr int kTcMaxK = 64;    // input features handled (padded to a multiple of 8)
constexpr uint32_t kTcCols = 256;  // TMEM columns allocated per CTA
// Dynamic shared memory requested by every tensor-core kernel here: more than
// a third of the SM's 228 KB, so at most two CTAs (2 x 256 TMEM columns) share an SM.
constexpr size_t kTcSmemFloor = 80 * 1024;


struct LinearTcArgs {
  int64_t n;
  int k, kp;          // input features, padded to a multiple of 8
  const float* x;     // (n, k)
  const float* w;     // (64, k)
  const float* b;     // (64) or null
  float* y;           // (n, 64)
  int32_t* status;
};

// TMEM columns: D [0, 64), A_hi [64, 64 + kp), A_lo [64 + kp, 64 + 2 kp).
__global__ void __launch_bounds__(kTcRows) linear_tc_kernel(LinearTcArgs a) {
  extern __shared__ __align__(1024) uint8_t smem[];
  const int kp = a.kp;
  const uint32_t wbytes = (uint32_t)kTcN * kp * 4u;
  uint8_t* w_hi = smem;
  uint8_t* w_lo = smem + wbytes;
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem + 2 * wbytes);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(smem + 2 * wbytes + 8);
  const int t = threadIdx.x, warp = t >> 5;

  // weights -> TF32 hi/lo, K-major core-matrix layout
  for (int e = t; e < kTcN * kp; e += blockDim.x) {
    const int r = e / kp, c = e - r * kp;
    const float v = c < a.k ? a.w[(int64_t)r * a.k + c] : 0.0f;
    uint32_t hi, lo;
    tc::tf32_split(v, hi, lo);
    const uint32_t off = tc::kmajor_offset(r, c, kp);
    *reinterpret_cast<uint32_t*>(w_hi + off) = hi;
    *reinterpret_cast<uint32_t*>(w_lo + off) = lo;
  }
  if (warp == 0) {
    tc::tmem_alloc(tmem_slot, kTcCols);
    tc::tmem_relinquish();
  }
  if (t == 0) tc::mbar_init(bar, 1);
  tc::fence_proxy_async_smem();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tbase = *tmem_slot;
  const uint32_t lane_base = (uint32_t)(32 * warp);
  const uint32_t idesc = tc::idesc_tf32(kTcRows, kTcN);
  const uint32_t sbo = (uint32_t)(kp / 4) * 128u;
  const uint32_t a_hi_col = kTcN, a_lo_col = kTcN + kp;
  uint32_t phase = 0;
  bool ok = true;

  const int64_t n_tiles = (a.n + kTcRows - 1) / kTcRows;
  for (int64_t tile = blockIdx.x; tile < n_tiles; tile += gridDim.x) {
    const int64_t row = tile * kTcRows + t;
    const bool live = row < a.n;
    // A rows: this thread's row, split, into its own lane
    for (int c0 = 0; c0 < kp; c0 += 8) {
      uint32_t hi[8], lo[8];
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const int c = c0 + i;
        const float v = (live && c < a.k) ? a.x[row * a.k + c] : 0.0f;
        tc::tf32_split(v, hi[i], lo[i]);
      }
      tc::tmem_st8(tc::taddr(tbase, lane_base, a_hi_col + c0), hi);
      tc::tmem_st8(tc::taddr(tbase, lane_base, a_lo_col + c0), lo);
    }
    tc::tmem_wait_st();
    tc::fence_before_sync();
    __syncthreads();
    if (t == 0) {
      tc::fence_after_sync();
      const uint32_t d = tc::taddr(tbase, 0, 0);
      const uint32_t s_hi = tc::smem_u32(w_hi), s_lo = tc::smem_u32(w_lo);
      uint32_t acc = 0;
      for (int ks = 0; ks < kp / 8; ++ks) {   // a_hi * w_hi
        tc::mma_ts(d, tc::taddr(tbase, 0, a_hi_col + 8 * ks), tc::smem_desc(s_hi + 256u * ks, 128u, sbo),
                   idesc, acc);
        acc = 1;
      }
      for (int ks = 0; ks < kp / 8; ++ks)     // a_lo * w_hi
        tc::mma_ts(d, tc::taddr(tbase, 0, a_lo_col + 8 * ks), tc::smem_desc(s_hi + 256u * ks, 128u, sbo),
                   idesc, 1);
      for (int ks = 0; ks < kp / 8; ++ks)     // a_hi * w_lo
        tc::mma_ts(d, tc::taddr(tbase, 0, a_hi_col + 8 * ks), tc::smem_desc(s_lo + 256u * ks, 128u, sbo),
                   idesc, 1);
      tc::mma_commit(bar);
    }
    const bool got = tc::mbar_wait_bounded(bar, phase);
    phase ^= 1u;
    if (!__syncthreads_and(got)) {
      ok = false;
      break;
    }
    tc::fence_after_sync();
    // D row -> bias -> y
#pragma unroll
    for (int c0 = 0; c0 < kTcN; c0 += 16) {
      float v[16];
      tc::tmem_ld16(tc::taddr(tbase, lane_base, c0), v);
      tc::tmem_wait_ld();
      if (live) {
#pragma unroll
        for (int i = 0; i < 16; i += 4) {
          float4 o;
          o.x = v[i] + (a.b ? a.b[c0 + i] : 0.0f);
          o.y = v[i + 1] + (a.b ? a.b[c0 + i + 1] : 0.0f);
          o.z = v[i + 2] + (a.b ? a.b[c0 + i + 2] : 0.0f);
          o.w = v[i + 3] + (a.b ? a.b[c0 + i + 3] : 0.0f);
          *reinterpret_cast<float4*>(a.y + row * kTcN + c0 + i) = o;
        }
      }
    }
    tc::fence_before_sync();
    __syncthreads();
  }
  if (!ok) {
    if (t == 0) atomicOr(a.status, SN_STATUS_TIMEOUT);
    // drain: the commit of the last batch may still be pending
    (void)tc::mbar_wait_bounded(bar, phase ^ 1u);
    __syncthreads();
  }
  tc::fence_after_sync();
  if (warp == 0) tc::tmem_dealloc(tbase, kTcCols);
}

}  // namespace sn

using namespace sn;

extern "C" {

int sn_linear_tc(int64_t n, int k, const float* x, const float* w, const float* b, float* y,
                 int32_t* status, void* stream) {
  SN_REQUIRE(n >= 0, "linear_tc: n < 0");
  SN_REQUIRE(k >= 1 && k <= kTcMaxK, "linear_tc: k = %d outside 1..%d", k, kTcMaxK);
  SN_REQUIRE(w && status && (n == 0 || (x && y)), "linear_tc: null buffer");
  if (n == 0) return SN_OK;
  LinearTcArgs a;
  a.n = n;
  a.k = k;
  a.kp = (k + 7) / 8 * 8;
  a.x = x;
  a.w = w;
  a.b = b;
  a.y = y;
  a.status = status;
  // The shared-memory request also caps residency at two CTAs per SM, so the
  // two 256-column TMEM allocations per SM never wait on each other.
  const size_t smem = kTcSmemFloor;
  SN_TRY(ensure_smem_limit(reinterpret_cast<const void*>(linear_tc_kernel), smem, "linear_tc"));
  const int64_t n_tiles = (n + kTcRows - 1) / kTcRows;
  const int64_t grid = n_tiles < 2LL * num_sms() ? n_tiles : 2LL * num_sms();
  linear_tc_kernel<<<(unsigned)grid, kTcRows, smem, as_stream(stream)>>>(a);
  return check_launch("linear_tc");
}

}  // extern "C"
