// Block-wide and multi-tile exclusive scans of int32 (1024 threads x 4
// items = one 4096-entry tile), shared by the packing, occupancy and mesh
// kernels.  Internal linkage: each translation unit that includes this gets
// its own copies of the kernels.
#pragma once

#include "common.cuh"

namespace sn {
namespace {

constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;

// Exclusive scan of v[] (ITEMS consecutive entries per thread, thread-major);
// returns the block total.  Requires blockDim.x == kScanThreads.
__device__ int block_exclusive_scan(int (&v)[kScanItems]) {
  __shared__ int warp_tot[kScanThreads / 32];
  int run = 0;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) {
    int t = v[i];
    v[i] = run;
    run += t;
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int incl = run;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  if (lane == 31) warp_tot[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    int w = warp_tot[lane];
    int wi = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, wi, o);
      if (lane >= o) wi += y;
    }
    warp_tot[lane] = wi - w;  // exclusive warp offsets
  }
  __syncthreads();
  const int off = warp_tot[warp] + incl - run;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) v[i] += off;
  int total = warp_tot[31];
  // the last warp's exclusive offset + its inclusive total = block total
  __shared__ int s_total;
  if (threadIdx.x == kScanThreads - 1) s_total = off + run;
  __syncthreads();
  total = s_total;
  __syncthreads();
  return total;
}

__global__ void __launch_bounds__(kScanThreads)
scan_tile_reduce(const int32_t* __restrict__ in, int64_t n, int32_t* __restrict__ tile_sums,
                 const int32_t* __restrict__ live = nullptr) {
  // live (nullable, device): only entries below *live count (the rest read as 0)
  if (live) n = min(n, (int64_t)*live);
  const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
  if ((int64_t)blockIdx.x * kScanTile >= n) {
    if (threadIdx.x == 0) tile_sums[blockIdx.x] = 0;
    return;
  }
  int s = 0;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i)
    if (base + i < n) s += in[base + i];
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

// Single block: exclusive scan of the tile sums in place; writes the total.
__global__ void __launch_bounds__(kScanThreads)
scan_tile_offsets(int32_t* __restrict__ tile_sums, int64_t n_tiles, int32_t* __restrict__ total,
                  const int32_t* __restrict__ live = nullptr, int64_t n = 0) {
  // live: only the tiles holding entries below min(*live, n) (the rest are 0)
  if (live) {
    const int64_t m = min(n, (int64_t)*live);
    n_tiles = min(n_tiles, (m + kScanTile - 1) / kScanTile);
  }
  int carry = 0;
  for (int64_t t0 = 0; t0 < n_tiles; t0 += kScanTile) {
    int v[kScanItems];
    const int64_t base = t0 + (int64_t)threadIdx.x * kScanItems;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) v[i] = (base + i < n_tiles) ? tile_sums[base + i] : 0;
    int tot = block_exclusive_scan(v);
#pragma unroll
    for (int i = 0; i < kScanItems; ++i)
      if (base + i < n_tiles) tile_sums[base + i] = v[i] + carry;
    carry += tot;
    __syncthreads();
  }
  if (threadIdx.x == 0 && total) *total = carry;
}

}  // namespace
}  // namespace sn
