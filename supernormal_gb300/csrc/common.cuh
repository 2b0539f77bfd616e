// Shared device/host helpers for the supernormal_gb300 CUDA library.
//
// Every exported entry point is `extern "C"`, takes raw device pointers,
// element counts and a `cudaStream_t` (passed as `void*`), writes into
// caller-allocated buffers and returns an `SN_*` status code.  A failing
// status leaves a human-readable message retrievable with sn_last_error().
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <stdarg.h>

#include "../../include/supernormal_gb300.h"

namespace sn {

// ---------------------------------------------------------------------------
// error reporting
// ---------------------------------------------------------------------------
void set_error(const char* fmt, ...);
void count_launches(int k);

// Records k kernel launches (for the launch counter) and checks for errors.
inline int check_launch(const char* what, int k = 1) {
  count_launches(k);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error("%s: CUDA launch failed: %s", what, cudaGetErrorString(e));
    return SN_ERR_CUDA;
  }
  return SN_OK;
}

#define SN_REQUIRE(cond, ...)          \
  do {                                 \
    if (!(cond)) {                     \
      ::sn::set_error(__VA_ARGS__);    \
      return SN_ERR_INVALID;           \
    }                                  \
  } while (0)

#define SN_TRY(expr)                   \
  do {                                 \
    int _st = (expr);                  \
    if (_st != SN_OK) return _st;      \
  } while (0)

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

// Number of SMs of the current device (cached per process; single-GPU use).
int num_sms();

// Raises a kernel's dynamic shared-memory limit to `bytes` once per (device,
// kernel); later calls only look the pair up, so launches made while a stream
// is being captured issue no attribute calls.
int ensure_smem_limit(const void* fn, size_t bytes, const char* what);

inline unsigned int div_up(int64_t a, int64_t b) {
  return (unsigned int)((a + b - 1) / b);
}

// Grid size for a grid-stride kernel: enough blocks to cover n, capped at a
// whole number of waves over all SMs.
inline unsigned int stride_grid(int64_t n, int threads, int blocks_per_sm) {
  int64_t need = (n + threads - 1) / threads;
  int64_t cap = (int64_t)num_sms() * blocks_per_sm;
  if (need < 1) need = 1;
  return (unsigned int)(need < cap ? need : cap);
}

// ---------------------------------------------------------------------------
// device helpers
// ---------------------------------------------------------------------------
struct f3 {
  float x, y, z;
};

__device__ __forceinline__ f3 mk(float x, float y, float z) { return f3{x, y, z}; }

// Counter-based uniform random numbers in [0, 1): a 64-bit mix of
// (seed, stream, index).  Used only where the reference draws from
// torch.rand / torch.randint and the exact stream is not part of the
// contract (jitter, cell sampling).
__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
__device__ __forceinline__ float uniform01(uint64_t seed, uint64_t stream, uint64_t idx) {
  uint64_t h = mix64(seed ^ mix64(stream * 0x632BE59BD9B4E019ull + idx));
  return (float)(h >> 40) * (1.0f / 16777216.0f);  // 24 random bits
}
__device__ __forceinline__ uint32_t uniform_u32(uint64_t seed, uint64_t stream, uint64_t idx) {
  return (uint32_t)(mix64(seed ^ mix64(stream * 0x632BE59BD9B4E019ull + idx)) >> 32);
}

// torch.nn.Softplus(beta, threshold) forward and its derivative
// (torch/nn/modules/activation.py Softplus; ATen softplus kernel semantics).
__device__ __forceinline__ float softplus_fwd(float x, float beta, float threshold) {
  float bx = x * beta;
  return bx > threshold ? x : log1pf(expf(bx)) / beta;
}
__device__ __forceinline__ float softplus_grad(float x, float beta, float threshold) {
  float bx = x * beta;
  if (bx > threshold) return 1.0f;
  float z = expf(bx);
  return z / (z + 1.0f);
}
// Both at once (one exponential); the same values as the two functions above.
__device__ __forceinline__ void softplus_fwd_grad(float x, float beta, float threshold, float& y,
                                                  float& dy) {
  const float bx = x * beta;
  if (bx > threshold) {
    y = x;
    dy = 1.0f;
    return;
  }
  const float z = expf(bx);
  y = log1pf(z) / beta;
  dy = z / (z + 1.0f);
}
// Softplus and its derivative through the hardware exp2/log2 approximations
// (__expf, __logf, __fdividef): y = log(1 + z) / beta, dy = z / (1 + z),
// z = exp(beta x).  Against the accurate pair above the absolute error of y
// stays below 4e-9 for beta = 100 and z < 1, and within a few ulp beyond.
__device__ __forceinline__ void softplus_fwd_grad_fast(float x, float beta, float inv_beta,
                                                       float threshold, float& y, float& dy) {
  const float bx = x * beta;
  if (bx > threshold) {
    y = x;
    dy = 1.0f;
    return;
  }
  const float z = __expf(bx);
  const float u = 1.0f + z;
  y = __logf(u) * inv_beta;
  dy = __fdividef(z, u);
}
__device__ __forceinline__ float sigmoidf_(float x) { return 1.0f / (1.0f + expf(-x)); }

}  // namespace sn
