// Optimiser step of the SuperNormal training loop: torch.optim.Adam
// (betas 0.9/0.999, eps 1e-8, no weight decay; exp_runner.py:97,205-207)
// over one flat parameter buffer, with the learning-rate schedule of
// Runner.update_learning_rate (exp_runner.py:270-279) evaluated on the
// device so a captured step needs no host input.  The gradient buffer is
// zeroed as it is consumed (optimizer.zero_grad fused into the step).
#include "common.cuh"

#include <math.h>

namespace sn {

// iter holds the current iteration k; writes lr(k) and the Adam step k+1,
// then advances iter.
__global__ void lr_schedule_kernel(int32_t* __restrict__ iter, float* __restrict__ lr,
                                   int32_t* __restrict__ adam_step, float base_lr, int warm_up_end,
                                   int end_iter, float alpha) {
  const int k = *iter;
  double factor;
  if (k < warm_up_end) {
    factor = (double)k / (double)warm_up_end;
  } else {
    const double progress = (double)(k - warm_up_end) / (double)(end_iter - warm_up_end);
    factor = (cos(M_PI * progress) + 1.0) * 0.5 * (1.0 - alpha) + alpha;
  }
  *lr = (float)(base_lr * factor);
  *adam_step = k + 1;
  *iter = k + 1;
}

// Marching step of iteration *iter on the log schedule of exp_runner.py:81-83,149:
// 10 ** (log10(start) - (log10(start) - log10(end)) / end_iter * iter) in double,
// rounded once to float (the reference passes the numpy float64 to the marcher's
// float argument).
__global__ void step_size_schedule_kernel(const int32_t* __restrict__ iter, double start, double end,
                                          int end_iter, float* __restrict__ step) {
  const double slop = (log10(start) - log10(end)) / (double)end_iter;
  *step = (float)pow(10.0, log10(start) - slop * (double)*iter);
}

struct AdamArgs {
  int64_t n;
  float* p;
  float* g;
  float* m;
  float* v;
  __half* p_half;  // optional low-precision mirror of p
  const float* lr_dev;
  const int32_t* step_dev;
  float lr;
  int step;
  float beta1, beta2, eps;
  int zero_grad;
};

__device__ __forceinline__ void adam_one(float& p, float& m, float& v, float g, float omb1,
                                         float b2, float omb2, float step_size, float bc2s,
                                         float eps) {
  m = __fmaf_rn(omb1, __fsub_rn(g, m), m);
  v = __fmaf_rn(__fmul_rn(omb2, g), g, __fmul_rn(v, b2));
  const float denom = __fadd_rn(__fdiv_rn(sqrtf(v), bc2s), eps);
  p = __fmaf_rn(-step_size, __fdiv_rn(m, denom), p);
}

__global__ void __launch_bounds__(256) adam_kernel(AdamArgs a) {
  // bias corrections (torch.optim.Adam, double precision) once per block: FP64
  // throughput is a small fraction of FP32 here, so not once per thread
  __shared__ float s_step_size, s_bc2s;
  if (threadIdx.x == 0) {
    const float lr = a.lr_dev ? *a.lr_dev : a.lr;
    const int step = a.step_dev ? *a.step_dev : a.step;
    const double bc1 = 1.0 - pow((double)a.beta1, (double)step);
    const double bc2 = 1.0 - pow((double)a.beta2, (double)step);
    s_step_size = (float)((double)lr / bc1);
    s_bc2s = (float)sqrt(bc2);
  }
  __syncthreads();
  const float step_size = s_step_size, bc2s = s_bc2s;
  const float omb1 = 1.0f - a.beta1, omb2 = 1.0f - a.beta2;
  const int64_t n4 = a.n >> 2;
  float4* p4 = reinterpret_cast<float4*>(a.p);
  float4* g4 = reinterpret_cast<float4*>(a.g);
  float4* m4 = reinterpret_cast<float4*>(a.m);
  float4* v4 = reinterpret_cast<float4*>(a.v);
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n4; i += stride) {
    // the moments are next read by the next step's Adam: streamed (evict
    // first), so the table and its gradient, which the field kernels gather
    // and reduce into next, keep their L2 lines
    float4 p = p4[i], g = g4[i], m = __ldcs(m4 + i), v = __ldcs(v4 + i);
    adam_one(p.x, m.x, v.x, g.x, omb1, a.beta2, omb2, step_size, bc2s, a.eps);
    adam_one(p.y, m.y, v.y, g.y, omb1, a.beta2, omb2, step_size, bc2s, a.eps);
    adam_one(p.z, m.z, v.z, g.z, omb1, a.beta2, omb2, step_size, bc2s, a.eps);
    adam_one(p.w, m.w, v.w, g.w, omb1, a.beta2, omb2, step_size, bc2s, a.eps);
    p4[i] = p;
    __stcs(m4 + i, m);
    __stcs(v4 + i, v);
    if (a.zero_grad) g4[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    if (a.p_half) {
      __half2* h2 = reinterpret_cast<__half2*>(a.p_half) + 2 * i;
      h2[0] = __floats2half2_rn(p.x, p.y);
      h2[1] = __floats2half2_rn(p.z, p.w);
    }
  }
  for (int64_t i = 4 * n4 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < a.n; i += stride) {
    float p = a.p[i], m = a.m[i], v = a.v[i];
    adam_one(p, m, v, a.g[i], omb1, a.beta2, omb2, step_size, bc2s, a.eps);
    a.p[i] = p;
    a.m[i] = m;
    a.v[i] = v;
    if (a.zero_grad) a.g[i] = 0.0f;
    if (a.p_half) a.p_half[i] = __float2half_rn(p);
  }
}

}  // namespace sn

using namespace sn;

extern "C" {

int sn_lr_schedule(int32_t* iter, float* lr, int32_t* adam_step, float base_lr, int warm_up_end,
                   int end_iter, float alpha, void* stream) {
  SN_REQUIRE(iter && lr && adam_step, "lr_schedule: null buffer");
  SN_REQUIRE(warm_up_end >= 0 && end_iter > warm_up_end, "lr_schedule: need end_iter > warm_up_end");
  lr_schedule_kernel<<<1, 1, 0, as_stream(stream)>>>(iter, lr, adam_step, base_lr, warm_up_end,
                                                     end_iter, alpha);
  return check_launch("lr_schedule");
}

int sn_step_size_schedule(const int32_t* iter, double start_step, double end_step, int end_iter,
                          float* step, void* stream) {
  SN_REQUIRE(iter && step, "step_size_schedule: null buffer");
  SN_REQUIRE(start_step > 0.0 && end_step > 0.0 && end_iter > 0, "step_size_schedule: bad schedule");
  step_size_schedule_kernel<<<1, 1, 0, as_stream(stream)>>>(iter, start_step, end_step, end_iter, step);
  return check_launch("step_size_schedule");
}

int sn_adam_step(int64_t n, float* param, float* grad, float* exp_avg, float* exp_avg_sq,
                 void* param_half, const float* lr_dev, const int32_t* step_dev, float lr, int step,
                 float beta1, float beta2, float eps, int zero_grad, void* stream) {
  SN_REQUIRE(n >= 0, "adam: n < 0");
  SN_REQUIRE(param && grad && exp_avg && exp_avg_sq, "adam: null buffer");
  SN_REQUIRE(step_dev != nullptr || step >= 1, "adam: step must be >= 1");
  SN_REQUIRE((((uintptr_t)param | (uintptr_t)grad | (uintptr_t)exp_avg | (uintptr_t)exp_avg_sq) & 15) == 0,
             "adam: buffers must be 16-byte aligned");
  if (n == 0) return SN_OK;
  AdamArgs a;
  a.n = n;
  a.p = param;
  a.g = grad;
  a.m = exp_avg;
  a.v = exp_avg_sq;
  a.p_half = reinterpret_cast<__half*>(param_half);
  a.lr_dev = lr_dev;
  a.step_dev = step_dev;
  a.lr = lr;
  a.step = step;
  a.beta1 = beta1;
  a.beta2 = beta2;
  a.eps = eps;
  a.zero_grad = zero_grad;
  // 4 blocks of 256 threads per SM: measured against 8 and 16 (0.0737 / 0.079 /
  // 0.090 ms per step on the bench's 12.6 M parameters)
  adam_kernel<<<stride_grid((n + 3) / 4, 256, 4), 256, 0, as_stream(stream)>>>(a);
  return check_launch("adam_step");
}

}  // extern "C"
