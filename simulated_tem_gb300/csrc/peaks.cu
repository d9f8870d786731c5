// Arithmetic-pipe peak microbenchmarks for the roofline of the imaging kernels.
//
// The phase-field and column-integration kernels are bound by the FP32 FMA pipe
// and the MUFU (special function) pipe, not by HBM or the tensor cores, and
// their FP64 variants by the FP64 pipe.  None of these peaks is in the
// generated peak file, so they are measured here on the same GPU, in the
// same process, right before the kernels they normalise.
//
// Each kernel runs 8 independent dependency chains per thread over a grid of
// 8 CTAs x 256 threads per SM so that every pipe is saturated; the timed
// region is bracketed by CUDA events on the launching stream.
#include <cuda_runtime.h>
#include <cstdio>

namespace {

constexpr int kChains = 8;
constexpr int kIters = 4096;
constexpr int kThreads = 256;

__global__ void fp32_fma_kernel(float* out, float b, float c) {
  float a[kChains];
#pragma unroll
  for (int i = 0; i < kChains; ++i) a[i] = threadIdx.x * 1e-3f + i;
  for (int it = 0; it < kIters; ++it) {
#pragma unroll
    for (int i = 0; i < kChains; ++i) a[i] = fmaf(a[i], b, c);
  }
  float s = 0.f;
#pragma unroll
  for (int i = 0; i < kChains; ++i) s += a[i];
  if (s == 1234.5f) out[blockIdx.x] = s;  // keeps the chains alive
}

// The same on packed FP32x2 multiply-adds (two FMAs per instruction), the form the
// column integrator uses.
__global__ void fp32x2_fma_kernel(float* out, float b, float c) {
  float2 a[kChains];
#pragma unroll
  for (int i = 0; i < kChains; ++i) a[i] = make_float2(threadIdx.x * 1e-3f + i, threadIdx.x * 2e-3f + i);
  const float2 b2 = make_float2(b, b), c2 = make_float2(c, c);
  for (int it = 0; it < kIters; ++it) {
#pragma unroll
    for (int i = 0; i < kChains; ++i) a[i] = __ffma2_rn(a[i], b2, c2);
  }
  float s = 0.f;
#pragma unroll
  for (int i = 0; i < kChains; ++i) s += a[i].x + a[i].y;
  if (s == 1234.5f) out[blockIdx.x] = s;
}

__global__ void fp64_fma_kernel(double* out, double b, double c) {
  double a[kChains];
#pragma unroll
  for (int i = 0; i < kChains; ++i) a[i] = threadIdx.x * 1e-3 + i;
  for (int it = 0; it < kIters / 8; ++it) {
#pragma unroll
    for (int i = 0; i < kChains; ++i) a[i] = fma(a[i], b, c);
  }
  double s = 0.0;
#pragma unroll
  for (int i = 0; i < kChains; ++i) s += a[i];
  if (s == 1234.5) out[blockIdx.x] = s;
}

__device__ __forceinline__ float mufu_ex2(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

__device__ __forceinline__ float mufu_sin(float x) {
  float y;
  asm("sin.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

template <int kOp>
__global__ void mufu_kernel(float* out) {
  float a[kChains];
#pragma unroll
  for (int i = 0; i < kChains; ++i) a[i] = -0.5f - 1e-4f * (threadIdx.x + i);
  for (int it = 0; it < kIters / 4; ++it) {
#pragma unroll
    for (int i = 0; i < kChains; ++i) a[i] = (kOp == 0) ? mufu_ex2(a[i]) : mufu_sin(a[i]);
  }
  float s = 0.f;
#pragma unroll
  for (int i = 0; i < kChains; ++i) s += a[i];
  if (s == 1234.5f) out[blockIdx.x] = s;
}

template <typename F>
double time_ms(F&& launch, cudaStream_t st) {
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  launch();  // warm-up
  launch();
  cudaStreamSynchronize(st);
  float best = 1e30f;
  for (int rep = 0; rep < 5; ++rep) {
    cudaEventRecord(e0, st);
    launch();
    cudaEventRecord(e1, st);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best) best = ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return best;
}

}  // namespace

// out[0] FP32 FMA-pipe TFLOP/s on scalar FMAs (2 flops per FMA), out[1] FP64 TFLOP/s,
// out[2] MUFU ex2 Gop/s, out[3] MUFU sin Gop/s, out[4] FP32 TFLOP/s on packed FP32x2
// FMAs (4 flops per instruction).  Returns 0 or a CUDA error code.
extern "C" int stp_measure_peaks(double* out) {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 1;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int blocks = sms * 8;
  const double threads = double(blocks) * kThreads;
  void* scratch = nullptr;
  if (cudaMalloc(&scratch, blocks * sizeof(double)) != cudaSuccess) return 2;
  cudaStream_t st;
  cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);

  double ms = time_ms([&] { fp32_fma_kernel<<<blocks, kThreads, 0, st>>>((float*)scratch, 0.999f, 1e-3f); }, st);
  out[0] = 2.0 * kChains * kIters * threads / (ms * 1e-3) / 1e12;
  ms = time_ms([&] { fp64_fma_kernel<<<blocks, kThreads, 0, st>>>((double*)scratch, 0.999, 1e-3); }, st);
  out[1] = 2.0 * kChains * (kIters / 8) * threads / (ms * 1e-3) / 1e12;
  ms = time_ms([&] { mufu_kernel<0><<<blocks, kThreads, 0, st>>>((float*)scratch); }, st);
  out[2] = double(kChains) * (kIters / 4) * threads / (ms * 1e-3) / 1e9;
  ms = time_ms([&] { mufu_kernel<1><<<blocks, kThreads, 0, st>>>((float*)scratch); }, st);
  out[3] = double(kChains) * (kIters / 4) * threads / (ms * 1e-3) / 1e9;

  ms = time_ms([&] { fp32x2_fma_kernel<<<blocks, kThreads, 0, st>>>((float*)scratch, 0.999f, 1e-3f); }, st);
  out[4] = 4.0 * kChains * kIters * threads / (ms * 1e-3) / 1e12;

  cudaError_t err = cudaStreamSynchronize(st);
  cudaStreamDestroy(st);
  cudaFree(scratch);
  return err == cudaSuccess ? 0 : int(err);
}
