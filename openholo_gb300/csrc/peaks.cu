// Issue-rate microbenchmarks: the compute-side roofline denominators.
//
// The HBM and BF16-tensor peaks of the roofline come from measured copy and
// GEMM runs; the kernels here measure the other two rates the library's
// kernels are bound by, on the GPU they run on:
//   FFMA   FP32 fused multiply-adds, scalar (one warp instruction = 32 FMAs);
//          also the SM's peak warp-instruction issue rate (one instruction per
//          scheduler per clock);
//   FFMA2  packed two-lane FP32 FMAs (one warp instruction = 64 FMAs);
//   MUFU   sin.approx.f32 results (the multi-function unit that also serves
//          the approximate rsqrt, reciprocal and ex2).
// Each kernel runs independent dependency chains, eight per thread, over a
// grid of whole waves, and is timed with CUDA events after a warm-up launch.
#include <cuda_runtime.h>
#include <algorithm>
#include "context.h"
#include "oh_common.cuh"

namespace oh {

constexpr int kPeakChains = 8;
constexpr int kPeakUnroll = 16;

__global__ void __launch_bounds__(256) peak_ffma(float* sink, int iters, float a, float b) {
  float x[kPeakChains];
#pragma unroll
  for (int c = 0; c < kPeakChains; ++c) x[c] = (float)(threadIdx.x + c) * 1e-3f;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int u = 0; u < kPeakUnroll; ++u)
#pragma unroll
      for (int c = 0; c < kPeakChains; ++c) x[c] = fmaf(x[c], a, b);
  }
  float s = 0.f;
#pragma unroll
  for (int c = 0; c < kPeakChains; ++c) s += x[c];
  if (s == 1234.5f) sink[blockIdx.x] = s;      // never true for the arguments used; keeps the chains live
}

__global__ void __launch_bounds__(256) peak_ffma2(float* sink, int iters, float a, float b) {
  float2 x[kPeakChains];
#pragma unroll
  for (int c = 0; c < kPeakChains; ++c) x[c] = make_float2((float)(threadIdx.x + c) * 1e-3f, (float)c * 1e-3f);
  const float2 a2 = make_float2(a, a), b2 = make_float2(b, b);
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int u = 0; u < kPeakUnroll; ++u)
#pragma unroll
      for (int c = 0; c < kPeakChains; ++c) {
#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 1000
        x[c] = __ffma2_rn(x[c], a2, b2);
#else
        x[c] = make_float2(fmaf(x[c].x, a, b), fmaf(x[c].y, a, b));
#endif
      }
  }
  float s = 0.f;
#pragma unroll
  for (int c = 0; c < kPeakChains; ++c) s += x[c].x + x[c].y;
  if (s == 1234.5f) sink[blockIdx.x] = s;
}

__global__ void __launch_bounds__(256) peak_mufu(float* sink, int iters) {
  float x[kPeakChains];
#pragma unroll
  for (int c = 0; c < kPeakChains; ++c) x[c] = (float)(threadIdx.x + c) * 1e-3f;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int u = 0; u < kPeakUnroll; ++u)
#pragma unroll
      for (int c = 0; c < kPeakChains; ++c) asm volatile("sin.approx.ftz.f32 %0, %0;" : "+f"(x[c]));
  }
  float s = 0.f;
#pragma unroll
  for (int c = 0; c < kPeakChains; ++c) s += x[c];
  if (s == 1234.5f) sink[blockIdx.x] = s;
}

}  // namespace oh

using namespace oh;

extern "C" oh_status oh_measure_issue_peaks(int device, double* ffma_per_s, double* ffma2_per_s,
                                            double* mufu_per_s, double* sm_mhz_hint) {
  if (!ffma_per_s || !ffma2_per_s || !mufu_per_s) return fail(OH_ERR_INVALID_ARG, "null output");
  int prev = -1;
  cudaGetDevice(&prev);
  OH_CUDA_TRY(cudaSetDevice(device));
  const int sms = sm_count();
  const int blocks = sms * 8, threads = 256;        // 64 warps per SM: eight resident blocks
  float* sink = nullptr;
  cudaStream_t st = nullptr;
  cudaEvent_t a = nullptr, b = nullptr;
  oh_status rc = OH_OK;
  auto cleanup = [&]() {
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
    if (st) cudaStreamDestroy(st);
    if (sink) cudaFree(sink);
    if (prev >= 0) cudaSetDevice(prev);
  };
  cudaError_t e = cudaMalloc(&sink, sizeof(float) * blocks);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreate(&a);
  if (e == cudaSuccess) e = cudaEventCreate(&b);
  if (e != cudaSuccess) { rc = cuda_fail(e, "peak set-up"); cleanup(); return rc; }
  const int iters = 4096;
  const double per_thread = (double)iters * kPeakUnroll * kPeakChains;
  const double warps = (double)blocks * threads / 32.0;
  double ms[3] = {0, 0, 0};
  for (int kind = 0; kind < 3; ++kind) {
    float best = 1e30f;
    for (int rep = 0; rep < 3; ++rep) {        // rep 0 warms up; the best of the others counts
      cudaEventRecord(a, st);
      if (kind == 0) peak_ffma<<<blocks, threads, 0, st>>>(sink, iters, 0.999f, 1e-4f);
      else if (kind == 1) peak_ffma2<<<blocks, threads, 0, st>>>(sink, iters, 0.999f, 1e-4f);
      else peak_mufu<<<blocks, threads, 0, st>>>(sink, iters);
      note_launch();
      cudaEventRecord(b, st);
      e = cudaEventSynchronize(b);
      if (e != cudaSuccess) { rc = cuda_fail(e, "peak kernel"); cleanup(); return rc; }
      float t = 0.f;
      cudaEventElapsedTime(&t, a, b);
      if (rep > 0) best = std::min(best, t);
    }
    ms[kind] = best;
  }
  *ffma_per_s = warps * per_thread / (ms[0] * 1e-3);      // warp instructions per second
  *ffma2_per_s = warps * per_thread / (ms[1] * 1e-3);
  *mufu_per_s = warps * 32.0 * per_thread / (ms[2] * 1e-3);   // results (thread operations) per second
  if (sm_mhz_hint) {
    // FFMA runs at four warp instructions per SM per clock
    *sm_mhz_hint = *ffma_per_s / (4.0 * sms) / 1e6;
  }
  cleanup();
  return OH_OK;
}
