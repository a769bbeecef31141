// Shared device/host helpers: complex arithmetic on float2/double2, error
// plumbing and the launch counter.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <string>
#include "../../include/oh.h"

namespace oh {

template <typename R> struct cplx_of;
template <> struct cplx_of<float>  { typedef float2  type; };
template <> struct cplx_of<double> { typedef double2 type; };

__host__ __device__ __forceinline__ float2  mk(float x, float y)   { return make_float2(x, y); }
__host__ __device__ __forceinline__ double2 mk(double x, double y) { return make_double2(x, y); }

template <typename C> __host__ __device__ __forceinline__ C cadd(C a, C b) { C r; r.x = a.x + b.x; r.y = a.y + b.y; return r; }
template <typename C> __host__ __device__ __forceinline__ C csub(C a, C b) { C r; r.x = a.x - b.x; r.y = a.y - b.y; return r; }
template <typename C> __host__ __device__ __forceinline__ C cmul(C a, C b) {
  C r; r.x = a.x * b.x - a.y * b.y; r.y = a.x * b.y + a.y * b.x; return r;
}
// a * conj(b)
template <typename C> __host__ __device__ __forceinline__ C cmulc(C a, C b) {
  C r; r.x = a.x * b.x + a.y * b.y; r.y = a.y * b.x - a.x * b.y; return r;
}
template <typename C, typename R> __host__ __device__ __forceinline__ C cscale(C a, R s) { C r; r.x = a.x * s; r.y = a.y * s; return r; }
// s a + b, s real
template <typename C, typename R> __host__ __device__ __forceinline__ C caxpy(R s, C a, C b) {
  C r; r.x = s * a.x + b.x; r.y = s * a.y + b.y; return r;
}
#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 1000
// FP32 complex add, subtract, real scale and real axpy as one packed two-lane
// instruction each (sm_100 family); per component the rounding is that of
// the scalar operation (a - b = a + (-1) b, the product exact)
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.f, -1.f), a); }
__device__ __forceinline__ float2 cscale(float2 a, float s) { return __fmul2_rn(a, make_float2(s, s)); }
__device__ __forceinline__ float2 caxpy(float s, float2 a, float2 b) { return __ffma2_rn(make_float2(s, s), a, b); }
#endif
// multiply by -i (forward) or +i (inverse): sgn = -1 -> -i*a, sgn = +1 -> i*a
template <int SGN, typename C> __host__ __device__ __forceinline__ C cmul_i(C a) {
  C r; if (SGN < 0) { r.x = a.y; r.y = -a.x; } else { r.x = -a.y; r.y = a.x; } return r;
}
// a + cmul_i<SGN>(b) and a + s cmul_i<SGN>(b), component by component (the
// swapped halves of b do not form a packed pair)
template <int SGN, typename C> __host__ __device__ __forceinline__ C cadd_i(C a, C b) {
  C r; if (SGN < 0) { r.x = a.x + b.y; r.y = a.y - b.x; } else { r.x = a.x - b.y; r.y = a.y + b.x; } return r;
}
template <int SGN, typename C, typename R> __host__ __device__ __forceinline__ C caxpy_i(R s, C b, C a) {
  C r; if (SGN < 0) { r.x = a.x + s * b.y; r.y = a.y - s * b.x; } else { r.x = a.x - s * b.y; r.y = a.y + s * b.x; }
  return r;
}

// Error-path test hook: spin on a device flag that nothing sets, for at most
// `cycles` SM clocks.  Returns false when the bound ran out (always, unless
// the flag were set), so the caller takes its bounded-wait error path.
__device__ __forceinline__ bool stall_on_unset_flag(const int* flag, long long cycles) {
  const long long t0 = clock64();
  while (*((volatile const int*)flag) == 0) {
    if (clock64() - t0 > cycles) return false;
  }
  return true;
}
// kernel_mask bits of oh_ctx_set_test_stall
constexpr int kStallDepthmapColumn = 1, kStallPointSumGemm = 2, kStallConvolution = 4, kStallDepthmapBatch = 8;

// Launch accounting (read through oh_kernel_launch_count()).
void note_launch(int n = 1);
// Kernels launched by this library so far (all threads).
uint64_t launches_so_far();

// Streaming multiprocessors of the current device (queried once per device
// and cached); grid sizes that aim at whole waves are multiples of it.
int sm_count();

// Per-thread last-error message.
void set_error(const std::string& msg);
oh_status fail(oh_status s, const std::string& msg);
oh_status cuda_fail(cudaError_t e, const char* what);

}  // namespace oh

#define OH_CUDA_TRY(expr)                                  \
  do {                                                     \
    cudaError_t _e = (expr);                               \
    if (_e != cudaSuccess) return ::oh::cuda_fail(_e, #expr); \
  } while (0)

#define OH_TRY(expr)                     \
  do {                                   \
    oh_status _s = (expr);               \
    if (_s != OH_OK) return _s;          \
  } while (0)

// Check the launch that was just enqueued.
#define OH_LAUNCH_CHECK()                                      \
  do {                                                         \
    ::oh::note_launch();                                       \
    cudaError_t _e = cudaGetLastError();                       \
    if (_e != cudaSuccess) return ::oh::cuda_fail(_e, "kernel launch"); \
  } while (0)
