// Hologram encoders (OpenHolo_Encoding/fn_encoding.m:29-98), the phase-only
// uint8 encoding of Hologram_WRP.m:57-60 and the uint8 normalisations of
// Write_Result_image (HologramGenerator.cpp:528-565) and ophNormalize
// (oph_common.cpp:92-115).  Global maxima/minima use a two-level reduction
// (block partials, then one block), so results are deterministic.
#include <algorithm>
#include <cmath>
#include "context.h"
#include "fft_kernels.cuh"

namespace oh {

template <typename R> __device__ __forceinline__ R ratan2(R y, R x);
template <> __device__ __forceinline__ float ratan2<float>(float y, float x) { return atan2f(y, x); }
template <> __device__ __forceinline__ double ratan2<double>(double y, double x) { return atan2(y, x); }

enum RedOp { RED_MAX_ABS = 0, RED_MINMAX_REAL = 1, RED_MAX_NI = 2, RED_MAX_PHASE = 3, RED_MINMAX_SSB = 4 };

// Block partial reductions: out[2*b] = min, out[2*b+1] = max of the mapped value.
template <typename R>
__global__ void __launch_bounds__(256) reduce_partial(const void* __restrict__ in, size_t n, int op, const R* __restrict__ refp, R* __restrict__ part) {
  typedef typename cplx_of<R>::type C;
  __shared__ R smin[256], smax[256];
  R mn = (R)INFINITY, mx = -(R)INFINITY;
  const R ref = refp ? refp[1] : (R)0;
  auto take = [&](C c) {
    R v;
    if (op == RED_MAX_ABS) v = hypot(c.x, c.y);
    else if (op == RED_MAX_NI) { R re = c.x + ref; v = re * re + c.y * c.y; }
    else if (op == RED_MAX_PHASE) v = ratan2<R>(c.y, c.x) + (R)3.14159265358979323846;
    else v = c.x;   // RED_MINMAX_SSB: real part
    mn = v < mn ? v : mn;
    mx = v > mx ? v : mx;
  };
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (op == RED_MINMAX_REAL) {
    for (; i < n; i += stride) {
      const R v = static_cast<const R*>(in)[i];
      mn = v < mn ? v : mn;
      mx = v > mx ? v : mx;
    }
  } else {
    // four independent loads in flight per thread before the math
    const C* src = static_cast<const C*>(in);
    for (; i + 3 * stride < n; i += 4 * stride) {
      C c[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) c[q] = src[i + q * stride];
#pragma unroll
      for (int q = 0; q < 4; ++q) take(c[q]);
    }
    for (; i < n; i += stride) take(src[i]);
  }
  smin[threadIdx.x] = mn; smax[threadIdx.x] = mx;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      smin[threadIdx.x] = min(smin[threadIdx.x], smin[threadIdx.x + s]);
      smax[threadIdx.x] = max(smax[threadIdx.x], smax[threadIdx.x + s]);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) { part[2 * blockIdx.x] = smin[0]; part[2 * blockIdx.x + 1] = smax[0]; }
}

template <typename R>
__global__ void reduce_final(R* part, int nb) {
  __shared__ R smin[256], smax[256];
  R mn = (R)INFINITY, mx = -(R)INFINITY;
  for (int i = threadIdx.x; i < nb; i += blockDim.x) { mn = min(mn, part[2 * i]); mx = max(mx, part[2 * i + 1]); }
  smin[threadIdx.x] = mn; smax[threadIdx.x] = mx;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      smin[threadIdx.x] = min(smin[threadIdx.x], smin[threadIdx.x + s]);
      smax[threadIdx.x] = max(smax[threadIdx.x], smax[threadIdx.x + s]);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) { part[0] = smin[0]; part[1] = smax[0]; }
}

// Enqueue a min/max reduction; result (min,max) lands in red[0], red[1] on the device.
template <typename R>
static oh_status reduce(oh_ctx* ctx, const void* in, size_t n, int op, const R* refp, R** red, cudaStream_t st, const char* slot) {
  // 16 blocks of 256 threads per SM: one load in flight per thread, so the
  // thread count sets how many bytes are in flight (512 blocks kept the read
  // of a 66 MB field near a quarter of the HBM bandwidth)
  const int nb = (int)std::max<size_t>(1, std::min<size_t>((n + 255) / 256, oh::sm_count() * 16));
  void* ptr;
  OH_TRY(scratch(ctx, slot, sizeof(R) * 2 * nb, &ptr));
  *red = (R*)ptr;
  KernelTimer kt(ctx, "reduce", st);
  reduce_partial<R><<<nb, 256, 0, st>>>(in, n, op, refp, *red);
  OH_LAUNCH_CHECK();
  reduce_final<R><<<1, 256, 0, st>>>(*red, nb);
  OH_LAUNCH_CHECK();
  return OH_OK;
}

// Reference value max|U| read on the device by the map kernels.
template <typename R>
__global__ void __launch_bounds__(256) encode_map(int kind, int nx, int ny, const typename cplx_of<R>::type* __restrict__ U,
                                                  const R* __restrict__ red1, const R* __restrict__ red2, void* __restrict__ out) {
  typedef typename cplx_of<R>::type C;
  const R pi = (R)3.14159265358979323846;
  const size_t n = (size_t)nx * ny;
  auto emit = [&](size_t i, C u) {
    R* o = static_cast<R*>(out);
    switch (kind) {
      case OH_ENC_REAL: o[i] = u.x; break;
      case OH_ENC_AMPLITUDE: o[i] = hypot(u.x, u.y); break;
      case OH_ENC_PHASE_TO_AMP: o[i] = ratan2<R>(u.y, u.x) + pi / ((R)2 * pi); break;   // fn_encoding.m:57 as written
      case OH_ENC_NUM_INTERFERENCE: {
        const R ref = red1[1];
        const R re = u.x + ref;
        o[i] = (re * re + u.y * u.y) / red2[1];
      } break;
      case OH_ENC_BURCKHARDT: {
        const R m = red1[1];
        const R cr = u.x / m, ci = u.y / m;
        const R ph = ratan2<R>(ci, cr) + pi;
        const R am = hypot(cr, ci);
        const R s3 = (R)1.7320508075688772935;
        R a1 = 0, a2 = 0, a3 = 0;
        if (ph >= 0 && ph < 2 * pi / 3) {
          a1 = am * (cos(ph) + sin(ph) / s3);
          a2 = 2 * sin(ph) / s3;
        } else if (ph >= 2 * pi / 3 && ph < 4 * pi / 3) {
          a2 = am * (cos(ph - 2 * pi / 3) + sin(ph - 2 * pi / 3) / s3);
          a3 = 2 * sin(ph - 2 * pi / 3) / s3;
        } else if (ph >= 4 * pi / 3 && ph < 2 * pi) {
          a3 = am * (cos(ph - 4 * pi / 3) + sin(ph - 4 * pi / 3) / s3);
          a1 = 2 * sin(ph - 4 * pi / 3) / s3;
        }
        const size_t r = i / nx, c = i - r * nx;
        R* row = o + r * (size_t)(3 * nx);
        row[3 * c] = a1; row[3 * c + 1] = a2; row[3 * c + 2] = a3;
      } break;
      case OH_ENC_TWO_PHASE: {
        const R m = red1[1];
        const R cr = u.x / m, ci = u.y / m;
        const R am = hypot(cr, ci);
        const R ph = ratan2<R>(ci, cr) + pi;
        // MATLAB's acos of a rounding-level 1+eps is complex; its real part is 0
        const R del = acos(am < (R)1 ? am : (R)1);
        const size_t r = i / nx, c = i - r * nx;
        R* row = o + r * (size_t)(2 * nx);
        row[2 * c] = ph + del; row[2 * c + 1] = ph - del;
      } break;
      case OH_ENC_PHASE_ONLY_U8: {
        const R ph = ratan2<R>(u.y, u.x) + pi;
        R v = (R)255 * ph / red1[1];
        // MATLAB uint8(): round half away from zero, saturate
        v = v < 0 ? 0 : (v > 255 ? 255 : v);
        static_cast<uint8_t*>(out)[i] = (uint8_t)floor(v + (R)0.5);
      } break;
      default: break;
    }
  };
  // four independent loads in flight per thread before the math
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  for (; i + 3 * stride < n; i += 4 * stride) {
    C u[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) u[q] = U[i + q * stride];
#pragma unroll
    for (int q = 0; q < 4; ++q) emit(i + q * stride, u[q]);
  }
  for (; i < n; i += stride) emit(i, U[i]);
}

// SSB: zero half of the centred spectrum (fn_encoding.m:33-41).
template <typename R>
__global__ void ssb_mask(int kind, int nx, int ny, typename cplx_of<R>::type* A) {
  const size_t n = (size_t)nx * ny;
  const int hx = nx / 2, hy = ny / 2;   // MATLAB floor(N/2), 1-based -> 0-based start hx-1
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int r = (int)(i / nx), c = (int)(i - (size_t)r * nx);
    bool zero = false;
    if (kind == OH_ENC_SSB_LEFT) zero = c >= hx - 1;
    else if (kind == OH_ENC_SSB_RIGHT) zero = c <= hx - 1;
    else if (kind == OH_ENC_SSB_TOP) zero = r >= hy - 1;
    else if (kind == OH_ENC_SSB_BOTTOM) zero = r <= hy - 1;
    if (zero) { A[i].x = 0; A[i].y = 0; }
  }
}

template <typename R>
__global__ void ssb_finish(size_t n, const typename cplx_of<R>::type* A, const R* red, R* out) {
  const R mn = red[0], rng = red[1] - red[0];
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    out[i] = (A[i].x - mn) / rng;
}

template <typename R>
__global__ void normalize_u8_kernel(int nx, int ny, const R* __restrict__ in, const R* __restrict__ red, uint8_t* __restrict__ out, int round_half) {
  const size_t n = (size_t)nx * ny;
  const R mn = red[0], mx = red[1];
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    if (round_half) {
      // ophNormalize: float math, +0.5, vertical flip
      const int r = (int)(i / nx), c = (int)(i - (size_t)r * nx);
      float v = (((float)in[i] - (float)mn) / ((float)mx - (float)mn)) * 255.f + 0.5f;
      out[(size_t)(ny - r - 1) * nx + c] = (uint8_t)(unsigned)v;
    } else {
      // Write_Result_image: (uint)((v - min)/(max - min)*255) in double
      double v = ((double)in[i] - (double)mn) / ((double)mx - (double)mn) * 255.0;
      out[i] = (uint8_t)(unsigned)v;
    }
  }
}

template <typename R>
static oh_status run_encode(oh_ctx* ctx, int kind, int nx, int ny, const void* field, void* out, cudaStream_t st) {
  typedef typename cplx_of<R>::type C;
  const size_t n = (size_t)nx * ny;
  const int grid = (int)std::min<size_t>((n + 255) / 256, oh::sm_count() * 16);
  R* red1 = nullptr;
  R* red2 = nullptr;
  if (kind >= OH_ENC_SSB_LEFT && kind <= OH_ENC_SSB_BOTTOM) {
    void* ptr;
    OH_TRY(scratch(ctx, "enc.ssb", n * sizeof(C), &ptr));
    C* A = (C*)ptr;
    const int prec = sizeof(R) == 8 ? 1 : 0;
    OH_TRY(fft2d_enqueue(ctx, prec, nx, ny, field, A, nullptr, -1, 1, 0, st));
    ssb_mask<R><<<grid, 256, 0, st>>>(kind, nx, ny, A);
    OH_LAUNCH_CHECK();
    OH_TRY(fft2d_enqueue(ctx, prec, nx, ny, A, A, nullptr, 1, 1, 1, st));
    OH_TRY(reduce<R>(ctx, A, n, RED_MINMAX_SSB, (const R*)nullptr, &red1, st, "enc.red1"));
    ssb_finish<R><<<grid, 256, 0, st>>>(n, A, red1, (R*)out);
    OH_LAUNCH_CHECK();
    return OH_OK;
  }
  if (kind == OH_ENC_NUM_INTERFERENCE || kind == OH_ENC_BURCKHARDT || kind == OH_ENC_TWO_PHASE)
    OH_TRY(reduce<R>(ctx, field, n, RED_MAX_ABS, (const R*)nullptr, &red1, st, "enc.red1"));
  if (kind == OH_ENC_NUM_INTERFERENCE) {
    // max |U + max|U||^2, the reference value read on the device
    OH_TRY(reduce<R>(ctx, field, n, RED_MAX_NI, red1, &red2, st, "enc.red2"));
  }
  if (kind == OH_ENC_PHASE_ONLY_U8) OH_TRY(reduce<R>(ctx, field, n, RED_MAX_PHASE, (const R*)nullptr, &red1, st, "enc.red1"));
  KernelTimer kt(ctx, "encode_map", st);
  encode_map<R><<<grid, 256, 0, st>>>(kind, nx, ny, (const C*)field, red1, red2, out);
  OH_LAUNCH_CHECK();
  return OH_OK;
}

}  // namespace oh

using namespace oh;

extern "C" {

oh_status oh_encode(oh_ctx* ctx, oh_precision prec, int kind, int nx, int ny, const void* field, void* out, void* stream) {
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  CallScope cs(ctx, st);
  OH_TRY(cs.status());
  if (nx < 1 || ny < 1 || !field || !out) return fail(OH_ERR_INVALID_ARG, "oh_encode: bad size or null buffer");
  if (kind < OH_ENC_REAL || kind > OH_ENC_AMPLITUDE) return fail(OH_ERR_INVALID_ARG, "oh_encode: unknown encoding");
  if (prec == OH_FP64) return run_encode<double>(ctx, kind, nx, ny, field, out, st);
  return run_encode<float>(ctx, kind, nx, ny, field, out, st);
}

oh_status oh_normalize_u8(oh_ctx* ctx, oh_precision prec, int nx, int ny, const void* in, uint8_t* out, int round_half,
                          void* stream) {
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  CallScope cs(ctx, st);
  OH_TRY(cs.status());
  if (nx < 1 || ny < 1 || !in || !out) return fail(OH_ERR_INVALID_ARG, "oh_normalize_u8: bad size or null buffer");
  const size_t n = (size_t)nx * ny;
  const int grid = (int)std::min<size_t>((n + 255) / 256, oh::sm_count() * 16);
  if (prec == OH_FP64) {
    double* red;
    OH_TRY(reduce<double>(ctx, in, n, RED_MINMAX_REAL, (const double*)nullptr, &red, st, "norm.red"));
    normalize_u8_kernel<double><<<grid, 256, 0, st>>>(nx, ny, (const double*)in, red, out, round_half);
  } else {
    float* red;
    OH_TRY(reduce<float>(ctx, in, n, RED_MINMAX_REAL, (const float*)nullptr, &red, st, "norm.red"));
    normalize_u8_kernel<float><<<grid, 256, 0, st>>>(nx, ny, (const float*)in, red, out, round_half);
  }
  OH_LAUNCH_CHECK();
  return OH_OK;
}

}  // extern "C"
