// The learned surrogate around the plain layered angular-spectrum method
// (no reference counterpart; the plain method is HologramGenerator::
// Calc_Holo_GPU, HologramGenerator_GPU.cpp:246-302, built here as
// dm_row_pass / dm_col_fast):
//   1. the U-Net predicts the complex field on a mid plane z_mid between the
//      layers from the RGB-D frame;
//   2. optionally the plain method computes the same mid-plane field (its
//      layers propagated over z' - z_mid) and judges the prediction: the PSNR
//      of the mid-plane intensity |F|^2 (peak = max of the plain one), and
//      when it is below the threshold the plain field replaces the
//      prediction for this frame;
//   3. the chosen field is carried over z_mid to the hologram plane by the
//      same padded angular-spectrum pass, crop and symmetrization encoding as
//      the plain frame (oh_depthmap_propagate_field's path).
// Also here: the seeded RGB-D scene generator that feeds training.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>
#include "context.h"
#include "unet.cuh"

namespace oh {

namespace {

__host__ __device__ __forceinline__ uint64_t sm_fin(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
// value idx of the SplitMix64 stream of `seed`: finaliser of seed + (idx+1) * golden
__host__ __device__ __forceinline__ uint64_t sm_at(uint64_t seed, uint64_t idx) {
  return sm_fin(seed + (idx + 1ull) * 0x9E3779B97F4A7C15ull);
}
// double in [0, 1) from value i of stream `stream` of `seed` (53 bits)
__host__ __device__ __forceinline__ double sm_uniform(uint64_t seed, uint64_t stream, uint64_t i) {
  const uint64_t s = sm_at(seed, stream);
  return (double)(sm_at(s, i) >> 11) * (1.0 / 9007199254740992.0);
}

constexpr int kGaussInt = 20, kGaussDepth = 8;
constexpr int kGaussTotal = 3 * kGaussInt + kGaussDepth;

// Channel sums of one frame's Gaussians: R, G, B intensity (streams 3, 1, 5;
// 20 Gaussians, sigma 20-200 px scaled by min(h, w)/1080, amplitude 0.2-1)
// and depth (stream 2; 8 Gaussians, sigma 200-600 px scaled).  Block-wide
// maxima (and the depth minimum) go to mm[frame][5] through integer atomics
// on the non-negative float bits.
__global__ void __launch_bounds__(256) scene_sums(uint64_t seed, int h, int w, float4* __restrict__ sums,
                                                  unsigned* __restrict__ mm) {
  __shared__ float g[kGaussTotal][4];     // cx, cy, 1/(2 sigma^2), amplitude
  const int f = blockIdx.y;
  const uint64_t fs = seed + (uint64_t)f;
  const double scale = (double)min(h, w) / 1080.0;
  for (int k = threadIdx.x; k < kGaussTotal; k += blockDim.x) {
    int stream, j, chan;
    double s0, s1;
    if (k < 3 * kGaussInt) {
      chan = k / kGaussInt; j = k % kGaussInt;
      stream = chan == 0 ? 3 : chan == 1 ? 1 : 5;
      s0 = 20.0 * scale; s1 = 200.0 * scale;
    } else {
      j = k - 3 * kGaussInt; stream = 2; s0 = 200.0 * scale; s1 = 600.0 * scale;
    }
    const double ux = sm_uniform(fs, stream, 4 * j), uy = sm_uniform(fs, stream, 4 * j + 1);
    const double us = sm_uniform(fs, stream, 4 * j + 2), ua = sm_uniform(fs, stream, 4 * j + 3);
    const double sg = s0 + us * (s1 - s0);
    g[k][0] = (float)(ux * w);
    g[k][1] = (float)(uy * h);
    g[k][2] = (float)(1.0 / (2.0 * sg * sg));
    g[k][3] = (float)(0.2 + ua * 0.8);
  }
  __syncthreads();
  float mx0 = 0.f, mx1 = 0.f, mx2 = 0.f, mx3 = 0.f, mn3 = 3.4e38f;
  const long long np = (long long)h * w;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < np; p += (long long)gridDim.x * blockDim.x) {
    const float x = (float)(p % w), y = (float)(p / w);
    float acc[4];
    auto sum = [&](int k0, int k1) {
      float a = 0.f;
      for (int k = k0; k < k1; ++k) {
        const float dx = x - g[k][0], dy = y - g[k][1];
        a += g[k][3] * __expf(-(dx * dx + dy * dy) * g[k][2]);
      }
      return a;
    };
    acc[0] = sum(0, kGaussInt);
    acc[1] = sum(kGaussInt, 2 * kGaussInt);
    acc[2] = sum(2 * kGaussInt, 3 * kGaussInt);
    acc[3] = sum(3 * kGaussInt, kGaussTotal);
    sums[(long long)f * np + p] = make_float4(acc[0], acc[1], acc[2], acc[3]);
    mx0 = fmaxf(mx0, acc[0]); mx1 = fmaxf(mx1, acc[1]); mx2 = fmaxf(mx2, acc[2]);
    mx3 = fmaxf(mx3, acc[3]); mn3 = fminf(mn3, acc[3]);
  }
  unsigned* m = mm + 5 * f;
  atomicMax(m + 0, __float_as_uint(mx0));
  atomicMax(m + 1, __float_as_uint(mx1));
  atomicMax(m + 2, __float_as_uint(mx2));
  atomicMax(m + 3, __float_as_uint(mx3));
  atomicMin(m + 4, __float_as_uint(mn3));
}

__global__ void scene_quantize(int h, int w, const float4* __restrict__ sums, const unsigned* __restrict__ mm,
                               uchar4* __restrict__ rgbd) {
  const int f = blockIdx.y;
  const long long np = (long long)h * w;
  const unsigned* m = mm + 5 * f;
  const float i0 = 255.f / __uint_as_float(m[0]), i1 = 255.f / __uint_as_float(m[1]), i2 = 255.f / __uint_as_float(m[2]);
  const float dmin = __uint_as_float(m[4]), dr = fmaxf(__uint_as_float(m[3]) - dmin, 1e-30f);
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < np; p += (long long)gridDim.x * blockDim.x) {
    const float4 s = sums[(long long)f * np + p];
    auto q = [](float v) { return (unsigned char)fminf(fmaxf(rintf(v), 0.f), 255.f); };
    rgbd[(long long)f * np + p] = make_uchar4(q(s.x * i0), q(s.y * i1), q(s.z * i2), q(255.f * (s.w - dmin) / dr));
  }
}

// G and depth planes of an RGB-D frame (the plain method's inputs).
__global__ void rgbd_split(const uchar4* __restrict__ rgbd, long long np, uint8_t* __restrict__ g, uint8_t* __restrict__ d) {
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < np; p += (long long)gridDim.x * blockDim.x) {
    const uchar4 v = rgbd[p];
    g[p] = v.y;
    d[p] = v.w;
  }
}

// Comparison of the predicted mid-plane field a with the plain one b:
// acc[0] = sum |a - b|^2, acc[1] = sum |b|^2, acc[2] = sum (|a|^2 - |b|^2)^2;
// mx[0] = max |b|^2, mx[1] = max |a - b| (float bits).
__global__ void __launch_bounds__(256) sg_compare(const float2* __restrict__ a, const float2* __restrict__ b, long long np,
                                                  double* __restrict__ acc, unsigned* __restrict__ mx) {
  double s0 = 0, s1 = 0, s2 = 0;
  float m0 = 0.f, m1 = 0.f;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < np; p += (long long)gridDim.x * blockDim.x) {
    const float2 x = a[p], y = b[p];
    const float dx = x.x - y.x, dy = x.y - y.y;
    const float ia = x.x * x.x + x.y * x.y, ib = y.x * y.x + y.y * y.y;
    s0 += (double)(dx * dx + dy * dy);
    s1 += (double)ib;
    s2 += (double)(ia - ib) * (double)(ia - ib);
    m0 = fmaxf(m0, ib);
    m1 = fmaxf(m1, sqrtf(dx * dx + dy * dy));
  }
  __shared__ double red[3][8];
  __shared__ float redm[2][8];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    s0 += __shfl_xor_sync(0xffffffffu, s0, o);
    s1 += __shfl_xor_sync(0xffffffffu, s1, o);
    s2 += __shfl_xor_sync(0xffffffffu, s2, o);
    m0 = fmaxf(m0, __shfl_xor_sync(0xffffffffu, m0, o));
    m1 = fmaxf(m1, __shfl_xor_sync(0xffffffffu, m1, o));
  }
  const int wp = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) { red[0][wp] = s0; red[1][wp] = s1; red[2][wp] = s2; redm[0][wp] = m0; redm[1][wp] = m1; }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int k = 1; k < (int)(blockDim.x >> 5); ++k) {
      s0 += red[0][k]; s1 += red[1][k]; s2 += red[2][k];
      m0 = fmaxf(m0, redm[0][k]); m1 = fmaxf(m1, redm[1][k]);
    }
    atomicAdd(acc + 0, s0);
    atomicAdd(acc + 1, s1);
    atomicAdd(acc + 2, s2);
    atomicMax(mx + 0, __float_as_uint(m0));
    atomicMax(mx + 1, __float_as_uint(m1));
  }
}

}  // namespace

oh_status unet_forward(oh_unet* u, const uint8_t* rgbd, int n, int h, int w, float2* out, cudaStream_t st);
oh_status unet_validate_size(const oh_unet* u, int n, int h, int w);
oh_status depthmap_enqueue_f32(oh_ctx* ctx, const oh_depthmap_params* p, const uint8_t* img, const uint8_t* depth,
                               void* fringe, void* field, const void* src, double src_z, cudaStream_t st);
oh_ctx* unet_ctx(const oh_unet* u);

namespace {

// The plain method's field on the mid plane: the frame's layers propagated
// over z' - z_mid (levels shifted by -z_mid), with no single-sideband crop
// (the full field) and the reference constant source phase 1.  Inputs: the
// G and depth planes of rgbd.
oh_status surrogate_mid_field(oh_ctx* ctx, const oh_depthmap_params* p, double z_mid, const uint8_t* rgbd,
                              void* field_mid, cudaStream_t st) {
  if (!p || !rgbd || !field_mid) return fail(OH_ERR_INVALID_ARG, "null argument");
  const long long np = (long long)p->pnx * p->pny;
  void* ptr;
  OH_TRY(scratch(ctx, "sg.planes", (size_t)np * 2 + (size_t)np * sizeof(float) + 512, &ptr));
  uint8_t* g = static_cast<uint8_t*>(ptr);
  uint8_t* d = g + np;
  float* fr = reinterpret_cast<float*>(static_cast<char*>(ptr) + ((2 * np + 255) & ~255LL));
  {
    KernelTimer kt(ctx, "rgbd_split", st);
    rgbd_split<<<(int)std::min<long long>((np + 255) / 256, (long long)sm_count() * 8), 256, 0, st>>>(
        reinterpret_cast<const uchar4*>(rgbd), np, g, d);
    OH_LAUNCH_CHECK();
  }
  oh_depthmap_params q = *p;
  q.near_depthmap -= z_mid;
  q.far_depthmap -= z_mid;
  q.sig_location_x = 0;
  q.sig_location_y = 0;
  q.phase_mode = OH_PHASE_REFERENCE;
  q.rand_phase_re = 1.0;
  q.rand_phase_im = 0.0;
  q.transform_viewing_window = 0;
  return depthmap_enqueue_f32(ctx, &q, g, d, fr, field_mid, nullptr, 0.0, st);
}

}  // namespace

}  // namespace oh

using namespace oh;

extern "C" {

oh_status oh_scene_rgbd(oh_ctx* ctx, uint64_t seed, int n, int h, int w, uint8_t* rgbd, void* stream) {
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  CallScope cs(ctx, st);
  OH_TRY(cs.status());
  if (n < 1 || h < 1 || w < 1 || n > 65535 || !rgbd) return fail(OH_ERR_INVALID_ARG, "scene: bad sizes or null output");
  const long long np = (long long)h * w;
  void* ptr;
  OH_TRY(scratch(ctx, "scene.sums", (size_t)n * np * sizeof(float4) + 256 + (size_t)n * 5 * sizeof(unsigned), &ptr));
  float4* sums = static_cast<float4*>(ptr);
  unsigned* mm = reinterpret_cast<unsigned*>(static_cast<char*>(ptr) + (((size_t)n * np * sizeof(float4) + 255) & ~(size_t)255));
  // maxima start at +0.0, the depth minimum at the largest finite float
  std::vector<unsigned> init(5 * (size_t)n, 0u);
  for (int f = 0; f < n; ++f) init[5 * f + 4] = 0x7f7fffffu;
  OH_CUDA_TRY(cudaMemcpyAsync(mm, init.data(), init.size() * sizeof(unsigned), cudaMemcpyHostToDevice, st));
  const int bx = (int)std::min<long long>((np + 255) / 256, (long long)sm_count() * 4);
  {
    KernelTimer kt(ctx, "scene_sums", st);
    scene_sums<<<dim3(bx, n), 256, 0, st>>>(seed, h, w, sums, mm);
    OH_LAUNCH_CHECK();
  }
  KernelTimer kt(ctx, "scene_quantize", st);
  scene_quantize<<<dim3(bx, n), 256, 0, st>>>(h, w, sums, mm, reinterpret_cast<uchar4*>(rgbd));
  OH_LAUNCH_CHECK();
  return OH_OK;
}

oh_status oh_surrogate_mid_field(oh_ctx* ctx, const oh_depthmap_params* p, double z_mid, const uint8_t* rgbd,
                                 void* field_mid, void* stream) {
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  CallScope cs(ctx, st);
  OH_TRY(cs.status());
  return surrogate_mid_field(ctx, p, z_mid, rgbd, field_mid, st);
}

oh_status oh_surrogate_generate(oh_ctx* ctx, oh_unet* net, const oh_surrogate_params* sp, const uint8_t* rgbd,
                                void* fringe_out, void* field_mid_out, oh_surrogate_report* rep, void* stream) {
  if (!ctx || !net || !sp || !rgbd || !fringe_out) return fail(OH_ERR_INVALID_ARG, "null argument");
  if (unet_ctx(net) != ctx) return fail(OH_ERR_INVALID_ARG, "the network belongs to another context");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  CallScope cs(ctx, st);
  OH_TRY(cs.status());
  const oh_depthmap_params* p = &sp->dm;
  const long long np = (long long)p->pnx * p->pny;
  OH_TRY(tc_arch_check());
  OH_TRY(unet_validate_size(net, 1, p->pny, p->pnx));
  void* pred;
  OH_TRY(scratch(ctx, "sg.pred", (size_t)np * sizeof(float2), &pred));
  OH_TRY(unet_forward(net, rgbd, 1, p->pny, p->pnx, static_cast<float2*>(pred), st));
  const void* chosen = pred;
  oh_surrogate_report r{};
  r.psnr_db = -1.f;
  if (sp->check) {
    void* plain;
    void* accp;
    OH_TRY(scratch(ctx, "sg.plain", (size_t)np * sizeof(float2), &plain));
    OH_TRY(scratch(ctx, "sg.acc", 64, &accp));
    OH_TRY(surrogate_mid_field(ctx, p, sp->z_mid, rgbd, plain, st));
    double* acc = static_cast<double*>(accp);
    unsigned* mx = reinterpret_cast<unsigned*>(acc + 3);
    OH_CUDA_TRY(cudaMemsetAsync(accp, 0, 64, st));
    {
      KernelTimer kt(ctx, "sg_compare", st);
      sg_compare<<<(int)std::min<long long>((np + 255) / 256, (long long)sm_count() * 4), 256, 0, st>>>(
          static_cast<const float2*>(pred), static_cast<const float2*>(plain), np, acc, mx);
      OH_LAUNCH_CHECK();
    }
    double h_acc[3];
    unsigned h_mx[2];
    OH_CUDA_TRY(cudaMemcpyAsync(h_acc, acc, sizeof(h_acc), cudaMemcpyDeviceToHost, st));
    OH_CUDA_TRY(cudaMemcpyAsync(h_mx, mx, sizeof(h_mx), cudaMemcpyDeviceToHost, st));
    OH_CUDA_TRY(cudaStreamSynchronize(st));
    float peak, maxerr;
    std::memcpy(&peak, &h_mx[0], 4);
    std::memcpy(&maxerr, &h_mx[1], 4);
    const double mse = h_acc[2] / (double)np;
    r.psnr_db = mse > 0 ? (float)(10.0 * std::log10((double)peak * peak / mse)) : 999.f;
    r.rel_err = h_acc[1] > 0 ? (float)std::sqrt(h_acc[0] / h_acc[1]) : 0.f;
    r.max_abs_err = peak > 0 ? maxerr / std::sqrt(peak) : 0.f;
    r.rms_err = peak > 0 ? (float)(std::sqrt(h_acc[0] / (double)np) / std::sqrt((double)peak)) : 0.f;
    r.checked = 1;
    if (!(r.psnr_db >= sp->psnr_threshold_db)) {
      r.fell_back = 1;
      chosen = plain;
    }
  }
  if (field_mid_out)
    OH_CUDA_TRY(cudaMemcpyAsync(field_mid_out, chosen, (size_t)np * sizeof(float2), cudaMemcpyDeviceToDevice, st));
  oh_depthmap_params q = *p;
  q.transform_viewing_window = 0;
  OH_TRY(depthmap_enqueue_f32(ctx, &q, nullptr, nullptr, fringe_out, nullptr, chosen, sp->z_mid, st));
  if (rep) *rep = r;
  return OH_OK;
}

}  // extern "C"
