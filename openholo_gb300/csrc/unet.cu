// The learned surrogate's network: a 4-level U-Net (3x3 convolutions, ReLU,
// 2x2 average pooling, nearest 2x upsampling with skip concatenation, a 1x1
// head) with BF16 weights and activations and FP32 accumulation, trained by
// Adam.  No reference counterpart: it predicts the mid-plane complex field
// of the plain layered angular-spectrum method
// (HologramGenerator_GPU.cpp:246-302), which produces its training targets.
//
// Every convolution of the forward and backward passes runs on the tcgen05
// tensor cores (unet_conv.cu); the CUDA-core kernels here do the layout work
// (input packing, pooling, upsampling and their adjoints fused with the ReLU
// masks), the 1x1 head fused with the loss and its gradients, the bias
// gradients and the Adam update (which also writes the BF16 weight copies
// the convolutions read: [cout][taps*cin] for the forward pass and
// [cin][taps*cout] for the input gradient).
//
// Memory (owned by the network, allocated at creation for its maximum batch
// and frame size): FP32 master weights, Adam moments, per-layer FP32 weight
// gradients dW^T[taps*cin][cout], BF16 weight copies, and the activations of
// one batch (NHWC BF16; level l has c_l = 32 << l channels; the encoder
// output of levels 0-2 lives in the first c_l channels of its concatenation
// buffer, whose last c_{l+1} channels receive the upsampled level below).
#include <cuda_bf16.h>
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>
#include "context.h"
#include "unet.cuh"

namespace oh {

namespace {

constexpr int kLevels = 4;
constexpr int kInCh = 4, kOutCh = 2, kInPad = 32;

// per-layer kernel-timer names (OH_UNET_LAYER_TIMING=1 at creation)
constexpr const char* kLayerTimerNames[3][15] = {
    {"fwd_enc0a", "fwd_enc0b", "fwd_enc1a", "fwd_enc1b", "fwd_enc2a", "fwd_enc2b", "fwd_enc3a", "fwd_enc3b",
     "fwd_dec2a", "fwd_dec2b", "fwd_dec1a", "fwd_dec1b", "fwd_dec0a", "fwd_dec0b", "fwd_head"},
    {"dgrad_enc0a", "dgrad_enc0b", "dgrad_enc1a", "dgrad_enc1b", "dgrad_enc2a", "dgrad_enc2b", "dgrad_enc3a",
     "dgrad_enc3b", "dgrad_dec2a", "dgrad_dec2b", "dgrad_dec1a", "dgrad_dec1b", "dgrad_dec0a", "dgrad_dec0b",
     "dgrad_head"},
    {"wgrad_enc0a", "wgrad_enc0b", "wgrad_enc1a", "wgrad_enc1b", "wgrad_enc2a", "wgrad_enc2b", "wgrad_enc3a",
     "wgrad_enc3b", "wgrad_dec2a", "wgrad_dec2b", "wgrad_dec1a", "wgrad_dec1b", "wgrad_dec0a", "wgrad_dec0b",
     "wgrad_head"}};

struct Layer {
  int cin, cin_pad, cout, taps;
  const char* tn[3] = {"unet_conv_fwd", "unet_conv_dgrad", "unet_conv_wgrad"};   // timer names
  size_t off_w, off_b;            // offsets in the flat FP32 parameter array
  float* dwt;                     // [taps*cin_pad][cout]
  float* db;                      // [cout]
  __nv_bfloat16* wf;              // [cout][taps*cin_pad]
  __nv_bfloat16* wd;              // [cin_pad][taps*cout]
};

__device__ __forceinline__ float bf(const __nv_bfloat16 v) { return __bfloat162float(v); }

// rgbd uint8 [n][h][w][4] -> BF16 [n][h][w][32]: channels 0-2 = R,G,B / 255,
// channel 3 = depth_lut[depth byte], channels 4-31 zero.
__global__ void unet_pack_input(const uint8_t* __restrict__ rgbd, const float* __restrict__ lut, long long npix,
                                __nv_bfloat16* __restrict__ out) {
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < npix; p += (long long)gridDim.x * blockDim.x) {
    const uchar4 v = reinterpret_cast<const uchar4*>(rgbd)[p];
    uint4 o[4];
    __nv_bfloat162* ob = reinterpret_cast<__nv_bfloat162*>(o);
    ob[0] = __floats2bfloat162_rn(v.x * (1.f / 255.f), v.y * (1.f / 255.f));
    ob[1] = __floats2bfloat162_rn(v.z * (1.f / 255.f), lut[v.w]);
#pragma unroll
    for (int i = 2; i < 16; ++i) ob[i] = __floats2bfloat162_rn(0.f, 0.f);
    uint4* dst = reinterpret_cast<uint4*>(out + p * kInPad);
#pragma unroll
    for (int i = 0; i < 4; ++i) dst[i] = o[i];
  }
}

// 2x2 average pooling: dst[n][y][x][c] = mean of src[n][2y+a][2x+b][c]
// (c < C, eight channels per thread).
__global__ void unet_pool(const __nv_bfloat16* __restrict__ src, int src_cs, int C, int H, int W, int n,
                          __nv_bfloat16* __restrict__ dst, int dst_cs) {
  const int h = H / 2, w = W / 2, c8 = C / 8;
  const long long total = (long long)n * h * w * c8;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
    const int c = (int)(i % c8) * 8;
    long long p = i / c8;
    const int x = (int)(p % w); p /= w;
    const int y = (int)(p % h);
    const int b = (int)(p / h);
    float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
#pragma unroll
    for (int dy = 0; dy < 2; ++dy)
#pragma unroll
      for (int dx = 0; dx < 2; ++dx) {
        const uint4 v = *reinterpret_cast<const uint4*>(src + (((size_t)b * H + 2 * y + dy) * W + 2 * x + dx) * src_cs + c);
        const __nv_bfloat162* vb = reinterpret_cast<const __nv_bfloat162*>(&v);
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          const float2 f = __bfloat1622float2(vb[e]);
          acc[2 * e] += f.x;
          acc[2 * e + 1] += f.y;
        }
      }
    uint4 o;
    __nv_bfloat162* ob = reinterpret_cast<__nv_bfloat162*>(&o);
#pragma unroll
    for (int e = 0; e < 4; ++e) ob[e] = __floats2bfloat162_rn(0.25f * acc[2 * e], 0.25f * acc[2 * e + 1]);
    *reinterpret_cast<uint4*>(dst + (((size_t)b * h + y) * w + x) * dst_cs + c) = o;
  }
}

// nearest 2x upsampling into channels [off, off + C) of dst:
// dst[n][Y][X][off + c] = src[n][Y/2][X/2][c], src h x w, dst 2h x 2w.
__global__ void unet_up(const __nv_bfloat16* __restrict__ src, int src_cs, int C, int h, int w, int n,
                        __nv_bfloat16* __restrict__ dst, int dst_cs, int off) {
  const int H = 2 * h, W = 2 * w, c8 = C / 8;
  const long long total = (long long)n * H * W * c8;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
    const int c = (int)(i % c8) * 8;
    long long p = i / c8;
    const int X = (int)(p % W); p /= W;
    const int Y = (int)(p % H);
    const int b = (int)(p / H);
    const uint4 v = *reinterpret_cast<const uint4*>(src + (((size_t)b * h + Y / 2) * w + X / 2) * src_cs + c);
    *reinterpret_cast<uint4*>(dst + (((size_t)b * H + Y) * W + X) * dst_cs + off + c) = v;
  }
}

// adjoint of the upsampling, times the ReLU mask of its source:
// out[n][y][x][c] = (sum_{a,b} d[n][2y+a][2x+b][off + c]) * (mask[n][y][x][c] > 0)
__global__ void unet_up_back_mask(const __nv_bfloat16* __restrict__ d, int d_cs, int off, int C, int h, int w, int n,
                                  const __nv_bfloat16* __restrict__ mask, int mask_cs,
                                  __nv_bfloat16* __restrict__ out, int out_cs) {
  const int H = 2 * h, W = 2 * w, c8 = C / 8;
  const long long total = (long long)n * h * w * c8;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
    const int c = (int)(i % c8) * 8;
    long long p = i / c8;
    const int x = (int)(p % w); p /= w;
    const int y = (int)(p % h);
    const int b = (int)(p / h);
    float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
#pragma unroll
    for (int dy = 0; dy < 2; ++dy)
#pragma unroll
      for (int dx = 0; dx < 2; ++dx) {
        const uint4 v = *reinterpret_cast<const uint4*>(d + (((size_t)b * H + 2 * y + dy) * W + 2 * x + dx) * d_cs + off + c);
        const __nv_bfloat162* vb = reinterpret_cast<const __nv_bfloat162*>(&v);
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          const float2 f = __bfloat1622float2(vb[e]);
          acc[2 * e] += f.x;
          acc[2 * e + 1] += f.y;
        }
      }
    const size_t q = ((size_t)b * h + y) * w + x;
    const uint4 mv = *reinterpret_cast<const uint4*>(mask + q * mask_cs + c);
    const __nv_bfloat162* mb = reinterpret_cast<const __nv_bfloat162*>(&mv);
    uint4 o;
    __nv_bfloat162* ob = reinterpret_cast<__nv_bfloat162*>(&o);
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const float2 m = __bfloat1622float2(mb[e]);
      ob[e] = __floats2bfloat162_rn(m.x > 0.f ? acc[2 * e] : 0.f, m.y > 0.f ? acc[2 * e + 1] : 0.f);
    }
    *reinterpret_cast<uint4*>(out + q * out_cs + c) = o;
  }
}

// gradient of an encoder output that feeds both the skip connection and the
// pooling, times its ReLU mask:
// out[n][Y][X][c] = (skip[n][Y][X][c] + dpool[n][Y/2][X/2][c] / 4) * (mask[n][Y][X][c] > 0)
__global__ void unet_skip_pool_back_mask(const __nv_bfloat16* __restrict__ skip, int skip_cs,
                                         const __nv_bfloat16* __restrict__ dpool, int dpool_cs, int C, int H, int W,
                                         int n, const __nv_bfloat16* __restrict__ mask, int mask_cs,
                                         __nv_bfloat16* __restrict__ out, int out_cs) {
  const int h = H / 2, w = W / 2, c8 = C / 8;
  const long long total = (long long)n * H * W * c8;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
    const int c = (int)(i % c8) * 8;
    long long p = i / c8;
    const int X = (int)(p % W); p /= W;
    const int Y = (int)(p % H);
    const int b = (int)(p / H);
    const size_t q = ((size_t)b * H + Y) * W + X;
    const uint4 sv = *reinterpret_cast<const uint4*>(skip + q * skip_cs + c);
    const uint4 pv = *reinterpret_cast<const uint4*>(dpool + (((size_t)b * h + Y / 2) * w + X / 2) * dpool_cs + c);
    const uint4 mv = *reinterpret_cast<const uint4*>(mask + q * mask_cs + c);
    const __nv_bfloat162* sb = reinterpret_cast<const __nv_bfloat162*>(&sv);
    const __nv_bfloat162* pb = reinterpret_cast<const __nv_bfloat162*>(&pv);
    const __nv_bfloat162* mb = reinterpret_cast<const __nv_bfloat162*>(&mv);
    uint4 o;
    __nv_bfloat162* ob = reinterpret_cast<__nv_bfloat162*>(&o);
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const float2 s = __bfloat1622float2(sb[e]), d = __bfloat1622float2(pb[e]), m = __bfloat1622float2(mb[e]);
      ob[e] = __floats2bfloat162_rn(m.x > 0.f ? s.x + 0.25f * d.x : 0.f, m.y > 0.f ? s.y + 0.25f * d.y : 0.f);
    }
    *reinterpret_cast<uint4*>(out + q * out_cs + c) = o;
  }
}

// bias gradient: db[c] += sum over pixels of dz[p][c] (C a multiple of 8,
// at most 256).  Thread t takes channels 8 (t % (C/8)) .. + 7 of pixel lane
// t / (C/8) with one 16-byte load per pixel; the lanes are summed in shared
// memory and added with one atomic per channel and block.
__global__ void __launch_bounds__(256) unet_bias_grad(const __nv_bfloat16* __restrict__ dz, int cs, int C, long long npix,
                                                      float* __restrict__ db) {
  __shared__ float red[256][9];
  const int c8n = C / 8;
  const int lanes = 256 / c8n;
  const int c8 = threadIdx.x % c8n, r = threadIdx.x / c8n;
  float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  if (r < lanes) {
    for (long long p = blockIdx.x * (long long)lanes + r; p < npix; p += (long long)gridDim.x * lanes) {
      const uint4 v = *reinterpret_cast<const uint4*>(dz + p * cs + 8 * c8);
      const __nv_bfloat162* vb = reinterpret_cast<const __nv_bfloat162*>(&v);
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const float2 f = __bfloat1622float2(vb[e]);
        acc[2 * e] += f.x;
        acc[2 * e + 1] += f.y;
      }
    }
  }
#pragma unroll
  for (int e = 0; e < 8; ++e) red[threadIdx.x][e] = acc[e];
  __syncthreads();
  if (threadIdx.x < C) {
    const int cc8 = threadIdx.x / 8, e = threadIdx.x % 8;
    float sum = 0.f;
    for (int k = 0; k < lanes; ++k) sum += red[k * c8n + cc8][e];
    atomicAdd(db + threadIdx.x, sum);
  }
}

// 1x1 head (32 -> 2 channels, FP32 weights): pred[p][k] = b[k] + sum_c W[k][c] x[p][c].
// Inference: out[p] = scale * pred[p] (float2).  Training (target != null):
// loss += sum (pred - target/scale)^2 / count, dpred = 2 (pred - t) / count,
// head gradients (dW[k][c] = sum dpred[k] x[c], db[k] = sum dpred[k]) and the
// gradient of x times its ReLU mask, dx[p][c] = sum_k dpred[k] W[k][c] (x > 0).
constexpr int kHeadThreads = 256;
__global__ void __launch_bounds__(kHeadThreads) unet_head(const __nv_bfloat16* __restrict__ x, long long npix,
                                                          const float* __restrict__ Wb, float scale,
                                                          float2* __restrict__ out, const float2* __restrict__ target,
                                                          float inv_count, float* __restrict__ loss,
                                                          float* __restrict__ gW, __nv_bfloat16* __restrict__ dx) {
  __shared__ float w[2 * 32 + 2];
  for (int i = threadIdx.x; i < 66; i += blockDim.x) w[i] = Wb[i];
  __syncthreads();
  const bool train = target != nullptr;
  float gacc[66];
  if (train) {
#pragma unroll
    for (int i = 0; i < 66; ++i) gacc[i] = 0.f;
  }
  float lacc = 0.f;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < npix; p += (long long)gridDim.x * blockDim.x) {
    float xv[32];
    const uint4* xp = reinterpret_cast<const uint4*>(x + p * 32);
#pragma unroll
    for (int g = 0; g < 4; ++g) {
      const uint4 v = xp[g];
      const __nv_bfloat162* vb = reinterpret_cast<const __nv_bfloat162*>(&v);
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const float2 f = __bfloat1622float2(vb[e]);
        xv[g * 8 + 2 * e] = f.x;
        xv[g * 8 + 2 * e + 1] = f.y;
      }
    }
    float p0 = w[64], p1 = w[65];
#pragma unroll
    for (int c = 0; c < 32; ++c) { p0 = fmaf(w[c], xv[c], p0); p1 = fmaf(w[32 + c], xv[c], p1); }
    if (!train) {
      out[p] = make_float2(scale * p0, scale * p1);
      continue;
    }
    const float2 t = target[p];
    const float e0 = p0 - t.x / scale, e1 = p1 - t.y / scale;
    lacc += e0 * e0 + e1 * e1;
    const float d0 = 2.f * e0 * inv_count, d1 = 2.f * e1 * inv_count;
#pragma unroll
    for (int c = 0; c < 32; ++c) { gacc[c] = fmaf(d0, xv[c], gacc[c]); gacc[32 + c] = fmaf(d1, xv[c], gacc[32 + c]); }
    gacc[64] += d0;
    gacc[65] += d1;
    uint4 o[4];
    __nv_bfloat162* ob = reinterpret_cast<__nv_bfloat162*>(o);
#pragma unroll
    for (int c = 0; c < 32; c += 2) {
      const float g0 = xv[c] > 0.f ? d0 * w[c] + d1 * w[32 + c] : 0.f;
      const float g1 = xv[c + 1] > 0.f ? d0 * w[c + 1] + d1 * w[33 + c] : 0.f;
      ob[c / 2] = __floats2bfloat162_rn(g0, g1);
    }
    uint4* dp = reinterpret_cast<uint4*>(dx + p * 32);
#pragma unroll
    for (int g = 0; g < 4; ++g) dp[g] = o[g];
  }
  if (!train) return;
  // block reduction of the 66 gradient sums and the loss
  __shared__ float red[kHeadThreads / 32][67];
  const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
#pragma unroll
  for (int i = 0; i < 66; ++i) {
    float v = gacc[i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) red[wp][i] = v;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) lacc += __shfl_xor_sync(0xffffffffu, lacc, o);
  if (lane == 0) red[wp][66] = lacc;
  __syncthreads();
  if (threadIdx.x < 67) {
    float s = 0.f;
    for (int k = 0; k < kHeadThreads / 32; ++k) s += red[k][threadIdx.x];
    if (threadIdx.x < 66) atomicAdd(gW + threadIdx.x, s);
    else atomicAdd(loss, s * inv_count);
  }
}

// Adam on one layer: master weights [cout][taps][cin] and bias; gradients
// dW^T[taps*cin_pad][cout] (the head's: [cout][cin], rowmajor_grad = 1) and
// db[cout]; writes the BF16 copies
// wf[co][t*cin_pad + ci] and (wd != null) wd[ci][t*cout + co].
struct AdamHyper { float lr, b1, b2, eps, c1, c2; };   // c1 = 1/(1-b1^t), c2 = 1/(1-b2^t)

__global__ void unet_adam_layer(float* __restrict__ W, float* __restrict__ m, float* __restrict__ v,
                                const float* __restrict__ dwt, const float* __restrict__ db, int cout, int taps, int cin,
                                int cin_pad, AdamHyper h, int update, int rowmajor_grad, __nv_bfloat16* __restrict__ wf,
                                __nv_bfloat16* __restrict__ wd) {
  const long long nw = (long long)cout * taps * cin;
  const long long total = nw + cout;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
    float g;
    int co = 0, t = 0, ci = 0;
    if (i < nw) {
      ci = (int)(i % cin);
      t = (int)((i / cin) % taps);
      co = (int)(i / ((long long)cin * taps));
      g = rowmajor_grad ? dwt[(size_t)co * cin + ci] : dwt[((size_t)t * cin_pad + ci) * cout + co];
    } else {
      g = db[i - nw];
    }
    float wv = W[i];
    if (update) {
      const float mi = h.b1 * m[i] + (1.f - h.b1) * g;
      const float vi = h.b2 * v[i] + (1.f - h.b2) * g * g;
      m[i] = mi;
      v[i] = vi;
      wv -= h.lr * (mi * h.c1) / (sqrtf(vi * h.c2) + h.eps);
      W[i] = wv;
    }
    if (i < nw) {
      const __nv_bfloat16 b = __float2bfloat16_rn(wv);
      wf[(size_t)co * taps * cin_pad + (size_t)t * cin_pad + ci] = b;
      if (wd) wd[(size_t)ci * taps * cout + (size_t)t * cout + co] = b;
    }
  }
}

inline int grid_for(long long work, int threads = 256) {
  const long long g = (work + threads - 1) / threads;
  return (int)std::max(1LL, std::min<long long>(g, (long long)sm_count() * 16));
}

}  // namespace

}  // namespace oh

struct oh_unet {
  oh_ctx* ctx = nullptr;
  int chans[oh::kLevels] = {32, 64, 128, 256};
  int max_n = 0, max_h = 0, max_w = 0;
  float out_scale = 1.f;
  std::vector<oh::Layer> layers;      // enc0a, enc0b, ..., enc3b, dec2a, dec2b, ..., dec0b, head
  size_t n_params = 0;
  float* P = nullptr;                 // FP32 master parameters (flat)
  float* M = nullptr;
  float* V = nullptr;
  float* G = nullptr;                 // gradient arena (dW^T and db of every layer; head: [2][32] + [2])
  size_t g_floats = 0;
  __nv_bfloat16* wbuf = nullptr;      // BF16 weight copies
  float* lut = nullptr;               // [256] depth channel values
  float* loss = nullptr;              // device scalar
  int step = 0;
  // activations
  std::vector<void*> allocs;
  __nv_bfloat16* in0 = nullptr;
  __nv_bfloat16* A[oh::kLevels] = {};       // encoder conv a outputs
  __nv_bfloat16* CAT[oh::kLevels] = {};     // levels 0-2: [E_l | up(D_{l+1})]; level 3: E_3 alone
  __nv_bfloat16* P_[oh::kLevels] = {};      // pooled inputs of levels 1-3
  __nv_bfloat16* DA[oh::kLevels] = {};      // decoder conv a outputs (levels 0-2)
  __nv_bfloat16* D[oh::kLevels] = {};       // decoder conv b outputs (levels 0-2)
  __nv_bfloat16* dCAT[oh::kLevels] = {};    // gradients of the concatenations (levels 0-2)
  __nv_bfloat16* dZ1 = nullptr;             // gradient scratch, largest level
  __nv_bfloat16* dZ2 = nullptr;
  __nv_bfloat16* dP[oh::kLevels] = {};      // gradients of the pooled inputs (levels 1-3)
};

namespace oh {
namespace {

int cat_cs(const oh_unet* u, int l) { return l < kLevels - 1 ? u->chans[l] + u->chans[l + 1] : u->chans[l]; }

oh_status dev_alloc(oh_unet* u, size_t bytes, void** p) {
  cudaError_t e = cudaMalloc(p, std::max<size_t>(bytes, 256));
  if (e != cudaSuccess) { cudaGetLastError(); return fail(OH_ERR_ALLOC, std::string("U-Net buffer of ") + std::to_string(bytes) + " bytes"); }
  u->allocs.push_back(*p);
  return OH_OK;
}

uint64_t sm64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

// He-normal initial weights from a SplitMix64 stream (Box-Muller), zero biases.
void init_params(const oh_unet* u, uint64_t seed, std::vector<float>& host) {
  host.assign(u->n_params, 0.f);
  uint64_t s = sm64(seed);
  auto unif = [&]() { s = sm64(s); return ((s >> 11) + 0.5) * (1.0 / 9007199254740992.0); };
  for (const Layer& L : u->layers) {
    const size_t nw = (size_t)L.cout * L.taps * L.cin;
    const double sd = std::sqrt(2.0 / (L.taps * L.cin)) * (L.taps == 1 ? 0.1 : 1.0);
    for (size_t i = 0; i < nw; ++i) {
      const double a = unif(), b = unif();
      host[L.off_w + i] = (float)(sd * std::sqrt(-2.0 * std::log(a)) * std::cos(2.0 * M_PI * b));
    }
  }
}

}  // namespace

// Pixels of a level for a batch of n frames of h x w.
static inline long long lvl_pix(int n, int h, int w, int l) { return (long long)n * (h >> l) * (w >> l); }

oh_status unet_validate_size(const oh_unet* u, int n, int h, int w) {
  if (n < 1 || h < 8 || w < 8 || n > u->max_n || h > u->max_h || w > u->max_w)
    return fail(OH_ERR_INVALID_ARG, "U-Net: batch or frame size outside 1..max (and at least 8 x 8)");
  if (h % 8 || w % 8) return fail(OH_ERR_UNSUPPORTED_SIZE, "U-Net: frame sides must be multiples of 8 (three 2x poolings)");
  for (int l = 0; l < kLevels; ++l) {
    const int wl = w >> l;
    if (wl < 128 && 128 % wl) return fail(OH_ERR_UNSUPPORTED_SIZE, "U-Net: level widths below 128 must divide 128");
  }
  return OH_OK;
}

// Forward pass of a batch; the activations stay for the backward pass.
// out (nullable) receives scale * prediction as float2 [n][h][w].
oh_status unet_forward(oh_unet* u, const uint8_t* rgbd, int n, int h, int w, float2* out, cudaStream_t st) {
  oh_ctx* ctx = u->ctx;
  const long long np0 = lvl_pix(n, h, w, 0);
  {
    KernelTimer kt(ctx, "unet_pack_input", st);
    unet_pack_input<<<grid_for(np0), 256, 0, st>>>(rgbd, u->lut, np0, u->in0);
    OH_LAUNCH_CHECK();
  }
  auto conv = [&](const Layer& L, const void* x, int x_cs, int hl, int wl, void* y, int y_cs) {
    ConvDesc d{};
    d.taps = L.taps; d.sign = 1; d.n = n; d.h = hl; d.w = wl; d.cin = L.cin_pad; d.cout = L.cout;
    d.x = x; d.x_cs = x_cs; d.w_mat = L.wf; d.bias = u->P + L.off_b; d.relu = 1;
    d.out = y; d.out_cs = y_cs;
    return conv_enqueue(ctx, d, st, L.tn[0]);
  };
  // encoder
  const void* xin = u->in0;
  int xin_cs = kInPad;
  for (int l = 0; l < kLevels; ++l) {
    const int hl = h >> l, wl = w >> l, c = u->chans[l];
    OH_TRY(conv(u->layers[2 * l], xin, xin_cs, hl, wl, u->A[l], c));
    OH_TRY(conv(u->layers[2 * l + 1], u->A[l], c, hl, wl, u->CAT[l], cat_cs(u, l)));
    if (l + 1 < kLevels) {
      KernelTimer kt(ctx, "unet_pool", st);
      unet_pool<<<grid_for(lvl_pix(n, h, w, l + 1) * c / 8), 256, 0, st>>>(u->CAT[l], cat_cs(u, l), c, hl, wl, n,
                                                                           u->P_[l + 1], c);
      OH_LAUNCH_CHECK();
      xin = u->P_[l + 1];
      xin_cs = c;
    }
  }
  // decoder
  const __nv_bfloat16* below = u->CAT[kLevels - 1];
  int below_cs = u->chans[kLevels - 1];
  for (int l = kLevels - 2; l >= 0; --l) {
    const int hl = h >> l, wl = w >> l, c = u->chans[l], cb = u->chans[l + 1];
    {
      KernelTimer kt(ctx, "unet_up", st);
      unet_up<<<grid_for(lvl_pix(n, h, w, l) * cb / 8), 256, 0, st>>>(below, below_cs, cb, hl / 2, wl / 2, n, u->CAT[l],
                                                                      cat_cs(u, l), c);
      OH_LAUNCH_CHECK();
    }
    const Layer& La = u->layers[2 * kLevels + 2 * (kLevels - 2 - l)];
    const Layer& Lb = u->layers[2 * kLevels + 2 * (kLevels - 2 - l) + 1];
    OH_TRY(conv(La, u->CAT[l], cat_cs(u, l), hl, wl, u->DA[l], c));
    OH_TRY(conv(Lb, u->DA[l], c, hl, wl, u->D[l], c));
    below = u->D[l];
    below_cs = c;
  }
  if (out) {
    const Layer& H = u->layers.back();
    KernelTimer kt(ctx, "unet_head", st);
    unet_head<<<grid_for(np0, kHeadThreads), kHeadThreads, 0, st>>>(u->D[0], np0, u->P + H.off_w, u->out_scale, out,
                                                                    nullptr, 0.f, nullptr, nullptr, nullptr);
    OH_LAUNCH_CHECK();
  }
  return OH_OK;
}

// Loss and every gradient of the batch whose forward pass just ran.
oh_status unet_backward(oh_unet* u, const float2* target, int n, int h, int w, cudaStream_t st) {
  oh_ctx* ctx = u->ctx;
  OH_CUDA_TRY(cudaMemsetAsync(u->G, 0, u->g_floats * sizeof(float), st));
  OH_CUDA_TRY(cudaMemsetAsync(u->loss, 0, sizeof(float), st));
  const long long np0 = lvl_pix(n, h, w, 0);
  const Layer& H = u->layers.back();
  {
    KernelTimer kt(ctx, "unet_head_loss", st);
    unet_head<<<grid_for(np0, kHeadThreads), kHeadThreads, 0, st>>>(u->D[0], np0, u->P + H.off_w, u->out_scale,
                                                                    nullptr, target, 1.f / (2.f * (float)np0), u->loss,
                                                                    H.dwt, u->dZ1);
    OH_LAUNCH_CHECK();
  }
  auto wgrad = [&](const Layer& L, const void* x, int x_cs, const void* dz, int hl, int wl) -> oh_status {
    WgradDesc d{};
    d.taps = L.taps; d.n = n; d.h = hl; d.w = wl; d.cin = L.cin_pad; d.cout = L.cout;
    d.x = x; d.x_cs = x_cs; d.dz = dz; d.dz_cs = L.cout; d.dwt = L.dwt;
    OH_TRY(wgrad_enqueue(ctx, d, st, L.tn[2]));
    KernelTimer kt(ctx, "unet_bias_grad", st);
    const long long np = (long long)n * hl * wl;
    unet_bias_grad<<<grid_for(np * L.cout / 8), 256, 0, st>>>(
        static_cast<const __nv_bfloat16*>(dz), L.cout, L.cout, np, L.db);
    OH_LAUNCH_CHECK();
    return OH_OK;
  };
  auto dgrad = [&](const Layer& L, const void* dz, int hl, int wl, const void* mask, int mask_cs, void* out,
                   int out_cs) -> oh_status {
    ConvDesc d{};
    d.taps = L.taps; d.sign = -1; d.n = n; d.h = hl; d.w = wl; d.cin = L.cout; d.cout = L.cin_pad;
    d.x = dz; d.x_cs = L.cout; d.w_mat = L.wd; d.bias = nullptr; d.relu = 0; d.mask = mask; d.mask_cs = mask_cs;
    d.out = out; d.out_cs = out_cs;
    return conv_enqueue(ctx, d, st, L.tn[1]);
  };
  // decoder, top level first: dZ1 holds the gradient of dec{l}b's pre-activation
  for (int l = 0; l < kLevels - 1; ++l) {
    const int hl = h >> l, wl = w >> l, c = u->chans[l], cb = u->chans[l + 1];
    const Layer& La = u->layers[2 * kLevels + 2 * (kLevels - 2 - l)];
    const Layer& Lb = u->layers[2 * kLevels + 2 * (kLevels - 2 - l) + 1];
    OH_TRY(wgrad(Lb, u->DA[l], c, u->dZ1, hl, wl));
    OH_TRY(dgrad(Lb, u->dZ1, hl, wl, u->DA[l], c, u->dZ2, c));
    OH_TRY(wgrad(La, u->CAT[l], cat_cs(u, l), u->dZ2, hl, wl));
    OH_TRY(dgrad(La, u->dZ2, hl, wl, nullptr, 0, u->dCAT[l], cat_cs(u, l)));
    // gradient of the level below's output (decoder l+1, or the bottleneck), masked
    const __nv_bfloat16* mask = l + 1 < kLevels - 1 ? u->D[l + 1] : u->CAT[kLevels - 1];
    KernelTimer kt(ctx, "unet_up_back", st);
    unet_up_back_mask<<<grid_for(lvl_pix(n, h, w, l + 1) * cb / 8), 256, 0, st>>>(
        u->dCAT[l], cat_cs(u, l), c, cb, hl / 2, wl / 2, n, mask, cb, u->dZ1, cb);
    OH_LAUNCH_CHECK();
  }
  // encoder, bottleneck first: dZ1 holds the gradient of enc{l}b's pre-activation
  for (int l = kLevels - 1; l >= 0; --l) {
    const int hl = h >> l, wl = w >> l, c = u->chans[l];
    const Layer& La = u->layers[2 * l];
    const Layer& Lb = u->layers[2 * l + 1];
    if (l < kLevels - 1) {
      KernelTimer kt(ctx, "unet_skip_pool_back", st);
      unet_skip_pool_back_mask<<<grid_for(lvl_pix(n, h, w, l) * c / 8), 256, 0, st>>>(
          u->dCAT[l], cat_cs(u, l), u->dP[l + 1], c, c, hl, wl, n, u->CAT[l], cat_cs(u, l), u->dZ1, c);
      OH_LAUNCH_CHECK();
    }
    OH_TRY(wgrad(Lb, u->A[l], c, u->dZ1, hl, wl));
    OH_TRY(dgrad(Lb, u->dZ1, hl, wl, u->A[l], c, u->dZ2, c));
    const void* xin = l == 0 ? (const void*)u->in0 : (const void*)u->P_[l];
    const int xin_cs = l == 0 ? kInPad : u->chans[l - 1];
    OH_TRY(wgrad(La, xin, xin_cs, u->dZ2, hl, wl));
    if (l > 0) OH_TRY(dgrad(La, u->dZ2, hl, wl, nullptr, 0, u->dP[l], u->chans[l - 1]));
  }
  return OH_OK;
}

oh_status unet_adam(oh_unet* u, float lr, float b1, float b2, float eps, int update, cudaStream_t st) {
  AdamHyper hp{lr, b1, b2, eps, 1.f, 1.f};
  if (update) {
    u->step += 1;
    hp.c1 = (float)(1.0 / (1.0 - std::pow((double)b1, u->step)));
    hp.c2 = (float)(1.0 / (1.0 - std::pow((double)b2, u->step)));
  }
  for (size_t i = 0; i < u->layers.size(); ++i) {
    const Layer& L = u->layers[i];
    const long long total = (long long)L.cout * L.taps * L.cin + L.cout;
    if (L.taps == 1) {
      // head: FP32 gradients [2][32] + [2] in place, no BF16 copies
      if (!update) continue;
      KernelTimer kt(u->ctx, "unet_adam", st);
      unet_adam_layer<<<1, 128, 0, st>>>(u->P + L.off_w, u->M + L.off_w, u->V + L.off_w, L.dwt, L.db, L.cout, 1, L.cin,
                                         L.cin_pad, hp, 1, 1, L.wf, nullptr);
      OH_LAUNCH_CHECK();
      continue;
    }
    KernelTimer kt(u->ctx, "unet_adam", st);
    unet_adam_layer<<<grid_for(total), 256, 0, st>>>(u->P + L.off_w, u->M + L.off_w, u->V + L.off_w, L.dwt, L.db, L.cout,
                                                     L.taps, L.cin, L.cin_pad, hp, update, 0, L.wf,
                                                     i == 0 ? nullptr : L.wd);
    OH_LAUNCH_CHECK();
  }
  return OH_OK;
}

oh_ctx* unet_ctx(const oh_unet* u) { return u ? u->ctx : nullptr; }

}  // namespace oh

using namespace oh;

extern "C" {

void oh_unet_config_default(oh_unet_config* c) {
  if (!c) return;
  std::memset(c, 0, sizeof(*c));
  c->max_batch = 1;
  c->max_height = 1024;
  c->max_width = 1024;
  c->seed = 1;
  c->out_scale = 1.f;
  for (int b = 0; b < 256; ++b) c->depth_lut[b] = b / 255.f;
}

oh_status oh_unet_create(oh_ctx* ctx, const oh_unet_config* cfg, oh_unet** out) {
  if (!ctx || !cfg || !out) return fail(OH_ERR_INVALID_ARG, "null argument");
  *out = nullptr;
  if (cfg->max_batch < 1 || cfg->max_height < 8 || cfg->max_width < 8 || cfg->max_height % 8 || cfg->max_width % 8)
    return fail(OH_ERR_INVALID_ARG, "U-Net: maximum batch >= 1 and frame sides multiples of 8");
  if (!(cfg->out_scale > 0.f)) return fail(OH_ERR_INVALID_ARG, "U-Net: out_scale must be positive");
  int prev = -1;
  cudaGetDevice(&prev);
  OH_CUDA_TRY(cudaSetDevice(ctx->device));
  oh_unet* u = new oh_unet();
  u->ctx = ctx;
  u->max_n = cfg->max_batch; u->max_h = cfg->max_height; u->max_w = cfg->max_width;
  u->out_scale = cfg->out_scale;
  // layers in parameter order
  auto add = [&](int cin, int cout, int taps) {
    Layer L{};
    L.cin = cin; L.cin_pad = (cin + 31) / 32 * 32; L.cout = cout; L.taps = taps;
    L.off_w = u->n_params; u->n_params += (size_t)cout * taps * cin;
    L.off_b = u->n_params; u->n_params += cout;
    u->layers.push_back(L);
  };
  int cprev = kInCh;
  for (int l = 0; l < kLevels; ++l) { add(cprev, u->chans[l], 9); add(u->chans[l], u->chans[l], 9); cprev = u->chans[l]; }
  for (int l = kLevels - 2; l >= 0; --l) { add(u->chans[l] + u->chans[l + 1], u->chans[l], 9); add(u->chans[l], u->chans[l], 9); }
  add(u->chans[0], kOutCh, 1);
  {
    const char* ev = std::getenv("OH_UNET_LAYER_TIMING");
    if (ev && std::atoi(ev) != 0)
      for (size_t i = 0; i < u->layers.size(); ++i)
        for (int k = 0; k < 3; ++k) u->layers[i].tn[k] = kLayerTimerNames[k][i];
  }
  oh_status rc = OH_OK;
  auto cleanup = [&]() {
    for (void* p : u->allocs) cudaFree(p);
    delete u;
    if (prev >= 0) cudaSetDevice(prev);
  };
  auto A = [&](size_t bytes, void** p) { if (rc == OH_OK) rc = dev_alloc(u, bytes, p); };
  void* p = nullptr;
  A(u->n_params * 4, &p); u->P = (float*)p;
  A(u->n_params * 4, &p); u->M = (float*)p;
  A(u->n_params * 4, &p); u->V = (float*)p;
  // gradient arena and BF16 copies
  size_t gf = 0, wb = 0;
  for (Layer& L : u->layers) { gf += (size_t)L.taps * L.cin_pad * L.cout + L.cout; wb += 2 * (size_t)L.taps * L.cin_pad * L.cout; }
  u->g_floats = gf;
  A(gf * 4, &p); u->G = (float*)p;
  A(wb * 2, &p); u->wbuf = (__nv_bfloat16*)p;
  A(256 * 4, &p); u->lut = (float*)p;
  A(256, &p); u->loss = (float*)p;
  if (rc != OH_OK) { cleanup(); return rc; }
  {
    float* g = u->G;
    __nv_bfloat16* wbp = u->wbuf;
    for (Layer& L : u->layers) {
      const size_t nk = (size_t)L.taps * L.cin_pad * L.cout;
      L.dwt = g; g += nk;
      L.db = g; g += L.cout;
      L.wf = wbp; wbp += nk;
      L.wd = wbp; wbp += nk;
    }
    // the head's gradient is [2][32] + [2] contiguous (the head kernel's layout)
    Layer& Hd = u->layers.back();
    Hd.db = Hd.dwt + (size_t)kOutCh * u->chans[0];
  }
  // activations
  const int n = u->max_n, h = u->max_h, w = u->max_w;
  A((size_t)lvl_pix(n, h, w, 0) * kInPad * 2, &p); u->in0 = (__nv_bfloat16*)p;
  size_t dz_max = 0;
  for (int l = 0; l < kLevels; ++l) {
    const size_t np = (size_t)lvl_pix(n, h, w, l), c = u->chans[l];
    A(np * c * 2, &p); u->A[l] = (__nv_bfloat16*)p;
    A(np * cat_cs(u, l) * 2, &p); u->CAT[l] = (__nv_bfloat16*)p;
    if (l > 0) {
      A(np * u->chans[l - 1] * 2, &p); u->P_[l] = (__nv_bfloat16*)p;
      A(np * u->chans[l - 1] * 2, &p); u->dP[l] = (__nv_bfloat16*)p;
    }
    if (l < kLevels - 1) {
      A(np * c * 2, &p); u->DA[l] = (__nv_bfloat16*)p;
      A(np * c * 2, &p); u->D[l] = (__nv_bfloat16*)p;
      A(np * cat_cs(u, l) * 2, &p); u->dCAT[l] = (__nv_bfloat16*)p;
    }
    dz_max = std::max(dz_max, np * c * 2);
  }
  A(dz_max, &p); u->dZ1 = (__nv_bfloat16*)p;
  A(dz_max, &p); u->dZ2 = (__nv_bfloat16*)p;
  if (rc != OH_OK) { cleanup(); return rc; }
  // initial parameters, BF16 copies, depth table
  std::vector<float> host;
  init_params(u, cfg->seed, host);
  cudaError_t e = cudaMemcpy(u->P, host.data(), host.size() * 4, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(u->M, 0, u->n_params * 4);
  if (e == cudaSuccess) e = cudaMemset(u->V, 0, u->n_params * 4);
  if (e == cudaSuccess) e = cudaMemset(u->G, 0, u->g_floats * 4);
  if (e == cudaSuccess) e = cudaMemset(u->wbuf, 0, wb * 2);
  if (e == cudaSuccess) e = cudaMemcpy(u->lut, cfg->depth_lut, 256 * 4, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) { rc = cuda_fail(e, "U-Net initialisation"); cleanup(); return rc; }
  rc = unet_adam(u, 0.f, 0.9f, 0.999f, 1e-8f, 0, nullptr);     // BF16 copies of the initial weights
  if (rc == OH_OK) { e = cudaDeviceSynchronize(); if (e != cudaSuccess) rc = cuda_fail(e, "U-Net initialisation"); }
  if (rc != OH_OK) { cleanup(); return rc; }
  if (prev >= 0) cudaSetDevice(prev);
  *out = u;
  return OH_OK;
}

oh_status oh_unet_destroy(oh_unet* u) {
  if (!u) return OH_OK;
  int prev = -1;
  cudaGetDevice(&prev);
  cudaSetDevice(u->ctx->device);
  cudaDeviceSynchronize();
  for (void* p : u->allocs) cudaFree(p);
  if (prev >= 0) cudaSetDevice(prev);
  delete u;
  return OH_OK;
}

size_t oh_unet_param_count(const oh_unet* u) { return u ? u->n_params : 0; }

oh_status oh_unet_get_params(oh_unet* u, float* host) {
  if (!u || !host) return fail(OH_ERR_INVALID_ARG, "null argument");
  CallScope cs(u->ctx, nullptr);
  OH_TRY(cs.status());
  OH_CUDA_TRY(cudaDeviceSynchronize());
  OH_CUDA_TRY(cudaMemcpy(host, u->P, u->n_params * 4, cudaMemcpyDeviceToHost));
  return OH_OK;
}

oh_status oh_unet_set_params(oh_unet* u, const float* host) {
  if (!u || !host) return fail(OH_ERR_INVALID_ARG, "null argument");
  CallScope cs(u->ctx, nullptr);
  OH_TRY(cs.status());
  OH_CUDA_TRY(cudaDeviceSynchronize());
  OH_CUDA_TRY(cudaMemcpy(u->P, host, u->n_params * 4, cudaMemcpyHostToDevice));
  OH_CUDA_TRY(cudaMemset(u->M, 0, u->n_params * 4));
  OH_CUDA_TRY(cudaMemset(u->V, 0, u->n_params * 4));
  u->step = 0;
  OH_TRY(unet_adam(u, 0.f, 0.9f, 0.999f, 1e-8f, 0, nullptr));
  OH_CUDA_TRY(cudaDeviceSynchronize());
  return OH_OK;
}

oh_status oh_unet_get_grads(oh_unet* u, float* host) {
  if (!u || !host) return fail(OH_ERR_INVALID_ARG, "null argument");
  CallScope cs(u->ctx, nullptr);
  OH_TRY(cs.status());
  OH_CUDA_TRY(cudaDeviceSynchronize());
  std::vector<float> g(u->g_floats);
  OH_CUDA_TRY(cudaMemcpy(g.data(), u->G, u->g_floats * 4, cudaMemcpyDeviceToHost));
  size_t go = 0;
  for (const Layer& L : u->layers) {
    const size_t nk = (size_t)L.taps * L.cin_pad * L.cout;
    const float* dwt = g.data() + go;
    const float* db = dwt + (L.taps == 1 ? (size_t)L.cout * L.cin : nk);
    for (int co = 0; co < L.cout; ++co)
      for (int t = 0; t < L.taps; ++t)
        for (int ci = 0; ci < L.cin; ++ci) {
          const size_t dst = L.off_w + ((size_t)co * L.taps + t) * L.cin + ci;
          // the head's gradient is [cout][cin]; the convolutions' dW^T[t*cin_pad + ci][co]
          host[dst] = L.taps == 1 ? dwt[(size_t)co * L.cin + ci] : dwt[((size_t)t * L.cin_pad + ci) * L.cout + co];
        }
    for (int co = 0; co < L.cout; ++co) host[L.off_b + co] = db[co];
    go += nk + L.cout;
  }
  return OH_OK;
}

oh_status oh_unet_forward(oh_unet* u, const uint8_t* rgbd, int n, int h, int w, void* field_out, void* stream) {
  if (!u || !rgbd || !field_out) return fail(OH_ERR_INVALID_ARG, "null argument");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  CallScope cs(u->ctx, st);
  OH_TRY(cs.status());
  OH_TRY(tc_arch_check());
  OH_TRY(unet_validate_size(u, n, h, w));
  return unet_forward(u, rgbd, n, h, w, static_cast<float2*>(field_out), st);
}

oh_status oh_unet_compute_grads(oh_unet* u, const uint8_t* rgbd, const void* target, int n, int h, int w,
                                float* loss_out, void* stream) {
  if (!u || !rgbd || !target) return fail(OH_ERR_INVALID_ARG, "null argument");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  CallScope cs(u->ctx, st);
  OH_TRY(cs.status());
  OH_TRY(tc_arch_check());
  OH_TRY(unet_validate_size(u, n, h, w));
  OH_TRY(unet_forward(u, rgbd, n, h, w, nullptr, st));
  OH_TRY(unet_backward(u, static_cast<const float2*>(target), n, h, w, st));
  if (loss_out) OH_CUDA_TRY(cudaMemcpyAsync(loss_out, u->loss, sizeof(float), cudaMemcpyDeviceToDevice, st));
  return OH_OK;
}

oh_status oh_unet_adam_step(oh_unet* u, float lr, float beta1, float beta2, float eps, void* stream) {
  if (!u) return fail(OH_ERR_INVALID_ARG, "null argument");
  if (!(lr >= 0.f) || !(beta1 >= 0.f && beta1 < 1.f) || !(beta2 >= 0.f && beta2 < 1.f) || !(eps > 0.f))
    return fail(OH_ERR_INVALID_ARG, "Adam: lr >= 0, betas in [0, 1), eps > 0");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  CallScope cs(u->ctx, st);
  OH_TRY(cs.status());
  return unet_adam(u, lr, beta1, beta2, eps, 1, st);
}

oh_status oh_unet_train_step(oh_unet* u, const uint8_t* rgbd, const void* target, int n, int h, int w, float lr,
                             float* loss_out, void* stream) {
  OH_TRY(oh_unet_compute_grads(u, rgbd, target, n, h, w, loss_out, stream));
  return oh_unet_adam_step(u, lr, 0.9f, 0.999f, 1e-8f, stream);
}

}  // extern "C"
