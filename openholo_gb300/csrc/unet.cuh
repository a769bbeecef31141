// Shared declarations of the learned surrogate: the tensor-core convolution
// launchers (unet_conv.cu) used by the U-Net (unet.cu).
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include "context.h"

namespace oh {

// Device-side arguments of conv_fwd_tc.
struct ConvArgs {
  int taps, cin, cout, w, h, n;
  int bx, by, tiles_x, tiles_y;
  int sign;                        // +1: forward, -1: input gradient (taps mirrored)
  const float* bias;               // nullable [cout]
  int relu;
  const __nv_bfloat16* mask;       // nullable: output multiplied by (mask > 0)
  int mask_cs;
  __nv_bfloat16* out;
  int out_cs;
  int* err;
  const int* stall_flag;           // error-path test hook (oh_ctx_set_test_stall), null otherwise
  long long stall_cycles;
};

// Device-side arguments of conv_wgrad_tc.
struct WgArgs {
  int taps, cin, cout, w, h, n;
  int bx, by, tiles_x, tiles_y;
  float* dwt;                      // [taps*cin][cout], accumulated
  int* err;
  const int* stall_flag;           // error-path test hook, null otherwise
  long long stall_cycles;
};

// One convolution (forward, or input gradient with sign = -1 and the
// transposed weight matrix).  Tensors are NHWC BF16 with channel strides
// x_cs / out_cs / mask_cs (elements, multiples of 8); w_mat is BF16
// [cout][taps*cin]; bias FP32 [cout] or null.
struct ConvDesc {
  int taps, sign, n, h, w, cin, cout;
  const void* x; int x_cs;
  const void* w_mat;
  const float* bias;
  int relu;
  const void* mask; int mask_cs;
  void* out; int out_cs;
};

// Weight gradient dW^T[taps*cin][cout] += X (tap-shifted) ^T dZ over all pixels.
struct WgradDesc {
  int taps, n, h, w, cin, cout;
  const void* x; int x_cs;
  const void* dz; int dz_cs;
  float* dwt;
};

oh_status tc_arch_check();
oh_status conv_enqueue(oh_ctx* ctx, const ConvDesc& d, cudaStream_t st, const char* timer_name);
oh_status wgrad_enqueue(oh_ctx* ctx, const WgradDesc& d, cudaStream_t st, const char* timer_name);

}  // namespace oh
