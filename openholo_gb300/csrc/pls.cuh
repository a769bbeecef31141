// Shared declarations of the point-light-source summation (pls.cu, pls_tc.cu).
#pragma once
#include <cstdint>
#include "context.h"

namespace oh {

struct PlsGeom {
  int nx, ny, mode, use_amp;
  double k, dpx, dpy, dox, doy, sox, soy, z, ph;
};

// Per point, FP64-prepared: x and y phases in 2^-64 turns as a n^2 + b n + g
// with n = column - mx (row - my); the y part carries ph (and k|dz| for
// Huygens).  u, v: the point in pixel units; dz: |z_k + z|; rk: Huygens
// remainder factor; (ar, ai): the amplitude applied to each term.
struct PlsPt {
  unsigned long long ax, bx, gx;
  unsigned long long ay, by, gy;
  int mx, my;
  float u, v, dz, rk;
  float ar, ai;
};

// top 32 bits of a n^2 + b n + g (mod 2^64): the phase in 2^-32 turns
__device__ __forceinline__ uint32_t pls_turns(unsigned long long a, unsigned long long b, unsigned long long g,
                                              int n) {
  const unsigned long long nn = (unsigned long long)((long long)n * (long long)n);
  const unsigned long long t = a * nn + b * (unsigned long long)(long long)n + g;
  return (uint32_t)(t >> 32);
}

// (cos, sin)(2 pi t 2^-32) with the sign folded: returns -(cos, sin) of the
// reduced angle, so callers subtract.  t is mapped to [1, 2) by its top 23
// bits, then to [-0.5, 0.5) turns (7.5e-7 rad resolution).
__device__ __forceinline__ void pls_cis_neg(uint32_t t, float* c, float* s) {
  const float f = __uint_as_float(0x3F800000u | (t >> 9)) - 1.5f;
  __sincosf(6.28318530717958647692f * f, s, c);
}

// Tensor-core engine for FRESNEL / CGH_FRESNEL (FP32 output).  Returns
// OH_ERR_UNSUPPORTED_SIZE for shapes it does not take.
oh_status pls_tensor_enqueue(oh_ctx* ctx, const PlsGeom& g, const PlsPt* pts, int n, void* out, cudaStream_t st);

}  // namespace oh
