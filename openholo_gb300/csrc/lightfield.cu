// Light field to complex field, fn_convertLightField2ComplexField.m:1-11
// (OpenHolo_LFCGH) with fn_myfft2.m (fftshift(fft2(ifftshift(.)))): the
// (s, t) view of an Nv x Nu x Nt x Ns light field, times exp(i phase) (the
// MATLAB code draws phase = 2 pi rand per sample), becomes the centred 2-D
// FFT filling block rows t Nv .. (t+1) Nv - 1, columns s Nu .. (s+1) Nu - 1
// of the Nt Nv x Ns Nu field.
//
// All views are transformed together: the pack kernel writes view b = t Ns + s
// (ifftshift applied) at columns b Nu .. of an Nv x (Nt Ns Nu) array, so one
// row-FFT launch (length Nu) and one column-FFT launch (length Nv) transform
// every view; the unpack kernel applies fftshift while placing each view's
// block.
#include <cmath>
#include "context.h"
#include "fft_kernels.cuh"

namespace oh {

namespace {

struct LFGeom { int nu, nv, ns, nt; unsigned long long seed; };

// numpy ifftshift / fftshift source indices along an axis of length n
__device__ __forceinline__ int ifs_src(int k, int n) { int j = k + n / 2; return j >= n ? j - n : j; }
__device__ __forceinline__ int fs_src(int k, int n) { int j = k + (n + 1) / 2; return j >= n ? j - n : j; }

template <typename R>
__global__ void lf_pack(LFGeom g, const float* __restrict__ lf, const float* __restrict__ phase,
                        typename cplx_of<R>::type* __restrict__ x) {
  const int B = g.ns * g.nt;
  const size_t row = (size_t)B * g.nu;
  const size_t n = row * g.nv;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int v = (int)(i / row);
    const int c = (int)(i - (size_t)v * row);
    const int b = c / g.nu, u = c - b * g.nu;
    const size_t src = ((size_t)b * g.nv + ifs_src(v, g.nv)) * g.nu + ifs_src(u, g.nu);
    const R ph = phase ? (R)phase[src] : (R)6.283185307179586476925286766559 * (R)u24_at(g.seed, src);
    R s, co;
    sincos(ph, &s, &co);
    const R a = (R)lf[src];
    x[i] = mk(a * co, a * s);
  }
}

template <typename R>
__global__ void lf_unpack(LFGeom g, const typename cplx_of<R>::type* __restrict__ x,
                          typename cplx_of<R>::type* __restrict__ field) {
  const size_t W = (size_t)g.ns * g.nu;
  const size_t n = W * g.nt * g.nv;
  const size_t row = (size_t)g.ns * g.nt * g.nu;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int r = (int)(i / W), c = (int)(i - (size_t)r * W);
    const int t = r / g.nv, v = r - t * g.nv;
    const int s = c / g.nu, u = c - s * g.nu;
    const int b = t * g.ns + s;
    field[i] = x[(size_t)fs_src(v, g.nv) * row + (size_t)b * g.nu + fs_src(u, g.nu)];
  }
}

template <typename R>
oh_status run_lightfield(oh_ctx* ctx, const LFGeom& g, const float* lf, const float* phase, void* field,
                         cudaStream_t st) {
  typedef typename cplx_of<R>::type C;
  const int prec = sizeof(R) == 8 ? 1 : 0;
  const int B = g.ns * g.nt;
  void* xp;
  OH_TRY(scratch(ctx, "lf.views", (size_t)B * g.nu * g.nv * sizeof(C), &xp));
  const int grid = oh::sm_count() * 8;
  KernelTimer kt(ctx, "lightfield", st);
  lf_pack<R><<<grid, 256, 0, st>>>(g, lf, phase, static_cast<C*>(xp));
  OH_LAUNCH_CHECK();
  OH_TRY(fft_rows_enqueue(ctx, prec, g.nu, g.nv * B, xp, xp, -1, 0, st));
  OH_TRY(fft_cols_enqueue(ctx, prec, B * g.nu, g.nv, xp, -1, 0, st));
  lf_unpack<R><<<grid, 256, 0, st>>>(g, static_cast<const C*>(xp), static_cast<C*>(field));
  OH_LAUNCH_CHECK();
  return OH_OK;
}

}  // namespace

}  // namespace oh

using namespace oh;

extern "C" oh_status oh_lightfield_to_field(oh_ctx* ctx, oh_precision prec, int nu, int nv, int ns, int nt,
                                            const float* lf, const float* phase, uint64_t seed, void* field,
                                            void* stream) {
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  CallScope cs(ctx, st);
  OH_TRY(cs.status());
  if (nu < 1 || nv < 1 || ns < 1 || nt < 1) return fail(OH_ERR_INVALID_ARG, "light-field sizes must be positive");
  if ((long long)nu * ns * nt > (1ll << 30) || (long long)nv * nu * ns * nt > (1ll << 31))
    return fail(OH_ERR_UNSUPPORTED_SIZE, "light field too large");
  if (!lf || !field) return fail(OH_ERR_INVALID_ARG, "light field and output are required");
  const LFGeom g{nu, nv, ns, nt, (unsigned long long)seed};
  if (prec == OH_FP64) return run_lightfield<double>(ctx, g, lf, phase, field, st);
  return run_lightfield<float>(ctx, g, lf, phase, field, st);
}
