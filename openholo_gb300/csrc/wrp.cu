// Wavefront-recording-plane (WRP) accumulation and Fresnel-convolution
// propagation.
//
// OPHWRP::SingleWRP (OpenHolo_WRP/openwrp_console_ver 1.0/openwrp/WRP.cpp:75-140):
//   per point: dz = z_wrp - z_k, w = int(|lambda dz / dp^2 / 2 + 0.5|)*2 - 1,
//   tx = int(x/dp) + Nx/2, ty = int(y/dp) + Ny/2, and for wx, wy in [-w, w):
//   r = sign(dz) sqrt((wx dp)^2 + (wy dp)^2 + dz^2),
//   WRP[ty+wy][tx+wx] += (cos, sin)(k r) / (r + 0.05)   (pixels inside the plane)
// The reference adds with a racy AddPixel (cwo.cpp:4298-4308); here every
// contribution is an atomic float2/double2 add.  FP32 mode evaluates k r as
// k dz (reduced mod 2 pi in double, once per point) + k rho^2/(|r| + |dz|)
// (at most tens of rad, exact in float to ~1e-5 rad).
//
// CWO::Diffract(z, CWO_FRESNEL_CONV) (cwo.cpp:2198-2279, DiffractConv
// FRESNEL_CONV cwo.cpp:2872-2898): zero-pad the Nx x Ny field into a
// 2Nx x 2Ny grid at offset (Nx/2, Ny/2), FFT, multiply by the FFT of the
// sampled Fresnel impulse response, inverse FFT with 1/(2Nx 2Ny), crop the
// centre back.  The impulse response is written from the mathematics
//   h(x,y) = exp(i k z)/(i lambda z) exp(i pi (x^2+y^2)/(lambda z)) dp^2
// (the DLL's kernel/coefficient bodies are not in the tree), sampled with
// its origin at index (0,0) so that the convolution output is aligned with
// the input; its spectrum is cached per (size, pitch, lambda, z).
#include <cmath>
#include <cstring>
#include "context.h"
#include "fft_kernels.cuh"

namespace oh {

struct WRPGeom { int nx, ny; double dp, lambda, z; int fixed_w; };

template <typename R>
__global__ void __launch_bounds__(256) wrp_accumulate_kernel(WRPGeom g, const double* __restrict__ xyz, int n,
                                                            typename cplx_of<R>::type* __restrict__ wrp) {
  typedef typename cplx_of<R>::type C;
  const double two_pi = 6.283185307179586476925286766559;
  const float wl = (float)g.lambda, dpx = (float)g.dp;
  const double kd = (double)(float)(2.0 * M_PI / g.lambda);   // GetWaveNum() as float (WRP.cpp:78)
  for (int k = blockIdx.x; k < n; k += gridDim.x) {
    const double px = xyz[3 * k], py = xyz[3 * k + 1], pz = xyz[3 * k + 2];
    const float dzf = (float)((double)(float)g.z - pz);
    int w;
    if (g.fixed_w > 0) w = g.fixed_w;
    else { float tw = (float)(int)fabsf(wl * dzf / dpx / dpx / 2 + 0.5f) * 2 - 1; w = (int)tw; }
    if (w <= 0) continue;
    const int tx = (int)(px / (double)dpx) + (g.nx >> 1);
    const int ty = (int)(py / (double)dpx) + (g.ny >> 1);
    const double dz = (double)(float)g.z - pz;
    const double sgn = dz > 0.0 ? 1.0 : -1.0;
    // k*dz reduced once per point
    const double kdz = kd * fabs(dz);
    const R base = (R)(kdz - two_pi * rint(kdz / two_pi));
    const int side = 2 * w;
    const int total = side * side;
    for (int i = threadIdx.x; i < total; i += blockDim.x) {
      const int wy = i / side - w, wx = i % side - w;
      const int X = tx + wx, Y = ty + wy;
      if (X < 0 || X >= g.nx || Y < 0 || Y >= g.ny) continue;
      C v;
      if constexpr (sizeof(R) == 4) {
        const float ddx = (float)wx * dpx, ddy = (float)wy * dpx;
        const float rho2 = ddx * ddx + ddy * ddy;
        const float adz = (float)fabs(dz);
        const float ar = sqrtf(rho2 + adz * adz);
        const float extra = (float)kd * rho2 / (ar + adz);      // k (|r| - |dz|)
        float ph = base + extra;
        ph = sgn > 0 ? ph : -ph;
        float sn, cs;
        sincosf(ph, &sn, &cs);
        const float inv = 1.f / ((float)sgn * ar + 0.05f);
        v = mk(cs * inv, sn * inv);
      } else {
        const double ddx = wx * (double)dpx, ddy = wy * (double)dpx;
        const double r = sgn * sqrt(ddx * ddx + ddy * ddy + dz * dz);
        double sn, cs;
        sincos(kd * r, &sn, &cs);
        v = mk(cs / (r + 0.05), sn / (r + 0.05));
      }
      C* dst = wrp + (size_t)Y * g.nx + X;
      atomicAdd(&dst->x, v.x);
      atomicAdd(&dst->y, v.y);
    }
  }
}

template <typename R>
__global__ void fresnel_pad(int nx, int ny, const typename cplx_of<R>::type* __restrict__ in,
                            typename cplx_of<R>::type* __restrict__ out) {
  const int NX = 2 * nx, NY = 2 * ny, ox = nx / 2, oy = ny / 2;
  const size_t n = (size_t)NX * NY;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int r = (int)(i / NX), c = (int)(i - (size_t)r * NX);
    const int rr = r - oy, cc = c - ox;
    typename cplx_of<R>::type v = mk((R)0, (R)0);
    if (rr >= 0 && rr < ny && cc >= 0 && cc < nx) v = in[(size_t)rr * nx + cc];
    out[i] = v;
  }
}

// Sampled impulse response with origin at index 0 (wrap-around coordinates).
template <typename R>
__global__ void fresnel_kernel_sample(int NX, int NY, double dp, double lambda, double z, typename cplx_of<R>::type* b) {
  const double two_pi = 6.283185307179586476925286766559;
  const double k = two_pi / lambda;
  const size_t n = (size_t)NX * NY;
  // exp(i k z) / (i lambda z) * dp^2
  const double kz = k * z - two_pi * rint(k * z / two_pi);
  double s0, c0;
  sincos(kz, &s0, &c0);
  const double amp = dp * dp / (lambda * z);
  // 1/i = -i
  const double cre = amp * s0, cim = -amp * c0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int r = (int)(i / NX), c = (int)(i - (size_t)r * NX);
    const int jx = c < NX / 2 ? c : c - NX, jy = r < NY / 2 ? r : r - NY;
    const double x = jx * dp, y = jy * dp;
    double ph = M_PI * (x * x + y * y) / (lambda * z);
    ph -= two_pi * rint(ph / two_pi);
    double s, co;
    sincos(ph, &s, &co);
    b[i] = mk((R)(cre * co - cim * s), (R)(cre * s + cim * co));
  }
}

template <typename R>
__global__ void cmul_inplace(size_t n, typename cplx_of<R>::type* a, const typename cplx_of<R>::type* b) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) a[i] = cmul(a[i], b[i]);
}

template <typename R>
__global__ void fresnel_crop(int nx, int ny, const typename cplx_of<R>::type* __restrict__ in, typename cplx_of<R>::type* __restrict__ out) {
  const int NX = 2 * nx, ox = nx / 2, oy = ny / 2;
  const size_t n = (size_t)nx * ny;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int r = (int)(i / nx), c = (int)(i - (size_t)r * nx);
    out[i] = in[(size_t)(r + oy) * NX + c + ox];
  }
}

template <typename R>
static oh_status run_fresnel(oh_ctx* ctx, int nx, int ny, double dp, double lambda, double z, void* field, cudaStream_t st) {
  typedef typename cplx_of<R>::type C;
  const int prec = sizeof(R) == 8 ? 1 : 0;
  const int NX = 2 * nx, NY = 2 * ny;
  const size_t n2 = (size_t)NX * NY;
  void* pa;
  void* pb;
  OH_TRY(scratch(ctx, "fr.a", n2 * sizeof(C), &pa));
  // one cached transfer-function spectrum per context, keyed by its parameters
  char key[160];
  std::snprintf(key, sizeof(key), "%d:%d:%d:%.17g:%.17g:%.17g", prec, NX, NY, dp, lambda, z);
  void* prev_b = nullptr;
  {
    auto it = ctx->scratch.find("fr.B");
    if (it != ctx->scratch.end()) prev_b = it->second.p;
  }
  OH_TRY(scratch(ctx, "fr.B", n2 * sizeof(C), &pb));
  const bool have = prev_b == pb && ctx->fresnel_key == key;
  ctx->fresnel_key = key;
  const int grid = 152 * 8;
  if (!have) {
    fresnel_kernel_sample<R><<<grid, 256, 0, st>>>(NX, NY, dp, lambda, z, (C*)pb);
    OH_LAUNCH_CHECK();
    OH_TRY(fft2d_enqueue(ctx, prec, NX, NY, pb, pb, nullptr, -1, 0, 0, st));
  }
  {
    KernelTimer kt(ctx, "fresnel_pad", st);
    fresnel_pad<R><<<grid, 256, 0, st>>>(nx, ny, (const C*)field, (C*)pa);
    OH_LAUNCH_CHECK();
  }
  OH_TRY(fft2d_enqueue(ctx, prec, NX, NY, pa, pa, nullptr, -1, 0, 0, st));
  {
    KernelTimer kt(ctx, "fresnel_mul", st);
    cmul_inplace<R><<<grid, 256, 0, st>>>(n2, (C*)pa, (const C*)pb);
    OH_LAUNCH_CHECK();
  }
  OH_TRY(fft2d_enqueue(ctx, prec, NX, NY, pa, pa, nullptr, 1, 0, 1, st));
  {
    KernelTimer kt(ctx, "fresnel_crop", st);
    fresnel_crop<R><<<grid, 256, 0, st>>>(nx, ny, (const C*)pa, (C*)field);
    OH_LAUNCH_CHECK();
  }
  return OH_OK;
}

}  // namespace oh

using namespace oh;

extern "C" {

oh_status oh_wrp_accumulate(oh_ctx* ctx, oh_precision prec, const oh_wrp_params* p, const double* xyz, int n_points,
                            void* wrp, void* stream) {
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  CallScope cs(ctx, st);
  OH_TRY(cs.status());
  if (!p || p->nx < 1 || p->ny < 1 || !(p->pitch > 0) || !(p->lambda > 0) || p->window < 0)
    return fail(OH_ERR_INVALID_ARG, "bad WRP parameters");
  if (n_points < 0 || (n_points > 0 && !xyz) || !wrp) return fail(OH_ERR_INVALID_ARG, "bad WRP buffers");
  if (n_points == 0) return OH_OK;
  WRPGeom g{p->nx, p->ny, p->pitch, p->lambda, p->z_wrp, p->window};
  const int grid = std::min(n_points, 152 * 32);
  KernelTimer kt(ctx, "wrp_accumulate", st);
  if (prec == OH_FP64) wrp_accumulate_kernel<double><<<grid, 256, 0, st>>>(g, xyz, n_points, (double2*)wrp);
  else wrp_accumulate_kernel<float><<<grid, 256, 0, st>>>(g, xyz, n_points, (float2*)wrp);
  OH_LAUNCH_CHECK();
  return OH_OK;
}

oh_status oh_fresnel_propagate(oh_ctx* ctx, oh_precision prec, int nx, int ny, double pitch, double lambda, double z,
                               void* field, void* stream) {
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  CallScope cs(ctx, st);
  OH_TRY(cs.status());
  if (nx < 1 || ny < 1 || !field || !(pitch > 0) || !(lambda > 0) || z == 0.0)
    return fail(OH_ERR_INVALID_ARG, "bad Fresnel propagation arguments");
  if (prec == OH_FP64) return run_fresnel<double>(ctx, nx, ny, pitch, lambda, z, field, st);
  return run_fresnel<float>(ctx, nx, ny, pitch, lambda, z, field, st);
}

}  // extern "C"
