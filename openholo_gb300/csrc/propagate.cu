// Free-space propagation in the forms of the reference's MATLAB tools:
//
//   OH_PROP_FRESNEL_TF      FresnelPropagation.m:1-16 (WRP_matlab_ver 1.0):
//     out = ifft2(fft2(U) .* H),  H = exp(i k z) exp(-i pi lambda z (fx^2 + fy^2))
//     on the FFT-ordered grid fx = [0 .. floor((Nx-1)/2), -ceil((Nx+1)/2)+1 .. -1] / (Nx dx).
//   OH_PROP_AS_BANDLIMITED  fn_FresnelPropagation_as.m:1-48 (OpenHolo_MeshCGH):
//     zero-pad to 2Nx x 2Ny with the field at (round(Ny/2)-1, round(Nx/2)-1)
//     (0-based), A = fftshift(fft2(ifftshift(pad))), multiply by
//     exp(i 2 pi z sqrt(1/lambda^2 - a^2 - b^2)) with a = (m + 1 - Nxx/2) / (Nxx dx)
//     (m 0-based, so the kernel's zero frequency sits one sample before the
//     spectrum's, as in the MATLAB source), zeroed where the Matsushima band
//     limit |a z / sqrt(...)| > 1 / (2 da) (or the same for b) holds;
//     fftshift(ifft2(ifftshift(.))) and crop the field window back.
//
// Both run on the shared-memory FFT engine (2-D transform = row pass +
// column-strip pass).  FP64 evaluates the transfer functions directly.
// FP32 never forms the large phases in float: the Fresnel kernel is the
// product of per-axis tables (phases reduced in FP64), and the angular-
// spectrum phase is split as
//   2 pi z sqrt(q) = 2 pi z / lambda - pi lambda z (a^2 + b^2) - 2 pi (z / lambda) g(s),
//   s = lambda^2 (a^2 + b^2),  g(s) = s^2 / (2 (1 + sqrt(1 - s))^2),
// with the first two terms tabulated per axis in FP64 and the small residual
// (a few rad at most) in FP32.  Evanescent components (q < 0) follow MATLAB's
// complex square root: kernel exp(-2 pi z sqrt(-q)).
#include <cmath>
#include "context.h"
#include "fft_kernels.cuh"

namespace oh {

namespace {

// MATLAB FFT-order frequency index of bin j of n
__host__ __device__ inline int fft_order_index(int j, int n) { return j <= (n - 1) / 2 ? j : j - n; }

__device__ __forceinline__ double2 cis_turns(double t) {
  t -= rint(t);
  double s, c;
  sincospi(2.0 * t, &s, &c);
  return make_double2(c, s);
}

// Per-axis tables (FP64): TF form hx[j] = exp(-i pi lambda z fx_j^2);
// AS form ax[m] = exp(-i pi lambda z a_m^2) and a_m itself.
struct PropAxis { int n; double df; };

__global__ void prop_axis_tables(int method, PropAxis X, PropAxis Y, double lambda, double z, double fold_t,
                                 double2* __restrict__ tx, double2* __restrict__ ty,
                                 double* __restrict__ fxv, double* __restrict__ fyv) {
  const int tot = X.n + Y.n;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < tot; e += gridDim.x * blockDim.x) {
    const bool isx = e < X.n;
    const PropAxis A = isx ? X : Y;
    const int m = isx ? e : e - X.n;
    const double f = method == OH_PROP_FRESNEL_TF ? fft_order_index(m, A.n) * A.df
                                                  : (double)(m + 1 - A.n / 2) * A.df;
    // exp(-i pi lambda z f^2); the x table also carries the constant phase fold_t (turns)
    const double2 v = cis_turns(-0.5 * lambda * z * f * f + (isx ? fold_t : 0.0));
    if (isx) { tx[m] = v; fxv[m] = f; }
    else { ty[m] = v; fyv[m] = f; }
  }
}

template <typename R>
__global__ void prop_tf_multiply(int nx, int ny, const double2* __restrict__ tx, const double2* __restrict__ ty,
                                 double cre, double cim, typename cplx_of<R>::type* __restrict__ u) {
  const size_t n = (size_t)nx * ny;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int r = (int)(i / nx), c = (int)(i - (size_t)r * nx);
    if constexpr (sizeof(R) == 8) {
      const double2 a = tx[c], b = ty[r];
      const double hr = a.x * b.x - a.y * b.y, hi = a.x * b.y + a.y * b.x;
      const double kr = cre * hr - cim * hi, ki = cre * hi + cim * hr;
      const double ur = u[i].x, ui = u[i].y;
      u[i].x = ur * kr - ui * ki;
      u[i].y = ur * ki + ui * kr;
    } else {
      // tx carries exp(i k z) (folded in by the table kernel)
      const float2 a = make_float2((float)tx[c].x, (float)tx[c].y), b = make_float2((float)ty[r].x, (float)ty[r].y);
      u[i] = cmul(u[i], cmul(a, b));
    }
  }
}

struct ASGeom {
  int NX, NY;
  double lambda, z, dal, dbl;
};

// Band-limited angular-spectrum kernel at spatial frequencies (a, b); ta, tb
// are the per-axis tables exp(-i pi lambda z a^2) (ta also carries exp(2 pi i z / lambda)).
template <typename R>
__device__ __forceinline__ void as_kernel(const ASGeom& g, R a, R b, const double2& ta, const double2& tb,
                                          R* kr, R* ki) {
  const R il = (R)(1.0 / g.lambda), zz = (R)g.z;
  const R q = il * il - a * a - b * b;
  const R aq = sqrt(fabs(q));
  // Matsushima limits (the MATLAB source's abs(-a z / sqrt(q)) > 1 / (2 da))
  const R la = fabs(a * zz) / aq, lb = fabs(b * zz) / aq;
  if (!(la <= (R)(0.5 / g.dal)) || !(lb <= (R)(0.5 / g.dbl))) { *kr = 0; *ki = 0; return; }
  if (q < (R)0) {                         // evanescent: exp(-2 pi z sqrt(-q))
    *kr = exp((R)(-2.0 * M_PI) * zz * aq);
    *ki = 0;
    return;
  }
  if constexpr (sizeof(R) == 8) {
    double s, c;
    const double t = g.z * aq;            // turns
    sincospi(2.0 * (t - rint(t)), &s, &c);
    *kr = c; *ki = s;
  } else {
    // carrier and paraxial part from the FP64 tables, non-paraxial residual in FP32
    const float2 h = cmul(make_float2((float)ta.x, (float)ta.y), make_float2((float)tb.x, (float)tb.y));
    const float sv = (float)(g.lambda * g.lambda) * (a * a + b * b);
    const float den = 1.f + sqrtf(1.f - sv);
    const float res = -(float)(g.z / g.lambda) * sv * sv / (2.f * den * den);   // turns
    float sn, cs;
    sincospif(2.f * res, &sn, &cs);
    *kr = h.x * cs - h.y * sn;
    *ki = h.x * sn + h.y * cs;
  }
}

template <typename R>
__global__ void prop_as_multiply(ASGeom g, const double2* __restrict__ ta, const double2* __restrict__ tb,
                                 const double* __restrict__ av, const double* __restrict__ bv,
                                 typename cplx_of<R>::type* __restrict__ u) {
  const size_t n = (size_t)g.NX * g.NY;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int r = (int)(i / g.NX), c = (int)(i - (size_t)r * g.NX);
    R kr, ki;
    as_kernel<R>(g, (R)av[c], (R)bv[r], ta[c], tb[r], &kr, &ki);
    const R ur = u[i].x, ui = u[i].y;
    u[i].x = ur * kr - ui * ki;
    u[i].y = ur * ki + ui * kr;
  }
}

template <typename R>
__global__ void prop_pad(int nx, int ny, int sx, int sy, const typename cplx_of<R>::type* __restrict__ in,
                         typename cplx_of<R>::type* __restrict__ out) {
  const int NX = 2 * nx, NY = 2 * ny;
  const size_t n = (size_t)NX * NY;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int r = (int)(i / NX) - sy, c = (int)(i % NX) - sx;
    typename cplx_of<R>::type v = mk((R)0, (R)0);
    if (r >= 0 && r < ny && c >= 0 && c < nx) v = in[(size_t)r * nx + c];
    out[i] = v;
  }
}

template <typename R>
__global__ void prop_crop(int nx, int ny, int sx, int sy, const typename cplx_of<R>::type* __restrict__ in,
                          typename cplx_of<R>::type* __restrict__ out) {
  const size_t n = (size_t)nx * ny;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int r = (int)(i / nx), c = (int)(i % nx);
    out[i] = in[(size_t)(r + sy) * (2 * nx) + c + sx];
  }
}

// MATLAB round(x / 2) - 1 for positive integers (halves away from zero)
inline int matlab_start(int n) { return (n + 1) / 2 - 1; }

template <typename R>
oh_status run_propagate(oh_ctx* ctx, int method, int nx, int ny, double dx, double dy, double z, double lambda,
                        void* field, cudaStream_t st) {
  typedef typename cplx_of<R>::type C;
  const int prec = sizeof(R) == 8 ? 1 : 0;
  const bool as = method == OH_PROP_AS_BANDLIMITED;
  const int NX = as ? 2 * nx : nx, NY = as ? 2 * ny : ny;
  void* tp;
  OH_TRY(scratch(ctx, "prop.tab", (size_t)(NX + NY) * (sizeof(double2) + sizeof(double)), &tp));
  double2* tx = static_cast<double2*>(tp);
  double2* ty = tx + NX;
  double* fxv = reinterpret_cast<double*>(ty + NY);
  double* fyv = fxv + NX;
  const PropAxis X{NX, 1.0 / (NX * dx)}, Y{NY, 1.0 / (NY * dy)};
  const int grid = oh::sm_count() * 8;
  const double zt = z / lambda;                 // exp(i k z) = exp(2 pi i z / lambda)
  const double carrier = zt - std::rint(zt);
  {
    // FP32 folds the constant phase into the x table; FP64 applies it separately (TF) or
    // evaluates the whole phase per sample (AS)
    KernelTimer kt(ctx, "prop_tables", st);
    prop_axis_tables<<<(NX + NY + 255) / 256, 256, 0, st>>>(method, X, Y, lambda, z, prec ? 0.0 : carrier, tx, ty,
                                                             fxv, fyv);
    OH_LAUNCH_CHECK();
  }
  if (!as) {
    OH_TRY(fft2d_enqueue(ctx, prec, nx, ny, field, field, nullptr, -1, 0, 0, st));
    const double cre = std::cos(2.0 * M_PI * carrier), cim = std::sin(2.0 * M_PI * carrier);
    {
      KernelTimer kt(ctx, "prop_tf_multiply", st);
      prop_tf_multiply<R><<<grid, 256, 0, st>>>(nx, ny, tx, ty, cre, cim, static_cast<C*>(field));
      OH_LAUNCH_CHECK();
    }
    return fft2d_enqueue(ctx, prec, nx, ny, field, field, nullptr, 1, 0, 1, st);
  }
  void* pp;
  OH_TRY(scratch(ctx, "prop.pad", (size_t)NX * NY * sizeof(C), &pp));
  const int sx = matlab_start(nx), sy = matlab_start(ny);
  {
    KernelTimer kt(ctx, "prop_pad", st);
    prop_pad<R><<<grid, 256, 0, st>>>(nx, ny, sx, sy, static_cast<const C*>(field), static_cast<C*>(pp));
    OH_LAUNCH_CHECK();
  }
  OH_TRY(fft2d_enqueue(ctx, prec, NX, NY, pp, pp, nullptr, -1, 1, 0, st));
  ASGeom g;
  g.NX = NX; g.NY = NY; g.lambda = lambda; g.z = z; g.dal = X.df; g.dbl = Y.df;
  {
    KernelTimer kt(ctx, "prop_as_multiply", st);
    prop_as_multiply<R><<<grid, 256, 0, st>>>(g, tx, ty, fxv, fyv, static_cast<C*>(pp));
    OH_LAUNCH_CHECK();
  }
  OH_TRY(fft2d_enqueue(ctx, prec, NX, NY, pp, pp, nullptr, 1, 1, 1, st));
  KernelTimer kt(ctx, "prop_crop", st);
  prop_crop<R><<<grid, 256, 0, st>>>(nx, ny, sx, sy, static_cast<const C*>(pp), static_cast<C*>(field));
  OH_LAUNCH_CHECK();
  return OH_OK;
}

}  // namespace

}  // namespace oh

using namespace oh;

extern "C" oh_status oh_propagate(oh_ctx* ctx, oh_precision prec, int method, int nx, int ny, double dx, double dy,
                                  double z, double lambda, void* field, void* stream) {
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  CallScope cs(ctx, st);
  OH_TRY(cs.status());
  if (method != OH_PROP_FRESNEL_TF && method != OH_PROP_AS_BANDLIMITED)
    return fail(OH_ERR_INVALID_ARG, "unknown propagation method");
  if (nx < 1 || ny < 1 || !field || !(dx > 0) || !(dy > 0) || !(lambda > 0))
    return fail(OH_ERR_INVALID_ARG, "bad propagation arguments");
  if (prec == OH_FP64) return run_propagate<double>(ctx, method, nx, ny, dx, dy, z, lambda, field, st);
  return run_propagate<float>(ctx, method, nx, ny, dx, dy, z, lambda, field, st);
}
