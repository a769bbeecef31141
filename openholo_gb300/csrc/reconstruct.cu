// Eye-model reconstruction of a fringe, HologramGenerator::ReconstructImage
// (OpenHolo_DepthMap/Hologram/src/HologramGenerator_CPU.cpp:414-614), one frame:
//
//   Test_Propagation_to_Eye_Pupil (:486-538): H = S F S (fringe) * exp(i pi (xe^2 + ye^2) / (lambda f))
//     on the eye-pupil grid pp_e = lambda f / (pn pp), xe = -E/2 + pp_e x, ye = (E/2 - pp_e) - pp_e y;
//   Reconstruction (:543-614): circular shift by (-round(cx / pp_ex), round(cy / pp_ey)),
//     times exp(i pi (xe^2 + ye^2) / (lambda f_eff)), the eye-lens anti-aliasing mask
//     r < |lambda f_eff / (2 max(pp_ex, pp_ey))| and the pupil mask r < D/2, then S F S again
//     and the magnitude (the retina-plane phase factor does not change it);
//   f_eye = L (f - d) / (L + (f - d)), f_eff = f_eye L / (f_eye - L), L = eye length, d = focus distance.
//
// S is the reference's CPU fftShift, out[(i - n/2) mod n] = in[i] per axis
// (the inverse of numpy's fftshift for odd n, equal for even n); F is the
// unnormalised forward FFT.  The pixel counts and pitches are divided by
// test_pixel_number_scale, and the fringe is read as the first pnx' pny'
// values in row-major order (the reference indexes its full-size buffer that
// way).  The two lens phases reach ~1e4 rad, so they are per-axis tables with
// FP64-reduced phases; the masks are evaluated in FP64.
#include <cmath>
#include "context.h"
#include "fft_kernels.cuh"

namespace oh {

namespace {

struct EyeGrid { int nx, ny; double ppx_e, ppy_e, Ex, Ey; };

__device__ __forceinline__ double2 cis_tn(double t) {
  t -= rint(t);
  double s, c;
  sincospi(2.0 * t, &s, &c);
  return make_double2(c, s);
}

__device__ __forceinline__ double eye_xe(const EyeGrid& g, int x) { return -g.Ex / 2.0 + g.ppx_e * x; }
__device__ __forceinline__ double eye_ye(const EyeGrid& g, int y) { return (g.Ey / 2.0 - g.ppy_e) - g.ppy_e * y; }

// per axis: exp(i pi v^2 / (lambda f)) and exp(i pi v^2 / (lambda f_eff)), v = xe or ye
__global__ void eye_tables(EyeGrid g, double lambda, double f, double feff, double2* __restrict__ t1x,
                           double2* __restrict__ t1y, double2* __restrict__ t2x, double2* __restrict__ t2y) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < g.nx + g.ny; e += gridDim.x * blockDim.x) {
    const bool isx = e < g.nx;
    const int m = isx ? e : e - g.nx;
    const double v = isx ? eye_xe(g, m) : eye_ye(g, m);
    const double a = v * v / (2.0 * lambda * f), b = v * v / (2.0 * lambda * feff);   // turns
    if (isx) { t1x[m] = cis_tn(a); t2x[m] = cis_tn(b); }
    else { t1y[m] = cis_tn(a); t2y[m] = cis_tn(b); }
  }
}

// S: out[k] = in[(k + n/2) mod n] per axis
__device__ __forceinline__ int s_src(int k, int n) { int j = k + n / 2; return j >= n ? j - n : j; }

template <typename R>
__global__ void eye_pack(int nx, int ny, const R* __restrict__ fringe, typename cplx_of<R>::type* __restrict__ buf) {
  const size_t n = (size_t)nx * ny;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int y = (int)(i / nx), x = (int)(i - (size_t)y * nx);
    buf[i] = mk(fringe[(size_t)s_src(y, ny) * nx + s_src(x, nx)], (R)0);
  }
}

template <typename R>
__device__ __forceinline__ typename cplx_of<R>::type cmul_d(typename cplx_of<R>::type u, double2 a, double2 b) {
  const double hr = a.x * b.x - a.y * b.y, hi = a.x * b.y + a.y * b.x;
  if constexpr (sizeof(R) == 8) {
    return mk(u.x * hr - u.y * hi, u.x * hi + u.y * hr);
  } else {
    const float fr = (float)hr, fi = (float)hi;
    return mk(u.x * fr - u.y * fi, u.x * fi + u.y * fr);
  }
}

// H[k] = S(F)[k] * lens(k)
template <typename R>
__global__ void eye_lens(EyeGrid g, const typename cplx_of<R>::type* __restrict__ spec, const double2* __restrict__ t1x,
                         const double2* __restrict__ t1y, typename cplx_of<R>::type* __restrict__ h) {
  const size_t n = (size_t)g.nx * g.ny;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int y = (int)(i / g.nx), x = (int)(i - (size_t)y * g.nx);
    h[i] = cmul_d<R>(spec[(size_t)s_src(y, g.ny) * g.nx + s_src(x, g.nx)], t1x[x], t1y[y]);
  }
}

// buf[k] = B[S(k)], B[p] = H[(p - shift) mod n] * eye lens(p) * masks(p)
template <typename R>
__global__ void eye_pupil(EyeGrid g, int shx, int shy, double r_alias, double r_pupil,
                          const typename cplx_of<R>::type* __restrict__ h, const double2* __restrict__ t2x,
                          const double2* __restrict__ t2y, typename cplx_of<R>::type* __restrict__ buf) {
  const size_t n = (size_t)g.nx * g.ny;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int y = (int)(i / g.nx), x = (int)(i - (size_t)y * g.nx);
    const int px = s_src(x, g.nx), py = s_src(y, g.ny);
    const double xe = eye_xe(g, px), ye = eye_ye(g, py);
    const double r = sqrt(xe * xe + ye * ye);
    typename cplx_of<R>::type v = mk((R)0, (R)0);
    if (r < r_alias && r < r_pupil) {
      int sx = (px - shx) % g.nx; if (sx < 0) sx += g.nx;
      int sy = (py - shy) % g.ny; if (sy < 0) sy += g.ny;
      v = cmul_d<R>(h[(size_t)sy * g.nx + sx], t2x[px], t2y[py]);
    }
    buf[i] = v;
  }
}

template <typename R>
__global__ void eye_magnitude(int nx, int ny, const typename cplx_of<R>::type* __restrict__ spec, R* __restrict__ out) {
  const size_t n = (size_t)nx * ny;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int y = (int)(i / nx), x = (int)(i - (size_t)y * nx);
    const typename cplx_of<R>::type v = spec[(size_t)s_src(y, ny) * nx + s_src(x, nx)];
    out[i] = hypot(v.x, v.y);
  }
}

template <typename R>
oh_status run_eye(oh_ctx* ctx, const oh_eye_params* p, const void* fringe, void* out, cudaStream_t st) {
  typedef typename cplx_of<R>::type C;
  const int prec = sizeof(R) == 8 ? 1 : 0;
  const int s = p->pixel_scale;
  const int nx = p->pnx / s, ny = p->pny / s;
  if (nx < 1 || ny < 1) return fail(OH_ERR_INVALID_ARG, "pixel counts below the scale");
  const double ppx = p->ppx / s, ppy = p->ppy / s;
  const double lam = p->lambda, f = p->field_lens, L = p->eye_length;
  EyeGrid g;
  g.nx = nx; g.ny = ny;
  g.ppx_e = lam * f / (nx * ppx);
  g.ppy_e = lam * f / (ny * ppy);
  g.Ex = g.ppx_e * nx;
  g.Ey = g.ppy_e * ny;
  const double fe = L * (f - p->focus_distance) / (L + (f - p->focus_distance));
  const double feff = fe * L / (fe - L);
  const int shx = -(int)std::round(p->eye_center_x / g.ppx_e);
  const int shy = (int)std::round(p->eye_center_y / g.ppy_e);
  const double r_alias = std::fabs(lam * feff / (2.0 * std::max(g.ppx_e, g.ppy_e)));
  const double r_pupil = p->eye_pupil_diameter / 2.0;
  const size_t npx = (size_t)nx * ny;
  void* tp;
  OH_TRY(scratch(ctx, "eye.tab", (size_t)2 * (nx + ny) * sizeof(double2), &tp));
  double2* t1x = static_cast<double2*>(tp);
  double2* t1y = t1x + nx;
  double2* t2x = t1y + ny;
  double2* t2y = t2x + nx;
  void* a;
  void* b;
  OH_TRY(scratch(ctx, "eye.a", npx * sizeof(C), &a));
  OH_TRY(scratch(ctx, "eye.b", npx * sizeof(C), &b));
  const int grid = oh::sm_count() * 8;
  KernelTimer kt(ctx, "eye_reconstruct", st);
  eye_tables<<<(nx + ny + 255) / 256, 256, 0, st>>>(g, lam, f, feff, t1x, t1y, t2x, t2y);
  OH_LAUNCH_CHECK();
  eye_pack<R><<<grid, 256, 0, st>>>(nx, ny, static_cast<const R*>(fringe), static_cast<C*>(a));
  OH_LAUNCH_CHECK();
  OH_TRY(fft2d_enqueue(ctx, prec, nx, ny, a, a, nullptr, -1, 0, 0, st));
  eye_lens<R><<<grid, 256, 0, st>>>(g, static_cast<const C*>(a), t1x, t1y, static_cast<C*>(b));
  OH_LAUNCH_CHECK();
  eye_pupil<R><<<grid, 256, 0, st>>>(g, shx, shy, r_alias, r_pupil, static_cast<const C*>(b), t2x, t2y,
                                     static_cast<C*>(a));
  OH_LAUNCH_CHECK();
  OH_TRY(fft2d_enqueue(ctx, prec, nx, ny, a, a, nullptr, -1, 0, 0, st));
  eye_magnitude<R><<<grid, 256, 0, st>>>(nx, ny, static_cast<const C*>(a), static_cast<R*>(out));
  OH_LAUNCH_CHECK();
  return OH_OK;
}

}  // namespace

}  // namespace oh

using namespace oh;

extern "C" oh_status oh_reconstruct_eye(oh_ctx* ctx, oh_precision prec, const oh_eye_params* p, const void* fringe,
                                        void* out, void* stream) {
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  CallScope cs(ctx, st);
  OH_TRY(cs.status());
  if (!p || p->pnx < 1 || p->pny < 1 || p->pixel_scale < 1 || !(p->ppx > 0) || !(p->ppy > 0) || !(p->lambda > 0))
    return fail(OH_ERR_INVALID_ARG, "bad eye-model parameters");
  if (!(p->field_lens != p->focus_distance) || !(p->eye_length > 0))
    return fail(OH_ERR_INVALID_ARG, "focus distance equals the field-lens focal length, or eye length <= 0");
  if (!fringe || !out) return fail(OH_ERR_INVALID_ARG, "fringe and out are required");
  if (prec == OH_FP64) return run_eye<double>(ctx, p, fringe, out, st);
  return run_eye<float>(ctx, p, fringe, out, st);
}
