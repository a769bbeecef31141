// Texture/depth wavefront-recording plane: CWO++'s cwoTexDep::WRP
// (OpenHolo_WRP/openwrp_console_ver 1.0/cwo/src/cwoTexDep.cpp).
//
// OH_TEXDEP_SINGLE (cwoTexDep.cpp:29-75): every texel with tex = int(value)
// != 0 adds tex exp(i k r) at (tx + wx, ty + wy), wx, wy in [-w, w),
// r = z + ((wx px)^2 + (wy py)^2) / (2 z), w = int(|z| tan(asin(lambda/(2 px))) / px),
// inside the plane only.  The window is the same for every texel and
// separable, exp(i k z) kx(wx) ky(wy), so the scatter equals a 2-D
// convolution of the texture with it, done as a row pass (texture * kx) and
// a column pass (* ky, times exp(i k z), added into the field): O(N w)
// instead of O(N w^2).  kx, ky are tabulated with FP64-reduced phases.
//
// OH_TEXDEP_RANGE (cwoTexDep.cpp:78-136): texels whose dep lies in
// [lo, hi) use dz = z + (hi - dep) dz_step, w = int(int(|dz| tan(asin(lambda/(2 px)))/px) / 1.4),
// a half zone plate wy in [-w, 0), wx in [-w, w), r = (dx^2 + dy^2) / (2 dz).
// The reference takes dep from the texture value when a depth image is
// loaded (it copies the pixel into dep before reading the depth image into
// the same variable) and 0 without one: dep_from_texture = 1 keeps that,
// 0 uses the depth image.  The window depends on the texel, so each output
// pixel gathers the texels whose windows cover it (no atomics); the
// per-level window and phase coefficient are computed in FP64 on the host.
//
// lambda and the pitches enter as the float values the reference holds;
// phases are reduced in FP64 or evaluated in turns (the reference forms
// k r in float).
#include <cmath>
#include "context.h"

namespace oh {

namespace {

struct TexGeom {
  int nx, ny, w;            // single mode: half-width
  int lo, hi, W;            // range mode: dep range, widest window
  int dep_from_texture;
};

__device__ __forceinline__ double2 cis_t(double t) {
  t -= rint(t);
  double s, c;
  sincospi(2.0 * t, &s, &c);
  return make_double2(c, s);
}

// kx[m], ky[m] for offsets m - w, exp(i k (off p)^2 / (2 z)); entry 2w of kx holds exp(i k z)
__global__ void texdep_tables(int w, double k_turn, double px, double py, double z, double2* __restrict__ kx,
                              double2* __restrict__ ky) {
  const int n = 2 * w;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e <= 2 * n; e += gridDim.x * blockDim.x) {
    if (e < n) {
      const double d = (e - w) * px;
      kx[e] = cis_t(k_turn * d * d / (2.0 * z));
    } else if (e < 2 * n) {
      const double d = (e - n - w) * py;
      ky[e - n] = cis_t(k_turn * d * d / (2.0 * z));
    } else {
      kx[n] = cis_t(k_turn * z);
    }
  }
}

template <typename R> struct V2;
template <> struct V2<float> { typedef float2 T; };
template <> struct V2<double> { typedef double2 T; };

template <typename R>
__global__ void texdep_rows(TexGeom g, const uint8_t* __restrict__ tex, const double2* __restrict__ kx,
                            typename V2<R>::T* __restrict__ t) {
  const int n = 2 * g.w;
  const size_t tot = (size_t)g.nx * g.ny;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < tot; i += (size_t)gridDim.x * blockDim.x) {
    const int y = (int)(i / g.nx), x = (int)(i - (size_t)y * g.nx);
    R re = 0, im = 0;
    // texel tx = x + w - m for m in [0, 2w), inside the row
    const int m_lo = max(0, x + g.w - (g.nx - 1)), m_hi = min(n, x + g.w + 1);
    const uint8_t* row = tex + (size_t)y * g.nx;
    for (int m = m_lo; m < m_hi; ++m) {
      const R v = (R)row[x + g.w - m];
      if (v != (R)0) {
        re += v * (R)kx[m].x;
        im += v * (R)kx[m].y;
      }
    }
    t[i].x = re;
    t[i].y = im;
  }
}

template <typename R>
__global__ void texdep_cols(TexGeom g, const typename V2<R>::T* __restrict__ t, const double2* __restrict__ ky,
                            const double2* __restrict__ kx, typename V2<R>::T* __restrict__ out) {
  const int n = 2 * g.w;
  const size_t tot = (size_t)g.nx * g.ny;
  const R c0r = (R)kx[n].x, c0i = (R)kx[n].y;      // exp(i k z)
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < tot; i += (size_t)gridDim.x * blockDim.x) {
    const int y = (int)(i / g.nx), x = (int)(i - (size_t)y * g.nx);
    R re = 0, im = 0;
    const int m_lo = max(0, y + g.w - (g.ny - 1)), m_hi = min(n, y + g.w + 1);
    for (int m = m_lo; m < m_hi; ++m) {
      const typename V2<R>::T a = t[(size_t)(y + g.w - m) * g.nx + x];
      const R kr = (R)ky[m].x, ki = (R)ky[m].y;
      re += a.x * kr - a.y * ki;
      im += a.x * ki + a.y * kr;
    }
    out[i].x += re * c0r - im * c0i;
    out[i].y += re * c0i + im * c0r;
  }
}

// per dep level: half-width and phase coefficient k / (2 dz) / (2 pi), turns per m^2 (w = 0: level unused)
struct LevelTab { int w[256]; double coef[256]; };

template <typename R>
__global__ void texdep_range(TexGeom g, double px, double py, const uint8_t* __restrict__ tex,
                             const uint8_t* __restrict__ dep, const LevelTab lt, typename V2<R>::T* __restrict__ out) {
  __shared__ int sw[256];
  __shared__ R sc[256];
  for (int e = threadIdx.x; e < 256; e += blockDim.x) { sw[e] = lt.w[e]; sc[e] = (R)lt.coef[e]; }
  __syncthreads();
  const R pxr = (R)px, pyr = (R)py;
  const size_t tot = (size_t)g.nx * g.ny;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < tot; i += (size_t)gridDim.x * blockDim.x) {
    const int y = (int)(i / g.nx), x = (int)(i - (size_t)y * g.nx);
    R re = 0, im = 0;
    // texels (tx, ty) with x - tx in [-w, w) and y - ty in [-w, 0): ty in (y, y + w], tx in (x - w, x + w]
    const int ty_hi = min(g.ny - 1, y + g.W);
    const int tx_lo = max(0, x - g.W + 1), tx_hi = min(g.nx - 1, x + g.W);
    for (int ty = y + 1; ty <= ty_hi; ++ty) {
      const uint8_t* trow = tex + (size_t)ty * g.nx;
      const int wy = y - ty;
      for (int tx = tx_lo; tx <= tx_hi; ++tx) {
        const int tv = trow[tx];
        if (tv == 0) continue;
        const int d = g.dep_from_texture ? tv : (dep ? (int)dep[(size_t)ty * g.nx + tx] : 0);
        if (d < g.lo || d >= g.hi) continue;
        const int w = sw[d];
        const int wx = x - tx;
        if (wx < -w || wx >= w || wy < -w) continue;
        const R dx = (R)wx * pxr, dy = (R)wy * pyr;
        R t = sc[d] * (dx * dx + dy * dy);      // turns
        t -= rint(t);
        R sn, cs;
        if constexpr (sizeof(R) == 8) sincospi(2.0 * t, &sn, &cs);
        else sincospif(2.f * t, &sn, &cs);
        re += (R)tv * cs;
        im += (R)tv * sn;
      }
    }
    out[i].x += re;
    out[i].y += im;
  }
}

template <typename R>
oh_status run_texdep(oh_ctx* ctx, int mode, const oh_texdep_params* p, const uint8_t* tex, const uint8_t* dep,
                     void* field, cudaStream_t st) {
  typedef typename V2<R>::T C;
  // float-held wavelength and pitches, as in the reference
  const double lam = (double)(float)p->lambda, px = (double)(float)p->px, py = (double)(float)p->py;
  const double k_turn = 1.0 / lam;                              // k / (2 pi)
  const double tn = std::tan(std::asin(lam / (2.0 * px)));     // half-width = int(|dz| tn / px)
  TexGeom g{p->nx, p->ny, 0, p->range_lo, p->range_hi, 0, p->dep_from_texture ? 1 : 0};
  const int grid = oh::sm_count() * 8;
  if (mode == OH_TEXDEP_SINGLE) {
    if (p->z == 0.0) return fail(OH_ERR_INVALID_ARG, "z must be non-zero");
    const double wd = std::fabs(p->z) * tn / px;
    if (wd > 1e6) return fail(OH_ERR_UNSUPPORTED_SIZE, "window half-width above 10^6 pixels");
    g.w = (int)wd;
    if (g.w <= 0) return OH_OK;
    void* tp;
    OH_TRY(scratch(ctx, "texdep.tab", (size_t)(4 * g.w + 1) * sizeof(double2), &tp));
    double2* kx = static_cast<double2*>(tp);
    double2* ky = kx + 2 * g.w + 1;
    void* bp;
    OH_TRY(scratch(ctx, "texdep.rows", (size_t)p->nx * p->ny * sizeof(C), &bp));
    KernelTimer kt(ctx, "texdep_single", st);
    texdep_tables<<<(4 * g.w + 256) / 256, 256, 0, st>>>(g.w, k_turn, px, py, p->z, kx, ky);
    OH_LAUNCH_CHECK();
    texdep_rows<R><<<grid, 256, 0, st>>>(g, tex, kx, static_cast<C*>(bp));
    OH_LAUNCH_CHECK();
    texdep_cols<R><<<grid, 256, 0, st>>>(g, static_cast<const C*>(bp), ky, kx, static_cast<C*>(field));
    OH_LAUNCH_CHECK();
    return OH_OK;
  }
  LevelTab lt;
  int W = 0;
  for (int d = 0; d < 256; ++d) {
    lt.w[d] = 0;
    lt.coef[d] = 0.0;
    if (d < p->range_lo || d >= p->range_hi) continue;
    const double dz = p->z + (p->range_hi - d) * p->dz_step;
    if (dz == 0.0) continue;
    const double wd = std::fabs(dz) * tn / px;
    if (wd > 1e6) return fail(OH_ERR_UNSUPPORTED_SIZE, "window half-width above 10^6 pixels");
    const int w = (int)((double)(int)wd / 1.4);    // the reference's (float)tw / 1.4 divides in double
    lt.w[d] = w;
    lt.coef[d] = k_turn / (2.0 * dz);
    W = std::max(W, w);
  }
  if (W <= 0) return OH_OK;
  if (W > 4096) return fail(OH_ERR_UNSUPPORTED_SIZE, "range-mode window half-width above 4096 pixels");
  g.W = W;
  KernelTimer kt(ctx, "texdep_range", st);
  texdep_range<R><<<grid, 256, 0, st>>>(g, px, py, tex, dep, lt, static_cast<C*>(field));
  OH_LAUNCH_CHECK();
  return OH_OK;
}

}  // namespace

}  // namespace oh

using namespace oh;

extern "C" oh_status oh_texdep_wrp(oh_ctx* ctx, oh_precision prec, int mode, const oh_texdep_params* p,
                                   const uint8_t* tex, const uint8_t* dep, void* field, void* stream) {
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  CallScope cs(ctx, st);
  OH_TRY(cs.status());
  if (!p || p->nx < 1 || p->ny < 1 || !(p->px > 0) || !(p->py > 0) || !(p->lambda > 0) || !(p->lambda < 2 * p->px))
    return fail(OH_ERR_INVALID_ARG, "bad texture-WRP parameters (pitch, wavelength < 2 pitch)");
  if (mode != OH_TEXDEP_SINGLE && mode != OH_TEXDEP_RANGE) return fail(OH_ERR_INVALID_ARG, "unknown texture-WRP mode");
  if (!tex || !field) return fail(OH_ERR_INVALID_ARG, "texture and field are required");
  if (prec == OH_FP64) return run_texdep<double>(ctx, mode, p, tex, dep, field, st);
  return run_texdep<float>(ctx, mode, p, tex, dep, field, st);
}
