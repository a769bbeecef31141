// Point-light-source summation: the per-pixel point sums of CWO++'s cwoPLS
// class (OpenHolo_WRP/openwrp_console_ver 1.0/cwo/src/cwoPLS.cpp):
//   Huygens    :316-368   U = sum_k exp(i (k r + ph)) / r
//   Fresnel    :370-424   U = sum_k exp(i (k rho^2 / (2 dz) + ph))
//   CGHFresnel :472-520   I = sum_k cos(k rho^2 / (2 dz) + ph)
// with dx = (j - Nx/2) dpx + dox - (x_k + sox), dy = (i - Ny/2) dpy + doy -
// (y_k + soy), rho^2 = dx^2 + dy^2, dz = z_k + z.
//
// FP32 phases.  The paraxial phase k rho^2 / (2 dz) reaches thousands of
// radians, so it is never formed in float.  Per point, with u = the point's
// column in pixel units, m = rint(u), d = u - m and n = j - m,
//   k dx^2 / (2 dz) / (2 pi) = alpha n^2 + beta n + gamma   (turns),
//   alpha = k dpx^2 / (4 pi dz), beta = -2 alpha d, gamma = alpha d^2,
// and alpha, beta, gamma are held as 64-bit fixed-point fractions of a turn
// (computed in FP64 once per point).  alpha n^2 + beta n + gamma mod 1 is
// then exact integer arithmetic; its top 32 bits give the x phase, likewise
// y, and the two add as 32-bit integers (wrap-around = mod one turn).
// Huygens adds the FP64-reduced k|dz| to the y part and evaluates the small
// non-paraxial remainder
//   k (r - |dz| - rho^2 / (2|dz|)) = -k rho^4 / (2 |dz| (r + |dz|)^2)
// in float (a few rad at most for scenes the paraxial sum is used on).
//
// Engines.  Fresnel and CGHFresnel factor into per-point x and y terms,
// U = e^{i ph} Ey^T diag(a) Ex, a complex matrix product over the points:
// pls_gemm_f32 runs it on the CUDA cores (64x64 output tiles, FP32) and the
// tensor-core engine (pls_tc.cu) with split BF16 operands.  pls_direct_f32
// evaluates every term (all modes; Huygens always).  FP64 evaluates every
// term in double precision.
#include <cmath>
#include "context.h"
#include "pls.cuh"

namespace oh {

__device__ __forceinline__ unsigned long long frac_to_fixed(double t) {
  double f = t - floor(t);
  if (f >= 1.0) f = 0.0;
  return __double2ull_rz(f * 18446744073709551616.0);
}

__global__ void pls_prep(PlsGeom g, const oh_pls_point* __restrict__ pts, int n, PlsPt* __restrict__ out) {
  const double inv2pi = 0.15915494309189533576888376337251;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const oh_pls_point p = pts[k];
    PlsPt q;
    const double dz = (double)p.z + g.z;
    const double adz = fabs(dz);
    const double dzp = g.mode == OH_PLS_HUYGENS ? adz : dz;       // paraxial denominator
    const bool ok = dzp != 0.0;
    const double c = ok ? g.k / (2.0 * dzp) * inv2pi : 0.0;      // turns per m^2
    const double u = ((double)p.x + g.sox - g.dox) / g.dpx + (double)(g.nx >> 1);
    const double v = ((double)p.y + g.soy - g.doy) / g.dpy + (double)(g.ny >> 1);
    const double ul = fmin(fmax(u, -1e9), 1e9), vl = fmin(fmax(v, -1e9), 1e9);
    q.mx = (int)rint(ul);
    q.my = (int)rint(vl);
    const double du = ul - q.mx, dv = vl - q.my;
    const double cx = c * g.dpx * g.dpx, cy = c * g.dpy * g.dpy;
    q.ax = frac_to_fixed(cx);
    q.bx = frac_to_fixed(-2.0 * cx * du);
    q.gx = frac_to_fixed(cx * du * du);
    double base = g.ph * inv2pi;
    if (g.mode == OH_PLS_HUYGENS) base += g.k * adz * inv2pi - rint(g.k * adz * inv2pi);
    q.ay = frac_to_fixed(cy);
    q.by = frac_to_fixed(-2.0 * cy * dv);
    q.gy = frac_to_fixed(cy * dv * dv + base);
    q.u = (float)ul;
    q.v = (float)vl;
    q.dz = (float)adz;
    // Huygens remainder factor -k / (2 |dz|) / (2 pi), turns per m^4 / (r + |dz|)^2
    q.rk = ok ? (float)(-g.k / (2.0 * adz) * inv2pi) : 0.f;
    q.ar = ok ? (g.use_amp ? p.a_re : 1.f) : 0.f;
    q.ai = ok ? (g.use_amp ? p.a_im : 0.f) : 0.f;
    out[k] = q;
  }
}

constexpr int kPlsTX = 32, kPlsTY = 8, kPlsPts = 64;

template <int MODE>
__global__ void __launch_bounds__(kPlsTX * kPlsTY) pls_direct_f32(PlsGeom g, const PlsPt* __restrict__ pts, int n,
                                                                  float2* __restrict__ outc, float* __restrict__ outr,
                                                                  int accumulate) {
  __shared__ uint32_t sTx[kPlsPts][kPlsTX];
  __shared__ uint32_t sTy[kPlsPts][kPlsTY];
  __shared__ float4 sP[kPlsPts];     // u, v, |dz|, rk
  __shared__ float2 sA[kPlsPts];
  const int tx = threadIdx.x % kPlsTX, ty = threadIdx.x / kPlsTX;
  const int j = blockIdx.x * kPlsTX + tx, i = blockIdx.y * kPlsTY + ty;
  const float fj = (float)j, fi = (float)i;
  const float dpx = (float)g.dpx, dpy = (float)g.dpy;
  float re = 0.f, im = 0.f;
  for (int k0 = 0; k0 < n; k0 += kPlsPts) {
    const int cnt = min(kPlsPts, n - k0);
    __syncthreads();
    for (int e = threadIdx.x; e < cnt * kPlsTX; e += blockDim.x) {
      const int kk = e / kPlsTX, c = e - kk * kPlsTX;
      const PlsPt& q = pts[k0 + kk];
      sTx[kk][c] = pls_turns(q.ax, q.bx, q.gx, blockIdx.x * kPlsTX + c - q.mx);
    }
    for (int e = threadIdx.x; e < cnt * kPlsTY; e += blockDim.x) {
      const int kk = e / kPlsTY, r = e - kk * kPlsTY;
      const PlsPt& q = pts[k0 + kk];
      sTy[kk][r] = pls_turns(q.ay, q.by, q.gy, blockIdx.y * kPlsTY + r - q.my);
    }
    for (int e = threadIdx.x; e < cnt; e += blockDim.x) {
      const PlsPt& q = pts[k0 + e];
      sP[e] = make_float4(q.u, q.v, q.dz, q.rk);
      sA[e] = make_float2(q.ar, q.ai);
    }
    __syncthreads();
#pragma unroll 4
    for (int kk = 0; kk < cnt; ++kk) {
      const uint32_t t = sTx[kk][tx] + sTy[kk][ty];
      float cs, sn;
      float2 a = sA[kk];
      if constexpr (MODE == OH_PLS_HUYGENS) {
        const float4 q = sP[kk];
        const float dx = (fj - q.x) * dpx, dy = (fi - q.y) * dpy;
        const float rho2 = fmaf(dx, dx, dy * dy);
        const float r2 = fmaf(q.z, q.z, rho2);
        const float rinv = rsqrtf(r2);
        const float s = fmaf(r2, rinv, q.z);                       // r + |dz|
        const float rem = q.w * rho2 * rho2 * __fdividef(1.f, s * s); // turns
        float f = __uint_as_float(0x3F800000u | (t >> 9)) - 1.5f + rem;
        f -= rintf(f);
        __sincosf(6.28318530717958647692f * f, &sn, &cs);
        a.x *= -rinv;     // -1/r: the half-turn offset of the [1, 2) mapping
        a.y *= -rinv;
      } else {
        pls_cis_neg(t, &cs, &sn);
        a.x = -a.x;
        a.y = -a.y;
      }
      if constexpr (MODE == OH_PLS_CGH_FRESNEL) {
        re = fmaf(a.x, cs, fmaf(-a.y, sn, re));
      } else {
        re = fmaf(a.x, cs, fmaf(-a.y, sn, re));
        im = fmaf(a.x, sn, fmaf(a.y, cs, im));
      }
    }
  }
  if (j < g.nx && i < g.ny) {
    const size_t o = (size_t)i * g.nx + j;
    if constexpr (MODE == OH_PLS_CGH_FRESNEL) {
      outr[o] = accumulate ? outr[o] + re : re;
    } else {
      if (accumulate) { const float2 v = outc[o]; outc[o] = make_float2(v.x + re, v.y + im); }
      else outc[o] = make_float2(re, im);
    }
  }
}

// Factor tables for the matrix-product engines: ex[k][j] = e^{2 pi i tx},
// ey[k][i] = a_k e^{2 pi i ty} (ty carries ph).
__global__ void pls_tables(PlsGeom g, const PlsPt* __restrict__ pts, int n, float2* __restrict__ ex,
                           float2* __restrict__ ey) {
  const long long tot_x = (long long)n * g.nx, tot = tot_x + (long long)n * g.ny;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < tot; e += (long long)gridDim.x * blockDim.x) {
    float c, s;
    if (e < tot_x) {
      const int k = (int)(e / g.nx), j = (int)(e - (long long)k * g.nx);
      const PlsPt& q = pts[k];
      pls_cis_neg(pls_turns(q.ax, q.bx, q.gx, j - q.mx), &c, &s);
      ex[e] = make_float2(-c, -s);
    } else {
      const long long f = e - tot_x;
      const int k = (int)(f / g.ny), i = (int)(f - (long long)k * g.ny);
      const PlsPt& q = pts[k];
      pls_cis_neg(pls_turns(q.ay, q.by, q.gy, i - q.my), &c, &s);
      ey[f] = make_float2(-(q.ar * c - q.ai * s), -(q.ar * s + q.ai * c));
    }
  }
}

// C[i][j] (+)= sum_k ey[k][i] ex[k][j]; 64x64 tile per block, 4x4 complex
// outputs per thread, 16 points per shared-memory step.
constexpr int kGB = 64, kGK = 16;

template <int MODE>
__global__ void __launch_bounds__(256) pls_gemm_f32(PlsGeom g, const float2* __restrict__ ex,
                                                   const float2* __restrict__ ey, int n,
                                                   float2* __restrict__ outc, float* __restrict__ outr,
                                                   int accumulate) {
  __shared__ float2 sX[kGK][kGB];
  __shared__ float2 sY[kGK][kGB];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int j0 = blockIdx.x * kGB, i0 = blockIdx.y * kGB;
  float2 acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) acc[a][b] = make_float2(0.f, 0.f);
  for (int k0 = 0; k0 < n; k0 += kGK) {
    __syncthreads();
    for (int e = threadIdx.x; e < kGK * kGB; e += 256) {
      const int kk = e / kGB, c = e - kk * kGB;
      const int k = k0 + kk;
      const bool okk = k < n;
      sX[kk][c] = okk && j0 + c < g.nx ? ex[(size_t)k * g.nx + j0 + c] : make_float2(0.f, 0.f);
      sY[kk][c] = okk && i0 + c < g.ny ? ey[(size_t)k * g.ny + i0 + c] : make_float2(0.f, 0.f);
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < kGK; ++kk) {
      float2 y[4], x[4];
#pragma unroll
      for (int a = 0; a < 4; ++a) y[a] = sY[kk][ty + 16 * a];
#pragma unroll
      for (int b = 0; b < 4; ++b) x[b] = sX[kk][tx + 16 * b];
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) {
          acc[a][b].x = fmaf(y[a].x, x[b].x, fmaf(-y[a].y, x[b].y, acc[a][b].x));
          acc[a][b].y = fmaf(y[a].x, x[b].y, fmaf(y[a].y, x[b].x, acc[a][b].y));
        }
    }
  }
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    const int i = i0 + ty + 16 * a;
    if (i >= g.ny) continue;
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      const int j = j0 + tx + 16 * b;
      if (j >= g.nx) continue;
      const size_t o = (size_t)i * g.nx + j;
      if constexpr (MODE == OH_PLS_CGH_FRESNEL) {
        outr[o] = accumulate ? outr[o] + acc[a][b].x : acc[a][b].x;
      } else {
        if (accumulate) { const float2 v = outc[o]; outc[o] = make_float2(v.x + acc[a][b].x, v.y + acc[a][b].y); }
        else outc[o] = acc[a][b];
      }
    }
  }
}

// FP64: every term in double precision, as the restated reference formulas.
template <int MODE>
__global__ void __launch_bounds__(256) pls_direct_f64(PlsGeom g, const oh_pls_point* __restrict__ pts, int n,
                                                     double2* __restrict__ outc, double* __restrict__ outr) {
  __shared__ double sP[kPlsPts][5];
  const int tx = threadIdx.x % kPlsTX, ty = threadIdx.x / kPlsTX;
  const int j = blockIdx.x * kPlsTX + tx, i = blockIdx.y * kPlsTY + ty;
  const double X = (double)(j - (g.nx >> 1)) * g.dpx + g.dox;
  const double Y = (double)(i - (g.ny >> 1)) * g.dpy + g.doy;
  double re = 0.0, im = 0.0;
  for (int k0 = 0; k0 < n; k0 += kPlsPts) {
    const int cnt = min(kPlsPts, n - k0);
    __syncthreads();
    for (int e = threadIdx.x; e < cnt; e += blockDim.x) {
      const oh_pls_point p = pts[k0 + e];
      sP[e][0] = (double)p.x + g.sox;
      sP[e][1] = (double)p.y + g.soy;
      sP[e][2] = (double)p.z + g.z;
      sP[e][3] = g.use_amp ? (double)p.a_re : 1.0;
      sP[e][4] = g.use_amp ? (double)p.a_im : 0.0;
    }
    __syncthreads();
    for (int kk = 0; kk < cnt; ++kk) {
      const double dx = X - sP[kk][0], dy = Y - sP[kk][1], dz = sP[kk][2];
      double ph, amp = 1.0;
      if constexpr (MODE == OH_PLS_HUYGENS) {
        const double r = sqrt(dx * dx + dy * dy + dz * dz);
        ph = g.k * r + g.ph;
        amp = 1.0 / r;
      } else {
        if (dz == 0.0) continue;
        ph = g.k * (dx * dx + dy * dy) / (2.0 * dz) + g.ph;
      }
      double s, c;
      sincos(ph, &s, &c);
      const double ar = sP[kk][3] * amp, ai = sP[kk][4] * amp;
      re += ar * c - ai * s;
      im += ar * s + ai * c;
    }
  }
  if (j < g.nx && i < g.ny) {
    const size_t o = (size_t)i * g.nx + j;
    if constexpr (MODE == OH_PLS_CGH_FRESNEL) outr[o] = re;
    else outc[o] = make_double2(re, im);
  }
}

static oh_status validate_pls(const oh_pls_params* p, const oh_pls_point* pts, int n, void* out) {
  if (!p) return fail(OH_ERR_INVALID_ARG, "null PLS params");
  if (p->nx < 1 || p->ny < 1) return fail(OH_ERR_INVALID_ARG, "nx/ny must be positive");
  if (!(p->dst_px > 0) || !(p->dst_py > 0) || !(p->lambda > 0)) return fail(OH_ERR_INVALID_ARG, "pitch and wavelength must be positive");
  if (p->mode < OH_PLS_HUYGENS || p->mode > OH_PLS_CGH_FRESNEL) return fail(OH_ERR_INVALID_ARG, "unknown PLS mode");
  if (p->engine < OH_PLS_ENGINE_AUTO || p->engine > OH_PLS_ENGINE_TENSOR) return fail(OH_ERR_INVALID_ARG, "unknown PLS engine");
  if (n < 0 || (n > 0 && !pts) || !out) return fail(OH_ERR_INVALID_ARG, "bad PLS buffers");
  return OH_OK;
}

template <class F>
static void with_pls_mode(int mode, F&& f) {
  if (mode == OH_PLS_HUYGENS) f(std::integral_constant<int, OH_PLS_HUYGENS>{});
  else if (mode == OH_PLS_FRESNEL) f(std::integral_constant<int, OH_PLS_FRESNEL>{});
  else f(std::integral_constant<int, OH_PLS_CGH_FRESNEL>{});
}

static oh_status run_pls(oh_ctx* ctx, int prec, const oh_pls_params* p, const oh_pls_point* pts, int n, void* out,
                         cudaStream_t st) {
  PlsGeom g;
  g.nx = p->nx; g.ny = p->ny; g.mode = p->mode; g.use_amp = p->use_amplitude ? 1 : 0;
  g.k = 2.0 * M_PI / p->lambda;
  g.dpx = p->dst_px; g.dpy = p->dst_py; g.dox = p->dst_ox; g.doy = p->dst_oy;
  g.sox = p->src_ox; g.soy = p->src_oy; g.z = p->z; g.ph = p->phase;
  const size_t npix = (size_t)p->nx * p->ny;
  const bool real_out = p->mode == OH_PLS_CGH_FRESNEL;
  if (n == 0) {
    OH_CUDA_TRY(cudaMemsetAsync(out, 0, npix * (real_out ? 1 : 2) * (prec ? 8 : 4), st));
    return OH_OK;
  }
  dim3 grid((p->nx + kPlsTX - 1) / kPlsTX, (p->ny + kPlsTY - 1) / kPlsTY);
  oh_status rs = OH_OK;
  if (prec) {
    with_pls_mode(p->mode, [&](auto mc) {
      constexpr int M = decltype(mc)::value;
      KernelTimer kt(ctx, "pls_direct_f64", st);
      pls_direct_f64<M><<<grid, kPlsTX * kPlsTY, 0, st>>>(g, pts, n, (double2*)out, (double*)out);
      note_launch();
      cudaError_t e = cudaGetLastError();
      if (e != cudaSuccess) rs = cuda_fail(e, "pls_direct_f64 launch");
    });
    return rs;
  }
  void* pp;
  OH_TRY(scratch(ctx, "pls.pts", (size_t)n * sizeof(PlsPt), &pp));
  PlsPt* q = static_cast<PlsPt*>(pp);
  {
    KernelTimer kt(ctx, "pls_prep", st);
    pls_prep<<<std::min((n + 63) / 64, oh::sm_count() * 32), 64, 0, st>>>(g, pts, n, q);
    OH_LAUNCH_CHECK();
  }
  int engine = p->engine;
  if (p->mode == OH_PLS_HUYGENS) engine = OH_PLS_ENGINE_DIRECT;
  if (engine == OH_PLS_ENGINE_AUTO) engine = OH_PLS_ENGINE_TENSOR;
  if (engine == OH_PLS_ENGINE_TENSOR) {
    const oh_status ts = pls_tensor_enqueue(ctx, g, q, n, out, st);
    if (ts != OH_ERR_UNSUPPORTED_SIZE || p->engine == OH_PLS_ENGINE_TENSOR) return ts;
    engine = OH_PLS_ENGINE_GEMM;     // automatic choice: shapes the tensor engine does not take
  }
  if (engine == OH_PLS_ENGINE_DIRECT) {
    with_pls_mode(p->mode, [&](auto mc) {
      constexpr int M = decltype(mc)::value;
      KernelTimer kt(ctx, "pls_direct_f32", st);
      pls_direct_f32<M><<<grid, kPlsTX * kPlsTY, 0, st>>>(g, q, n, (float2*)out, (float*)out, 0);
      note_launch();
      cudaError_t e = cudaGetLastError();
      if (e != cudaSuccess) rs = cuda_fail(e, "pls_direct_f32 launch");
    });
    return rs;
  }
  // CUDA-core matrix product over point chunks (tables <= 256 MiB)
  const size_t per_pt = (size_t)(p->nx + p->ny) * sizeof(float2);
  const int chunk = (int)std::max<size_t>(16, std::min<size_t>((size_t)n, ((size_t)256 << 20) / per_pt));
  void* tp;
  OH_TRY(scratch(ctx, "pls.tables", (size_t)chunk * per_pt, &tp));
  float2* ex = static_cast<float2*>(tp);
  float2* ey = ex + (size_t)chunk * p->nx;
  dim3 gg((p->nx + kGB - 1) / kGB, (p->ny + kGB - 1) / kGB);
  for (int k0 = 0; k0 < n; k0 += chunk) {
    const int cnt = std::min(chunk, n - k0);
    {
      KernelTimer kt(ctx, "pls_tables", st);
      pls_tables<<<oh::sm_count() * 8, 256, 0, st>>>(g, q + k0, cnt, ex, ey);
      OH_LAUNCH_CHECK();
    }
    with_pls_mode(p->mode, [&](auto mc) {
      constexpr int M = decltype(mc)::value;
      if constexpr (M != OH_PLS_HUYGENS) {
        KernelTimer kt(ctx, "pls_gemm_f32", st);
        pls_gemm_f32<M><<<gg, 256, 0, st>>>(g, ex, ey, cnt, (float2*)out, (float*)out, k0 > 0);
        note_launch();
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) rs = cuda_fail(e, "pls_gemm_f32 launch");
      }
    });
    OH_TRY(rs);
  }
  return OH_OK;
}

}  // namespace oh

using namespace oh;

extern "C" oh_status oh_pls(oh_ctx* ctx, oh_precision prec, const oh_pls_params* p, const oh_pls_point* pts,
                            int n_points, void* out, void* stream) {
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  CallScope cs(ctx, st);
  OH_TRY(cs.status());
  OH_TRY(validate_pls(p, pts, n_points, out));
  return run_pls(ctx, prec == OH_FP64 ? 1 : 0, p, pts, n_points, out, st);
}
