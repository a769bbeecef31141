// Wavefront-recording-plane (WRP) accumulation.
//
// OPHWRP::SingleWRP (OpenHolo_WRP/openwrp_console_ver 1.0/openwrp/WRP.cpp:75-140):
//   per point: dz = z_wrp - z_k, w = int(|lambda dz / dp^2 / 2 + 0.5|)*2 - 1,
//   tx = int(x/dp) + Nx/2, ty = int(y/dp) + Ny/2, and for wx, wy in [-w, w):
//   r = sign(dz) sqrt((wx dp)^2 + (wy dp)^2 + dz^2),
//   WRP[ty+wy][tx+wx] += (cos, sin)(k r) / (r + 0.05)   (pixels inside the plane)
// The reference adds with a racy AddPixel (cwo.cpp:4298-4308).  Here a fixed
// window is summed race-free per 64x64 plane tile (wrp_tile*); the formula
// window (w varies per point) is added with float2/double2 atomics.  FP32
// evaluates k r as k dz (reduced mod 2 pi in double, once per point) +
// k rho^2/(|r| + |dz|) (at most tens of rad, exact in float to ~1e-5 rad).
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

// ---- tiled accumulation for fixed windows ------------------------------------
// Points are binned by the 64x64 plane tiles their window overlaps (count,
// scan, fill); one block per tile sums its points' window pixels and adds the
// tile to the plane once, with no global atomics.  FP64 sums in a
// shared-memory copy of the tile; FP32 keeps each thread's pixels in
// registers.
constexpr int kWrpTile = 64;

// Per point: window centre and half-width; exact-path terms (base = k|dz|
// reduced to radians); the FP64 path's dz; and, when the window is paraxial
// enough (series = 1), the polynomial coefficients of the series evaluation
// below in u = rho^2 / dz^2 = (wx sx)^2 + (wy sx)^2, sx = dp / |dz|.
struct WrpPt {
  int tx, ty, w, series;
  float base, adz, sgn, sx;
  float base_t, c1, c2, c3;          // phase in turns: base_t + u (c1 + u (c2 + u c3))
  float a0c, a1c, a2c, pad0;         // amplitude: a0c + u (a1c + u a2c)
  double dz, pad1;
};

__device__ __forceinline__ void wrp_point(const WRPGeom& g, const double* xyz, int k, WrpPt* o) {
  const double two_pi = 6.283185307179586476925286766559;
  const float dpx = (float)g.dp;
  const double kd = (double)(float)(2.0 * M_PI / g.lambda);
  const double px = xyz[3 * k], py = xyz[3 * k + 1], pz = xyz[3 * k + 2];
  // centres far outside the plane are clamped so that c +- w cannot overflow
  const double lim = 1 << 29;
  o->tx = (int)fmin(fmax(px / (double)dpx, -lim), lim) + (g.nx >> 1);
  o->ty = (int)fmin(fmax(py / (double)dpx, -lim), lim) + (g.ny >> 1);
  o->w = g.fixed_w;
  const double dz = (double)(float)g.z - pz;
  o->dz = dz;
  o->sgn = dz > 0.0 ? 1.f : -1.f;
  o->adz = (float)fabs(dz);
  const double kdz = kd * fabs(dz);
  o->base = (float)(kdz - two_pi * rint(kdz / two_pi));
  // Series form: with u = rho^2 / dz^2 and t = sqrt(1 + u) - 1 = u (1/2 - u/8 + u^2/16) + O(5 u^4 / 128),
  //   sgn k|r| / (2 pi) = sgn turns (1 + t),  turns = k|dz| / (2 pi),
  //   1 / (sgn |r| + 0.05) = (1 / a0) / (1 + e),  a0 = sgn |dz| + 0.05,  e = ea t,  ea = sgn |dz| / a0,
  //   1 / (1 + e) = 1 - ea u / 2 + (ea / 8 + ea^2 / 4) u^2 - (ea / 16 + ea^2 / 8 + ea^3 / 8) u^3 + ...,
  // used when the dropped terms stay below 1e-6 rad (phase) and 1e-8 relative
  // (amplitude) over the whole window.
  const double adz = fabs(dz), sg = dz > 0.0 ? 1.0 : -1.0;
  const double a0 = sg * adz + 0.05;
  const double rho2max = 2.0 * (double)g.fixed_w * g.fixed_w * (double)dpx * dpx;
  const double umax = adz > 0.0 ? rho2max / (adz * adz) : 1.0;
  const double ea = fabs(a0) > 1e-6 ? sg * adz / a0 : 0.0;
  const double aea = fabs(ea);
  const double u3 = umax * umax * umax;
  o->series = (adz > 0.0 && fabs(a0) > 1e-6 && umax < 0.05 &&
               kdz * (5.0 / 128.0) * umax * u3 < 1e-6 &&
               (aea / 16.0 + aea * aea / 8.0 + aea * aea * aea / 8.0) * u3 < 1e-8) ? 1 : 0;
  const double turns = kdz / two_pi;
  o->base_t = (float)(sg * (turns - rint(turns)));
  o->c1 = (float)(sg * turns * 0.5);
  o->c2 = (float)(sg * turns * -0.125);
  o->c3 = (float)(sg * turns * 0.0625);
  o->sx = adz > 0.0 ? (float)((double)dpx / adz) : 0.f;
  const double ia0 = fabs(a0) > 1e-6 ? 1.0 / a0 : 0.0;
  o->a0c = (float)ia0;
  o->a1c = (float)(-ia0 * ea * 0.5);
  o->a2c = (float)(ia0 * (ea * 0.125 + ea * ea * 0.25));
  o->pad0 = 0.f;
  o->pad1 = 0.0;
}

// tile index range [t0, t1] along one axis for the window [c - w, c + w) clipped to [0, n)
__device__ __forceinline__ bool wrp_tile_range(int c, int w, int n, int* t0, int* t1) {
  const int lo = max(c - w, 0), hi = min(c + w, n);
  if (lo >= hi) return false;
  *t0 = lo / kWrpTile;
  *t1 = (hi - 1) / kWrpTile;
  return true;
}

__global__ void wrp_prep(WRPGeom g, const double* __restrict__ xyz, int n, WrpPt* __restrict__ pts,
                         int* __restrict__ count, int tiles_x) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    WrpPt q;
    wrp_point(g, xyz, k, &q);
    pts[k] = q;
    int x0, x1, y0, y1;
    if (!wrp_tile_range(q.tx, q.w, g.nx, &x0, &x1) || !wrp_tile_range(q.ty, q.w, g.ny, &y0, &y1)) continue;
    for (int ty = y0; ty <= y1; ++ty)
      for (int tx = x0; tx <= x1; ++tx) atomicAdd(&count[ty * tiles_x + tx], 1);
  }
}

// exclusive scan of count[0..n) into start[0..n], single block
__global__ void wrp_scan(const int* __restrict__ count, int* __restrict__ start, int* __restrict__ cursor, int n) {
  __shared__ int part[1024];
  const int per = (n + blockDim.x - 1) / blockDim.x;
  const int b = threadIdx.x * per, e = min(b + per, n);
  int sum = 0;
  for (int i = b; i < e; ++i) sum += count[i];
  part[threadIdx.x] = sum;
  __syncthreads();
  for (int off = 1; off < blockDim.x; off <<= 1) {
    int v = threadIdx.x >= off ? part[threadIdx.x - off] : 0;
    __syncthreads();
    part[threadIdx.x] += v;
    __syncthreads();
  }
  int run = part[threadIdx.x] - sum;
  for (int i = b; i < e; ++i) { start[i] = run; cursor[i] = run; run += count[i]; }
  if (threadIdx.x == blockDim.x - 1) start[n] = part[threadIdx.x];
}

__global__ void wrp_fill(WRPGeom g, const WrpPt* __restrict__ pts, int n, int* __restrict__ cursor,
                         int* __restrict__ list, int tiles_x) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const WrpPt q = pts[k];
    int x0, x1, y0, y1;
    if (!wrp_tile_range(q.tx, q.w, g.nx, &x0, &x1) || !wrp_tile_range(q.ty, q.w, g.ny, &y0, &y1)) continue;
    for (int ty = y0; ty <= y1; ++ty)
      for (int tx = x0; tx <= x1; ++tx) list[atomicAdd(&cursor[ty * tiles_x + tx], 1)] = k;
  }
}

// FP64 tile: shared-memory accumulators (double atomics on shared memory).
template <typename R>
__global__ void __launch_bounds__(256) wrp_tile(WRPGeom g, const WrpPt* __restrict__ pts, const int* __restrict__ start,
                                               const int* __restrict__ list, int tiles_x,
                                               typename cplx_of<R>::type* __restrict__ wrp) {
  typedef typename cplx_of<R>::type C;
  __shared__ R acc_re[kWrpTile * kWrpTile];
  __shared__ R acc_im[kWrpTile * kWrpTile];
  const int tile = blockIdx.x;
  const int X0 = (tile % tiles_x) * kWrpTile, Y0 = (tile / tiles_x) * kWrpTile;
  for (int i = threadIdx.x; i < kWrpTile * kWrpTile; i += blockDim.x) { acc_re[i] = 0; acc_im[i] = 0; }
  __syncthreads();
  const float dpx = (float)g.dp;
  const double kd = (double)(float)(2.0 * M_PI / g.lambda);
  const int b = start[tile], e = start[tile + 1];
  for (int li = b; li < e; ++li) {
    const WrpPt q = pts[list[li]];
    // window x range [tx - w, tx + w) intersected with this tile and the plane
    const int xa = max(max(q.tx - q.w, X0), 0), xb = min(min(q.tx + q.w, X0 + kWrpTile), g.nx);
    const int ya = max(max(q.ty - q.w, Y0), 0), yb = min(min(q.ty + q.w, Y0 + kWrpTile), g.ny);
    const int wd = xb - xa, area = wd * (yb - ya);
    for (int i = threadIdx.x; i < area; i += blockDim.x) {
      const int yy = i / wd, xx = i - yy * wd;
      const int X = xa + xx, Y = ya + yy;
      const int wx = X - q.tx, wy = Y - q.ty;
      R re, im;
      if constexpr (sizeof(R) == 4) {
        const float ddx = (float)wx * dpx, ddy = (float)wy * dpx;
        const float rho2 = ddx * ddx + ddy * ddy;
        const float ar = sqrtf(rho2 + q.adz * q.adz);
        float ph = q.base + (float)kd * rho2 / (ar + q.adz);
        ph = q.sgn > 0 ? ph : -ph;
        float sn, cs;
        sincosf(ph, &sn, &cs);
        const float inv = 1.f / (q.sgn * ar + 0.05f);
        re = cs * inv; im = sn * inv;
      } else {
        const double ddx = wx * (double)dpx, ddy = wy * (double)dpx;
        const double r = (q.dz > 0.0 ? 1.0 : -1.0) * sqrt(ddx * ddx + ddy * ddy + q.dz * q.dz);
        double sn, cs;
        sincos(kd * r, &sn, &cs);
        re = cs / (r + 0.05); im = sn / (r + 0.05);
      }
      const int o = (Y - Y0) * kWrpTile + (X - X0);
      atomicAdd(&acc_re[o], re);
      atomicAdd(&acc_im[o], im);
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < kWrpTile * kWrpTile; i += blockDim.x) {
    const int X = X0 + i % kWrpTile, Y = Y0 + i / kWrpTile;
    if (X < g.nx && Y < g.ny) {
      C* d = wrp + (size_t)Y * g.nx + X;
      C v = *d;
      v.x += acc_re[i];
      v.y += acc_im[i];
      *d = v;
    }
  }
}

// One window pixel in FP32 at (squared) distance rho2 from the point's axis:
//   k|r| = base + k rho^2 / (|r| + |dz|),   value = (cos, sin)(sgn k|r|) / (sgn |r| + 0.05)
// with one MUFU reciprocal shared by the phase and the amplitude, and the
// phase reduced to [-pi, pi] by a two-term Cody-Waite split of 2 pi before
// the hardware sine/cosine (absolute error ~4e-7 on that interval).
__device__ __forceinline__ float2 wrp_term_f32(float rho2, const WrpPt& q, float kf) {
  const float a2 = fmaf(q.adz, q.adz, rho2);
  const float ar = a2 * rsqrtf(a2);
  const float s = ar + q.adz;
  const float d = fmaf(q.sgn, ar, 0.05f);
  const float inv = __fdividef(1.f, s * d);
  float ph = q.base + kf * rho2 * (d * inv);
  ph = q.sgn > 0.f ? ph : -ph;
  const float n = rintf(ph * 0.159154943091895336f);            // 1 / (2 pi)
  float red = fmaf(n, -6.28318548202514648f, ph);              // 2 pi rounded to float
  red = fmaf(n, 1.74845553146951862e-7f, red);                 // 2 pi - float(2 pi)
  float sn, cs;
  __sincosf(red, &sn, &cs);
  const float amp = s * inv;
  return make_float2(cs * amp, sn * amp);
}

// FP32 tile: each thread owns 16 pixels of the tile (below) and keeps their
// sums in registers; no atomics.  The tile's point records are staged in
// shared memory in chunks of kWrpChunk.
constexpr int kWrpChunk = 128;
static_assert(sizeof(WrpPt) % 16 == 0, "point records are copied as float4");

__global__ void __launch_bounds__(256) wrp_tile_f32(WRPGeom g, const WrpPt* __restrict__ pts,
                                                   const int* __restrict__ start, const int* __restrict__ list,
                                                   int tiles_x, float2* __restrict__ wrp) {
  constexpr int kRows = kWrpTile * kWrpTile / 256;
  constexpr int kParts = (int)(sizeof(WrpPt) / 16);
  __shared__ __align__(16) WrpPt sp[kWrpChunk];
  const int tile = blockIdx.x;
  const int X0 = (tile % tiles_x) * kWrpTile, Y0 = (tile / tiles_x) * kWrpTile;
  // warp w owns columns 8w..8w+7 of the tile; lane l column 8w + l % 8, rows l / 8 + 4 j
  const int c = 8 * (threadIdx.x >> 5) + (threadIdx.x & 7), r0 = (threadIdx.x & 31) >> 3;
  float2 acc[kRows];
#pragma unroll
  for (int j = 0; j < kRows; ++j) acc[j] = make_float2(0.f, 0.f);
  const float dpx = (float)g.dp;
  const float kf = (float)(2.0 * M_PI / g.lambda);
  const int X = X0 + c;
  const int b = start[tile], e = start[tile + 1];
  for (int c0 = b; c0 < e; c0 += kWrpChunk) {
    const int nc = min(kWrpChunk, e - c0);
    __syncthreads();                                  // the previous chunk is consumed
    for (int i = threadIdx.x; i < nc * kParts; i += blockDim.x) {
      const int k = i / kParts, part = i - k * kParts;
      reinterpret_cast<float4*>(sp + k)[part] = reinterpret_cast<const float4*>(pts + __ldg(list + c0 + k))[part];
    }
    __syncthreads();
    for (int li = 0; li < nc; ++li) {
      const WrpPt& q = sp[li];
      const int wx = X - q.tx;
      if (wx < -q.w || wx >= q.w || X >= g.nx) continue;
      const int wy0 = Y0 + r0 - q.ty;                 // wy of row j is wy0 + 4 j
      // row j is in the window and the plane iff 0 <= wy0 + 4 j + w < vlim
      const int v0 = wy0 + q.w;
      const int vlim = min(2 * q.w, g.ny - q.ty + q.w);
      if (vlim <= 0) continue;
      if (q.series) {
        const float sx = q.sx;
        const float xs = (float)wx * sx;
        const float xs2 = xs * xs;
        const float ys0 = (float)wy0 * sx, s4 = 4.f * sx;
        const float bt = q.base_t, c1 = q.c1, c2 = q.c2, c3 = q.c3, a0 = q.a0c, a1 = q.a1c, a2 = q.a2c;
        // rows j = 4h .. 4h+3 span v0 + 16h .. v0 + 16h + 12: a group the window
        // misses is skipped; the others are evaluated without branches (four
        // independent chains) and rows outside the window get amplitude 0
#pragma unroll
        for (int h = 0; h < kRows / 4; ++h) {
          const int vh = v0 + 16 * h;
          if (vh + 12 < 0 || vh >= vlim) continue;
#pragma unroll
          for (int jj = 0; jj < 4; ++jj) {
            const int j = 4 * h + jj;
            const bool in = (unsigned)(vh + 4 * jj) < (unsigned)vlim;
            const float ys = fmaf((float)j, s4, ys0);
            const float u = fmaf(ys, ys, xs2);
            float f = fmaf(u, fmaf(u, fmaf(u, c3, c2), c1), bt);
            f -= rintf(f);
            float sn, cs;
            __sincosf(6.28318530717958647692f * f, &sn, &cs);
            const float amp = in ? fmaf(u, fmaf(u, a2, a1), a0) : 0.f;
            acc[j].x = fmaf(cs, amp, acc[j].x);
            acc[j].y = fmaf(sn, amp, acc[j].y);
          }
        }
      } else {
        const float ddx = (float)wx * dpx;
        const float dx2 = ddx * ddx;
#pragma unroll
        for (int j = 0; j < kRows; ++j) {
          const int wy = wy0 + 4 * j;
          if ((unsigned)(v0 + 4 * j) < (unsigned)vlim) {
            const float ddy = (float)wy * dpx;
            const float2 v = wrp_term_f32(fmaf(ddy, ddy, dx2), q, kf);
            acc[j].x += v.x;
            acc[j].y += v.y;
          }
        }
      }
    }
  }
  if (X >= g.nx) return;
#pragma unroll
  for (int j = 0; j < kRows; ++j) {
    const int Y = Y0 + r0 + 4 * j;
    if (Y < g.ny) {
      float2* d = wrp + (size_t)Y * g.nx + X;
      float2 v = *d;
      v.x += acc[j].x;
      v.y += acc[j].y;
      *d = v;
    }
  }
}

// ---- MATLAB fn_wrp (fn_wrp.m:13-36, WRP_matlab_ver 1.0) ----------------------
// Per point: dz = z_wrp - z, N = round(|lambda dz / dp^2 / 2| + 0.5) * 2 - 1
// (odd), centre (round(x/dp) + (res-1)/2, round(y/dp) + (res-1)/2) (MATLAB
// 1-based), sub-hologram exp(i phase) exp(i k r) / r with r = sign(dz)
// sqrt(dz^2 + xr^2 + yr^2) over the N x N offsets (a - (N-1)/2) dp; the
// first index follows x.  Window pixels outside the res x res plane are
// dropped; points with dz = 0 (r = 0) are skipped.  Each block takes whole
// points and adds the part of the window inside the plane with atomics.
struct WrpMGeom { int res; double dp, lambda, z; };

__device__ __forceinline__ double mround(double x) { return x < 0 ? -floor(-x + 0.5) : floor(x + 0.5); }

template <typename R>
__global__ void __launch_bounds__(256) wrp_matlab_kernel(WrpMGeom g, const double* __restrict__ xyz,
                                                        const double* __restrict__ phase, int n,
                                                        typename cplx_of<R>::type* __restrict__ holo) {
  const double two_pi = 6.283185307179586476925286766559;
  const double k = two_pi / g.lambda;
  const long long res = g.res;
  for (int o = blockIdx.x; o < n; o += gridDim.x) {
    const double px = xyz[3 * o], py = xyz[3 * o + 1], pz = xyz[3 * o + 2];
    const double dz = g.z - pz;
    if (dz == 0.0) continue;
    const double nd = mround(fabs(g.lambda * dz / (g.dp * g.dp) / 2.0) + 0.5) * 2.0 - 1.0;
    if (!(nd >= 1.0) || nd > 4.0e9) continue;
    const long long N = (long long)nd;
    const double lim = 4.0e18;
    const long long cx = (long long)fmin(fmax(mround(px / g.dp), -lim), lim) + (res - 1) / 2;
    const long long cy = (long long)fmin(fmax(mround(py / g.dp), -lim), lim) + (res - 1) / 2;
    // plane row i takes window row a = i + a0, a in [0, N)
    const long long a0 = (N + 1) / 2 - cx, b0 = (N + 1) / 2 - cy;
    const long long i_lo = a0 < 0 ? -a0 : 0, i_hi = N - a0 < res ? N - a0 : res;
    const long long j_lo = b0 < 0 ? -b0 : 0, j_hi = N - b0 < res ? N - b0 : res;
    if (i_lo >= i_hi || j_lo >= j_hi) continue;
    const int h = (int)(i_hi - i_lo), w = (int)(j_hi - j_lo);
    const double ph0 = phase ? phase[o] : 0.0;
    const double sg = dz > 0.0 ? 1.0 : -1.0, adz = fabs(dz);
    const long long half = (N - 1) / 2;
    // FP32: sign(dz) k |r| + ph = sign(dz) (k|dz| + k rho^2 / (|r| + |dz|)) + ph, constant part reduced in FP64
    double base = sg * k * adz + ph0;
    base -= two_pi * rint(base / two_pi);
    const float basef = (float)base, kf = (float)k, adzf = (float)adz, sgf = (float)sg, dpf = (float)g.dp;
    for (int e = threadIdx.x; e < h * w; e += blockDim.x) {
      const int ii = e / w, jj = e - ii * w;
      const long long i = i_lo + ii, j = j_lo + jj;
      const long long a = i + a0 - half, b = j + b0 - half;      // offsets from the window centre
      typename cplx_of<R>::type v;
      if constexpr (sizeof(R) == 8) {
        const double xr = (double)a * g.dp, yr = (double)b * g.dp;
        const double r = sg * sqrt(dz * dz + xr * xr + yr * yr);
        double sn, cs;
        sincos(k * r + ph0, &sn, &cs);
        v = mk(cs / r, sn / r);
      } else {
        const float xr = (float)a * dpf, yr = (float)b * dpf;
        const float rho2 = fmaf(xr, xr, yr * yr);
        const float ar = sqrtf(fmaf(adzf, adzf, rho2));
        float ph = fmaf(sgf * kf, rho2 / (ar + adzf), basef);
        float sn, cs;
        sincosf(ph, &sn, &cs);
        const float inv = sgf / ar;
        v = mk(cs * inv, sn * inv);
      }
      typename cplx_of<R>::type* d = holo + i * res + j;
      atomicAdd(&d->x, v.x);
      atomicAdd(&d->y, v.y);
    }
  }
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
  const int tiles_x = (p->nx + kWrpTile - 1) / kWrpTile, tiles_y = (p->ny + kWrpTile - 1) / kWrpTile;
  const int span = p->window > 0 ? (2 * p->window + kWrpTile - 1) / kWrpTile + 1 : 0;  // tiles per axis a window touches
  const size_t cap = (size_t)n_points * std::min(span, tiles_x) * std::min(span, tiles_y);
  if (p->window > 0 && p->window < (1 << 28) && cap < (size_t)INT32_MAX) {
    // fixed windows: binned, tiled accumulation
    const int ntiles = tiles_x * tiles_y;
    void* ptr;
    const size_t off_cnt = ((size_t)n_points * sizeof(WrpPt) + 255) & ~(size_t)255;
    const size_t off_start = off_cnt + (((size_t)ntiles * 4 + 255) & ~(size_t)255);
    const size_t off_cur = off_start + (((size_t)(ntiles + 1) * 4 + 255) & ~(size_t)255);
    const size_t off_list = off_cur + (((size_t)ntiles * 4 + 255) & ~(size_t)255);
    OH_TRY(scratch(ctx, "wrp.bins", off_list + cap * sizeof(int), &ptr));
    char* base = (char*)ptr;
    WrpPt* pts = (WrpPt*)base;
    int* cnt = (int*)(base + off_cnt);
    int* start = (int*)(base + off_start);
    int* cur = (int*)(base + off_cur);
    int* list = (int*)(base + off_list);
    KernelTimer kt(ctx, "wrp_accumulate", st);
    OH_CUDA_TRY(cudaMemsetAsync(cnt, 0, (size_t)ntiles * 4, st));
    const int g1 = std::min((n_points + 255) / 256, 152 * 8);
    wrp_prep<<<g1, 256, 0, st>>>(g, xyz, n_points, pts, cnt, tiles_x);
    OH_LAUNCH_CHECK();
    wrp_scan<<<1, 1024, 0, st>>>(cnt, start, cur, ntiles);
    OH_LAUNCH_CHECK();
    wrp_fill<<<g1, 256, 0, st>>>(g, pts, n_points, cur, list, tiles_x);
    OH_LAUNCH_CHECK();
    if (prec == OH_FP64) wrp_tile<double><<<ntiles, 256, 0, st>>>(g, pts, start, list, tiles_x, (double2*)wrp);
    else wrp_tile_f32<<<ntiles, 256, 0, st>>>(g, pts, start, list, tiles_x, (float2*)wrp);
    OH_LAUNCH_CHECK();
    return OH_OK;
  }
  const int grid = std::min(n_points, 152 * 32);
  KernelTimer kt(ctx, "wrp_accumulate", st);
  if (prec == OH_FP64) wrp_accumulate_kernel<double><<<grid, 256, 0, st>>>(g, xyz, n_points, (double2*)wrp);
  else wrp_accumulate_kernel<float><<<grid, 256, 0, st>>>(g, xyz, n_points, (float2*)wrp);
  OH_LAUNCH_CHECK();
  return OH_OK;
}

oh_status oh_wrp_matlab(oh_ctx* ctx, oh_precision prec, int res, double pitch, double lambda, double z_wrp,
                        const double* xyz, const double* phase, int n_points, void* holo, void* stream) {
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  CallScope cs(ctx, st);
  OH_TRY(cs.status());
  if (res < 1 || !(pitch > 0) || !(lambda > 0)) return fail(OH_ERR_INVALID_ARG, "bad fn_wrp parameters");
  if (n_points < 0 || (n_points > 0 && !xyz) || !holo) return fail(OH_ERR_INVALID_ARG, "bad fn_wrp buffers");
  if (n_points == 0) return OH_OK;
  WrpMGeom g{res, pitch, lambda, z_wrp};
  KernelTimer kt(ctx, "wrp_matlab", st);
  const int grid = std::min(n_points, 152 * 16);
  if (prec == OH_FP64) wrp_matlab_kernel<double><<<grid, 256, 0, st>>>(g, xyz, phase, n_points, (double2*)holo);
  else wrp_matlab_kernel<float><<<grid, 256, 0, st>>>(g, xyz, phase, n_points, (float2*)holo);
  OH_LAUNCH_CHECK();
  return OH_OK;
}

}  // extern "C"
