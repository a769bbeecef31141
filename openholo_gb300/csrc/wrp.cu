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
#include <cuda_bf16.h>
#include <cmath>
#include <cstdlib>
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
// enough (series >= 1), the polynomial coefficients of the series evaluation
// below in u = rho^2 / dz^2 = ux + uy, ux = (wx sx)^2, uy = (wy sx)^2,
// sx = dp / |dz|.  series = 2 marks windows that are also separable to
// within the bounds of the tensor-core form (wrp_tc):
//   e^{2 pi i phase} amp = a0 e^{2 pi i (base_t + fy)} Ay  e^{2 pi i fx} Ax  (1 + i kappa ux uy),
//   f(u) = u (c1 + u (c2 + u c3)),  A(u) = 1 + u (alpha + u beta),  kappa = 2 pi 2 c2.
struct WrpPt {
  int tx, ty, w, series;
  float base, adz, sgn, sx;
  float base_t, c1, c2, c3;          // phase in turns: base_t + u (c1 + u (c2 + u c3))
  float a0c, a1c, a2c, kappa;        // amplitude: a0c + u (a1c + u a2c); cross-term factor (rad)
  double dz;
  float alpha, beta;                 // per-axis amplitude factors: a1c / a0c, a2c / a0c
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
  // FP64 only for the phase reduction; the rest in FP32 (FP64 is a small
  // fraction of FP32 throughput here)
  const double kdz = kd * fabs(dz);
  const double turns = kdz * 0.15915494309189533576888376337251;      // k|dz| / (2 pi)
  const double tfrac = turns - rint(turns);
  o->base = (float)(two_pi * tfrac);
  // Series form: with u = rho^2 / dz^2 and t = sqrt(1 + u) - 1 = u (1/2 - u/8 + u^2/16) + O(5 u^4 / 128),
  //   sgn k|r| / (2 pi) = sgn turns (1 + t),  turns = k|dz| / (2 pi),
  //   1 / (sgn |r| + 0.05) = (1 / a0) / (1 + e),  a0 = sgn |dz| + 0.05,  e = ea t,  ea = sgn |dz| / a0,
  //   1 / (1 + e) = 1 - ea u / 2 + (ea / 8 + ea^2 / 4) u^2 - (ea / 16 + ea^2 / 8 + ea^3 / 8) u^3 + ...,
  // used when the dropped terms stay below 1e-6 rad (phase) and 1e-8 relative
  // (amplitude) over the whole window.
  const float adz = (float)fabs(dz), sg = dz > 0.0 ? 1.f : -1.f;
  const float a0 = sg * adz + 0.05f;
  const float rho2max = 2.f * (float)g.fixed_w * (float)g.fixed_w * dpx * dpx;
  const float umax = adz > 0.f ? rho2max / (adz * adz) : 1.f;
  const float ea = fabsf(a0) > 1e-6f ? sg * adz / a0 : 0.f;
  const float aea = fabsf(ea);
  const float u3 = umax * umax * umax;
  const float kdzf = (float)kdz;
  o->series = (adz > 0.f && fabsf(a0) > 1e-6f && umax < 0.05f && kdzf * (5.f / 128.f) * umax * u3 < 1e-6f &&
               (aea / 16.f + aea * aea / 8.f + aea * aea * aea / 8.f) * u3 < 1e-8f) ? 1 : 0;
  const float st = (float)(dz > 0.0 ? turns : -turns);               // sgn turns; the c's are its exact scalings
  o->base_t = (float)(dz > 0.0 ? tfrac : -tfrac);
  o->c1 = st * 0.5f;
  o->c2 = st * -0.125f;
  o->c3 = st * 0.0625f;
  o->sx = adz > 0.f ? dpx / adz : 0.f;
  const float ia0 = fabsf(a0) > 1e-6f ? 1.f / a0 : 0.f;
  o->a0c = ia0;
  o->a1c = -ia0 * ea * 0.5f;
  o->a2c = ia0 * (ea * 0.125f + ea * ea * 0.25f);
  // separable form: the dropped terms at the window corner (ux = uy = (w sx)^2)
  //   phase cross term to second order (kappa ux uy)^2 / 2, the c3 cross terms
  //   2 pi 3 c3 ux uy (ux + uy), the amplitude cross term (alpha^2 - 2 beta) ux uy
  const float two_pi_f = 6.28318530717958647692f;
  const float al = -ea * 0.5f, be = ea * 0.125f + ea * ea * 0.25f;
  const float kap = two_pi_f * 2.f * o->c2;
  const float uc = adz > 0.f ? (float)g.fixed_w * (float)g.fixed_w * dpx * dpx / (adz * adz) : 1.f;
  const float t1 = kap * uc * uc, t2 = two_pi_f * 3.f * fabsf(o->c3) * uc * uc * 2.f * uc;
  const float t3 = fabsf(al * al - 2.f * be) * uc * uc;
  if (o->series && g.fixed_w > 0 && 0.5f * t1 * t1 < 3e-5f && t2 < 1e-5f && t3 < 1e-6f) o->series = 2;
  o->kappa = kap;
  o->alpha = al;
  o->beta = be;
}

// Two binnings share one count / start / list layout: 64 x 64 tiles for the
// direct tile kernels (bins [0, nd)) and, for points the tensor-core form
// takes (series == 2 and use_tc), 64-column x 128-row regions (bins
// [nd, nd + regions)).
constexpr int kTcW = 64, kTcH = 128;

struct WrpBins {
  int tiles_x, nd;          // direct tiles across, direct bin count
  int regions_x;            // tensor regions across
  int use_tc;
};

// bin index range [t0, t1] along one axis for the window [c - w, c + w) clipped to [0, n)
__device__ __forceinline__ bool wrp_bin_range(int c, int w, int n, int size, int* t0, int* t1) {
  const int lo = max(c - w, 0), hi = min(c + w, n);
  if (lo >= hi) return false;
  *t0 = lo / size;
  *t1 = (hi - 1) / size;
  return true;
}

// calls f(bin) for every bin the point's window touches
template <class F>
__device__ __forceinline__ void wrp_for_bins(const WRPGeom& g, const WrpBins& b, const WrpPt& q, F f) {
  const bool tc = b.use_tc && q.series == 2;
  const int bw = tc ? kTcW : kWrpTile, bh = tc ? kTcH : kWrpTile;
  int x0, x1, y0, y1;
  if (!wrp_bin_range(q.tx, q.w, g.nx, bw, &x0, &x1) || !wrp_bin_range(q.ty, q.w, g.ny, bh, &y0, &y1)) return;
  for (int ty = y0; ty <= y1; ++ty)
    for (int tx = x0; tx <= x1; ++tx) f(tc ? b.nd + ty * b.regions_x + tx : ty * b.tiles_x + tx);
}

// Bin counters and cursors are replicated kWrpRep times (replicas of one bin
// a whole counter array apart): about 600 points share a plane-region
// counter, and the replicas split that contention.  The replica of point k
// is (k / 256) mod kWrpRep, so runs of consecutive points stay together in a
// bin's list (the window kernels read the point records in list order, and
// records of nearby points share cache lines).
constexpr int kWrpRep = 8;
__device__ __forceinline__ int wrp_replica(int k) { return (k >> 8) & (kWrpRep - 1); }

__global__ void wrp_prep(WRPGeom g, const double* __restrict__ xyz, int n, WrpPt* __restrict__ pts,
                         int* __restrict__ count, int nbins, WrpBins bins) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    WrpPt q;
    wrp_point(g, xyz, k, &q);
    pts[k] = q;
    int* c = count + (size_t)wrp_replica(k) * nbins;
    wrp_for_bins(g, bins, q, [&](int t) { atomicAdd(&c[t], 1); });
  }
}

// Exclusive scan of the replicated counts in (bin, replica) order, single
// block: cursor[r * n + t] = first list slot of replica r of bin t,
// start[t] = first slot of bin t, start[n] = total.
__global__ void wrp_scan(const int* __restrict__ count, int* __restrict__ start, int* __restrict__ cursor, int n) {
  __shared__ int part[1024];
  const int m = n * kWrpRep;
  const int per = (m + blockDim.x - 1) / blockDim.x;
  const int b = threadIdx.x * per, e = min(b + per, m);
  auto at = [&](int i) { return (size_t)(i % kWrpRep) * n + i / kWrpRep; };   // i = t kWrpRep + r
  int sum = 0;
  for (int i = b; i < e; ++i) sum += count[at(i)];
  part[threadIdx.x] = sum;
  __syncthreads();
  for (int off = 1; off < blockDim.x; off <<= 1) {
    int v = threadIdx.x >= off ? part[threadIdx.x - off] : 0;
    __syncthreads();
    part[threadIdx.x] += v;
    __syncthreads();
  }
  int run = part[threadIdx.x] - sum;
  for (int i = b; i < e; ++i) {
    if (i % kWrpRep == 0) start[i / kWrpRep] = run;
    cursor[at(i)] = run;
    run += count[at(i)];
  }
  if (threadIdx.x == blockDim.x - 1) start[n] = part[threadIdx.x];
}

__global__ void wrp_fill(WRPGeom g, const WrpPt* __restrict__ pts, int n, int* __restrict__ cursor, int nbins,
                         int* __restrict__ list, WrpBins bins) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const WrpPt q = pts[k];
    int* c = cursor + (size_t)wrp_replica(k) * nbins;
    wrp_for_bins(g, bins, q, [&](int t) { list[atomicAdd(&c[t], 1)] = k; });
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
  if (b == e) return;                               // no window reaches this tile
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

// ---- tensor-core form of the fixed-window sum (series == 2 points) ---------
// Over a 128-row x 64-column plane region, the separable windows make the sum
//   W[y][x] = sum_p L0_p[y] R0_p[x] + L1_p[y] R1_p[x],
//   L0 = a0 e^{2 pi i (base_t + f(uy))} A(uy),  L1 = uy L0,
//   R0 = e^{2 pi i f(ux)} A(ux),                R1 = i kappa ux R0
// (zero outside each window) a complex matrix product with K = 2 per point.
// Embedded in reals as in the point-sum GEMM (K column 2k / 2k+1 = Re / Im of
// term k; B rows 2x / 2x+1 give Re / Im of column x), C = A B^T is the
// region's complex64 sum, M = 128, N = 128, K = 4 per point.  BF16 high and
// low parts, three products (Ahi Bhi + Ahi Blo + Alo Bhi), FP32 in TMEM.
//
// One CTA per region, 288 threads.  Warps 0-7 write the operands of 8 points
// (K = 32) per stage straight into shared memory, in the layout a TMA load
// with 64-byte swizzle would give, then arrive on the stage's full barrier:
// thread t takes point slot t & 7, A rows (t >> 3) + 32 m (m < 4) and B
// columns (t >> 3) + 32 m (m < 2), so its swizzled offsets are fixed.  Warp 8
// issues tcgen05.mma (M 128, N 128, K 16) and releases stages with
// tcgen05.commit; warps 4-7 read the accumulator (tcgen05.ld) and add the
// region into the plane.  Waits are bounded: on timeout the CTA sets the
// device error word, skips the add, waits for its MMAs and frees TMEM.
namespace tcw {

constexpr int kRows = kTcH, kCols = kTcW;             // region
constexpr int kBK = 32, kPts = kBK / 4, kStages = 2;
constexpr int kTile = 128 * kBK * 2;                   // 8 KB: 128 rows x 32 BF16
constexpr int kStageBytes = 4 * kTile;                 // Ahi, Alo, Bhi, Blo
constexpr int kTmemCols = 128;
constexpr int kProducerWarps = 8, kThreads = 32 * kProducerWarps + 32;   // + the MMA warp
constexpr int kSmemBytes = kStages * kStageBytes + 1024 + 256;
constexpr long long kWaitCycles = 2000000000LL;

__device__ __forceinline__ uint32_t su32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mb_init(uint64_t* b, uint32_t n) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(su32(b)), "r"(n) : "memory");
}
__device__ __forceinline__ void mb_arrive(uint64_t* b) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(su32(b)) : "memory");
}
__device__ __forceinline__ bool mb_try(uint64_t* b, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(su32(b)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ bool mb_wait(uint64_t* b, uint32_t parity) {
  const long long t0 = clock64();
  while (!mb_try(b, parity)) {
    if (clock64() - t0 > kWaitCycles) return false;
  }
  return true;
}
// K-major tile, rows of 32 BF16 (64 bytes), 64-byte swizzle, 8-row atoms 512 bytes apart
__device__ __forceinline__ uint64_t sw_desc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFF) >> 4);
  d |= (uint64_t)1 << 16;
  d |= (uint64_t)((8 * kBK * 2) >> 4) << 32;
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)4 << 61;
  return d;
}
// kind::f16, D FP32, A and B BF16, K-major, N = 128, M = 128
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(128 >> 3) << 17) |
                            ((uint32_t)(128 >> 4) << 24);
__device__ __forceinline__ void umma(uint32_t tmem, uint64_t a, uint64_t b, uint32_t accum) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(tmem),
      "l"(a), "l"(b), "r"(kIdesc), "r"(accum)
      : "memory");
}
__device__ __forceinline__ void umma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(su32(bar))
               : "memory");
}
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t* r) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
      "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// Byte offset of point slot j (4 BF16 = 8 bytes) in row r of a [128][32] BF16
// tile with 64-byte swizzle: 16-byte chunk c of the row lands at c ^ ((r >> 1) & 3).
__device__ __forceinline__ int sw_off(int r, int j) {
  return r * 64 + (((j >> 1) ^ ((r >> 1) & 3)) << 4) + ((j & 1) << 3);
}

// BF16 high / low parts of four values, written as 8 bytes each
__device__ __forceinline__ void put4(unsigned char* hi, unsigned char* lo, int off, float a, float b, float c,
                                     float d) {
  const __nv_bfloat162 h0 = __floats2bfloat162_rn(a, b), h1 = __floats2bfloat162_rn(c, d);
  const __nv_bfloat162 l0 = __floats2bfloat162_rn(a - __low2float(h0), b - __high2float(h0));
  const __nv_bfloat162 l1 = __floats2bfloat162_rn(c - __low2float(h1), d - __high2float(h1));
  uint2 vh, vl;
  vh.x = *reinterpret_cast<const uint32_t*>(&h0);
  vh.y = *reinterpret_cast<const uint32_t*>(&h1);
  vl.x = *reinterpret_cast<const uint32_t*>(&l0);
  vl.y = *reinterpret_cast<const uint32_t*>(&l1);
  *reinterpret_cast<uint2*>(hi + off) = vh;
  *reinterpret_cast<uint2*>(lo + off) = vl;
}

__device__ __forceinline__ float frac_turns(float f) { return f - rintf(f); }

// BF16 high / low parts of (a, b, c, d) packed as two bf16x2 words each
struct Split4 { uint32_t h01, h23, l01, l23; };
__device__ __forceinline__ Split4 split4(float a, float b, float c, float d) {
  const __nv_bfloat162 h0 = __floats2bfloat162_rn(a, b), h1 = __floats2bfloat162_rn(c, d);
  const __nv_bfloat162 l0 = __floats2bfloat162_rn(a - __low2float(h0), b - __high2float(h0));
  const __nv_bfloat162 l1 = __floats2bfloat162_rn(c - __low2float(h1), d - __high2float(h1));
  Split4 r;
  r.h01 = *reinterpret_cast<const uint32_t*>(&h0);
  r.h23 = *reinterpret_cast<const uint32_t*>(&h1);
  r.l01 = *reinterpret_cast<const uint32_t*>(&l0);
  r.l23 = *reinterpret_cast<const uint32_t*>(&l1);
  return r;
}

// the fields of a point record the operand builders use (held in registers)
struct Rec {
  int tx, ty, w;
  float sx, base_t, c1, c2, c3, a0c, alpha, beta, kappa;
};
// the point list entry of slot k (-1 past the region's end)
__device__ __forceinline__ int list_at(const int* __restrict__ list, int k, int e) {
  return k < e ? __ldg(list + k) : -1;
}
__device__ __forceinline__ Rec load_rec_at(const WrpPt* __restrict__ pts, int idx) {
  Rec r;
  if (idx >= 0) {
    const WrpPt* q = pts + idx;
    r.tx = q->tx; r.ty = q->ty; r.w = q->w;
    r.sx = q->sx; r.base_t = q->base_t; r.c1 = q->c1; r.c2 = q->c2; r.c3 = q->c3;
    r.a0c = q->a0c; r.alpha = q->alpha; r.beta = q->beta; r.kappa = q->kappa;
  } else {
    r.tx = r.ty = 0; r.w = 0;                       // empty slot: every item writes zeros
    r.sx = r.base_t = r.c1 = r.c2 = r.c3 = r.a0c = r.alpha = r.beta = r.kappa = 0.f;
  }
  return r;
}
__device__ __forceinline__ Rec load_rec(const WrpPt* __restrict__ pts, const int* __restrict__ list, int k, int e) {
  Rec r;
  if (k < e) {
    const WrpPt* q = pts + __ldg(list + k);
    r.tx = q->tx; r.ty = q->ty; r.w = q->w;
    r.sx = q->sx; r.base_t = q->base_t; r.c1 = q->c1; r.c2 = q->c2; r.c3 = q->c3;
    r.a0c = q->a0c; r.alpha = q->alpha; r.beta = q->beta; r.kappa = q->kappa;
  } else {
    r.tx = r.ty = 0; r.w = 0;                       // empty slot: every item writes zeros
    r.sx = r.base_t = r.c1 = r.c2 = r.c3 = r.a0c = r.alpha = r.beta = r.kappa = 0.f;
  }
  return r;
}

}  // namespace tcw

__global__ void __launch_bounds__(tcw::kThreads, 3) wrp_tc(WRPGeom g, const WrpPt* __restrict__ pts,
                                                           const int* __restrict__ start,
                                                           const int* __restrict__ list, int regions_x,
                                                           float2* __restrict__ wrp, int* err) {
  using namespace tcw;
  extern __shared__ unsigned char smem_raw[];
  const uint32_t raw = su32(smem_raw);
  unsigned char* base = smem_raw + (((raw + 1023u) & ~1023u) - raw);
  uint64_t* bars = reinterpret_cast<uint64_t*>(base + kStages * kStageBytes);
  uint64_t* full = bars;                 // [kStages], one arrival per producer warp
  uint64_t* empty = bars + kStages;      // [kStages], tcgen05.commit
  uint64_t* done = bars + 2 * kStages;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2 * kStages + 1);
  int* abort_flag = reinterpret_cast<int*>(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int region = blockIdx.x;
  const int X0 = (region % regions_x) * kCols, Y0 = (region / regions_x) * kRows;
  const int b = start[region], e = start[region + 1];
  if (b == e) return;                    // uniform: no window reaches this region
  const int npts = e - b;
  const int nst = (npts + kPts - 1) / kPts;

  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) { mb_init(&full[s], kProducerWarps); mb_init(&empty[s], 1); }
    mb_init(done, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(tmem_slot)),
                 "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;

  if (warp < kProducerWarps) {
    // producers: point slot j, A rows rb + 32 m, B columns rb + 32 m; the
    // record of this stage's point sits in registers, the next stage's is
    // loaded while this stage is built
    const int pt = threadIdx.x;
    const int j = pt & (kPts - 1), rb = pt >> 3;
    int offA[4], YA[4], offB0[2], offB1[2], XB[2];
#pragma unroll
    for (int m = 0; m < 4; ++m) { offA[m] = sw_off(rb + 32 * m, j); YA[m] = Y0 + rb + 32 * m; }
#pragma unroll
    for (int m = 0; m < 2; ++m) {
      offB0[m] = sw_off(2 * (rb + 32 * m), j);
      offB1[m] = sw_off(2 * (rb + 32 * m) + 1, j);
      XB[m] = X0 + rb + 32 * m;
    }
    // two-level prefetch: the list entry two stages ahead, the record of the
    // next stage (its address known a stage in advance), so the dependent
    // list -> record loads are not on one stage's critical path
    Rec q = load_rec(pts, list, b + j, e);
    int idx_next = list_at(list, b + kPts + j, e);
    for (int it = 0; it < nst; ++it) {
      const int s = it % kStages;
      const uint32_t ph = (uint32_t)((it / kStages) & 1);
      bool ok = true;
      if (lane == 0) ok = mb_wait(&empty[s], ph ^ 1u) && !*((volatile int*)abort_flag);
      ok = __shfl_sync(0xffffffffu, ok ? 1 : 0, 0) != 0;
      if (!ok) {
        if (lane == 0) atomicExch(abort_flag, 1);
        break;
      }
      unsigned char* sAh = base + s * kStageBytes;
      unsigned char* sAl = sAh + kTile;
      unsigned char* sBh = sAh + 2 * kTile;
      unsigned char* sBl = sAh + 3 * kTile;
      const Rec qn = load_rec_at(pts, idx_next);
      idx_next = list_at(list, b + (it + 2) * kPts + j, e);
      // A: branch-free, rows outside the window (or the plane) get amplitude 0
#pragma unroll
      for (int m = 0; m < 4; ++m) {
        const int wy = YA[m] - q.ty;
        const bool in = YA[m] < g.ny && (unsigned)(wy + q.w) < (unsigned)(2 * q.w);
        const float ys = (float)wy * q.sx, uy = ys * ys;
        const float f = frac_turns(fmaf(uy, fmaf(uy, fmaf(uy, q.c3, q.c2), q.c1), q.base_t));
        float sn, cs;
        __sincosf(6.28318530717958647692f * f, &sn, &cs);
        const float amp = in ? q.a0c * fmaf(uy, fmaf(uy, q.beta, q.alpha), 1.f) : 0.f;
        const float v0 = amp * cs, v1 = amp * sn;
        put4(sAh, sAl, offA[m], v0, v1, uy * v0, uy * v1);
      }
      // B: R1 = i kappa ux R0; row 2x: (R0x, -R0y, R1x, -R1y), row 2x+1:
      // (R0y, R0x, R1y, R1x), from one split by swapping halves and flipping signs
#pragma unroll
      for (int m = 0; m < 2; ++m) {
        const int wx = XB[m] - q.tx;
        const bool in = XB[m] < g.nx && (unsigned)(wx + q.w) < (unsigned)(2 * q.w);
        const float xs = (float)wx * q.sx, ux = xs * xs;
        const float f = frac_turns(ux * fmaf(ux, fmaf(ux, q.c3, q.c2), q.c1));
        float sn, cs;
        __sincosf(6.28318530717958647692f * f, &sn, &cs);
        const float amp = in ? fmaf(ux, fmaf(ux, q.beta, q.alpha), 1.f) : 0.f;
        const float r0x = amp * cs, r0y = amp * sn;
        const float kx = q.kappa * ux;
        const Split4 v = split4(r0x, r0y, -kx * r0y, kx * r0x);
        const uint32_t neg_hi = 0x80000000u;               // sign of the second BF16 of a pair
        *reinterpret_cast<uint2*>(sBh + offB0[m]) = make_uint2(v.h01 ^ neg_hi, v.h23 ^ neg_hi);
        *reinterpret_cast<uint2*>(sBl + offB0[m]) = make_uint2(v.l01 ^ neg_hi, v.l23 ^ neg_hi);
        *reinterpret_cast<uint2*>(sBh + offB1[m]) = make_uint2(__byte_perm(v.h01, 0, 0x1032), __byte_perm(v.h23, 0, 0x1032));
        *reinterpret_cast<uint2*>(sBl + offB1[m]) = make_uint2(__byte_perm(v.l01, 0, 0x1032), __byte_perm(v.l23, 0, 0x1032));
      }
      // generic-proxy writes -> visible to the tensor core's async proxy
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      __syncwarp();
      if (lane == 0) mb_arrive(&full[s]);
      q = qn;
    }
  } else if (threadIdx.x == 32 * kProducerWarps) {
    // MMA issuer
    for (int it = 0; it < nst; ++it) {
      const int s = it % kStages;
      const uint32_t ph = (uint32_t)((it / kStages) & 1);
      if (!mb_wait(&full[s], ph) || *((volatile int*)abort_flag)) {
        atomicExch(abort_flag, 1);
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      unsigned char* st0 = base + s * kStageBytes;
      const uint64_t ah = sw_desc(su32(st0)), al = sw_desc(su32(st0 + kTile));
      const uint64_t bh = sw_desc(su32(st0 + 2 * kTile)), bl = sw_desc(su32(st0 + 3 * kTile));
#pragma unroll
      for (int kk = 0; kk < kBK / 16; ++kk) {
        const uint64_t adv = (uint64_t)((kk * 32) >> 4);
        umma(tmem, ah + adv, bh + adv, (it | kk) ? 1u : 0u);
        umma(tmem, ah + adv, bl + adv, 1u);
        umma(tmem, al + adv, bh + adv, 1u);
      }
      umma_commit(&empty[s]);
    }
    umma_commit(done);                   // arrives when every MMA issued above has completed
  }
  // epilogue: warps 4-7 own TMEM lanes 32 (warp - 4) .. + 31 = region rows
  __syncwarp();
  const bool epi = warp >= 4 && warp < 8;
  bool ok_done = true;
  if (epi) ok_done = mb_wait(done, 0);
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const bool good = __syncthreads_and(ok_done && !*((volatile int*)abort_flag));
  if (good && epi) {
    const int r = 32 * (warp - 4) + lane;
    const int Y = Y0 + r;
#pragma unroll 1
    for (int c = 0; c < 2 * kCols / 32; ++c) {
      uint32_t v[32];
      tmem_ld32(tmem + ((uint32_t)(32 * (warp - 4)) << 16) + (uint32_t)(c * 32), v);
      if (Y < g.ny) {
        float2* dst = wrp + (size_t)Y * g.nx + X0 + 16 * c;
#pragma unroll
        for (int q = 0; q < 16; ++q) {
          if (X0 + 16 * c + q < g.nx) {
            float2 o = dst[q];
            o.x += __uint_as_float(v[2 * q]);
            o.y += __uint_as_float(v[2 * q + 1]);
            dst[q] = o;
          }
        }
      }
    }
  } else if (!good && threadIdx.x == 0) {
    atomicOr(err, 4);
  }
  // the MMAs must have finished reading shared memory and TMEM before exit
  if (!good && threadIdx.x == 0) mb_wait(done, 0);
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 1) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
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
  const int regions_x = (p->nx + kTcW - 1) / kTcW, regions_y = (p->ny + kTcH - 1) / kTcH;
  // bins a window touches per axis: direct tiles, tensor regions
  const int span = p->window > 0 ? (2 * p->window + kWrpTile - 1) / kWrpTile + 1 : 0;
  const int span_rx = p->window > 0 ? (2 * p->window + kTcW - 1) / kTcW + 1 : 0;
  const int span_ry = p->window > 0 ? (2 * p->window + kTcH - 1) / kTcH + 1 : 0;
  const size_t cap_d = (size_t)std::min(span, tiles_x) * std::min(span, tiles_y);
  const size_t cap_t = (size_t)std::min(span_rx, regions_x) * std::min(span_ry, regions_y);
  const size_t cap = (size_t)n_points * std::max(cap_d, cap_t);
  if (p->window > 0 && p->window < (1 << 28) && cap < (size_t)INT32_MAX) {
    // fixed windows: binned, tiled accumulation; in FP32 the separable points
    // go to the tensor-core form (OH_WRP_ENGINE=direct keeps every point on
    // the direct tile kernel)
    bool use_tc = prec != OH_FP64;
    if (const char* ev = std::getenv("OH_WRP_ENGINE")) use_tc = use_tc && std::strcmp(ev, "direct") != 0;
    if (use_tc) {
      int dev = 0, major = 0, minor = 0;
      OH_CUDA_TRY(cudaGetDevice(&dev));
      OH_CUDA_TRY(cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev));
      OH_CUDA_TRY(cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev));
      use_tc = major == 10 && minor == 3;
    }
    const int ntiles = tiles_x * tiles_y, nregions = regions_x * regions_y;
    const int nbins = ntiles + (use_tc ? nregions : 0);
    void* ptr;
    const size_t off_cnt = ((size_t)n_points * sizeof(WrpPt) + 255) & ~(size_t)255;
    const size_t off_start = off_cnt + (((size_t)nbins * kWrpRep * 4 + 255) & ~(size_t)255);
    const size_t off_cur = off_start + (((size_t)(nbins + 1) * 4 + 255) & ~(size_t)255);
    const size_t off_list = off_cur + (((size_t)nbins * kWrpRep * 4 + 255) & ~(size_t)255);
    OH_TRY(scratch(ctx, "wrp.bins", off_list + cap * sizeof(int), &ptr));
    char* base = (char*)ptr;
    WrpPt* pts = (WrpPt*)base;
    int* cnt = (int*)(base + off_cnt);
    int* start = (int*)(base + off_start);
    int* cur = (int*)(base + off_cur);
    int* list = (int*)(base + off_list);
    const WrpBins bins{tiles_x, ntiles, regions_x, use_tc ? 1 : 0};
    if (use_tc)
      OH_CUDA_TRY(cudaFuncSetAttribute(wrp_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, tcw::kSmemBytes));
    KernelTimer kt(ctx, "wrp_accumulate", st);
    OH_CUDA_TRY(cudaMemsetAsync(cnt, 0, (size_t)nbins * kWrpRep * 4, st));
    const int g1 = std::min((n_points + 255) / 256, oh::sm_count() * 8);
    wrp_prep<<<g1, 256, 0, st>>>(g, xyz, n_points, pts, cnt, nbins, bins);
    OH_LAUNCH_CHECK();
    wrp_scan<<<1, 1024, 0, st>>>(cnt, start, cur, nbins);
    OH_LAUNCH_CHECK();
    wrp_fill<<<g1, 256, 0, st>>>(g, pts, n_points, cur, nbins, list, bins);
    OH_LAUNCH_CHECK();
    if (use_tc) {
      KernelTimer kt2(ctx, "wrp_tc", st);
      wrp_tc<<<nregions, tcw::kThreads, tcw::kSmemBytes, st>>>(g, pts, start + ntiles, list, regions_x,
                                                              (float2*)wrp, ctx->dev_err);
      OH_LAUNCH_CHECK();
    }
    {
      KernelTimer kt3(ctx, "wrp_tile", st);
      if (prec == OH_FP64) wrp_tile<double><<<ntiles, 256, 0, st>>>(g, pts, start, list, tiles_x, (double2*)wrp);
      else wrp_tile_f32<<<ntiles, 256, 0, st>>>(g, pts, start, list, tiles_x, (float2*)wrp);
      OH_LAUNCH_CHECK();
    }
    return OH_OK;
  }
  const int grid = std::min(n_points, oh::sm_count() * 32);
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
  const int grid = std::min(n_points, oh::sm_count() * 16);
  if (prec == OH_FP64) wrp_matlab_kernel<double><<<grid, 256, 0, st>>>(g, xyz, phase, n_points, (double2*)holo);
  else wrp_matlab_kernel<float><<<grid, 256, 0, st>>>(g, xyz, phase, n_points, (float2*)holo);
  OH_LAUNCH_CHECK();
  return OH_OK;
}

}  // extern "C"
