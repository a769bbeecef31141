// Point-cloud hologram: sum over points of a_j exp(i phi_j) per SLM pixel,
//   phi_j = k r_j - k X sin(tx) - k Y sin(ty),  r_j = |(X,Y,0) - (x_j,y_j,z_j)|
// with the KETI geometry of ophGenCghPointCloud (ophgen_pointcloud.cpp:195-249)
// and ophKernelCghPointCloud_cuda (ophgen_pointcloud_gpu.cpp:391-416):
//   X = (col + 0.5) px - Nx px / 2,  Y = Ny py / 2 - (row + 0.5) py,
//   x_j = x sx, y_j = y sy, z_j = z sz + offsetDepth.
// The KETI fringe is Re of the same sum, accumulated into the caller's
// buffer (dst += ...).
//
// FP32 path: k r_j reaches 1e6 rad, far beyond float resolution, so the
// phase is split exactly into FP64-reduced tables plus a small FP32 residual.
// With a per-point anchor distance rb = sqrt(y^2 + z^2) (SLM-centre row),
//   r_y = sqrt(dy^2 + z^2)   (per point and row),
//   r_x = sqrt(dx^2 + rb^2)  (per point and column),
//   k r = k (r_x - rb) - k X sin tx                  table A[point][col]
//       + k r_y        - k Y sin ty                  table B[point][row]
//       + k (r - r_y) - k (r_x - rb)                 FP32 residual
// and, with E = r_y - rb (tabulated per point and row), the residual is
// evaluated without cancellation as
//   -k E dx^2 [(r_x + r) + (r_y + rb)] / ((r + r_y)(r_x + rb)(r_x + r)),
// bounded by about k |E| / 2: a few rad for paraxial scenes, ~1e3 rad for
// the strongly off-axis KETI sample over its full 1 mm SLM.
// FP64 path: the direct formula in double precision.
#include <algorithm>
#include <cmath>
#include <mutex>
#include <vector>
#include "context.h"
#include "fft_kernels.cuh"

namespace oh {

struct PCGeom {
  double k, px, py, hlx, hly, sx, sy, sz, off, stx, sty;
  int nx, ny;
};

constexpr int kPcChunk = 32768;    // points per table chunk
constexpr int kPcTX = 32, kPcTY = 8, kPcPts = 64;

// Per point: x_j, rb, amplitude; per point and column: A, r_x; per point
// and row: B, r_y, E = r_y - rb.  One block per point (grid-stride), so the
// point's FP64 terms are formed once per thread and the table rows are
// written coalesced.
//
// FP64 is slow on this part (about 1/64 of the FP32 rate), so only the large
// phase terms use it.  With d = dx (or dy) and R = rb (or |z|),
//   k (sqrt(d^2 + R^2) - R) = k d^2 / (2R) - k d^4 / (2R (r + R)^2),
// the paraxial part (up to ~1e3 rad; k R up to ~1e6 rad) in FP64, reduced
// mod 2 pi, the remainder in FP32.  The remainder is at most k d^4 / (8 R^3)
// over the point's rows or columns; where that bound reaches 4 rad the point
// keeps the all-FP64 form (strongly off-axis or near scenes).
__global__ void pc_tables(PCGeom g, const float4* __restrict__ pts, int n, float4* __restrict__ prm,
                          float* __restrict__ A, float* __restrict__ RX, float* __restrict__ B,
                          float* __restrict__ RY, float* __restrict__ E) {
  const double two_pi = 6.283185307179586476925286766559;
  const double inv_two_pi = 0.15915494309189533576888376337251;
  for (int j = blockIdx.x; j < n; j += gridDim.x) {
    const float4 p = pts[j];
    const double x = (double)p.x * g.sx, y = (double)p.y * g.sy, z = (double)p.z * g.sz + g.off;
    const double rb = sqrt(y * y + z * z), az = fabs(z);
    if (threadIdx.x == 0) prm[j] = make_float4((float)x, (float)rb, p.w, 0.f);
    const float kf = (float)g.k;
    // x table
    {
      const double X0 = 0.5 * g.px - g.hlx, X1 = ((double)g.nx - 0.5) * g.px - g.hlx;
      const double dm = fmax(fabs(X0 - x), fabs(X1 - x));
      const bool fast = rb > 0.0 && g.k * (dm * dm) * (dm * dm) < 32.0 * rb * rb * rb;
      const double ca = g.k / (2.0 * rb);
      const float rbf = (float)rb;
      for (int c = threadIdx.x; c < g.nx; c += blockDim.x) {
        const double X = ((double)c + 0.5) * g.px - g.hlx;
        const double dx = X - x, dx2 = dx * dx;
        const size_t idx = (size_t)j * g.nx + c;
        if (fast) {
          double ph = fma(ca, dx2, -g.k * X * g.stx);
          ph -= two_pi * rint(ph * inv_two_pi);
          const float rxf = sqrtf((float)(dx2 + rb * rb));
          const float sx = rxf + rbf, d2 = (float)dx2;
          A[idx] = (float)ph - kf * d2 * d2 / (2.f * rbf * sx * sx);
          RX[idx] = rxf;
        } else {
          const double rx = sqrt(dx2 + rb * rb);
          double ph = g.k * (dx2 / (rx + rb)) - g.k * X * g.stx;      // k (r_x - rb) - k X sin tx
          ph -= two_pi * rint(ph / two_pi);
          A[idx] = (float)ph;
          RX[idx] = (float)rx;
        }
      }
    }
    // y table
    {
      const double Y0 = g.hly - 0.5 * g.py, Y1 = g.hly - ((double)g.ny - 0.5) * g.py;
      const double dm = fmax(fabs(Y0 - y), fabs(Y1 - y));
      const bool fast = az > 0.0 && g.k * (dm * dm) * (dm * dm) < 32.0 * az * az * az;
      double kz = g.k * az;
      kz -= two_pi * rint(kz * inv_two_pi);
      const double cb = g.k / (2.0 * az);
      const float azf = (float)az, rbf = (float)rb;
      for (int r = threadIdx.x; r < g.ny; r += blockDim.x) {
        const double Y = g.hly - ((double)r + 0.5) * g.py;
        const double dy = Y - y, dy2 = dy * dy;
        const size_t idx = (size_t)j * g.ny + r;
        if (fast) {
          double ph = kz + fma(cb, dy2, -g.k * Y * g.sty);
          ph -= two_pi * rint(ph * inv_two_pi);
          const float ryf = sqrtf((float)(dy2 + z * z));
          const float sy = ryf + azf, d2 = (float)dy2;
          B[idx] = (float)ph - kf * d2 * d2 / (2.f * azf * sy * sy);
          RY[idx] = ryf;
          E[idx] = (float)((dy - y) * (dy + y)) / (ryf + rbf);           // r_y - rb without cancellation
        } else {
          const double ry = sqrt(dy2 + z * z);
          const double kr = g.k * ry;
          double ph = (kr - two_pi * rint(kr / two_pi)) - g.k * Y * g.sty;
          ph -= two_pi * rint(ph / two_pi);
          B[idx] = (float)ph;
          RY[idx] = (float)ry;
          E[idx] = (float)((dy2 - y * y) / (ry + rb));
        }
      }
    }
  }
}

// A 32 x 16 pixel tile per 128-thread block: thread (tx, ty) owns column tx
// and rows ty + 4 i (i < 4), so each point's column terms (x table, r_x, dx)
// serve four pixels; points streamed through shared memory in chunks.
// (2048 blocks at 1024 x 1024: about two full waves at 7 blocks per SM.)
constexpr int kPcFTY = 4, kPcRows = 4;
constexpr int kPcTR = kPcFTY * kPcRows;    // tile rows

__device__ __forceinline__ float pc_sqrt_approx(float a) {
  float r;
  asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(a));
  return r;
}

__device__ __forceinline__ float pc_rcp_approx(float a) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(a));
  return r;
}

inline dim3 pc_grid_f32(int nx, int ny) { return dim3((nx + kPcTX - 1) / kPcTX, (ny + kPcTR - 1) / kPcTR); }

// sin and cos of two phases in [-pi, pi]: the cosine on the FMA pipe (packed
// two-lane FP32), the sine on the MUFU unit, which also serves the square
// root and the reciprocal; with both on the MUFU unit it bounds the kernel,
// with both on the FMA pipe that pipe does.  cos x = Q(x^2), a degree-6
// polynomial in x^2 fitted here as a near-minimax approximation on [-pi, pi]
// (Lawson-reweighted least squares on Chebyshev nodes); measured with FP32
// Horner evaluation: |error| <= 4.2e-7 over [-pi, pi].
__device__ __forceinline__ void pc_sincos2(float2 x, float2* sn, float2* cs) {
  *sn = make_float2(__sinf(x.x), __sinf(x.y));
  const float2 t = __fmul2_rn(x, x);
  float2 q = make_float2(1.7247606e-09f, 1.7247606e-09f);
  q = __ffma2_rn(q, t, make_float2(-2.7079776e-07f, -2.7079776e-07f));
  q = __ffma2_rn(q, t, make_float2(2.4769966e-05f, 2.4769966e-05f));
  q = __ffma2_rn(q, t, make_float2(-1.3887808e-03f, -1.3887808e-03f));
  q = __ffma2_rn(q, t, make_float2(4.1666489e-02f, 4.1666489e-02f));
  q = __ffma2_rn(q, t, make_float2(-4.9999988e-01f, -4.9999988e-01f));
  *cs = __ffma2_rn(q, t, make_float2(1.f, 1.f));
}

__device__ __forceinline__ float2 f2(float v) { return make_float2(v, v); }

__global__ void __launch_bounds__(kPcTX * kPcFTY) pc_direct_f32(PCGeom g, const float4* __restrict__ prm,
                                                              const float* __restrict__ A, const float* __restrict__ RX,
                                                              const float* __restrict__ B, const float* __restrict__ RY,
                                                              const float* __restrict__ E, int n,
                                                              float2* __restrict__ field, float* __restrict__ fringe,
                                                              int accumulate_field) {
  // per point: column terms [point][column]; row terms [point][ty][i] for
  // tile row ty + kPcFTY i, so a thread reads its four rows with one 16-byte load
  __shared__ float sA[kPcPts][kPcTX];
  __shared__ float sX[kPcPts][kPcTX];
  __shared__ __align__(16) float sB[kPcPts][kPcTR];
  __shared__ __align__(16) float sR[kPcPts][kPcTR];
  __shared__ __align__(16) float sE[kPcPts][kPcTR];
  __shared__ float4 sP[kPcPts];
  static_assert(kPcRows == 4, "four rows per thread: two packed pairs");
  const int tx = threadIdx.x % kPcTX, ty = threadIdx.x / kPcTX;
  const int col = blockIdx.x * kPcTX + tx, row0 = blockIdx.y * kPcTR + ty;
  const float X = (float)(((double)col + 0.5) * g.px - g.hlx);
  const float nk = (float)(-g.k);
  const float inv2pi = 0.15915494309189533577f, two_pi = 6.28318530717958647692f;
  float2 re01 = f2(0.f), im01 = f2(0.f), re23 = f2(0.f), im23 = f2(0.f);
  for (int j0 = 0; j0 < n; j0 += kPcPts) {
    const int cnt = min(kPcPts, n - j0);
    __syncthreads();
    for (int i = threadIdx.x; i < cnt * kPcTX; i += blockDim.x) {
      int j = i / kPcTX, c = i - j * kPcTX;
      int cc = blockIdx.x * kPcTX + c;
      size_t o = (size_t)(j0 + j) * g.nx + cc;
      sA[j][c] = cc < g.nx ? A[o] : 0.f;
      sX[j][c] = cc < g.nx ? RX[o] : 1.f;
    }
    for (int i = threadIdx.x; i < cnt * kPcTR; i += blockDim.x) {
      int j = i / kPcTR, r = i - j * kPcTR;          // tile row r = ty' + kPcFTY i'
      int rr = blockIdx.y * kPcTR + r;
      const int slot = (r % kPcFTY) * kPcRows + r / kPcFTY;
      size_t o = (size_t)(j0 + j) * g.ny + rr;
      sB[j][slot] = rr < g.ny ? B[o] : 0.f;
      sR[j][slot] = rr < g.ny ? RY[o] : 1.f;
      sE[j][slot] = rr < g.ny ? E[o] : 0.f;
    }
    for (int i = threadIdx.x; i < cnt; i += blockDim.x) sP[i] = prm[j0 + i];
    __syncthreads();
#pragma unroll 2
    for (int j = 0; j < cnt; ++j) {
      const float4 p = sP[j];                     // x_j, rb, amplitude
      const float dx = X - p.x;
      const float dx2 = dx * dx;
      const float ndx2 = nk * dx2;
      const float rx = sX[j][tx], a = sA[j][tx];
      const float rxb = rx + p.y;
      const float4 ry4 = *reinterpret_cast<const float4*>(&sR[j][ty * kPcRows]);
      const float4 e4 = *reinterpret_cast<const float4*>(&sE[j][ty * kPcRows]);
      const float4 b4 = *reinterpret_cast<const float4*>(&sB[j][ty * kPcRows]);
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const float2 ry = h ? make_float2(ry4.z, ry4.w) : make_float2(ry4.x, ry4.y);
        const float2 ee = h ? make_float2(e4.z, e4.w) : make_float2(e4.x, e4.y);
        const float2 bb = h ? make_float2(b4.z, b4.w) : make_float2(b4.x, b4.y);
        const float2 t = __ffma2_rn(ry, ry, f2(dx2));
        const float2 rr = make_float2(pc_sqrt_approx(t.x), pc_sqrt_approx(t.y));
        const float2 s1 = __fadd2_rn(f2(rx), rr);                           // r_x + r
        const float2 num = __fadd2_rn(s1, __fadd2_rn(ry, f2(p.y)));          // (r_x + r) + (r_y + rb)
        const float2 den = __fmul2_rn(__fmul2_rn(__fadd2_rn(rr, ry), f2(rxb)), s1);
        const float2 q = __fmul2_rn(num, make_float2(pc_rcp_approx(den.x), pc_rcp_approx(den.y)));
        const float2 rem = __fmul2_rn(__fmul2_rn(f2(ndx2), ee), q);
        float2 ph = __fadd2_rn(__fadd2_rn(f2(a), bb), rem);
        const float2 k = __fmul2_rn(ph, f2(inv2pi));
        ph = __ffma2_rn(f2(-two_pi), make_float2(rintf(k.x), rintf(k.y)), ph);
        float2 sn, cs;
        pc_sincos2(ph, &sn, &cs);
        if (h) { re23 = __ffma2_rn(f2(p.z), cs, re23); im23 = __ffma2_rn(f2(p.z), sn, im23); }
        else { re01 = __ffma2_rn(f2(p.z), cs, re01); im01 = __ffma2_rn(f2(p.z), sn, im01); }
      }
    }
  }
  if (col >= g.nx) return;
  const float re[kPcRows] = {re01.x, re01.y, re23.x, re23.y};
  const float im[kPcRows] = {im01.x, im01.y, im23.x, im23.y};
#pragma unroll
  for (int i = 0; i < kPcRows; ++i) {
    const int row = row0 + kPcFTY * i;
    if (row < g.ny) {
      const size_t o = (size_t)row * g.nx + col;
      if (field) {
        if (accumulate_field) { float2 f = field[o]; field[o] = make_float2(f.x + re[i], f.y + im[i]); }
        else field[o] = make_float2(re[i], im[i]);
      }
      if (fringe) fringe[o] += re[i];
    }
  }
}

__global__ void __launch_bounds__(256) pc_direct_f64(PCGeom g, const float4* __restrict__ pts, int n,
                                                    double2* __restrict__ field, double* __restrict__ fringe) {
  __shared__ double4 sP[kPcPts];
  const int tx = threadIdx.x % kPcTX, ty = threadIdx.x / kPcTX;
  const int col = blockIdx.x * kPcTX + tx, row = blockIdx.y * kPcTY + ty;
  const double X = ((double)col + 0.5) * g.px - g.hlx;
  const double Y = g.hly - ((double)row + 0.5) * g.py;
  const double ref = g.k * X * g.stx + g.k * Y * g.sty;
  double re = 0.0, im = 0.0;
  for (int j0 = 0; j0 < n; j0 += kPcPts) {
    const int cnt = min(kPcPts, n - j0);
    __syncthreads();
    for (int i = threadIdx.x; i < cnt; i += blockDim.x) {
      float4 p = pts[j0 + i];
      sP[i] = make_double4((double)p.x * g.sx, (double)p.y * g.sy, (double)p.z * g.sz + g.off, (double)p.w);
    }
    __syncthreads();
    for (int j = 0; j < cnt; ++j) {
      const double4 p = sP[j];
      const double dx = X - p.x, dy = Y - p.y;
      const double r = sqrt(dx * dx + dy * dy + p.z * p.z);
      double sn, cs;
      sincos(g.k * r - ref, &sn, &cs);
      re += p.w * cs;
      im += p.w * sn;
    }
  }
  if (col < g.nx && row < g.ny) {
    const size_t o = (size_t)row * g.nx + col;
    if (field) field[o] = make_double2(re, im);
    if (fringe) fringe[o] += re;
  }
}

static oh_status validate_pc(const oh_pc_params* p, int n) {
  if (!p) return fail(OH_ERR_INVALID_ARG, "null point-cloud params");
  if (p->nx < 1 || p->ny < 1) return fail(OH_ERR_INVALID_ARG, "nx/ny must be positive");
  if (n < 0) return fail(OH_ERR_INVALID_ARG, "negative point count");
  if (!(p->lambda > 0) || !(p->pitch_x > 0) || !(p->pitch_y > 0)) return fail(OH_ERR_INVALID_ARG, "pitch and wavelength must be positive");
  return OH_OK;
}

static PCGeom make_geom(const oh_pc_params* p) {
  PCGeom g;
  g.k = 2.0 * M_PI / p->lambda;
  g.px = p->pitch_x; g.py = p->pitch_y;
  g.hlx = p->pitch_x * p->nx / 2.0; g.hly = p->pitch_y * p->ny / 2.0;
  g.sx = p->scale_x; g.sy = p->scale_y; g.sz = p->scale_z; g.off = p->offset_depth;
  g.stx = std::sin(p->tilt_x_deg * M_PI / 180.0);
  g.sty = std::sin(p->tilt_y_deg * M_PI / 180.0);
  g.nx = p->nx; g.ny = p->ny;
  return g;
}

oh_status pointcloud_enqueue(oh_ctx* ctx, int prec, const oh_pc_params* p, const float* xyza, int n,
                             void* field, void* fringe, cudaStream_t st) {
  PCGeom g = make_geom(p);
  dim3 grid((p->nx + kPcTX - 1) / kPcTX, (p->ny + kPcTY - 1) / kPcTY);
  const float4* pts = reinterpret_cast<const float4*>(xyza);
  if (n == 0) {
    if (field) OH_CUDA_TRY(cudaMemsetAsync(field, 0, (size_t)p->nx * p->ny * (prec ? 16 : 8), st));
    return OH_OK;
  }
  if (prec) {
    KernelTimer kt(ctx, "pc_direct_f64", st);
    pc_direct_f64<<<grid, kPcTX * kPcTY, 0, st>>>(g, pts, n, (double2*)field, (double*)fringe);
    OH_LAUNCH_CHECK();
    return OH_OK;
  }
  const int chunk = std::min(n, kPcChunk);
  void* ptr;
  OH_TRY(scratch(ctx, "pc.tables", (size_t)chunk * (sizeof(float4) + sizeof(float) * (2 * (size_t)p->nx + 3 * (size_t)p->ny)) + 1024, &ptr));
  float4* prm = (float4*)ptr;
  float* A = (float*)(prm + chunk);
  float* RX = A + (size_t)chunk * p->nx;
  float* B = RX + (size_t)chunk * p->nx;
  float* RY = B + (size_t)chunk * p->ny;
  float* E = RY + (size_t)chunk * p->ny;
  for (int j0 = 0; j0 < n; j0 += chunk) {
    const int cnt = std::min(chunk, n - j0);
    {
      KernelTimer kt(ctx, "pc_tables", st);
      pc_tables<<<std::max(1, std::min(cnt, oh::sm_count() * 8)), 256, 0, st>>>(g, pts + j0, cnt, prm, A, RX, B, RY, E);
      OH_LAUNCH_CHECK();
    }
    KernelTimer kt(ctx, "pc_direct_f32", st);
    pc_direct_f32<<<pc_grid_f32(p->nx, p->ny), kPcTX * kPcFTY, 0, st>>>(g, prm, A, RX, B, RY, E, cnt, (float2*)field, (float*)fringe, j0 > 0);
    OH_LAUNCH_CHECK();
  }
  return OH_OK;
}

// ---- allocation-free variant -------------------------------------------------
// Scratch for oh_pointcloud_noalloc: the per-chunk phase tables live in this
// file-scope device array (held by every GPU that loads the library).  Host
// code must not use the symbol as a device address; set-up below looks the
// address up once per device with cudaGetSymbolAddress.
constexpr size_t kNoAllocScratchBytes = (size_t)OH_PC_NOALLOC_SCRATCH_BYTES;
constexpr int kNoAllocMinChunk = 64;
static __device__ __align__(256) unsigned char g_pc_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
static std::mutex g_noalloc_mu;
static void* g_noalloc_ptr[kMaxDevices] = {nullptr};
static unsigned long long g_noalloc_ctx_id[kMaxDevices] = {0};

// Unique id of the CUDA context current on this thread (0 if unknown).  A
// device reset destroys the primary context and the module with it, so the
// scratch array's address is cached per context id, not per device index.
static unsigned long long current_ctx_id() {
  typedef int (*get_current_t)(void**);
  typedef int (*get_id_t)(void*, unsigned long long*);
  static get_current_t get_current = nullptr;
  static get_id_t get_id = nullptr;
  static bool looked_up = false;
  if (!looked_up) {
    looked_up = true;
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = (get_current_t)f;
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = (get_id_t)f;
    cudaGetLastError();
  }
  void* c = nullptr;
  unsigned long long id = 0;
  if (!get_current || !get_id || get_current(&c) != 0 || !c || get_id(c, &id) != 0) return 0;
  return id;
}

// Device address of the scratch array in the current device's context.  The
// first call in a context (the first call on a device, and the first after
// a device reset) looks the address up with cudaGetSymbolAddress.
static oh_status noalloc_scratch(void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  if (dev < 0 || dev >= kMaxDevices) return fail(OH_ERR_INVALID_ARG, "device index above the supported maximum");
  e = cudaSetDevice(dev);   // makes the device's primary context current
  if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
  const unsigned long long id = current_ctx_id();
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_ptr[dev] || id == 0 || g_noalloc_ctx_id[dev] != id) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_pc_noalloc_scratch);
    if (e != cudaSuccess || !p) return cuda_fail(e == cudaSuccess ? cudaErrorInvalidSymbol : e, "cudaGetSymbolAddress(point-cloud scratch)");
    g_noalloc_ptr[dev] = p;
    g_noalloc_ctx_id[dev] = id;
  }
  *out = g_noalloc_ptr[dev];
  return OH_OK;
}

}  // namespace oh

using namespace oh;

extern "C" {

oh_status oh_pointcloud_noalloc(const oh_pc_params* p, const float* xyza, int n_points, void* field_out,
                                void* fringe_out, void* stream) {
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  OH_TRY(validate_pc(p, n_points));
  if (!field_out && !fringe_out) return fail(OH_ERR_INVALID_ARG, "need field_out or fringe_out");
  if (n_points > 0 && !xyza) return fail(OH_ERR_INVALID_ARG, "null points");
  // one chunk of tables needs 16 B + 4 B x (2 nx + 3 ny) per point
  const size_t per_point = sizeof(float4) + sizeof(float) * (2 * (size_t)p->nx + 3 * (size_t)p->ny);
  if (per_point * kNoAllocMinChunk > kNoAllocScratchBytes)
    return fail(OH_ERR_UNSUPPORTED_SIZE, "oh_pointcloud_noalloc: field " + std::to_string(p->nx) + "x" + std::to_string(p->ny) +
                                             " needs more than the fixed scratch of " + std::to_string(kNoAllocScratchBytes) +
                                             " bytes (limit: 2*nx + 3*ny <= " +
                                             std::to_string((kNoAllocScratchBytes / kNoAllocMinChunk - sizeof(float4)) / sizeof(float)) + ")");
  void* base = nullptr;
  OH_TRY(noalloc_scratch(&base));
  PCGeom g = make_geom(p);
  const float4* pts = reinterpret_cast<const float4*>(xyza);
  if (n_points == 0) {
    if (field_out) OH_CUDA_TRY(cudaMemsetAsync(field_out, 0, (size_t)p->nx * p->ny * sizeof(float2), st));
    return OH_OK;
  }
  const int chunk = (int)std::min<size_t>((size_t)n_points, kNoAllocScratchBytes / per_point);
  float4* prm = (float4*)base;
  float* A = (float*)(prm + chunk);
  float* RX = A + (size_t)chunk * p->nx;
  float* B = RX + (size_t)chunk * p->nx;
  float* RY = B + (size_t)chunk * p->ny;
  float* E = RY + (size_t)chunk * p->ny;
  for (int j0 = 0; j0 < n_points; j0 += chunk) {
    const int cnt = std::min(chunk, n_points - j0);
    pc_tables<<<std::max(1, std::min(cnt, oh::sm_count() * 8)), 256, 0, st>>>(g, pts + j0, cnt, prm, A, RX, B, RY, E);
    OH_LAUNCH_CHECK();
    pc_direct_f32<<<pc_grid_f32(p->nx, p->ny), kPcTX * kPcFTY, 0, st>>>(g, prm, A, RX, B, RY, E, cnt, (float2*)field_out, (float*)fringe_out,
                                                  j0 > 0);
    OH_LAUNCH_CHECK();
  }
  return OH_OK;
}


oh_status oh_pointcloud(oh_ctx* ctx, oh_precision prec, const oh_pc_params* p, const float* xyza, int n_points,
                        void* field_out, void* fringe_out, void* stream) {
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  CallScope cs(ctx, st);
  OH_TRY(cs.status());
  OH_TRY(validate_pc(p, n_points));
  if (!field_out && !fringe_out) return fail(OH_ERR_INVALID_ARG, "need field_out or fringe_out");
  if (n_points > 0 && !xyza) return fail(OH_ERR_INVALID_ARG, "null points");
  return pointcloud_enqueue(ctx, prec == OH_FP64 ? 1 : 0, p, xyza, n_points, field_out, fringe_out, st);
}

oh_status oh_pointcloud_host(oh_ctx* ctx, oh_precision prec, const oh_pc_params* p, const float* xyza_host,
                             int n_points, void* field_host, void* fringe_host, void* stream) {
  OH_TRY(validate_pc(p, n_points));
  if (!ctx) return fail(OH_ERR_INVALID_ARG, "null context");
  if (!field_host && !fringe_host) return fail(OH_ERR_INVALID_ARG, "need field_host or fringe_host");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  CallScope cs(ctx, st);
  OH_TRY(cs.status());
  const size_t npx = (size_t)p->nx * p->ny;
  const size_t es = prec == OH_FP64 ? 8 : 4;
  const size_t pbytes = (size_t)std::max(n_points, 1) * 16;
  void* ptr;
  OH_TRY(scratch(ctx, "host.pc", pbytes + npx * es * 3 + 1024, &ptr));
  char* base = (char*)ptr;
  float* d_pts = (float*)base;
  size_t off = (pbytes + 255) & ~(size_t)255;
  void* d_field = field_host ? base + off : nullptr;
  if (field_host) off += (npx * es * 2 + 255) & ~(size_t)255;
  void* d_fringe = fringe_host ? base + off : nullptr;
  if (n_points > 0) OH_CUDA_TRY(cudaMemcpyAsync(d_pts, xyza_host, (size_t)n_points * 16, cudaMemcpyHostToDevice, st));
  if (d_fringe) OH_CUDA_TRY(cudaMemcpyAsync(d_fringe, fringe_host, npx * es, cudaMemcpyHostToDevice, st));
  OH_TRY(pointcloud_enqueue(ctx, prec == OH_FP64 ? 1 : 0, p, d_pts, n_points, d_field, d_fringe, st));
  if (d_field) OH_CUDA_TRY(cudaMemcpyAsync(field_host, d_field, npx * es * 2, cudaMemcpyDeviceToHost, st));
  if (d_fringe) OH_CUDA_TRY(cudaMemcpyAsync(fringe_host, d_fringe, npx * es, cudaMemcpyDeviceToHost, st));
  OH_CUDA_TRY(cudaStreamSynchronize(st));
  return OH_OK;
}

}  // extern "C"
