// Fresnel-convolution propagation, CWO::Diffract(z, CWO_FRESNEL_CONV)
// (cwo.cpp:2198-2279; DiffractConv FRESNEL_CONV cwo.cpp:2872-2898): zero-pad
// the Nx x Ny field into a 2Nx x 2Ny grid at offset (Nx/2, Ny/2), FFT,
// multiply by the FFT of the sampled Fresnel impulse response, inverse FFT
// with 1/(2Nx 2Ny), crop the centre back.  The impulse response is written
// from the mathematics
//   h(x,y) = exp(i k z)/(i lambda z) exp(i pi (x^2+y^2)/(lambda z)) dp^2
// (the DLL's kernel/coefficient bodies are not in the tree), sampled with its
// origin at index (0,0) so that the convolution output is aligned with the
// input.
//
// h is separable, h = C gx(x) gy(y), so its spectrum is C Hx(u) Hy(v), Hx and
// Hy being the 1-D DFTs of the sampled chirps (computed once in FP64 and
// cached per size, pitch, lambda and z), and the padded 2-D convolution is a
// row convolution with C gx followed by a column convolution with gy.  In
// FP32, when 2Nx and 2Ny have compile-time FFT schedules, three kernels do
// the propagation without materialising the padded grid:
//   fr_rowconv         per row: x-FFT on the padded length, times C Hx,
//                      inverse x-FFT, crop to Nx, written as strips of two
//                      columns;
//   fr_col             per strip: the same along y with Hy / (4 Nx Ny),
//                      keeping the Ny cropped rows (in place in the strip);
//   fr_strips_to_rows  strips back to the row-major field.
// Each line enters its forward FFT rotated by half its padded length, so the
// data fill the first and last quarters (radix-16 stage-0 butterflies see 8 of
// 16 inputs); the rotation multiplies the spectrum by (-1)^u (and (-1)^v),
// which the tables undo.  FP64 and other sizes run the padded-grid path:
// pad, 2-D FFT, multiply by the cached 2-D spectrum, inverse 2-D FFT, crop.
#include <cmath>
#include <cstdio>
#include <cstring>
#include "context.h"
#include "fft_kernels.cuh"

namespace oh {

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
static oh_status run_fresnel_grid(oh_ctx* ctx, int nx, int ny, double dp, double lambda, double z, void* field, cudaStream_t st) {
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
  const int grid = oh::sm_count() * 8;
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

// ---- separable path (FP32) ------------------------------------------------

constexpr int kFrW = 2;      // columns per strip

struct FrArgs {
  int nx, ny;                // field size; the padded grid is 2nx x 2ny
  float2* field;             // read by fr_rowconv, written by fr_strips_to_rows
  float2* R;                 // strips [nx / kFrW][ny][kFrW]
  const float2* twx;         // plan twiddles of the two lengths
  const float2* twy;
  const float2* hxs;         // C (-1)^u Hx(u) at x-FFT storage position
  const float2* hys;         // (-1)^v Hy(v) / (4 nx ny), natural order
};

__host__ __device__ constexpr int fr_tw_entries(int n) { return kTwLo + (n + 63) / 64; }

template <int NY> struct FrColCfg {
  static constexpr int R0 = FastSched<NY>::r0;
  static constexpr int RL = FastSched<NY>::rlast;
  static constexpr int NBL = (NY / RL) * kFrW;        // last-stage butterflies in the strip
  static constexpr int KB = NBL > 768 ? 2 : 1;         // butterflies per thread
  static constexpr int T = ((NBL + KB - 1) / KB + 31) / 32 * 32;
  // two blocks per SM when two strips fit in shared memory (at 4320, 576
  // threads x 2 blocks cap the registers at 56 with a few spills; measured
  // still faster than 288 threads with two butterflies each)
  static constexpr int MINB = (NY * kFrW + fr_tw_entries(NY)) * 8 <= 113 * 1024 ? 2 : 1;
};

// One strip of kFrW columns (already convolved along x) per block: y-FFT,
// times Hy, inverse y-FFT, crop; the result overwrites the strip.  The last
// forward stage, Hy and the first stage of the inverse run in registers; the
// inverse is the adjoint of the forward network (storage order in, natural
// order out), and its last stage computes only the outputs of the crop and
// stores them straight into the strip.
template <int NY>
__global__ void __launch_bounds__(FrColCfg<NY>::T, FrColCfg<NY>::MINB) fr_col(FrArgs a) {
  typedef float2 C;
  typedef FrColCfg<NY> CF;
  constexpr int W = kFrW, T = CF::T, R0 = CF::R0, RL = CF::RL, KB = CF::KB;
  constexpr int R1 = FastSched<NY>::r1;
  constexpr int Q0 = NY / R0, QY = NY / 4;
  static_assert(FastSched<NY>::nstages == 3, "three-stage schedule expected");
  static_assert(R0 % 4 == 0, "stage-0 radix must split the line into quarters");
  extern __shared__ __align__(16) unsigned char smem[];
  C* buf = reinterpret_cast<C*>(smem);               // [NY][W]
  C* twlo = buf + NY * W;
  C* twhi = twlo + kTwLo;
  const int tid = threadIdx.x, s = blockIdx.x;
  C* strip = a.R + (size_t)s * a.ny * W;
  load_tw_split(twlo, twhi, a.twy, NY);
  __syncthreads();
  const TwSplit<C> tw{twlo, twhi};
  // stage 0 from global memory; rotated line: positions [QY, 3QY) are zero,
  // position p < QY holds row p + QY, p >= 3QY holds row p - 3QY
  for (int idx = tid; idx < Q0 * W; idx += T) {
    const int j = idx / W, w = idx - j * W;
    C x[R0];
#pragma unroll
    for (int t = 0; t < R0; ++t) {
      const int p = j + t * Q0;
      if (t < R0 / 4) x[t] = strip[(p + QY) * W + w];
      else if (t >= 3 * R0 / 4) x[t] = strip[(p - 3 * QY) * W + w];
      else x[t] = make_float2(0.f, 0.f);
    }
    if constexpr (R0 == 16) dft16_halfzero<-1>(x);
    else DFT<R0, -1, C>::run(x);
    if (j) {
      C wp[R0];
      twiddle_powers<R0, -1>(tw, j, wp);
#pragma unroll
      for (int f = 1; f < R0; ++f) x[f] = cmul(x[f], wp[f]);
    }
#pragma unroll
    for (int f = 0; f < R0; ++f) buf[(j + f * Q0) * W + w] = x[f];
  }
  __syncthreads();
  fstage_t<NY, R1, NY / R0, -1>(buf, W, 1, W, tw, true);
  __syncthreads();
  // last forward stage (stride 1, no twiddles), Hy, first inverse stage
#pragma unroll
  for (int kb = 0; kb < KB; ++kb) {
    const int bb = tid + kb * T;
    if (bb < CF::NBL) {
      const int b = bb / W, w = bb - b * W;
      C x[RL];
#pragma unroll
      for (int f = 0; f < RL; ++f) x[f] = buf[(b * RL + f) * W + w];
      DFT<RL, -1, C>::run(x);
#pragma unroll
      for (int f = 0; f < RL; ++f) x[f] = cmul(x[f], __ldg(a.hys + FastSched<NY>::iperm(b * RL + f)));
      DFT<RL, 1, C>::run(x);
#pragma unroll
      for (int f = 0; f < RL; ++f) buf[(b * RL + f) * W + w] = x[f];
    }
  }
  __syncthreads();
  fstage_adj<NY, R1, NY / R0>(buf, W, 1, W, tw, true);
  __syncthreads();
  // last inverse stage: output row r is sample QY + r = j + t Q0, t in [R0/4, 3R0/4)
  for (int idx = tid; idx < Q0 * W; idx += T) {
    const int j = idx / W, w = idx - j * W;
    C x[R0];
#pragma unroll
    for (int f = 0; f < R0; ++f) x[f] = buf[(j + f * Q0) * W + w];
    if (j) {
      C wp[R0];
      twiddle_powers<R0, 1>(tw, j, wp);
#pragma unroll
      for (int f = 1; f < R0; ++f) x[f] = cmul(x[f], wp[f]);
    }
    DFT<R0, 1, C>::run(x);
#pragma unroll
    for (int t = R0 / 4; t < 3 * R0 / 4; ++t) strip[(j + (t - R0 / 4) * Q0) * W + w] = x[t];
  }
}

// Shared-memory layout of fr_rowconv's two rows: element p of row l at
// l LS + (p / M1) BS + p % M1 + RP ((p % M1) / RL), M1 = NX / r0 (a stage-0
// block).  RP pads one element after every RL (an even last radix otherwise
// puts a half-warp of the last stage on few bank pairs), BS - M1 (1 + RP/RL)
// pads each block (middle-stage half-warps that cross a block), and LS makes
// the two rows of a stage-0 half-warp use other bank pairs.  The layouts
// were found by an exhaustive search over (RP, block pad, LS) minimising
// the shared-memory wavefronts of the three access patterns; other lengths
// keep LS = the padded length rounded to 8 mod 16 and no element pads.
template <int NX> struct FrRowPad {
  typedef FastSched<NX> S;
  static constexpr int M1 = NX / S::r0, RL = S::rlast;
  static constexpr int RP = NX == 7680 || NX == 4096 || NX == 2048 ? 1 : 0;
  static constexpr int PADB = NX == 7680 ? 14 : NX == 2048 ? 8 : NX == 3840 ? 15 : NX == 4320 ? 1 : 0;
  static constexpr int BS = M1 + RP * (M1 / RL) + PADB;
  static constexpr int LS = NX == 7680 ? 8168 : NX == 4096 ? 4360 : NX == 2048 ? 2440 : NX == 3840 ? 4088
                          : NX == 4320 ? 4344 : NX + ((8 - NX % 16) + 16) % 16;
  static constexpr int RLP = RL + RP;
  static constexpr int BPB = M1 / RL;                        // last-stage butterflies per block
  static_assert(RP == 0 || M1 % RL == 0, "the element pad needs whole last-stage groups per block");
  static_assert(LS >= S::r0 * BS, "rows must not overlap");
  // stored offset of j < M1 within its block
  __device__ __forceinline__ static int in_blk(int j) { return RP ? j + j / RL : j; }
};
template <int NX> constexpr int fr_row_stride() { return FrRowPad<NX>::LS; }

// Separable form, first pass: two rows per block, each convolved with hx on
// the padded length, cropped to nx columns and stored as strips
// [nx / kFrW][ny][kFrW].  Forward x-FFT of the rotated row (stage 0 straight
// from global memory, half its inputs zero), then in registers the last
// forward stage, C (-1)^u Hx(u) and the first stage of the inverse; the
// inverse is the adjoint of the forward network (storage order in, natural
// order out), and its last stage computes only the cropped outputs and
// stores them, thread pairs (one per row) filling 32-byte strip sectors.
template <int NX>
__global__ void __launch_bounds__(512) fr_rowconv(FrArgs a) {
  typedef float2 C;
  typedef FastSched<NX> S;
  constexpr int ROWS = 2, NT = 512;
  constexpr int R0 = S::r0, R1 = S::r1, RL = S::rlast, Q0 = NX / R0, Q = NX / 4;
  typedef FrRowPad<NX> FP;
  constexpr int LS = FP::LS;
  static_assert(S::nstages == 3, "three-stage schedule expected");
  static_assert(R0 % 4 == 0, "stage-0 radix must split the line into quarters");
  extern __shared__ __align__(16) unsigned char smem[];
  C* buf = reinterpret_cast<C*>(smem);               // [ROWS][LS]
  C* twlo = buf + ROWS * LS;
  C* twhi = twlo + kTwLo;
  const int r0 = ROWS * blockIdx.x, nx = a.nx, ny = a.ny;
  load_tw_split(twlo, twhi, a.twx, NX);
  __syncthreads();
  const TwSplit<C> tw{twlo, twhi};
  const C* src = a.field + (size_t)r0 * nx;
  // stage 0: rotated line, position p < Q holds column p + Q, p >= 3Q column p - 3Q
  for (int idx = threadIdx.x; idx < ROWS * Q0; idx += NT) {
    const int j = idx >> 1, l = idx & 1;
    C x[R0];
#pragma unroll
    for (int t = 0; t < R0; ++t) {
      const int p = j + t * Q0;
      if (t < R0 / 4) x[t] = src[(size_t)l * nx + p + Q];
      else if (t >= 3 * R0 / 4) x[t] = src[(size_t)l * nx + p - 3 * Q];
      else x[t] = make_float2(0.f, 0.f);
    }
    if constexpr (R0 == 16) dft16_halfzero<-1>(x);
    else DFT<R0, -1, C>::run(x);
    if (j) {
      C wp[R0];
      twiddle_powers<R0, -1>(tw, j, wp);
#pragma unroll
      for (int f = 1; f < R0; ++f) x[f] = cmul(x[f], wp[f]);
    }
    C* bl = buf + l * LS + FP::in_blk(j);
#pragma unroll
    for (int f = 0; f < R0; ++f) bl[f * FP::BS] = x[f];
  }
  __syncthreads();
  fstage_t<NX, R1, NX / R0, -1, C, TwSplit<C>, FP::BS, FP::RLP>(buf, ROWS, LS, 1, tw, false);
  __syncthreads();
  // last forward stage (no twiddles), the transfer function, first inverse stage
  constexpr int NBL = NX / RL;
  for (int idx = threadIdx.x; idx < ROWS * NBL; idx += NT) {
    const int l = idx / NBL, b = idx - l * NBL;
    C* p = buf + l * LS + (b / FP::BPB) * FP::BS + (b % FP::BPB) * FP::RLP;
    C x[RL];
#pragma unroll
    for (int f = 0; f < RL; ++f) x[f] = p[f];
    DFT<RL, -1, C>::run(x);
#pragma unroll
    for (int f = 0; f < RL; ++f) x[f] = cmul(x[f], __ldg(a.hxs + b * RL + f));
    DFT<RL, 1, C>::run(x);
#pragma unroll
    for (int f = 0; f < RL; ++f) p[f] = x[f];
  }
  __syncthreads();
  fstage_adj<NX, R1, NX / R0, C, TwSplit<C>, FP::BS, FP::RLP>(buf, ROWS, LS, 1, tw, false);
  __syncthreads();
  // last inverse stage: column c = sample Q + c = j + t Q0, t in [R0/4, 3R0/4)
  for (int idx = threadIdx.x; idx < ROWS * Q0; idx += NT) {
    const int j = idx >> 1, l = idx & 1;
    C x[R0];
    const C* bl = buf + l * LS + FP::in_blk(j);
#pragma unroll
    for (int f = 0; f < R0; ++f) x[f] = bl[f * FP::BS];
    if (j) {
      C wp[R0];
      twiddle_powers<R0, 1>(tw, j, wp);
#pragma unroll
      for (int f = 1; f < R0; ++f) x[f] = cmul(x[f], wp[f]);
    }
    DFT<R0, 1, C>::run(x);
#pragma unroll
    for (int t = R0 / 4; t < 3 * R0 / 4; ++t) {
      const int c = j + (t - R0 / 4) * Q0;
      a.R[((size_t)(c / kFrW) * ny + r0 + l) * kFrW + (c % kFrW)] = x[t];
    }
  }
}

// Separable form, last pass: strips [nx / kFrW][ny][kFrW] to the row-major
// field, through a 32-row x 64-column shared-memory tile.
__global__ void __launch_bounds__(256) fr_strips_to_rows(FrArgs a) {
  __shared__ float2 tile[32][64 + 1];
  const int x0 = blockIdx.x * 64, y0 = blockIdx.y * 32, nx = a.nx, ny = a.ny;
  const int ns = nx / kFrW;
  for (int i = threadIdx.x; i < 32 * 32; i += 256) {
    const int r = i & 31, s = i >> 5;                 // 32 strips x 32 rows, 16 bytes each; a warp
                                                      // reads 32 consecutive rows of one strip
    const int sg = x0 / kFrW + s, y = y0 + r;
    if (sg < ns && y < ny) {
      const float4 v = *reinterpret_cast<const float4*>(a.R + ((size_t)sg * ny + y) * kFrW);
      tile[r][2 * s] = make_float2(v.x, v.y);
      tile[r][2 * s + 1] = make_float2(v.z, v.w);
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < 32 * 64; i += 256) {
    const int c = i & 63, r = i >> 6;
    const int x = x0 + c, y = y0 + r;
    if (x < nx && y < ny) a.field[(size_t)y * nx + x] = tile[r][c];
  }
}

// exp(i pi x^2 / (lambda z)) at x = j dp, j = i (i < n/2) or i - n
__global__ void fr_chirp(int n, double dp, double lambda, double z, double2* g) {
  const double two_pi = 6.283185307179586476925286766559;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int j = i < n / 2 ? i : i - n;
    const double x = j * dp;
    double ph = M_PI * x * x / (lambda * z);
    ph -= two_pi * rint(ph / two_pi);
    double s, c;
    sincos(ph, &s, &c);
    g[i] = make_double2(c, s);
  }
}

__global__ void fr_tables(int NX, int NY, const double2* __restrict__ Hx, const double2* __restrict__ Hy,
                          const int* __restrict__ iperm_x, double cre, double cim, double scale,
                          float2* __restrict__ hxs, float2* __restrict__ hys) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < NX + NY; i += gridDim.x * blockDim.x) {
    if (i < NX) {
      const int u = iperm_x[i];
      const double sg = (u & 1) ? -1.0 : 1.0;
      const double2 h = Hx[u];
      hxs[i] = make_float2((float)(sg * (cre * h.x - cim * h.y)), (float)(sg * (cre * h.y + cim * h.x)));
    } else {
      const int v = i - NX;
      const double sg = (v & 1) ? -scale : scale;
      hys[v] = make_float2((float)(sg * Hy[v].x), (float)(sg * Hy[v].y));
    }
  }
}

typedef void (*FrKernel)(FrArgs);

struct FrKernels {
  FrKernel rowconv, col;
  int col_threads;
};

// The kernels for padded lengths NX = 2nx, NY = 2ny, or false.
static bool fr_pick(int NX, int NY, FrKernels* k) {
  std::memset(k, 0, sizeof(*k));
  with_fast_n(NX, [&](auto nc) {
    constexpr int N = decltype(nc)::value;
    if constexpr (N > 0) k->rowconv = fr_rowconv<N>;
  });
  with_fast_n(NY, [&](auto nc) {
    constexpr int N = decltype(nc)::value;
    if constexpr (N > 0) { k->col = fr_col<N>; k->col_threads = FrColCfg<N>::T; }
  });
  return k->rowconv && k->col;
}

static oh_status run_fresnel_separable(oh_ctx* ctx, int nx, int ny, double dp, double lambda, double z,
                                       float2* field, const FrKernels& k, cudaStream_t st) {
  const int NX = 2 * nx, NY = 2 * ny;
  FFTPlan px, py;
  OH_TRY(get_plan(ctx, NX, 0, &px));
  OH_TRY(get_plan(ctx, NY, 0, &py));
  // strip buffer first: growing the scratch arena drops every cached key
  void* rbuf;
  OH_TRY(scratch(ctx, "fr.R", (size_t)ny * NX * sizeof(float2), &rbuf));
  // cached tables: FP64 chirps / spectra, then the FP32 factors
  const size_t tab_bytes = (size_t)(NX + NY) * (sizeof(double2) + sizeof(float2));
  char key[160];
  std::snprintf(key, sizeof(key), "sep:%d:%d:%.17g:%.17g:%.17g", NX, NY, dp, lambda, z);
  void* prev = nullptr;
  {
    auto it = ctx->scratch.find("fr.tab");
    if (it != ctx->scratch.end()) prev = it->second.p;
  }
  void* tab;
  OH_TRY(scratch(ctx, "fr.tab", tab_bytes, &tab));
  double2* gx = static_cast<double2*>(tab);
  double2* gy = gx + NX;
  float2* hxs = reinterpret_cast<float2*>(gy + NY);
  float2* hys = hxs + NX;
  if (!(prev == tab && ctx->fresnel_key == key)) {
    ctx->fresnel_key = key;
    fr_chirp<<<(NX + 255) / 256, 256, 0, st>>>(NX, dp, lambda, z, gx);
    OH_LAUNCH_CHECK();
    fr_chirp<<<(NY + 255) / 256, 256, 0, st>>>(NY, dp, lambda, z, gy);
    OH_LAUNCH_CHECK();
    OH_TRY(fft_rows_enqueue(ctx, 1, NX, 1, gx, gx, -1, 0, st));
    OH_TRY(fft_rows_enqueue(ctx, 1, NY, 1, gy, gy, -1, 0, st));
    const double two_pi = 6.283185307179586476925286766559;
    const double k = two_pi / lambda;
    const double kz = k * z - two_pi * std::rint(k * z / two_pi);
    const double amp = dp * dp / (lambda * z);
    fr_tables<<<(NX + NY + 255) / 256, 256, 0, st>>>(NX, NY, gx, gy, px.iperm, amp * std::sin(kz),
                                                      -amp * std::cos(kz), 1.0 / ((double)NX * (double)NY), hxs, hys);
    OH_LAUNCH_CHECK();
  }
  FrArgs a{nx, ny, field, static_cast<float2*>(rbuf), static_cast<const float2*>(px.tw),
           static_cast<const float2*>(py.tw), hxs, hys};
  const int scol = (NY * kFrW + fr_tw_entries(NY)) * (int)sizeof(float2);
  // rows convolved with hx and cropped to nx, then the nx / 2 strips with
  // hy (cropped to ny in place), then strips to rows
  int row_ls = NX;
  with_fast_n(NX, [&](auto nc) {
    if constexpr (decltype(nc)::value > 0) row_ls = fr_row_stride<decltype(nc)::value>();
  });
  const int srow = (2 * row_ls + fr_tw_entries(NX)) * (int)sizeof(float2);
  OH_CUDA_TRY(cudaFuncSetAttribute(k.rowconv, cudaFuncAttributeMaxDynamicSharedMemorySize, srow));
  OH_CUDA_TRY(cudaFuncSetAttribute(k.col, cudaFuncAttributeMaxDynamicSharedMemorySize, scol));
  {
    KernelTimer kt(ctx, "fresnel_rowconv", st);
    k.rowconv<<<ny / 2, 512, srow, st>>>(a);
    OH_LAUNCH_CHECK();
  }
  {
    KernelTimer kt(ctx, "fresnel_col", st);
    k.col<<<nx / kFrW, k.col_threads, scol, st>>>(a);
    OH_LAUNCH_CHECK();
  }
  {
    KernelTimer kt(ctx, "fresnel_to_rows", st);
    fr_strips_to_rows<<<dim3((nx + 63) / 64, (ny + 31) / 32), 256, 0, st>>>(a);
    OH_LAUNCH_CHECK();
  }
  return OH_OK;
}

template <typename R>
static oh_status run_fresnel(oh_ctx* ctx, int nx, int ny, double dp, double lambda, double z, void* field,
                             cudaStream_t st) {
  if constexpr (sizeof(R) == 4) {
    FrKernels k;
    const bool even = nx % 2 == 0 && ny % 2 == 0;
    int row_ls = 0;
    with_fast_n(2 * nx, [&](auto nc) {
      if constexpr (decltype(nc)::value > 0) row_ls = fr_row_stride<decltype(nc)::value>();
    });
    if (even && !getenv("OH_FRESNEL_GRID") && fr_pick(2 * nx, 2 * ny, &k) &&
        (size_t)(2 * row_ls + fr_tw_entries(2 * nx)) * sizeof(float2) <= max_smem_per_block())
      return run_fresnel_separable(ctx, nx, ny, dp, lambda, z, static_cast<float2*>(field), k, st);
  }
  return run_fresnel_grid<R>(ctx, nx, ny, dp, lambda, z, field, st);
}

}  // namespace oh

using namespace oh;

extern "C" {

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
