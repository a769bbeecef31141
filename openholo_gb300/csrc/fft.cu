// Generic 2-D / batched 1-D complex FFT built on the shared-memory engine
// (fft_core.cuh).  The 2-D transform is a row pass (each block owns whole
// rows) followed by a column pass (each block owns a strip of W adjacent
// columns, so global loads/stores are W*sizeof(complex)-byte segments).
//
// Shift semantics follow HologramKernel.cu:10-34 / :189-227:
//   out = shift(FFT2(shift(in))),  shift(a)[i][j] = a[(i-ny/2) mod ny][(j-nx/2) mod nx]
// (floor(n/2) on both sides).  The x shifts are applied by the row pass when
// loading/storing a row, the y shifts by the column pass, so no separate
// shift kernel runs and in == out is safe.
#include "context.h"
#include "fft_kernels.cuh"

namespace oh {

template <typename R, int SGN, int N>
__global__ void __launch_bounds__(256) fft_rows_kernel(const typename cplx_of<R>::type* __restrict__ in,
                                                       typename cplx_of<R>::type* __restrict__ out,
                                                       int nx, int ny, int rpb, int shift, R scale,
                                                       FFTPlan pl) {
  typedef typename cplx_of<R>::type C;
  extern __shared__ unsigned char smem_raw[];
  C* buf = reinterpret_cast<C*>(smem_raw);
  const int row0 = blockIdx.x * rpb;
  const int nrows = min(rpb, ny - row0);
  const int hx = shift ? nx / 2 : 0;
  for (int idx = threadIdx.x; idx < nrows * nx; idx += blockDim.x) {
    int l = idx / nx, j = idx - l * nx;
    int src = j - hx; if (src < 0) src += nx;
    buf[l * nx + j] = in[(size_t)(row0 + l) * nx + src];
  }
  block_fft_n<N, SGN>(buf, nrows, nx, 1, pl, false);
  for (int idx = threadIdx.x; idx < nrows * nx; idx += blockDim.x) {
    int l = idx / nx, k = idx - l * nx;
    int m = k - hx; if (m < 0) m += nx;     // out[k] = A[(k - hx) mod nx]
    C v = buf[l * nx + pl.perm[m]];
    out[(size_t)(row0 + l) * nx + k] = cscale(v, scale);
  }
}

// Column pass over strips of W columns.  aux (nullable) receives the
// unshifted transform FFT2(shift(in)) as cudaFFT leaves it in its input
// buffer (HologramKernel.cu:207-210).
template <typename R, int SGN, int N>
__global__ void __launch_bounds__(512) fft_cols_kernel(typename cplx_of<R>::type* data,
                                                       typename cplx_of<R>::type* aux,
                                                       int nx, int ny, int W, int shift, R scale,
                                                       FFTPlan pl) {
  typedef typename cplx_of<R>::type C;
  extern __shared__ unsigned char smem_raw[];
  C* buf = reinterpret_cast<C*>(smem_raw);
  const int x0 = blockIdx.x * W;
  const int hy = shift ? ny / 2 : 0;
  const int hx = shift ? nx / 2 : 0;
  for (int idx = threadIdx.x; idx < ny * W; idx += blockDim.x) {
    int i = idx / W, w = idx - i * W;
    int src = i - hy; if (src < 0) src += ny;
    buf[idx] = data[(size_t)src * nx + x0 + w];
  }
  block_fft_n<N, SGN>(buf, W, 1, W, pl, true);
  for (int idx = threadIdx.x; idx < ny * W; idx += blockDim.x) {
    int k = idx / W, w = idx - k * W;
    int m = k - hy; if (m < 0) m += ny;
    C v = buf[pl.perm[m] * W + w];
    data[(size_t)k * nx + x0 + w] = cscale(v, scale);
    if (aux) {
      C u = buf[pl.perm[k] * W + w];
      int xu = x0 + w - hx; if (xu < 0) xu += nx;
      aux[(size_t)k * nx + xu] = u;
    }
  }
}

template <typename R>
static oh_status launch_fft2d(oh_ctx* ctx, int nx, int ny, const void* in, void* out, void* aux,
                              int direction, int shift, int normalize, cudaStream_t st) {
  typedef typename cplx_of<R>::type C;
  const int prec = sizeof(R) == 8 ? 1 : 0;
  FFTPlan px, py;
  OH_TRY(get_plan(ctx, nx, prec, &px));
  OH_TRY(get_plan(ctx, ny, prec, &py));
  const size_t smax = max_smem_per_block();
  // rows
  int rpb = 1;
  while (rpb < 8 && (size_t)(rpb * 2) * nx * sizeof(C) <= 48 * 1024 && rpb * 2 * nx <= 4096) rpb *= 2;
  size_t srow = (size_t)rpb * nx * sizeof(C);
  if (srow > smax) return fail(OH_ERR_UNSUPPORTED_SIZE, "row length " + std::to_string(nx) + " exceeds shared memory");
  int W = pick_strip_width(nx, ny, sizeof(C), smax);
  if (W == 0) return fail(OH_ERR_UNSUPPORTED_SIZE, "column length " + std::to_string(ny) + " exceeds shared memory");
  size_t scol = (size_t)W * ny * sizeof(C);
  R scale = normalize ? (R)(1.0 / ((double)nx * (double)ny)) : (R)1;
  const C* cin = static_cast<const C*>(in);
  C* cout_ = static_cast<C*>(out);
  oh_status rs = OH_OK;
  auto rows = [&](auto sg) {
    constexpr int SG = decltype(sg)::value;
    with_fast_n_if<sizeof(R) == 4>(nx, [&](auto nc) {
      constexpr int NX = decltype(nc)::value;
      cudaError_t e = cudaFuncSetAttribute(fft_rows_kernel<R, SG, NX>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)srow);
      if (e != cudaSuccess) { rs = cuda_fail(e, "cudaFuncSetAttribute(fft_rows)"); return; }
      KernelTimer kt(ctx, "fft_rows", st);
      fft_rows_kernel<R, SG, NX><<<(ny + rpb - 1) / rpb, 256, srow, st>>>(cin, cout_, nx, ny, rpb, shift, (R)1, px);
      note_launch();
      if ((e = cudaGetLastError()) != cudaSuccess) rs = cuda_fail(e, "fft_rows launch");
    });
  };
  auto cols = [&](auto sg) {
    constexpr int SG = decltype(sg)::value;
    with_fast_n_if<sizeof(R) == 4>(ny, [&](auto nc) {
      constexpr int NY = decltype(nc)::value;
      cudaError_t e = cudaFuncSetAttribute(fft_cols_kernel<R, SG, NY>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)scol);
      if (e != cudaSuccess) { rs = cuda_fail(e, "cudaFuncSetAttribute(fft_cols)"); return; }
      KernelTimer kt(ctx, "fft_cols", st);
      fft_cols_kernel<R, SG, NY><<<nx / W, 512, scol, st>>>(cout_, static_cast<C*>(aux), nx, ny, W, shift, scale, py);
      note_launch();
      if ((e = cudaGetLastError()) != cudaSuccess) rs = cuda_fail(e, "fft_cols launch");
    });
  };
  if (direction < 0) { rows(std::integral_constant<int, -1>{}); OH_TRY(rs); cols(std::integral_constant<int, -1>{}); }
  else { rows(std::integral_constant<int, 1>{}); OH_TRY(rs); cols(std::integral_constant<int, 1>{}); }
  return rs;
}

template <typename R>
static oh_status launch_fft_rows(oh_ctx* ctx, int nx, int ny, const void* in, void* out,
                                 int direction, int normalize, cudaStream_t st) {
  typedef typename cplx_of<R>::type C;
  const int prec = sizeof(R) == 8 ? 1 : 0;
  FFTPlan px;
  OH_TRY(get_plan(ctx, nx, prec, &px));
  int rpb = 1;
  while (rpb < 8 && (size_t)(rpb * 2) * nx * sizeof(C) <= 48 * 1024 && rpb * 2 * nx <= 4096) rpb *= 2;
  size_t srow = (size_t)rpb * nx * sizeof(C);
  if (srow > max_smem_per_block()) return fail(OH_ERR_UNSUPPORTED_SIZE, "row length exceeds shared memory");
  R scale = normalize ? (R)(1.0 / (double)nx) : (R)1;
  if (direction < 0) {
    OH_CUDA_TRY(cudaFuncSetAttribute(fft_rows_kernel<R, -1, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)srow));
    fft_rows_kernel<R, -1, 0><<<(ny + rpb - 1) / rpb, 256, srow, st>>>(static_cast<const C*>(in), static_cast<C*>(out), nx, ny, rpb, 0, scale, px);
  } else {
    OH_CUDA_TRY(cudaFuncSetAttribute(fft_rows_kernel<R, 1, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)srow));
    fft_rows_kernel<R, 1, 0><<<(ny + rpb - 1) / rpb, 256, srow, st>>>(static_cast<const C*>(in), static_cast<C*>(out), nx, ny, rpb, 0, scale, px);
  }
  OH_LAUNCH_CHECK();
  return OH_OK;
}

oh_status fft2d_enqueue(oh_ctx* ctx, int prec, int nx, int ny, const void* in, void* out, void* aux,
                        int direction, int shift, int normalize, cudaStream_t st) {
  if (prec) return launch_fft2d<double>(ctx, nx, ny, in, out, aux, direction, shift, normalize, st);
  return launch_fft2d<float>(ctx, nx, ny, in, out, aux, direction, shift, normalize, st);
}

template <typename R>
static oh_status launch_fft_cols(oh_ctx* ctx, int nx, int ny, void* data, int direction, int normalize,
                                 cudaStream_t st) {
  typedef typename cplx_of<R>::type C;
  const int prec = sizeof(R) == 8 ? 1 : 0;
  FFTPlan py;
  OH_TRY(get_plan(ctx, ny, prec, &py));
  const int W = pick_strip_width(nx, ny, sizeof(C), max_smem_per_block());
  if (W == 0) return fail(OH_ERR_UNSUPPORTED_SIZE, "column length " + std::to_string(ny) + " exceeds shared memory");
  const size_t scol = (size_t)W * ny * sizeof(C);
  const R scale = normalize ? (R)(1.0 / (double)ny) : (R)1;
  if (direction < 0) {
    OH_CUDA_TRY(cudaFuncSetAttribute(fft_cols_kernel<R, -1, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)scol));
    fft_cols_kernel<R, -1, 0><<<nx / W, 512, scol, st>>>(static_cast<C*>(data), nullptr, nx, ny, W, 0, scale, py);
  } else {
    OH_CUDA_TRY(cudaFuncSetAttribute(fft_cols_kernel<R, 1, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)scol));
    fft_cols_kernel<R, 1, 0><<<nx / W, 512, scol, st>>>(static_cast<C*>(data), nullptr, nx, ny, W, 0, scale, py);
  }
  OH_LAUNCH_CHECK();
  return OH_OK;
}

oh_status fft_cols_enqueue(oh_ctx* ctx, int prec, int nx, int ny, void* data, int direction, int normalize,
                           cudaStream_t st) {
  if (prec) return launch_fft_cols<double>(ctx, nx, ny, data, direction, normalize, st);
  return launch_fft_cols<float>(ctx, nx, ny, data, direction, normalize, st);
}

oh_status fft_rows_enqueue(oh_ctx* ctx, int prec, int nx, int ny, const void* in, void* out, int direction,
                           int normalize, cudaStream_t st) {
  if (prec) return launch_fft_rows<double>(ctx, nx, ny, in, out, direction, normalize, st);
  return launch_fft_rows<float>(ctx, nx, ny, in, out, direction, normalize, st);
}

int pick_strip_width(int nx, int ny, size_t esz, size_t smax) {
  // widest strip (<= 8 columns) that divides nx and fits in shared memory
  const int cands[4] = {8, 4, 2, 1};
  for (int W : cands) {
    if (nx % W) continue;
    if ((size_t)W * ny * esz <= smax) return W;
  }
  return 0;
}

}  // namespace oh

using namespace oh;

extern "C" {

int oh_fft_supported(int n, oh_precision prec) {
  int radix[kMaxStages], nst;
  if (n < 1 || !factorize(n, radix, &nst)) return 0;
  size_t esz = prec == OH_FP64 ? sizeof(double2) : sizeof(float2);
  return (size_t)n * esz <= max_smem_per_block() ? 1 : 0;
}

oh_status oh_fft2d(oh_ctx* ctx, oh_precision prec, int nx, int ny, const void* in, void* out,
                   int direction, int shift, int normalize, void* stream) {
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  CallScope cs(ctx, st);
  OH_TRY(cs.status());
  if (nx < 1 || ny < 1 || !in || !out) return fail(OH_ERR_INVALID_ARG, "oh_fft2d: bad size or null buffer");
  if (direction != -1 && direction != 1) return fail(OH_ERR_INVALID_ARG, "oh_fft2d: direction must be -1 or +1");
  return fft2d_enqueue(ctx, prec == OH_FP64 ? 1 : 0, nx, ny, in, out, nullptr, direction, shift, normalize, st);
}

oh_status oh_fft1d_rows(oh_ctx* ctx, oh_precision prec, int nx, int ny, const void* in, void* out,
                        int direction, int normalize, void* stream) {
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  CallScope cs(ctx, st);
  OH_TRY(cs.status());
  if (nx < 1 || ny < 1 || !in || !out) return fail(OH_ERR_INVALID_ARG, "oh_fft1d_rows: bad size or null buffer");
  if (direction != -1 && direction != 1) return fail(OH_ERR_INVALID_ARG, "oh_fft1d_rows: direction must be -1 or +1");
  if (prec == OH_FP64) return launch_fft_rows<double>(ctx, nx, ny, in, out, direction, normalize, st);
  return launch_fft_rows<float>(ctx, nx, ny, in, out, direction, normalize, st);
}

}  // extern "C"
