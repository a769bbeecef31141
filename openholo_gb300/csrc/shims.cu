// Reference-signature depth-map launchers (include/oh_reference_shims.h).
// The element-wise launchers are FP64 restatements of the reference kernels
// (HologramKernel.cu:49-187); cudaFFT runs this library's mixed-radix FFT
// with the shifts folded into its load/store index maps.  A process-wide
// context per device holds the FFT plans.
#include <mutex>
#include <vector>
#include "context.h"
#include "fft_kernels.cuh"
#include "../../include/oh_reference_shims.h"

namespace oh {

static thread_local oh_status t_shim_status = OH_OK;
static std::mutex g_shim_mu;
static std::vector<oh_ctx*> g_shim_ctx;

static oh_ctx* shim_ctx() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
  std::lock_guard<std::mutex> lk(g_shim_mu);
  if ((int)g_shim_ctx.size() <= dev) g_shim_ctx.resize(dev + 1, nullptr);
  if (!g_shim_ctx[dev]) {
    oh_ctx* c = nullptr;
    if (oh_ctx_create(&c, dev) != OH_OK) return nullptr;
    g_shim_ctx[dev] = c;
  }
  return g_shim_ctx[dev];
}

static inline int nblocks(long long n) { return (int)std::min<long long>((n + 511) / 512, (long long)oh::sm_count() * 64); }

__global__ void shim_depth_sources(double2* u, const unsigned char* img, const unsigned char* dimg, const double* didx,
                                   int dtr, double2 rp, double2 cp, long long n, int flag, unsigned int defq) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    const double im = (double)img[t] / 255.0;
    const double di = flag == 1 ? didx[t] : (double)defq - (double)dimg[t];
    const double alpha = (double)img[t] > 0.0 ? 1.0 : 0.0;
    double2 v = make_double2(im * alpha * (di == (double)dtr ? 1.0 : 0.0), 0.0);
    const double2 tmp = cmul(rp, cp);
    u[t] = cmul(v, tmp);
  }
}

__global__ void shim_as(const double2* in, double2* acc, int pnx, long long n, double ppx, double ppy, double ssx, double ssy,
                        double lambda, double k, double d) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(t % pnx), y = (int)(t / pnx);
    const double fxx = (-1.0 / (2.0 * ppx)) + (1.0 / ssx) * (double)x;
    const double fyy = (1.0 / (2.0 * ppy)) - (1.0 / ssy) - (1.0 / ssy) * (double)y;
    double sval = sqrt(1 - (lambda * fxx) * (lambda * fxx) - (lambda * fyy) * (lambda * fyy));
    sval *= k * d;
    double s, c;
    sincos(sval, &s, &c);
    const int mask = ((fxx * fxx + fyy * fyy) < (k * k)) ? 1 : 0;
    double2 uf = make_double2(0.0, 0.0);
    if (mask) uf = cmul(make_double2(c, s), in[t]);
    acc[t] = cadd(acc[t], uf);
  }
}

__global__ void shim_crop(const double2* in, double2* out, int nx, long long n, int x1, int x2, int y1, int y2) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(t % nx), y = (int)(t / nx);
    if (x >= x1 && x <= x2 && y >= y1 && y <= y2) out[t] = in[t];
  }
}

__global__ void shim_fringe(const double2* in, double2* out, int nx, long long n, int sx, int sy, double ssx, double ssy,
                            double ppx, double ppy, double pi) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    double2 shift = make_double2(1.0, 0.0);
    const int r = (int)(t / nx), c = (int)(t % nx);
    if (sy != 0) {
      const double yy = (ssy / 2.0) - ppy * (double)r - ppy;
      const double ph = sy == 1 ? 2.0 * pi * (yy / (4.0 * ppy)) : 2.0 * pi * (-yy / (4.0 * ppy));
      double s, co; sincos(ph, &s, &co);
      shift = cmul(shift, make_double2(co, s));
    }
    if (sx != 0) {
      const double xx = (-ssx / 2.0) - ppx * (double)c - ppx;
      const double ph = sx == -1 ? 2.0 * pi * (-xx / (4.0 * ppx)) : 2.0 * pi * (xx / (4.0 * ppx));
      double s, co; sincos(ph, &s, &co);
      shift = cmul(shift, make_double2(co, s));
    }
    out[t] = cmul(in[t], shift);
  }
}

__global__ void shim_depth_quan(double* didx, const unsigned char* dimg, long long n, int dtr, double d1, double d2,
                                double nd, double farv, double nearv) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    const double src = double(dimg[t]) / 255.0;
    const double dmap = (1.0 - src) * (farv - nearv) + nearv;
    int td;
    if (dtr < nd - 1) td = (dmap >= d1 ? 1 : 0) * (dmap < d2 ? 1 : 0);
    else td = (dmap >= d1 ? 1 : 0) * (dmap <= d2 ? 1 : 0);
    didx[t] = didx[t] + (double)(td * (dtr + 1));
  }
}

static void shim_done(cudaError_t e, const char* what) {
  note_launch();
  if (e != cudaSuccess) { t_shim_status = cuda_fail(e, what); }
  else t_shim_status = OH_OK;
}

}  // namespace oh

using namespace oh;

extern "C" {

oh_status oh_shim_last_status(void) { return t_shim_status; }

void cudaFFT(struct CUstream_st* stream, int nx, int ny, oh_c128* in_field, oh_c128* output_field, int direction,
             bool bNormalized) {
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  oh_ctx* ctx = shim_ctx();
  if (!ctx) { t_shim_status = fail(OH_ERR_CUDA, "cudaFFT: no CUDA device"); return; }
  if (nx < 1 || ny < 1 || !in_field || !output_field) { t_shim_status = fail(OH_ERR_INVALID_ARG, "cudaFFT: bad arguments"); return; }
  CallScope cs(ctx, st);
  if (cs.status() != OH_OK) { t_shim_status = cs.status(); return; }
  // row pass in -> out (x shift), column pass on out (y shift) with the
  // unshifted transform also written back into in_field
  t_shim_status = fft2d_enqueue(ctx, 1, nx, ny, in_field, output_field, in_field, direction == -1 ? -1 : 1, 1,
                                bNormalized ? 1 : 0, st);
}

void cudaDepthHoloKernel(struct CUstream_st* stream, int pnx, int pny, oh_c128* u_o_gpu, unsigned char* img_src_gpu,
                         unsigned char* dimg_src_gpu, double* depth_index_gpu, int dtr, double rand_phase_val_a,
                         double rand_phase_val_b, double carrier_phase_delay_a, double carrier_phase_delay_b,
                         int flag_change_depth_quan, unsigned int default_depth_quan) {
  const long long n = (long long)pnx * pny;
  if (n <= 0) { t_shim_status = OH_OK; return; }
  shim_depth_sources<<<nblocks(n), 512, 0, reinterpret_cast<cudaStream_t>(stream)>>>(
      (double2*)u_o_gpu, img_src_gpu, dimg_src_gpu, depth_index_gpu, dtr, make_double2(rand_phase_val_a, rand_phase_val_b),
      make_double2(carrier_phase_delay_a, carrier_phase_delay_b), n, flag_change_depth_quan, default_depth_quan);
  shim_done(cudaGetLastError(), "cudaDepthHoloKernel");
}

void cudaPropagation_AngularSpKernel(struct CUstream_st* stream, int pnx, int pny, oh_c128* input_d, oh_c128* u_complex,
                                     double ppx, double ppy, double ssx, double ssy, double lambda, double params_k,
                                     double propagation_dist) {
  const long long n = (long long)pnx * pny;
  if (n <= 0) { t_shim_status = OH_OK; return; }
  shim_as<<<nblocks(n), 512, 0, reinterpret_cast<cudaStream_t>(stream)>>>((const double2*)input_d, (double2*)u_complex, pnx, n,
                                                                           ppx, ppy, ssx, ssy, lambda, params_k, propagation_dist);
  shim_done(cudaGetLastError(), "cudaPropagation_AngularSpKernel");
}

void cudaCropFringe(struct CUstream_st* stream, int nx, int ny, oh_c128* in_field, oh_c128* out_field, int cropx1, int cropx2,
                    int cropy1, int cropy2) {
  const long long n = (long long)nx * ny;
  if (n <= 0) { t_shim_status = OH_OK; return; }
  shim_crop<<<nblocks(n), 512, 0, reinterpret_cast<cudaStream_t>(stream)>>>((const double2*)in_field, (double2*)out_field, nx, n,
                                                                             cropx1, cropx2, cropy1, cropy2);
  shim_done(cudaGetLastError(), "cudaCropFringe");
}

void cudaGetFringe(struct CUstream_st* stream, int pnx, int pny, oh_c128* in_field, oh_c128* out_field, int sig_locationx,
                   int sig_locationy, double ssx, double ssy, double ppx, double ppy, double PI) {
  const long long n = (long long)pnx * pny;
  if (n <= 0) { t_shim_status = OH_OK; return; }
  shim_fringe<<<nblocks(n), 512, 0, reinterpret_cast<cudaStream_t>(stream)>>>((const double2*)in_field, (double2*)out_field, pnx, n,
                                                                              sig_locationx, sig_locationy, ssx, ssy, ppx, ppy, PI);
  shim_done(cudaGetLastError(), "cudaGetFringe");
}

void cudaChangeDepthQuanKernel(struct CUstream_st* stream, int pnx, int pny, double* depth_index_gpu,
                               unsigned char* dimg_src_gpu, int dtr, double d1, double d2, double params_num_of_depth,
                               double params_far_depthmap, double params_near_depthmap) {
  const long long n = (long long)pnx * pny;
  if (n <= 0) { t_shim_status = OH_OK; return; }
  shim_depth_quan<<<nblocks(n), 512, 0, reinterpret_cast<cudaStream_t>(stream)>>>(depth_index_gpu, dimg_src_gpu, n, dtr, d1, d2,
                                                                                   params_num_of_depth, params_far_depthmap,
                                                                                   params_near_depthmap);
  shim_done(cudaGetLastError(), "cudaChangeDepthQuanKernel");
}

}  // extern "C"
