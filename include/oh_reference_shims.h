/*
 * oh_reference_shims.h — drop-in replacements for the depth-map CUDA
 * launchers that HologramGenerator's GPU path binds
 * (declared OpenHolo_DepthMap/Hologram/src/HologramGenerator_GPU.cpp:31-150,
 *  defined OpenHolo_DepthMap/Hologram/src/HologramKernel.cu:189-274).
 *
 * Same symbol names, argument order and meaning, same FP64 complex layout
 * (cufftDoubleComplex == oh_c128), so the reference's host code links
 * against liboh_gb300.so unchanged.  Differences that a caller can observe:
 *   - every launcher enqueues on `stream` only (the reference runs cuFFT on
 *     the legacy default stream and synchronises the device inside cudaFFT);
 *   - failures are not silent: the launcher returns early and the message
 *     is available from oh_last_error() / oh_shim_last_status().
 * Device buffers stay caller-owned, as in the reference (init_GPU,
 * HologramGenerator_GPU.cpp:157-185).
 */
#ifndef OH_REFERENCE_SHIMS_H
#define OH_REFERENCE_SHIMS_H

#include <stdbool.h>
#include "oh.h"

#ifdef __cplusplus
extern "C" {
#endif

struct CUstream_st;

/* HologramKernel.cu:189-227: out = fftshift(FFT(fftshift(in))) [/ (nx ny)];
 * direction -1 forward, otherwise inverse.  As in the reference, in_field
 * receives the unshifted transform FFT(fftshift(in)) (it is the cuFFT
 * output buffer there). */
void cudaFFT(struct CUstream_st* stream, int nx, int ny, oh_c128* in_field, oh_c128* output_field,
             int direction, bool bNormalized);

/* HologramKernel.cu:229-236 / depth_sources_kernel :49-72 */
void cudaDepthHoloKernel(struct CUstream_st* stream, int pnx, int pny, oh_c128* u_o_gpu,
                         unsigned char* img_src_gpu, unsigned char* dimg_src_gpu, double* depth_index_gpu,
                         int dtr, double rand_phase_val_a, double rand_phase_val_b,
                         double carrier_phase_delay_a, double carrier_phase_delay_b,
                         int flag_change_depth_quan, unsigned int default_depth_quan);

/* HologramKernel.cu:238-245 / propagation_angularsp_kernel :75-103 */
void cudaPropagation_AngularSpKernel(struct CUstream_st* stream, int pnx, int pny, oh_c128* input_d,
                                     oh_c128* u_complex, double ppx, double ppy, double ssx, double ssy,
                                     double lambda, double params_k, double propagation_dist);

/* HologramKernel.cu:247-254 / cropFringe :106-118 */
void cudaCropFringe(struct CUstream_st* stream, int nx, int ny, oh_c128* in_field, oh_c128* out_field,
                    int cropx1, int cropx2, int cropy1, int cropy2);

/* HologramKernel.cu:256-264 / getFringe :121-166 */
void cudaGetFringe(struct CUstream_st* stream, int pnx, int pny, oh_c128* in_field, oh_c128* out_field,
                   int sig_locationx, int sig_locationy, double ssx, double ssy, double ppx, double ppy,
                   double PI);

/* HologramKernel.cu:266-274 / change_depth_quan_kernel :168-187 */
void cudaChangeDepthQuanKernel(struct CUstream_st* stream, int pnx, int pny, double* depth_index_gpu,
                               unsigned char* dimg_src_gpu, int dtr, double d1, double d2,
                               double params_num_of_depth, double params_far_depthmap,
                               double params_near_depthmap);

/* Status of the last shim call on this host thread (the shims return void). */
oh_status oh_shim_last_status(void);

#ifdef __cplusplus
}
#endif
#endif /* OH_REFERENCE_SHIMS_H */
