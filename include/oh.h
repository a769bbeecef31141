/*
 * oh.h — C ABI of the GB300-native hologram-generation library (liboh_gb300.so).
 *
 * Every entry point takes plain pointers and sizes, returns an oh_status and
 * never calls exit().  Device pointers are caller-owned; temporary device
 * memory lives in a per-context scratch arena.  Work is enqueued on the
 * caller's stream; no call synchronises the host unless its name ends in
 * _host (those copy host buffers in and out and return when the result is on
 * the host).
 *
 * The operators mirror the reference's hot path:
 *   - layered angular-spectrum depth-map CGH + symmetrization encoding
 *       (OpenHolo_DepthMap/Hologram/src/HologramGenerator.cpp:261-294,391-522,
 *        HologramGenerator_GPU.cpp:246-368, HologramKernel.cu:49-187)
 *   - point-cloud Rayleigh-Sommerfeld / Fresnel summation
 *       (OpenHolo_KETI/.../ophgen_pointcloud/ophgen_pointcloud.cpp:195-365,
 *        .../ophgen_pointcloud_gpu/ophgen_pointcloud_gpu.cpp:391-503)
 *   - WRP accumulation + Fresnel-convolution propagation
 *       (OpenHolo_WRP/openwrp_console_ver 1.0/openwrp/WRP.cpp:65-140,
 *        cwo/src/cwo.cpp:2198-2279,2872-2898)
 *   - encoders (OpenHolo_Encoding/fn_encoding.m:29-98, Hologram_WRP.m:57-60)
 * The reference-signature launchers (cudaFFT, cudaDepthHoloKernel, ...) are
 * declared separately in oh_reference_shims.h.
 */
#ifndef OH_GB300_H
#define OH_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum oh_status {
  OH_OK = 0,
  OH_ERR_INVALID_ARG = 1,      /* null pointer, non-positive size, bad enum */
  OH_ERR_UNSUPPORTED_SIZE = 2, /* transform length has no plan (see oh_fft_supported) */
  OH_ERR_CUDA = 3,             /* a CUDA runtime call failed; see oh_last_error() */
  OH_ERR_ALLOC = 4,            /* scratch allocation failed */
  OH_ERR_TIMEOUT = 5,          /* a bounded device-side wait ran out */
  OH_ERR_IO = 6                /* a file could not be read or parsed */
} oh_status;

typedef enum oh_precision { OH_FP32 = 0, OH_FP64 = 1 } oh_precision;

typedef struct oh_ctx oh_ctx;   /* opaque; one per device, thread-safe */

/* Interleaved complex values (same layout as float2/double2, cufftComplex). */
typedef struct oh_c64  { float  x, y; } oh_c64;
typedef struct oh_c128 { double x, y; } oh_c128;

/* ---- context ---------------------------------------------------------- */
oh_status   oh_ctx_create(oh_ctx** ctx, int device);
oh_status   oh_ctx_destroy(oh_ctx* ctx);
/* Bytes currently held by the context's scratch arena. */
size_t      oh_ctx_scratch_bytes(const oh_ctx* ctx);
oh_status   oh_ctx_release_scratch(oh_ctx* ctx);
const char* oh_status_string(oh_status s);
/* Message of the last failing call on this host thread ("" if none). */
const char* oh_last_error(void);
/* Number of kernels this library has launched since load (all contexts). */
uint64_t    oh_kernel_launch_count(void);
/* Per-kernel device timing: while enabled, every kernel this context
 * launches is bracketed by CUDA events on its stream.  oh_ctx_read_timing
 * waits for the recorded events, accumulates milliseconds and launch counts
 * per kernel name, fills up to `cap` entries and returns the number of
 * kernel names (reset != 0 clears the totals). */
oh_status   oh_ctx_set_timing(oh_ctx* ctx, int on);
int         oh_ctx_read_timing(oh_ctx* ctx, int reset, const char** names,
                               double* ms, long* launches, int cap);
const char* oh_version(void);
/* Issue-rate microbenchmarks on `device` (no reference counterpart): the
 * compute-side roofline denominators.  Times eight independent dependency
 * chains per thread over whole waves with CUDA events (best of two after a
 * warm-up) and returns scalar FP32 FMA warp instructions per second (also the
 * peak warp-instruction issue rate), packed two-lane FP32 FMA warp
 * instructions per second, and sin.approx.f32 results per second (the
 * multi-function unit).  sm_mhz_hint (nullable) receives the SM clock implied
 * by the FMA rate at four warp instructions per SM per clock.  Synchronous. */
oh_status   oh_measure_issue_peaks(int device, double* ffma_per_s, double* ffma2_per_s,
                                   double* mufu_per_s, double* sm_mhz_hint);
/* Upper bound on the depth-map layer buffer (the row pass's strips of every
 * depth layer, pny * 2 pnx * 8 bytes per layer at pad 2 in FP32): frames whose
 * layers would exceed it run the row and column passes in chunks of layers,
 * handing the spectrum accumulators on between chunks (FP32 frames with
 * compile-time column lengths and the default render list; others keep one
 * buffer for all layers).  Results are the same either way.  0 restores
 * the default of 8 GiB. */
oh_status   oh_ctx_set_depthmap_layer_limit(oh_ctx* ctx, size_t bytes);
/* Depth-map batches (no reference counterpart): 1 (default) runs a batch
 * whose frames the persistent batch kernel carries (FP32, padded lengths
 * 1024, 1536, 2048, 3072 and 4096 along both axes, evenly spaced layers, the
 * SSB crop of a 2x pad, one layer buffer) as one launch of that kernel; 0
 * runs every batch as per-frame launches.  Results are the same either way. */
oh_status   oh_ctx_set_depthmap_batch_mode(oh_ctx* ctx, int persistent);
/* Error-path test hook (no reference counterpart).  While set, the kernels
 * selected by kernel_mask (1: depth-map column pass, 2: point-sum tensor-core
 * GEMM, 4: tensor-core convolutions, 8: the persistent depth-map batch
 * kernel, outside graph replay) first wait on a device flag that nothing
 * sets, for at most `cycles` SM clocks, and then take their bounded-wait error
 * path: they let their copies and tensor-core operations land, free their
 * tensor memory, set the context's error word and return without writing
 * results, so oh_ctx_device_status reports OH_ERR_TIMEOUT.  cycles = 0 turns
 * the hook off.  For testing the error path; never set in production. */
oh_status   oh_ctx_set_test_stall(oh_ctx* ctx, int kernel_mask, long long cycles);
/* Synchronises `stream` and reports OH_ERR_TIMEOUT if a kernel of this
 * context gave up a bounded wait since the last check (the flag is then
 * cleared); OH_OK otherwise. */
oh_status   oh_ctx_device_status(oh_ctx* ctx, void* stream);

/* ---- FFT ----------------------------------------------------------------
 * Mixed-radix complex FFT (radices 2,3,4,5,8 + generic odd prime), computed
 * in shared memory by this library's own kernels.
 * direction: -1 forward (e^{-2 pi i jk/n}), +1 inverse (unnormalised unless
 * normalize != 0, then scaled by 1/(nx*ny)).
 * shift != 0 computes fftshift(FFT(fftshift(x))) as HologramKernel.cu:10-34,
 * 189-227 does (shift by floor(n/2) on both sides).
 * in == out is allowed. */
int       oh_fft_supported(int n, oh_precision prec);
oh_status oh_fft2d(oh_ctx* ctx, oh_precision prec, int nx, int ny,
                   const void* in, void* out, int direction, int shift,
                   int normalize, void* stream);
/* Batched 1-D transforms along contiguous rows (ny rows of length nx). */
oh_status oh_fft1d_rows(oh_ctx* ctx, oh_precision prec, int nx, int ny,
                        const void* in, void* out, int direction, int normalize,
                        void* stream);

/* ---- depth-map layered angular-spectrum CGH ------------------------------
 * Field order follows HologramParams (HologramGenerator.h:100-120) plus the
 * config_openholo.txt switches that HologramGenerator reads. */
typedef enum oh_phase_mode {
  OH_PHASE_REFERENCE = 0,  /* constant per-layer phase rand_phase (RANDOM_PHASE=0 -> 1+0i) */
  OH_PHASE_ARRAY = 1,      /* per-pixel phase in radians, float32 [pny][pnx] */
  OH_PHASE_SEEDED = 2      /* per-pixel phase 2*pi*u, u from SplitMix64(seed, pixel index) */
} oh_phase_mode;

typedef struct oh_depthmap_params {
  int    pnx, pny;               /* SLM pixel counts (input image size) */
  double ppx, ppy;               /* SLM pixel pitch [m] */
  double lambda;                 /* wavelength [m] */
  double field_lens;             /* FIELD_LENS [m] (viewing-window transform) */
  double near_depthmap, far_depthmap;
  int    num_of_depth;           /* depth levels */
  int    flag_change_depth_quantization;   /* 1: bin dmap into num_of_depth levels */
  int    default_depth_quantization;       /* 256 in the reference config */
  int    transform_viewing_window;         /* 1: z' = -f z/(z-f); 0: z' = z */
  int    pad;                    /* 1: reference grid, 2: 2x zero-padded grid */
  int    sig_location_x, sig_location_y;   /* Encoding_Symmetrization(ivec2(x,y)) */
  int    phase_mode;             /* oh_phase_mode */
  uint64_t seed;                 /* OH_PHASE_SEEDED */
  double rand_phase_re, rand_phase_im;     /* OH_PHASE_REFERENCE constant */
  const int* render_depth;       /* 1-based levels to render (host array); NULL = 1..num_of_depth */
  int    n_render_depth;
} oh_depthmap_params;

/* Fill p with the reference defaults used by config_openholo.txt-like runs. */
void      oh_depthmap_params_default(oh_depthmap_params* p);

/* Parse a config_openholo.txt file (positional format, arithmetic
 * expressions allowed in the pixel-count and pitch lines, as
 * HologramGenerator::readConfig, HologramGenerator.cpp:65-229, reads it).
 * render_depth storage is owned by the library (valid until the next call
 * on this thread). */
oh_status oh_depthmap_read_config(const char* path, oh_depthmap_params* p);

/* Full frame: img/depth uint8 [pny][pnx] on the device, phase float32
 * [pny][pnx] (only for OH_PHASE_ARRAY, else NULL).
 * fringe_out: real fringe [pny][pnx] (float for OH_FP32, double for OH_FP64),
 *   the u255_fringe_ of HologramGenerator (before uint8 normalisation).
 * field_out (nullable): complex hologram h before taking the real part,
 *   [pny][pnx] oh_c64/oh_c128.
 * spectrum_out (nullable): accumulated frequency-domain field U_complex
 *   [P*pny][P*pnx] (P = pad) before encoding. */
oh_status oh_depthmap_generate(oh_ctx* ctx, oh_precision prec,
                               const oh_depthmap_params* p,
                               const uint8_t* img, const uint8_t* depth,
                               const float* phase, void* fringe_out,
                               void* field_out, void* spectrum_out,
                               void* stream);
/* One complex source field instead of the image/depth layers (no reference
 * counterpart; the learned surrogate's second step): field_in [pny][pnx]
 * (oh_c64 for OH_FP32, oh_c128 for OH_FP64, device) taken as a single layer
 * at distance z (the layer's z'), then the same padded angular-spectrum
 * propagation, crop and encoding as oh_depthmap_generate with parameters p
 * (pad, pitch, wavelength, sig_location; the level and phase fields are
 * unused).  The carrier exp(i k z) multiplies the source as it does a layer. */
oh_status oh_depthmap_propagate_field(oh_ctx* ctx, oh_precision prec, const oh_depthmap_params* p,
                                      const void* field_in, double z, void* fringe_out, void* field_out,
                                      void* spectrum_out, void* stream);
/* Same with host buffers, on the given stream; waits for the frame.
 * Page-locked buffers (cudaHostAlloc / cudaHostRegister) are used through
 * their device mappings: the passes read the inputs and write the fringe in
 * host memory, with no copies; pageable ones are copied in and out.  When
 * every buffer is page-locked and the stream is not the legacy default
 * stream, the first call with given parameters and buffers also captures its
 * passes into a CUDA graph that later identical calls replay (the library's
 * per-kernel timing and the test-stall hook turn this off). */
oh_status oh_depthmap_generate_host(oh_ctx* ctx, oh_precision prec,
                                    const oh_depthmap_params* p,
                                    const uint8_t* img_host,
                                    const uint8_t* depth_host,
                                    const float* phase_host,
                                    void* fringe_host, void* stream);
/* Batch of depth-map frames (frames differ in size, layer count, wavelength
 * and every other parameter).  No reference counterpart: the reference
 * generates one frame per call.  Each frame is what oh_depthmap_generate
 * computes for the same arguments (fringe required, field nullable), in
 * array order on `stream`; the scratch is sized once for the largest frame.
 * flags OH_BATCH_GRAPH: the first call with a given frame array (parameters
 * and buffer addresses) runs the frames and also captures them into a CUDA
 * graph; later calls with an identical array launch that graph, reading
 * whatever the input buffers then hold.  Graph mode needs a stream other
 * than the legacy default stream and must not be called while the caller is
 * capturing `stream`; otherwise the frames run without a graph. */
typedef struct oh_depthmap_frame {
  oh_depthmap_params params;
  const uint8_t* img;       /* device [pny][pnx] */
  const uint8_t* depth;     /* device [pny][pnx] */
  const float*   phase;     /* device, OH_PHASE_ARRAY only */
  void*          fringe;    /* device [pny][pnx] float (FP32) / double (FP64) */
  void*          field;     /* nullable */
} oh_depthmap_frame;
#define OH_BATCH_GRAPH 1u
oh_status oh_depthmap_generate_batch(oh_ctx* ctx, oh_precision prec,
                                     const oh_depthmap_frame* frames, int n_frames,
                                     unsigned flags, void* stream);

/* Autotuner of the persistent batch kernel (no reference counterpart).  For
 * each padded length the kernel carries that has square frames in `frames`
 * (same rules as oh_depthmap_generate_batch), times those frames as a batch
 * `reps` times per candidate and keeps the fastest settings: blocks per SM
 * (1, 2), pipeline lag between a frame's passes (0, 1), columns per column
 * block (1, 2), row pairs per row item (1, 2, 4), column blocks per column
 * item (1, 2) and output rows per output item (1, 2, 4, 8), by coordinate
 * descent from the current entry (a change must gain 1 %).  Entries are kept
 * per (padded length, compute capability, SM count) in the context, used by
 * every later batch, and written to the tune file when one is set.  The
 * frames' outputs hold the last trial's results (equal to a normal run's).
 * The FFT radix order is not a tuning parameter: the fused passes fix it
 * (radix-16 first stage over the zero half, a last stage of 256 butterflies
 * per row). */
oh_status oh_depthmap_autotune_batch(oh_ctx* ctx, const oh_depthmap_frame* frames, int n, int reps,
                                     void* stream);
/* The settings batches of padded length padded_len use on the context's
 * device: {blocks per SM, lag, column width, row pairs per item, column
 * blocks per item, output rows per item}; *ms (nullable) = the tuned batch
 * time, 0 for the defaults. */
oh_status oh_depthmap_batch_tuning(oh_ctx* ctx, int padded_len, int settings[6], double* ms);
/* Tune file: loads its entries (if the file exists) and makes later
 * autotune calls rewrite it; NULL or "" sets no file.  One line per entry:
 * key ctas_per_sm lag col_w row_pairs col_blocks out_rows ms. */
oh_status oh_ctx_set_autotune_file(oh_ctx* ctx, const char* path);


/* Layer index per depth byte (256 entries, 0 = no layer), exactly the
 * reference's binning (change_depth_quan_*, HologramGenerator_CPU.cpp:74-103)
 * and the z' of each level (dlevel_transform_).  z_out holds num_of_depth
 * doubles. */
oh_status oh_depthmap_levels(const oh_depthmap_params* p, int16_t lut_out[256],
                             double* z_out);

/* Triangle-mesh hologram by analytic angular spectra (OpenHolo_MeshCGH,
 * fn_genH.m:1-53 with fn_AS_shading.m or, continuous != 0, fn_AS_continuous.m
 * and fn_FindVertexNormalVector.m).  tris: host array [n][9] of vertex
 * coordinates (x1 y1 z1 x2 y2 z2 x3 y3 z3, metres); back-facing triangles
 * (normal z <= 0) contribute nothing.  field: device oh_c128 [ny][nx], the
 * hologram fftshift(fft2(fftshift(G))); spectrum (nullable): the summed
 * angular spectrum G.  FP64 only; pitches must exceed the wavelength. */
typedef struct oh_mesh_params {
  int    nx, ny;
  double dx, dy, lambda;
  double illu[3];           /* shadingParam.illu */
  int    continuous;        /* shadingParam.con */
} oh_mesh_params;
oh_status oh_mesh_hologram(oh_ctx* ctx, const oh_mesh_params* p, const double* tris, int n_tris,
                           void* field, void* spectrum, void* stream);

/* Light field to complex field (fn_convertLightField2ComplexField.m:1-11,
 * LF-CGH): view (s, t) of the light field, times exp(i phase), becomes the
 * centred 2-D FFT (fftshift(fft2(ifftshift(.))), fn_myfft2.m) in block rows
 * t nv.., columns s nu.. of field [nt*nv][ns*nu] (oh_c64 for OH_FP32, oh_c128
 * for OH_FP64).  lf and phase: float [nt][ns][nv][nu] on the device; phase in
 * radians replaces MATLAB's 2*pi*rand, or is NULL for the seeded generator
 * 2 pi u24(seed, index) (SplitMix64, the same generator as the depth map's
 * seeded phase). */
oh_status oh_lightfield_to_field(oh_ctx* ctx, oh_precision prec, int nu, int nv, int ns, int nt,
                                 const float* lf, const float* phase, uint64_t seed,
                                 void* field, void* stream);

/* Eye-model reconstruction of a fringe (HologramGenerator::ReconstructImage,
 * HologramGenerator_CPU.cpp:414-614), one frame: propagation to the eye pupil
 * through the field lens, eye position shift, eye lens focused at
 * focus_distance with its anti-aliasing and pupil masks, propagation to the
 * retina; out = magnitude [pny/s][pnx/s] (s = pixel_scale, the reference's
 * test_pixel_number_scale).  fringe: real [pny][pnx] (float / double), read as
 * the first (pnx/s)(pny/s) values in row-major order as the reference does.
 * A focus or eye-position sweep is one call per value. */
typedef struct oh_eye_params {
  int    pnx, pny;             /* SLM pixels (before scaling) */
  double ppx, ppy;             /* SLM pitch */
  double lambda;
  double field_lens;           /* FIELD_LENS */
  int    pixel_scale;          /* test_pixel_number_scale (>= 1) */
  double eye_length, eye_pupil_diameter;
  double eye_center_x, eye_center_y;
  double focus_distance;
} oh_eye_params;
oh_status oh_reconstruct_eye(oh_ctx* ctx, oh_precision prec, const oh_eye_params* p,
                             const void* fringe, void* out, void* stream);

/* ---- point cloud -----------------------------------------------------------
 * Field order mirrors OphSpec (ophgen_pointcloud.h:45-70). */
typedef struct oh_pc_params {
  double scale_x, scale_y, scale_z;   /* pointCloudScale{X,Y,Z} */
  double offset_depth;                /* offsetDepth */
  double pitch_x, pitch_y;            /* samplingPitch{X,Y} */
  int    nx, ny;
  double lambda;
  double tilt_x_deg, tilt_y_deg;      /* tiltAngle{X,Y} in degrees */
} oh_pc_params;

/* Points are float4 (x, y, z, amplitude) in scene units before scaling.
 * field_out (nullable): complex field sum_j a_j exp(i phi_j) [ny][nx],
 * fringe_out (nullable): KETI fringe, dst += sum_j a_j cos(phi_j) [ny][nx]
 *   (accumulated into the caller's buffer, as the reference does).
 * phi_j = k r_j - k X sin(tx) - k Y sin(ty), r exact.
 * Precision: OH_FP32 -> oh_c64/float outputs, OH_FP64 -> oh_c128/double. */
oh_status oh_pointcloud(oh_ctx* ctx, oh_precision prec, const oh_pc_params* p,
                        const float* xyza, int n_points, void* field_out,
                        void* fringe_out, void* stream);
/* Host-buffer form (the ophGenCghPointCloud drop-in path). */
oh_status oh_pointcloud_host(oh_ctx* ctx, oh_precision prec,
                             const oh_pc_params* p, const float* xyza_host,
                             int n_points, void* field_host, void* fringe_host,
                             void* stream);

/* Allocation-free point-cloud summation (FP32).  This entry point has no
 * counterpart in the reference.  It exists for callers that cannot allocate
 * device memory once they are running: an SLM or display loop working under
 * a fixed device-memory budget, or a host framework that owns every device
 * allocation through its own pool, where a cudaMalloc inside the library
 * would synchronise the device or fail.  It takes no context and calls no
 * cudaMalloc, cudaFree or other allocating routine: its working tables live
 * in a file-scope device array of OH_PC_NOALLOC_SCRATCH_BYTES (16 MiB) that
 * every GPU loading the library holds until the process exits.
 *   - Limit: fields with 2*nx + 3*ny <= 65532 (at least 64 points per table
 *     chunk); larger fields are rejected with OH_ERR_UNSUPPORTED_SIZE.  Any
 *     number of points is accepted (processed in chunks).
 *   - The first call on a device looks up the array's device address
 *     (cudaGetSymbolAddress) with that device current; make that first call
 *     before any stream capture.  The address is cached per CUDA context,
 *     so after a device reset the next call looks it up again (again
 *     outside any capture).
 *   - Every call shares the one array and leaves the last call's tables in
 *     it; calls that overlap on the GPU (different streams or host threads)
 *     race on it.  Outputs are written in full (field) or accumulated
 *     (fringe, as oh_pointcloud does), so no state needs clearing.
 * Arguments and results are those of oh_pointcloud with OH_FP32. */
#define OH_PC_NOALLOC_SCRATCH_BYTES (16u << 20)
oh_status oh_pointcloud_noalloc(const oh_pc_params* p, const float* xyza, int n_points,
                                void* field_out, void* fringe_out, void* stream);

/* ---- tensor-core convolutions (the learned surrogate's building blocks) ----
 * No reference counterpart.  NHWC BF16 tensors on the device with channel
 * strides x_cs / mask_cs / out_cs (elements, multiples of 8; tensors 16-byte
 * aligned), n images of h x w pixels; widths below 128 must divide 128.
 * oh_conv2d_bf16: out[p][co] = act(bias[co] + sum_{t, ci} x[p + sign*off_t][ci] W[co][t*cin + ci])
 *   taps 9 (3x3, zero padding 1; off_t = (t%3 - 1, t/3 - 1)) or 1; cin and
 *   cout multiples of 32 (cout <= 1024); W BF16 [cout][taps*cin]; bias FP32
 *   or NULL; relu != 0 applies max(., 0); mask (nullable) zeroes outputs
 *   where mask[p][co] <= 0.  sign = -1 with W[ci][t*cout + co] (the layer's
 *   weights transposed) gives the gradient with respect to the layer input.
 *   FP32 accumulation on the tcgen05 tensor cores, BF16 output.
 * oh_conv2d_wgrad_bf16: dwt[t*cin + ci][co] += sum_p x[p + off_t][ci] dz[p][co]
 *   (FP32, accumulated: zero it first); cout 32, 64, 128 or 256; widths
 *   below 64 must divide 64. */
oh_status oh_conv2d_bf16(oh_ctx* ctx, int taps, int sign, int n, int h, int w, int cin, int cout,
                         const void* x, int x_cs, const void* wmat, const float* bias, int relu,
                         const void* mask, int mask_cs, void* out, int out_cs, void* stream);
oh_status oh_conv2d_wgrad_bf16(oh_ctx* ctx, int taps, int n, int h, int w, int cin, int cout,
                               const void* x, int x_cs, const void* dz, int dz_cs, float* dwt,
                               void* stream);

/* ---- learned surrogate: U-Net (no reference counterpart) ---------------------
 * A 4-level U-Net mapping an RGB-D frame to the complex mid-plane field of the
 * plain layered angular-spectrum method: encoder levels of 32, 64, 128 and
 * 256 channels (3x3 convolution + ReLU, twice; 2x2 average pooling between
 * levels), decoder levels that upsample (nearest, 2x), concatenate the
 * encoder output of the same level and apply two 3x3 convolutions + ReLU, and
 * a 1x1 head to 2 channels (re, im).  BF16 weights and activations, FP32
 * accumulation on the tcgen05 tensor cores, FP32 master weights, Adam.
 * Input: rgbd uint8 [n][h][w][4] on the device (R, G, B and a depth byte; the
 * depth channel is depth_lut[byte]); output: field float2 [n][h][w] =
 * out_scale * (head output).  h and w multiples of 8; level widths w >> l
 * below 128 must divide 128.  The network owns its device memory (weights,
 * optimizer state and the activations of max_batch frames of
 * max_height x max_width), allocated by oh_unet_create.
 * Parameters are exchanged as one flat FP32 array, layer by layer (enc0a,
 * enc0b, ..., enc3b, dec2a, dec2b, dec1a, dec1b, dec0a, dec0b, head), each
 * W[cout][taps][cin] then b[cout]; enc0a has cin = 4, dec{l}a has
 * cin = c_l + c_{l+1} (encoder channels first). */
typedef struct oh_unet oh_unet;
typedef struct oh_unet_config {
  int max_batch, max_height, max_width;
  uint64_t seed;                 /* He-normal initial weights from a SplitMix64 stream */
  float out_scale;               /* field units per head output unit */
  float depth_lut[256];          /* depth byte -> input channel 3 */
} oh_unet_config;
void      oh_unet_config_default(oh_unet_config* cfg);
oh_status oh_unet_create(oh_ctx* ctx, const oh_unet_config* cfg, oh_unet** net);
oh_status oh_unet_destroy(oh_unet* net);
size_t    oh_unet_param_count(const oh_unet* net);
/* Synchronous copies of the flat parameter array (set also resets Adam). */
oh_status oh_unet_get_params(oh_unet* net, float* host);
oh_status oh_unet_set_params(oh_unet* net, const float* host);
/* Inference: field_out float2 [n][h][w] (device). */
oh_status oh_unet_forward(oh_unet* net, const uint8_t* rgbd, int n, int h, int w, void* field_out,
                          void* stream);
/* Forward and backward pass of a batch against target float2 [n][h][w]
 * (device): loss = mean over pixels and both components of
 * (head output - target / out_scale)^2, written to loss_out (device float,
 * nullable); the gradients stay in the network (oh_unet_get_grads copies
 * them out in the flat parameter layout, synchronously). */
oh_status oh_unet_compute_grads(oh_unet* net, const uint8_t* rgbd, const void* target, int n, int h,
                                int w, float* loss_out, void* stream);
oh_status oh_unet_get_grads(oh_unet* net, float* host);
/* Adam update from the last computed gradients (bias-corrected). */
oh_status oh_unet_adam_step(oh_unet* net, float lr, float beta1, float beta2, float eps, void* stream);
/* compute_grads + adam_step (beta1 0.9, beta2 0.999, eps 1e-8). */
oh_status oh_unet_train_step(oh_unet* net, const uint8_t* rgbd, const void* target, int n, int h, int w,
                             float lr, float* loss_out, void* stream);

/* Seeded synthetic RGB-D frames (training and test inputs; no reference
 * counterpart): rgbd uint8 [n][h][w][4], frame f from seed + f.  R, G and B
 * are sums of 20 Gaussians (SplitMix64 streams 3, 1 and 5; centres uniform
 * over the frame, sigma 20-200 px times min(h, w)/1080, amplitude 0.2-1),
 * each scaled by its maximum to 0-255; the depth byte is a sum of 8 broad
 * Gaussians (stream 2, sigma 200-600 px scaled) rescaled min..max to 0-255.
 * FP32 evaluation (the FP64 twin may differ by one level at rounding ties). */
oh_status oh_scene_rgbd(oh_ctx* ctx, uint64_t seed, int n, int h, int w, uint8_t* rgbd, void* stream);

/* The learned surrogate around the plain layered angular-spectrum method.
 * dm: the plain frame's parameters (pnx x pny is the network's frame; the G
 * byte of rgbd is the intensity image and the depth byte the depth map;
 * the source phase is the reference constant 1).  z_mid: the mid plane.
 * oh_surrogate_mid_field: the plain method's field on the mid plane (its
 *   layers propagated over z' - z_mid, full spectrum) -> oh_c64 [pny][pnx];
 *   the network's training target.
 * oh_surrogate_generate: the network's mid-plane field, carried over z_mid
 *   to the hologram plane with the plain frame's padding, crop and encoding
 *   (fringe_out float [pny][pnx]; field_mid_out, nullable, receives the
 *   mid-plane field used).  check != 0 also computes the plain mid-plane
 *   field, reports the PSNR of the mid-plane intensity |F|^2 (peak: the plain
 *   field's maximum intensity) and the complex errors relative to it, and
 *   when the PSNR is below psnr_threshold_db uses the plain field for this
 *   frame (fell_back = 1); with check the call synchronises `stream` to read
 *   the comparison. */
typedef struct oh_surrogate_params {
  oh_depthmap_params dm;
  double z_mid;
  float  psnr_threshold_db;
  int    check;
} oh_surrogate_params;
typedef struct oh_surrogate_report {
  int   checked, fell_back;
  float psnr_db;          /* mid-plane intensity PSNR against the plain method */
  float rel_err;          /* ||F_net - F|| / ||F|| */
  float max_abs_err;      /* max |F_net - F| / max |F| */
  float rms_err;          /* rms |F_net - F| / max |F| */
} oh_surrogate_report;
oh_status oh_surrogate_mid_field(oh_ctx* ctx, const oh_depthmap_params* p, double z_mid, const uint8_t* rgbd,
                                 void* field_mid, void* stream);
oh_status oh_surrogate_generate(oh_ctx* ctx, oh_unet* net, const oh_surrogate_params* sp, const uint8_t* rgbd,
                                void* fringe_out, void* field_mid_out, oh_surrogate_report* rep, void* stream);

/* ---- propagation in the MATLAB tools' forms --------------------------------
 * OH_PROP_FRESNEL_TF (FresnelPropagation.m:1-16): ifft2(fft2(U) .* H) with
 *   H = exp(i k z) exp(-i pi lambda z (fx^2 + fy^2)) on the FFT-ordered grid; no padding.
 * OH_PROP_AS_BANDLIMITED (fn_FresnelPropagation_as.m:1-48): 2x zero pad with
 *   the field at (round(ny/2)-1, round(nx/2)-1), centred FFT, angular-spectrum
 *   kernel exp(i 2 pi z sqrt(1/lambda^2 - a^2 - b^2)) with the Matsushima band
 *   limit, centred inverse FFT, crop.
 * In place on field [ny][nx] (oh_c64 for OH_FP32, oh_c128 for OH_FP64). */
#define OH_PROP_FRESNEL_TF 0
#define OH_PROP_AS_BANDLIMITED 1
oh_status oh_propagate(oh_ctx* ctx, oh_precision prec, int method, int nx, int ny,
                       double dx, double dy, double z, double lambda,
                       void* field, void* stream);

/* ---- point-light-source summation (cwoPLS) -------------------------------
 * The per-pixel point sums of CWO++'s cwoPLS class
 * (OpenHolo_WRP/openwrp_console_ver 1.0/cwo/src/cwoPLS.cpp), pixel (i, j):
 *   dx = (j - nx/2) dst_px + dst_ox - (x_k + src_ox)
 *   dy = (i - ny/2) dst_py + dst_oy - (y_k + src_oy),   dz = z_k + z
 *   OH_PLS_HUYGENS     (cwoPLS.cpp:316-368)  U = sum_k exp(i (k r + ph)) / r
 *   OH_PLS_FRESNEL     (cwoPLS.cpp:370-424)  U = sum_k exp(i (k (dx^2+dy^2)/(2 dz) + ph))
 *   OH_PLS_CGH_FRESNEL (cwoPLS.cpp:472-520)  I = sum_k cos(k (dx^2+dy^2)/(2 dz) + ph)
 * (nx/2 = nx >> 1).  Points use the cwoObjPoint layout (cwo_lib.h:469-474).
 * The reference ignores the amplitude a_k; use_amplitude = 1 multiplies each
 * term by it.  out is written (not accumulated): complex [ny][nx] for
 * HUYGENS/FRESNEL, real [ny][nx] for CGH_FRESNEL; oh_c64/float for OH_FP32,
 * oh_c128/double for OH_FP64.
 * Engines (FP32): FRESNEL and CGH_FRESNEL factor into x and y phase tables,
 * U = e^{i ph} Ey^T diag(a) Ex, a complex matrix product over the points;
 * OH_PLS_ENGINE_AUTO runs it on the tensor cores where available (BF16
 * operands split into high and low parts, three products, FP32 accumulation;
 * relative error ~1e-5), OH_PLS_ENGINE_GEMM on the CUDA cores in FP32,
 * OH_PLS_ENGINE_DIRECT evaluates every term.  HUYGENS is always direct. */
typedef struct oh_pls_point { float a_re, a_im; float x, y, z; } oh_pls_point;
typedef enum oh_pls_mode { OH_PLS_HUYGENS = 0, OH_PLS_FRESNEL = 1, OH_PLS_CGH_FRESNEL = 2 } oh_pls_mode;
typedef enum oh_pls_engine {
  OH_PLS_ENGINE_AUTO = 0, OH_PLS_ENGINE_DIRECT = 1, OH_PLS_ENGINE_GEMM = 2, OH_PLS_ENGINE_TENSOR = 3
} oh_pls_engine;
typedef struct oh_pls_params {
  int    nx, ny;
  double dst_px, dst_py;    /* GetDstPx/GetDstPy: hologram pitch */
  double dst_ox, dst_oy;    /* GetDstOx/GetDstOy: hologram offset */
  double src_ox, src_oy;    /* GetOx/GetOy: point offset */
  double lambda;
  double z;                 /* added to every point's z */
  double phase;             /* ph, radians */
  int    mode;              /* oh_pls_mode */
  int    use_amplitude;
  int    engine;            /* oh_pls_engine */
} oh_pls_params;
oh_status oh_pls(oh_ctx* ctx, oh_precision prec, const oh_pls_params* p,
                 const oh_pls_point* pts, int n_points, void* out, void* stream);

/* ---- WRP ------------------------------------------------------------------ */
typedef struct oh_wrp_params {
  int    nx, ny;          /* WRP / hologram grid */
  double pitch;           /* dpx = dpy */
  double lambda;
  double z_wrp;           /* WRP plane position */
  int    window;          /* 0: reference formula int(|lambda dz/(2p^2)+0.5|)*2-1, >0: fixed half-width */
} oh_wrp_params;
/* OPHWRP::SingleWRP (WRP.cpp:75-140): points double3 (x,y,z); adds into wrp
 * (caller zeroes it, as CWO::Create does). */
oh_status oh_wrp_accumulate(oh_ctx* ctx, oh_precision prec,
                            const oh_wrp_params* p, const double* xyz,
                            int n_points, void* wrp, void* stream);
/* MATLAB fn_wrp (fn_wrp.m:13-36): per point an odd N x N window,
 * N = round(|lambda dz / pitch^2 / 2| + 0.5) * 2 - 1, dz = z_wrp - z, of
 * exp(i phase[k]) exp(i k r) / r (r signed with dz, no +0.05), centred at
 * (round(x/pitch) + (res-1)/2, round(y/pitch) + (res-1)/2) (1-based, first
 * index along x), added into holo [res][res] (caller zeroes it).  phase
 * (radians, nullable = 0) replaces MATLAB's rand * 2 pi.  Points are double3. */
oh_status oh_wrp_matlab(oh_ctx* ctx, oh_precision prec, int res, double pitch, double lambda,
                        double z_wrp, const double* xyz, const double* phase, int n_points,
                        void* holo, void* stream);
/* Texture/depth WRP, cwoTexDep::WRP (cwoTexDep.cpp:29-136).  tex, dep:
 * uint8 [ny][nx] on the device (dep nullable); field [ny][nx] accumulated
 * (oh_c64 for OH_FP32, oh_c128 for OH_FP64).
 *   OH_TEXDEP_SINGLE: WRP(z), full zone plates of half-width
 *     int(|z| tan(asin(lambda/(2 px))) / px); r = z + rho^2 / (2 z).
 *   OH_TEXDEP_RANGE: WRP(z, dz_step, {range_lo, range_hi}), texels with dep in
 *     [lo, hi), dz = z + (hi - dep) dz_step, half zone plates (wy < 0) of
 *     half-width int(int(...) / 1.4), r = rho^2 / (2 dz).  dep_from_texture = 1
 *     reproduces the reference, which takes dep from the texture value when
 *     a depth image is given (0 without one); 0 reads dep from the depth image. */
#define OH_TEXDEP_SINGLE 0
#define OH_TEXDEP_RANGE 1
typedef struct oh_texdep_params {
  int    nx, ny;
  double px, py, lambda;
  double z, dz_step;
  int    range_lo, range_hi;
  int    dep_from_texture;
} oh_texdep_params;
oh_status oh_texdep_wrp(oh_ctx* ctx, oh_precision prec, int mode, const oh_texdep_params* p,
                        const uint8_t* tex, const uint8_t* dep, void* field, void* stream);

/* CWO::Diffract(z, CWO_FRESNEL_CONV) with the default zero-pad expansion
 * (cwo.cpp:2198-2279, 2872-2898), in place on field [ny][nx]. */
oh_status oh_fresnel_propagate(oh_ctx* ctx, oh_precision prec, int nx, int ny,
                               double pitch, double lambda, double z,
                               void* field, void* stream);

/* ---- encoders ------------------------------------------------------------- */
typedef enum oh_encoding {
  OH_ENC_REAL = 0,            /* real(U) */
  OH_ENC_PHASE_TO_AMP = 1,    /* angle(U) + pi/(2*pi) (fn_encoding.m:57) */
  OH_ENC_NUM_INTERFERENCE = 2,/* |U + max|U||^2 / max */
  OH_ENC_BURCKHARDT = 3,      /* [ny][3nx] */
  OH_ENC_TWO_PHASE = 4,       /* [ny][2nx] */
  OH_ENC_SSB_LEFT = 5, OH_ENC_SSB_RIGHT = 6, OH_ENC_SSB_TOP = 7, OH_ENC_SSB_BOTTOM = 8,
  OH_ENC_PHASE_ONLY_U8 = 9,   /* uint8(255*(angle+pi)/max(angle+pi)) (Hologram_WRP.m:57-60) */
  OH_ENC_AMPLITUDE = 10       /* |U| */
} oh_encoding;
/* field: complex [ny][nx]; out: float/double (or uint8 for PHASE_ONLY_U8). */
oh_status oh_encode(oh_ctx* ctx, oh_precision prec, int kind, int nx, int ny,
                    const void* field, void* out, void* stream);
/* min/max normalisation to uint8 as HologramGenerator::Write_Result_image
 * (truncating, HologramGenerator.cpp:528-565) when round_half == 0, or
 * ophNormalize with +0.5 rounding and vertical flip (oph_common.cpp:92-115)
 * when round_half != 0. */
oh_status oh_normalize_u8(oh_ctx* ctx, oh_precision prec, int nx, int ny,
                          const void* in, uint8_t* out, int round_half,
                          void* stream);

#ifdef __cplusplus
}
#endif
#endif /* OH_GB300_H */
