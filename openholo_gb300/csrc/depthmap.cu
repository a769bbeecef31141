// Layered angular-spectrum depth-map CGH with symmetrization encoding.
//
// Reference path (OpenHolo_DepthMap/Hologram/src):
//   GetDepthValues / change_depth_quan   HologramGenerator.cpp:391-417, HologramKernel.cu:168-187
//   TransformViewingWindow                HologramGenerator.cpp:423-435
//   Calc_Holo_GPU                         HologramGenerator_GPU.cpp:246-302
//     per layer: depth_sources_kernel (mask * rand_phase * carrier) -> cudaFFT
//     (fftshift.FFT.fftshift) -> propagation_angularsp_kernel (U += H*F)
//   Encoding_Symmetrization / encoding_GPU HologramGenerator.cpp:481-522, HologramGenerator_GPU.cpp:338-368
//     cropFringe -> cudaFFT(inverse, 1/N) -> getFringe -> real part
//
// GB300 structure (4 launches per frame, whatever the layer count):
//   dm_setup     per-layer tables (FP64 phase reduction, rounded to the
//                compute precision) and per-frame flags
//   dm_row_pass  one block per image row: builds every layer's masked source
//                row on the fly from the uint8 image/depth bytes, x-FFTs only
//                the layers present in that row and stores them column-strip
//                tiled; absent (layer,row) pairs are flagged, not written
//   dm_col_pass  one block per strip of W spectrum columns: for every layer
//                y-FFT + angular-spectrum multiply-accumulate into registers;
//                then SSB crop, inverse y-FFT, keep the output rows, apply the
//                y shift phase and 1/N
//   dm_out_pass  one block per output row: inverse x-FFT, crop the padding,
//                x shift phase, real part
// The 2x zero-padding (pad = 2) never materialises: padded rows are skipped
// and padded columns are zeros written straight into shared memory.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cmath>
#include <cstring>
#include <type_traits>
#include <vector>
#include "context.h"
#include "dm_batch.h"
#include "dm_kernels.cuh"

namespace oh {

template <typename R, int KMAX, int NY>
__global__ void __launch_bounds__(512) dm_col_pass(DMArgs<R> a) {
  typedef typename cplx_of<R>::type C;
  extern __shared__ unsigned char smem_raw[];
  const int W = a.W;
  const int Py = a.Py;
  C* buf = reinterpret_cast<C*>(smem_raw);
  C* exw = buf + (size_t)Py * W;                  // [W]
  R* lfxw = reinterpret_cast<R*>(exw + W);        // [W]
  int* kyp = reinterpret_cast<int*>(lfxw + W);    // [Py] spectrum row held at storage position
  const int s = blockIdx.x;
  const int kx0 = s * W;
  const int T = blockDim.x;
  const int nel = Py * W;
  for (int p = threadIdx.x; p < Py; p += T) {
    int ky = a.ply.iperm[p] + a.hy; if (ky >= Py) ky -= Py;   // S[ky] = B[(ky - hy) mod Py]
    kyp[p] = ky;
  }
  for (int w = threadIdx.x; w < W; w += T) lfxw[w] = a.lfx[kx0 + w];
  C acc[KMAX];
#pragma unroll
  for (int k = 0; k < KMAX; ++k) acc[k] = mk((R)0, (R)0);
  __syncthreads();

  for (int e = 0; e < a.n_entries; ++e) {
    const int u = a.uslot_of_entry[e];
    if (!a.slot_any[u]) continue;
    const uint8_t* occ = a.occ + (size_t)u * a.occ_stride;
    const C* src = a.Rbuf + ((size_t)u * a.nstrips + s) * a.pny * W;
    for (int idx = threadIdx.x; idx < nel; idx += T) {
      const int i = idx / W, w = idx - i * W;
      int y = i - a.hy; if (y < 0) y += Py;
      const int yl = y - a.oy;
      C val = mk((R)0, (R)0);
      if (yl >= 0 && yl < a.pny && occ[yl]) val = src[(size_t)yl * W + w];
      buf[idx] = val;
    }
    if constexpr (sizeof(R) == 4) {
      for (int w = threadIdx.x; w < W; w += T) exw[w] = a.exc[(size_t)e * a.Px + kx0 + w];
    } else {
      for (int w = threadIdx.x; w < W; w += T) exw[w] = a.cst[e];
    }
    block_fft_n<NY, -1>(buf, W, 1, W, a.ply, true);
    const R kz = a.kzp[e];
    const C* eyr = a.ey + (size_t)e * Py;
#pragma unroll
    for (int k = 0; k < KMAX; ++k) {
      const int idx = threadIdx.x + k * T;
      if (idx < nel) {
        const int p = idx / W, w = idx - p * W;
        const int ky = kyp[p];
        const R sv = lfxw[w] + a.lfy[ky];
        C h;
        if constexpr (sizeof(R) == 4) {
          // residual of k z' (1 - sqrt(1-s)) beyond the separable s/2 term:
          // k z' s^2 / (2 (1 + sqrt(1-s))^2), |.| < a few rad
          const R rt = sqrt((R)1 - sv);
          const R den = (R)1 + rt;
          const R psi = kz * sv * sv / ((R)2 * den * den);
          float sn, cs;
          __sincosf(psi, &sn, &cs);
          C g = cmul(exw[w], eyr[ky]);
          h = cmul(g, mk(cs, sn));
        } else {
          // direct reference formula H = exp(i k d sqrt(1 - s)), d = -z'
          const double sval = sqrt(1.0 - (double)sv) * (-(double)kz);
          double sn, cs;
          sincos(sval, &sn, &cs);
          h = cmul(exw[w], mk((R)cs, (R)sn));
        }
        acc[k] = cadd(acc[k], cmul(h, buf[idx]));
      }
    }
    __syncthreads();
  }

  // SSB crop + move the spectrum into the inverse-transform input order:
  // b[i] = Uc[(i - hy) mod Py]  ->  spectrum row ky goes to i = (ky + hy) mod Py
#pragma unroll
  for (int k = 0; k < KMAX; ++k) {
    const int idx = threadIdx.x + k * T;
    if (idx < nel) {
      const int p = idx / W, w = idx - p * W;
      const int ky = kyp[p];
      const int kx = kx0 + w;
      if (a.spectrum) a.spectrum[(size_t)ky * a.Px + kx] = acc[k];
      const bool keep = kx >= a.cx1 && kx <= a.cx2 && ky >= a.cy1 && ky <= a.cy2;
      int i = ky + a.hy; if (i >= Py) i -= Py;
      // each storage slot is written exactly once (ky is a permutation)
      buf[i * W + w] = keep ? acc[k] : mk((R)0, (R)0);
    }
  }
  block_fft_n<NY, 1>(buf, W, 1, W, a.ply, true);
  for (int idx = threadIdx.x; idx < a.pny * W; idx += T) {
    const int yl = idx / W, w = idx - yl * W;
    int m = a.oy + yl - a.hy; if (m < 0) m += Py;   // out[y] = B[(y - hy) mod Py]
    const C val = cmul(buf[a.ply.perm[m] * W + w], a.shy[yl]);
    a.V[(size_t)yl * a.Px + kx0 + w] = val;
  }
}

// ---------------------------------------------------------------------------
// host side

struct Levels {
  double dstep;
  std::vector<double> dlevel;     // num_of_depth entries
  std::vector<double> ztrans;     // z' per level
  int16_t lut[256];               // depth byte -> level index dtr (1-based), 0 = none
};

// GetDepthValues (HologramGenerator.cpp:391-408) with the per-pixel binning
// of change_depth_quan_* evaluated once per depth byte.  The level list is
// built by repeated addition while val <= far, as the reference does; when
// rounding stops it one level short of num_of_depth the addition continues
// (the reference would read past the end of dlevel_ there).
static oh_status compute_levels(const oh_depthmap_params* p, Levels* L) {
  const double nearv = std::min(p->near_depthmap, p->far_depthmap);
  const double farv = std::max(p->near_depthmap, p->far_depthmap);
  const int nd = p->num_of_depth;
  L->dlevel.clear();
  if (nd > 1) {
    L->dstep = (farv - nearv) / (nd - 1);
    double val = nearv;
    while (val <= farv && (int)L->dlevel.size() < nd) { L->dlevel.push_back(val); val += L->dstep; }
    while ((int)L->dlevel.size() < nd) { L->dlevel.push_back(val); val += L->dstep; }
  } else {
    L->dstep = (farv + nearv) / 2;
    L->dlevel.push_back(farv - nearv);
  }
  L->ztrans.resize(nd);
  for (int i = 0; i < nd; ++i) {
    const double d = L->dlevel[i];
    L->ztrans[i] = p->transform_viewing_window ? -p->field_lens * d / (d - p->field_lens) : d;
  }
  for (int b = 0; b < 256; ++b) {
    long idx;
    if (p->flag_change_depth_quantization == 1) {
      const double dmap_src = double(b) / 255.0;
      const double dmap = (1.0 - dmap_src) * (farv - nearv) + nearv;
      idx = 0;
      for (int dtr = 0; dtr < nd; ++dtr) {
        const double t = L->dlevel[dtr];
        const double d1 = t - L->dstep / 2.0;
        const double d2 = t + L->dstep / 2.0;
        int hit;
        if (dtr < nd - 1) hit = (dmap >= d1 ? 1 : 0) * (dmap < d2 ? 1 : 0);
        else hit = (dmap >= d1 ? 1 : 0) * (dmap <= d2 ? 1 : 0);
        idx += (long)hit * (dtr + 1);
      }
    } else {
      idx = (long)p->default_depth_quantization - b;
    }
    L->lut[b] = (idx >= 1 && idx <= 32767) ? (int16_t)idx : (int16_t)0;
  }
  return OH_OK;
}

static oh_status validate(const oh_depthmap_params* p) {
  if (!p) return fail(OH_ERR_INVALID_ARG, "null depth-map params");
  if (p->pnx < 1 || p->pny < 1) return fail(OH_ERR_INVALID_ARG, "pnx/pny must be positive");
  if (p->pad != 1 && p->pad != 2) return fail(OH_ERR_INVALID_ARG, "pad must be 1 or 2");
  if (!(p->ppx > 0) || !(p->ppy > 0) || !(p->lambda > 0)) return fail(OH_ERR_INVALID_ARG, "pitch and wavelength must be positive");
  if (p->num_of_depth < 1 || p->num_of_depth > 4096) return fail(OH_ERR_INVALID_ARG, "num_of_depth out of range");
  if (p->phase_mode < 0 || p->phase_mode > 2) return fail(OH_ERR_INVALID_ARG, "bad phase_mode");
  if (p->sig_location_x < -1 || p->sig_location_x > 1 || p->sig_location_y < -1 || p->sig_location_y > 1)
    return fail(OH_ERR_INVALID_ARG, "sig_location components must be -1, 0 or 1");
  if (p->render_depth && p->n_render_depth < 1) return fail(OH_ERR_INVALID_ARG, "empty render_depth list");
  return OH_OK;
}

// Enqueues one frame.  With info set, fills it (scratch needs, arguments,
// set-up constants, pass configuration) and returns without allocating or
// launching anything.
// src (nullable): a complex source field [pny][pnx] (oh_c64 / oh_c128) taken
// as the one layer, at z' = src_z, instead of the image/depth layers.
template <typename R, int KMAX>
static oh_status run_depthmap(oh_ctx* ctx, const oh_depthmap_params* p, const uint8_t* img,
                              const uint8_t* depth, const float* phase, void* fringe, void* field,
                              void* spectrum, cudaStream_t st, FrameInfo<R>* info = nullptr,
                              const void* src = nullptr, double src_z = 0.0) {
  typedef typename cplx_of<R>::type C;
  const int prec = sizeof(R) == 8 ? 1 : 0;
  Levels L;
  OH_TRY(compute_levels(p, &L));
  int nd = p->num_of_depth;
  std::vector<int> render;
  if (src) {
    nd = 1;
    L.ztrans.assign(1, src_z);
    for (int b = 0; b < 256; ++b) L.lut[b] = 0;
    render.push_back(1);
  } else if (p->render_depth) render.assign(p->render_depth, p->render_depth + p->n_render_depth);
  else for (int i = 1; i <= nd; ++i) render.push_back(i);
  if ((int)render.size() > kMaxEntries) return fail(OH_ERR_INVALID_ARG, "more than 256 render_depth entries");
  for (int d : render) if (d < 1 || d > nd) return fail(OH_ERR_INVALID_ARG, "render_depth entry outside 1..num_of_depth");

  DMSetup su;
  std::memset(&su, 0, sizeof(su));
  std::vector<int> udtr;              // unique level numbers in first-seen order
  std::vector<int> uslot_of_dtr(nd + 1, -1);
  for (size_t e = 0; e < render.size(); ++e) {
    int d = render[e];
    if (uslot_of_dtr[d] < 0) { uslot_of_dtr[d] = (int)udtr.size(); udtr.push_back(d); }
    su.uslot_of_entry[e] = (int16_t)uslot_of_dtr[d];
    const double z = L.ztrans[d - 1];
    su.zp[e] = z;
    const double k = 2.0 * M_PI / p->lambda;
    // rand_phase * carrier exp(i k z') (HologramGenerator_GPU.cpp:267-273)
    double rre = 1.0, rim = 0.0;
    if (p->phase_mode == OH_PHASE_REFERENCE && !src) { rre = p->rand_phase_re; rim = p->rand_phase_im; }
    double cre = std::cos(k * z), cim = std::sin(k * z);
    double are = rre * cre - rim * cim, aim = rre * cim + rim * cre;
    if (prec == 0) {
      // fp32 path folds the constant exp(-i k z') of H into the entry constant
      double hre = std::cos(-k * z), him = std::sin(-k * z);
      double bre = are * hre - aim * him, bim = are * him + aim * hre;
      are = bre; aim = bim;
    }
    su.cre[e] = are; su.cim[e] = aim;
  }
  su.n_entries = (int)render.size();
  su.n_uslots = (int)udtr.size();
  for (int b = 0; b < 256; ++b) {
    int d = L.lut[b];
    su.lut[b] = (d >= 1 && d <= nd) ? (int16_t)uslot_of_dtr[d] : (int16_t)-1;
  }

  DMArgs<R> a;
  std::memset(&a, 0, sizeof(a));
  a.pnx = p->pnx; a.pny = p->pny;
  a.Px = p->pad * p->pnx; a.Py = p->pad * p->pny;
  a.ox = (a.Px - a.pnx) / 2; a.oy = (a.Py - a.pny) / 2;
  a.hx = a.Px / 2; a.hy = a.Py / 2;
  a.n_entries = su.n_entries; a.n_uslots = su.n_uslots;
  a.slot0 = 0; a.slot1 = su.n_uslots; a.e0 = 0; a.e1 = su.n_entries;
  a.chunk_first = 1; a.chunk_last = 1; a.accbuf = nullptr;
  a.ppx = p->ppx; a.ppy = p->ppy;
  a.ssx = p->ppx * a.Px; a.ssy = p->ppy * a.Py;
  a.lambda = p->lambda; a.k = 2.0 * M_PI / p->lambda;
  a.img = img; a.depth = depth; a.phase = phase;
  a.src = static_cast<const C*>(src);
  a.phase_mode = p->phase_mode; a.seed = p->seed;
  a.sig_x = p->sig_location_x; a.sig_y = p->sig_location_y;
  // Encoding_Symmetrization crop window (HologramGenerator.cpp:486-514), on the padded grid
  {
    int cropx1, cropx2, cropy1, cropy2;
    if (p->sig_location_y == 0) { cropy1 = 1; cropy2 = a.Py; }
    else { int cropy = a.Py / 2; cropy1 = cropy - cropy / 2; cropy2 = cropy1 + cropy - 1; }
    if (p->sig_location_x == 0) { cropx1 = 1; cropx2 = a.Px; }
    else { int cropx = a.Px / 2; cropx1 = cropx - cropx / 2; cropx2 = cropx1 + cropx - 1; }
    a.cx1 = cropx1 - 1; a.cx2 = cropx2 - 1; a.cy1 = cropy1 - 1; a.cy2 = cropy2 - 1;
  }
  OH_TRY(get_plan(ctx, a.Px, prec, &a.plx));
  OH_TRY(get_plan(ctx, a.Py, prec, &a.ply));

  const size_t smax = max_smem_per_block();
  const int T = 512;
  const int occ_stride = (a.pny + 15) & ~15;
  a.occ_stride = occ_stride;
  a.err = ctx->dev_err;
  if (ctx->stall_mask & kStallDepthmapColumn) { a.stall_flag = ctx->dev_err + 1; a.stall_cycles = ctx->stall_cycles; }
  // FP32 with a compile-time FFT length: bulk-copy pipelined column pass
  // (dm_col_fast) with the widest strip whose shared-memory layout fits
  int Wfast = 0, col_tab = 0, col_py = a.Py;      // col_py: stored column length of the fast pass
  bool fastlen = false;
  with_fast_n(a.Py, [&](auto nc) { fastlen = decltype(nc)::value > 0; });
  if (prec == 0 && fastlen) {
    // strips of two spectrum columns (two blocks per SM)
    with_fast_n(a.Py, [&](auto nc) {
      if constexpr (decltype(nc)::value > 0) {
        col_tab = col_tab_entries<decltype(nc)::value>();
        col_py = col_len<decltype(nc)::value>();
      }
    });
    if (a.Px % 2 == 0 &&
        (size_t)col_layout(col_py, a.pny, 2, kColStripW, false, occ_stride, su.n_entries, col_tab).total <= smax)
      Wfast = 2;
  }
  int W = Wfast;
  if (W == 0) {
    for (int cand : {8, 4, 2, 1}) {
      if (a.Px % cand) continue;
      size_t sm = (size_t)cand * a.Py * sizeof(C) + cand * (sizeof(C) + sizeof(R)) + (size_t)a.Py * sizeof(int);
      if (sm <= smax && cand * a.Py <= T * KMAX) { W = cand; break; }
    }
  }
  if (W == 0) return fail(OH_ERR_UNSUPPORTED_SIZE, "padded column length " + std::to_string(a.Py) + " too long for the column pass");
  a.W = W; a.nstrips = a.Px / W;
  a.lw = W == 8 ? 3 : W == 4 ? 2 : W == 2 ? 1 : 0;
  a.ey_perm = Wfast ? 1 : 0;
  // Render entries evenly spaced in z' with one entry constant: the fast
  // column pass accumulates with the layer-step recurrence (the transfer
  // function is exp(i z' Phi(fx, fy)) times that constant, so consecutive
  // entries differ by the factor exp(-i dz Phi)).  OH_DM_LAYER_STEP=0 keeps
  // the per-layer evaluation.
  a.horner = 0;
  if (Wfast && su.n_entries >= 2) {
    const char* ev = std::getenv("OH_DM_LAYER_STEP");
    const int n = su.n_entries;
    const double dz = (su.zp[n - 1] - su.zp[0]) / (n - 1);
    const double k = 2.0 * M_PI / p->lambda;
    bool even = dz != 0.0 && !(ev && std::atoi(ev) == 0);
    for (int e = 0; e < n && even; ++e) {
      if (std::fabs(su.zp[e] - (su.zp[0] + e * dz)) * k > 1e-7) even = false;
      if (std::fabs(su.cre[e] - su.cre[0]) > 1e-12 || std::fabs(su.cim[e] - su.cim[0]) > 1e-12) even = false;
    }
    if (even) { a.horner = 1; a.dz = dz; a.kdz_pi = (float)(k * dz / M_PI); }
  }
  bool fastx = false;
  with_fast_n(a.Px, [&](auto nc) { fastx = decltype(nc)::value > 0; });
  a.xs = (prec == 0 && fastx && Wfast) ? 1 : 0;
  int r0x = 0, r0y = 0;
  with_fast_n(a.Px, [&](auto nc) { if constexpr (decltype(nc)::value > 0) r0x = FastSched<decltype(nc)::value>::r0; });
  with_fast_n(a.Py, [&](auto nc) { if constexpr (decltype(nc)::value > 0) r0y = FastSched<decltype(nc)::value>::r0; });
  // Last-stage outputs of the fast column pass that can reach the SSB crop:
  // storage position p = b RL + f holds spectrum row ky = (k_low(b) + (Py/RL) f + hy) mod Py
  // (the last radix is the most significant output digit), k_low < Py/RL.
  a.fkeep = 0xffffffffu;
  if (Wfast && !spectrum) {
    int rl = 0;
    with_fast_n(a.Py, [&](auto nc) { if constexpr (decltype(nc)::value > 0) rl = FastSched<decltype(nc)::value>::rlast; });
    if (rl > 0 && rl <= 32) {
      const int q = a.Py / rl;
      uint32_t m = 0;
      for (int f = 0; f < rl; ++f)
        for (int kl = 0; kl < q; ++kl) {
          const int ky = (kl + q * f + a.hy) % a.Py;
          if (ky >= a.cy1 && ky <= a.cy2) { m |= 1u << f; break; }
        }
      a.fkeep = m;
    }
  }
  a.hzx = (p->pad == 2 && r0x == 16 && (a.Px % 16) == 0 && a.ox * 4 == a.Px && a.hx * 2 == a.Px) ? 1 : 0;
  a.hzy = (p->pad == 2 && r0y == 16 && (a.Py % 16) == 0 && a.oy * 4 == a.Py && a.hy * 2 == a.Py) ? 1 : 0;
  // fast column pass: one-column blocks over the two-column strips where
  // that turns one block per SM into two
  // layer chunks: when the strips of every layer slot would exceed the
  // context's layer-buffer limit, the fast FP32 path runs the row and column
  // passes per chunk of slots, the column pass handing its accumulators on
  // through a buffer of one spectrum (slots must map one to one onto render
  // entries, as with the default render list)
  const size_t per_slot = (size_t)a.pny * a.Px * sizeof(C);
  const size_t nU_ = su.n_uslots, nE_ = su.n_entries;
  size_t lc = nU_;
  bool identity = nU_ == nE_;
  for (size_t e = 0; e < nE_ && identity; ++e) identity = su.uslot_of_entry[e] == (int16_t)e;
  if (Wfast && identity && nU_ > 1 && nU_ * per_slot > ctx->dm_layer_limit)
    lc = std::max<size_t>(1, ctx->dm_layer_limit / per_slot);
  const int nchunks = (int)((nU_ + lc - 1) / lc);
  int wcol = Wfast;
  if (Wfast) {
    bool narrow = false;
    with_fast_n(a.Py, [&](auto nc) {
      if constexpr (decltype(nc)::value > 0) narrow = col_narrow_ok<decltype(nc)::value>();
    });
    const bool step = a.horner != 0;
    auto two_fit = [&](int w) {
      return 2 * ((size_t)col_layout(col_py, a.pny, w, kColStripW, step, occ_stride, su.n_entries, col_tab).total +
                  1024) <= (size_t)228 * 1024;
    };
    const char* ev = std::getenv("OH_DM_COL_NARROW");
    // the extended kernel (layer chunks, test hook) takes whole strips
    const bool ext_mode = (ctx->stall_mask & kStallDepthmapColumn) != 0 || nchunks > 1;
    if (narrow && !(ev && std::atoi(ev) == 0) && !ext_mode && !two_fit(2) && two_fit(1)) wcol = 1;
  }
  // the column pass's two-buffer pipeline (its layer-step SSB form without
  // layer chunks or the test hook, at the lengths where it keeps two blocks
  // per SM): the kernel decides the same way at compile time
  bool col_p2 = false;
  if (Wfast && a.horner) {
    const bool ext_mode = (ctx->stall_mask & kStallDepthmapColumn) != 0 || nchunks > 1;
    with_fast_n(a.Py, [&](auto nc) {
      constexpr int NY = decltype(nc)::value;
      if constexpr (NY > 0)
        col_p2 = a.fkeep == col_ssb_keep<NY>() && !ext_mode && (wcol == 2 ? col_pipe2<NY, 2>() : col_pipe2<NY, 1>());
    });
  }
  const size_t smem_col =
      Wfast ? (size_t)col_layout(col_py, a.pny, wcol, kColStripW, a.horner != 0, occ_stride, su.n_entries, col_tab,
                                 col_p2).total
            : (size_t)W * a.Py * sizeof(C) + W * (sizeof(C) + sizeof(R)) + (size_t)a.Py * sizeof(int);
  int row_tab = 0, row_ls = a.Px;
  with_fast_n_if<sizeof(R) == 4>(a.Px, [&](auto nc) {
    if constexpr (decltype(nc)::value > 0) {
      row_tab = FastSched<decltype(nc)::value>::tab1_entries;
      row_ls = RowPad<decltype(nc)::value>::LSMAX;
    }
  });
  const size_t smem_row = kRowPair * ((size_t)row_ls * sizeof(C) + (size_t)a.pnx * sizeof(C) +
                                      (size_t)((a.pnx + 7) & ~7) * sizeof(int16_t)) +
                          16 * sizeof(uint32_t) + (kTwLo + (size_t)(a.Px + 63) / 64 + row_tab) * sizeof(C);
  const size_t smem_out = (size_t)a.Px * sizeof(C) + (kTwLo + (size_t)(a.Px + 63) / 64) * sizeof(C);
  if (smem_row > smax || smem_out > smax) return fail(OH_ERR_UNSUPPORTED_SIZE, "padded row length " + std::to_string(a.Px) + " exceeds shared memory");

  // scratch
  void* ptr;
  const size_t nE = su.n_entries, nU = su.n_uslots;
  size_t bytes_acc = 0;
  if (nchunks > 1) {
    with_fast_n(a.Py, [&](auto nc) {
      constexpr int NY = decltype(nc)::value;
      if constexpr (NY > 0) {
        const bool step = a.horner != 0;
        const size_t blocks = wcol == 1 ? (size_t)a.Px : (size_t)a.nstrips;
        size_t per_block;
        if (wcol == 1) per_block = step ? (size_t)ColCfg<NY, 1, true>::T * ColCfg<NY, 1, true>::KB * ColCfg<NY, 1, true>::RL
                                        : (size_t)ColCfg<NY, 1, false>::T * ColCfg<NY, 1, false>::KB * ColCfg<NY, 1, false>::RL;
        else per_block = step ? (size_t)ColCfg<NY, 2, true>::T * ColCfg<NY, 2, true>::KB * ColCfg<NY, 2, true>::RL
                              : (size_t)ColCfg<NY, 2, false>::T * ColCfg<NY, 2, false>::KB * ColCfg<NY, 2, false>::RL;
        bytes_acc = blocks * per_block * sizeof(C);
      }
    });
  }
  const size_t bytes_R = std::min(nU, lc) * per_slot, bytes_V = (size_t)a.pny * a.Px * sizeof(C),
               bytes_occ = std::min(nU, lc) * (size_t)occ_stride + 16;
  // small tables share one buffer
  size_t off = 0;
  auto carve = [&](size_t bytes) { size_t o = off; off += (bytes + 255) & ~(size_t)255; return o; };
  size_t o_lut = carve(256 * sizeof(int16_t)), o_use = carve(nE * sizeof(int16_t)), o_kz = carve(nE * sizeof(R)),
         o_cst = carve(nE * sizeof(C)), o_exc = carve(prec ? 0 : nE * a.Px * sizeof(C)),
         o_ey = carve(prec ? 0 : nE * a.Py * sizeof(C)),
         o_eth = carve(a.ey_perm ? nE * a.Py * sizeof(R) : 0), o_lfx = carve(a.Px * sizeof(R)), o_lfy = carve(a.Py * sizeof(R)), o_lfyp = carve(a.Py * sizeof(R)),
         o_shy = carve(a.pny * sizeof(C)), o_shx = carve(a.pnx * sizeof(C)), o_any = carve(nU * sizeof(int)),
         o_dxh = carve(a.horner ? a.Px * sizeof(C) : 0), o_dyh = carve(a.horner ? a.Py * sizeof(C) : 0);
  if (info) {
    info->sz = DMScratch{bytes_R, bytes_V, bytes_occ, off, bytes_acc};
    DMArgs<R> b = a;
    auto at = [](size_t o) { return reinterpret_cast<char*>(o); };
    b.lut = (int16_t*)at(o_lut); b.uslot_of_entry = (int16_t*)at(o_use); b.kzp = (R*)at(o_kz);
    b.cst = (C*)at(o_cst); b.exc = (C*)at(o_exc); b.ey = (C*)at(o_ey); b.eth = (R*)at(o_eth);
    b.lfx = (R*)at(o_lfx); b.lfy = (R*)at(o_lfy); b.lfyp = (R*)at(o_lfyp); b.shy = (C*)at(o_shy); b.shx = (C*)at(o_shx);
    b.slot_any = (int*)at(o_any);
    b.dxh = a.horner ? (C*)at(o_dxh) : nullptr;
    b.dyh = a.horner ? (C*)at(o_dyh) : nullptr;
    b.fringe = (R*)fringe; b.field = (C*)field; b.spectrum = (C*)spectrum;
    info->a = b;
    info->su = su;
    info->Wfast = Wfast; info->wcol = wcol; info->nchunks = nchunks;
    info->smem_row = smem_row; info->smem_col = smem_col; info->smem_out = smem_out;
    return OH_OK;
  }
  OH_TRY(scratch(ctx, "dm.R", bytes_R, &ptr)); a.Rbuf = (C*)ptr;
  OH_TRY(scratch(ctx, "dm.V", bytes_V, &ptr)); a.V = (C*)ptr;
  OH_TRY(scratch(ctx, "dm.occ", bytes_occ, &ptr)); a.occ = (uint8_t*)ptr;
  if (bytes_acc) { OH_TRY(scratch(ctx, "dm.acc", bytes_acc, &ptr)); a.accbuf = (C*)ptr; }
  OH_TRY(scratch(ctx, "dm.tables", off, &ptr));
  char* base = (char*)ptr;
  a.lut = (int16_t*)(base + o_lut); a.uslot_of_entry = (int16_t*)(base + o_use); a.kzp = (R*)(base + o_kz);
  a.cst = (C*)(base + o_cst); a.exc = (C*)(base + o_exc); a.ey = (C*)(base + o_ey);
  a.eth = (R*)(base + o_eth);
  a.lfx = (R*)(base + o_lfx); a.lfy = (R*)(base + o_lfy); a.lfyp = (R*)(base + o_lfyp); a.shy = (C*)(base + o_shy); a.shx = (C*)(base + o_shx);
  a.slot_any = (int*)(base + o_any);
  a.dxh = a.horner ? (C*)(base + o_dxh) : nullptr;
  a.dyh = a.horner ? (C*)(base + o_dyh) : nullptr;
  a.fringe = (R*)fringe; a.field = (C*)field; a.spectrum = (C*)spectrum;

  {
    // the tables depend only on the parameters: rebuild them when those (or
    // the scratch buffer holding them) change, else only reset the per-frame
    // layer flags
    struct Key {
      DMSetup su;
      int prec, pnx, pny, Px, Py, sig_x, sig_y, ey_perm, horner, src_mode;
      double ppx, ppy, lambda;
      const void* tables;
      const void* iperm;
    } key;
    std::memset(&key, 0, sizeof(key));
    key.su = su;
    key.prec = prec; key.pnx = a.pnx; key.pny = a.pny; key.Px = a.Px; key.Py = a.Py;
    key.sig_x = a.sig_x; key.sig_y = a.sig_y; key.ey_perm = a.ey_perm; key.horner = a.horner;
    key.src_mode = src ? 1 : 0;
    key.ppx = a.ppx; key.ppy = a.ppy; key.lambda = a.lambda;
    key.tables = base; key.iperm = a.ply.iperm;
    std::string ks(reinterpret_cast<const char*>(&key), sizeof(key));
    if (ks == ctx->dm_setup_key && !ctx->force_dm_setup) {
      OH_CUDA_TRY(cudaMemsetAsync(a.slot_any, 0, nU * sizeof(int), st));
    } else {
      KernelTimer kt(ctx, prec ? "dm_setup_f64" : "dm_setup", st);
      dm_setup<R><<<64, 256, 0, st>>>(a, su);
      OH_LAUNCH_CHECK();
      ctx->dm_setup_key = ks;
    }
  }
  // the FP32 path uses the compile-time FFT schedules; FP64 the generic engine
  oh_status rs = OH_OK;
  for (int chunk = 0; chunk < nchunks; ++chunk) {
  a.slot0 = (int)(chunk * lc);
  a.slot1 = (int)std::min(nU, (chunk + 1) * lc);
  a.e0 = nchunks > 1 ? a.slot0 : 0;
  a.e1 = nchunks > 1 ? a.slot1 : (int)nE;
  a.chunk_first = chunk == 0;
  a.chunk_last = chunk == nchunks - 1;
  with_fast_n_if<sizeof(R) == 4>(a.Px, [&](auto nc) {
    constexpr int NX = decltype(nc)::value;
    cudaError_t e = cudaFuncSetAttribute(dm_row_pass<R, NX>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_row);
    if (e != cudaSuccess) { rs = cuda_fail(e, "cudaFuncSetAttribute(dm_row_pass)"); return; }
    KernelTimer kt(ctx, prec ? "dm_row_pass_f64" : "dm_row_pass", st);
    dm_row_pass<R, NX><<<(a.pny + kRowPair - 1) / kRowPair, 512, smem_row, st>>>(a);
    note_launch();
    e = cudaGetLastError();
    if (e != cudaSuccess) rs = cuda_fail(e, "dm_row_pass launch");
  });
  OH_TRY(rs);
  if constexpr (sizeof(R) == 4) {
    if (Wfast) {
      with_fast_n(a.Py, [&](auto nc) {
        constexpr int NY = decltype(nc)::value;
        if constexpr (NY > 0) {
          auto launch = [&](auto kern, int threads, int blocks) {
            cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_col);
            if (e == cudaSuccess) e = cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
            if (e != cudaSuccess) { rs = cuda_fail(e, "cudaFuncSetAttribute(dm_col_fast)"); return; }
            KernelTimer kt(ctx, "dm_col_pass", st);
            kern<<<blocks, threads, smem_col, st>>>(a);
            note_launch();
            if ((e = cudaGetLastError()) != cudaSuccess) rs = cuda_fail(e, "dm_col_fast launch");
          };
          // the layer-step form with the SSB crop of a 2x-padded frame: the
          // output mask as a compile-time constant
          const bool ssb = a.horner && a.fkeep == col_ssb_keep<NY>();
          // layer chunks or the test hook: the extended kernel (runtime SSB mask)
          const bool ext = nchunks > 1 || a.stall_flag;
          bool done = false;
          if constexpr (col_narrow_ok<NY>()) {
            if (wcol == 1) {
              if (ssb) launch(dm_col_fast<NY, 1, true, true>, ColCfg<NY, 1, true>::T, a.Px);
              else if (a.horner) launch(dm_col_fast<NY, 1, true>, ColCfg<NY, 1, true>::T, a.Px);
              else launch(dm_col_fast<NY, 1, false>, ColCfg<NY, 1, false>::T, a.Px);
              done = true;
            }
          }
          if (!done) {
            if (ext && a.horner) launch(dm_col_fast<NY, 2, true, false, true>, ColCfg<NY, 2, true>::T, a.nstrips);
            else if (ext) launch(dm_col_fast<NY, 2, false, false, true>, ColCfg<NY, 2, false>::T, a.nstrips);
            else if (ssb) launch(dm_col_fast<NY, 2, true, true>, ColCfg<NY, 2, true>::T, a.nstrips);
            else if (a.horner) launch(dm_col_fast<NY, 2, true>, ColCfg<NY, 2, true>::T, a.nstrips);
            else launch(dm_col_fast<NY, 2, false>, ColCfg<NY, 2, false>::T, a.nstrips);
          }
        }
      });
      OH_TRY(rs);
    }
  }
  }   // layer chunks
  if (!Wfast) {
    cudaError_t e = cudaFuncSetAttribute(dm_col_pass<R, KMAX, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_col);
    if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(dm_col_pass)");
    KernelTimer kt(ctx, prec ? "dm_col_pass_f64" : "dm_col_pass", st);
    dm_col_pass<R, KMAX, 0><<<a.nstrips, T, smem_col, st>>>(a);
    OH_LAUNCH_CHECK();
  }
  with_fast_n_if<sizeof(R) == 4>(a.Px, [&](auto nc) {
    constexpr int NX = decltype(nc)::value;
    cudaError_t e = cudaFuncSetAttribute(dm_out_pass<R, NX>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_out);
    if (e != cudaSuccess) { rs = cuda_fail(e, "cudaFuncSetAttribute(dm_out_pass)"); return; }
    KernelTimer kt(ctx, prec ? "dm_out_pass_f64" : "dm_out_pass", st);
    dm_out_pass<R, NX><<<a.pny, 256, smem_out, st>>>(a);
    note_launch();
    e = cudaGetLastError();
    if (e != cudaSuccess) rs = cuda_fail(e, "dm_out_pass launch");
  });
  OH_TRY(rs);
  return OH_OK;
}

// One FP32 frame with the caller holding the context (the surrogate's two
// uses: image/depth layers, or one complex source field at src_z).
oh_status depthmap_enqueue_f32(oh_ctx* ctx, const oh_depthmap_params* p, const uint8_t* img, const uint8_t* depth,
                               void* fringe, void* field, const void* src, double src_z, cudaStream_t st) {
  OH_TRY(validate(p));
  if (!fringe || (!src && (!img || !depth))) return fail(OH_ERR_INVALID_ARG, "depth-map frame: missing buffers");
  return run_depthmap<float, 36>(ctx, p, img, depth, nullptr, fringe, field, nullptr, st, nullptr, src, src_z);
}

// The planning half of run_depthmap for one FP32 frame (dm_batch.h).
oh_status depthmap_frame_info(oh_ctx* ctx, const oh_depthmap_frame& f, cudaStream_t st, FrameInfo<float>* info) {
  return run_depthmap<float, 36>(ctx, &f.params, f.img, f.depth, f.phase, f.fringe, f.field, nullptr, st, info);
}

oh_status depthmap_validate(const oh_depthmap_params* p) { return validate(p); }

}  // namespace oh

using namespace oh;

extern "C" {

void oh_depthmap_params_default(oh_depthmap_params* p) {
  if (!p) return;
  std::memset(p, 0, sizeof(*p));
  p->pnx = 1920; p->pny = 1080;
  p->ppx = 8e-6; p->ppy = 8e-6;
  p->lambda = 532e-9;
  p->field_lens = 1000e-3;
  p->near_depthmap = 0.30; p->far_depthmap = 0.35;
  p->num_of_depth = 32;
  p->flag_change_depth_quantization = 1;
  p->default_depth_quantization = 256;
  p->transform_viewing_window = 0;
  p->pad = 2;
  p->sig_location_x = 0; p->sig_location_y = 1;
  p->phase_mode = OH_PHASE_REFERENCE;
  p->seed = 0;
  p->rand_phase_re = 1.0; p->rand_phase_im = 0.0;
  p->render_depth = nullptr; p->n_render_depth = 0;
}

oh_status oh_depthmap_levels(const oh_depthmap_params* p, int16_t lut_out[256], double* z_out) {
  OH_TRY(validate(p));
  Levels L;
  OH_TRY(compute_levels(p, &L));
  if (lut_out) std::memcpy(lut_out, L.lut, sizeof(L.lut));
  if (z_out) for (int i = 0; i < p->num_of_depth; ++i) z_out[i] = L.ztrans[i];
  return OH_OK;
}

oh_status oh_depthmap_generate(oh_ctx* ctx, oh_precision prec, const oh_depthmap_params* p,
                               const uint8_t* img, const uint8_t* depth, const float* phase,
                               void* fringe_out, void* field_out, void* spectrum_out, void* stream) {
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  CallScope cs(ctx, st);
  OH_TRY(cs.status());
  OH_TRY(validate(p));
  if (!img || !depth || !fringe_out) return fail(OH_ERR_INVALID_ARG, "img, depth and fringe_out are required");
  if (p->phase_mode == OH_PHASE_ARRAY && !phase) return fail(OH_ERR_INVALID_ARG, "OH_PHASE_ARRAY needs a phase array");
  if (prec == OH_FP64) return run_depthmap<double, 18>(ctx, p, img, depth, phase, fringe_out, field_out, spectrum_out, st);
  return run_depthmap<float, 36>(ctx, p, img, depth, phase, fringe_out, field_out, spectrum_out, st);
}

oh_status oh_depthmap_propagate_field(oh_ctx* ctx, oh_precision prec, const oh_depthmap_params* p,
                                      const void* field_in, double z, void* fringe_out, void* field_out,
                                      void* spectrum_out, void* stream) {
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  CallScope cs(ctx, st);
  OH_TRY(cs.status());
  OH_TRY(validate(p));
  if (!field_in || !fringe_out) return fail(OH_ERR_INVALID_ARG, "field_in and fringe_out are required");
  if (!std::isfinite(z)) return fail(OH_ERR_INVALID_ARG, "propagation distance must be finite");
  if (prec == OH_FP64)
    return run_depthmap<double, 18>(ctx, p, nullptr, nullptr, nullptr, fringe_out, field_out, spectrum_out, st, nullptr,
                                    field_in, z);
  return run_depthmap<float, 36>(ctx, p, nullptr, nullptr, nullptr, fringe_out, field_out, spectrum_out, st, nullptr,
                                 field_in, z);
}

oh_status oh_depthmap_generate_batch(oh_ctx* ctx, oh_precision prec, const oh_depthmap_frame* frames, int n,
                                     unsigned flags, void* stream) {
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  CallScope cs(ctx, st);
  OH_TRY(cs.status());
  if (n < 0 || (n > 0 && !frames)) return fail(OH_ERR_INVALID_ARG, "bad frame array");
  if (flags & ~OH_BATCH_GRAPH) return fail(OH_ERR_INVALID_ARG, "unknown batch flags");
  for (int i = 0; i < n; ++i) {
    const oh_depthmap_frame& f = frames[i];
    OH_TRY(validate(&f.params));
    if (!f.img || !f.depth || !f.fringe)
      return fail(OH_ERR_INVALID_ARG, "frame " + std::to_string(i) + ": img, depth and fringe are required");
    if (f.params.phase_mode == OH_PHASE_ARRAY && !f.phase)
      return fail(OH_ERR_INVALID_ARG, "frame " + std::to_string(i) + ": OH_PHASE_ARRAY needs a phase array");
  }
  if (n == 0) return OH_OK;
  const bool fp64 = prec == OH_FP64;
  // key: precision and the whole frame array (parameters, buffer addresses,
  // render-depth lists)
  std::string key = std::to_string((int)fp64) + ":" + std::to_string(n) + ":";
  key.append(reinterpret_cast<const char*>(frames), (size_t)n * sizeof(oh_depthmap_frame));
  for (int i = 0; i < n; ++i)
    if (frames[i].params.render_depth)
      key.append(reinterpret_cast<const char*>(frames[i].params.render_depth),
                 (size_t)frames[i].params.n_render_depth * sizeof(int));
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (st) OH_CUDA_TRY(cudaStreamIsCapturing(st, &cap));
  if (!fp64 && ctx->dm_batch_persistent && cap == cudaStreamCaptureStatusNone) {
    // every frame in one launch of the persistent batch kernel
    bool handled = false;
    OH_TRY(batch_persistent(ctx, frames, n, flags, key, st, &handled));
    if (handled) return OH_OK;
  }
  auto run_all = [&](DMScratch* sizes) -> oh_status {
    for (int i = 0; i < n; ++i) {
      const oh_depthmap_frame& f = frames[i];
      if (fp64) {
        FrameInfo<double> fi;
        OH_TRY((run_depthmap<double, 18>(ctx, &f.params, f.img, f.depth, f.phase, f.fringe, f.field, nullptr, st,
                                         sizes ? &fi : nullptr)));
        if (sizes) sizes[i] = fi.sz;
      } else {
        FrameInfo<float> fi;
        OH_TRY((run_depthmap<float, 36>(ctx, &f.params, f.img, f.depth, f.phase, f.fringe, f.field, nullptr, st,
                                        sizes ? &fi : nullptr)));
        if (sizes) sizes[i] = fi.sz;
      }
    }
    return OH_OK;
  };
  // size the scratch once for the largest frame
  std::vector<DMScratch> sz(n);
  OH_TRY(run_all(sz.data()));
  DMScratch mx{0, 0, 0, 0, 0};
  for (const DMScratch& z : sz) {
    mx.R = std::max(mx.R, z.R); mx.V = std::max(mx.V, z.V);
    mx.occ = std::max(mx.occ, z.occ); mx.tables = std::max(mx.tables, z.tables);
    mx.acc = std::max(mx.acc, z.acc);
  }
  void* ptr;
  OH_TRY(scratch(ctx, "dm.R", mx.R, &ptr));
  OH_TRY(scratch(ctx, "dm.V", mx.V, &ptr));
  OH_TRY(scratch(ctx, "dm.occ", mx.occ, &ptr));
  if (mx.acc) OH_TRY(scratch(ctx, "dm.acc", mx.acc, &ptr));
  OH_TRY(scratch(ctx, "dm.tables", mx.tables, &ptr));
  const bool graph = (flags & OH_BATCH_GRAPH) && st != nullptr && cap == cudaStreamCaptureStatusNone;
  if (!graph) return run_all(nullptr);
  auto it = ctx->graphs.find(key);
  if (it != ctx->graphs.end()) {
    OH_CUDA_TRY(cudaGraphLaunch(it->second.exec, st));
    note_launch(it->second.launches);           // kernels inside the graph
    ctx->dm_setup_key = it->second.dm_key;    // the tables the graph leaves in scratch
    return OH_OK;
  }
  OH_TRY(run_all(nullptr));                   // this call's frames
  if (ctx->graphs.size() >= 16) drop_graphs(ctx);
  // capture the same launches for the next calls: tables are rebuilt inside
  // the graph for every frame, timing events are left out
  const bool timing = ctx->timing;
  ctx->timing = false;
  ctx->force_dm_setup = true;
  cudaGraph_t g = nullptr;
  oh_status rs = OH_OK;
  const uint64_t l0 = launches_so_far();
  cudaError_t e = cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed);
  if (e != cudaSuccess) rs = cuda_fail(e, "cudaStreamBeginCapture");
  else {
    rs = run_all(nullptr);
    e = cudaStreamEndCapture(st, &g);
    if (rs == OH_OK && e != cudaSuccess) rs = cuda_fail(e, "cudaStreamEndCapture");
  }
  ctx->timing = timing;
  ctx->force_dm_setup = false;
  if (rs == OH_OK) {
    cudaGraphExec_t ex = nullptr;
    e = cudaGraphInstantiate(&ex, g, 0);
    if (e != cudaSuccess) rs = cuda_fail(e, "cudaGraphInstantiate");
    else ctx->graphs[key] = oh_ctx::Graph{ex, ctx->dm_setup_key, (int)(launches_so_far() - l0)};
  }
  if (g) cudaGraphDestroy(g);
  return rs;
}

oh_status oh_depthmap_generate_host(oh_ctx* ctx, oh_precision prec, const oh_depthmap_params* p,
                                    const uint8_t* img_host, const uint8_t* depth_host,
                                    const float* phase_host, void* fringe_host, void* stream) {
  OH_TRY(validate(p));
  if (!ctx || !img_host || !depth_host || !fringe_host) return fail(OH_ERR_INVALID_ARG, "null argument");
  if (p->phase_mode == OH_PHASE_ARRAY && !phase_host) return fail(OH_ERR_INVALID_ARG, "OH_PHASE_ARRAY needs a phase array");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  CallScope cs(ctx, st);
  OH_TRY(cs.status());
  const size_t n = (size_t)p->pnx * p->pny;
  const size_t fsz = n * (prec == OH_FP64 ? sizeof(double) : sizeof(float));
  void* dev;
  OH_TRY(scratch(ctx, "host.io", 2 * n + (phase_host ? 4 * n : 0) + fsz + 1024, &dev));
  // Page-locked (or registered) buffers are used through their device
  // mappings: the row pass reads the image, depth (and phase) bytes straight
  // from host memory and the output kernel writes the fringe there, with no
  // copy before or after the passes (1920x1080: 1.141 -> 1.130 ms per call
  // against copying the inputs first).  Pageable buffers get the copies.
  auto mapped = [](const void* h) -> void* {
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, h) != cudaSuccess) { cudaGetLastError(); return nullptr; }
    return at.type == cudaMemoryTypeHost ? at.devicePointer : nullptr;
  };
  void* fringe_mapped = mapped(fringe_host);
  uint8_t* d_img = (uint8_t*)dev;
  uint8_t* d_depth = d_img + n;
  size_t off = (2 * n + 255) & ~(size_t)255;
  float* d_phase = phase_host ? (float*)((char*)dev + off) : nullptr;
  if (phase_host) off += (4 * n + 255) & ~(size_t)255;
  void* d_fringe = (char*)dev + off;
  const uint8_t* img_mapped = (const uint8_t*)mapped(img_host);
  const uint8_t* depth_mapped = (const uint8_t*)mapped(depth_host);
  const float* phase_mapped = phase_host ? (const float*)mapped(phase_host) : nullptr;
  auto enqueue = [&]() -> oh_status {
    const uint8_t* di = img_mapped;
    const uint8_t* dd = depth_mapped;
    const float* dp = phase_mapped;
    if (!di) { OH_CUDA_TRY(cudaMemcpyAsync(d_img, img_host, n, cudaMemcpyHostToDevice, st)); di = d_img; }
    if (!dd) { OH_CUDA_TRY(cudaMemcpyAsync(d_depth, depth_host, n, cudaMemcpyHostToDevice, st)); dd = d_depth; }
    if (phase_host && !dp) {
      OH_CUDA_TRY(cudaMemcpyAsync(d_phase, phase_host, 4 * n, cudaMemcpyHostToDevice, st));
      dp = d_phase;
    }
    void* out = fringe_mapped ? fringe_mapped : d_fringe;
    if (prec == OH_FP64) OH_TRY((run_depthmap<double, 18>(ctx, p, di, dd, dp, out, nullptr, nullptr, st)));
    else OH_TRY((run_depthmap<float, 36>(ctx, p, di, dd, dp, out, nullptr, nullptr, st)));
    if (!fringe_mapped) OH_CUDA_TRY(cudaMemcpyAsync(fringe_host, d_fringe, fsz, cudaMemcpyDeviceToHost, st));
    return OH_OK;
  };
  // Repeated frames with the same parameters and page-locked host buffers
  // replay one CUDA graph of the copies and the passes (one launch instead
  // of the per-call planning and five enqueues).  The graph expects the
  // parameter tables its capture found in scratch; when another frame has
  // replaced them, the frame runs directly and is captured again.
  bool graphable = st != nullptr && fringe_mapped && img_mapped && depth_mapped && (!phase_host || phase_mapped) &&
                   !ctx->timing && !ctx->stall_mask;
  if (graphable) {
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    OH_CUDA_TRY(cudaStreamIsCapturing(st, &cap));
    graphable = cap == cudaStreamCaptureStatusNone;
  }
  if (!graphable) {
    OH_TRY(enqueue());
    OH_CUDA_TRY(cudaStreamSynchronize(st));
    return OH_OK;
  }
  std::string key = "host:" + std::to_string((int)prec) + ":";
  key.append(reinterpret_cast<const char*>(p), sizeof(*p));
  if (p->render_depth)
    key.append(reinterpret_cast<const char*>(p->render_depth), (size_t)p->n_render_depth * sizeof(int));
  const void* ptrs[4] = {img_host, depth_host, phase_host, fringe_host};
  key.append(reinterpret_cast<const char*>(ptrs), sizeof(ptrs));
  auto it = ctx->frame_graphs.find(key);
  if (it != ctx->frame_graphs.end() && it->second.dm_key == ctx->dm_setup_key) {
    OH_CUDA_TRY(cudaGraphLaunch(it->second.exec, st));
    note_launch(it->second.launches);
    OH_CUDA_TRY(cudaStreamSynchronize(st));
    return OH_OK;
  }
  if (it != ctx->frame_graphs.end()) {
    cudaGraphExecDestroy(it->second.exec);
    ctx->frame_graphs.erase(it);
  }
  OH_TRY(enqueue());                          // this call's frame (builds the tables when needed)
  if (ctx->frame_graphs.size() >= 16) {
    for (auto& kv : ctx->frame_graphs) cudaGraphExecDestroy(kv.second.exec);
    ctx->frame_graphs.clear();
  }
  // capture the same work for the next calls (launched kernels are counted
  // when the graph runs, not while it is captured)
  const uint64_t l0 = launches_so_far();
  cudaGraph_t g = nullptr;
  oh_status rs = OH_OK;
  cudaError_t e = cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed);
  if (e != cudaSuccess) rs = cuda_fail(e, "cudaStreamBeginCapture");
  else {
    rs = enqueue();
    e = cudaStreamEndCapture(st, &g);
    if (rs == OH_OK && e != cudaSuccess) rs = cuda_fail(e, "cudaStreamEndCapture");
  }
  const int captured = (int)(launches_so_far() - l0);
  note_launch(-captured);
  if (rs == OH_OK) {
    cudaGraphExec_t ex = nullptr;
    e = cudaGraphInstantiate(&ex, g, 0);
    if (e != cudaSuccess) rs = cuda_fail(e, "cudaGraphInstantiate");
    else ctx->frame_graphs[key] = oh_ctx::Graph{ex, ctx->dm_setup_key, captured};
  }
  if (g) cudaGraphDestroy(g);
  OH_TRY(rs);
  OH_CUDA_TRY(cudaStreamSynchronize(st));
  return OH_OK;
}

}  // extern "C"
