// Fast column pass of the depth-map pipeline (FP32, compile-time FFT length).
//
// One block owns a strip of W spectrum columns for the whole frame.  For each
// non-empty layer it
//   1. waits for the layer's data in a shared-memory staging buffer: the
//      strip of row-pass output (pny x W complex, contiguous), the row
//      occupancy flags and the layer's Ey row.  One thread issues the three
//      copies with cp.async.bulk on an mbarrier one layer ahead (double
//      buffered), so the loads overlap the previous layer's FFT;
//   2. runs FFT stage 0 straight from the staging buffer (only the pny image
//      rows are read; padded rows are implicit zeros) into the work buffer,
//      then the remaining stages in place, twiddles from a two-level
//      shared-memory table;
//   3. multiplies by the layer's transfer function and accumulates into
//      registers (fixed element ownership across layers).  When the layers
//      are evenly spaced in z' (H_l = H_last D^(last - l) with one step factor
//      D per element), step 3 is the recurrence acc = acc D + x instead, with
//      no per-layer Ey row and no per-layer sine/cosine, and the last layer's
//      H is applied once in the epilogue.
// The epilogue applies the SSB crop, the inverse y-FFT and the y shift phase
// and writes the pny output rows of the strip.
//
// Every mbarrier wait is bounded (about one second of SM clock); on timeout
// the block sets the frame's error word, waits (bounded) for its own copies
// still in flight and leaves the layer loop.
#pragma once
#include "async_copy.cuh"
#include "fft_fast.cuh"

namespace oh {

struct ColLayout {
  int buf, stg, ey0, ey1, occ, g, twlo, twhi, tab, exw, lfxw, list, mbar, stg1, occ1, total;
};

// Twiddle-table entries of the middle forward stage of the column FFT
// (W^(j f) per butterfly offset j and output f: one load per twiddle instead
// of two loads and a product), or 0 when they would take more than 8 KB.
// (A table for stage 0 as well raises the register pressure there, where the
// accumulators are live, into spills.)
template <int NY>
constexpr int col_tab_entries() {
  constexpr int R0 = FastSched<NY>::r0, R1 = FastSched<NY>::r1;
  constexpr int n = (NY / R0 / R1) * stage_tab_stride(R1);
  return n * 8 <= 8192 ? n : 0;
}

__host__ __device__ constexpr int col_take(int* o, int bytes) {
  const int r = *o;
  *o += (bytes + 127) & ~127;
  return r;
}

// W: spectrum columns a block transforms; sw: columns per strip of the row
// pass output (the staging buffer holds a whole strip); step: the layer-step
// variant (its region holds D, float2 per element, instead of g and two Ey
// rows); pipe2: the two-buffer pipeline (see dm_col_body), whose step region
// is the second work buffer, plus a second staging buffer and flag row
__host__ __device__ constexpr ColLayout col_layout(int Py, int pny, int W, int sw, bool step, int occ_stride,
                                                   int n_entries, int tab_entries, bool pipe2 = false) {
  ColLayout L{};
  int o = 0;
  L.buf = col_take(&o, Py * W * 8);
  L.stg = col_take(&o, pny * sw * 8);
  const int gb = (Py * W * 4 + 127) & ~127, eb = (Py * 4 + 127) & ~127;
  L.g = col_take(&o, step ? Py * W * 8 : gb + 2 * eb);
  L.ey0 = L.g + gb;
  L.ey1 = L.ey0 + eb;
  L.occ = col_take(&o, occ_stride);
  L.twlo = col_take(&o, kTwLo * 8);
  L.twhi = col_take(&o, ((Py + 63) / 64) * 8);
  L.tab = col_take(&o, tab_entries * 8);
  L.exw = col_take(&o, W * 8);
  L.lfxw = col_take(&o, W * 4);
  L.list = col_take(&o, n_entries * 2 + 2);
  L.mbar = col_take(&o, 24);
  L.stg1 = pipe2 ? col_take(&o, pny * sw * 8) : 0;
  L.occ1 = pipe2 ? col_take(&o, occ_stride) : 0;
  L.total = o;
  return L;
}


// Column buffer layout: with an even last radix RL the last stage's 16
// threads of a half-warp (butterflies b, inputs b RL + f) would all hit one
// bank pair, so one element of padding follows every RL elements (element p
// sits at p + p / RL; RL + 1 is odd).  Q0 = NY / r0 and the middle stage's
// block size NY / r0 are multiples of RL, so every stage still addresses its
// inputs with fixed strides (col_pad: the padded length, 0 pad for odd RL).
template <int NY> constexpr bool col_padded() { return FastSched<NY>::rlast % 2 == 0; }
template <int NY> constexpr int col_len() { return col_padded<NY>() ? NY + NY / FastSched<NY>::rlast : NY; }

// Threads per block for a strip of W columns: one thread per last-stage
// butterfly (NY/RL per column), two when that would exceed 768 threads.
constexpr int kColStripW = 2;     // columns per strip of the row pass output

// Last-stage butterflies per thread: the block has as many threads as the
// smaller of the first two stages has butterflies (each stage then keeps all
// its threads busy in one round), within 768 threads; e.g. 2048 = 16 16 8
// takes 256 threads with two last-stage butterflies each instead of 512
// threads of which the first two stages use half.
template <int NY, int W> constexpr int col_kb() {
  constexpr int nbl = (NY / FastSched<NY>::rlast) * W;
  constexpr int i0 = NY / FastSched<NY>::r0, i1 = NY / FastSched<NY>::r1;
  constexpr int mi = W * (i0 < i1 ? i0 : i1);
  int kb = nbl > 768 ? 2 : 1;
  while (kb < 4 && nbl % (2 * kb) == 0 && nbl / (2 * kb) >= mi) kb *= 2;
  return kb;
}

// TT > 0: a block of exactly TT threads (the persistent batch kernel's
// block size), each taking ceil(NBL / TT) last-stage butterflies.
template <int NY, int W, bool STEP, int TT = 0> struct ColCfg {
  static constexpr int RL = FastSched<NY>::rlast;
  static constexpr int NBL = (NY / RL) * W;          // last-stage butterflies of the block's columns
  static constexpr int KB = TT > 0 ? (NBL + TT - 1) / TT : col_kb<NY, W>();   // butterflies per thread
  static constexpr int T = TT > 0 ? TT : ((NBL + KB - 1) / KB + 31) / 32 * 32;
  // two blocks per SM when two fit in shared memory (2x padding, pny =
  // NY / 2); otherwise one, and the register cap that two would impose
  // (spills at the longer lengths) is lifted
  static constexpr int SMEM =
      col_layout(col_len<NY>(), NY / 2, W, kColStripW, STEP, ((NY / 2) + 15) & ~15, kMaxEntries,
                 col_tab_entries<NY>()).total;
  static constexpr int FIT = (228 * 1024) / (SMEM + 1024);                // blocks per SM by shared memory
  static constexpr int MINB = FIT >= 3 && T <= 256 ? 3 : (FIT >= 2 ? 2 : 1);
};

// The two-buffer pipeline (layer-step form with the SSB crop): taken where
// it keeps two blocks per SM and the one-buffer kernel has two as well (2x
// padding, up to kMaxEntries render entries).
template <int NY, int W> constexpr bool col_pipe2() {
  constexpr int pny = NY / 2;
  constexpr int total = col_layout(col_len<NY>(), pny, W, kColStripW, true, (pny + 15) & ~15, kMaxEntries,
                                   col_tab_entries<NY>(), true).total;
  return ColCfg<NY, W, true>::MINB == 2 && 2 * (total + 1024 + 512) <= 228 * 1024;
}

// The step factor D = H(z' - dz) / H(z') = Dx(fx) Dy(fy) exp(-i k dz g) of
// one spectrum element, g = s^2 / (2 (1 + sqrt(1 - s))^2), s = (lambda fx)^2
// + (lambda fy)^2 (one expression for every variant, so they agree bit for bit).
__device__ __forceinline__ float2 col_step_factor(float2 dx, float2 dy, float lfx, float lfy, float kdz_pi) {
  const float sv = lfx + lfy;
  const float den = 1.f + sqrtf(1.f - sv);
  const float g = sv * sv * __fdividef(0.5f, den * den);
  float sn, cs;
  sincospif(-kdz_pi * g, &sn, &cs);
  return cmul(cmul(dx, dy), make_float2(cs, sn));
}

// One-column blocks (W = 1) over two-column strips, for the lengths where a
// two-column block's shared memory leaves one block per SM and the second
// read of each strip still hits L2 (measured faster at 3072 to 4096; at 4096
// 5.02 -> 4.66 ms for a 64-layer frame)
template <int NY> constexpr bool col_narrow_ok() { return NY >= 3072 && NY <= 4096; }

// Last-stage outputs f (bit f) that can reach the SSB crop of a 2x-padded
// grid with the signal shifted along y (crop rows (NY/2 - NY/4) .. +NY/2 - 1
// on the 1-based padded grid, spectrum row at storage position b RL + f =
// (k_low + (NY/RL) f + NY/2) mod NY, k_low < NY/RL): the mask the host
// derives from the crop window for that case.
template <int NY> constexpr uint32_t col_ssb_keep() {
  constexpr int RL = FastSched<NY>::rlast, q = NY / RL;
  const int cropy = NY / 2, cy1 = cropy - cropy / 2 - 1, cy2 = cy1 + cropy - 1;
  uint32_t m = 0;
  for (int f = 0; f < RL; ++f)
    for (int kl = 0; kl < q; ++kl) {
      const int ky = (kl + q * f + NY / 2) % NY;
      if (ky >= cy1 && ky <= cy2) { m |= 1u << f; break; }
    }
  return m;
}

// STEP: evenly spaced layers, accumulated with the layer-step recurrence.
// SSB: the output mask is col_ssb_keep<NY>() at compile time, so the last
// stage's small DFT computes only the outputs that reach the crop.
// EXT: the layer-chunk hand-over of the accumulators and the error-path
// test hook; the frames that need neither run the kernel without them.
// Block body for column block blk (a strip, or one column of a strip when
// W = 1).  TT: see ColCfg.  PERSIST: the block goes on to other work after
// this one, so its mbarriers are invalidated at the end.
// PIPE2 (layer-step form with the SSB crop): two work buffers and two
// staging buffers.  Layer k's last stage and layer k+1's stage 0 share one
// barrier phase (they use different work buffers), so a layer takes two
// block barriers instead of three; the strip of layer k+2 is requested as
// soon as stage 0 of layer k has read its buffer; the step factors of the
// thread's own outputs are held in registers.
template <int NY, int W, bool STEP, bool SSB, bool EXT, int TT, bool PERSIST, bool PIPE2 = false>
__device__ __forceinline__ void dm_col_body(const DMArgs<float>& a, int blk) {
  static_assert(!PIPE2 || (STEP && SSB && !EXT), "the two-buffer pipeline is the layer-step SSB form");
  typedef float2 C;
  typedef ColCfg<NY, W, STEP, TT> CF;
  constexpr int SW = kColStripW;
  static_assert(W == 1 || W == SW, "a block takes one column or a whole strip");
  constexpr int T = CF::T;
  constexpr int R0 = FastSched<NY>::r0;
  constexpr int RL = CF::RL;
  constexpr int KB = CF::KB;
  constexpr int Q0 = NY / R0;
  static_assert(FastSched<NY>::nstages == 3, "fast column pass expects a three-stage schedule");
  extern __shared__ __align__(128) unsigned char smem[];
  constexpr int kTab = col_tab_entries<NY>();
  constexpr int R1 = FastSched<NY>::r1;
  const ColLayout Lo = col_layout(col_len<NY>(), a.pny, W, SW, STEP, a.occ_stride, a.n_entries, kTab, PIPE2);
  // padded layout (see col_padded): element p at p + p / RL
  constexpr bool PADL = col_padded<NY>();
  constexpr int RLP = PADL ? RL + 1 : RL;                     // stored length of RL elements
  constexpr int Q0P = PADL ? Q0 + Q0 / RL : Q0;               // stored stride of stage-0 outputs
  constexpr int M1 = NY / R0, M1P = PADL ? M1 + M1 / RL : M1; // middle-stage block, stored
  auto pidx = [](int p) { return PADL ? p + p / RL : p; };
  C* buf = reinterpret_cast<C*>(smem + Lo.buf);
  C* const stg = reinterpret_cast<C*>(smem + Lo.stg);            // row-pass strip of the layer (single buffer)
  uint8_t* const occ = smem + Lo.occ;                             // its row flags
  float* const ey0 = reinterpret_cast<float*>(smem + Lo.ey0);    // Ey phase rows, double buffered
  float* const ey1 = reinterpret_cast<float*>(smem + Lo.ey1);
  float* gsm = reinterpret_cast<float*>(smem + Lo.g);            // per element, buffer order
  C* twlo = reinterpret_cast<C*>(smem + Lo.twlo);
  C* twhi = reinterpret_cast<C*>(smem + Lo.twhi);
  C* const tab1 = reinterpret_cast<C*>(smem + Lo.tab);            // stage 1: [NY/R0/R1][R1-1]
  C* exw = reinterpret_cast<C*>(smem + Lo.exw);
  float* lfxw = reinterpret_cast<float*>(smem + Lo.lfxw);
  ColShared* const csh = dm_col_shared();
  int* const kxw = csh->kxw;      // spectrum column of each strip column
  C* const dxw = csh->dxw;        // its Dx factor (layer-step form)
  // active render entries of this chunk, list[0..nact); list[-1] holds the
  // entry before the first (the previous chunk's last active one, or one less
  // than the first), so the layer-step gap is e - list[k - 1] for every k
  int16_t* list = reinterpret_cast<int16_t*>(smem + Lo.list) + 1;
  uint64_t* mbar = reinterpret_cast<uint64_t*>(smem + Lo.mbar);  // [0] strip+flags, [1],[2] Ey
  int& s_nact = csh->nact;
  int& s_last = csh->last;

  const int tid = threadIdx.x;
  const int s = blk / (SW / W);                      // row-pass strip
  const int csel = (blk % (SW / W)) * W;              // first of its columns this block takes
  const int kx0 = blk * W;
  const int pny = a.pny;
  if (tid < 32) {
    // this chunk's active entries, the last active entry before it (the
    // layer-step gap) and the last active entry of the frame (its transfer
    // function finishes the recurrence): warp 0 reads the layer flags of 32
    // entries at a time and compacts them with ballots
    const unsigned lt = (1u << tid) - 1u;
    int n = 0, prev = -1, last = -1, first = -1;
    for (int base = 0; base < a.n_entries; base += 32) {
      const int e = base + tid;
      const bool act = e < a.n_entries && a.slot_any[a.uslot_of_entry[e]] != 0;
      const unsigned m = __ballot_sync(0xffffffffu, act);
      const unsigned mc = __ballot_sync(0xffffffffu, act && e >= a.e0 && e < a.e1);
      const unsigned mp = __ballot_sync(0xffffffffu, act && e < a.e0);
      if ((mc >> tid) & 1u) list[n + __popc(mc & lt)] = (int16_t)e;
      if (mc && first < 0) first = base + __ffs(mc) - 1;
      n += __popc(mc);
      if (mp) prev = base + 31 - __clz(mp);
      if (m) last = base + 31 - __clz(m);
    }
    if (tid == 0) {
      mbar_init(&mbar[0], 1);
      mbar_init(&mbar[1], 1);
      mbar_init(&mbar[2], 1);
      fence_mbar_init();
      s_nact = n;
      s_last = last;
      list[-1] = (int16_t)(prev >= 0 ? prev : (n > 0 ? first - 1 : 0));
    }
  }
  load_tw_split(twlo, twhi, static_cast<const C*>(a.ply.tw), NY);
  if constexpr (kTab > 0) fill_stage_tab<NY, R1, NY / R0, -1>(tab1, static_cast<const C*>(a.ply.tw));
  if (tid < W) {
    // strip column kx0 + w is either spectrum column kx0 + w or, when the row
    // pass stored its output in FFT storage order, column iperm + hx
    int kx = kx0 + tid;
    if (a.xs) { kx = a.plx.iperm[kx0 + tid] + a.hx; if (kx >= a.Px) kx -= a.Px; }
    kxw[tid] = kx;
    lfxw[tid] = a.lfx[kx];
    if (STEP) dxw[tid] = a.dxh[kx];
  }
  __syncthreads();
  constexpr bool horner = STEP;
  const int nact = s_nact;
  const uint32_t fkeep = SSB ? col_ssb_keep<NY>() : a.fkeep;
  const TwSplit<C> tw{twlo, twhi};
  const uint32_t strip_bytes = (uint32_t)(pny * SW * 8);

  auto issue_strip = [&](int k) {
    const int u = a.uslot_of_entry[list[k]] - (EXT ? a.slot0 : 0);      // slot within this chunk's buffers
    mbar_expect_tx(&mbar[0], strip_bytes + (uint32_t)a.occ_stride);
    bulk_g2s(stg, a.Rbuf + ((size_t)u * a.nstrips + s) * pny * SW, strip_bytes, &mbar[0]);
    bulk_g2s(occ, a.occ + (size_t)u * a.occ_stride, (uint32_t)a.occ_stride, &mbar[0]);
  };
  // PIPE2: strip j goes to staging buffer j & 1 on mbar[j & 1]
  C* const stg1 = reinterpret_cast<C*>(smem + Lo.stg1);
  uint8_t* const occ1 = smem + Lo.occ1;
  auto issue_strip2 = [&](int j) {
    const int u = a.uslot_of_entry[list[j]];
    uint64_t* const bar = &mbar[j & 1];
    mbar_expect_tx(bar, strip_bytes + (uint32_t)a.occ_stride);
    bulk_g2s((j & 1) ? stg1 : stg, a.Rbuf + ((size_t)u * a.nstrips + s) * pny * SW, strip_bytes, bar);
    bulk_g2s((j & 1) ? occ1 : occ, a.occ + (size_t)u * a.occ_stride, (uint32_t)a.occ_stride, bar);
  };
  auto issue_ey = [&](int k) {
    const int e = list[k];
    uint64_t* bar = (k & 1) ? &mbar[2] : &mbar[1];
    mbar_expect_tx(bar, (uint32_t)(NY * 4));
    bulk_g2s((k & 1) ? ey1 : ey0, a.eth + (size_t)e * NY, (uint32_t)(NY * 4), bar);
  };
  // the first layer's copies fly while the tables below are built
  if (tid == 0 && nact > 0) {
    issue_strip(0);
    if (PIPE2 && nact > 1) issue_strip2(1);
    if (!horner) issue_ey(0);
  }

  // layer-independent part of the angular-spectrum residual phase:
  // psi = k z' g,  g = s^2 / (2 (1 + sqrt(1 - s))^2),  s = (lambda fx)^2 + (lambda fy)^2.
  // With the layer-step recurrence the region holds instead the step factor
  // D = H(z' - dz) / H(z') = Dx(fx) Dy(fy) exp(-i k dz g).  Each thread loads
  // the fy terms of kDB elements before using them.
  C* const dsm = reinterpret_cast<C*>(smem + Lo.g);
  constexpr int kDB = 4;
  for (int i0 = tid; i0 < (PIPE2 ? 0 : NY * W); i0 += kDB * T) {
    float lfy[kDB];
    C dyv[kDB];
#pragma unroll
    for (int q = 0; q < kDB; ++q) {
      const int idx = i0 + q * T;
      const int p = idx < NY * W ? idx / W : 0;
      lfy[q] = a.lfyp[p];
      if constexpr (horner) dyv[q] = a.dyh[p];
    }
#pragma unroll
    for (int q = 0; q < kDB; ++q) {
      const int idx = i0 + q * T;
      if (idx >= NY * W) break;
      const int p = idx / W, w = idx - p * W;
      if constexpr (horner) {
        dsm[pidx(p) * W + w] = col_step_factor(dxw[w], dyv[q], lfxw[w], lfy[q], a.kdz_pi);
      } else {
        const float sv = lfxw[w] + lfy[q];
        const float den = 1.f + sqrtf(1.f - sv);
        gsm[pidx(p) * W + w] = sv * sv * __fdividef(0.5f, den * den);
      }
    }
  }

  // accumulators: last-stage butterfly bb = tid + kb*T of the strip (bb = b*W + w),
  // outputs f at storage position p = b*RL + f of line w
  C acc[KB][RL];
#pragma unroll
  for (int kb = 0; kb < KB; ++kb)
#pragma unroll
    for (int f = 0; f < RL; ++f) acc[kb][f] = make_float2(0.f, 0.f);
  if (EXT && !a.chunk_first) {
    // the accumulators of the earlier layer chunks
    const C* accb = a.accbuf + (size_t)blk * KB * RL * T + tid;
#pragma unroll
    for (int kb = 0; kb < KB; ++kb)
#pragma unroll
      for (int f = 0; f < RL; ++f) acc[kb][f] = accb[(kb * RL + f) * T];
  }
  if (EXT && a.stall_flag) {
    // error-path test hook: wait on a flag that nothing sets, then leave as a
    // timed-out copy wait does (the first layer's copies land first)
    const bool stalled = tid == 0 && !stall_on_unset_flag(a.stall_flag, a.stall_cycles);
    if (__syncthreads_or(stalled)) {
      if (tid == 0) atomicOr(a.err, 1);
      if (nact > 0) {
        mbar_wait_bounded(&mbar[0], 0u);
        if (!horner) mbar_wait_bounded(&mbar[1], 0u);
      }
      return;
    }
  }

  // stage 0 of one layer from staging buffer (sg, oc) into work buffer bf:
  // inputs j + t*Q0 of the y-shifted line
  auto stage0 = [&](const C* sg, const uint8_t* oc, C* bf) {
    for (int idx = tid; idx < Q0 * W; idx += T) {
      const int j = idx / W, w = idx - j * W;
      C x[R0];
      if (R0 == 16 && a.hzy) {
        // 2x padding: inputs t = 4..11 are rows of the zero band; with
        // hy = NY/2 and oy = NY/4 the image row of input t is
        // j + (t + 4) Q0 (t < 4) or j + (t - 12) Q0 (t >= 12)
#pragma unroll
        for (int t = 0; t < R0; ++t) {
          if (t >= 4 && t < 12) { x[t] = make_float2(0.f, 0.f); continue; }
          const int yl = j + (t < 4 ? t + 4 : t - 12) * Q0;
          x[t] = oc[yl] ? sg[yl * SW + csel + w] : make_float2(0.f, 0.f);
        }
        dft16_halfzero<-1>(x);
      } else {
#pragma unroll
        for (int t = 0; t < R0; ++t) {
          int y = j + t * Q0 - a.hy;
          if (y < 0) y += NY;
          const int yl = y - a.oy;
          C v = make_float2(0.f, 0.f);
          if (yl >= 0 && yl < pny && oc[yl]) v = sg[yl * SW + csel + w];
          x[t] = v;
        }
        DFT<R0, -1, C>::run(x);
      }
      if (j) {
        C wp[R0];
        twiddle_powers<R0, -1>(tw, j, wp);
#pragma unroll
        for (int f = 1; f < R0; ++f) x[f] = cmul(x[f], wp[f]);
      }
#pragma unroll
      for (int f = 0; f < R0; ++f) bf[(pidx(j) + f * Q0P) * W + w] = x[f];
    }
  };
  auto middle = [&](C* bf) {
    if constexpr (kTab > 0) fstage_tab<NY, R1, M1, -1, C, M1P, RLP>(bf, W, 1, W, tab1, true);
    else fstage_t<NY, R1, NY / R0, -1>(bf, W, 1, W, tw, true);
  };
  static_assert(kTab > 0 || !PADL, "the padded layout needs the middle stage's table");
  if constexpr (PIPE2) {
    C* const buf1 = reinterpret_cast<C*>(smem + Lo.g);
    // step factors of this thread's kept outputs
    C dreg[KB][RL];
#pragma unroll
    for (int kb = 0; kb < KB; ++kb) {
      const int bb = tid + kb * T;
#pragma unroll
      for (int f = 0; f < RL; ++f) {
        dreg[kb][f] = make_float2(0.f, 0.f);
        if (bb < CF::NBL && ((fkeep >> f) & 1u)) {
          const int b = bb / W, w = bb - b * W, p = b * RL + f;
          dreg[kb][f] = col_step_factor(dxw[w], a.dyh[p], lfxw[w], a.lfyp[p], a.kdz_pi);
        }
      }
    }
    // layers without pixels since the previous one (acc D^(gap - 1)), then
    // the last stage of work buffer bf fused with acc = acc D + x
    auto last = [&](const C* bf, int gap) {
#pragma unroll
      for (int kb = 0; kb < KB; ++kb) {
        const int bb = tid + kb * T;
        if (bb < CF::NBL) {
          const int b = bb / W, w = bb - b * W;
          for (int r = 1; r < gap; ++r) {
#pragma unroll
            for (int f = 0; f < RL; ++f)
              if ((fkeep >> f) & 1u) acc[kb][f] = cmul(acc[kb][f], dreg[kb][f]);
          }
          C x[RL];
#pragma unroll
          for (int f = 0; f < RL; ++f) x[f] = bf[(b * RLP + f) * W + w];
          DFT<RL, -1, C>::run(x);
#pragma unroll
          for (int f = 0; f < RL; ++f) {
            if (!((fkeep >> f) & 1u)) continue;
            const C d = dreg[kb][f];
            const C t = acc[kb][f];
            acc[kb][f] = make_float2(fmaf(t.x, d.x, fmaf(-t.y, d.y, x[f].x)), fmaf(t.x, d.y, fmaf(t.y, d.x, x[f].y)));
          }
        }
      }
    };
    // a wait for strip j ran out: flag it, let the copies in flight (strips
    // j and j + 1) land, leave
    auto bail = [&](int j) {
      if (tid == 0) atomicOr(a.err, 1);
      for (int q = j; q < nact && q <= j + 1; ++q) mbar_wait_bounded(&mbar[q & 1], (uint32_t)((q >> 1) & 1));
    };
    if (nact > 0) {
      const bool ok = mbar_wait_bounded(&mbar[0], 0u);
      if (__syncthreads_or(!ok)) { bail(0); return; }
      stage0(stg, occ, buf);
      __syncthreads();
      if (tid == 0 && nact > 2) {
        fence_proxy_async_smem();
        issue_strip2(2);
      }
      middle(buf);
      __syncthreads();
    }
    for (int k = 0; k < nact; ++k) {
      C* const bk = (k & 1) ? buf1 : buf;
      C* const bn = (k & 1) ? buf : buf1;
      last(bk, list[k] - list[k - 1]);
      bool ok = true;
      if (k + 1 < nact) {
        const int j = k + 1;
        ok = mbar_wait_bounded(&mbar[j & 1], (uint32_t)((j >> 1) & 1));
        if (ok) stage0((j & 1) ? stg1 : stg, (j & 1) ? occ1 : occ, bn);
      }
      if (__syncthreads_or(!ok)) { bail(k + 1); return; }
      if (k + 1 < nact) {
        if (tid == 0 && k + 3 < nact) {
          fence_proxy_async_smem();
          issue_strip2(k + 3);       // into the buffer stage 0 of layer k+1 has just read
        }
        middle(bn);
        __syncthreads();
      }
    }
  } else {
    for (int k = 0; k < nact; ++k) {
      // one barrier: layer k's strip and Ey have landed, and the previous
      // layer's last stage no longer reads the work buffer
      uint64_t* const bar_e = (k & 1) ? &mbar[2] : &mbar[1];
      bool ok = mbar_wait_bounded(&mbar[0], (uint32_t)(k & 1));
      ok = ok && (horner || mbar_wait_bounded(bar_e, (uint32_t)((k >> 1) & 1)));
      if (__syncthreads_or(!ok)) {
        if (tid == 0) atomicOr(a.err, 1);
        // let this block's copies still in flight land before leaving
        mbar_wait_bounded(&mbar[0], (uint32_t)(k & 1));
        if (!horner) mbar_wait_bounded(bar_e, (uint32_t)((k >> 1) & 1));
        return;
      }
      if (tid == 0 && k + 1 < nact && !horner) {
        // Ey buffer (k+1)&1 was last read by layer k-1, finished before the barrier
        fence_proxy_async_smem();
        issue_ey(k + 1);
      }
      const int e = list[k];
      if (tid < W && !horner) exw[tid] = a.exc[(size_t)e * a.Px + kxw[tid]];
      const int gap = e - list[k - 1];
      if constexpr (horner) {
        // layers without pixels since the previous one: acc D^(gap - 1)
        for (int r = 1; r < gap; ++r) {
#pragma unroll
          for (int kb = 0; kb < KB; ++kb) {
            const int bb = tid + kb * T;
            if (bb < CF::NBL) {
              const int b = bb / W, w = bb - b * W;
#pragma unroll
              for (int f = 0; f < RL; ++f) acc[kb][f] = cmul(acc[kb][f], dsm[(b * RLP + f) * W + w]);
            }
          }
        }
      }
      stage0(stg, occ, buf);
      // middle stage(s); the leading barrier also frees the strip buffer
      __syncthreads();
      if (tid == 0 && k + 1 < nact) {
        fence_proxy_async_smem();
        issue_strip(k + 1);
      }
      middle(buf);
      __syncthreads();
      // last stage (stride 1, no twiddles) fused with the transfer-function
      // multiply-accumulate: either acc += H x per layer, or the recurrence
      // acc = acc D^gap + x over the evenly spaced layers (H of the last layer
      // applied once in the epilogue)
      const float kz = a.kzp[e];
      const float* eth = (k & 1) ? ey1 : ey0;       // storage order
      const float inv2pi = 0.15915494309189533577f, two_pi = 6.28318530717958647692f;
#pragma unroll
      for (int kb = 0; kb < KB; ++kb) {
        const int bb = tid + kb * T;
        if (bb < CF::NBL) {
          const int b = bb / W, w = bb - b * W;
          C x[RL];
#pragma unroll
          for (int f = 0; f < RL; ++f) x[f] = buf[(b * RLP + f) * W + w];
          DFT<RL, -1, C>::run(x);
          if constexpr (horner) {
#pragma unroll
            for (int f = 0; f < RL; ++f) {
              if (!((fkeep >> f) & 1u)) continue;         // outside the SSB crop for every b
              const C d = dsm[(b * RLP + f) * W + w];
              const C t = acc[kb][f];
              acc[kb][f] = make_float2(fmaf(t.x, d.x, fmaf(-t.y, d.y, x[f].x)), fmaf(t.x, d.y, fmaf(t.y, d.x, x[f].y)));
            }
            continue;
          }
          const C ex = exw[w];
#pragma unroll
          for (int f = 0; f < RL; ++f) {
            if (!((fkeep >> f) & 1u)) continue;           // outside the SSB crop for every b
            const int p = b * RL + f;
            // H = C Ex exp(i (pi lambda z' fy^2 + k z' g)), both phase parts reduced
            float ph = fmaf(kz, gsm[(b * RLP + f) * W + w], eth[p]);
            ph = fmaf(-two_pi, rintf(ph * inv2pi), ph);
            float sn, cs;
            __sincosf(ph, &sn, &cs);
            const C h = cmul(ex, make_float2(cs, sn));
            acc[kb][f] = cadd(acc[kb][f], cmul(h, x[f]));
          }
        }
      }
    }
  }
  if (EXT && !a.chunk_last) {
    // more layer chunks follow: hand the accumulators on (this chunk's
    // copies have all landed: the last layer's strip was waited for above)
    C* accb = a.accbuf + (size_t)blk * KB * RL * T + tid;
#pragma unroll
    for (int kb = 0; kb < KB; ++kb)
#pragma unroll
      for (int f = 0; f < RL; ++f) accb[(kb * RL + f) * T] = acc[kb][f];
    return;
  }
  __syncthreads();

  // recurrence: apply the last layer's transfer function
  //   H = C Ex exp(i (pi lambda z' fy^2 + k z' g)), as in the per-layer form
  if (horner && s_last >= 0) {
    const int e = s_last;
    const float kz = a.kzp[e];
    const float inv2pi = 0.15915494309189533577f, two_pi = 6.28318530717958647692f;
#pragma unroll
    for (int kb = 0; kb < KB; ++kb) {
      const int bb = tid + kb * T;
      if (bb < CF::NBL) {
        const int b = bb / W, w = bb - b * W;
        const C ex = a.exc[(size_t)e * a.Px + kxw[w]];
#pragma unroll
        for (int f = 0; f < RL; ++f) {
          const int p = b * RL + f;
          const float sv = lfxw[w] + a.lfyp[p];
          const float den = 1.f + sqrtf(1.f - sv);
          const float g = sv * sv * __fdividef(0.5f, den * den);
          float ph = fmaf(kz, g, a.eth[(size_t)e * NY + p]);
          ph = fmaf(-two_pi, rintf(ph * inv2pi), ph);
          float sn, cs;
          __sincosf(ph, &sn, &cs);
          acc[kb][f] = cmul(acc[kb][f], cmul(ex, make_float2(cs, sn)));
        }
      }
    }
  }

  // SSB crop, then the inverse y-FFT.  Spectrum row ky sits in the inverse
  // line at (ky + hy) mod NY = iperm(p) for storage position p: the
  // accumulators are in the forward FFT's storage order, the input order of
  // the adjoint network, whose first stage (the adjoint of the last forward
  // stage) runs here in registers; the output comes out in natural order.
#pragma unroll
  for (int kb = 0; kb < KB; ++kb) {
    const int bb = tid + kb * T;
    if (bb < CF::NBL) {
      const int b = bb / W, w = bb - b * W;
      const int kx = kxw[w];
      C x[RL];
#pragma unroll
      for (int f = 0; f < RL; ++f) {
        int ky = FastSched<NY>::iperm(b * RL + f) + a.hy;      // spectrum row at storage position
        if (ky >= NY) ky -= NY;
        if (a.spectrum) a.spectrum[(size_t)ky * a.Px + kx] = acc[kb][f];
        const bool keep = kx >= a.cx1 && kx <= a.cx2 && ky >= a.cy1 && ky <= a.cy2 &&
                          (!PIPE2 || ((fkeep >> f) & 1u));
        x[f] = keep ? acc[kb][f] : make_float2(0.f, 0.f);
      }
      DFT<RL, 1, C>::run(x);
#pragma unroll
      for (int f = 0; f < RL; ++f) buf[(b * RLP + f) * W + w] = x[f];
    }
  }
  __syncthreads();
  fstage_adj<NY, R1, M1, C, TwSplit<C>, M1P, RLP>(buf, W, 1, W, tw, true);
  __syncthreads();
  fstage_adj<NY, R0, NY, C, TwSplit<C>, col_len<NY>(), Q0P, PADL ? RL : 0>(buf, W, 1, W, tw, true);
  __syncthreads();
  for (int idx = tid; idx < pny * W; idx += T) {
    const int yl = idx / W, w = idx - yl * W;
    int m = a.oy + yl - a.hy;
    if (m < 0) m += NY;
    a.V[(size_t)yl * a.Px + kx0 + w] = cmul(buf[pidx(m) * W + w], a.shy[yl]);
  }
  if constexpr (PERSIST) {
    __syncthreads();
    if (tid == 0) {
      mbar_inval(&mbar[0]);
      mbar_inval(&mbar[1]);
      mbar_inval(&mbar[2]);
    }
  }
}

template <int NY, int W, bool STEP, bool SSB = false, bool EXT = false>
__global__ void __launch_bounds__(ColCfg<NY, W, STEP>::T, ColCfg<NY, W, STEP>::MINB) dm_col_fast(DMArgs<float> a) {
  dm_col_body<NY, W, STEP, SSB, EXT, 0, false, STEP && SSB && !EXT && col_pipe2<NY, W>()>(a, blockIdx.x);
}

}  // namespace oh
