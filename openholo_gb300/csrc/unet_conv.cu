// Implicit-GEMM convolutions on the tcgen05 tensor cores (BF16 operands,
// FP32 accumulation in TMEM), the compute core of the learned surrogate.
//
// Activations are NHWC BF16 with a channel stride that is a multiple of 32
// (64 bytes), so 32 channels of one pixel are one 64-byte line of a
// 64-byte-swizzled shared-memory tile.
//
// conv_fwd_tc: Y[p][co] = sum_{tap, ci} X[p + s*off(tap)][ci] W[co][tap*cin + ci]
//   GEMM with M = 128 pixels (a bx x by patch), N = BN output channels,
//   K = taps x cin in 32-channel steps.  The A tile of a K step is one TMA
//   load of the 4-D activation map at the tap's offset: out-of-range pixels
//   read as zero, which is the convolution's zero padding.  When a tile is
//   128 pixels of one image row, one 136-pixel load of the row at dy (from
//   x - 1) serves all three dx taps: their A operands start 0, 1 and 2 pixel
//   rows into it, so each K step of 32 channels loads a third of the input.  s = +1 is the
//   forward convolution; s = -1 with the transposed weight matrix
//   Wt[ci][tap*cout + co] is the gradient with respect to the input (dgrad).
//   Epilogue: + bias, ReLU, multiplication by (mask > 0) (the ReLU derivative
//   of the layer below, for dgrad), BF16 store with an output channel stride
//   (so a layer can write straight into one half of a concatenation buffer).
// conv_wgrad_tc: dW^T[tap*cin + ci][co] += sum_p X[p + off(tap)][ci] dZ[p][co]
//   GEMM with M = 128 rows of the (tap, ci) space (four 32-channel groups,
//   each its own TMA load at its tap's offset), N = cout, K = pixels in
//   64-pixel steps; both operands are MN-major (channels contiguous), K split
//   across CTAs, partial sums added with vector reductions.
//
// Roles (128 threads): thread 0 issues TMA loads into a ring of stages,
// thread 32 issues tcgen05.mma and releases stages with tcgen05.commit, all
// four warps read the accumulator (warp w owns TMEM lanes 32w..32w+31).  Every
// mbarrier wait gives up after about one second of SM clock: the CTA then
// sets the device error word, lets its copies and MMAs land, frees TMEM and
// returns.  Pipeline waits (a stage's copies, a stage's release) also give
// up as soon as the other role has aborted; the final waits for the MMAs and
// for copies still in flight keep the full bound.
#include <cuda_bf16.h>
#include <algorithm>
#include <cstdlib>
#include "context.h"
#include "tc_common.cuh"
#include "unet.cuh"

namespace oh {

namespace {

constexpr int kConvThreads = 128;
constexpr long long kWaitCycles = 2000000000LL;      // ~1 s at 2 GHz

__device__ __forceinline__ bool wait_live(uint64_t* b, uint32_t parity, const int* abort) {
  const long long t0 = clock64();
  while (!tc::mb_try(b, parity)) {
    if (*((volatile const int*)abort) || clock64() - t0 > kWaitCycles) return false;
  }
  return true;
}

constexpr int pow2_at_least(int n) { return n <= 32 ? 32 : n <= 64 ? 64 : n <= 128 ? 128 : n <= 256 ? 256 : 512; }

template <int BN, bool HALO = false> struct FwdCfg {
  // HALO: one 136-pixel row box per (dy, 32 channels) serves the three dx
  // taps, whose A operands start 0, 1 and 2 pixel rows into it
  static constexpr int kABox = HALO ? 136 * 64 : 128 * 64;
  static constexpr int kA = (kABox + 1023) / 1024 * 1024;
  static constexpr int kBBox = BN * 64;                // BN rows x 32 K
  static constexpr int kBStride = (kBBox + 1023) / 1024 * 1024;
  static constexpr int kTapsPerStage = HALO ? 3 : 1;
  static constexpr int kB = kTapsPerStage * kBStride;
  static constexpr int kStage = kA + kB;
  static constexpr int kStagesRaw = (BN <= 64 ? 80 : 200) * 1024 / kStage;
  static constexpr int kStages = HALO ? (kStagesRaw < 2 ? 2 : kStagesRaw > 6 ? 6 : kStagesRaw) : (BN >= 192 ? 5 : 6);
  static constexpr int kTmemBuf = pow2_at_least(BN);  // columns of one accumulator
  static constexpr int kTmem = 2 * kTmemBuf;          // two accumulators: MMA and epilogue overlap
  static constexpr int kThreads = 192;                // warp 0 TMA, warp 1 MMA, warps 2-5 epilogue
  static constexpr int kSmem = kStages * kStage + 1024 + 256;
};

// Persistent CTAs: CTA i takes pixel tiles i, i + gridDim.x, ... of output
// channel tile blockIdx.y.  The TMA producer streams the K steps of all its
// tiles through one ring of stages; the MMA issuer accumulates tile j into
// TMEM buffer j & 1 and commits it to the epilogue warps, which drain it
// (bias, ReLU, mask, BF16 store) while the next tile accumulates in the
// other buffer.
template <int BN, bool HALO>
__global__ void __launch_bounds__(FwdCfg<BN, HALO>::kThreads) conv_fwd_tc(const __grid_constant__ CUtensorMap mX,
                                                                          const __grid_constant__ CUtensorMap mW,
                                                                          ConvArgs a) {
  typedef FwdCfg<BN, HALO> Cfg;
  extern __shared__ unsigned char smem_raw[];
  const uint32_t raw = tc::su32(smem_raw);
  unsigned char* base = smem_raw + (((raw + 1023u) & ~1023u) - raw);
  uint64_t* full = reinterpret_cast<uint64_t*>(base + Cfg::kStages * Cfg::kStage);
  uint64_t* empty = full + Cfg::kStages;
  uint64_t* tfull = empty + Cfg::kStages;              // [2] accumulator ready (MMA commit)
  uint64_t* tempty = tfull + 2;                        // [2] accumulator drained (4 epilogue warps)
  uint64_t* done = tempty + 2;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(done + 1);
  int* abort_flag = reinterpret_cast<int*>(tmem_slot + 1);
  int* issued = abort_flag + 1;
  int* consumed = abort_flag + 2;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  const long long tiles = (long long)a.n * a.tiles_y * a.tiles_x;
  const int ntl = blockIdx.x < tiles ? (int)((tiles - 1 - blockIdx.x) / gridDim.x + 1) : 0;
  const int co0 = blockIdx.y * BN;
  const int cchunks = a.cin >> 5;
  const int nk = (HALO ? 3 : a.taps) * cchunks;
  const long long nsteps = (long long)ntl * nk;

  if (threadIdx.x == 0) {
    for (int s = 0; s < Cfg::kStages; ++s) { tc::mb_init(&full[s], 1); tc::mb_init(&empty[s], 1); }
    for (int b = 0; b < 2; ++b) { tc::mb_init(&tfull[b], 1); tc::mb_init(&tempty[b], 4); }
    tc::mb_init(done, 1);
    *abort_flag = 0; *issued = 0; *consumed = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __shared__ float sbias[BN];               // this CTA's output-channel biases (0 without bias)
  for (int c = threadIdx.x; c < BN; c += blockDim.x)
    sbias[c] = (a.bias && co0 + c < a.cout) ? a.bias[co0 + c] : 0.f;
  if (warp == 1) tc::tmem_alloc(tmem_slot, Cfg::kTmem);
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t tmem = *tmem_slot;

  auto tile_origin = [&](int j, int* img, int* x0, int* y0) {
    long long t = blockIdx.x + (long long)j * gridDim.x;
    const int tx = (int)(t % a.tiles_x); t /= a.tiles_x;
    const int ty = (int)(t % a.tiles_y);
    *img = (int)(t / a.tiles_y);
    *x0 = tx * a.bx; *y0 = ty * a.by;
  };

  if (warp == 0) {
    if (lane == 0) {
      long long g = 0;
      for (int j = 0; j < ntl && g >= 0; ++j) {
        int img, x0, y0;
        tile_origin(j, &img, &x0, &y0);
        for (int it = 0; it < nk; ++it, ++g) {
          const int s = (int)(g % Cfg::kStages);
          const uint32_t ph = (uint32_t)((g / Cfg::kStages) & 1);
          if (!wait_live(&empty[s], ph ^ 1u, abort_flag) || *((volatile int*)abort_flag)) {
            atomicExch(abort_flag, 1);
            *issued = (int)g;
            g = -1;
            break;
          }
          unsigned char* st = base + s * Cfg::kStage;
          if constexpr (HALO) {
            // row y0 + dy' from x0 - 1: the dx' = -1, 0, +1 taps start 0, 1, 2 rows in
            const int dyi = it / cchunks, cc = it - dyi * cchunks;
            const int dyp = dyi - 1;
            tc::mb_expect_tx(&full[s], (uint32_t)(Cfg::kABox + 3 * Cfg::kBBox));
            tc::tma_load_4d(st, &mX, cc * 32, x0 - 1, y0 + dyp, img, &full[s]);
#pragma unroll
            for (int j = 0; j < 3; ++j) {
              const int tap = 3 * (1 + a.sign * dyp) + (1 + a.sign * (j - 1));
              tc::tma_load_2d(st + Cfg::kA + j * Cfg::kBStride, &mW, tap * a.cin + cc * 32, co0, &full[s]);
            }
          } else {
            const int tap = it / cchunks, cc = it - tap * cchunks;
            int dx = 0, dy = 0;
            if (a.taps == 9) { dx = (tap % 3 - 1) * a.sign; dy = (tap / 3 - 1) * a.sign; }
            tc::mb_expect_tx(&full[s], (uint32_t)Cfg::kStage);
            tc::tma_load_4d(st, &mX, cc * 32, x0 + dx, y0 + dy, img, &full[s]);
            tc::tma_load_2d(st + Cfg::kA, &mW, tap * a.cin + cc * 32, co0, &full[s]);
          }
        }
      }
      if (g >= 0) *issued = (int)nsteps;
    }
  } else if (warp == 1) {
    if (lane == 0) {
      constexpr uint32_t idesc = tc::idesc_bf16(128, BN, 0, 0);
      long long g = 0;
      bool stop = false;
      if (a.stall_flag && !stall_on_unset_flag(a.stall_flag, a.stall_cycles)) {
        atomicExch(abort_flag, 1);
        stop = true;
      }
      for (int j = 0; j < ntl && !stop; ++j) {
        const int b = j & 1;
        if (!wait_live(&tempty[b], (uint32_t)(((j >> 1) & 1) ^ 1), abort_flag)) {
          atomicExch(abort_flag, 1);
          break;
        }
        tc::fence_after();
        const uint32_t acc = tmem + (uint32_t)(b * Cfg::kTmemBuf);
        for (int it = 0; it < nk; ++it, ++g) {
          const int s = (int)(g % Cfg::kStages);
          const uint32_t ph = (uint32_t)((g / Cfg::kStages) & 1);
          if (!wait_live(&full[s], ph, abort_flag) || *((volatile int*)abort_flag)) {
            atomicExch(abort_flag, 1);
            stop = true;
            break;
          }
          tc::fence_after();
          const uint32_t sa = tc::su32(base + s * Cfg::kStage);
#pragma unroll
          for (int j = 0; j < Cfg::kTapsPerStage; ++j) {
            // HALO: tap dx' = j - 1 starts j pixel rows (64 bytes each) into the
            // row box; the swizzle follows the absolute shared-memory address,
            // which the TMA write and the MMA read share, so the start address
            // simply moves (matrix base offset 0)
            const uint64_t da = tc::desc_sw64(sa + (HALO ? j * 64 : 0), 16, 512);
            const uint64_t db = tc::desc_sw64(sa + Cfg::kA + j * Cfg::kBStride, 16, 512);
#pragma unroll
            for (int kk = 0; kk < 2; ++kk) {
              const uint64_t adv = (uint64_t)((kk * 32) >> 4);      // 16 BF16 = 32 bytes along K
              tc::umma_bf16(acc, da + adv, db + adv, idesc, (it | j | kk) ? 1u : 0u);
            }
          }
          tc::umma_commit(&empty[s]);
        }
        if (!stop) tc::umma_commit(&tfull[b]);
      }
      *consumed = (int)g;
      tc::umma_commit(done);                             // arrives when every MMA issued above has completed
    }
  } else {
    // epilogue warps 2-5: TMEM lane quarter (warp % 4) = pixels 32 (warp % 4) .. + 31 of the tile
    const int q = warp & 3;
    const int m = q * 32 + lane;
    for (int j = 0; j < ntl; ++j) {
      const int b = j & 1;
      bool ok = true;
      if (lane == 0) ok = wait_live(&tfull[b], (uint32_t)((j >> 1) & 1), abort_flag);
      ok = __shfl_sync(0xffffffffu, ok ? 1 : 0, 0) != 0;
      if (!ok) break;
      tc::fence_after();
      int img, x0, y0;
      tile_origin(j, &img, &x0, &y0);
      const int px = x0 + (m % a.bx), py = y0 + (m / a.bx);
      const bool inside = px < a.w && py < a.h;
      const size_t pix = ((size_t)img * a.h + py) * a.w + px;
#pragma unroll 1
      for (int c = 0; c < BN / 32; ++c) {
        uint32_t r[32];
        tc::tmem_ld32(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(b * Cfg::kTmemBuf + c * 32), r);
        const int cb = co0 + c * 32;
        if (!inside || cb >= a.cout) continue;
        float v[32];
#pragma unroll
        for (int e = 0; e < 32; ++e) v[e] = __uint_as_float(r[e]);
#pragma unroll
        for (int e = 0; e < 32; ++e) v[e] += sbias[c * 32 + e];
        if (a.relu) {
#pragma unroll
          for (int e = 0; e < 32; ++e) v[e] = fmaxf(v[e], 0.f);
        }
        if (a.mask) {
          const uint4* mp = reinterpret_cast<const uint4*>(a.mask + pix * a.mask_cs + cb);
#pragma unroll
          for (int g4 = 0; g4 < 4; ++g4) {
            const uint4 mv = __ldg(mp + g4);
            const __nv_bfloat162* mb = reinterpret_cast<const __nv_bfloat162*>(&mv);
#pragma unroll
            for (int e = 0; e < 4; ++e) {
              const float2 f = __bfloat1622float2(mb[e]);
              if (!(f.x > 0.f)) v[g4 * 8 + 2 * e] = 0.f;
              if (!(f.y > 0.f)) v[g4 * 8 + 2 * e + 1] = 0.f;
            }
          }
        }
        uint4* op = reinterpret_cast<uint4*>(a.out + pix * a.out_cs + cb);
#pragma unroll
        for (int g4 = 0; g4 < 4; ++g4) {
          uint4 o;
          __nv_bfloat162* ob = reinterpret_cast<__nv_bfloat162*>(&o);
#pragma unroll
          for (int e = 0; e < 4; ++e) ob[e] = __floats2bfloat162_rn(v[g4 * 8 + 2 * e], v[g4 * 8 + 2 * e + 1]);
          op[g4] = o;
        }
      }
      tc::fence_before();
      __syncwarp();
      if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(tc::su32(&tempty[b])) : "memory");
    }
  }
  __syncwarp();
  // every MMA issued has completed before TMEM is freed; copies issued but
  // not consumed land before the CTA exits
  if (threadIdx.x == 0) tc::mb_wait(done, 0, kWaitCycles);
  __syncthreads();
  if (threadIdx.x == 0) {
    if (*((volatile int*)abort_flag)) atomicOr(a.err, 2);
    for (int g = *consumed; g < *issued; ++g)
      tc::mb_wait(&full[g % Cfg::kStages], (uint32_t)((g / Cfg::kStages) & 1), kWaitCycles);
  }
  tc::fence_before();
  __syncthreads();
  if (warp == 1) {
    tc::fence_after();
    tc::tmem_dealloc(tmem, Cfg::kTmem);
  }
}

template <int BN> struct WgCfg {
  static constexpr int kKp = 64;                       // pixels per K step
  static constexpr int kBox = kKp * 64;                // one 32-channel group of kKp pixels
  static constexpr int kA = 4 * kBox;                  // four (tap, 32-channel) groups
  static constexpr int kB = (BN / 32) * kBox;
  static constexpr int kStage = kA + kB;
  static constexpr int kStages = BN >= 256 ? 4 : 5;
  static constexpr int kTmem = BN < 32 ? 32 : BN;
  static constexpr int kSmem = kStages * kStage + 1024 + 256;
};

template <int BN>
__global__ void __launch_bounds__(kConvThreads) conv_wgrad_tc(const __grid_constant__ CUtensorMap mX,
                                                              const __grid_constant__ CUtensorMap mD, WgArgs a) {
  typedef WgCfg<BN> Cfg;
  extern __shared__ unsigned char smem_raw[];
  const uint32_t raw = tc::su32(smem_raw);
  unsigned char* base = smem_raw + (((raw + 1023u) & ~1023u) - raw);
  uint64_t* full = reinterpret_cast<uint64_t*>(base + Cfg::kStages * Cfg::kStage);
  uint64_t* empty = full + Cfg::kStages;
  uint64_t* done = empty + Cfg::kStages;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(done + 1);
  int* abort_flag = reinterpret_cast<int*>(tmem_slot + 1);
  int* issued = abort_flag + 1;
  int* consumed = abort_flag + 2;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  const int cchunks = a.cin >> 5;
  const int groups = a.taps * cchunks;
  const int g0 = blockIdx.x * 4;
  const long long kb_total = (long long)a.n * a.tiles_y * a.tiles_x;
  const int kb0 = (int)(kb_total * blockIdx.y / gridDim.y);
  const int kb1 = (int)(kb_total * (blockIdx.y + 1) / gridDim.y);
  const int nk = kb1 - kb0;

  if (threadIdx.x == 0) {
    for (int s = 0; s < Cfg::kStages; ++s) { tc::mb_init(&full[s], 1); tc::mb_init(&empty[s], 1); }
    tc::mb_init(done, 1);
    *abort_flag = 0; *issued = 0; *consumed = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) tc::tmem_alloc(tmem_slot, Cfg::kTmem);
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t tmem = *tmem_slot;

  if (threadIdx.x == 0) {
    int it = 0;
    for (; it < nk; ++it) {
      const int s = it % Cfg::kStages;
      const uint32_t ph = (uint32_t)((it / Cfg::kStages) & 1);
      if (!wait_live(&empty[s], ph ^ 1u, abort_flag) || *((volatile int*)abort_flag)) {
        atomicExch(abort_flag, 1);
        break;
      }
      int kb = kb0 + it;
      const int tx = kb % a.tiles_x; kb /= a.tiles_x;
      const int ty = kb % a.tiles_y;
      const int img = kb / a.tiles_y;
      const int x0 = tx * a.bx, y0 = ty * a.by;
      unsigned char* st = base + s * Cfg::kStage;
      tc::mb_expect_tx(&full[s], (uint32_t)Cfg::kStage);
#pragma unroll
      for (int g = 0; g < 4; ++g) {
        const int gg = min(g0 + g, groups - 1);     // rows past the last group: loaded, never stored
        const int tap = gg / cchunks, cc = gg - tap * cchunks;
        int dx = 0, dy = 0;
        if (a.taps == 9) { dx = tap % 3 - 1; dy = tap / 3 - 1; }
        tc::tma_load_4d(st + g * Cfg::kBox, &mX, cc * 32, x0 + dx, y0 + dy, img, &full[s]);
      }
#pragma unroll
      for (int j = 0; j < BN / 32; ++j)
        tc::tma_load_4d(st + Cfg::kA + j * Cfg::kBox, &mD, j * 32, x0, y0, img, &full[s]);
    }
    *issued = it;
  } else if (threadIdx.x == 32) {
    constexpr uint32_t idesc = tc::idesc_bf16(128, BN, 1, 1);
    int it = 0;
    bool stalled = false;
    if (a.stall_flag && !stall_on_unset_flag(a.stall_flag, a.stall_cycles)) {
      atomicExch(abort_flag, 1);
      stalled = true;
    }
    for (; it < nk && !stalled; ++it) {
      const int s = it % Cfg::kStages;
      const uint32_t ph = (uint32_t)((it / Cfg::kStages) & 1);
      if (!wait_live(&full[s], ph, abort_flag) || *((volatile int*)abort_flag)) {
        atomicExch(abort_flag, 1);
        break;
      }
      tc::fence_after();
      const uint32_t sa = tc::su32(base + s * Cfg::kStage);
#pragma unroll
      for (int kk = 0; kk < Cfg::kKp / 16; ++kk) {
        // 16 pixels = two 8-line K groups, 1024 bytes
        const uint64_t da = tc::desc_sw64(sa + kk * 1024, Cfg::kBox, 512);
        const uint64_t db = tc::desc_sw64(sa + Cfg::kA + kk * 1024, Cfg::kBox, 512);
        tc::umma_bf16(tmem, da, db, idesc, (it | kk) ? 1u : 0u);
      }
      tc::umma_commit(&empty[s]);
    }
    *consumed = it;
    tc::umma_commit(done);
  }
  __syncwarp();
  const bool ok_done = tc::mb_wait(done, 0, kWaitCycles);
  tc::fence_after();
  const bool good = __syncthreads_and(ok_done && !*((volatile int*)abort_flag));
  if (good && nk > 0) {
    const int m = warp * 32 + lane;
    const int row = g0 * 32 + m;                      // (tap, ci) row of dW^T
    const bool live = row < groups * 32;
#pragma unroll 1
    for (int c = 0; c < BN / 32; ++c) {
      uint32_t r[32];
      tc::tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(c * 32), r);
      if (!live) continue;
      float* dst = a.dwt + (size_t)row * a.cout + c * 32;
#pragma unroll
      for (int q = 0; q < 32; q += 4)
        asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(dst + q), "f"(__uint_as_float(r[q])),
                     "f"(__uint_as_float(r[q + 1])), "f"(__uint_as_float(r[q + 2])), "f"(__uint_as_float(r[q + 3]))
                     : "memory");
    }
  } else if (!good && threadIdx.x == 0) {
    atomicOr(a.err, 2);
  }
  if (threadIdx.x == 0) {
    for (int it = *consumed; it < *issued; ++it)
      tc::mb_wait(&full[it % Cfg::kStages], (uint32_t)((it / Cfg::kStages) & 1), kWaitCycles);
  }
  tc::fence_before();
  __syncthreads();
  if (warp == 1) {
    tc::fence_after();
    tc::tmem_dealloc(tmem, Cfg::kTmem);
  }
}

// Weight gradient over whole 64-pixel rows (3x3, w >= 64): one CTA per
// (32-channel input chunk cc, group of dy rows) and K range.  Per K step
// (64 pixels of one row) it loads, for each of its dy, one 72-pixel row box
// of X starting at x - 1, and the dZ tile once.  The A operand of dy reads
// that box with a leading-dimension offset of one pixel row (64 bytes):
// M group g (rows 32 g .. 32 g + 31) is the box shifted by g pixels, i.e.
// the taps dx = g - 1 for g < 3 (group 3 is computed and dropped).  One
// accumulator per dy shares the dZ tile.
template <int BN> struct WgHCfg {
  static constexpr int kABox = 72 * 64;
  static constexpr int kAStride = (kABox + 1023) / 1024 * 1024;
  static constexpr int kTmemBuf = pow2_at_least(BN);
  static constexpr int kNdy = (512 / kTmemBuf) >= 3 ? 3 : 2;   // dy rows per CTA (accumulators)
  static constexpr int kTmem = pow2_at_least(kNdy * kTmemBuf) > 512 ? 512 : pow2_at_least(kNdy * kTmemBuf);
  static constexpr int kBBox = 64 * 64;                // 64 pixels x 32 channels of dZ
  static constexpr int kA = kNdy * kAStride;
  static constexpr int kB = (BN / 32) * kBBox;
  static constexpr int kStage = kA + kB;
  static constexpr int kStagesRaw = 200 * 1024 / kStage;
  static constexpr int kStages = kStagesRaw > 6 ? 6 : kStagesRaw;
  static constexpr int kSmem = kStages * kStage + 1024 + 256;
};

template <int BN>
__global__ void __launch_bounds__(kConvThreads) conv_wgrad_halo(const __grid_constant__ CUtensorMap mX,
                                                                const __grid_constant__ CUtensorMap mD, WgArgs a) {
  typedef WgHCfg<BN> Cfg;
  extern __shared__ unsigned char smem_raw[];
  const uint32_t raw = tc::su32(smem_raw);
  unsigned char* base = smem_raw + (((raw + 1023u) & ~1023u) - raw);
  uint64_t* full = reinterpret_cast<uint64_t*>(base + Cfg::kStages * Cfg::kStage);
  uint64_t* empty = full + Cfg::kStages;
  uint64_t* done = empty + Cfg::kStages;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(done + 1);
  int* abort_flag = reinterpret_cast<int*>(tmem_slot + 1);
  int* issued = abort_flag + 1;
  int* consumed = abort_flag + 2;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  const int cchunks = a.cin >> 5;
  const int cc = blockIdx.x % cchunks;
  const int dy0 = (blockIdx.x / cchunks) * Cfg::kNdy;           // first dy index (0..2) of this CTA
  const int ndy = min(Cfg::kNdy, 3 - dy0);
  const long long kb_total = (long long)a.n * a.tiles_y * a.tiles_x;
  const int kb0 = (int)(kb_total * blockIdx.y / gridDim.y);
  const int kb1 = (int)(kb_total * (blockIdx.y + 1) / gridDim.y);
  const int nk = kb1 - kb0;

  if (threadIdx.x == 0) {
    for (int s = 0; s < Cfg::kStages; ++s) { tc::mb_init(&full[s], 1); tc::mb_init(&empty[s], 1); }
    tc::mb_init(done, 1);
    *abort_flag = 0; *issued = 0; *consumed = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) tc::tmem_alloc(tmem_slot, Cfg::kTmem);
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t tmem = *tmem_slot;

  if (threadIdx.x == 0) {
    int it = 0;
    for (; it < nk; ++it) {
      const int s = it % Cfg::kStages;
      const uint32_t ph = (uint32_t)((it / Cfg::kStages) & 1);
      if (!wait_live(&empty[s], ph ^ 1u, abort_flag) || *((volatile int*)abort_flag)) {
        atomicExch(abort_flag, 1);
        break;
      }
      int kb = kb0 + it;
      const int tx = kb % a.tiles_x; kb /= a.tiles_x;
      const int ty = kb % a.tiles_y;
      const int img = kb / a.tiles_y;
      const int x0 = tx * a.bx, y0 = ty * a.by;
      unsigned char* st = base + s * Cfg::kStage;
      tc::mb_expect_tx(&full[s], (uint32_t)(ndy * Cfg::kABox + Cfg::kB));
      for (int d = 0; d < ndy; ++d)
        tc::tma_load_4d(st + d * Cfg::kAStride, &mX, cc * 32, x0 - 1, y0 + (dy0 + d - 1), img, &full[s]);
#pragma unroll
      for (int j = 0; j < BN / 32; ++j)
        tc::tma_load_4d(st + Cfg::kA + j * Cfg::kBBox, &mD, j * 32, x0, y0, img, &full[s]);
    }
    *issued = it;
  } else if (threadIdx.x == 32) {
    constexpr uint32_t idesc = tc::idesc_bf16(128, BN, 1, 1);
    int it = 0;
    bool stalled = false;
    if (a.stall_flag && !stall_on_unset_flag(a.stall_flag, a.stall_cycles)) {
      atomicExch(abort_flag, 1);
      stalled = true;
    }
    for (; it < nk && !stalled; ++it) {
      const int s = it % Cfg::kStages;
      const uint32_t ph = (uint32_t)((it / Cfg::kStages) & 1);
      if (!wait_live(&full[s], ph, abort_flag) || *((volatile int*)abort_flag)) {
        atomicExch(abort_flag, 1);
        break;
      }
      tc::fence_after();
      const uint32_t sa = tc::su32(base + s * Cfg::kStage);
      for (int d = 0; d < ndy; ++d) {
#pragma unroll
        for (int kk = 0; kk < 4; ++kk) {
          // 16 pixels = two 8-row K groups, 1024 bytes; M groups one pixel row apart
          const uint64_t da = tc::desc_sw64(sa + d * Cfg::kAStride + kk * 1024, 64, 512);
          const uint64_t db = tc::desc_sw64(sa + Cfg::kA + kk * 1024, Cfg::kBBox, 512);
          tc::umma_bf16(tmem + (uint32_t)(d * Cfg::kTmemBuf), da, db, idesc, (it | kk) ? 1u : 0u);
        }
      }
      tc::umma_commit(&empty[s]);
    }
    *consumed = it;
    tc::umma_commit(done);
  }
  __syncwarp();
  const bool ok_done = tc::mb_wait(done, 0, kWaitCycles);
  tc::fence_after();
  const bool good = __syncthreads_and(ok_done && !*((volatile int*)abort_flag));
  if (good && nk > 0 && warp < 3) {
    // warp g = tap dx = g - 1 of each dy: dW^T row (3 dy + g) cin + cc 32 + lane
    for (int d = 0; d < ndy; ++d) {
      const int tap = 3 * (dy0 + d) + warp;
      const int row = tap * a.cin + cc * 32 + lane;
#pragma unroll 1
      for (int c = 0; c < BN / 32; ++c) {
        uint32_t r[32];
        tc::tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(d * Cfg::kTmemBuf + c * 32), r);
        float* dst = a.dwt + (size_t)row * a.cout + c * 32;
#pragma unroll
        for (int q = 0; q < 32; q += 4)
          asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(dst + q), "f"(__uint_as_float(r[q])),
                       "f"(__uint_as_float(r[q + 1])), "f"(__uint_as_float(r[q + 2])), "f"(__uint_as_float(r[q + 3]))
                       : "memory");
      }
    }
  } else if (!good && threadIdx.x == 0) {
    atomicOr(a.err, 2);
  }
  if (threadIdx.x == 0) {
    for (int it = *consumed; it < *issued; ++it)
      tc::mb_wait(&full[it % Cfg::kStages], (uint32_t)((it / Cfg::kStages) & 1), kWaitCycles);
  }
  tc::fence_before();
  __syncthreads();
  if (warp == 1) {
    tc::fence_after();
    tc::tmem_dealloc(tmem, Cfg::kTmem);
  }
}

template <int BN>
oh_status launch_wgrad_halo(const CUtensorMap& mX, const CUtensorMap& mD, const WgArgs& a, long long kb_total,
                            cudaStream_t st) {
  typedef WgHCfg<BN> Cfg;
  OH_CUDA_TRY(cudaFuncSetAttribute(conv_wgrad_halo<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize, Cfg::kSmem));
  const int gx = (a.cin / 32) * ((3 + Cfg::kNdy - 1) / Cfg::kNdy);
  long long splits = std::max(1LL, (4LL * sm_count() + gx - 1) / gx);
  splits = std::min(splits, std::max(1LL, kb_total / 16));
  splits = std::min(splits, 65535LL);
  conv_wgrad_halo<BN><<<dim3(gx, (int)splits), kConvThreads, Cfg::kSmem, st>>>(mX, mD, a);
  OH_LAUNCH_CHECK();
  return OH_OK;
}

// Patch of `pixels` pixels for an image row of width w: bx = min(w, pixels),
// by = pixels / bx; widths below `pixels` must divide it.
bool patch_shape(int w, int pixels, int* bx, int* by) {
  if (w >= pixels) { *bx = pixels; *by = 1; return true; }
  if (pixels % w) return false;
  *bx = w; *by = pixels / w;
  return true;
}

template <int BN, bool HALO>
oh_status launch_fwd(const CUtensorMap& mX, const CUtensorMap& mW, const ConvArgs& a, long long tiles, cudaStream_t st) {
  typedef FwdCfg<BN, HALO> Cfg;
  OH_CUDA_TRY(cudaFuncSetAttribute(conv_fwd_tc<BN, HALO>, cudaFuncAttributeMaxDynamicSharedMemorySize, Cfg::kSmem));
  // persistent grid: the CTAs that fit on an SM by shared memory and tensor
  // memory (512 columns), at most four, times the SMs, spread over the
  // output-channel tiles
  const int by_smem = (int)((228 * 1024) / (Cfg::kSmem + 1024));
  const int per_sm = std::max(1, std::min(4, std::min(by_smem, 512 / Cfg::kTmem)));
  const int ctiles = (a.cout + BN - 1) / BN;
  const long long want = std::max(1LL, (long long)sm_count() * per_sm / ctiles);
  const int gx = (int)std::min(tiles, want);
  conv_fwd_tc<BN, HALO><<<dim3(gx, ctiles), Cfg::kThreads, Cfg::kSmem, st>>>(mX, mW, a);
  OH_LAUNCH_CHECK();
  return OH_OK;
}

template <int BN>
oh_status launch_wgrad(const CUtensorMap& mX, const CUtensorMap& mD, const WgArgs& a, int mtiles, int splits,
                       cudaStream_t st) {
  typedef WgCfg<BN> Cfg;
  OH_CUDA_TRY(cudaFuncSetAttribute(conv_wgrad_tc<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize, Cfg::kSmem));
  conv_wgrad_tc<BN><<<dim3(mtiles, splits), kConvThreads, Cfg::kSmem, st>>>(mX, mD, a);
  OH_LAUNCH_CHECK();
  return OH_OK;
}

}  // namespace

oh_status tc_arch_check() {
  int dev = 0, major = 0, minor = 0;
  OH_CUDA_TRY(cudaGetDevice(&dev));
  OH_CUDA_TRY(cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev));
  OH_CUDA_TRY(cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev));
  if (major != 10 || minor != 3) return fail(OH_ERR_UNSUPPORTED_SIZE, "the tensor-core convolutions are built for sm_103a");
  return OH_OK;
}

oh_status conv_enqueue(oh_ctx* ctx, const ConvDesc& d, cudaStream_t st, const char* timer_name) {
  if (d.cin % 32 || d.cin <= 0 || d.cout <= 0 || d.cout % 32 || d.cout > 1024 || (d.taps != 9 && d.taps != 1))
    return fail(OH_ERR_INVALID_ARG, "convolution: cin and cout must be positive multiples of 32 (cout <= 1024), taps 1 or 9");
  if (d.x_cs % 8 || d.out_cs % 8 || (d.mask && (d.mask_cs % 8 || d.mask_cs < d.cout)) || d.x_cs < d.cin ||
      d.out_cs < d.cout)
    return fail(OH_ERR_INVALID_ARG, "convolution: channel strides must be multiples of 8 and cover the channels");
  if (!d.x || !d.w_mat || !d.out) return fail(OH_ERR_INVALID_ARG, "convolution: null tensor");
  if ((reinterpret_cast<uintptr_t>(d.x) | reinterpret_cast<uintptr_t>(d.w_mat) | reinterpret_cast<uintptr_t>(d.out) |
       reinterpret_cast<uintptr_t>(d.mask)) & 15)
    return fail(OH_ERR_INVALID_ARG, "convolution: tensors must be 16-byte aligned");
  OH_TRY(tc_arch_check());
  ConvArgs a{};
  if (!patch_shape(d.w, 128, &a.bx, &a.by)) return fail(OH_ERR_UNSUPPORTED_SIZE, "convolution: widths below 128 must divide 128");
  a.taps = d.taps; a.cin = d.cin; a.cout = d.cout; a.w = d.w; a.h = d.h; a.n = d.n;
  a.tiles_x = (d.w + a.bx - 1) / a.bx; a.tiles_y = (d.h + a.by - 1) / a.by;
  a.sign = d.sign;
  a.bias = d.bias; a.relu = d.relu;
  a.mask = reinterpret_cast<const __nv_bfloat16*>(d.mask); a.mask_cs = d.mask_cs;
  a.out = reinterpret_cast<__nv_bfloat16*>(d.out); a.out_cs = d.out_cs;
  a.err = ctx->dev_err;
  if (ctx->stall_mask & kStallConvolution) { a.stall_flag = ctx->dev_err + 1; a.stall_cycles = ctx->stall_cycles; }
  const long long tiles = (long long)a.tiles_x * a.tiles_y * d.n;
  if (tiles > 0x7fffffffLL) return fail(OH_ERR_UNSUPPORTED_SIZE, "convolution: too many pixel tiles");
  // output-channel tile: all of cout up to 256 (384 as two halves), else the
  // largest of 256, 192, 128, 96, 64, 32 that divides it; halved while the
  // pixel tiles alone cannot fill two CTAs per SM
  int bn = 32;
  for (int c : {256, 192, 128, 96, 64})
    if (d.cout % c == 0) { bn = c; break; }
  while ((bn == 256 || bn == 128 || bn == 64 || bn == 192) && tiles * ((d.cout + bn - 1) / bn) < 2LL * sm_count())
    bn /= 2;
  // 3x3 over whole 128-pixel rows: one halo row box per (dy, 32 channels)
  const char* hv = std::getenv("OH_CONV_HALO");
  const bool halo = d.taps == 9 && a.by == 1 && a.bx == 128 && !(hv && std::atoi(hv) == 0);
  CUtensorMap mX, mW;
  OH_TRY(tc::map_act4d(&mX, d.x, d.cin, d.x_cs, d.w, d.h, d.n, halo ? 136 : a.bx, a.by));
  OH_TRY(tc::map_mat2d(&mW, d.w_mat, d.taps * d.cin, d.cout, bn));
  KernelTimer kt(ctx, timer_name, st);
  switch (bn) {
    case 32: return halo ? launch_fwd<32, true>(mX, mW, a, tiles, st) : launch_fwd<32, false>(mX, mW, a, tiles, st);
    case 64: return halo ? launch_fwd<64, true>(mX, mW, a, tiles, st) : launch_fwd<64, false>(mX, mW, a, tiles, st);
    case 96: return halo ? launch_fwd<96, true>(mX, mW, a, tiles, st) : launch_fwd<96, false>(mX, mW, a, tiles, st);
    case 128: return halo ? launch_fwd<128, true>(mX, mW, a, tiles, st) : launch_fwd<128, false>(mX, mW, a, tiles, st);
    case 192: return halo ? launch_fwd<192, true>(mX, mW, a, tiles, st) : launch_fwd<192, false>(mX, mW, a, tiles, st);
    default: return halo ? launch_fwd<256, true>(mX, mW, a, tiles, st) : launch_fwd<256, false>(mX, mW, a, tiles, st);
  }
}

oh_status wgrad_enqueue(oh_ctx* ctx, const WgradDesc& d, cudaStream_t st, const char* timer_name) {
  if (d.cin % 32 || d.cin <= 0 || (d.cout != 32 && d.cout != 64 && d.cout != 128 && d.cout != 256) ||
      (d.taps != 9 && d.taps != 1))
    return fail(OH_ERR_INVALID_ARG, "weight gradient: cin a positive multiple of 32, cout 32, 64, 128 or 256, taps 1 or 9");
  if (d.x_cs % 8 || d.dz_cs % 8 || d.x_cs < d.cin || d.dz_cs < d.cout)
    return fail(OH_ERR_INVALID_ARG, "weight gradient: channel strides must be multiples of 8 and cover the channels");
  if (!d.x || !d.dz || !d.dwt) return fail(OH_ERR_INVALID_ARG, "weight gradient: null tensor");
  if ((reinterpret_cast<uintptr_t>(d.x) | reinterpret_cast<uintptr_t>(d.dz) | reinterpret_cast<uintptr_t>(d.dwt)) & 15)
    return fail(OH_ERR_INVALID_ARG, "weight gradient: tensors must be 16-byte aligned");
  OH_TRY(tc_arch_check());
  WgArgs a{};
  if (!patch_shape(d.w, 64, &a.bx, &a.by)) return fail(OH_ERR_UNSUPPORTED_SIZE, "weight gradient: widths below 64 must divide 64");
  a.taps = d.taps; a.cin = d.cin; a.cout = d.cout; a.w = d.w; a.h = d.h; a.n = d.n;
  a.tiles_x = (d.w + a.bx - 1) / a.bx; a.tiles_y = (d.h + a.by - 1) / a.by;
  a.dwt = d.dwt;
  a.err = ctx->dev_err;
  if (ctx->stall_mask & kStallConvolution) { a.stall_flag = ctx->dev_err + 1; a.stall_cycles = ctx->stall_cycles; }
  const int groups = d.taps * (d.cin / 32);
  const int mtiles = (groups + 3) / 4;
  const long long kb_total = (long long)a.tiles_x * a.tiles_y * d.n;
  // 3x3 over whole 64-pixel rows: one row box per (dy, 32 channels) feeds the three dx taps
  const char* hv = std::getenv("OH_CONV_HALO");
  if (d.taps == 9 && a.by == 1 && a.bx == 64 && d.cout <= 128 && !(hv && std::atoi(hv) == 0)) {
    CUtensorMap mX, mD;
    OH_TRY(tc::map_act4d(&mX, d.x, d.cin, d.x_cs, d.w, d.h, d.n, 72, 1));
    OH_TRY(tc::map_act4d(&mD, d.dz, d.cout, d.dz_cs, d.w, d.h, d.n, 64, 1));
    KernelTimer kt(ctx, timer_name, st);
    switch (d.cout) {
      case 32: return launch_wgrad_halo<32>(mX, mD, a, kb_total, st);
      case 64: return launch_wgrad_halo<64>(mX, mD, a, kb_total, st);
      default: return launch_wgrad_halo<128>(mX, mD, a, kb_total, st);
    }
  }
  // K splits: about four CTAs per SM over all M tiles, each with at least 16 K steps
  long long splits = std::max(1LL, (4LL * sm_count() + mtiles - 1) / mtiles);
  splits = std::min(splits, std::max(1LL, kb_total / 16));
  splits = std::min(splits, 65535LL);
  CUtensorMap mX, mD;
  OH_TRY(tc::map_act4d(&mX, d.x, d.cin, d.x_cs, d.w, d.h, d.n, a.bx, a.by));
  OH_TRY(tc::map_act4d(&mD, d.dz, d.cout, d.dz_cs, d.w, d.h, d.n, a.bx, a.by));
  KernelTimer kt(ctx, timer_name, st);
  switch (d.cout) {
    case 32: return launch_wgrad<32>(mX, mD, a, mtiles, (int)splits, st);
    case 64: return launch_wgrad<64>(mX, mD, a, mtiles, (int)splits, st);
    case 128: return launch_wgrad<128>(mX, mD, a, mtiles, (int)splits, st);
    default: return launch_wgrad<256>(mX, mD, a, mtiles, (int)splits, st);
  }
}

}  // namespace oh

using namespace oh;

extern "C" {

oh_status oh_conv2d_bf16(oh_ctx* ctx, int taps, int sign, int n, int h, int w, int cin, int cout, const void* x,
                         int x_cs, const void* wmat, const float* bias, int relu, const void* mask, int mask_cs,
                         void* out, int out_cs, void* stream) {
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  CallScope cs(ctx, st);
  OH_TRY(cs.status());
  if (n < 1 || h < 1 || w < 1 || (sign != 1 && sign != -1)) return fail(OH_ERR_INVALID_ARG, "convolution: bad sizes or sign");
  ConvDesc d{};
  d.taps = taps; d.sign = sign; d.n = n; d.h = h; d.w = w; d.cin = cin; d.cout = cout;
  d.x = x; d.x_cs = x_cs; d.w_mat = wmat; d.bias = bias; d.relu = relu; d.mask = mask; d.mask_cs = mask_cs;
  d.out = out; d.out_cs = out_cs;
  return conv_enqueue(ctx, d, st, "conv_fwd_tc");
}

oh_status oh_conv2d_wgrad_bf16(oh_ctx* ctx, int taps, int n, int h, int w, int cin, int cout, const void* x, int x_cs,
                               const void* dz, int dz_cs, float* dwt, void* stream) {
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  CallScope cs(ctx, st);
  OH_TRY(cs.status());
  if (n < 1 || h < 1 || w < 1) return fail(OH_ERR_INVALID_ARG, "weight gradient: bad sizes");
  WgradDesc d{};
  d.taps = taps; d.n = n; d.h = h; d.w = w; d.cin = cin; d.cout = cout;
  d.x = x; d.x_cs = x_cs; d.dz = dz; d.dz_cs = dz_cs; d.dwt = dwt;
  return wgrad_enqueue(ctx, d, st, "conv_wgrad_tc");
}

}  // extern "C"
