// Tensor-core engine of the paraxial point-light-source sum (cwoPLS::Fresnel,
// cwoPLS.cpp:370-424, and CGHFresnel, :472-520).
//
// U[i][j] = sum_k Ey[k][i] Ex[k][j] (Ey carries a_k e^{i ph}) is a complex
// matrix product.  Embedded in reals (point k -> columns 2k, 2k+1):
//   A[i][2k] = Re Ey, A[i][2k+1] = Im Ey                       (M = Ny rows)
//   B[2j][2k] = Re Ex, B[2j][2k+1] = -Im Ex,
//   B[2j+1][2k] = Im Ex, B[2j+1][2k+1] = Re Ex                 (N = 2 Nx rows)
//   C = A B^T:  C[i][2j] = Re U[i][j], C[i][2j+1] = Im U[i][j]
// so C is the complex64 field itself.  Each operand is split into BF16 high
// and low parts (x = hi + lo + O(2^-17 x)); C = Ahi Bhi + Ahi Blo + Alo Bhi in
// FP32 (relative error ~1e-5).
//
// Kernel: one CTA per 128 x 256 tile of C (and per K split), 4 warps.
// Thread 0 loads K-slices of 32 (Ahi, Alo, Bhi, Blo: 48 KB, four stages) with
// TMA (64-byte swizzle); thread 32 issues tcgen05.mma (M=128, N=256, K=16,
// BF16 -> FP32 in 256 TMEM columns) and releases each stage with
// tcgen05.commit; all four warps then read the accumulator with tcgen05.ld
// (warp w owns TMEM lanes 32w..32w+31) and store (or, with K splits, add)
// the tile.  Every mbarrier wait gives up after about a second, sets the
// context's device error word and lets the CTA drain and free its TMEM.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cmath>
#include <mutex>
#include "pls.cuh"

namespace oh {

namespace {

constexpr int kBM = 128, kBN = 256, kBK = 32, kStages = 4;
constexpr int kTileA = kBM * kBK * 2;                 // 8 KB
constexpr int kTileB = kBN * kBK * 2;                 // 16 KB
constexpr int kStageBytes = 2 * kTileA + 2 * kTileB;  // 48 KB
constexpr int kTmemCols = 256;
constexpr int kSmemBytes = kStages * kStageBytes + 1024 /*alignment*/ + 256 /*barriers*/;
constexpr long long kWaitCycles = 2000000000LL;       // ~1 s at 2 GHz

__device__ __forceinline__ uint32_t su32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mb_init(uint64_t* b, uint32_t n) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(su32(b)), "r"(n) : "memory");
}
__device__ __forceinline__ void mb_expect_tx(uint64_t* b, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(su32(b)), "r"(bytes) : "memory");
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

// as mb_wait, also giving up as soon as another role has set *abort
__device__ __forceinline__ bool mb_wait_live(uint64_t* b, uint32_t parity, const int* abort) {
  const long long t0 = clock64();
  while (!mb_try(b, parity)) {
    if (*((volatile const int*)abort) || clock64() - t0 > kWaitCycles) return false;
  }
  return true;
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int c0, int c1, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          su32(dst)),
      "l"(map), "r"(c0), "r"(c1), "r"(su32(bar))
      : "memory");
}

// Shared-memory matrix descriptor: K-major tile with 64-byte swizzle (rows of
// kBK = 32 BF16), 8-row atoms 512 bytes apart (SBO), version 1, layout SWIZZLE_64B.
__device__ __forceinline__ uint64_t sw_desc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFF) >> 4);
  d |= (uint64_t)1 << 16;                 // leading byte offset (unused for swizzled K-major)
  d |= (uint64_t)((8 * kBK * 2) >> 4) << 32;   // stride byte offset: 8 rows
  d |= (uint64_t)1 << 46;                 // descriptor version
  d |= (uint64_t)4 << 61;                 // SWIZZLE_64B
  return d;
}

// Instruction descriptor, kind::f16: D FP32, A and B BF16, both K-major,
// N = 256, M = 128.
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kBN >> 3) << 17) |
                            ((uint32_t)(kBM >> 4) << 24);

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

struct TcArgs {
  int kb_total;     // 64-wide K blocks of the product
  int splits;       // K splits (gridDim.z): split z takes blocks [z kb_total / splits, (z+1) kb_total / splits)
  int mode;         // OH_PLS_FRESNEL (complex out) or OH_PLS_CGH_FRESNEL (real out)
  int rows, cols;   // C extent: Ny x 2 Nx
  int atomic;       // add into out (K splits or point chunks)
  int vec4;         // out rows start on 16-byte boundaries (base aligned, cols % 4 == 0)
  float* out;
  int* err;
  const int* stall_flag;   // error-path test hook (oh_ctx_set_test_stall), null otherwise
  long long stall_cycles;
};

__global__ void __launch_bounds__(128, 1) pls_tc_gemm(const __grid_constant__ CUtensorMap mAhi,
                                                      const __grid_constant__ CUtensorMap mAlo,
                                                      const __grid_constant__ CUtensorMap mBhi,
                                                      const __grid_constant__ CUtensorMap mBlo, TcArgs a) {
  extern __shared__ unsigned char smem_raw[];
  const uint32_t raw = su32(smem_raw);
  const uint32_t pad = ((raw + 1023u) & ~1023u) - raw;
  unsigned char* base = smem_raw + pad;
  uint64_t* bars = reinterpret_cast<uint64_t*>(base + kStages * kStageBytes);
  uint64_t* full = bars;                // [kStages]
  uint64_t* empty = bars + kStages;     // [kStages]
  uint64_t* done = bars + 2 * kStages;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2 * kStages + 1);
  int* abort_flag = reinterpret_cast<int*>(tmem_slot + 1);
  int* issued = abort_flag + 1;
  int* consumed = abort_flag + 2;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int n0 = blockIdx.x * kBN, m0 = blockIdx.y * kBM;
  const int kb0 = (int)((long long)blockIdx.z * a.kb_total / a.splits);
  const int nkb = (int)((long long)(blockIdx.z + 1) * a.kb_total / a.splits) - kb0;

  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) { mb_init(&full[s], 1); mb_init(&empty[s], 1); }
    mb_init(done, 1);
    *abort_flag = 0;
    *issued = 0;
    *consumed = 0;
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

  auto sA = [&](int s, int lo) { return base + s * kStageBytes + lo * kTileA; };
  auto sB = [&](int s, int lo) { return base + s * kStageBytes + 2 * kTileA + lo * kTileB; };

  if (threadIdx.x == 0) {
    // producer
    int it = 0;
    for (; it < nkb; ++it) {
      const int s = it % kStages;
      const uint32_t ph = (uint32_t)((it / kStages) & 1);
      if (!mb_wait_live(&empty[s], ph ^ 1u, abort_flag) || *((volatile int*)abort_flag)) {
        atomicExch(abort_flag, 1);
        break;
      }
      mb_expect_tx(&full[s], (uint32_t)kStageBytes);
      const int kx = (kb0 + it) * kBK;
      tma_load_2d(sA(s, 0), &mAhi, kx, m0, &full[s]);
      tma_load_2d(sA(s, 1), &mAlo, kx, m0, &full[s]);
      tma_load_2d(sB(s, 0), &mBhi, kx, n0, &full[s]);
      tma_load_2d(sB(s, 1), &mBlo, kx, n0, &full[s]);
    }
    *issued = it;
  } else if (threadIdx.x == 32) {
    // MMA issuer
    int it = 0;
    bool stalled = false;
    if (a.stall_flag && !stall_on_unset_flag(a.stall_flag, a.stall_cycles)) {
      atomicExch(abort_flag, 1);         // nothing consumed; the drain lets issued copies land
      stalled = true;
    }
    for (; it < nkb && !stalled; ++it) {
      const int s = it % kStages;
      const uint32_t ph = (uint32_t)((it / kStages) & 1);
      if (!mb_wait(&full[s], ph)) {
        atomicExch(abort_flag, 1);
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint64_t ah = sw_desc(su32(sA(s, 0))), al = sw_desc(su32(sA(s, 1)));
      const uint64_t bh = sw_desc(su32(sB(s, 0))), bl = sw_desc(su32(sB(s, 1)));
#pragma unroll
      for (int kk = 0; kk < kBK / 16; ++kk) {
        const uint64_t adv = (uint64_t)((kk * 32) >> 4);     // 16 BF16 = 32 bytes along K
        umma(tmem, ah + adv, bh + adv, (it | kk) ? 1u : 0u);
        umma(tmem, ah + adv, bl + adv, 1u);
        umma(tmem, al + adv, bh + adv, 1u);
      }
      umma_commit(&empty[s]);
    }
    *consumed = it;
    umma_commit(done);      // arrives once every MMA issued above has completed
  }
  // epilogue: all four warps
  __syncwarp();
  const bool ok_done = mb_wait(done, 0);
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const bool good = __syncthreads_and(ok_done && !*((volatile int*)abort_flag));
  if (good) {
    const int row = m0 + warp * 32 + lane;
#pragma unroll 1
    for (int c = 0; c < kBN / 32; ++c) {
      uint32_t r[32];
      tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(c * 32), r);
      if (row < a.rows) {
        const int col0 = n0 + c * 32;
        if (a.mode == OH_PLS_CGH_FRESNEL) {
          float* dst = a.out + (size_t)row * (a.cols >> 1) + (col0 >> 1);
#pragma unroll
          for (int q = 0; q < 32; q += 2) {
            if (col0 + q < a.cols) {
              const float v = __uint_as_float(r[q]);
              if (a.atomic) atomicAdd(dst + (q >> 1), v);
              else dst[q >> 1] = v;
            }
          }
        } else {
          float* dst = a.out + (size_t)row * a.cols + col0;
          if (a.atomic && a.vec4 && col0 + 32 <= a.cols) {
            // 16-byte aligned rows: vector reductions
#pragma unroll
            for (int q = 0; q < 32; q += 4)
              asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(dst + q), "f"(__uint_as_float(r[q])),
                           "f"(__uint_as_float(r[q + 1])), "f"(__uint_as_float(r[q + 2])), "f"(__uint_as_float(r[q + 3]))
                           : "memory");
          } else {
#pragma unroll
            for (int q = 0; q < 32; ++q) {
              if (col0 + q < a.cols) {
                const float v = __uint_as_float(r[q]);
                if (a.atomic) atomicAdd(dst + q, v);
                else dst[q] = v;
              }
            }
          }
        }
      }
    }
  } else if (threadIdx.x == 0) {
    atomicOr(a.err, 2);
  }
  // drain: copies the MMA side did not consume must land before exit
  if (threadIdx.x == 0) {
    for (int it = *consumed; it < *issued; ++it) mb_wait(&full[it % kStages], (uint32_t)((it / kStages) & 1));
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 1) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
  }
}

// Operand tables for points [0, n): A (rows M_pad, K_pad) and B (rows N_pad,
// K_pad), BF16 high and low parts, zero outside the data.  Grid: x over point
// slots, y over A rows then B row pairs; each thread writes BF16 pairs.
__device__ __forceinline__ void split2(float x, float y, __nv_bfloat162* hi, __nv_bfloat162* lo) {
  const __nv_bfloat162 h = __floats2bfloat162_rn(x, y);
  *hi = h;
  *lo = __floats2bfloat162_rn(x - __low2float(h), y - __high2float(h));
}

constexpr int kTabRows = 16;     // table rows per thread (A rows, or B row pairs)

__global__ void __launch_bounds__(256) pls_tc_tables(PlsGeom g, const PlsPt* __restrict__ pts, int n, int kpad,
                                                     int mpad, __nv_bfloat16* __restrict__ ahi,
                                                     __nv_bfloat16* __restrict__ alo, __nv_bfloat16* __restrict__ bhi,
                                                     __nv_bfloat16* __restrict__ blo) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;      // point slot
  if (k >= kpad / 2) return;
  const int r0 = blockIdx.y * kTabRows;                      // mpad is a multiple of kTabRows
  const bool live = k < n;
  if (r0 < mpad) {
    unsigned long long qa = 0, qb = 0, qg = 0;
    int qm = 0;
    float ar = 0.f, ai = 0.f;
    if (live) {
      const PlsPt& q = pts[k];
      qa = q.ay; qb = q.by; qg = q.gy; qm = q.my; ar = q.ar; ai = q.ai;
    }
#pragma unroll 4
    for (int r = r0; r < r0 + kTabRows; ++r) {
      float re = 0.f, im = 0.f;
      if (live && r < g.ny) {
        float c, s;
        pls_cis_neg(pls_turns(qa, qb, qg, r - qm), &c, &s);
        re = -(ar * c - ai * s);
        im = -(ar * s + ai * c);
      }
      const size_t o = (size_t)r * kpad + 2 * k;
      split2(re, im, reinterpret_cast<__nv_bfloat162*>(ahi + o), reinterpret_cast<__nv_bfloat162*>(alo + o));
    }
  } else {
    unsigned long long qa = 0, qb = 0, qg = 0;
    int qm = 0;
    if (live) {
      const PlsPt& q = pts[k];
      qa = q.ax; qb = q.bx; qg = q.gx; qm = q.mx;
    }
    const int j0 = r0 - mpad;
#pragma unroll 4
    for (int j = j0; j < j0 + kTabRows; ++j) {
      float re = 0.f, im = 0.f;
      if (live && j < g.nx) {
        float c, s;
        pls_cis_neg(pls_turns(qa, qb, qg, j - qm), &c, &s);
        re = -c;
        im = -s;
      }
      const size_t o0 = (size_t)(2 * j) * kpad + 2 * k, o1 = o0 + kpad;
      split2(re, -im, reinterpret_cast<__nv_bfloat162*>(bhi + o0), reinterpret_cast<__nv_bfloat162*>(blo + o0));
      split2(im, re, reinterpret_cast<__nv_bfloat162*>(bhi + o1), reinterpret_cast<__nv_bfloat162*>(blo + o1));
    }
  }
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

oh_status encode_fn(EncodeTiledFn* out) {
  static std::mutex mu;
  static EncodeTiledFn fn = nullptr;
  std::lock_guard<std::mutex> lk(mu);
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q);
    if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !p)
      return fail(OH_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
    fn = reinterpret_cast<EncodeTiledFn>(p);
  }
  *out = fn;
  return OH_OK;
}

// 2-D BF16 tensor [rows][kpad], box 64 (K) x box_rows, 128-byte swizzle
oh_status make_map(CUtensorMap* m, void* ptr, int kpad, int rows, int box_rows) {
  EncodeTiledFn fn;
  OH_TRY(encode_fn(&fn));
  const cuuint64_t dims[2] = {(cuuint64_t)kpad, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {(cuuint64_t)kpad * 2};
  const cuuint32_t box[2] = {(cuuint32_t)kBK, (cuuint32_t)box_rows};
  const cuuint32_t estr[2] = {1, 1};
  const CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, ptr, dims, strides, box, estr,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(OH_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
  return OH_OK;
}

}  // namespace

oh_status pls_tensor_enqueue(oh_ctx* ctx, const PlsGeom& g, const PlsPt* pts, int n, void* out, cudaStream_t st) {
  if (g.mode != OH_PLS_FRESNEL && g.mode != OH_PLS_CGH_FRESNEL)
    return fail(OH_ERR_UNSUPPORTED_SIZE, "the tensor engine covers FRESNEL and CGH_FRESNEL");
  int dev = 0, major = 0, minor = 0;
  OH_CUDA_TRY(cudaGetDevice(&dev));
  OH_CUDA_TRY(cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev));
  OH_CUDA_TRY(cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev));
  if (major != 10 || minor != 3) return fail(OH_ERR_UNSUPPORTED_SIZE, "the tensor engine is built for sm_103a");
  const int mpad = (g.ny + kBM - 1) / kBM * kBM;
  const int npad = (2 * g.nx + kBN - 1) / kBN * kBN;
  if ((mpad + npad / 2) / kTabRows > 65535) return fail(OH_ERR_UNSUPPORTED_SIZE, "field too large for the tensor engine");
  // points per chunk: tables (mpad + npad) x 2 x 2 bytes per K column, <= 512 MiB
  const size_t per_k = (size_t)(mpad + npad) * 4;
  const size_t fit = ((size_t)512 << 20) / (per_k * 2);
  const int chunk_pts = (size_t)n <= fit ? n : (int)std::max<size_t>(32, fit / 32 * 32);
  const int kpad_max = (std::min(chunk_pts, n) * 2 + kBK - 1) / kBK * kBK;
  void* tp;
  OH_TRY(scratch(ctx, "pls.tc", (size_t)kpad_max * per_k, &tp));
  __nv_bfloat16* ahi = static_cast<__nv_bfloat16*>(tp);
  __nv_bfloat16* alo = ahi + (size_t)mpad * kpad_max;
  __nv_bfloat16* bhi = alo + (size_t)mpad * kpad_max;
  __nv_bfloat16* blo = bhi + (size_t)npad * kpad_max;
  int* err = ctx->dev_err;
  const int tiles = (mpad / kBM) * (npad / kBN);
  const int nchunks = (n + chunk_pts - 1) / chunk_pts;
  bool atomic = nchunks > 1;
  OH_CUDA_TRY(cudaFuncSetAttribute(pls_tc_gemm, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes));
  for (int c0 = 0; c0 < n; c0 += chunk_pts) {
    const int cnt = std::min(chunk_pts, n - c0);
    const int kpad = (cnt * 2 + kBK - 1) / kBK * kBK;
    const int kb_total = kpad / kBK;
    // K splits: the fewest that fill the SMs' waves to 95 % (each split keeps
    // at least 8 K blocks), else the best filling
    int splits = 1;
    {
      const int sms = oh::sm_count();
      const int smax = std::max(1, kb_total / 8);
      double best = -1.0;
      for (int sp = 1; sp <= std::min(smax, 32); ++sp) {
        const long long ctas = (long long)tiles * sp;
        const long long waves = (ctas + sms - 1) / sms;
        const double eff = (double)ctas / (double)(waves * sms);
        if (eff > best + 1e-9) { best = eff; splits = sp; }
        if (eff >= 0.95) break;
      }
    }
    if (splits > 1) atomic = true;
    if (atomic && c0 == 0)
      OH_CUDA_TRY(cudaMemsetAsync(out, 0, (size_t)g.ny * g.nx * (g.mode == OH_PLS_CGH_FRESNEL ? 4 : 8), st));
    {
      KernelTimer kt(ctx, "pls_tc_tables", st);
      const dim3 tg((kpad / 2 + 255) / 256, (mpad + npad / 2) / kTabRows);
      pls_tc_tables<<<tg, 256, 0, st>>>(g, pts + c0, cnt, kpad, mpad, ahi, alo, bhi, blo);
      OH_LAUNCH_CHECK();
    }
    CUtensorMap mAhi, mAlo, mBhi, mBlo;
    OH_TRY(make_map(&mAhi, ahi, kpad, mpad, kBM));
    OH_TRY(make_map(&mAlo, alo, kpad, mpad, kBM));
    OH_TRY(make_map(&mBhi, bhi, kpad, npad, kBN));
    OH_TRY(make_map(&mBlo, blo, kpad, npad, kBN));
    const int vec4 = ((reinterpret_cast<uintptr_t>(out) & 15) == 0 && ((2 * g.nx) & 3) == 0) ? 1 : 0;
    TcArgs a{kb_total, splits, g.mode, g.ny, 2 * g.nx, atomic ? 1 : 0, vec4, static_cast<float*>(out), err,
             (ctx->stall_mask & kStallPointSumGemm) ? ctx->dev_err + 1 : nullptr, ctx->stall_cycles};
    KernelTimer kt(ctx, "pls_tc_gemm", st);
    pls_tc_gemm<<<dim3(npad / kBN, mpad / kBM, splits), 128, kSmemBytes, st>>>(mAhi, mAlo, mBhi, mBlo, a);
    OH_LAUNCH_CHECK();
  }
  return OH_OK;
}

}  // namespace oh
