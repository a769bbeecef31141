// Persistent batch kernel of the depth-map pipeline (the scheduling rules
// are in dm_batch.h).  Replaces the reference's per-frame loop
// (OpenHolo_DepthMap/Hologram/src/HologramGenerator.cpp:261-294: one
// GenerateHologram per frame, each a chain of per-layer launches) by one
// launch for the whole batch.  The pass bodies are the per-frame kernels'
// (dm_kernels.cuh, dm_col_fast.cuh) run with 256 threads, so every frame's
// results equal the per-frame path's bit for bit.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <vector>
#include "dm_batch.h"

namespace oh {

namespace {

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Wait until *ctr >= target; false when the launch aborted or the wait ran
// past `limit` SM clocks.
__device__ __forceinline__ bool wait_count(const unsigned* ctr, unsigned target, const unsigned* abort,
                                           long long limit) {
  if (ld_acquire(ctr) >= target) return true;
  const long long t0 = clock64();
  for (;;) {
    __nanosleep(100);
    if (ld_acquire(ctr) >= target) return true;
    if (*(volatile const unsigned*)abort) return false;
    if (clock64() - t0 > limit) return false;
  }
}

template <int C>
__device__ __forceinline__ void run_row(const DMArgs<float>& a, int first, int count) {
  for (int b = first; b < first + count; ++b) {
    if (b > first) __syncthreads();
    dm_row_body<float, kBatchLens[C], kBatchThreads>(a, b);
  }
}
template <int C, int W>
__device__ __forceinline__ void run_col(const DMArgs<float>& a, int first, int count) {
  for (int b = first; b < first + count; ++b) {
    if (b > first) __syncthreads();
    dm_col_body<kBatchLens[C], W, true, true, false, kBatchThreads, true>(a, b);
  }
}
template <int C>
__device__ __forceinline__ void run_out(const DMArgs<float>& a, int first, int count) {
  for (int b = first; b < first + count; ++b) {
    if (b > first) __syncthreads();
    dm_out_body<float, kBatchLens[C]>(a, b);
  }
}
// one item of length class C
template <int C>
__device__ __forceinline__ void run_item(const DMArgs<float>& a, int kind, bool two_col, int first, int count) {
  if (kind == kItemRow) { run_row<C>(a, first, count); return; }
  if (kind == kItemOut) { run_out<C>(a, first, count); return; }
  if constexpr (batch_col_w_ok(C, 2)) {
    if (two_col) { run_col<C, 2>(a, first, count); return; }
  }
  run_col<C, 1>(a, first, count);
}

}  // namespace

__global__ void __launch_bounds__(kBatchThreads, 2) dm_batch_kernel(BatchLaunch L) {
  __shared__ __align__(16) unsigned char s_args[sizeof(DMArgs<float>)];
  __shared__ int4 s_item;
  __shared__ int s_go, s_load;
  const DMArgs<float>& a = *reinterpret_cast<const DMArgs<float>*>(s_args);
  const int tid = threadIdx.x;
  unsigned* const ticket = L.ctl;
  unsigned* const abort = L.ctl + 1;
  unsigned* const done = L.ctl + kBatchCtlHead;
  unsigned next = 0;
  int cur = -1;
  if (tid == 0) {
    if (L.stall_flag && !stall_on_unset_flag(L.stall_flag, L.stall_cycles)) atomicOr(abort, 1u);
    next = atomicAdd(ticket, 1u);
  }
  for (;;) {
    if (tid == 0) {
      int go = 0, load = 0;
      int4 it = make_int4(0, 0, 0, 0);
      if (next < (unsigned)L.n_items && !*(volatile unsigned*)abort) {
        it = L.items[next];
        next = atomicAdd(ticket, 1u);            // the next ticket's latency hides behind this item
        const BatchFrame& F = L.frames[it.x];
        const int kind = it.y & 15;
        bool ok;
        if (kind == kItemRow) {
          ok = F.dep_row < 0 ||
               wait_count(&done[3 * F.dep_row + kItemCol], (unsigned)L.frames[F.dep_row].n_items[kItemCol], abort,
                          L.wait_cycles);
        } else if (kind == kItemCol) {
          ok = wait_count(&done[3 * it.x + kItemRow], (unsigned)F.n_items[kItemRow], abort, L.wait_cycles) &&
               (F.dep_col < 0 || wait_count(&done[3 * F.dep_col + kItemOut],
                                            (unsigned)L.frames[F.dep_col].n_items[kItemOut], abort, L.wait_cycles));
        } else {
          ok = wait_count(&done[3 * it.x + kItemCol], (unsigned)F.n_items[kItemCol], abort, L.wait_cycles);
        }
        if (ok) {
          go = 1;
          load = it.x != cur;
          cur = it.x;
          // the producers' generic-proxy writes before the bulk copies this
          // thread issues (column items read R through cp.async.bulk)
          __threadfence();
          asm volatile("fence.proxy.async.global;" ::: "memory");
        } else {
          atomicOr(abort, 1u);
        }
      }
      s_item = it;
      s_go = go;
      s_load = load;
    }
    __syncthreads();
    if (!s_go) break;
    const int4 it = s_item;
    if (s_load) {
      const int4* src = reinterpret_cast<const int4*>(&L.frames[it.x].a);
      int4* dst = reinterpret_cast<int4*>(s_args);
      for (int i = tid; i < (int)(sizeof(DMArgs<float>) / 16); i += kBatchThreads) dst[i] = src[i];
      __syncthreads();
    }
    const int kind = it.y & 15;
    const bool two_col = (it.y >> 8) & 1;
    switch ((it.y >> 4) & 15) {
      case 0: run_item<0>(a, kind, two_col, it.z, it.w); break;
      case 1: run_item<1>(a, kind, two_col, it.z, it.w); break;
      case 2: run_item<2>(a, kind, two_col, it.z, it.w); break;
      case 3: run_item<3>(a, kind, two_col, it.z, it.w); break;
      case 4: run_item<4>(a, kind, two_col, it.z, it.w); break;
      default: break;
    }
    // shared memory written by generic stores here may be filled by bulk
    // copies in this block's next item
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      __threadfence();
      atomicAdd(&done[3 * it.x + kind], 1u);
    }
  }
  if (tid == 0 && *(volatile unsigned*)abort) atomicOr(L.err, 1);
}

// Tables of every frame: blockIdx.y = frame.
__global__ void __launch_bounds__(256) dm_batch_setup(const BatchFrame* frames, const DMSetup* su) {
  const int f = blockIdx.y;
  dm_setup_body<float>(frames[f].a, su[f], blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x);
}

int dm_batch_occupancy(size_t smem) {
  int nb = 0;
  if (cudaFuncSetAttribute(dm_batch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, dm_batch_kernel, kBatchThreads, smem) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return nb;
}

oh_status dm_batch_launch(const BatchLaunch& L, cudaStream_t st) {
  cudaError_t e = cudaFuncSetAttribute(dm_batch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L.smem);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(dm_batch_kernel, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
  if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(dm_batch_kernel)");
  dm_batch_kernel<<<L.grid, kBatchThreads, L.smem, st>>>(L);
  note_launch();
  if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(e, "dm_batch_kernel launch");
  return OH_OK;
}

oh_status dm_batch_setup_launch(const BatchFrame* frames, const DMSetup* su, int n, cudaStream_t st) {
  dm_batch_setup<<<dim3(32, n), 256, 0, st>>>(frames, su);
  note_launch();
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "dm_batch_setup launch");
  return OH_OK;
}


// ---------------------------------------------------------------------------
// host planner: the batch as one list of items, its tables and control block

namespace {

int batch_class(int len) {
  for (int c = 0; c < kBatchNumLens; ++c)
    if (kBatchLens[c] == len) return c;
  return -1;
}

// Column pass variant the batch kernel carries: the layer-step form with the
// SSB crop of a 2x-padded frame.
bool batch_col_ok(const FrameInfo<float>& fi) {
  const DMArgs<float>& a = fi.a;
  bool ssb = false;
  with_fast_n(a.Py, [&](auto nc) {
    if constexpr (decltype(nc)::value > 0) ssb = a.horner && a.fkeep == col_ssb_keep<decltype(nc)::value>();
  });
  return ssb;
}

struct BatchPlan : oh_ctx::BatchPlanBase {
  bool eligible = true;       // false: some frame is outside the batch kernel (per-frame launches)
  void* dev = nullptr;        // frames, items, set-up constants, tables
  void* ctl = nullptr;        // ticket, abort, counters, per-frame layer flags (cleared per batch)
  size_t ctl_bytes = 0;
  BatchLaunch L{};
  cudaGraphExec_t exec = nullptr;
  ~BatchPlan() override {
    if (exec) cudaGraphExecDestroy(exec);
    if (dev) cudaFree(dev);
    if (ctl) cudaFree(ctl);
  }
};

std::string tune_key(int len) {
  int dev = 0, maj = 0, mnr = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&maj, cudaDevAttrComputeCapabilityMajor, dev);
  cudaDeviceGetAttribute(&mnr, cudaDevAttrComputeCapabilityMinor, dev);
  return "sm_" + std::to_string(maj) + std::to_string(mnr) + ":" + std::to_string(sm_count()) + ":" +
         std::to_string(len);
}

}  // namespace

// Settings for a batch: the tuned entry of the length class with the most
// work (model bytes) sets the launch-wide ones (blocks per SM, lag); item
// sizes come from each frame's own class.
struct BatchSettings {
  int ctas_per_sm = 2, lag = 1;
  oh_ctx::BatchTune per[kBatchNumLens];
};

static int batch_width(const BatchSettings& bs, int cls) {
  const int w = bs.per[cls].col_w;
  return w && batch_col_w_ok(cls, w) ? w : batch_col_w(cls);
}

// Shared memory of a column block of width w for this frame (the layer-step
// form the batch kernel carries).
static size_t batch_col_smem(const DMArgs<float>& a, int w) {
  size_t b = 0;
  with_fast_n(a.Py, [&](auto nc) {
    constexpr int NY = decltype(nc)::value;
    if constexpr (NY > 0)
      b = (size_t)col_layout(col_len<NY>(), a.pny, w, kColStripW, true, a.occ_stride, a.n_entries,
                             col_tab_entries<NY>()).total;
  });
  return b;
}

// Tuned settings for padded length len on the current device, or the
// defaults.
static oh_ctx::BatchTune batch_tune_for(oh_ctx* ctx, int len) {
  auto it = ctx->batch_tune.find(tune_key(len));
  return it == ctx->batch_tune.end() ? oh_ctx::BatchTune{} : it->second;
}

// Builds the plan for `frames` (all eligible), runs the table set-up on st.
static oh_status batch_plan_build(oh_ctx* ctx, const oh_depthmap_frame* frames, int n,
                                  const std::vector<FrameInfo<float>>& fi, const BatchSettings& bs,
                                  cudaStream_t st, std::unique_ptr<BatchPlan>* out) {
  std::unique_ptr<BatchPlan> P(new BatchPlan());
  const int lag = bs.lag;
  const int nring = 2 * lag + 1;
  size_t maxR = 0, maxV = 0, maxO = 0, smem = 0, tables = 0, slots = 0;
  for (int i = 0; i < n; ++i) {
    maxR = std::max(maxR, fi[i].sz.R);
    maxV = std::max(maxV, fi[i].sz.V);
    maxO = std::max(maxO, fi[i].sz.occ);
    const int yc = batch_class(fi[i].a.Py);
    smem = std::max({smem, fi[i].smem_row, batch_col_smem(fi[i].a, batch_width(bs, yc)), fi[i].smem_out});
    tables += (fi[i].sz.tables + 255) & ~(size_t)255;
    slots += (size_t)fi[i].a.n_uslots;
  }
  maxR = (maxR + 255) & ~(size_t)255;
  maxV = (maxV + 255) & ~(size_t)255;
  maxO = (maxO + 255) & ~(size_t)255;
  const int occ = dm_batch_occupancy(smem);
  if (occ < 1) return fail(OH_ERR_UNSUPPORTED_SIZE, "batch kernel: shared memory");
  void *bR, *bV, *bO;
  OH_TRY(scratch(ctx, "dm.bR", maxR * nring, &bR));
  OH_TRY(scratch(ctx, "dm.bV", maxV * nring, &bV));
  OH_TRY(scratch(ctx, "dm.bocc", maxO * nring, &bO));

  // items, pipelined: step s holds the row items of frame s, the column
  // items of frame s - lag and the output items of frame s - 2 lag
  std::vector<BatchFrame> bf(n);
  std::vector<std::vector<int4>> rows(n), cols(n), outs(n);
  for (int i = 0; i < n; ++i) {
    const DMArgs<float>& a = fi[i].a;
    const int xc = batch_class(a.Px), yc = batch_class(a.Py);
    const oh_ctx::BatchTune& tx = bs.per[xc];
    const oh_ctx::BatchTune& ty = bs.per[yc];
    const int npairs = (a.pny + kRowPair - 1) / kRowPair;
    const int wc = batch_width(bs, yc);
    const int ncolb = wc == 1 ? a.Px : a.nstrips;
    for (int b = 0; b < npairs; b += tx.row_pairs)
      rows[i].push_back(make_int4(i, kItemRow | xc << 4, b, std::min(tx.row_pairs, npairs - b)));
    for (int b = 0; b < ncolb; b += ty.col_blocks)
      cols[i].push_back(make_int4(i, kItemCol | yc << 4 | (wc == 2) << 8, b, std::min(ty.col_blocks, ncolb - b)));
    for (int b = 0; b < a.pny; b += tx.out_rows)
      outs[i].push_back(make_int4(i, kItemOut | xc << 4, b, std::min(tx.out_rows, a.pny - b)));
    BatchFrame& F = bf[i];
    std::memset(&F, 0, sizeof(F));
    F.xcls = xc; F.ycls = yc;
    F.n_items[kItemRow] = (int)rows[i].size();
    F.n_items[kItemCol] = (int)cols[i].size();
    F.n_items[kItemOut] = (int)outs[i].size();
    F.dep_row = i >= nring ? i - nring : -1;
    F.dep_col = i >= nring ? i - nring : -1;
  }
  std::vector<int4> items;
  for (int s = 0; s < n + 2 * lag; ++s) {
    if (s < n) items.insert(items.end(), rows[s].begin(), rows[s].end());
    if (s - lag >= 0 && s - lag < n) items.insert(items.end(), cols[s - lag].begin(), cols[s - lag].end());
    if (s - 2 * lag >= 0 && s - 2 * lag < n) items.insert(items.end(), outs[s - 2 * lag].begin(), outs[s - 2 * lag].end());
  }

  // device memory: [frames][set-up constants][items][tables], and the
  // control block [head][3 counters per frame][layer flags of every frame]
  auto up = [](size_t b) { return (b + 255) & ~(size_t)255; };
  const size_t o_fr = 0, o_su = up(o_fr + n * sizeof(BatchFrame)), o_it = up(o_su + n * sizeof(DMSetup)),
               o_tab = up(o_it + items.size() * sizeof(int4)), dev_bytes = o_tab + tables;
  OH_CUDA_TRY(cudaMalloc(&P->dev, dev_bytes));
  const size_t o_any = up((kBatchCtlHead + 3 * (size_t)n) * sizeof(unsigned));
  P->ctl_bytes = o_any + slots * sizeof(int);
  OH_CUDA_TRY(cudaMalloc(&P->ctl, P->ctl_bytes));
  char* dev = static_cast<char*>(P->dev);
  char* ctl = static_cast<char*>(P->ctl);
  std::vector<DMSetup> su(n);
  size_t toff = o_tab, aoff = o_any;
  for (int i = 0; i < n; ++i) {
    DMArgs<float> a = fi[i].a;
    relocate_tables(&a, dev + toff);
    toff += up(fi[i].sz.tables);
    a.slot_any = reinterpret_cast<int*>(ctl + aoff);
    aoff += (size_t)a.n_uslots * sizeof(int);
    a.Rbuf = reinterpret_cast<float2*>(static_cast<char*>(bR) + (i % nring) * maxR);
    a.V = reinterpret_cast<float2*>(static_cast<char*>(bV) + (i % nring) * maxV);
    a.occ = static_cast<uint8_t*>(bO) + (i % nring) * maxO;
    a.err = reinterpret_cast<int*>(ctl + sizeof(unsigned));       // the launch's abort word
    a.stall_flag = nullptr;
    bf[i].a = a;
    su[i] = fi[i].su;
  }
  OH_CUDA_TRY(cudaMemcpy(dev + o_fr, bf.data(), n * sizeof(BatchFrame), cudaMemcpyHostToDevice));
  OH_CUDA_TRY(cudaMemcpy(dev + o_su, su.data(), n * sizeof(DMSetup), cudaMemcpyHostToDevice));
  OH_CUDA_TRY(cudaMemcpy(dev + o_it, items.data(), items.size() * sizeof(int4), cudaMemcpyHostToDevice));
  {
    KernelTimer kt(ctx, "dm_batch_setup", st);
    OH_TRY(dm_batch_setup_launch(reinterpret_cast<const BatchFrame*>(dev + o_fr),
                                 reinterpret_cast<const DMSetup*>(dev + o_su), n, st));
  }
  BatchLaunch& L = P->L;
  L.frames = reinterpret_cast<const BatchFrame*>(dev + o_fr);
  L.items = reinterpret_cast<const int4*>(dev + o_it);
  L.n_items = (int)items.size();
  L.ctl = reinterpret_cast<unsigned*>(ctl);
  L.err = ctx->dev_err;
  L.stall_flag = nullptr;
  L.stall_cycles = 0;
  L.wait_cycles = 2000000000LL;
  L.grid = sm_count() * std::min(occ, std::max(1, bs.ctas_per_sm));
  L.smem = smem;
  *out = std::move(P);
  return OH_OK;
}

// The persistent path of oh_depthmap_generate_batch.  *handled = false when
// some frame is outside what the batch kernel carries (FP32 fast lengths of
// kBatchLens, layer-step column form with the SSB crop, one layer buffer),
// and the caller runs the per-frame launches instead.
// Plans every frame; *ok = false when some frame is outside the batch kernel.
static oh_status batch_frame_infos(oh_ctx* ctx, const oh_depthmap_frame* frames, int n, cudaStream_t st,
                                   std::vector<FrameInfo<float>>* fi, bool* ok) {
  fi->assign(n, FrameInfo<float>());
  *ok = true;
  for (int i = 0; i < n; ++i) {
    const oh_depthmap_frame& f = frames[i];
    OH_TRY(depthmap_frame_info(ctx, f, st, &(*fi)[i]));
    const FrameInfo<float>& x = (*fi)[i];
    if (batch_class(x.a.Px) < 0 || batch_class(x.a.Py) < 0 || !x.Wfast || !x.a.xs || x.nchunks != 1 ||
        !batch_col_ok(x))
      *ok = false;
  }
  return OH_OK;
}

// Settings of a batch: each class's tuned entry; the launch-wide ones from
// the class with the most work.
static BatchSettings batch_settings(oh_ctx* ctx, const std::vector<FrameInfo<float>>& fi) {
  BatchSettings bs;
  double best = -1.0;
  for (int c = 0; c < kBatchNumLens; ++c) bs.per[c] = batch_tune_for(ctx, kBatchLens[c]);
  std::vector<double> work(kBatchNumLens, 0.0);
  for (const FrameInfo<float>& x : fi)
    work[batch_class(std::max(x.a.Px, x.a.Py))] += (double)x.a.Px * x.a.Py * (x.a.n_entries + 1);
  for (int c = 0; c < kBatchNumLens; ++c)
    if (work[c] > best) { best = work[c]; bs.ctas_per_sm = bs.per[c].ctas_per_sm; bs.lag = bs.per[c].lag; }
  return bs;
}

oh_status batch_persistent(oh_ctx* ctx, const oh_depthmap_frame* frames, int n, unsigned flags,
                                  const std::string& key, cudaStream_t st, bool* handled) {
  *handled = false;
  auto it = ctx->batch_plans.find(key);
  BatchPlan* P = it == ctx->batch_plans.end() ? nullptr : static_cast<BatchPlan*>(it->second.get());
  const bool stall = (ctx->stall_mask & kStallDepthmapBatch) != 0;
  if (P && !P->eligible) return OH_OK;
  if (!P) {
    std::vector<FrameInfo<float>> fi;
    bool ok = false;
    OH_TRY(batch_frame_infos(ctx, frames, n, st, &fi, &ok));
    if (!ok) {
      if (ctx->batch_plans.size() >= 16) ctx->batch_plans.clear();
      std::unique_ptr<BatchPlan> no(new BatchPlan());
      no->eligible = false;
      ctx->batch_plans[key] = std::move(no);
      return OH_OK;
    }
    const BatchSettings bs = batch_settings(ctx, fi);
    std::unique_ptr<BatchPlan> np;
    OH_TRY(batch_plan_build(ctx, frames, n, fi, bs, st, &np));
    if (ctx->batch_plans.size() >= 16) ctx->batch_plans.clear();
    P = np.get();
    ctx->batch_plans[key] = std::move(np);
  }
  *handled = true;
  bool graph = (flags & OH_BATCH_GRAPH) && st != nullptr && !stall;
  if (graph && !P->exec) {
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed);
    oh_status rs = OH_OK;
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamBeginCapture");
    e = cudaMemsetAsync(P->ctl, 0, P->ctl_bytes, st);
    if (e != cudaSuccess) rs = cuda_fail(e, "cudaMemsetAsync (batch control)");
    else rs = dm_batch_launch(P->L, st);
    e = cudaStreamEndCapture(st, &g);
    if (rs == OH_OK && e != cudaSuccess) rs = cuda_fail(e, "cudaStreamEndCapture");
    if (rs == OH_OK) {
      e = cudaGraphInstantiate(&P->exec, g, 0);
      if (e != cudaSuccess) { P->exec = nullptr; rs = cuda_fail(e, "cudaGraphInstantiate"); }
    }
    if (g) cudaGraphDestroy(g);
    OH_TRY(rs);
  }
  if (graph) {
    OH_CUDA_TRY(cudaGraphLaunch(P->exec, st));
    note_launch(1);
    return OH_OK;
  }
  OH_CUDA_TRY(cudaMemsetAsync(P->ctl, 0, P->ctl_bytes, st));
  BatchLaunch L = P->L;
  if (stall) { L.stall_flag = ctx->dev_err + 1; L.stall_cycles = ctx->stall_cycles; }
  KernelTimer kt(ctx, "dm_batch", st);
  return dm_batch_launch(L, st);
}

// ---- autotuner: per padded length and device, the batch kernel's blocks
// per SM, pipeline lag, column-block width and item sizes, chosen by timing
// the frames of that length (coordinate descent from the current entry;
// a change must gain 1 %).  Entries persist in the context's tune file.

static oh_status batch_trial(oh_ctx* ctx, const oh_depthmap_frame* frames, const std::vector<FrameInfo<float>>& fi,
                             const BatchSettings& bs, int reps, cudaStream_t st, double* ms) {
  std::unique_ptr<BatchPlan> P;
  OH_TRY(batch_plan_build(ctx, frames, (int)fi.size(), fi, bs, st, &P));
  auto run = [&]() -> oh_status {
    OH_CUDA_TRY(cudaMemsetAsync(P->ctl, 0, P->ctl_bytes, st));
    return dm_batch_launch(P->L, st);
  };
  OH_TRY(run());
  cudaEvent_t a = nullptr, b = nullptr;
  OH_CUDA_TRY(cudaEventCreate(&a));
  OH_CUDA_TRY(cudaEventCreate(&b));
  oh_status rs = OH_OK;
  cudaEventRecord(a, st);
  for (int r = 0; r < reps && rs == OH_OK; ++r) rs = run();
  cudaEventRecord(b, st);
  cudaError_t e = cudaEventSynchronize(b);
  float t = 0.f;
  if (rs == OH_OK && e == cudaSuccess) e = cudaEventElapsedTime(&t, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  OH_TRY(rs);
  if (e != cudaSuccess) return cuda_fail(e, "autotune timing");
  unsigned abort_word = 0;
  OH_CUDA_TRY(cudaMemcpy(&abort_word, static_cast<unsigned*>(P->ctl) + 1, sizeof(unsigned), cudaMemcpyDeviceToHost));
  if (abort_word) return fail(OH_ERR_TIMEOUT, "batch kernel wait ran out while tuning");
  *ms = (double)t / reps;
  return OH_OK;
}

static oh_status tune_save(oh_ctx* ctx) {
  if (ctx->tune_file.empty()) return OH_OK;
  FILE* f = std::fopen(ctx->tune_file.c_str(), "w");
  if (!f) return fail(OH_ERR_IO, "cannot write tune file " + ctx->tune_file);
  std::fprintf(f, "# depth-map batch kernel settings: key ctas_per_sm lag col_w row_pairs col_blocks out_rows ms\n");
  for (const auto& kv : ctx->batch_tune) {
    const oh_ctx::BatchTune& t = kv.second;
    std::fprintf(f, "%s %d %d %d %d %d %d %.6f\n", kv.first.c_str(), t.ctas_per_sm, t.lag, t.col_w, t.row_pairs,
                 t.col_blocks, t.out_rows, t.ms);
  }
  std::fclose(f);
  return OH_OK;
}

static oh_status batch_autotune(oh_ctx* ctx, const oh_depthmap_frame* frames, int n, int reps, cudaStream_t st) {
  std::vector<FrameInfo<float>> fi;
  bool ok = false;
  OH_TRY(batch_frame_infos(ctx, frames, n, st, &fi, &ok));
  if (!ok) return fail(OH_ERR_UNSUPPORTED_SIZE, "autotune: a frame is outside what the batch kernel carries");
  for (int c = 0; c < kBatchNumLens; ++c) {
    // the square frames of this length
    std::vector<oh_depthmap_frame> sub;
    std::vector<FrameInfo<float>> sfi;
    for (int i = 0; i < n; ++i)
      if (fi[i].a.Px == kBatchLens[c] && fi[i].a.Py == kBatchLens[c]) { sub.push_back(frames[i]); sfi.push_back(fi[i]); }
    if (sub.empty()) continue;
    oh_ctx::BatchTune cur = batch_tune_for(ctx, kBatchLens[c]);
    auto settings = [&](const oh_ctx::BatchTune& t) {
      BatchSettings bs;
      for (int k = 0; k < kBatchNumLens; ++k) bs.per[k] = batch_tune_for(ctx, kBatchLens[k]);
      bs.per[c] = t;
      bs.ctas_per_sm = t.ctas_per_sm;
      bs.lag = t.lag;
      return bs;
    };
    double best = 0.0;
    OH_TRY(batch_trial(ctx, sub.data(), sfi, settings(cur), reps, st, &best));
    const int def_w = batch_col_w(c);
    struct Knob { int oh_ctx::BatchTune::*field; std::vector<int> vals; };
    const Knob knobs[] = {{&oh_ctx::BatchTune::ctas_per_sm, {1, 2}}, {&oh_ctx::BatchTune::lag, {0, 1}},
                          {&oh_ctx::BatchTune::col_w, {def_w, 3 - def_w}}, {&oh_ctx::BatchTune::row_pairs, {1, 2, 4}},
                          {&oh_ctx::BatchTune::col_blocks, {1, 2}}, {&oh_ctx::BatchTune::out_rows, {1, 2, 4, 8}}};
    for (const Knob& kn : knobs) {
      for (int v : kn.vals) {
        oh_ctx::BatchTune t = cur;
        const int now = cur.*(kn.field) ? cur.*(kn.field) : def_w;
        if (v == now) continue;
        if (kn.field == &oh_ctx::BatchTune::col_w && !batch_col_w_ok(c, v)) continue;
        t.*(kn.field) = v;
        double ms = 0.0;
        oh_status rs = batch_trial(ctx, sub.data(), sfi, settings(t), reps, st, &ms);
        if (rs == OH_ERR_UNSUPPORTED_SIZE) continue;        // e.g. a width whose shared memory does not fit
        OH_TRY(rs);
        if (ms < best * 0.99) { best = ms; cur = t; }
      }
    }
    cur.ms = best;
    ctx->batch_tune[tune_key(kBatchLens[c])] = cur;
  }
  OH_CUDA_TRY(cudaStreamSynchronize(st));
  ctx->batch_plans.clear();             // later batches plan with the new settings
  return tune_save(ctx);
}


}  // namespace oh

using namespace oh;

extern "C" {

oh_status oh_depthmap_autotune_batch(oh_ctx* ctx, const oh_depthmap_frame* frames, int n, int reps, void* stream) {
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  CallScope cs(ctx, st);
  OH_TRY(cs.status());
  if (n < 1 || !frames) return fail(OH_ERR_INVALID_ARG, "autotune: empty frame array");
  if (reps < 1 || reps > 100) return fail(OH_ERR_INVALID_ARG, "autotune: reps must be 1..100");
  for (int i = 0; i < n; ++i) {
    OH_TRY(depthmap_validate(&frames[i].params));
    if (!frames[i].img || !frames[i].depth || !frames[i].fringe)
      return fail(OH_ERR_INVALID_ARG, "frame " + std::to_string(i) + ": img, depth and fringe are required");
    if (frames[i].params.phase_mode == OH_PHASE_ARRAY && !frames[i].phase)
      return fail(OH_ERR_INVALID_ARG, "frame " + std::to_string(i) + ": OH_PHASE_ARRAY needs a phase array");
  }
  if (st) {
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    OH_CUDA_TRY(cudaStreamIsCapturing(st, &cap));
    if (cap != cudaStreamCaptureStatusNone) return fail(OH_ERR_INVALID_ARG, "autotune: stream is capturing");
  }
  return batch_autotune(ctx, frames, n, reps, st);
}

oh_status oh_depthmap_batch_tuning(oh_ctx* ctx, int padded_len, int settings[6], double* ms) {
  if (!ctx || !settings) return fail(OH_ERR_INVALID_ARG, "null argument");
  std::lock_guard<std::mutex> lk(ctx->mu);
  int prev = 0;
  cudaGetDevice(&prev);
  cudaSetDevice(ctx->device);
  const oh_ctx::BatchTune t = batch_tune_for(ctx, padded_len);
  cudaSetDevice(prev);
  const int cls = batch_class(padded_len);
  settings[0] = t.ctas_per_sm; settings[1] = t.lag; settings[2] = t.col_w ? t.col_w : (cls >= 0 ? batch_col_w(cls) : 0);
  settings[3] = t.row_pairs; settings[4] = t.col_blocks; settings[5] = t.out_rows;
  if (ms) *ms = t.ms;
  return OH_OK;
}

oh_status oh_ctx_set_autotune_file(oh_ctx* ctx, const char* path) {
  if (!ctx) return fail(OH_ERR_INVALID_ARG, "null context");
  std::lock_guard<std::mutex> lk(ctx->mu);
  ctx->tune_file = path ? path : "";
  if (ctx->tune_file.empty()) return OH_OK;
  FILE* f = std::fopen(ctx->tune_file.c_str(), "r");
  if (!f) return OH_OK;                  // written by the first autotune
  char line[512];
  while (std::fgets(line, sizeof(line), f)) {
    if (line[0] == '#') continue;
    char key[256];
    oh_ctx::BatchTune t;
    if (std::sscanf(line, "%255s %d %d %d %d %d %d %lf", key, &t.ctas_per_sm, &t.lag, &t.col_w, &t.row_pairs,
                    &t.col_blocks, &t.out_rows, &t.ms) != 8 ||
        t.ctas_per_sm < 1 || t.ctas_per_sm > 2 || t.lag < 0 || t.lag > 1 || t.col_w < 0 || t.col_w > 2 ||
        t.row_pairs < 1 || t.row_pairs > 64 || t.col_blocks < 1 || t.col_blocks > 64 || t.out_rows < 1 ||
        t.out_rows > 64) {
      std::fclose(f);
      return fail(OH_ERR_IO, "malformed tune file line: " + std::string(line));
    }
    ctx->batch_tune[key] = t;
  }
  std::fclose(f);
  int prev = 0;
  cudaGetDevice(&prev);
  cudaSetDevice(ctx->device);
  cudaDeviceSynchronize();               // plans built with the old settings may still run
  ctx->batch_plans.clear();
  cudaSetDevice(prev);
  return OH_OK;
}

}  // extern "C"
