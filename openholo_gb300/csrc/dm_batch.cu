// Persistent batch kernel of the depth-map pipeline (the scheduling rules
// are in dm_batch.h).  Replaces the reference's per-frame loop
// (OpenHolo_DepthMap/Hologram/src/HologramGenerator.cpp:261-294: one
// GenerateHologram per frame, each a chain of per-layer launches) by one
// launch for the whole batch.  The pass bodies are the per-frame kernels'
// (dm_kernels.cuh, dm_col_fast.cuh) run with 256 threads, so every frame's
// results equal the per-frame path's bit for bit.
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

}  // namespace oh
