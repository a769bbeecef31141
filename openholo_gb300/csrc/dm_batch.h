// Persistent batch kernel of the depth-map pipeline: declarations shared by
// the per-frame pipeline (depthmap.cu) and the batch kernel with its host
// planner and autotuner (dm_batch.cu).
//
// A batch of frames becomes one list of work items, each a range of blocks
// of one pass of one frame (row pairs, column strips or output rows).  One
// launch of dm_batch_kernel, one or two blocks per SM, takes items from the
// list in order through a global ticket counter.  Before an item's body runs
// its block waits, bounded, until the items it reads from have finished
// (per-frame completion counters):
//   column items of frame f: every row item of f, and every output item of
//     the frame that last used f's V ring slot;
//   output items of f: every column item of f;
//   row items of f: every column item of the frame that last used f's R and
//     occupancy ring slot.
// An item's block only waits on items taken before its own, and a block
// that has taken an item is resident, so the oldest unfinished item always
// progresses.  A wait that runs out (about a second of SM clock, or the
// error-path test hook) sets the launch's abort word and the context's
// error word; every block then stops at its next item.
#pragma once
#include <string>
#include <type_traits>
#include "dm_kernels.cuh"

namespace oh {

// Scratch bytes one frame needs: R strips, V rows, occupancy flags, tables.
struct DMScratch { size_t R, V, occ, tables, acc; };

// Everything run_depthmap decides for one frame before it allocates: the
// scratch sizes, the kernel arguments (their table pointers hold offsets
// into the frame's table region, see relocate_tables), the per-frame set-up
// constants, and the pass configuration.
template <typename R> struct FrameInfo {
  DMScratch sz;
  DMArgs<R> a;
  DMSetup su;
  int Wfast = 0, wcol = 0, nchunks = 1;
  size_t smem_row = 0, smem_col = 0, smem_out = 0;
};

// Adds the base of a table region to the offsets FrameInfo::a holds.
template <typename R> void relocate_tables(DMArgs<R>* a, char* base) {
  auto rel = [&](auto*& p) { p = reinterpret_cast<std::remove_reference_t<decltype(p)>>(base + reinterpret_cast<size_t>(p)); };
  rel(a->lut); rel(a->uslot_of_entry); rel(a->kzp); rel(a->cst); rel(a->exc); rel(a->ey); rel(a->eth);
  rel(a->lfx); rel(a->lfy); rel(a->lfyp); rel(a->shy); rel(a->shx); rel(a->slot_any);
  if (a->dxh) rel(a->dxh);
  if (a->dyh) rel(a->dyh);
}

// The planning half of run_depthmap (depthmap.cu) for one FP32 frame: fills
// info without allocating or launching anything.
oh_status depthmap_frame_info(oh_ctx* ctx, const oh_depthmap_frame& f, cudaStream_t st, FrameInfo<float>* info);
oh_status depthmap_validate(const oh_depthmap_params* p);
// The persistent path of oh_depthmap_generate_batch (dm_batch.cu): *handled
// = false when some frame is outside what the batch kernel carries.
oh_status batch_persistent(oh_ctx* ctx, const oh_depthmap_frame* frames, int n, unsigned flags,
                           const std::string& key, cudaStream_t st, bool* handled);

// Padded lengths (Px and Py) the batch kernel carries, as length classes.
constexpr int kBatchLens[] = {1024, 1536, 2048, 3072, 4096};
constexpr int kBatchNumLens = 5;
constexpr int kBatchThreads = 256;
// Default columns per column block for each class: one-column blocks over
// the two-column strips at 3072 and 4096 (as the per-frame pass picks
// there), whole strips below.  The autotuner may pick the other width.
__host__ __device__ constexpr int batch_col_w(int cls) { return cls >= 3 ? 1 : 2; }
// Widths the kernel carries: both below 3072; one column at 3072 and 4096,
// where a two-column block would need 136-178 KB of shared memory (one block
// per SM) and spill its accumulators at 256 threads.
__host__ __device__ constexpr bool batch_col_w_ok(int cls, int w) { return w == 1 || (w == 2 && cls < 3); }

enum : int { kItemRow = 0, kItemCol = 1, kItemOut = 2 };

// 16-byte aligned: the kernel copies `a` into shared memory as int4 words.
struct alignas(16) BatchFrame {
  DMArgs<float> a;
  int xcls, ycls;          // classes of Px and Py
  int n_items[3];          // row, column and output items
  int dep_row;             // frame whose column items free this frame's R/occ slot (-1: none)
  int dep_col;             // frame whose output items free this frame's V slot (-1: none)
};
static_assert(sizeof(DMArgs<float>) % 16 == 0, "frame arguments are copied as int4 words");
static_assert(sizeof(BatchFrame) % 16 == 0, "frame records keep 16-byte alignment");

// Item: x = frame, y = kind | class << 4 | (column blocks of two columns) << 8,
// z = first block, w = blocks.
struct BatchLaunch {
  const BatchFrame* frames;
  const int4* items;
  int n_items;
  unsigned* ctl;           // [0] ticket, [1] abort, [2..3] unused, then 3 counters per frame
  int* err;                // context error word
  const int* stall_flag;   // error-path test hook: a flag nothing sets (or null)
  long long stall_cycles;
  long long wait_cycles;   // bound of a dependency wait
  int grid;
  size_t smem;
};

constexpr int kBatchCtlHead = 4;

oh_status dm_batch_launch(const BatchLaunch& L, cudaStream_t st);
oh_status dm_batch_setup_launch(const BatchFrame* frames, const DMSetup* su, int n, cudaStream_t st);
// Resident blocks per SM of the batch kernel with `smem` bytes of dynamic
// shared memory (0 when it does not fit).
int dm_batch_occupancy(size_t smem);

}  // namespace oh
