// Host runtime: per-device context with an FFT plan cache and a named
// scratch arena.  Calls on one context are serialised by a mutex, and every
// call orders its stream after the previous call's work through an event, so
// the shared scratch is never used by two streams at once.
#pragma once
#include <cuda_runtime.h>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <utility>
#include <vector>
#include "fft_core.cuh"

struct oh_ctx {
  int device = 0;
  std::mutex mu;
  cudaEvent_t last_done = nullptr;   // recorded at the end of every call
  int* dev_err = nullptr;             // [0]: set by kernels whose bounded waits ran out; [1]: a flag nothing sets
  // error-path test hook (oh_ctx_set_test_stall): kernels in stall_mask wait
  // on dev_err[1] for at most stall_cycles SM clocks before their first stage
  // depth-map layer buffer (row-pass strips of every layer slot): frames
  // whose strips would exceed this run in layer chunks (fast FP32 path)
  size_t dm_layer_limit = (size_t)8 << 30;
  int stall_mask = 0;
  long long stall_cycles = 0;
  std::string dm_setup_key;           // parameters of the depth-map tables now in scratch
  std::string fresnel_key;            // parameters of the Fresnel spectrum in scratch "fr.B"
  bool force_dm_setup = false;        // rebuild the depth-map tables even when cached (graph capture)
  // captured depth-map batches: key -> executable graph and the table key it leaves behind
  struct Graph { cudaGraphExec_t exec = nullptr; std::string dm_key; int launches = 0; };
  std::map<std::string, Graph> graphs;
  // host-buffer frames: key (parameters, host pointers) -> graph of copies and passes
  std::map<std::string, Graph> frame_graphs;
  // persistent depth-map batches: key -> plan (descriptors, tables, graph)
  struct BatchPlanBase { virtual ~BatchPlanBase() = default; };
  std::map<std::string, std::unique_ptr<BatchPlanBase>> batch_plans;
  // persistent batch kernel: 0 off (per-frame launches); tuned settings per
  // (padded length, device) and the file they persist in (empty: none)
  int dm_batch_persistent = 1;
  // col_w 0: the class's default column-block width
  struct BatchTune { int ctas_per_sm = 2, lag = 1, col_w = 0, row_pairs = 1, col_blocks = 1, out_rows = 2; double ms = 0; };
  std::map<std::string, BatchTune> batch_tune;
  std::string tune_file;
  struct Buf { void* p = nullptr; size_t bytes = 0; };
  std::map<std::string, Buf> scratch;
  struct PlanBufs { oh::FFTPlan plan; void* tw = nullptr; int* perm = nullptr; int* iperm = nullptr; };
  std::map<std::pair<int, int>, PlanBufs> plans;   // key (n, precision)
  // optional per-kernel timing: events recorded around each launch on the
  // launching stream while `timing` is set
  bool timing = false;
  struct Mark { const char* name; cudaEvent_t a, b; };
  std::vector<Mark> marks;
  std::vector<cudaEvent_t> event_pool;
  std::map<std::string, std::pair<double, long>> timing_acc;   // name -> (ms, launches)
};

namespace oh {

// Scoped guard: locks the context, makes its device current and orders
// `stream` after the context's previous call.  On destruction records the
// completion event on the stream.
class CallScope {
 public:
  CallScope(oh_ctx* ctx, cudaStream_t stream);
  ~CallScope();
  oh_status status() const { return st_; }
 private:
  oh_ctx* ctx_;
  cudaStream_t stream_;
  int prev_dev_ = -1;
  oh_status st_ = OH_OK;
  std::unique_lock<std::mutex> lk_;
};

// Returns a device buffer of at least `bytes` under `name`, growing it if
// needed (growth synchronises the device before freeing the old buffer).
oh_status scratch(oh_ctx* ctx, const char* name, size_t bytes, void** out);

// Destroys every captured graph (they hold scratch addresses).
void drop_graphs(oh_ctx* ctx);

// Plan for length n in precision prec (0 = fp32, 1 = fp64); built on first
// use.  Fails with OH_ERR_UNSUPPORTED_SIZE when n cannot be factored.
oh_status get_plan(oh_ctx* ctx, int n, int prec, FFTPlan* out);

// Radix schedule for n (empty when unsupported).
bool factorize(int n, int* radix, int* nst);

// Largest dynamic shared memory a block may use on this device.
size_t max_smem_per_block();

// Bracket one kernel launch with timing events when ctx->timing is set.
class KernelTimer {
 public:
  KernelTimer(oh_ctx* ctx, const char* name, cudaStream_t st);
  ~KernelTimer();
 private:
  oh_ctx* ctx_;
  const char* name_;
  cudaStream_t st_;
  cudaEvent_t a_ = nullptr;
};

}  // namespace oh
