// Context, scratch arena, FFT plan cache and error plumbing.
#include "context.h"
#include "fft_fast.cuh"

#include <atomic>
#include <cmath>
#include <cstring>
#include <vector>

namespace oh {

static std::atomic<uint64_t> g_launches{0};
static thread_local std::string t_last_error;

void note_launch(int n) { g_launches.fetch_add((uint64_t)n, std::memory_order_relaxed); }
uint64_t launches_so_far() { return g_launches.load(std::memory_order_relaxed); }
void set_error(const std::string& msg) { t_last_error = msg; }

int sm_count() {
  static std::atomic<int> cached[64];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) return 152;
  if (dev < 64) {
    const int c = cached[dev].load(std::memory_order_relaxed);
    if (c > 0) return c;
  }
  int n = 0;
  if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) {
    cudaGetLastError();
    n = 152;
  }
  if (dev < 64) cached[dev].store(n, std::memory_order_relaxed);
  return n;
}
oh_status fail(oh_status s, const std::string& msg) { t_last_error = msg; return s; }
oh_status cuda_fail(cudaError_t e, const char* what) {
  t_last_error = std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
  return OH_ERR_CUDA;
}

CallScope::CallScope(oh_ctx* ctx, cudaStream_t stream) : ctx_(ctx), stream_(stream) {
  if (!ctx) { st_ = fail(OH_ERR_INVALID_ARG, "null context"); return; }
  lk_ = std::unique_lock<std::mutex>(ctx->mu);
  t_last_error.clear();
  cudaGetDevice(&prev_dev_);
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e != cudaSuccess) { st_ = cuda_fail(e, "cudaSetDevice"); return; }
  e = cudaStreamWaitEvent(stream, ctx->last_done, 0);
  if (e != cudaSuccess) { st_ = cuda_fail(e, "cudaStreamWaitEvent"); return; }
}

CallScope::~CallScope() {
  if (ctx_ && st_ == OH_OK) cudaEventRecord(ctx_->last_done, stream_);
  if (prev_dev_ >= 0 && ctx_ && prev_dev_ != ctx_->device) cudaSetDevice(prev_dev_);
}

void drop_graphs(oh_ctx* ctx) {
  for (auto& kv : ctx->graphs)
    if (kv.second.exec) cudaGraphExecDestroy(kv.second.exec);
  ctx->graphs.clear();
  for (auto& kv : ctx->frame_graphs)
    if (kv.second.exec) cudaGraphExecDestroy(kv.second.exec);
  ctx->frame_graphs.clear();
  ctx->batch_plans.clear();
}

oh_status scratch(oh_ctx* ctx, const char* name, size_t bytes, void** out) {
  auto& b = ctx->scratch[name];
  if (b.bytes < bytes) {
    // captured depth-map graphs address the buffer being replaced
    // (and the host-buffer frame graphs address "host.io")
    if (b.p && (std::string(name).compare(0, 3, "dm.") == 0 || std::string(name) == "host.io")) drop_graphs(ctx);
    // the cached tables of a buffer being replaced are gone
    const std::string nm(name);
    if (nm == "dm.tables") ctx->dm_setup_key.clear();
    if (nm == "fr.B" || nm == "fr.tab") ctx->fresnel_key.clear();
    if (b.p) {
      cudaError_t e = cudaDeviceSynchronize();
      if (e != cudaSuccess) return cuda_fail(e, "cudaDeviceSynchronize (scratch growth)");
      cudaFree(b.p);
      b.p = nullptr; b.bytes = 0;
    }
    size_t sz = (bytes + 255) & ~(size_t)255;
    cudaError_t e = cudaMalloc(&b.p, sz);
    if (e != cudaSuccess) { b.p = nullptr; cudaGetLastError(); return fail(OH_ERR_ALLOC, std::string("scratch '") + name + "' of " + std::to_string(sz) + " bytes: " + cudaGetErrorString(e)); }
    b.bytes = sz;
  }
  *out = b.p;
  return OH_OK;
}

bool factorize(int n, int* radix, int* nst) {
  if (n < 1) return false;
  // lengths with a compile-time schedule use exactly that schedule
#define OH_SCHED_CASE(len, ...)                                   \
  if (n == len) {                                                  \
    const int rs[] = {__VA_ARGS__};                                \
    *nst = (int)(sizeof(rs) / sizeof(rs[0]));                      \
    for (int s = 0; s < *nst; ++s) radix[s] = rs[s];               \
    return true;                                                   \
  }
  OH_FAST_SCHEDULES(OH_SCHED_CASE)
#undef OH_SCHED_CASE
  int m = n, s = 0;
  int twos = 0;
  while (m % 2 == 0) { m /= 2; ++twos; }
  while (twos >= 3) { radix[s++] = 8; twos -= 3; }
  if (twos == 2) radix[s++] = 4;
  if (twos == 1) radix[s++] = 2;
  while (m % 5 == 0) { radix[s++] = 5; m /= 5; }
  while (m % 3 == 0) { radix[s++] = 3; m /= 3; }
  for (int p = 7; m > 1; p += 2) {
    if (p > kMaxGenericRadix) return false;
    while (m % p == 0) { radix[s++] = p; m /= p; }
    if (s > kMaxStages - 1) return false;
  }
  if (s == 0) radix[s++] = 1;   // n == 1: identity
  *nst = s;
  return true;
}

static void build_perm(int n, const int* radix, int nst, std::vector<int>& perm) {
  perm.assign(n, 0);
  // q_s = n / (r_0...r_s); X[k], k = f0 + r0 f1 + r0 r1 f2 + ..., sits at sum f_s q_s
  for (int k = 0; k < n; ++k) {
    int rem = k, pos = 0, prod = 1;
    for (int s = 0; s < nst; ++s) {
      int r = radix[s];
      prod *= r;
      int f = rem % r; rem /= r;
      pos += f * (n / prod);
    }
    perm[k] = pos;
  }
}

oh_status get_plan(oh_ctx* ctx, int n, int prec, FFTPlan* out) {
  auto key = std::make_pair(n, prec);
  auto it = ctx->plans.find(key);
  if (it != ctx->plans.end()) { *out = it->second.plan; return OH_OK; }
  oh_ctx::PlanBufs pb;
  FFTPlan& pl = pb.plan;
  std::memset(&pl, 0, sizeof(pl));
  pl.n = n;
  if (!factorize(n, pl.radix, &pl.nst))
    return fail(OH_ERR_UNSUPPORTED_SIZE, "FFT length " + std::to_string(n) + " has a prime factor above " + std::to_string(kMaxGenericRadix));
  if (pl.radix[0] == 1) pl.nst = 0;
  int m = n;
  for (int s = 0; s < pl.nst; ++s) {
    pl.q[s] = m / pl.radix[s];
    pl.tws[s] = n / m;
    m = pl.q[s];
  }
  std::vector<int> perm, iperm(n);
  if (pl.nst == 0) { perm.assign(n, 0); } else build_perm(n, pl.radix, pl.nst, perm);
  for (int k = 0; k < n; ++k) iperm[perm[k]] = k;
  // twiddles W_n^e = exp(-2 pi i e / n), evaluated in double with the angle
  // reduced to [0, pi/4] by symmetry so that both precisions get correctly
  // rounded-quality values.
  std::vector<double> c(n), sn(n);
  for (int e = 0; e < n; ++e) {
    // angle = 2 pi e / n; use integer arithmetic to fold into an octant
    long long num = 8LL * e;            // angle / (pi/4) = 8 e / n
    long long oct = num / n;            // 0..7
    long long rem = num - oct * n;      // angle within octant, in units of (pi/4)/n
    double a = (M_PI / 4.0) * (double)rem / (double)n;
    double ca = std::cos(a), sa = std::sin(a);
    double cb = std::cos(M_PI / 4.0 - a), sb = std::sin(M_PI / 4.0 - a);
    double cs, ss;
    switch (oct) {            // angle = oct*pi/4 + a
      case 0: cs = ca;  ss = sa;  break;
      case 1: cs = sb;  ss = cb;  break;   // pi/4 + a = pi/2 - (pi/4 - a)
      case 2: cs = -sa; ss = ca;  break;   // pi/2 + a
      case 3: cs = -cb; ss = sb;  break;   // pi - (pi/4 - a)
      case 4: cs = -ca; ss = -sa; break;   // pi + a
      case 5: cs = -sb; ss = -cb; break;   // 3pi/2 - (pi/4 - a)
      case 6: cs = sa;  ss = -ca; break;   // 3pi/2 + a
      default: cs = cb; ss = -sb; break;   // 2pi - (pi/4 - a)
    }
    c[e] = cs; sn[e] = -ss;   // forward twiddle exp(-i angle)
  }
  size_t esz = prec ? sizeof(double2) : sizeof(float2);
  cudaError_t e1 = cudaMalloc(&pb.tw, esz * n);
  cudaError_t e2 = cudaMalloc((void**)&pb.perm, sizeof(int) * n);
  cudaError_t e3 = cudaMalloc((void**)&pb.iperm, sizeof(int) * n);
  if (e1 != cudaSuccess || e2 != cudaSuccess || e3 != cudaSuccess) {
    cudaFree(pb.tw); cudaFree(pb.perm); cudaFree(pb.iperm); cudaGetLastError();
    return fail(OH_ERR_ALLOC, "FFT plan tables");
  }
  if (prec) {
    std::vector<double2> t(n);
    for (int e = 0; e < n; ++e) t[e] = make_double2(c[e], sn[e]);
    OH_CUDA_TRY(cudaMemcpy(pb.tw, t.data(), esz * n, cudaMemcpyHostToDevice));
  } else {
    std::vector<float2> t(n);
    for (int e = 0; e < n; ++e) t[e] = make_float2((float)c[e], (float)sn[e]);
    OH_CUDA_TRY(cudaMemcpy(pb.tw, t.data(), esz * n, cudaMemcpyHostToDevice));
  }
  OH_CUDA_TRY(cudaMemcpy(pb.perm, perm.data(), sizeof(int) * n, cudaMemcpyHostToDevice));
  OH_CUDA_TRY(cudaMemcpy(pb.iperm, iperm.data(), sizeof(int) * n, cudaMemcpyHostToDevice));
  pl.tw = pb.tw; pl.perm = pb.perm; pl.iperm = pb.iperm;
  ctx->plans[key] = pb;
  *out = pl;
  return OH_OK;
}

static cudaEvent_t pool_get(oh_ctx* ctx) {
  if (!ctx->event_pool.empty()) { cudaEvent_t e = ctx->event_pool.back(); ctx->event_pool.pop_back(); return e; }
  cudaEvent_t e = nullptr;
  if (cudaEventCreate(&e) != cudaSuccess) { cudaGetLastError(); return nullptr; }
  return e;
}

KernelTimer::KernelTimer(oh_ctx* ctx, const char* name, cudaStream_t st) : ctx_(ctx), name_(name), st_(st) {
  if (!ctx_ || !ctx_->timing) return;
  a_ = pool_get(ctx_);
  if (a_) cudaEventRecord(a_, st_);
}

KernelTimer::~KernelTimer() {
  if (!a_) return;
  cudaEvent_t b = pool_get(ctx_);
  if (!b) { ctx_->event_pool.push_back(a_); return; }
  cudaEventRecord(b, st_);
  ctx_->marks.push_back({name_, a_, b});
}

size_t max_smem_per_block() {
  int dev = 0, v = 0;
  cudaGetDevice(&dev);
  if (cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) { cudaGetLastError(); return 48 * 1024; }
  return (size_t)v;
}

}  // namespace oh

using namespace oh;

extern "C" {

oh_status oh_ctx_create(oh_ctx** ctx, int device) {
  if (!ctx) return fail(OH_ERR_INVALID_ARG, "ctx out pointer is null");
  *ctx = nullptr;
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDeviceCount");
  if (device < 0 || device >= ndev) return fail(OH_ERR_INVALID_ARG, "device index out of range");
  int prev = 0;
  cudaGetDevice(&prev);
  e = cudaSetDevice(device);
  if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
  oh_ctx* c = new oh_ctx();
  c->device = device;
  e = cudaEventCreateWithFlags(&c->last_done, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaMalloc(&c->dev_err, 2 * sizeof(int));
  if (e == cudaSuccess) e = cudaMemset(c->dev_err, 0, 2 * sizeof(int));
  cudaSetDevice(prev);
  if (e != cudaSuccess) { delete c; return cuda_fail(e, "context set-up"); }
  *ctx = c;
  return OH_OK;
}

oh_status oh_ctx_destroy(oh_ctx* ctx) {
  if (!ctx) return OH_OK;
  int prev = 0;
  cudaGetDevice(&prev);
  cudaSetDevice(ctx->device);
  cudaDeviceSynchronize();
  drop_graphs(ctx);
  for (auto& kv : ctx->scratch) cudaFree(kv.second.p);
  for (auto& kv : ctx->plans) { cudaFree(kv.second.tw); cudaFree(kv.second.perm); cudaFree(kv.second.iperm); }
  for (auto& m : ctx->marks) { cudaEventDestroy(m.a); cudaEventDestroy(m.b); }
  for (auto e : ctx->event_pool) cudaEventDestroy(e);
  cudaEventDestroy(ctx->last_done);
  cudaFree(ctx->dev_err);
  cudaSetDevice(prev);
  delete ctx;
  return OH_OK;
}

size_t oh_ctx_scratch_bytes(const oh_ctx* ctx) {
  if (!ctx) return 0;
  size_t s = 0;
  for (auto& kv : ctx->scratch) s += kv.second.bytes;
  return s;
}

oh_status oh_ctx_release_scratch(oh_ctx* ctx) {
  if (!ctx) return fail(OH_ERR_INVALID_ARG, "null context");
  std::lock_guard<std::mutex> lk(ctx->mu);
  int prev = 0;
  cudaGetDevice(&prev);
  cudaSetDevice(ctx->device);
  cudaDeviceSynchronize();
  drop_graphs(ctx);
  for (auto& kv : ctx->scratch) cudaFree(kv.second.p);
  ctx->scratch.clear();
  ctx->dm_setup_key.clear();
  ctx->fresnel_key.clear();
  cudaSetDevice(prev);
  return OH_OK;
}

const char* oh_status_string(oh_status s) {
  switch (s) {
    case OH_OK: return "OH_OK";
    case OH_ERR_INVALID_ARG: return "OH_ERR_INVALID_ARG";
    case OH_ERR_UNSUPPORTED_SIZE: return "OH_ERR_UNSUPPORTED_SIZE";
    case OH_ERR_CUDA: return "OH_ERR_CUDA";
    case OH_ERR_ALLOC: return "OH_ERR_ALLOC";
    case OH_ERR_TIMEOUT: return "OH_ERR_TIMEOUT";
    case OH_ERR_IO: return "OH_ERR_IO";
  }
  return "OH_ERR_UNKNOWN";
}

const char* oh_last_error(void) { return t_last_error.c_str(); }

oh_status oh_ctx_device_status(oh_ctx* ctx, void* stream) {
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  CallScope cs(ctx, st);
  OH_TRY(cs.status());
  int h = 0;
  OH_CUDA_TRY(cudaMemcpyAsync(&h, ctx->dev_err, sizeof(int), cudaMemcpyDeviceToHost, st));
  OH_CUDA_TRY(cudaStreamSynchronize(st));
  if (h) {
    OH_CUDA_TRY(cudaMemsetAsync(ctx->dev_err, 0, sizeof(int), st));
    return fail(OH_ERR_TIMEOUT, "a bounded device-side wait ran out (copy into shared memory did not complete)");
  }
  return OH_OK;
}

oh_status oh_ctx_set_depthmap_layer_limit(oh_ctx* ctx, size_t bytes) {
  if (!ctx) return fail(OH_ERR_INVALID_ARG, "null context");
  std::lock_guard<std::mutex> lk(ctx->mu);
  ctx->dm_layer_limit = bytes ? bytes : (size_t)8 << 30;
  return OH_OK;
}

oh_status oh_ctx_set_depthmap_batch_mode(oh_ctx* ctx, int persistent) {
  if (!ctx) return fail(OH_ERR_INVALID_ARG, "null context");
  if (persistent != 0 && persistent != 1) return fail(OH_ERR_INVALID_ARG, "batch mode must be 0 or 1");
  std::lock_guard<std::mutex> lk(ctx->mu);
  ctx->dm_batch_persistent = persistent;
  return OH_OK;
}

oh_status oh_ctx_set_test_stall(oh_ctx* ctx, int kernel_mask, long long cycles) {
  if (!ctx) return fail(OH_ERR_INVALID_ARG, "null context");
  if (kernel_mask < 0 || cycles < 0 || cycles > 4000000000LL)
    return fail(OH_ERR_INVALID_ARG, "test stall: mask >= 0 and 0 <= cycles <= 4e9");
  std::lock_guard<std::mutex> lk(ctx->mu);
  ctx->stall_mask = cycles > 0 ? kernel_mask : 0;
  ctx->stall_cycles = cycles;
  return OH_OK;
}

oh_status oh_ctx_set_timing(oh_ctx* ctx, int on) {
  if (!ctx) return fail(OH_ERR_INVALID_ARG, "null context");
  std::lock_guard<std::mutex> lk(ctx->mu);
  ctx->timing = on != 0;
  return OH_OK;
}

int oh_ctx_read_timing(oh_ctx* ctx, int reset, const char** names, double* ms, long* launches, int cap) {
  if (!ctx) return -1;
  std::lock_guard<std::mutex> lk(ctx->mu);
  int prev = 0;
  cudaGetDevice(&prev);
  cudaSetDevice(ctx->device);
  for (auto& m : ctx->marks) {
    float t = 0.f;
    cudaEventSynchronize(m.b);
    if (cudaEventElapsedTime(&t, m.a, m.b) != cudaSuccess) { cudaGetLastError(); t = 0.f; }
    auto& acc = ctx->timing_acc[m.name];
    acc.first += t;
    acc.second += 1;
    ctx->event_pool.push_back(m.a);
    ctx->event_pool.push_back(m.b);
  }
  ctx->marks.clear();
  cudaSetDevice(prev);
  int i = 0;
  for (auto& kv : ctx->timing_acc) {
    if (i < cap) {
      // names point into the map keys, valid until the next reset
      if (names) names[i] = kv.first.c_str();
      if (ms) ms[i] = kv.second.first;
      if (launches) launches[i] = kv.second.second;
    }
    ++i;
  }
  if (reset) {
    static thread_local std::vector<std::string> keep;
    keep.clear();
    for (auto& kv : ctx->timing_acc) keep.push_back(kv.first);
    if (names) for (int j = 0; j < i && j < cap; ++j) names[j] = keep[j].c_str();
    ctx->timing_acc.clear();
  }
  return i;
}
uint64_t oh_kernel_launch_count(void) { return g_launches.load(); }
const char* oh_version(void) { return "oh_gb300 0.1 (sm_103a)"; }

}  // extern "C"
