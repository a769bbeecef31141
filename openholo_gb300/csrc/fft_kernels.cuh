// Internal entry points shared between translation units.
#pragma once
#include <type_traits>
#include "context.h"
#include "fft_fast.cuh"

namespace oh {

// Enqueue out = [shift] FFT2 [shift] (in), optional aux = unshifted transform.
oh_status fft2d_enqueue(oh_ctx* ctx, int prec, int nx, int ny, const void* in, void* out, void* aux,
                        int direction, int shift, int normalize, cudaStream_t st);

// Enqueue ny independent length-nx transforms of contiguous rows (no shift).
oh_status fft_rows_enqueue(oh_ctx* ctx, int prec, int nx, int ny, const void* in, void* out, int direction,
                           int normalize, cudaStream_t st);

// Enqueue in-place transforms of the nx columns (length ny) of a [ny][nx]
// array (no shift).
oh_status fft_cols_enqueue(oh_ctx* ctx, int prec, int nx, int ny, void* data, int direction, int normalize,
                           cudaStream_t st);

// Widest column strip (8, 4, 2 or 1 columns) dividing nx whose ny-long
// complex lines fit in smax bytes of shared memory; 0 if none fits.
int pick_strip_width(int nx, int ny, size_t esz, size_t smax);

// SplitMix64 finaliser on a counter: the per-pixel random phase generator
// shared by the seeded depth-map mode and the synthetic scene generators.
__host__ __device__ __forceinline__ uint64_t splitmix64_at(uint64_t seed, uint64_t idx) {
  uint64_t z = seed + (idx + 1ull) * 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
// u in [0,1) with 24 random bits (exact in float)
__host__ __device__ __forceinline__ float u24_at(uint64_t seed, uint64_t idx) {
  return (float)(splitmix64_at(seed, idx) >> 40) * (1.0f / 16777216.0f);
}

// Calls f(std::integral_constant<int, n>) when n has a compile-time
// schedule, else f(std::integral_constant<int, 0>) (generic engine).
template <class F>
inline void with_fast_n(int n, F&& f) {
  switch (n) {
#define OH_WITH_CASE(len, ...) \
    case len: f(std::integral_constant<int, len>{}); return;
    OH_FAST_SCHEDULES(OH_WITH_CASE)
#undef OH_WITH_CASE
    default: f(std::integral_constant<int, 0>{}); return;
  }
}

// Same, restricted to the generic engine unless Enable (keeps FP64
// instantiations to one per kernel).
template <bool Enable, class F>
inline void with_fast_n_if(int n, F&& f) {
  if constexpr (Enable) with_fast_n(n, f);
  else f(std::integral_constant<int, 0>{});
}

}  // namespace oh
