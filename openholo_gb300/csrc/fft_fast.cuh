// Compile-time scheduled shared-memory FFT for the line lengths of the
// hologram workloads.  Same in-place decimation-in-frequency recursion and
// output order (perm table) as the generic engine in fft_core.cuh, but the
// radix schedule, strides and twiddle steps are template constants, so the
// butterfly index arithmetic compiles to shifts/multiplies and every stage
// is a straight-line radix-R kernel.  Radices 9 and 16 are split 3x3 / 4x4
// (Cooley-Tukey with constant twiddles); 6, 10, 12, 15 and 18 use the
// Good-Thomas prime-factor mapping (no internal twiddles).
//
// The schedules listed in OH_FAST_SCHEDULES are also what the host-side plan
// builder uses for these lengths, so both engines agree on output order.
#pragma once
#include "fft_core.cuh"

// length, then the radices in stage order
#define OH_FAST_SCHEDULES(X) \
  X(1024, 16, 16, 4)         \
  X(1080, 8, 9, 15)          \
  X(1536, 16, 16, 6)         \
  X(1920, 16, 8, 15)         \
  X(2048, 16, 16, 8)         \
  X(2160, 16, 9, 15)         \
  X(3072, 16, 16, 12)        \
  X(3840, 16, 16, 15)        \
  X(4096, 16, 16, 16)        \
  X(4320, 16, 18, 15)        \
  X(7680, 16, 16, 30)

namespace oh {

// ---- small DFTs on register arrays ----------------------------------------

template <int R, int SGN, typename C> struct DFT;

template <int SGN, typename C> struct DFT<2, SGN, C> {
  __device__ __forceinline__ static void run(C* x) { dft2<SGN>(x[0], x[1]); }
};
template <int SGN, typename C> struct DFT<3, SGN, C> {
  __device__ __forceinline__ static void run(C* x) { dft3<SGN>(x[0], x[1], x[2]); }
};
template <int SGN, typename C> struct DFT<4, SGN, C> {
  __device__ __forceinline__ static void run(C* x) { dft4<SGN>(x[0], x[1], x[2], x[3]); }
};
template <int SGN, typename C> struct DFT<5, SGN, C> {
  __device__ __forceinline__ static void run(C* x) { dft5<SGN>(x[0], x[1], x[2], x[3], x[4]); }
};
template <int SGN, typename C> struct DFT<8, SGN, C> {
  __device__ __forceinline__ static void run(C* x) { dft8<SGN>(x); }
};

// cos/sin(2 pi m / 16) and (2 pi m / 9), m = 0..4
__device__ __forceinline__ double w16c(int m) {
  return m == 0 ? 1.0 : m == 1 ? 0.9238795325112867561282 : m == 2 ? 0.7071067811865475244008
       : m == 3 ? 0.3826834323650897717285 : 0.0;
}
__device__ __forceinline__ double w16s(int m) {
  return m == 0 ? 0.0 : m == 1 ? 0.3826834323650897717285 : m == 2 ? 0.7071067811865475244008
       : m == 3 ? 0.9238795325112867561282 : 1.0;
}
__device__ __forceinline__ double w9c(int m) {
  return m == 0 ? 1.0 : m == 1 ? 0.7660444431189780352024 : m == 2 ? 0.1736481776669303488517
       : m == 3 ? -0.5 : -0.9396926207859083840541;
}
__device__ __forceinline__ double w9s(int m) {
  return m == 0 ? 0.0 : m == 1 ? 0.6427876096865393263226 : m == 2 ? 0.9848077530122080593667
       : m == 3 ? 0.8660254037844386467637 : 0.3420201433256687330441;
}

// multiply by W_N^m = exp(SGN * 2 pi i m / N) for N in {16, 9}, m small
template <int N, int SGN, typename C>
__device__ __forceinline__ C wmul(C a, int m) {
  typedef decltype(a.x) R;
  if (m == 0) return a;
  if (N == 16 && (m == 2 || m == 6)) {
    // W16^2 = h (1 + SGN i), W16^6 = -h (1 - SGN i), h = sqrt(1/2): a sum
    // and a difference, then one real scale
    const R h = (R)0.70710678118654752440;
    C u;
    if (m == 2) { u.x = a.x - (R)SGN * a.y; u.y = a.y + (R)SGN * a.x; return cscale(u, h); }
    u.x = a.x + (R)SGN * a.y; u.y = a.y - (R)SGN * a.x;
    return cscale(u, -h);
  }
  R c, s;
  if (N == 16) {
    // reduce m in [1, 9] to the first quadrant: W16^m for m = 4 is -i (fwd)
    if (m == 4) return cmul_i<SGN>(a);
    if (m < 4) { c = (R)w16c(m); s = (R)w16s(m); }
    else if (m < 8) { c = -(R)w16c(8 - m); s = (R)w16s(8 - m); }   // angle pi - a
    else if (m == 8) { C r; r.x = -a.x; r.y = -a.y; return r; }
    else { c = -(R)w16c(m - 8); s = -(R)w16s(m - 8); }              // angle pi + a
  } else {
    c = (R)w9c(m); s = (R)w9s(m);
  }
  C w; w.x = c; w.y = (R)SGN * s;
  return cmul(a, w);
}

// Cooley-Tukey N1 x N2 with constant twiddles W_N^{n2 k1}
template <int N1, int N2, int SGN, typename C>
__device__ __forceinline__ void dft_ct(C* x) {
  constexpr int N = N1 * N2;
  C a[N];
#pragma unroll
  for (int n2 = 0; n2 < N2; ++n2) {
    C v[N1];
#pragma unroll
    for (int n1 = 0; n1 < N1; ++n1) v[n1] = x[n2 + N2 * n1];
    DFT<N1, SGN, C>::run(v);
#pragma unroll
    for (int k1 = 0; k1 < N1; ++k1) a[n2 * N1 + k1] = wmul<N, SGN>(v[k1], n2 * k1);
  }
#pragma unroll
  for (int k1 = 0; k1 < N1; ++k1) {
    C v[N2];
#pragma unroll
    for (int n2 = 0; n2 < N2; ++n2) v[n2] = a[n2 * N1 + k1];
    DFT<N2, SGN, C>::run(v);
#pragma unroll
    for (int k2 = 0; k2 < N2; ++k2) x[k1 + N1 * k2] = v[k2];
  }
}

// Good-Thomas prime-factor N1 x N2 (gcd 1): n = (n1 N2 + n2 N1) mod N,
// X[k] = DFT_N2( DFT_N1 ) at (k mod N1, k mod N2)
template <int N1, int N2, int SGN, typename C>
__device__ __forceinline__ void dft_pfa(C* x) {
  constexpr int N = N1 * N2;
  C b[N];
#pragma unroll
  for (int n2 = 0; n2 < N2; ++n2) {
    C v[N1];
#pragma unroll
    for (int n1 = 0; n1 < N1; ++n1) v[n1] = x[(n1 * N2 + n2 * N1) % N];
    DFT<N1, SGN, C>::run(v);
#pragma unroll
    for (int k1 = 0; k1 < N1; ++k1) b[k1 * N2 + n2] = v[k1];
  }
#pragma unroll
  for (int k1 = 0; k1 < N1; ++k1) {
    DFT<N2, SGN, C>::run(b + k1 * N2);
  }
#pragma unroll
  for (int k = 0; k < N; ++k) x[k] = b[(k % N1) * N2 + (k % N2)];
}

template <int SGN, typename C> struct DFT<16, SGN, C> {
  __device__ __forceinline__ static void run(C* x) { dft_ct<4, 4, SGN>(x); }
};
template <int SGN, typename C> struct DFT<9, SGN, C> {
  __device__ __forceinline__ static void run(C* x) { dft_ct<3, 3, SGN>(x); }
};
template <int SGN, typename C> struct DFT<6, SGN, C> {
  __device__ __forceinline__ static void run(C* x) { dft_pfa<2, 3, SGN>(x); }
};
template <int SGN, typename C> struct DFT<10, SGN, C> {
  __device__ __forceinline__ static void run(C* x) { dft_pfa<2, 5, SGN>(x); }
};
template <int SGN, typename C> struct DFT<12, SGN, C> {
  __device__ __forceinline__ static void run(C* x) { dft_pfa<4, 3, SGN>(x); }
};
template <int SGN, typename C> struct DFT<15, SGN, C> {
  __device__ __forceinline__ static void run(C* x) { dft_pfa<3, 5, SGN>(x); }
};
template <int SGN, typename C> struct DFT<18, SGN, C> {
  __device__ __forceinline__ static void run(C* x) { dft_pfa<2, 9, SGN>(x); }
};
template <int SGN, typename C> struct DFT<30, SGN, C> {
  __device__ __forceinline__ static void run(C* x) { dft_pfa<2, 15, SGN>(x); }
};

// ---- twiddle sources: W_N^e = exp(-2 pi i e / N) ------------------------

template <typename C> struct TwTable {            // full table (global or shared)
  const C* t;
  __device__ __forceinline__ C operator()(int e) const { return t[e]; }
};
// entries of the low table of TwSplit: W^m for m < 64, then W^(4m) for m < 16
constexpr int kTwLo = 80;
template <typename C> struct TwSplit {            // W^e = W^(64 (e>>6)) * W^(e & 63)
  const C* lo;                                    // lo[m] = W_N^m, m < 64; lo[64 + m] = W_N^(4m), m < 16
  const C* hi;                                    // hi[m] = W_N^(64 m)
  __device__ __forceinline__ C operator()(int e) const { return cmul(hi[e >> 6], lo[e & 63]); }
  // W^(4e) = W^(64 (e>>4)) W^(4 (e & 15)): consecutive e read consecutive
  // entries (lo[4 (e & 15)] would put 16 consecutive e on four bank pairs)
  __device__ __forceinline__ C pow4(int e) const { return cmul(hi[e >> 4], lo[64 + (e & 15)]); }
};
// fill lo/hi (shared memory) from a full table; call with all threads, then sync
template <typename C>
__device__ __forceinline__ void load_tw_split(C* lo, C* hi, const C* tw, int n) {
  for (int m = threadIdx.x; m < kTwLo; m += blockDim.x) {
    const int e = m < 64 ? m : 4 * (m - 64);
    lo[m] = e < n ? tw[e] : tw[0];
  }
  for (int m = threadIdx.x; m < (n + 63) / 64; m += blockDim.x) hi[m] = tw[64 * m];
}
template <int SGN, typename C, class TW>
__device__ __forceinline__ C twid(const TW& tw, int e) {
  C w = tw(e);
  if (SGN > 0) w.y = -w.y;
  return w;
}
// W^(4e), conjugated for SGN > 0
template <int SGN, typename C, class TW>
__device__ __forceinline__ C twid4(const TW& tw, int e) {
  C w = tw(4 * e);
  if (SGN > 0) w.y = -w.y;
  return w;
}
template <int SGN, typename C>
__device__ __forceinline__ C twid4(const TwSplit<C>& tw, int e) {
  C w = tw.pow4(e);
  if (SGN > 0) w.y = -w.y;
  return w;
}

// Twiddles W^(e f), f = 1..R-1, from two fetches (W^e, W^4e) and products:
// W^(4a+b) = (W^4e)^a (W^e)^b; a few ulp of error for R <= 32.
template <int R, int SGN, typename C, class TW>
__device__ __forceinline__ void twiddle_powers(const TW& tw, int e, C* w) {
  w[1] = twid<SGN, C>(tw, e);
  if constexpr (R > 2) w[2] = cmul(w[1], w[1]);
  if constexpr (R > 3) w[3] = cmul(w[2], w[1]);
  if constexpr (R > 4) {
    w[4] = twid4<SGN, C>(tw, e);
#pragma unroll
    for (int f = 5; f < R; ++f) w[f] = cmul(w[f - 4], w[4]);
  }
}

// Forward/inverse DFT16 whose inputs 4..11 are zero (stage 0 of a 2x
// zero-padded line): inner length-4 DFTs over n1 see only n1 = 0 and 3.
template <int SGN, typename C>
__device__ __forceinline__ void dft16_halfzero(C* x) {
  C a[16];
#pragma unroll
  for (int n2 = 0; n2 < 4; ++n2) {
    const C x0 = x[n2], x3 = x[n2 + 12];
    // y_k = x0 + x3 * W4^(3k) = x0 + x3 * (-SGN i)^k
    C v[4];
    v[0] = cadd(x0, x3);
    v[1] = cadd_i<-SGN>(x0, x3);
    v[2] = csub(x0, x3);
    v[3] = cadd_i<SGN>(x0, x3);
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1) a[n2 * 4 + k1] = wmul<16, SGN>(v[k1], n2 * k1);
  }
#pragma unroll
  for (int k1 = 0; k1 < 4; ++k1) {
    C v[4] = {a[k1], a[4 + k1], a[8 + k1], a[12 + k1]};
    dft4<SGN>(v[0], v[1], v[2], v[3]);
#pragma unroll
    for (int k2 = 0; k2 < 4; ++k2) x[k1 + 4 * k2] = v[k2];
  }
}

// ---- one stage --------------------------------------------------------------

// BS / TS: stored block and input strides of a padded layout (M and M/R plain)
template <int N, int R, int M, int SGN, typename C, class TW, int BS = M, int TS = M / R>
__device__ __forceinline__ void fstage_t(C* buf, int nl, int ls, int es, const TW& tw, bool line_fastest) {
  constexpr int Q = M / R;
  constexpr int TWS = N / M;
  constexpr int NB = N / R;
  const int total = NB * nl;
  for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
    int line, b;
    if (line_fastest) { b = idx / nl; line = idx - b * nl; }
    else { line = idx / NB; b = idx - line * NB; }
    const int blk = b / Q, j = b - blk * Q;
    const int base = line * ls + (blk * BS + j) * es;
    const int st = TS * es;
    C x[R];
#pragma unroll
    for (int t = 0; t < R; ++t) x[t] = buf[base + t * st];
    DFT<R, SGN, C>::run(x);
    if (Q > 1 && j) {
      C w[R];
      twiddle_powers<R, SGN>(tw, j * TWS, w);
#pragma unroll
      for (int f = 1; f < R; ++f) x[f] = cmul(x[f], w[f]);
    }
#pragma unroll
    for (int t = 0; t < R; ++t) buf[base + t * st] = x[t];
  }
}

// Adjoint (transpose) of the forward stage fstage_t<N, R, M, -1>: inputs at
// j + f Q of each block times conj(W^(j f N/M)) for f >= 1, then DFT<R, +1>,
// outputs back at j + t Q.  The adjoint stages, run in reverse stage order on
// a line in the forward transform's storage order, compute its unnormalised
// inverse DFT with the output in natural order (the forward network maps x to
// P F x, its adjoint maps P y to F^H y = N F^-1 y).
//
// BS, TS and JG describe a padded layout: block blk starts at element blk BS,
// input t of a butterfly sits TS elements after input t - 1, and offset j is
// stored at j + j / JG (JG > 0) or j.
template <int N, int R, int M, typename C, class TW, int BS = M, int TS = M / R, int JG = 0>
__device__ __forceinline__ void fstage_adj(C* buf, int nl, int ls, int es, const TW& tw, bool line_fastest) {
  constexpr int Q = M / R;
  constexpr int TWS = N / M;
  constexpr int NB = N / R;
  const int total = NB * nl;
  for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
    int line, b;
    if (line_fastest) { b = idx / nl; line = idx - b * nl; }
    else { line = idx / NB; b = idx - line * NB; }
    const int blk = b / Q, j = b - blk * Q;
    const int base = line * ls + (blk * BS + (JG > 0 ? j + j / (JG > 0 ? JG : 1) : j)) * es;
    const int st = TS * es;
    C x[R];
#pragma unroll
    for (int t = 0; t < R; ++t) x[t] = buf[base + t * st];
    if (Q > 1 && j) {
      C w[R];
      twiddle_powers<R, 1>(tw, j * TWS, w);
#pragma unroll
      for (int f = 1; f < R; ++f) x[f] = cmul(x[f], w[f]);
    }
    DFT<R, 1, C>::run(x);
#pragma unroll
    for (int t = 0; t < R; ++t) buf[base + t * st] = x[t];
  }
}

// the adjoints of the stages (R, M), (Rest, M/R), ... in reverse order, each
// after a block barrier
template <int N, int M, typename C, class TW, int R, int... Rest>
__device__ __forceinline__ void fstages_adj(C* buf, int nl, int ls, int es, const TW& tw, bool line_fastest) {
  if constexpr (sizeof...(Rest) > 0) fstages_adj<N, M / R, C, TW, Rest...>(buf, nl, ls, es, tw, line_fastest);
  __syncthreads();
  fstage_adj<N, R, M>(buf, nl, ls, es, tw, line_fastest);
}

// Row stride of a per-stage twiddle table: R - 1 rounded up to odd, so that
// consecutive butterflies j read from distinct shared-memory bank pairs.
constexpr int stage_tab_stride(int R) { return (R - 1) | 1; }

// One stage with its twiddles from a per-stage table: tab[j S + f - 1] =
// W^(SGN j f N/M) for butterfly offset j < M/R, output f = 1..R-1, S =
// stage_tab_stride(R).  BS is the storage distance between consecutive
// blocks of M elements and TS that between a butterfly's inputs (M and M/R,
// or more for a padded layout).
template <int N, int R, int M, int SGN, typename C, int BS = M, int TS = M / R>
__device__ __forceinline__ void fstage_tab(C* buf, int nl, int ls, int es, const C* __restrict__ tab,
                                           bool line_fastest) {
  constexpr int Q = M / R;
  constexpr int NB = N / R;
  const int total = NB * nl;
  for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
    int line, b;
    if (line_fastest) { b = idx / nl; line = idx - b * nl; }
    else { line = idx / NB; b = idx - line * NB; }
    const int blk = b / Q, j = b - blk * Q;
    const int base = line * ls + (blk * BS + j) * es;
    const int st = TS * es;
    C x[R];
#pragma unroll
    for (int t = 0; t < R; ++t) x[t] = buf[base + t * st];
    DFT<R, SGN, C>::run(x);
    if (Q > 1 && j) {
      const C* tj = tab + j * stage_tab_stride(R) - 1;
#pragma unroll
      for (int f = 1; f < R; ++f) x[f] = cmul(x[f], tj[f]);
    }
#pragma unroll
    for (int t = 0; t < R; ++t) buf[base + t * st] = x[t];
  }
}

// Fill a per-stage table for fstage_tab from the full table tw (W_N^e,
// e < N); call with all threads, then sync.
template <int N, int R, int M, int SGN, typename C>
__device__ __forceinline__ void fill_stage_tab(C* tab, const C* __restrict__ tw) {
  constexpr int Q = M / R;
  constexpr int TWS = N / M;
  constexpr int TS = stage_tab_stride(R);
  for (int i = threadIdx.x; i < Q * TS; i += blockDim.x) {
    const int j = i / TS, f = i - j * TS + 1;
    C w = tw[(j * (f < R ? f : 0) * TWS) % N];       // f = R: the pad entry
    if (SGN > 0) w.y = -w.y;
    tab[i] = w;
  }
}

template <int N, int M, int SGN, typename C, class TW, int R, int... Rest>
__device__ __forceinline__ void fstages_t(C* buf, int nl, int ls, int es, const TW& tw, bool line_fastest) {
  __syncthreads();
  fstage_t<N, R, M, SGN>(buf, nl, ls, es, tw, line_fastest);
  if constexpr (sizeof...(Rest) > 0) fstages_t<N, M / R, SGN, C, TW, Rest...>(buf, nl, ls, es, tw, line_fastest);
}

template <int N, int R, int M, int SGN, typename C>
__device__ __forceinline__ void fstage(C* buf, int nl, int ls, int es, const C* __restrict__ tw,
                                       bool line_fastest) {
  constexpr int Q = M / R;         // stride of the butterfly inputs
  constexpr int TWS = N / M;       // twiddle step
  constexpr int NB = N / R;        // butterflies per line
  const int total = NB * nl;
  for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
    int line, b;
    if (line_fastest) { b = idx / nl; line = idx - b * nl; }
    else { line = idx / NB; b = idx - line * NB; }
    const int blk = b / Q, j = b - blk * Q;
    const int base = line * ls + (blk * M + j) * es;
    const int st = Q * es;
    C x[R];
#pragma unroll
    for (int t = 0; t < R; ++t) x[t] = buf[base + t * st];
    DFT<R, SGN, C>::run(x);
    if (Q > 1 && j) {
#pragma unroll
      for (int f = 1; f < R; ++f) x[f] = cmul(x[f], twiddle<SGN>(tw, j * f * TWS));
    }
#pragma unroll
    for (int t = 0; t < R; ++t) buf[base + t * st] = x[t];
  }
}

template <int N, int M, int SGN, typename C, int R, int... Rest>
__device__ __forceinline__ void fstages(C* buf, int nl, int ls, int es, const C* tw, bool line_fastest) {
  __syncthreads();
  fstage<N, R, M, SGN>(buf, nl, ls, es, tw, line_fastest);
  if constexpr (sizeof...(Rest) > 0) fstages<N, M / R, SGN, C, Rest...>(buf, nl, ls, es, tw, line_fastest);
}

// the first stage of the list with its table twiddles, then the others
template <int N, int M, int SGN, typename C, class TW, int R, int... Rest>
__device__ __forceinline__ void fstages_tab_first(C* buf, int nl, int ls, int es, const C* tab, const TW& tw,
                                                  bool line_fastest) {
  __syncthreads();
  fstage_tab<N, R, M, SGN>(buf, nl, ls, es, tab, line_fastest);
  if constexpr (sizeof...(Rest) > 0) fstages_t<N, M / R, SGN, C, TW, Rest...>(buf, nl, ls, es, tw, line_fastest);
}

// every stage of the list except the last one (block size M at entry)
template <int N, int M, int SGN, typename C, class TW, int R, int... Rest>
__device__ __forceinline__ void fstages_but_last(C* buf, int nl, int ls, int es, const TW& tw, bool line_fastest) {
  if constexpr (sizeof...(Rest) > 0) {
    __syncthreads();
    fstage_t<N, R, M, SGN>(buf, nl, ls, es, tw, line_fastest);
    fstages_but_last<N, M / R, SGN, C, TW, Rest...>(buf, nl, ls, es, tw, line_fastest);
  }
}

template <int D, int... Rs> struct FirstOr { static constexpr int value = D; };
template <int D, int R, int... Rs> struct FirstOr<D, R, Rs...> { static constexpr int value = R; };

template <int... Rs> struct LastOf;
template <int R> struct LastOf<R> { static constexpr int value = R; };
template <int R, int... Rs> struct LastOf<R, Rs...> { static constexpr int value = LastOf<Rs...>::value; };

template <int N, int R0, int... Rest>
struct SchedImpl {
  static constexpr bool ok = true;
  static constexpr int r0 = R0;
  static constexpr int r1 = FirstOr<1, Rest...>::value;
  static constexpr int nstages = 1 + (int)sizeof...(Rest);
  static constexpr int rlast = LastOf<R0, Rest...>::value;
  // stages 1 .. S-2 (the caller runs stage 0 and the last stage itself)
  template <int SGN, typename C, class TW>
  __device__ __forceinline__ static void run_middle(C* buf, int nl, int ls, int es, const TW& tw, bool lf) {
    if constexpr (sizeof...(Rest) > 0) fstages_but_last<N, N / R0, SGN, C, TW, Rest...>(buf, nl, ls, es, tw, lf);
  }
  template <int SGN, typename C>
  __device__ __forceinline__ static void run(C* buf, int nl, int ls, int es, const C* tw, bool lf) {
    fstages<N, N, SGN, C, R0, Rest...>(buf, nl, ls, es, tw, lf);
  }
  // all stages with a twiddle functor
  template <int SGN, typename C, class TW>
  __device__ __forceinline__ static void run_t(C* buf, int nl, int ls, int es, const TW& tw, bool lf) {
    fstages_t<N, N, SGN, C, TW, R0, Rest...>(buf, nl, ls, es, tw, lf);
  }
  // unnormalised inverse DFT of a line in this schedule's storage order,
  // output in natural order (the adjoint network)
  template <typename C, class TW>
  __device__ __forceinline__ static void run_adj(C* buf, int nl, int ls, int es, const TW& tw, bool lf) {
    fstages_adj<N, N, C, TW, R0, Rest...>(buf, nl, ls, es, tw, lf);
  }
  // every stage after the first (the caller ran stage 0 itself)
  template <int SGN, typename C, class TW>
  __device__ __forceinline__ static void run_rest(C* buf, int nl, int ls, int es, const TW& tw, bool lf) {
    if constexpr (sizeof...(Rest) > 0) fstages_t<N, N / R0, SGN, C, TW, Rest...>(buf, nl, ls, es, tw, lf);
  }
  // Output order of this schedule as arithmetic (the plan's perm / iperm
  // tables): X[k], k = f0 + r0 f1 + r0 r1 f2 + ..., sits at position
  // sum_s f_s N / (r0 ... r_s).
  __host__ __device__ __forceinline__ static constexpr int perm(int k) {
    constexpr int rs[] = {R0, Rest...};
    int pos = 0, q = N;
#pragma unroll
    for (int s = 0; s < nstages; ++s) {
      q /= rs[s];
      pos += (k % rs[s]) * q;
      k /= rs[s];
    }
    return pos;
  }
  __host__ __device__ __forceinline__ static constexpr int iperm(int pos) {
    constexpr int rs[] = {R0, Rest...};
    int k = 0, mul = 1, q = N;
#pragma unroll
    for (int s = 0; s < nstages; ++s) {
      q /= rs[s];
      const int f = pos / q;
      pos -= f * q;
      k += f * mul;
      mul *= rs[s];
    }
    return k;
  }
  // entries of the stage-1 twiddle table (fill_stage_tab<N, r1, N / r0>)
  static constexpr int tab1_entries = (N / R0 / r1) * stage_tab_stride(r1);
  // as run_rest, with stage 1's twiddles from its table tab1
  template <int SGN, typename C, class TW>
  __device__ __forceinline__ static void run_rest_tab(C* buf, int nl, int ls, int es, const C* tab1, const TW& tw,
                                                      bool lf) {
    if constexpr (sizeof...(Rest) > 0) fstages_tab_first<N, N / R0, SGN, C, TW, Rest...>(buf, nl, ls, es, tab1, tw, lf);
  }
};

template <int N> struct FastSched { static constexpr bool ok = false; };
#define OH_DEFINE_SCHED(n, ...) \
  template <> struct FastSched<n> : SchedImpl<n, __VA_ARGS__> {};
OH_FAST_SCHEDULES(OH_DEFINE_SCHED)
#undef OH_DEFINE_SCHED

// In-place transform of nl lines with the compile-time schedule for N when
// N > 0, else the generic engine; ends with __syncthreads().
template <int N, int SGN, typename C>
__device__ __forceinline__ void block_fft_n(C* buf, int nl, int ls, int es, const FFTPlan& pl, bool line_fastest) {
  if constexpr (N > 0) {
    FastSched<N>::template run<SGN>(buf, nl, ls, es, static_cast<const C*>(pl.tw), line_fastest);
    __syncthreads();
  } else {
    block_fft<SGN>(buf, nl, ls, es, pl, line_fastest);
  }
}

}  // namespace oh
