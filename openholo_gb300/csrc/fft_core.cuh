// Block-level mixed-radix FFT on data resident in shared memory.
//
// A length-n line (n = r0*r1*...*r_{S-1}, radices 2,3,4,5,8 and any other
// prime through a generic O(r^2) butterfly) is transformed in place with the
// decimation-in-frequency (Sande-Tukey) recursion:
//   stage s works on blocks of m_s = r_s*q_s elements; for j < q_s it takes
//   x[j + t*q_s], t < r_s, forms the r_s-point DFT y_f, multiplies y_f by
//   W_{m_s}^{j f} and stores it back at j + f*q_s.
// After the last stage the spectrum value X[k] sits at position perm[k]
// (mixed-radix digit reversal); callers read outputs through that table, so
// no reordering pass is needed.  Twiddles W_n^e = exp(-2 pi i e/n) come from
// a table of n entries built on the host in double precision; SGN = -1 runs
// the forward transform, SGN = +1 the inverse (conjugate twiddles).
//
// Lines are addressed as buf[line*ls + i*es], so the same code serves a
// contiguous row (ls = n, es = 1) and a strip of W interleaved columns
// (ls = 1, es = W).
#pragma once
#include "oh_common.cuh"

namespace oh {

constexpr int kMaxStages = 24;
constexpr int kMaxGenericRadix = 64;

struct FFTPlan {
  int n;
  int nst;
  int radix[kMaxStages];
  int q[kMaxStages];      // stride inside a block at stage s
  int tws[kMaxStages];    // twiddle index step n/m_s
  const void* tw;         // n complex twiddles W_n^e (precision of the kernel)
  const int* perm;        // perm[k]: position of X[k] after the last stage
  const int* iperm;       // iperm[pos]: frequency k stored at pos
};

// ---- small DFT kernels (forward SGN=-1, inverse SGN=+1) -------------------

template <int SGN, typename C>
__device__ __forceinline__ void dft2(C& a, C& b) {
  C t = a; a = cadd(t, b); b = csub(t, b);
}

template <int SGN, typename C>
__device__ __forceinline__ void dft4(C& x0, C& x1, C& x2, C& x3) {
  C t0 = cadd(x0, x2), t1 = csub(x0, x2), t2 = cadd(x1, x3), t3 = csub(x1, x3);
  x0 = cadd(t0, t2); x2 = csub(t0, t2);
  x1 = cadd_i<SGN>(t1, t3); x3 = cadd_i<-SGN>(t1, t3);   // forward: t1 -/+ i t3
}

template <int SGN, typename C>
__device__ __forceinline__ void dft3(C& x0, C& x1, C& x2) {
  typedef decltype(x0.x) R;
  const R c = (R)0.86602540378443864676;   // sqrt(3)/2
  C t = cadd(x1, x2), d = csub(x1, x2);
  C y0 = cadd(x0, t);
  C m = caxpy((R)-0.5, t, x0);
  // forward y1 = m - i c d, y2 = m + i c d
  x0 = y0; x1 = caxpy_i<SGN>(c, d, m); x2 = caxpy_i<-SGN>(c, d, m);
}

template <int SGN, typename C>
__device__ __forceinline__ void dft5(C& x0, C& x1, C& x2, C& x3, C& x4) {
  typedef decltype(x0.x) R;
  const R c1 = (R)0.30901699437494742410;   // cos(2pi/5)
  const R c2 = (R)-0.80901699437494742410;  // cos(4pi/5)
  const R s1 = (R)0.95105651629515357212;   // sin(2pi/5)
  const R s2 = (R)0.58778525229247312917;   // sin(4pi/5)
  C a1 = cadd(x1, x4), b1 = csub(x1, x4), a2 = cadd(x2, x3), b2 = csub(x2, x3);
  C y0 = cadd(x0, cadd(a1, a2));
  const C p1 = caxpy(c2, a2, caxpy(c1, a1, x0));
  const C p2 = caxpy(c1, a2, caxpy(c2, a1, x0));
  const C q1 = caxpy(s2, b2, cscale(b1, s1));
  const C q2 = caxpy(-s1, b2, cscale(b1, s2));
  x0 = y0;
  // forward: p -/+ i q
  x1 = cadd_i<SGN>(p1, q1); x4 = cadd_i<-SGN>(p1, q1);
  x2 = cadd_i<SGN>(p2, q2); x3 = cadd_i<-SGN>(p2, q2);
}

template <int SGN, typename C>
__device__ __forceinline__ void dft8(C* x) {
  typedef decltype(x[0].x) R;
  const R h = (R)0.70710678118654752440;
  C e0 = x[0], e1 = x[2], e2 = x[4], e3 = x[6];
  C o0 = x[1], o1 = x[3], o2 = x[5], o3 = x[7];
  dft4<SGN>(e0, e1, e2, e3);
  dft4<SGN>(o0, o1, o2, o3);
  // w8^k for k = 1,2,3 (forward e^{-i pi k/4})
  C w1, w3;
  w1.x = h; w1.y = (R)SGN * h;
  w3.x = -h; w3.y = (R)SGN * h;
  o1 = cmul(o1, w1);
  o3 = cmul(o3, w3);
  x[0] = cadd(e0, o0); x[4] = csub(e0, o0);
  x[1] = cadd(e1, o1); x[5] = csub(e1, o1);
  x[2] = cadd_i<SGN>(e2, o2); x[6] = cadd_i<-SGN>(e2, o2);
  x[3] = cadd(e3, o3); x[7] = csub(e3, o3);
}

template <int SGN, typename C>
__device__ __forceinline__ C twiddle(const C* tw, int e) {
  C w = tw[e];
  if (SGN > 0) w.y = -w.y;
  return w;
}

// One DIF stage over `nl` lines.  col_major selects the thread mapping:
// true -> line index fastest (interleaved column strips), false -> butterfly
// index fastest (contiguous rows).
template <int SGN, typename C>
__device__ __forceinline__ void fft_stage(C* buf, int nl, int ls, int es, int n,
                                          int r, int q, int tws, const C* tw,
                                          bool line_fastest) {
  const int nb = n / r;            // butterflies per line
  const int total = nb * nl;
  for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
    int line, b;
    if (line_fastest) { line = idx % nl; b = idx / nl; }
    else { b = idx % nb; line = idx / nb; }
    const int blk = b / q, j = b - blk * q;
    const int base = line * ls + (blk * r * q + j) * es;
    const int st = q * es;
    switch (r) {
      case 2: {
        C a = buf[base], c = buf[base + st];
        dft2<SGN>(a, c);
        if (j) c = cmul(c, twiddle<SGN>(tw, j * tws));
        buf[base] = a; buf[base + st] = c;
      } break;
      case 3: {
        C a = buf[base], c = buf[base + st], d = buf[base + 2 * st];
        dft3<SGN>(a, c, d);
        if (j) { c = cmul(c, twiddle<SGN>(tw, j * tws)); d = cmul(d, twiddle<SGN>(tw, 2 * j * tws)); }
        buf[base] = a; buf[base + st] = c; buf[base + 2 * st] = d;
      } break;
      case 4: {
        C x0 = buf[base], x1 = buf[base + st], x2 = buf[base + 2 * st], x3 = buf[base + 3 * st];
        dft4<SGN>(x0, x1, x2, x3);
        if (j) {
          const int e = j * tws;
          x1 = cmul(x1, twiddle<SGN>(tw, e));
          x2 = cmul(x2, twiddle<SGN>(tw, 2 * e));
          x3 = cmul(x3, twiddle<SGN>(tw, 3 * e));
        }
        buf[base] = x0; buf[base + st] = x1; buf[base + 2 * st] = x2; buf[base + 3 * st] = x3;
      } break;
      case 5: {
        C x0 = buf[base], x1 = buf[base + st], x2 = buf[base + 2 * st], x3 = buf[base + 3 * st], x4 = buf[base + 4 * st];
        dft5<SGN>(x0, x1, x2, x3, x4);
        if (j) {
          const int e = j * tws;
          x1 = cmul(x1, twiddle<SGN>(tw, e));
          x2 = cmul(x2, twiddle<SGN>(tw, 2 * e));
          x3 = cmul(x3, twiddle<SGN>(tw, 3 * e));
          x4 = cmul(x4, twiddle<SGN>(tw, 4 * e));
        }
        buf[base] = x0; buf[base + st] = x1; buf[base + 2 * st] = x2; buf[base + 3 * st] = x3; buf[base + 4 * st] = x4;
      } break;
      case 8: {
        C x[8];
#pragma unroll
        for (int t = 0; t < 8; ++t) x[t] = buf[base + t * st];
        dft8<SGN>(x);
        if (j) {
          const int e = j * tws;
#pragma unroll
          for (int t = 1; t < 8; ++t) x[t] = cmul(x[t], twiddle<SGN>(tw, t * e));
        }
#pragma unroll
        for (int t = 0; t < 8; ++t) buf[base + t * st] = x[t];
      } break;
      default: {
        // generic odd radix: y_f = sum_t x_t w_r^{t f}, w_r^m = W_n^{m n / r}
        C x[kMaxGenericRadix];
        for (int t = 0; t < r; ++t) x[t] = buf[base + t * st];
        const int step = n / r;
        for (int f = 0; f < r; ++f) {
          C acc = x[0];
          int m = 0;
          for (int t = 1; t < r; ++t) {
            m += f; if (m >= r) m -= r;
            acc = cadd(acc, cmul(x[t], twiddle<SGN>(tw, m * step)));
          }
          if (j && f) acc = cmul(acc, twiddle<SGN>(tw, f * j * tws));
          buf[base + f * st] = acc;
        }
      } break;
    }
  }
}

// Full in-place transform of nl lines; ends with __syncthreads().
template <int SGN, typename C>
__device__ void block_fft(C* buf, int nl, int ls, int es, const FFTPlan& pl,
                          bool line_fastest) {
  const C* tw = static_cast<const C*>(pl.tw);
  for (int s = 0; s < pl.nst; ++s) {
    __syncthreads();
    fft_stage<SGN>(buf, nl, ls, es, pl.n, pl.radix[s], pl.q[s], pl.tws[s], tw, line_fastest);
  }
  __syncthreads();
}

}  // namespace oh
