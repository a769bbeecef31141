// Device side of the depth-map pipeline shared by the per-frame launches
// (depthmap.cu) and the persistent batch kernel (dm_batch.cu): frame
// arguments, the table set-up, and the row, column and output passes as
// block bodies.  Each pass is a __device__ body taking the block index it
// works on; the per-frame kernels call it with blockIdx.x, the batch
// kernel with the index of a work item.
#pragma once
#include <cstdint>
#include "context.h"
#include "fft_kernels.cuh"

namespace oh {

constexpr int kMaxEntries = 256;

// Per-frame constants, passed by value to dm_setup (no host->device copy in
// the frame, so a frame can be captured in a CUDA graph).
struct DMSetup {
  int n_entries, n_uslots;
  int16_t uslot_of_entry[kMaxEntries];
  double zp[kMaxEntries];            // z' of each render entry
  double cre[kMaxEntries], cim[kMaxEntries];   // per-entry complex constant
  int16_t lut[256];                  // depth byte -> unique slot (-1: none)
};

template <typename R>
struct DMArgs {
  typedef typename cplx_of<R>::type C;
  int pnx, pny, Px, Py, ox, oy, hx, hy;
  int W, lw, nstrips, n_entries, n_uslots;     // lw = log2(W)
  int cx1, cx2, cy1, cy2;            // SSB crop window on the (padded) spectrum
  double ppx, ppy, ssx, ssy, lambda, k;
  const uint8_t* img;
  const uint8_t* depth;
  const float* phase;
  int phase_mode;
  uint64_t seed;
  const C* src;          // complex source field [pny][pnx] (one layer, img/depth unused) or null
  // device tables (written by dm_setup)
  int16_t* lut;          // 256
  int16_t* uslot_of_entry;
  R* kzp;                // k*z' per entry
  C* cst;                // per-entry constant
  C* exc;                // [entries][Px] cst*exp(i alpha fx^2)   (fp32 path)
  R* eth;                // [entries][Py] phase alpha fy^2 reduced to [-pi, pi], y storage order (fast passes)
  C* ey;                 // [entries][Py] exp(i alpha fy^2)       (fp32 path)
  R* lfx;                // [Px] (lambda fx)^2
  R* lfy;                // [Py] (lambda fy)^2
  R* lfyp;               // [Py] (lambda fy)^2 in FFT storage order (fast column pass)
  int ey_perm;           // 1: ey rows stored in FFT storage order (fast column pass)
  C* shy;                // [pny] y shift phase / (Px*Py)
  C* shx;                // [pnx] x shift phase
  int* slot_any;         // [uslots]
  uint8_t* occ;          // [uslots][pny]
  C* Rbuf;               // [uslots][nstrips][pny][W]
  C* V;                  // [pny][Px]
  R* fringe;             // [pny][pnx]
  C* field;              // [pny][pnx] or null
  C* spectrum;           // [Py][Px] or null
  int sig_x, sig_y;
  int occ_stride;        // bytes per layer row of occ (multiple of 16)
  int xs;                // 1: R and V columns are in the row FFT's storage order (fast passes), 0: kx order
  int hzx, hzy;          // 1: 2x padding with a radix-16 first stage (stage-0 inputs 4..11 are zero)
  int* err;              // device error word (bounded waits that ran out)
  const int* stall_flag; // error-path test hook: wait on this never-set flag before the first layer
  long long stall_cycles;
  // layer chunks (fast FP32 path): this launch pair covers layer slots (and
  // render entries) [slot0, slot1); R and occ hold only those slots; the
  // column pass's accumulators pass between chunks through accbuf
  int slot0, slot1;
  int e0, e1;            // render entries of this chunk (all entries when unchunked)
  int chunk_first, chunk_last;
  C* accbuf;
  // evenly spaced layers (fast column pass): step dz = z'_e - z'_(e-1) of the
  // render entries; D = Dx(fx) Dy(fy) exp(-i k dz g) per spectrum element
  int horner;
  uint32_t fkeep;        // fast column pass: bit f set when last-stage output f can fall in the SSB crop
  float kdz_pi;          // k dz / pi
  double dz;
  C* dxh;                // [Px] exp(-i pi lambda dz fx^2)
  C* dyh;                // [Py] exp(-i pi lambda dz fy^2), y storage order
  FFTPlan plx, ply;
};

__device__ __forceinline__ double2 cexp_d(double ph) {
  double s, c;
  sincos(ph, &s, &c);
  return make_double2(c, s);
}

// exp(i*ph) for large |ph|: reduce modulo 2 pi in double first.
__device__ __forceinline__ double2 cexp_reduced(double ph) {
  const double two_pi = 6.283185307179586476925286766559;
  double n = rint(ph / two_pi);
  return cexp_d(fma(-n, two_pi, ph));
}

// Tables of one frame; thread tid of nthr.
template <typename R>
__device__ __forceinline__ void dm_setup_body(const DMArgs<R>& a, const DMSetup& s, int tid, int nthr) {
  typedef typename cplx_of<R>::type C;
  const double pi = 3.14159265358979323846;
  for (int i = tid; i < 256; i += nthr) a.lut[i] = s.lut[i];
  for (int e = tid; e < s.n_entries; e += nthr) {
    a.uslot_of_entry[e] = s.uslot_of_entry[e];
    a.kzp[e] = (R)(a.k * s.zp[e]);
    a.cst[e] = mk((R)s.cre[e], (R)s.cim[e]);
  }
  for (int u = tid; u < s.n_uslots; u += nthr) a.slot_any[u] = 0;
  // reference frequency grid (HologramKernel.cu:85-86)
  for (int x = tid; x < a.Px; x += nthr) {
    double fx = (-1.0 / (2.0 * a.ppx)) + (1.0 / a.ssx) * (double)x;
    double l = a.lambda * fx;
    a.lfx[x] = (R)(l * l);
  }
  for (int y = tid; y < a.Py; y += nthr) {
    double fy = (1.0 / (2.0 * a.ppy)) - (1.0 / a.ssy) - (1.0 / a.ssy) * (double)y;
    double l = a.lambda * fy;
    a.lfy[y] = (R)(l * l);
    // storage position p of the column FFT output holds spectrum row ky(p)
    int ky = a.ply.iperm[y] + a.hy;
    if (ky >= a.Py) ky -= a.Py;
    double fyp = (1.0 / (2.0 * a.ppy)) - (1.0 / a.ssy) - (1.0 / a.ssy) * (double)ky;
    double lp = a.lambda * fyp;
    a.lfyp[y] = (R)(lp * lp);
  }
  if constexpr (sizeof(R) == 4) {
    // separable paraxial factors exp(i pi lambda z' f^2), reduced in double
    for (int idx = tid; idx < s.n_entries * a.Px; idx += nthr) {
      int e = idx / a.Px, x = idx - e * a.Px;
      double fx = (-1.0 / (2.0 * a.ppx)) + (1.0 / a.ssx) * (double)x;
      double2 v = cexp_reduced(pi * a.lambda * s.zp[e] * fx * fx);
      double2 c = make_double2(s.cre[e], s.cim[e]);
      a.exc[idx] = mk((R)(c.x * v.x - c.y * v.y), (R)(c.x * v.y + c.y * v.x));
    }
    if (a.horner) {
      for (int x = tid; x < a.Px; x += nthr) {
        double fx = (-1.0 / (2.0 * a.ppx)) + (1.0 / a.ssx) * (double)x;
        double2 v = cexp_reduced(-pi * a.lambda * a.dz * fx * fx);
        a.dxh[x] = mk((R)v.x, (R)v.y);
      }
      for (int p = tid; p < a.Py; p += nthr) {
        int y = a.ply.iperm[p] + a.hy;
        if (y >= a.Py) y -= a.Py;
        double fy = (1.0 / (2.0 * a.ppy)) - (1.0 / a.ssy) - (1.0 / a.ssy) * (double)y;
        double2 v = cexp_reduced(-pi * a.lambda * a.dz * fy * fy);
        a.dyh[p] = mk((R)v.x, (R)v.y);
      }
    }
    if (a.ey_perm) {
      const double two_pi = 6.283185307179586476925286766559;
      for (int idx = tid; idx < s.n_entries * a.Py; idx += nthr) {
        int e = idx / a.Py, p = idx - e * a.Py;
        int y = a.ply.iperm[p] + a.hy;
        if (y >= a.Py) y -= a.Py;
        double fy = (1.0 / (2.0 * a.ppy)) - (1.0 / a.ssy) - (1.0 / a.ssy) * (double)y;
        double ph = pi * a.lambda * s.zp[e] * fy * fy;
        a.eth[idx] = (R)(ph - two_pi * rint(ph / two_pi));
      }
    }
    for (int idx = tid; idx < s.n_entries * a.Py; idx += nthr) {
      int e = idx / a.Py, y = idx - e * a.Py;
      if (a.ey_perm) {
        y = a.ply.iperm[y] + a.hy;
        if (y >= a.Py) y -= a.Py;
      }
      double fy = (1.0 / (2.0 * a.ppy)) - (1.0 / a.ssy) - (1.0 / a.ssy) * (double)y;
      double2 v = cexp_reduced(pi * a.lambda * s.zp[e] * fy * fy);
      a.ey[idx] = mk((R)v.x, (R)v.y);
    }
  }
  // encoding shift phases (get_shift_phase_value, HologramGenerator_CPU.cpp:367-408)
  const double norm = 1.0 / ((double)a.Px * (double)a.Py);
  const double ssy0 = a.ppy * a.pny, ssx0 = a.ppx * a.pnx;
  for (int r = tid; r < a.pny; r += nthr) {
    double2 v = make_double2(1.0, 0.0);
    if (a.sig_y != 0) {
      double yy = (ssy0 / 2.0) - a.ppy * (double)r - a.ppy;
      double ph = a.sig_y == 1 ? 2.0 * pi * (yy / (4.0 * a.ppy)) : 2.0 * pi * (-yy / (4.0 * a.ppy));
      v = cexp_reduced(ph);
    }
    a.shy[r] = mk((R)(v.x * norm), (R)(v.y * norm));
  }
  for (int c = tid; c < a.pnx; c += nthr) {
    double2 v = make_double2(1.0, 0.0);
    if (a.sig_x != 0) {
      double xx = (-ssx0 / 2.0) - a.ppx * (double)c - a.ppx;
      double ph = a.sig_x == -1 ? 2.0 * pi * (-xx / (4.0 * a.ppx)) : 2.0 * pi * (xx / (4.0 * a.ppx));
      v = cexp_reduced(ph);
    }
    a.shx[c] = mk((R)v.x, (R)v.y);
  }
}

template <typename R>
__global__ void dm_setup(DMArgs<R> a, DMSetup s) {
  dm_setup_body<R>(a, s, blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x);
}

template <typename R>
__device__ __forceinline__ void sincos_r(R x, R* s, R* c);
template <> __device__ __forceinline__ void sincos_r<float>(float x, float* s, float* c) { sincosf(x, s, c); }
template <> __device__ __forceinline__ void sincos_r<double>(double x, double* s, double* c) { sincos(x, s, c); }

// Two image rows per block: their layer lines are transformed as a pair and
// stored together, so each strip receives 2*W contiguous complex values
// (a full 32-byte sector for W = 2).
constexpr int kRowPair = 2;

// two blocks per SM where two row pairs fit in shared memory (padded lengths
// up to 4320); the register cap that comes with it applies only there
template <int NX> constexpr int row_min_blocks() { return NX > 0 && NX <= 4320 ? 2 : 1; }

// Shared-memory layout of the row pass's fused path (three-stage schedules
// whose last stage has 256 butterflies per row, two rows, last stage stored
// straight from registers): element p of row l sits at l LS + (p / M1) BS +
// p % M1, M1 = NX / r0 (one stage-0 output block).  The block pad BS - M1
// puts consecutive blocks Q1 = M1 / r1 bank pairs apart, so the middle
// stage's half-warps (consecutive butterflies, across a block boundary) hit
// 16 distinct 8-byte bank pairs; the row stride LS does the same for the last
// stage (8 butterflies x 2 rows per half-warp).  Where no pad makes both
// conflict free the plain layout (LS = NX, BS = M1) is kept.
template <int NX, bool FAST = (NX > 0)> struct RowPad {
  static constexpr bool fusable = false;
  static constexpr int LS = NX, BS = 0, LSMAX = NX, RLP = 0, JG = 0, BPB = 1;
};
template <int NX> struct RowPad<NX, true> {
  typedef FastSched<NX> S;
  static constexpr bool fusable = S::nstages == 3 && NX / S::rlast == 256;
  static constexpr int M1 = NX / S::r0, Q1 = M1 / S::r1, RL = S::rlast, NB1 = NX / S::r1;
  static constexpr int BPB = M1 % RL == 0 ? M1 / RL : 0;    // last-stage butterflies per block
  // element p of a row at (p / M1) bs + (p % M1) + rp ((p % M1) / RL): rp = 1
  // pads every RL elements (an even RL puts a half-warp of the last stage
  // on one bank pair otherwise), bs - M1 (1 + rp / RL) pads every block
  static constexpr int at(int p, int bs, int rp) { return (p / M1) * bs + p % M1 + rp * ((p % M1) / RL); }
  static constexpr bool conflict_free(int bs, int ls, int rp) {
    if (BPB == 0 || Q1 != RL) return false;
    for (int h = 0; h < 2 * M1 / 16; ++h) {           // stage 0 stores, line-major: at most 2-way
      int seen = 0, twice = 0;                        // (the per-RL pad skips a pair every RL stores)
      for (int i = 0; i < 16; ++i) {
        const int idx = h * 16 + i, line = idx / M1, j = idx % M1;
        const int e = line * ls + at(j, bs, rp);
        if (twice & (1 << (e % 16))) return false;
        if (seen & (1 << (e % 16))) twice |= 1 << (e % 16);
        seen |= 1 << (e % 16);
      }
    }
    for (int h = 0; h < 2 * NB1 / 16; ++h) {          // middle stage, line-major
      int seen = 0;
      for (int i = 0; i < 16; ++i) {
        const int idx = h * 16 + i, line = idx / NB1, b = idx % NB1;
        const int e = line * ls + at((b / Q1) * M1 + b % Q1, bs, rp);
        if (seen & (1 << (e % 16))) return false;
        seen |= 1 << (e % 16);
      }
    }
    for (int h = 0; h < 512 / 16; ++h) {              // last stage, thread pairs = rows
      int seen = 0;
      for (int i = 0; i < 16; ++i) {
        const int idx = h * 16 + i, b = idx >> 1, l = idx & 1;
        const int e = l * ls + at(b * RL, bs, rp);
        if (seen & (1 << (e % 16))) return false;
        seen |= 1 << (e % 16);
      }
    }
    return true;
  }
  // first (rp, block pad, row stride) free of conflicts in the middle and
  // last stages (stage-0 stores at most 2-way), plain layout preferred;
  // packed as rp << 24 | pad << 16 | (ls - base), or -1
  static constexpr int search() {
    for (int rp = 0; rp <= (RL % 2 == 0 ? 1 : 0); ++rp)
      for (int pad = 0; pad < 16; ++pad) {
        const int bs = M1 + rp * (M1 / RL) + pad, base = S::r0 * bs;
        for (int d = 0; d < 16; ++d)
          if (conflict_free(bs, base + d, rp)) return rp << 24 | pad << 16 | d;
      }
    return -1;
  }
  static constexpr int found = fusable ? search() : -1;
  static constexpr bool padded = found >= 0;
  static constexpr int RP = padded ? found >> 24 : 0;
  static constexpr int BS = padded ? M1 + RP * (M1 / RL) + ((found >> 16) & 0xff) : M1;
  static constexpr int LS = padded ? S::r0 * BS + (found & 0xffff) : NX;
  static constexpr int RLP = RL + RP;                        // stored length of RL elements
  static constexpr int JG = RP ? RL : 0;                    // stage-0 offset j stored at j + j / JG
  static constexpr int LSMAX = LS > NX ? LS : NX;
};

// Static shared memory of the row and column bodies, one instance per
// kernel whatever the instantiations it inlines (a kernel that runs several
// lengths keeps its static shared memory small).
__device__ __forceinline__ int16_t* dm_row_slut() {
  __shared__ int16_t slut[256];
  return slut;
}
struct ColShared {
  int kxw[8];                 // spectrum column of each strip column
  float2 dxw[8];              // its Dx factor (layer-step form)
  int nact, last;
};
__device__ __forceinline__ ColShared* dm_col_shared() {
  __shared__ ColShared cs;
  return &cs;
}

// Row pair blk of a frame, NT threads (the fused last stage is written for
// 512 thread slots: 256 butterflies x 2 rows; fewer threads take several).
template <typename R, int NX, int NT>
__device__ __forceinline__ void dm_row_body(const DMArgs<R>& a, int blk) {
  typedef typename cplx_of<R>::type C;
  static_assert(512 % NT == 0, "row pass: 512 thread slots over NT threads");
  extern __shared__ unsigned char smem_raw[];
  const int Px = a.Px, pnx = a.pnx;
  const int lip = (pnx + 7) & ~7;                       // keeps 16-byte alignment
  typedef RowPad<NX> RP;
  const int lsmax = NX > 0 ? RP::LSMAX : Px;
  C* buf = reinterpret_cast<C*>(smem_raw);              // [2][lsmax]
  C* v = buf + 2 * lsmax;                               // [2][pnx] source values
  int16_t* li = reinterpret_cast<int16_t*>(v + 2 * pnx);   // [2][lip] layer slot per pixel
  uint32_t* mask = reinterpret_cast<uint32_t*>(li + 2 * lip);   // [2][8] layers present per row
  C* twlo = reinterpret_cast<C*>(mask + 16);            // kTwLo + ceil(Px/64) twiddles (fast path)
  C* twhi = twlo + kTwLo;
  C* tab1 = twhi + (Px + 63) / 64;                      // stage-1 twiddle table (fast path)
  const int r0 = blk * kRowPair;
  const int nrows = min(kRowPair, a.pny - r0);
  // fused last stage + strip store, in the padded layout
  const bool fused = RP::fusable && a.W == 2 && a.xs && nrows == 2;
  for (int i = threadIdx.x; i < 16; i += NT) mask[i] = 0u;
  int16_t* const slut = dm_row_slut();                  // depth byte -> layer slot
  for (int i = threadIdx.x; i < 256; i += NT) slut[i] = a.lut[i];
  if constexpr (NX > 0) {
    load_tw_split(twlo, twhi, static_cast<const C*>(a.plx.tw), NX);
    fill_stage_tab<NX, FastSched<NX>::r1, NX / FastSched<NX>::r0, -1>(tab1, static_cast<const C*>(a.plx.tw));
  }
  __syncthreads();
  // the image and depth bytes of up to kSetupPix pixels per thread are loaded
  // before any is used, so their latency is paid once
  constexpr int kSetupPix = 8;
  // layer-presence bits of slots 0..63 per row, gathered in registers and
  // OR-reduced per warp (one shared atomic per warp and word instead of one
  // per pixel, which all hit the same word); higher slots use the atomics
  uint32_t pm00 = 0u, pm01 = 0u, pm10 = 0u, pm11 = 0u;     // [row][word], scalars (no local memory)
  for (int base = 0; base < kRowPair * pnx; base += kSetupPix * NT) {
    uint8_t gb[kSetupPix], db[kSetupPix];
#pragma unroll
    for (int q = 0; q < kSetupPix; ++q) {
      const int idx = base + q * NT + threadIdx.x;
      const int l = idx / pnx, c = idx - l * pnx;
      gb[q] = 0; db[q] = 0;
      if (idx < kRowPair * pnx && l < nrows && !a.src) {
        const size_t off = (size_t)(r0 + l) * pnx + c;
        gb[q] = a.img[off];
        db[q] = a.depth[off];
      }
    }
#pragma unroll
    for (int q = 0; q < kSetupPix; ++q) {
      const int idx = base + q * NT + threadIdx.x;
      if (idx >= kRowPair * pnx) break;
      const int l = idx / pnx, c = idx - l * pnx;
      int u = -1;
      C val = mk((R)0, (R)0);
      if (l < nrows && a.src) {
        // a complex source field: every pixel in the one layer slot
        u = 0;
        val = a.src[(size_t)(r0 + l) * pnx + c];
        if (c == 0) atomicOr(&mask[l * 8], 1u);
      } else if (l < nrows) {
        const size_t off = (size_t)(r0 + l) * pnx + c;
        const uint8_t g = gb[q];
        u = g > 0 ? (int)slut[db[q]] : -1;
        if (u >= 0) {
          const R amp = (R)g / (R)255;
          if (a.phase_mode == OH_PHASE_REFERENCE) {
            val = mk(amp, (R)0);
          } else {
            R ph;
            if (a.phase_mode == OH_PHASE_ARRAY) ph = (R)a.phase[off];
            else ph = (R)u24_at(a.seed, off) * (R)6.283185307179586476925;
            R sn, cs;
            sincos_r<R>(ph, &sn, &cs);
            val = mk(amp * cs, amp * sn);
          }
          const uint32_t bit = 1u << (u & 31);
          if (u < 32) { if (l == 0) pm00 |= bit; else pm10 |= bit; }
          else if (u < 64) { if (l == 0) pm01 |= bit; else pm11 |= bit; }
          else atomicOr(&mask[l * 8 + (u >> 5)], bit);
        }
      }
      li[l * lip + c] = (int16_t)u;
      v[l * pnx + c] = val;
    }
  }
  {
    const uint32_t m00 = __reduce_or_sync(0xffffffffu, pm00), m01 = __reduce_or_sync(0xffffffffu, pm01);
    const uint32_t m10 = __reduce_or_sync(0xffffffffu, pm10), m11 = __reduce_or_sync(0xffffffffu, pm11);
    if ((threadIdx.x & 31) == 0) {
      if (m00) atomicOr(&mask[0], m00);
      if (m01) atomicOr(&mask[1], m01);
      if (m10) atomicOr(&mask[8], m10);
      if (m11) atomicOr(&mask[9], m11);
    }
  }
  __syncthreads();
  for (int u = a.slot0; u < a.slot1; ++u) {
    const bool p0 = (mask[u >> 5] >> (u & 31)) & 1u;
    const bool p1 = (mask[8 + (u >> 5)] >> (u & 31)) & 1u;
    const int ur = u - a.slot0;                       // slot within this chunk's buffers
    if (threadIdx.x < nrows) {
      const bool pr = threadIdx.x == 0 ? p0 : p1;
      a.occ[(size_t)ur * a.occ_stride + r0 + threadIdx.x] = pr ? 1 : 0;
    }
    if (!(p0 || p1)) continue;
    if (threadIdx.x == 0) a.slot_any[u] = 1;
    if constexpr (NX > 0) {
      // stage 0 straight from the source rows: inputs j + t*Q0 of each
      // x-shifted, zero-padded line a[j] = u[(j - hx) mod Px]
      constexpr int R0 = FastSched<NX>::r0;
      constexpr int Q0 = NX / R0;
      const TwSplit<C> tw{twlo, twhi};
      const int ls = fused ? RP::LS : Px, bs = fused ? RP::BS : Q0;
      for (int idx = threadIdx.x; idx < kRowPair * Q0; idx += NT) {
        const int l = idx / Q0, j = idx - l * Q0;
        const int16_t* lil = li + l * lip;
        const C* vl = v + l * pnx;
        C x[R0];
        if (R0 == 16 && a.hzx) {
          // 2x padding: inputs t = 4..11 fall in the zero columns; with
          // hx = NX/2 and ox = NX/4 the image column of input t is
          // j + (t + 4) Q0 (t < 4) or j + (t - 12) Q0 (t >= 12)
#pragma unroll
          for (int t = 0; t < R0; ++t) {
            if (t >= 4 && t < 12) { x[t] = mk((R)0, (R)0); continue; }
            const int c = j + (t < 4 ? t + 4 : t - 12) * Q0;
            x[t] = lil[c] == u ? vl[c] : mk((R)0, (R)0);
          }
          dft16_halfzero<-1>(x);
        } else {
#pragma unroll
          for (int t = 0; t < R0; ++t) {
            int xx = j + t * Q0 - a.hx;
            if (xx < 0) xx += NX;
            const int c = xx - a.ox;
            C val = mk((R)0, (R)0);
            if (c >= 0 && c < pnx && lil[c] == u) val = vl[c];
            x[t] = val;
          }
          DFT<R0, -1, C>::run(x);
        }
        if (j) {
          C wp[R0];
          twiddle_powers<R0, -1>(tw, j, wp);
#pragma unroll
          for (int f = 1; f < R0; ++f) x[f] = cmul(x[f], wp[f]);
        }
        C* bl = buf + l * ls + (fused && RP::JG > 0 ? j / (RP::JG > 0 ? RP::JG : 1) : 0);
#pragma unroll
        for (int f = 0; f < R0; ++f) bl[j + f * bs] = x[f];
      }
      if constexpr (RP::fusable) {
        if (fused) {
          // middle stage, then the last stage (no twiddles) straight from
          // registers into the strips: thread pair (2b, 2b+1) = rows r0, r0+1
          // of butterfly b; each writes 16 bytes (storage positions p, p+1 of
          // its row) of the same 32-byte strip sector
          constexpr int RL = FastSched<NX>::rlast;
          __syncthreads();
          fstage_tab<NX, FastSched<NX>::r1, NX / FastSched<NX>::r0, -1, C, RP::BS, RP::RLP>(buf, kRowPair, RP::LS, 1,
                                                                                           tab1, false);
          __syncthreads();
#pragma unroll
          for (int vi = 0; vi < 512 / NT; ++vi) {
            const int vt = threadIdx.x + vi * NT;
            const int b = vt >> 1, l = vt & 1;
            C x[RL];
            const C* src = buf + l * RP::LS + (b / RP::BPB) * RP::BS + (b % RP::BPB) * RP::RLP;
#pragma unroll
            for (int t = 0; t < RL; ++t) x[t] = src[t];
            DFT<RL, -1, C>::run(x);
            float4* d4 = reinterpret_cast<float4*>(a.Rbuf + (size_t)ur * a.nstrips * a.pny * 2);
            const size_t rowoff = (size_t)r0 + l;
            if constexpr (RL % 2 == 0) {
#pragma unroll
              for (int f = 0; f < RL; f += 2) {
                const int s2 = (b * RL + f) >> 1;
                d4[(size_t)s2 * a.pny + rowoff] = make_float4(x[f].x, x[f].y, x[f + 1].x, x[f + 1].y);
              }
            } else {
              // odd RL: even b also writes (its last, b+1's first), from lane + 2
              const C nxt0 = make_float2(__shfl_down_sync(0xffffffffu, x[0].x, 2),
                                         __shfl_down_sync(0xffffffffu, x[0].y, 2));
              const int f0 = b & 1;                     // first paired output
#pragma unroll
              for (int f = 0; f + 1 < RL; ++f) {
                if (((f - f0) & 1) == 0 && f >= f0) {
                  const int s2 = (b * RL + f) >> 1;
                  d4[(size_t)s2 * a.pny + rowoff] = make_float4(x[f].x, x[f].y, x[f + 1].x, x[f + 1].y);
                }
              }
              if (f0 == 0) {
                const int s2 = (b * RL + RL - 1) >> 1;
                d4[(size_t)s2 * a.pny + rowoff] = make_float4(x[RL - 1].x, x[RL - 1].y, nxt0.x, nxt0.y);
              }
            }
          }
          __syncthreads();
          continue;
        }
      }
      FastSched<NX>::template run_rest_tab<-1>(buf, kRowPair, Px, 1, tab1, tw, false);
      __syncthreads();
    } else {
      // shifted, zero-padded source lines: a[j] = u[(j - hx) mod Px]
      for (int idx = threadIdx.x; idx < kRowPair * Px; idx += NT) {
        const int l = idx / Px, j = idx - l * Px;
        int x = j - a.hx; if (x < 0) x += Px;
        const int c = x - a.ox;
        C val = mk((R)0, (R)0);
        if (c >= 0 && c < pnx && li[l * lip + c] == u) val = v[l * pnx + c];
        buf[idx] = val;
      }
      block_fft<-1>(buf, kRowPair, Px, 1, a.plx, false);
    }
    // store: strip s holds rows r0, r0+1 contiguously -> 2*W values per strip
    // (W is a power of two: index split with shifts)
    C* dst = a.Rbuf + (size_t)ur * a.nstrips * a.pny * a.W;
    const int W = a.W, lw = a.lw;
    if (sizeof(R) == 4 && W == 2 && nrows == 2 && a.xs) {
      // FP32, strips of two columns, FFT storage order: a thread pair moves
      // one strip's 2 x 2 block (32 contiguous bytes, one full sector), one
      // row each, with 16-byte accesses
      const float4* b4 = reinterpret_cast<const float4*>(buf);
      float4* d4 = reinterpret_cast<float4*>(dst);
      for (int idx = threadIdx.x; idx < Px; idx += NT) {
        const int st = idx >> 1, l = idx & 1;
        d4[(size_t)st * a.pny + r0 + l] = b4[l * (Px / 2) + st];
      }
      __syncthreads();
      continue;
    }
    for (int idx = threadIdx.x; idx < nrows * Px; idx += NT) {
      const int w = idx & (W - 1);
      const int t = idx >> lw;
      const int l = nrows == 2 ? (t & 1) : 0;
      const int s = nrows == 2 ? (t >> 1) : t;
      const int col = (s << lw) + w;                     // strip column
      C val;
      if (a.xs) {
        val = buf[l * Px + col];                         // FFT storage order
      } else {
        int m = col - a.hx; if (m < 0) m += Px;          // S[kx] = A[(kx - hx) mod Px]
        val = buf[l * Px + a.plx.perm[m]];
      }
      dst[((size_t)s * a.pny + r0 + l) * W + w] = val;
    }
    __syncthreads();
  }
}

template <typename R, int NX>
__global__ void __launch_bounds__(512, row_min_blocks<NX>()) dm_row_pass(DMArgs<R> a) {
  dm_row_body<R, NX, 512>(a, blockIdx.x);
}

// Output row yl of a frame (the block's threads stride over the row).
template <typename R, int NX>
__device__ __forceinline__ void dm_out_body(const DMArgs<R>& a, int yl) {
  typedef typename cplx_of<R>::type C;
  extern __shared__ unsigned char smem_raw[];
  C* buf = reinterpret_cast<C*>(smem_raw);
  C* twlo = buf + a.Px;
  C* twhi = twlo + kTwLo;
  const C* row = a.V + (size_t)yl * a.Px;
  if constexpr (NX > 0) load_tw_split(twlo, twhi, static_cast<const C*>(a.plx.tw), NX);
  if constexpr (NX > 0) {
    if (a.xs) {
      // V column p holds spectrum column kx = (iperm[p] + hx) mod Px, whose
      // place in the inverse line is (kx + hx) mod Px = iperm[p]: the row is
      // in the x-FFT's storage order, the input order of the adjoint network
      // (output in natural order)
      for (int p = threadIdx.x; p < NX; p += blockDim.x) buf[p] = row[p];
      FastSched<NX>::run_adj(buf, 1, NX, 1, TwSplit<C>{twlo, twhi}, false);
      __syncthreads();
      for (int c = threadIdx.x; c < a.pnx; c += blockDim.x) {
        int m = a.ox + c - a.hx; if (m < 0) m += NX;
        C h = buf[m];
        if (a.sig_x != 0) h = cmul(h, a.shx[c]);
        a.fringe[(size_t)yl * a.pnx + c] = h.x;
        if (a.field) a.field[(size_t)yl * a.pnx + c] = h;
      }
      return;
    }
  }
  if (a.xs) {
    // V column p holds spectrum column kx = (iperm[p] + hx) mod Px; the
    // inverse line wants it at j = (kx + hx) mod Px
    for (int p = threadIdx.x; p < a.Px; p += blockDim.x) {
      int kx = a.plx.iperm[p] + a.hx; if (kx >= a.Px) kx -= a.Px;
      int j = kx + a.hx; if (j >= a.Px) j -= a.Px;
      buf[j] = row[p];
    }
  } else {
    for (int j = threadIdx.x; j < a.Px; j += blockDim.x) {
      int kx = j - a.hx; if (kx < 0) kx += a.Px;
      buf[j] = row[kx];
    }
  }
  if constexpr (NX > 0) {
    FastSched<NX>::template run_t<1>(buf, 1, a.Px, 1, TwSplit<C>{twlo, twhi}, false);
    __syncthreads();
  } else {
    block_fft<1>(buf, 1, a.Px, 1, a.plx, false);
  }
  for (int c = threadIdx.x; c < a.pnx; c += blockDim.x) {
    int m = a.ox + c - a.hx; if (m < 0) m += a.Px;
    int pm;
    if constexpr (NX > 0) pm = FastSched<NX>::perm(m);
    else pm = a.plx.perm[m];
    C h = buf[pm];
    if (a.sig_x != 0) h = cmul(h, a.shx[c]);
    a.fringe[(size_t)yl * a.pnx + c] = h.x;
    if (a.field) a.field[(size_t)yl * a.pnx + c] = h;
  }
}

template <typename R, int NX>
__global__ void __launch_bounds__(256) dm_out_pass(DMArgs<R> a) {
  dm_out_body<R, NX>(a, blockIdx.x);
}

}  // namespace oh
#include "dm_col_fast.cuh"
