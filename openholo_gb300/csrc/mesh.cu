// Triangle-mesh CGH by analytic angular spectra (OpenHolo_MeshCGH):
// fn_genH.m:1-53 sums, over the frequency grid fx = -(m - Nx/2) / (Nx dx),
// fy = (r - Ny/2) / (Ny dy), fz = sqrt(1/lambda^2 - fx^2 - fy^2), the
// angular spectrum of every front-facing triangle, then takes
// fftshift(fft2(fftshift(.))).  Per triangle (fn_AS_shading.m, flat shading;
// fn_AS_continuous.m with fn_FindVertexNormalVector.m, continuous shading):
// rotate the frequencies into the triangle's plane (R from the normal), map
// the triangle to the reference triangle (0,0), (1,1), (1,0) (affine A),
// evaluate the reference triangle's analytic spectrum G0 at
// (inv(A') (fl - du)), with the source's special cases where a coordinate is
// exactly zero, and carry it back: G = J G0 e^{-i 2 pi (R'c)_3 / lambda}
// (flz / fz) e^{i 2 pi (flx c1 + fly c2 + flz c3)}, times 2 s + 0.1 (flat).
//
// The per-triangle set-up (normal, rotation, shift c, A, inv(A'), constants,
// illumination) runs on the host in FP64, in the operation order of the
// source.  The GPU evaluates the per-sample sums in FP64 (the phases reach
// ~1e5 turns and are reduced in turns before the sine and cosine).  The
// quantities that feed the source's exact-zero tests (fx, fy, fz, flx, fly,
// flux, fluy, inv(A') products) are formed with explicit round-to-nearest
// multiplies and adds in the source's order, so no fused multiply-add moves
// a sample into or out of a special case.
#include <cmath>
#include <vector>
#include "context.h"
#include "fft_kernels.cuh"

namespace oh {

namespace {

struct MeshTri {
  double R[6];          // rows 1 and 2 of the rotation
  double du1, du2;      // (1/lambda) (R13, R23)
  double tA[4];         // inv(A') row-major
  double c[3];          // local shift
  double gre, gim;      // J exp(-i 2 pi (R'c)_3 / lambda), J = 1/det(A)
  double wflat;         // flat: 2 s + 0.1; continuous: unused
  double a1, a2, a3;    // continuous: vertex illumination terms
};
constexpr int kTriDoubles = (int)(sizeof(MeshTri) / sizeof(double));
constexpr int kMeshChunk = 32;

struct MeshGeom { int nx, ny; double dfx, dfy, il2; int continuous; };

__device__ __forceinline__ double2 cd(double re, double im) { return make_double2(re, im); }
__device__ __forceinline__ double2 cm(double2 a, double2 b) { return cd(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
__device__ __forceinline__ double2 cdv(double2 a, double2 b) {
  const double den = b.x * b.x + b.y * b.y;
  return cd((a.x * b.x + a.y * b.y) / den, (a.y * b.x - a.x * b.y) / den);
}
__device__ __forceinline__ double2 cs(double2 a, double s) { return cd(a.x * s, a.y * s); }
__device__ __forceinline__ double2 ca(double2 a, double2 b) { return cd(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 cb(double2 a, double2 b) { return cd(a.x - b.x, a.y - b.y); }
// exp(-i 2 pi x), x in turns
__device__ __forceinline__ double2 em(double x) {
  const double t = x - rint(x);
  double s, c;
  sincospi(2.0 * t, &s, &c);
  return cd(c, -s);
}
__device__ __forceinline__ double2 csqrt_re(double q) { return q >= 0.0 ? cd(__dsqrt_rn(q), 0.0) : cd(0.0, __dsqrt_rn(-q)); }

__device__ __forceinline__ double2 g0_flat(double fa, double fb) {
  const double tp = 6.283185307179586476925286766559, tp2 = tp * tp;
  const double2 one = cd(1.0, 0.0);
  if (fa == fb && fa == 0.0) return cd(0.5, 0.0);
  if (fa == 0.0 && fb != 0.0) {
    const double2 a = cs(cb(one, em(fb)), 1.0 / ((tp * fb) * (tp * fb)));
    return cb(a, cd(0.0, 1.0 / (tp * fb)));
  }
  if (fa != 0.0 && fb == 0.0) {
    const double2 e = em(fa);
    return ca(cs(cb(e, one), 1.0 / ((tp * fa) * (tp * fa))), cs(cm(cd(0.0, 1.0), e), 1.0 / (tp * fa)));
  }
  if (fa == -fb && fb != 0.0) {
    const double2 ep = cd(em(fb).x, -em(fb).y);      // exp(+i 2 pi fb)
    return ca(cs(cb(one, ep), 1.0 / ((tp * fb) * (tp * fb))), cd(0.0, 1.0 / (tp * fb)));
  }
  const double2 a = cs(cb(em(fa), one), 1.0 / (tp2 * fa * fb));
  const double2 b = cs(cb(one, em(fa + fb)), 1.0 / (tp2 * fb * (fa + fb)));
  return ca(a, b);
}

__device__ __forceinline__ double2 g0_cont(double fa, double fb, double a1, double a2, double a3) {
  const double p = 3.14159265358979323846264338327950, p2 = p * p, p3 = p2 * p;
  const double2 I = cd(0.0, 1.0);
  double2 D1, D2, D3;
  if (fa == 0.0 && fb == 0.0) {
    D1 = cd(1.0 / 3.0, 0.0); D2 = cd(1.0 / 6.0, 0.0); D3 = cd(0.5, 0.0);
  } else if (fa == 0.0 && fb != 0.0) {
    const double y = fb, y3 = 8.0 * p3 * y * y * y, q3 = 4.0 * p3 * y * y * y;
    const double2 ey = em(y);
    D1 = ca(cs(ey, -(2.0 * p * y + 1.0) / y3), cs(cd(1.0, -2.0 * p2 * y * y), 1.0 / y3));
    D2 = cb(cs(cm(cd(-p * y, 1.0), ey), 1.0 / q3), cs(cd(p * y, 1.0), 1.0 / q3));
    D3 = ca(cs(ey, 1.0 / (2.0 * p * y)), cs(cd(1.0, -1.0), 1.0 / (2.0 * p * y)));
  } else if (fa != 0.0 && fb == 0.0) {
    const double x = fa, x3 = 8.0 * p3 * x * x * x;
    const double2 ex = em(x);
    D1 = ca(cs(cm(cd(4.0 * p * x, 4.0 * p2 * x * x - 2.0), ex), 1.0 / x3), cd(0.0, 1.0 / (4.0 * p3 * x * x * x)));
    D2 = cs(D1, 0.5);
    D3 = cs(cb(cm(cd(1.0, 2.0 * p * x), ex), cd(1.0, 0.0)), 1.0 / (4.0 * p2 * x * x));
  } else if (fa == -fb) {
    const double x = fa, x3 = 8.0 * p3 * x * x * x;
    const double2 ex = em(x);
    D1 = cb(cs(cm(cd(-2.0 * p * x, 1.0), ex), 1.0 / x3), cs(cd(0.0, 2.0 * p2 * x * x + 1.0), 1.0 / x3));
    D2 = ca(cs(cm(cd(0.0, -1.0), ex), 1.0 / x3), cs(cd(2.0 * p * x, -2.0 * p2 * x * x + 1.0), 1.0 / x3));
    D3 = ca(cs(cm(cd(0.0, -1.0), ex), 1.0 / (4.0 * p2 * x * x)), cs(cd(1.0, -2.0 * p * x), 1.0 / (4.0 * p2 * x * x)));
  } else {
    const double s = fa + fb;
    const double2 eab = em(s), ea = em(fa);
    D1 = ca(ca(cs(cm(eab, cb(I, cd(2.0 * p * s, 0.0))), 1.0 / (8.0 * p3 * fb * s * s)),
               cs(cm(ea, cd(2.0 * p * fa, -1.0)), 1.0 / (8.0 * p3 * fa * fa * fb))),
            cd(0.0, (2.0 * fa + fb) / (8.0 * p3 * fa * fa * s * s)));
    D2 = ca(ca(cs(cm(eab, cd(-2.0 * p * fb * s, fa + 2.0 * fb)), 1.0 / (8.0 * p3 * fb * fb * s * s)),
               cs(cm(ea, cd(0.0, -1.0)), 1.0 / (8.0 * p3 * fa * fb * fb))),
            cd(0.0, 1.0 / (8.0 * p3 * fa * s * s)));
    D3 = cb(ca(cs(eab, -1.0 / (4.0 * p2 * fb * s)), cs(ea, 1.0 / (4.0 * p2 * fa * fb))),
            cd(1.0 / (4.0 * p2 * fa * s), 0.0));
  }
  return ca(ca(cs(D1, a2 - a1), cs(D2, a3 - a2)), cs(D3, a1));
}

__global__ void __launch_bounds__(256) mesh_spectrum(MeshGeom g, const double* __restrict__ tris, int n,
                                                    double2* __restrict__ gg) {
  __shared__ double sT[kMeshChunk * kTriDoubles];
  const size_t tot = (size_t)g.nx * g.ny;
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  const bool live = i < tot;
  const int r = live ? (int)(i / g.nx) : 0, m = live ? (int)(i - (size_t)r * g.nx) : 0;
  // fx = -(m - nx/2) dfx, fy = (r - ny/2) dfy, fz = sqrt((1/lambda)^2 - fx^2 - fy^2)
  const double fx = __dmul_rn(-((double)m - (double)g.nx / 2.0), g.dfx);
  const double fy = __dmul_rn((double)r - (double)g.ny / 2.0, g.dfy);
  const double fz = __dsqrt_rn(__dsub_rn(__dsub_rn(g.il2, __dmul_rn(fx, fx)), __dmul_rn(fy, fy)));
  double2 acc = cd(0.0, 0.0);
  for (int t0 = 0; t0 < n; t0 += kMeshChunk) {
    const int cnt = min(kMeshChunk, n - t0);
    __syncthreads();
    for (int e = threadIdx.x; e < cnt * kTriDoubles; e += blockDim.x) sT[e] = tris[(size_t)t0 * kTriDoubles + e];
    __syncthreads();
    if (!live) continue;
    for (int k = 0; k < cnt; ++k) {
      const MeshTri& T = *reinterpret_cast<const MeshTri*>(sT + k * kTriDoubles);
      const double flx = __dadd_rn(__dadd_rn(__dmul_rn(T.R[0], fx), __dmul_rn(T.R[1], fy)), __dmul_rn(T.R[2], fz));
      const double fly = __dadd_rn(__dadd_rn(__dmul_rn(T.R[3], fx), __dmul_rn(T.R[4], fy)), __dmul_rn(T.R[5], fz));
      const double2 flz = csqrt_re(__dsub_rn(__dsub_rn(g.il2, __dmul_rn(flx, flx)), __dmul_rn(fly, fly)));
      const double flux = __dsub_rn(flx, T.du1), fluy = __dsub_rn(fly, T.du2);
      const double fa = __dadd_rn(__dmul_rn(T.tA[0], flux), __dmul_rn(T.tA[1], fluy));
      const double fb = __dadd_rn(__dmul_rn(T.tA[2], flux), __dmul_rn(T.tA[3], fluy));
      double2 G0 = g.continuous ? g0_cont(fa, fb, T.a1, T.a2, T.a3) : g0_flat(fa, fb);
      if (!g.continuous) G0 = cs(G0, T.wflat);
      const double2 Gl = cm(G0, cd(T.gre, T.gim));
      // exp(i 2 pi (flx c1 + fly c2 + flz c3)), flz possibly complex
      const double tre = flx * T.c[0] + fly * T.c[1] + flz.x * T.c[2];
      const double2 ph = cs(cd(em(tre).x, -em(tre).y), exp(-6.283185307179586476925286766559 * flz.y * T.c[2]));
      acc = ca(acc, cm(cm(Gl, cs(flz, 1.0 / fz)), ph));
    }
  }
  if (live) gg[i] = acc;
}

// host-side per-triangle set-up, in the operation order of the source
struct V3 { double x, y, z; };
static V3 sub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
static V3 cross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }

static bool setup_triangle(const double* v, V3 n, bool normalise, double lambda, const double* illu, bool continuous,
                           const double* nvrow, MeshTri* out) {
  if (!(n.z > 0)) return false;
  if (normalise) {
    const double nn = std::sqrt(n.x * n.x + n.y * n.y + n.z * n.z);
    n = {n.x / nn, n.y / nn, n.z / nn};
  }
  const double th = (n.x == 0 && n.z == 0) ? 0.0 : std::atan(n.x / n.z);
  const double ph = std::atan(n.y / std::sqrt(n.x * n.x + n.z * n.z));
  const double R[3][3] = {{std::cos(th), 0.0, -std::sin(th)},
                          {-std::sin(ph) * std::sin(th), std::cos(ph), -std::cos(th) * std::sin(ph)},
                          {std::cos(ph) * std::sin(th), std::sin(ph), std::cos(ph) * std::cos(th)}};
  double Xl[3][3];   // Xl[row][vertex] = R X
  for (int a = 0; a < 3; ++a)
    for (int k = 0; k < 3; ++k) Xl[a][k] = R[a][0] * v[3 * k] + R[a][1] * v[3 * k + 1] + R[a][2] * v[3 * k + 2];
  const double c[3] = {-Xl[0][0], -Xl[1][0], -Xl[2][0]};
  for (int a = 0; a < 3; ++a)
    for (int k = 0; k < 3; ++k) Xl[a][k] += c[a];
  if (Xl[0][2] * Xl[1][1] == Xl[1][2] * Xl[0][1]) return false;
  // Xld = Xl(1:2,:)' : Xld[vertex][coord]
  const double Xld[3][2] = {{Xl[0][0], Xl[1][0]}, {Xl[0][1], Xl[1][1]}, {Xl[0][2], Xl[1][2]}};
  const double b = Xld[2][0] * Xld[1][1] - Xld[2][1] * Xld[1][0];
  const double ref[3][2] = {{0.0, 0.0}, {1.0, 1.0}, {1.0, 0.0}};
  double A[2][2];
  for (int l = 0; l < 2; ++l)
    for (int m = 0; m < 2; ++m) A[l][m] = (ref[2][l] * Xld[1][1 - m] - ref[1][l] * Xld[2][1 - m]) / (b * ((m % 2) ? -1.0 : 1.0));
  // tA = inv(A'), closed form
  const double At[2][2] = {{A[0][0], A[1][0]}, {A[0][1], A[1][1]}};
  const double det = At[0][0] * At[1][1] - At[0][1] * At[1][0];
  out->tA[0] = At[1][1] / det; out->tA[1] = -At[0][1] / det;
  out->tA[2] = -At[1][0] / det; out->tA[3] = At[0][0] / det;
  for (int k = 0; k < 3; ++k) { out->R[k] = R[0][k]; out->R[3 + k] = R[1][k]; }
  out->du1 = (1.0 / lambda) * R[0][2];
  out->du2 = (1.0 / lambda) * R[1][2];
  for (int k = 0; k < 3; ++k) out->c[k] = c[k];
  const double J = 1.0 / (A[0][0] * A[1][1] - A[0][1] * A[1][0]);
  const double rc3 = R[0][2] * c[0] + R[1][2] * c[1] + R[2][2] * c[2];   // (R'c)_3
  const double t = rc3 / lambda;
  const double red = t - std::rint(t);
  out->gre = J * std::cos(-2.0 * M_PI * red);
  out->gim = J * std::sin(-2.0 * M_PI * red);
  if (!continuous) {
    double s = 1.0;
    if (!(illu[0] == 0 && illu[1] == 0 && illu[2] == 0)) {
      const double ni = std::sqrt(illu[0] * illu[0] + illu[1] * illu[1] + illu[2] * illu[2]);
      s = n.x * (illu[0] / ni) + n.y * (illu[1] / ni) + n.z * (illu[2] / ni);
      if (s < 0) s = 0;
    }
    out->wflat = 2.0 * s + 0.1;
    out->a1 = out->a2 = out->a3 = 0.0;
  } else {
    double av[3];
    for (int k = 0; k < 3; ++k) {
      av[k] = nvrow[3 * k] * illu[0] + nvrow[3 * k + 1] * illu[1] + nvrow[3 * k + 2] * illu[2] + 0.1;
      if (av[k] < 0) av[k] = 0;
    }
    out->a1 = av[0]; out->a2 = av[2]; out->a3 = av[1];
    out->wflat = 1.0;
  }
  return true;
}

// fn_FindVertexNormalVector: face normals (unnormalised: a common positive
// scale, which no later use depends on) and per-vertex averages over the
// triangles sharing the exact vertex; a vertex at the origin keeps a zero
// normal, as the source marks visited rows by zeroing them.
static void vertex_normals(const double* tris, int n, std::vector<V3>& na, std::vector<double>& nv) {
  na.resize(n);
  for (int i = 0; i < n; ++i) {
    const double* v = tris + 9 * (size_t)i;
    na[i] = cross(sub({v[0], v[1], v[2]}, {v[3], v[4], v[5]}), sub({v[6], v[7], v[8]}, {v[3], v[4], v[5]}));
  }
  std::vector<double> objv(tris, tris + 9 * (size_t)n);
  nv.assign(9 * (size_t)n, 0.0);
  const int nvx = 3 * n;
  for (int i = 0; i < nvx; ++i) {
    const double x = objv[3 * i], y = objv[3 * i + 1], z = objv[3 * i + 2];
    if (x == 0 && y == 0 && z == 0) continue;
    std::vector<int> idx;
    for (int j = 0; j < nvx; ++j)
      if (objv[3 * j] == x && objv[3 * j + 1] == y && objv[3 * j + 2] == z) idx.push_back(j);
    V3 s{0, 0, 0};
    for (int j : idx) {
      s.x += na[j / 3].x; s.y += na[j / 3].y; s.z += na[j / 3].z;
      objv[3 * j] = objv[3 * j + 1] = objv[3 * j + 2] = 0.0;
    }
    const double cnt = (double)idx.size();
    V3 avg{s.x / cnt, s.y / cnt, s.z / cnt};
    const double nn = std::sqrt(avg.x * avg.x + avg.y * avg.y + avg.z * avg.z);
    avg = {avg.x / nn, avg.y / nn, avg.z / nn};
    for (int j : idx) { nv[3 * j] = avg.x; nv[3 * j + 1] = avg.y; nv[3 * j + 2] = avg.z; }
  }
}

}  // namespace

}  // namespace oh

using namespace oh;

extern "C" oh_status oh_mesh_hologram(oh_ctx* ctx, const oh_mesh_params* p, const double* tris, int n_tris,
                                      void* field, void* spectrum, void* stream) {
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  CallScope cs(ctx, st);
  OH_TRY(cs.status());
  if (!p || p->nx < 1 || p->ny < 1 || !(p->dx > 0) || !(p->dy > 0) || !(p->lambda > 0))
    return fail(OH_ERR_INVALID_ARG, "bad mesh-hologram parameters");
  if (!(p->dx > p->lambda) || !(p->dy > p->lambda))
    return fail(OH_ERR_UNSUPPORTED_SIZE, "pitch must exceed the wavelength (no evanescent hologram-plane samples)");
  if (n_tris < 0 || (n_tris > 0 && !tris) || !field) return fail(OH_ERR_INVALID_ARG, "bad mesh buffers");
  const bool cont = p->continuous != 0;
  std::vector<V3> na;
  std::vector<double> nv;
  if (cont) vertex_normals(tris, n_tris, na, nv);
  std::vector<MeshTri> prep;
  prep.reserve((size_t)n_tris);
  for (int i = 0; i < n_tris; ++i) {
    const double* v = tris + 9 * (size_t)i;
    V3 nrm;
    if (cont) nrm = na[i];
    else nrm = cross(sub({v[3], v[4], v[5]}, {v[6], v[7], v[8]}), sub({v[0], v[1], v[2]}, {v[6], v[7], v[8]}));
    MeshTri t;
    if (setup_triangle(v, nrm, !cont, p->lambda, p->illu, cont, cont ? nv.data() + 9 * (size_t)i : nullptr, &t))
      prep.push_back(t);
  }
  const size_t npx = (size_t)p->nx * p->ny;
  double2* gg = static_cast<double2*>(spectrum ? spectrum : field);
  const int n = (int)prep.size();
  if (n > 0) {
    void* tp;
    OH_TRY(scratch(ctx, "mesh.tris", prep.size() * sizeof(MeshTri), &tp));
    OH_CUDA_TRY(cudaMemcpyAsync(tp, prep.data(), prep.size() * sizeof(MeshTri), cudaMemcpyHostToDevice, st));
    MeshGeom g{p->nx, p->ny, (1.0 / p->dx) / p->nx, (1.0 / p->dy) / p->ny, (1.0 / p->lambda) * (1.0 / p->lambda),
               cont ? 1 : 0};
    KernelTimer kt(ctx, "mesh_spectrum", st);
    mesh_spectrum<<<(unsigned)((npx + 255) / 256), 256, 0, st>>>(g, static_cast<const double*>(tp), n, gg);
    OH_LAUNCH_CHECK();
    OH_CUDA_TRY(cudaStreamSynchronize(st));     // the host staging vector is released on return
  } else {
    OH_CUDA_TRY(cudaMemsetAsync(gg, 0, npx * sizeof(double2), st));
  }
  if (spectrum) OH_CUDA_TRY(cudaMemcpyAsync(field, spectrum, npx * sizeof(double2), cudaMemcpyDeviceToDevice, st));
  // fftshift(fft2(fftshift(.))): the centred transform of the FFT engine
  return fft2d_enqueue(ctx, 1, p->nx, p->ny, field, field, nullptr, -1, 1, 0, st);
}
