/*
 * CPU oracle for the point-cloud and WRP paths — TEST INFRASTRUCTURE ONLY
 * (used by tests/, __graft_entry__.smoke() and bench.py's CPU baseline; the
 * library never links it).
 *
 * oracle_keti_f32   restates openholo::ophGenCghPointCloud
 *                   (OpenHolo_KETI/VS/Openholo_Generation_PointCloud_Library_beta_v1.0/
 *                    ophgen_pointcloud/ophgen_pointcloud.cpp:195-249) in the same
 *                   float arithmetic and operation order, single-threaded
 *                   (the reference's OpenMP loop races on dst, :221/:241).
 *                   Built with -ffp-contract=off it matches the compiled
 *                   reference bit for bit.
 * oracle_pc_f64     the same geometry in double precision, complex output
 *                   sum_j a_j exp(i phi_j), phi_j = k r_j - k X sin tx - k Y sin ty.
 * oracle_fresnel_f64 paraxial sum of cwoPLS::Fresnel (WRPC/cwo/src/cwoPLS.cpp:370-424)
 *                   with amplitude a_j and the exp(i k z) term.
 * oracle_wrp_f64    OPHWRP::SingleWRP (WRPC/openwrp/WRP.cpp:75-140) in double,
 *                   single-threaded; window half-width from the reference
 *                   formula (fixed_w == 0) or fixed.
 */
#include <math.h>
#include <stdint.h>
#include <string.h>

typedef struct {
  float scale_x, scale_y, scale_z, offset_depth, pitch_x, pitch_y;
  int nx, ny;
  float lambda, tilt_x, tilt_y;
} keti_spec;

void oracle_keti_f32(const float* xyza, int n, const keti_spec* s, float* dst) {
  const int Nx = s->nx, Ny = s->ny;
  float thetaX = s->tilt_x * (M_PI / 180.f);
  float thetaY = s->tilt_y * (M_PI / 180.f);
  float k = (2.f * M_PI) / s->lambda;
  float pixel_x = s->pitch_x, pixel_y = s->pitch_y;
  float Length_x = pixel_x * Nx, Length_y = pixel_y * Ny;
  for (int j = 0; j < n; ++j) {
    float x = xyza[4 * j + 0] * s->scale_x;
    float y = xyza[4 * j + 1] * s->scale_y;
    float z = xyza[4 * j + 2] * s->scale_z + s->offset_depth;
    float amplitude = xyza[4 * j + 3];
    for (int row = 0; row < Ny; ++row) {
      float SLM_y = (Length_y / 2) - ((float)row + 0.5f) * pixel_y;
      for (int col = 0; col < Nx; ++col) {
        float SLM_x = ((float)col + 0.5f) * pixel_x - (Length_x / 2);
        float r = sqrtf((SLM_x - x) * (SLM_x - x) + (SLM_y - y) * (SLM_y - y) + z * z);
        float phi = k * r - k * SLM_x * sinf(thetaX) - k * SLM_y * sinf(thetaY);
        float result = amplitude * cosf(phi);
        dst[col + row * Nx] += result;
      }
    }
  }
}

typedef struct {
  double scale_x, scale_y, scale_z, offset_depth, pitch_x, pitch_y;
  int nx, ny;
  double lambda, tilt_x_deg, tilt_y_deg;
} pc_params;

/* field: interleaved re,im [ny][nx] (overwritten); rows/cols restrict the
 * evaluated region (row0..row0+nrows) for sampled baselines. */
void oracle_pc_f64(const double* xyza, int n, const pc_params* p, double* field, int row0, int nrows) {
  const double k = 2.0 * M_PI / p->lambda;
  const double stx = sin(p->tilt_x_deg * M_PI / 180.0), sty = sin(p->tilt_y_deg * M_PI / 180.0);
  const double hlx = p->pitch_x * p->nx / 2.0, hly = p->pitch_y * p->ny / 2.0;
  for (int row = row0; row < row0 + nrows; ++row) {
    const double Y = hly - ((double)row + 0.5) * p->pitch_y;
    for (int col = 0; col < p->nx; ++col) {
      const double X = ((double)col + 0.5) * p->pitch_x - hlx;
      const double ref = k * X * stx + k * Y * sty;
      double re = 0.0, im = 0.0;
      for (int j = 0; j < n; ++j) {
        const double x = xyza[4 * j] * p->scale_x, y = xyza[4 * j + 1] * p->scale_y;
        const double z = xyza[4 * j + 2] * p->scale_z + p->offset_depth;
        const double dx = X - x, dy = Y - y;
        const double r = sqrt(dx * dx + dy * dy + z * z);
        const double ph = k * r - ref;
        re += xyza[4 * j + 3] * cos(ph);
        im += xyza[4 * j + 3] * sin(ph);
      }
      field[2 * ((size_t)row * p->nx + col)] = re;
      field[2 * ((size_t)row * p->nx + col) + 1] = im;
    }
  }
}

/* cwoPLS::Fresnel geometry: pixel (i,j) at ((j - Nx/2) dp, (i - Ny/2) dp),
 * phase k ((dx^2+dy^2)/(2 dz)) + k dz, amplitude a_j. */
void oracle_fresnel_f64(const double* xyza, int n, int nx, int ny, double dp, double lambda, double* field) {
  const double k = 2.0 * M_PI / lambda;
  for (int i = 0; i < ny; ++i)
    for (int j = 0; j < nx; ++j) {
      double re = 0.0, im = 0.0;
      for (int q = 0; q < n; ++q) {
        const double dx = (double)(j - nx / 2) * dp - xyza[4 * q];
        const double dy = (double)(i - ny / 2) * dp - xyza[4 * q + 1];
        const double dz = xyza[4 * q + 2];
        const double ph = k * ((dx * dx + dy * dy) / (2.0 * dz)) + k * dz;
        re += xyza[4 * q + 3] * cos(ph);
        im += xyza[4 * q + 3] * sin(ph);
      }
      field[2 * ((size_t)i * nx + j)] = re;
      field[2 * ((size_t)i * nx + j) + 1] = im;
    }
}

/* SingleWRP: wrp interleaved re,im [ny][nx], accumulated.  The wave number
 * is the float GetWaveNum() of the reference (WRP.cpp:78); the window size
 * uses the reference's float expression (WRP.cpp:110-112). */
void oracle_wrp_f64(const double* xyz, int n, int nx, int ny, double dp, double lambda, double z, int fixed_w,
                    double* wrp) {
  const float wl = (float)lambda, dpx = (float)dp;
  const double wn = (double)(float)(2.0 * M_PI / lambda);
  const int nxh = nx >> 1, nyh = ny >> 1;
  for (int q = 0; q < n; ++q) {
    const float dzf = (float)((double)(float)z - xyz[3 * q + 2]);
    int w;
    if (fixed_w > 0) w = fixed_w;
    else {
      float tw = (float)(int)fabsf(wl * dzf / dpx / dpx / 2 + 0.5f) * 2 - 1;
      w = (int)tw;
    }
    const int tx = (int)(xyz[3 * q] / (double)dpx) + nxh;
    const int ty = (int)(xyz[3 * q + 1] / (double)dpx) + nyh;
    const double dz = (double)(float)z - xyz[3 * q + 2];
    const double sign = dz > 0.0 ? 1.0 : -1.0;
    for (int wy = -w; wy < w; ++wy)
      for (int wx = -w; wx < w; ++wx) {
        const int X = tx + wx, Y = ty + wy;
        if (X < 0 || X >= nx || Y < 0 || Y >= ny) continue;
        const double ddx = wx * (double)dpx, ddy = wy * (double)dpx;
        const double r = sign * sqrt(ddx * ddx + ddy * ddy + dz * dz);
        wrp[2 * ((size_t)Y * nx + X)] += cos(wn * r) / (r + 0.05);
        wrp[2 * ((size_t)Y * nx + X) + 1] += sin(wn * r) / (r + 0.05);
      }
  }
}
