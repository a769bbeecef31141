// C++ drop-in for the KETI point-cloud library (include/oh_openholo_pointcloud.hpp).
// Loaders parse the reference's formats (ophgen_pointcloud.cpp:13-162):
//   .dat     first line N, then N lines "idx x y z phase amplitude", idx == line
//   .config  exactly 17 "title = value" lines in OphSpec order
// Generation runs on the GPU through oh_pointcloud_host (FP32 path).
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>
#include "../../include/oh.h"
#include "../../include/oh_openholo_pointcloud.hpp"

namespace {

std::mutex g_mu;
oh_ctx* g_ctx = nullptr;

oh_ctx* default_ctx() {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_ctx && oh_ctx_create(&g_ctx, 0) != OH_OK) g_ctx = nullptr;
  return g_ctx;
}

template <typename Fn>
int parse_dat(const char* path, Fn&& add) {
  FILE* f = std::fopen(path, "r");
  if (!f) return -1;
  int n = 0;
  if (std::fscanf(f, "%d", &n) != 1 || n < 0) { std::fclose(f); return -1; }
  for (int i = 0; i < n; ++i) {
    int idx;
    float x, y, z, ph, amp;
    if (std::fscanf(f, "%d %f %f %f %f %f", &idx, &x, &y, &z, &ph, &amp) != 6 || idx != i) { std::fclose(f); return -1; }
    add(x, y, z, amp, ph);
  }
  std::fclose(f);
  return n;
}

double run(const float* xyza, int n, const openholo::OphSpec& c, float* dst) {
  auto t0 = std::chrono::steady_clock::now();
  oh_pc_params p;
  p.scale_x = c.pointCloudScaleX; p.scale_y = c.pointCloudScaleY; p.scale_z = c.pointCloudScaleZ;
  p.offset_depth = c.offsetDepth;
  p.pitch_x = c.samplingPitchX; p.pitch_y = c.samplingPitchY;
  p.nx = c.nx; p.ny = c.ny;
  p.lambda = c.lambda;
  p.tilt_x_deg = c.tiltAngleX; p.tilt_y_deg = c.tiltAngleY;
  oh_ctx* ctx = default_ctx();
  if (!ctx || oh_pointcloud_host(ctx, OH_FP32, &p, xyza, n, nullptr, dst, nullptr) != OH_OK) return -1.0;
  return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

}  // namespace

namespace openholo {

int ophLoadPointCloud(char* inputData, OphPointCloud*& model) {
  std::vector<OphPointCloud> v;
  int n = ophLoadPointCloud(std::string(inputData ? inputData : ""), v);
  if (n < 0) return -1;
  model = (OphPointCloud*)std::malloc(sizeof(OphPointCloud) * (n > 0 ? n : 1));
  if (!model) return -1;
  for (int i = 0; i < n; ++i) model[i] = v[i];
  return n;
}

int ophLoadPointCloud(const std::string inputData, std::vector<OphPointCloud>& model) {
  return parse_dat(inputData.c_str(), [&](float x, float y, float z, float a, float ph) {
    model.push_back(OphPointCloud(x, y, z, a, ph));
  });
}

int ophLoadPointCloud(const std::string inputData, std::vector<float>& vertexArray, std::vector<float>& phaseArray,
                      std::vector<float>& amplitudeArray) {
  return parse_dat(inputData.c_str(), [&](float x, float y, float z, float a, float ph) {
    vertexArray.push_back(x); vertexArray.push_back(y); vertexArray.push_back(z);
    phaseArray.push_back(ph);
    amplitudeArray.push_back(a);
  });
}

bool ophLoadSpecConfig(char* inputData, OphSpec* config) {
  if (!inputData || !config) return false;
  FILE* f = std::fopen(inputData, "r");
  if (!f) return false;
  std::vector<std::string> values;
  char line[256];
  while (std::fgets(line, sizeof(line), f)) {
    char title[128], value[128];
    if (std::sscanf(line, "%127s = %127s", title, value) == 2) values.push_back(value);
    else values.push_back("");
  }
  std::fclose(f);
  if (values.size() != 17) return false;
  config->pointCloudScaleX = (float)std::atof(values[0].c_str());
  config->pointCloudScaleY = (float)std::atof(values[1].c_str());
  config->pointCloudScaleZ = (float)std::atof(values[2].c_str());
  config->offsetDepth = (float)std::atof(values[3].c_str());
  config->samplingPitchX = (float)std::atof(values[4].c_str());
  config->samplingPitchY = (float)std::atof(values[5].c_str());
  config->nx = std::atoi(values[6].c_str());
  config->ny = std::atoi(values[7].c_str());
  static thread_local std::string shape;
  shape = values[8];
  config->filterShapeFlag = &shape[0];
  config->filterXwidth = (float)std::atof(values[9].c_str());
  config->filterYwidth = (float)std::atof(values[10].c_str());
  config->focalLengthLensIn = (float)std::atof(values[11].c_str());
  config->focalLengthLensOut = (float)std::atof(values[12].c_str());
  config->focalLengthLenEyepiece = (float)std::atof(values[13].c_str());
  config->lambda = (float)std::atof(values[14].c_str());
  config->tiltAngleX = (float)std::atof(values[15].c_str());
  config->tiltAngleY = (float)std::atof(values[16].c_str());
  return true;
}

bool ophLoadSpecConfig(const std::string inputData, OphSpec& config) {
  return ophLoadSpecConfig(const_cast<char*>(inputData.c_str()), &config);
}

void ophSetScaleFactor(OphSpec& c, const float sx, const float sy, const float sz) {
  c.pointCloudScaleX = sx; c.pointCloudScaleY = sy; c.pointCloudScaleZ = sz;
}
void ophSetOffsetDepth(OphSpec& c, const float d) { c.offsetDepth = d; }
void ophSetSamplingPitch(OphSpec& c, const float px, const float py) { c.samplingPitchX = px; c.samplingPitchY = py; }
void ophSetImageSize(OphSpec& c, const int nx, const int ny) { c.nx = nx; c.ny = ny; }
void ophSetWaveLength(OphSpec& c, const float l) { c.lambda = l; }
void ophSetTiltAngle(OphSpec& c, const float tx, const float ty) { c.tiltAngleX = tx; c.tiltAngleY = ty; }

double ophGenCghPointCloud(const OphPointCloud* model, const int n_points, const OphSpec& config, float* dst) {
  std::vector<float> xyza((size_t)n_points * 4);
  for (int i = 0; i < n_points; ++i) {
    xyza[4 * i] = model[i].x; xyza[4 * i + 1] = model[i].y; xyza[4 * i + 2] = model[i].z;
    xyza[4 * i + 3] = model[i].amplitude;
  }
  return run(xyza.data(), n_points, config, dst);
}

double ophGenCghPointCloud(const std::vector<OphPointCloud>& model, const OphSpec& config, float* dst) {
  return ophGenCghPointCloud(model.data(), (int)model.size(), config, dst);
}

double ophGenCghPointCloud(const std::vector<float>& vertexArray, const std::vector<float>& amplitudeArray,
                           const OphSpec& config, float* dst) {
  const int n = (int)(vertexArray.size() / 3);
  std::vector<float> xyza((size_t)n * 4);
  for (int i = 0; i < n; ++i) {
    xyza[4 * i] = vertexArray[3 * i]; xyza[4 * i + 1] = vertexArray[3 * i + 1]; xyza[4 * i + 2] = vertexArray[3 * i + 2];
    xyza[4 * i + 3] = i < (int)amplitudeArray.size() ? amplitudeArray[i] : 0.f;
  }
  return run(xyza.data(), n, config, dst);
}

namespace gpu {
double ophGenCghPointCloud_cuda(const std::vector<float>& vertexArray, const std::vector<float>& amplitudeArray,
                                const OphSpec& config, float* dst) {
  return openholo::ophGenCghPointCloud(vertexArray, amplitudeArray, config, dst);
}
}  // namespace gpu

void ophSaveFileBmp(unsigned char* pixelbuffer, int w, int h, char* file_name) {
  if (!pixelbuffer || !file_name || w <= 0 || h <= 0) return;
  const int stride = (w + 3) & ~3;
  const unsigned palette = 256 * 4, hdr = 14 + 40;
  const unsigned offset = hdr + palette, image = (unsigned)stride * h;
  unsigned char fh[14] = {'B', 'M'};
  auto put32 = [](unsigned char* p, unsigned v) { p[0] = v & 255; p[1] = (v >> 8) & 255; p[2] = (v >> 16) & 255; p[3] = v >> 24; };
  auto put16 = [](unsigned char* p, unsigned v) { p[0] = v & 255; p[1] = (v >> 8) & 255; };
  put32(fh + 2, offset + image);
  put32(fh + 10, offset);
  unsigned char ih[40] = {0};
  put32(ih, 40); put32(ih + 4, (unsigned)w); put32(ih + 8, (unsigned)h);
  put16(ih + 12, 1); put16(ih + 14, 8); put32(ih + 20, image);
  put32(ih + 24, 2835); put32(ih + 28, 2835); put32(ih + 32, 256);
  std::string name = std::string(file_name) + ".bmp";
  FILE* f = std::fopen(name.c_str(), "wb");
  if (!f) return;
  std::fwrite(fh, 1, 14, f);
  std::fwrite(ih, 1, 40, f);
  for (int i = 0; i < 256; ++i) { unsigned char q[4] = {(unsigned char)i, (unsigned char)i, (unsigned char)i, 0}; std::fwrite(q, 1, 4, f); }
  std::vector<unsigned char> row(stride, 0);
  for (int r = 0; r < h; ++r) {
    std::memcpy(row.data(), pixelbuffer + (size_t)r * w, w);
    std::fwrite(row.data(), 1, stride, f);
  }
  std::fclose(f);
}

void ophNormalize(float* src, unsigned char* dst, const int nx, const int ny) {
  if (!src || !dst || nx <= 0 || ny <= 0) return;
  float mn = src[0], mx = src[0];
  for (long i = 0; i < (long)nx * ny; ++i) { mn = src[i] < mn ? src[i] : mn; mx = src[i] > mx ? src[i] : mx; }
  for (int y = 0; y < ny; ++y)
    for (int x = 0; x < nx; ++x) {
      float v = ((src[x + (long)y * nx] - mn) / (mx - mn)) * 255 + 0.5f;
      dst[x + (long)(ny - y - 1) * nx] = (unsigned char)v;
    }
}

}  // namespace openholo
