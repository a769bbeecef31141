// C entry points around the reference's own point-cloud routines, compiled
// together with the reference source file
//   OpenHolo_KETI/VS/Openholo_Generation_PointCloud_Library_beta_v1.0/ophgen_pointcloud/ophgen_pointcloud.cpp
// by oracle/build.py into oracle/_ref/.  Test infrastructure only: it is used
// to pin the oracle restatement and as the reference CPU baseline.
#include <vector>
#include "ophgen_pointcloud.h"

extern "C" {

// xyza: n x {x, y, z, amplitude}; spec fields in OphSpec order.  Returns the
// reference's own elapsed-seconds value.
double keti_ref_gen(const float* xyza, int n, const float* spec11, int nx, int ny, float* dst) {
  std::vector<openholo::OphPointCloud> model;
  model.reserve(n);
  for (int i = 0; i < n; ++i)
    model.push_back(openholo::OphPointCloud(xyza[4 * i], xyza[4 * i + 1], xyza[4 * i + 2], xyza[4 * i + 3], 0.f));
  openholo::OphSpec cfg;
  cfg.pointCloudScaleX = spec11[0];
  cfg.pointCloudScaleY = spec11[1];
  cfg.pointCloudScaleZ = spec11[2];
  cfg.offsetDepth = spec11[3];
  cfg.samplingPitchX = spec11[4];
  cfg.samplingPitchY = spec11[5];
  cfg.nx = nx;
  cfg.ny = ny;
  cfg.filterShapeFlag = nullptr;
  cfg.filterXwidth = cfg.filterYwidth = 0.f;
  cfg.focalLengthLensIn = cfg.focalLengthLensOut = cfg.focalLengthLenEyepiece = 0.f;
  cfg.lambda = spec11[6];
  cfg.tiltAngleX = spec11[7];
  cfg.tiltAngleY = spec11[8];
  return openholo::ophGenCghPointCloud(model.data(), n, cfg, dst);
}

// The reference's own loaders, for the .dat / .config fixtures.
int keti_ref_load_points(const char* path, float* xyzpa, int cap) {
  std::vector<openholo::OphPointCloud> model;
  int n = openholo::ophLoadPointCloud(std::string(path), model);
  if (n < 0) return n;
  for (int i = 0; i < n && i < cap; ++i) {
    xyzpa[5 * i] = model[i].x; xyzpa[5 * i + 1] = model[i].y; xyzpa[5 * i + 2] = model[i].z;
    xyzpa[5 * i + 3] = model[i].phase; xyzpa[5 * i + 4] = model[i].amplitude;
  }
  return n;
}

int keti_ref_load_spec(const char* path, float* out11, int* nxny) {
  openholo::OphSpec cfg;
  if (!openholo::ophLoadSpecConfig(std::string(path), cfg)) return 0;
  out11[0] = cfg.pointCloudScaleX; out11[1] = cfg.pointCloudScaleY; out11[2] = cfg.pointCloudScaleZ;
  out11[3] = cfg.offsetDepth; out11[4] = cfg.samplingPitchX; out11[5] = cfg.samplingPitchY;
  out11[6] = cfg.lambda; out11[7] = cfg.tiltAngleX; out11[8] = cfg.tiltAngleY;
  nxny[0] = cfg.nx; nxny[1] = cfg.ny;
  return 1;
}

}  // extern "C"
