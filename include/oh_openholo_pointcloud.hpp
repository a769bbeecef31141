/*
 * oh_openholo_pointcloud.hpp — C++ drop-in for the KETI point-cloud library
 * API (OpenHolo_KETI/VS/Openholo_Generation_PointCloud_Library_beta_v1.0/
 * ophgen_pointcloud/ophgen_pointcloud.h:19-207, ophgen_pointcloud_gpu/
 * ophgen_pointcloud_gpu.h:227-243, oph_common/oph_common.h).
 *
 * Same namespace, type layouts, names and argument meanings, so the
 * reference's example programs (example_cpu.cpp, example_gpu.cpp) compile
 * against this header and link against liboh_gb300.so.  The hologram is
 * computed on the GPU by this library's kernels in both the "CPU" and the
 * "GPU" entry points; like the reference, dst is accumulated (dst += ...),
 * so callers zero it first, and the return value is the elapsed seconds.
 * Loaders return -1 / false on failure without touching a null FILE*.
 */
#ifndef OH_OPENHOLO_POINTCLOUD_HPP
#define OH_OPENHOLO_POINTCLOUD_HPP

#include <string>
#include <vector>

namespace openholo {

typedef struct OphPointCloud {
  OphPointCloud() : x(0), y(0), z(0), amplitude(0), phase(0) {}
  OphPointCloud(const float x, const float y, const float z) : x(x), y(y), z(z), amplitude(0), phase(0) {}
  OphPointCloud(const float x, const float y, const float z, const float amp, const float phase)
      : x(x), y(y), z(z), amplitude(amp), phase(phase) {}
  float x;
  float y;
  float z;
  float amplitude;
  float phase;
} OphPC;

typedef struct OphConfig {
  float pointCloudScaleX;
  float pointCloudScaleY;
  float pointCloudScaleZ;
  float offsetDepth;
  float samplingPitchX;
  float samplingPitchY;
  int nx;
  int ny;
  char* filterShapeFlag;
  float filterXwidth;
  float filterYwidth;
  float focalLengthLensIn;
  float focalLengthLensOut;
  float focalLengthLenEyepiece;
  float lambda;
  float tiltAngleX;
  float tiltAngleY;
} OphSpec;

int ophLoadPointCloud(char* inputData, OphPointCloud*& model);
int ophLoadPointCloud(const std::string inputData, std::vector<OphPointCloud>& model);
int ophLoadPointCloud(const std::string inputData, std::vector<float>& vertexArray, std::vector<float>& phaseArray,
                      std::vector<float>& amplitudeArray);
bool ophLoadSpecConfig(char* inputData, OphSpec* config);
bool ophLoadSpecConfig(const std::string inputData, OphSpec& config);

void ophSetScaleFactor(OphSpec& config, const float scaleX, const float scaleY, const float scaleZ);
void ophSetOffsetDepth(OphSpec& config, const float offsetDepth);
void ophSetSamplingPitch(OphSpec& config, const float pitchX, const float pitchY);
void ophSetImageSize(OphSpec& config, const int n_x, const int n_y);
void ophSetWaveLength(OphSpec& config, const float lambda);
void ophSetTiltAngle(OphSpec& config, const float tiltAngleX, const float tiltAngleY);

double ophGenCghPointCloud(const OphPointCloud* model, const int n_points, const OphSpec& config, float* dst);
double ophGenCghPointCloud(const std::vector<OphPointCloud>& model, const OphSpec& config, float* dst);
double ophGenCghPointCloud(const std::vector<float>& vertexArray, const std::vector<float>& amplitudeArray,
                           const OphSpec& config, float* dst);

namespace gpu {
double ophGenCghPointCloud_cuda(const std::vector<float>& vertexArray, const std::vector<float>& amplitudeArray,
                                const OphSpec& config, float* dst);
}

/* oph_common.h: 8-bit grayscale BMP writer and min/max normalisation with
 * vertical flip (oph_common.cpp:49-115). */
void ophSaveFileBmp(unsigned char* pixelbuffer, int pic_width, int pic_height, char* file_name);
void ophNormalize(float* src, unsigned char* dst, const int nx, const int ny);

}  // namespace openholo

#endif
