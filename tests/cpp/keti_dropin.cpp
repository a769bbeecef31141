// Drives the KETI point-cloud API of include/oh_openholo_pointcloud.hpp the
// way the reference's example_cpu.cpp / example_gpu.cpp do (load spec, load
// points, zeroed fringe, ophGenCghPointCloud, normalise), then writes the raw
// fringe and the normalised image for the test to compare.
// usage: keti_dropin <points.dat> <spec.config> <out_prefix>
#include <cstdio>
#include <cstdlib>
#include <vector>
#include "oh_openholo_pointcloud.hpp"

int main(int argc, char** argv) {
  if (argc != 4) return 2;
  openholo::OphSpec config;
  if (!openholo::ophLoadSpecConfig(argv[2], &config)) return 3;
  openholo::OphPointCloud* model = nullptr;
  int n = openholo::ophLoadPointCloud(argv[1], model);
  if (n < 0) return 4;
  std::vector<float> fringe((size_t)config.nx * config.ny, 0.f), fringe_gpu(fringe.size(), 0.f);
  std::vector<unsigned char> img(fringe.size());
  double t = openholo::ophGenCghPointCloud(model, n, config, fringe.data());
  if (t < 0) return 5;
  std::vector<float> v, ph, amp;
  if (openholo::ophLoadPointCloud(std::string(argv[1]), v, ph, amp) != n) return 6;
  if (openholo::gpu::ophGenCghPointCloud_cuda(v, amp, config, fringe_gpu.data()) < 0) return 7;
  openholo::ophNormalize(fringe.data(), img.data(), config.nx, config.ny);
  std::string p(argv[3]);
  FILE* f = std::fopen((p + "_fringe.f32").c_str(), "wb");
  std::fwrite(fringe.data(), 4, fringe.size(), f);
  std::fclose(f);
  f = std::fopen((p + "_fringe_gpu.f32").c_str(), "wb");
  std::fwrite(fringe_gpu.data(), 4, fringe_gpu.size(), f);
  std::fclose(f);
  f = std::fopen((p + "_img.u8").c_str(), "wb");
  std::fwrite(img.data(), 1, img.size(), f);
  std::fclose(f);
  openholo::ophSaveFileBmp(img.data(), config.nx, config.ny, const_cast<char*>((p + "_img").c_str()));
  std::free(model);
  std::printf("points %d nx %d ny %d\n", n, config.nx, config.ny);
  return 0;
}
