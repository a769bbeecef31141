// OPHWRP drop-in (include/oh_openholo_wrp.hpp): the reference's WRP console
// class (WRP.h:19-61, WRP.cpp) over the C ABI, without CWO++.  The plane is a
// device buffer of res x res oh_c64 owned by the object; methods enqueue the
// library's kernels on the legacy default stream and wait for them, matching
// the reference's blocking calls.
#include <cuda_runtime.h>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>
#include "../../include/oh.h"
#include "../../include/oh_openholo_pointcloud.hpp"   // openholo::ophSaveFileBmp (keti_shim.cpp)
#include "../../include/oh_openholo_wrp.hpp"

struct OPHWRP::State {
  oh_ctx* ctx = nullptr;
  int res = 0;
  double lambda = 0.0, pitch = 0.0;
  oh_c64* plane = nullptr;   // device, res x res
};

OPHWRP::OPHWRP() : st_(new State) {}

OPHWRP::~OPHWRP() {
  if (st_) {
    if (st_->plane) cudaFree(st_->plane);
    if (st_->ctx) oh_ctx_destroy(st_->ctx);
    delete st_;
  }
  std::free(obj);
}

int OPHWRP::readxyz(std::string filename) {
  std::ifstream in(filename);
  if (!in) {
    std::fprintf(stderr, "can not read the file\n");
    return -1;
  }
  std::string line, tok;
  while (std::getline(in, line)) {
    std::istringstream ls(line);
    while (ls >> tok) vec_xyz.push_back((float)std::stod(tok));
  }
  const int num = (int)(vec_xyz.size() / 3);
  cwoObjPoint* op = (cwoObjPoint*)std::calloc((size_t)(num > 0 ? num : 1), sizeof(cwoObjPoint));
  if (!op) return -1;
  for (int i = 0; i < num; ++i) {
    op[i].x = vec_xyz[3 * i];
    op[i].y = vec_xyz[3 * i + 1];
    op[i].z = vec_xyz[3 * i + 2];
  }
  std::free(obj);
  obj = op;
  obj_num = num;
  return 0;
}

int OPHWRP::Setparameter(float m_wavelength, float m_pixelpitch, float m_resolution) {
  const int res = (int)m_resolution;
  if (res < 1 || !(m_pixelpitch > 0) || !(m_wavelength > 0)) { status_ = OH_ERR_INVALID_ARG; return -1; }
  if (!st_->ctx && (status_ = oh_ctx_create(&st_->ctx, 0)) != OH_OK) return -1;
  if (st_->plane && st_->res != res) { cudaFree(st_->plane); st_->plane = nullptr; }
  if (!st_->plane && cudaMalloc((void**)&st_->plane, (size_t)res * res * sizeof(oh_c64)) != cudaSuccess) {
    status_ = OH_ERR_ALLOC;
    return -1;
  }
  if (cudaMemset(st_->plane, 0, (size_t)res * res * sizeof(oh_c64)) != cudaSuccess) { status_ = OH_ERR_CUDA; return -1; }
  st_->res = res;
  st_->lambda = m_wavelength;
  st_->pitch = m_pixelpitch;
  status_ = OH_OK;
  return 0;
}

void OPHWRP::SingleWRP(float z) {
  if (!st_->plane) { status_ = OH_ERR_INVALID_ARG; return; }
  if (obj_num <= 0) { status_ = OH_OK; return; }
  std::vector<double> xyz((size_t)obj_num * 3);
  for (int i = 0; i < obj_num; ++i) {
    xyz[3 * i] = obj[i].x;
    xyz[3 * i + 1] = obj[i].y;
    xyz[3 * i + 2] = obj[i].z;
  }
  double* d = nullptr;
  if (cudaMalloc((void**)&d, xyz.size() * sizeof(double)) != cudaSuccess) { status_ = OH_ERR_ALLOC; return; }
  oh_wrp_params p;
  p.nx = p.ny = st_->res;
  p.pitch = st_->pitch;
  p.lambda = st_->lambda;
  p.z_wrp = z;
  p.window = 0;     // the reference's window formula
  status_ = cudaMemcpy(d, xyz.data(), xyz.size() * sizeof(double), cudaMemcpyHostToDevice) == cudaSuccess
                ? oh_wrp_accumulate(st_->ctx, OH_FP32, &p, d, obj_num, st_->plane, nullptr)
                : OH_ERR_CUDA;
  if (status_ == OH_OK && cudaDeviceSynchronize() != cudaSuccess) status_ = OH_ERR_CUDA;
  cudaFree(d);
}

int OPHWRP::Fresnelpropagation(float z) {
  if (!st_->plane) { status_ = OH_ERR_INVALID_ARG; return -1; }
  status_ = oh_fresnel_propagate(st_->ctx, OH_FP32, st_->res, st_->res, st_->pitch, st_->lambda, z, st_->plane,
                                 nullptr);
  if (status_ == OH_OK && cudaDeviceSynchronize() != cudaSuccess) status_ = OH_ERR_CUDA;
  return status_ == OH_OK ? 0 : -1;
}

int OPHWRP::SavetoImage(char* filename) {
  // CWO_SAVE_AS_ARG: phase, then ScaleReal(255) (min..max -> 0..255); the
  // phase-to-amplitude encoding is the phase plus a constant, which the
  // min-max scaling removes
  if (!st_->plane || !filename) { status_ = OH_ERR_INVALID_ARG; return -1; }
  const size_t n = (size_t)st_->res * st_->res;
  float* ph = nullptr;
  unsigned char* u8 = nullptr;
  if (cudaMalloc((void**)&ph, n * sizeof(float)) != cudaSuccess) { status_ = OH_ERR_ALLOC; return -1; }
  if (cudaMalloc((void**)&u8, n) != cudaSuccess) { cudaFree(ph); status_ = OH_ERR_ALLOC; return -1; }
  status_ = oh_encode(st_->ctx, OH_FP32, OH_ENC_PHASE_TO_AMP, st_->res, st_->res, st_->plane, ph, nullptr);
  if (status_ == OH_OK) status_ = oh_normalize_u8(st_->ctx, OH_FP32, st_->res, st_->res, ph, u8, 0, nullptr);
  std::vector<unsigned char> host(n);
  if (status_ == OH_OK && cudaMemcpy(host.data(), u8, n, cudaMemcpyDeviceToHost) != cudaSuccess) status_ = OH_ERR_CUDA;
  cudaFree(ph);
  cudaFree(u8);
  if (status_ != OH_OK) return -1;
  // the BMP writer appends ".bmp": strip it from the reference-style name
  std::string name(filename);
  if (name.size() > 4 && name.compare(name.size() - 4, 4, ".bmp") == 0) name.resize(name.size() - 4);
  std::vector<char> cname(name.begin(), name.end());
  cname.push_back('\0');
  openholo::ophSaveFileBmp(host.data(), st_->res, st_->res, cname.data());
  return 0;
}

int OPHWRP::GetField(oh_c64* host) const {
  if (!st_->plane || !host) return -1;
  return cudaMemcpy(host, st_->plane, (size_t)st_->res * st_->res * sizeof(oh_c64), cudaMemcpyDeviceToHost) ==
                 cudaSuccess
             ? 0
             : -1;
}
