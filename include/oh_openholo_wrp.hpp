// Drop-in for the reference's WRP console library class OPHWRP
// (OpenHolo_WRP/openwrp_console_ver 1.0/openwrp/WRP.h:19-61, WRP.cpp), without
// the CWO++ base class: the WRP plane lives on the GPU and every method runs
// the library's kernels through the C ABI (oh.h).
//
//   OPHWRP::readxyz(filename)          WRP.cpp:6-55   whitespace-separated x y z per point
//   OPHWRP::Setparameter(wl, pp, res)  WRP.cpp:56-64  res x res plane, pitch pp, wavelength wl
//   OPHWRP::SingleWRP(z)               WRP.cpp:75-140 oh_wrp_accumulate, reference-formula windows
//   OPHWRP::Fresnelpropagation(z)      WRP.cpp:65-68  oh_fresnel_propagate (CWO_FRESNEL_CONV)
//   OPHWRP::SavetoImage(filename)      WRP.cpp:70-74  phase (CWO_SAVE_AS_ARG) scaled to 0..255,
//                                                     8-bit grayscale BMP
// The point record keeps cwoObjPoint's layout (cwo_lib.h:469-474).
// Return codes follow the reference (0 on success, -1 on failure); the
// library's own status and message are available from OPHWRP::last_status()
// and oh_last_error().
#pragma once
#include <string>
#include <vector>
#include "oh.h"

#ifndef OH_CWO_TYPES_DEFINED
#define OH_CWO_TYPES_DEFINED
typedef struct cwoComplex { float cplx[2]; } cwoComplex;
typedef struct cwoObjPoint {
  cwoComplex a;
  float x, y, z;
} cwoObjPoint;
#endif

class OPHWRP {
 public:
  cwoObjPoint* obj = nullptr;
  int obj_num = 0;
  std::vector<float> vec_xyz;

  OPHWRP();
  ~OPHWRP();
  OPHWRP(const OPHWRP&) = delete;
  OPHWRP& operator=(const OPHWRP&) = delete;

  /** Adds the WRP of the loaded points at plane distance z (window from the reference formula). */
  void SingleWRP(float z);
  /** Reads the point cloud (x y z per point, whitespace-separated); -1 when the file cannot be read. */
  int readxyz(std::string filename);
  /** Wavelength, pixel pitch and resolution (res x res) of the WRP plane and hologram; clears the plane. */
  int Setparameter(float m_wavelength, float m_pixelpitch, float m_resolution);
  /** Writes the phase of the plane, scaled to 0..255, as an 8-bit BMP. */
  int SavetoImage(char* filename);
  /** Fresnel-convolution propagation of the plane by z (zero-padded 2x). */
  int Fresnelpropagation(float z);

  // additions without a reference counterpart
  /** Copies the plane (res x res oh_c64) to host memory; -1 before Setparameter. */
  int GetField(oh_c64* host) const;
  /** Status of the last library call made by this object. */
  oh_status last_status() const { return status_; }

 private:
  struct State;
  State* st_ = nullptr;
  oh_status status_ = OH_OK;
};
