// Written the way the reference's openwrp.cpp drives OPHWRP: read points,
// set parameters, build the WRP plane, save it, propagate, save again.  Also
// dumps the complex planes for the comparison with the oracle.
// usage: wrp_dropin <points.txt> <out prefix>
#include <cstdio>
#include <string>
#include <vector>
#include "oh_openholo_wrp.hpp"

static int dump(const OPHWRP& w, int res, const std::string& path) {
  std::vector<oh_c64> f((size_t)res * res);
  if (w.GetField(f.data()) != 0) return -1;
  FILE* fp = std::fopen(path.c_str(), "wb");
  if (!fp) return -1;
  std::fwrite(f.data(), sizeof(oh_c64), f.size(), fp);
  std::fclose(fp);
  return 0;
}

int main(int argc, char** argv) {
  if (argc < 3) return 2;
  const std::string out = argv[2];
  const int res = 129;
  OPHWRP oh_wrp;
  if (oh_wrp.readxyz(argv[1]) != 0) return 3;
  if (oh_wrp.Setparameter(532e-9f, 8.0e-6f, (float)res) != 0) return 4;
  oh_wrp.SingleWRP(0.5e-3f);
  if (oh_wrp.last_status() != OH_OK) return 5;
  if (dump(oh_wrp, res, out + "_wrp.c64") != 0) return 6;
  std::string t1 = out + "_wrp_table.bmp", t2 = out + "_wrp_result.bmp";
  if (oh_wrp.SavetoImage(&t1[0]) != 0) return 7;
  if (oh_wrp.Fresnelpropagation(0.05f) != 0) return 8;
  if (dump(oh_wrp, res, out + "_holo.c64") != 0) return 9;
  if (oh_wrp.SavetoImage(&t2[0]) != 0) return 10;
  if (oh_wrp.readxyz(out + "_missing.txt") != -1) return 11;   // unreadable file: -1, as the reference
  return 0;
}
