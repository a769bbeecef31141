// config_openholo.txt reader: the positional format of
// HologramGenerator::readConfig (OpenHolo_DepthMap/Hologram/src/
// HologramGenerator.cpp:65-229), read with the same sequence of stream
// extractions and getline calls.  The pixel-count and pitch lines are
// arithmetic expressions that the reference hands to QScriptEngine
// (:109-146); a small recursive-descent evaluator (+ - * / parentheses,
// unary signs, decimal/exponent literals) stands in for it.
#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdlib>
#include <fstream>
#include <random>
#include <regex>
#include <string>
#include <vector>
#include "../../include/oh.h"

namespace oh {
void set_error(const std::string& msg);
oh_status fail(oh_status s, const std::string& msg);
}

namespace {

struct Expr {
  const char* s;
  bool ok = true;
  void ws() { while (*s && std::isspace((unsigned char)*s)) ++s; }
  double prim() {
    ws();
    if (*s == '(') { ++s; double v = sum(); ws(); if (*s == ')') ++s; else ok = false; return v; }
    if (*s == '+') { ++s; return prim(); }
    if (*s == '-') { ++s; return -prim(); }
    char* end = nullptr;
    double v = std::strtod(s, &end);
    if (end == s) { ok = false; return 0.0; }
    s = end;
    return v;
  }
  double prod() {
    double v = prim();
    for (;;) {
      ws();
      if (*s == '*') { ++s; v *= prim(); }
      else if (*s == '/') { ++s; v /= prim(); }
      else return v;
    }
  }
  double sum() {
    double v = prod();
    for (;;) {
      ws();
      if (*s == '+') { ++s; v += prod(); }
      else if (*s == '-') { ++s; v -= prod(); }
      else return v;
    }
  }
};

bool eval_expr(const std::string& text, double* out) {
  Expr e{text.c_str()};
  double v = e.sum();
  e.ws();
  if (!e.ok || *e.s) return false;
  *out = v;
  return true;
}

thread_local std::vector<int> t_render;

}  // namespace

extern "C" oh_status oh_depthmap_read_config(const char* path, oh_depthmap_params* p) {
  using oh::fail;
  if (!path || !p) return fail(OH_ERR_INVALID_ARG, "null path or params");
  std::ifstream in(path);
  if (!in.is_open()) return fail(OH_ERR_IO, std::string("file not found: ") + path);
  oh_depthmap_params_default(p);
  std::string temp;
  for (int i = 0; i < 7; ++i) std::getline(in, temp, '\n');
  std::string source, img_prefix, depth_prefix, result_folder, result_prefix;
  bool static_image;
  unsigned start_frame, n_frames, n_digits;
  in >> source; std::getline(in, temp, '\n');
  in >> img_prefix; std::getline(in, temp, '\n');
  in >> depth_prefix; std::getline(in, temp, '\n');
  in >> result_folder; std::getline(in, temp, '\n');
  in >> result_prefix; std::getline(in, temp, '\n');
  in >> static_image; std::getline(in, temp, '\n');
  in >> start_frame; std::getline(in, temp, '\n');
  in >> n_frames; std::getline(in, temp, '\n');
  in >> n_digits; std::getline(in, temp, '\n');
  for (int i = 0; i < 3; ++i) std::getline(in, temp, '\n');
  int transform_method, propagation_method, encoding_method;
  in >> transform_method; std::getline(in, temp, '\n');
  in >> propagation_method; std::getline(in, temp, '\n');
  in >> encoding_method; std::getline(in, temp, '\n');
  for (int i = 0; i < 3; ++i) std::getline(in, temp, '\n');
  double field_lens, wavelength;
  in >> field_lens; std::getline(in, temp, '\n');
  in >> wavelength; std::getline(in, temp, '\n');
  double v[4];
  const char* names[4] = {"SLM_PIXEL_NUMBER_X", "SLM_PIXEL_NUMBER_Y", "SLM_PIXEL_PITCH_X", "SLM_PIXEL_PITCH_Y"};
  for (int i = 0; i < 4; ++i) {
    in >> temp;
    if (!eval_expr(temp, &v[i])) return fail(OH_ERR_IO, std::string("Error: ") + names[i]);
    std::getline(in, temp, '\n');
  }
  for (int i = 0; i < 3; ++i) std::getline(in, temp, '\n');
  double near_d, far_d;
  in >> near_d; std::getline(in, temp, '\n');
  in >> far_d; std::getline(in, temp, '\n');
  bool flag_change;
  unsigned def_q, num_q;
  in >> flag_change; std::getline(in, temp, '\n');
  in >> def_q; std::getline(in, temp, '\n');
  in >> num_q; std::getline(in, temp, '\n');
  std::getline(in, temp, '\n');
  std::string src = temp.substr(0, temp.find("//"));
  // trimmed()
  size_t a = src.find_first_not_of(" \t\r\n"), b = src.find_last_not_of(" \t\r\n");
  src = a == std::string::npos ? std::string() : src.substr(a, b - a + 1);
  t_render.clear();
  if (src.find(':') != std::string::npos) {
    std::smatch m;
    if (std::regex_search(src, m, std::regex("(\\d+):(\\d+)"))) {
      int s0 = std::stoi(m[1].str()), s1 = std::stoi(m[2].str());
      for (int k = s0; k <= s1; ++k) t_render.push_back(k);
    }
  } else {
    std::regex re("(\\d+)");
    for (auto it = std::sregex_iterator(src.begin(), src.end(), re); it != std::sregex_iterator(); ++it)
      t_render.push_back(std::stoi((*it)[1].str()));
  }
  if (t_render.empty()) return fail(OH_ERR_IO, "Error: RENDER_DEPTH");
  bool random_phase;
  in >> random_phase; std::getline(in, temp, '\n');
  if (in.fail()) return fail(OH_ERR_IO, "config file ended early or holds a malformed value");

  p->field_lens = field_lens;
  p->lambda = wavelength;
  p->pnx = (int)v[0];
  p->pny = (int)v[1];
  p->ppx = v[2];
  p->ppy = v[3];
  p->near_depthmap = std::min(near_d, far_d);
  p->far_depthmap = std::max(near_d, far_d);
  p->flag_change_depth_quantization = flag_change ? 1 : 0;
  p->default_depth_quantization = (int)def_q;
  p->num_of_depth = flag_change ? (int)num_q : (int)def_q;
  p->transform_viewing_window = transform_method == 0 ? 1 : 0;
  p->pad = 1;
  p->sig_location_x = 0;
  p->sig_location_y = 1;   // GenerateHologram: Encoding_Symmetrization(ivec2(0,1))
  p->phase_mode = OH_PHASE_REFERENCE;
  if (random_phase) {
    // get_rand_phase_value (HologramGenerator.cpp:457-473): a fresh engine per
    // call, so every layer gets the first draw of this library's engine
    std::default_random_engine generator;
    std::uniform_real_distribution<double> distribution(0.0, 1.0);
    double ph = 2 * M_PI * distribution(generator);
    p->rand_phase_re = std::cos(ph);
    p->rand_phase_im = std::sin(ph);
  } else {
    p->rand_phase_re = 1.0;
    p->rand_phase_im = 0.0;
  }
  p->render_depth = t_render.data();
  p->n_render_depth = (int)t_render.size();
  (void)propagation_method; (void)encoding_method;
  return OH_OK;
}
