// SIMPLE_PARSER-compatible reader of the reference's cfg files
// (src/util/SIMPLE_PARSER.cpp:64-168): "key = value" lines, '#' comments,
// keys and values trimmed and lowercased, numbers through atof, vectors as
// "a,b,c". Fills the grid, the step parameters and the per-solid paths and
// scalars that projects/rubberBall/main.cpp:63-141 reads.
#include <ctype.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <fstream>
#include <map>
#include <sstream>
#include <string>

#include "../../include/eulersf.h"

namespace esf {
void set_error(const char* fmt, ...);
}

namespace {
std::string trim(const std::string& in) {
  size_t s = 0, e = in.size();
  while (s < in.size() && isspace((unsigned char)in[s])) s++;
  while (e > s && isspace((unsigned char)in[e - 1])) e--;
  return in.substr(s, e - s);
}
std::string lower(std::string s) {
  for (char& c : s) c = (char)tolower((unsigned char)c);
  return s;
}
struct Cfg {
  std::map<std::string, std::string> v;
  bool has(const std::string& k) const { return v.count(k) > 0; }
  double f(const std::string& k, double d) const { return has(k) ? atof(v.at(k).c_str()) : d; }
  int i(const std::string& k, int d) const { return has(k) ? (int)atof(v.at(k).c_str()) : d; }
  std::string s(const std::string& k, const std::string& d) const { return has(k) ? v.at(k) : d; }
  void vec(const std::string& k, double* out, const double* d) const {
    if (!has(k)) {
      for (int q = 0; q < 3; q++) out[q] = d[q];
      return;
    }
    std::stringstream ss(v.at(k));
    std::string tok;
    for (int q = 0; q < 3; q++) {
      if (!std::getline(ss, tok, ',')) tok = "0";
      out[q] = atof(tok.c_str());
    }
  }
};
}  // namespace

extern "C" esf_status esf_parse_config(const char* path, esf_grid* grid, esf_params* p,
                                       int* num_solids, char* solid_paths, size_t stride,
                                       esf_solid_desc* solids, int max_solids) {
  if (!path || !grid || !p) return ESF_ERR_INVALID_ARG;
  std::ifstream in(path);
  if (!in.good()) {
    esf::set_error("esf_parse_config: cannot open %s", path);
    return ESF_ERR_IO;
  }
  Cfg c;
  std::string line;
  int lineNo = 0;
  while (std::getline(in, line)) {
    lineNo++;
    if (line.size() > 511) line.resize(511);  // the reference reads 512-byte lines
    if (line.empty() || line[0] == '#') continue;
    size_t pos = line.find('=');
    if (pos == std::string::npos) {
      if (!trim(line).empty()) {
        esf::set_error("esf_parse_config: %s:%d: unable to parse '%s'", path, lineNo, line.c_str());
        return ESF_ERR_IO;
      }
      continue;
    }
    c.v[lower(trim(line.substr(0, pos)))] = lower(trim(line.substr(pos + 1)));
  }
  grid->xRes = c.i("xres", 100);
  grid->yRes = c.i("yres", 100);
  grid->zRes = c.i("zres", 100);
  grid->dh = c.f("dh", 0.01);
  const double zero[3] = {0, 0, 0}, one[3] = {1, 1, 1};
  c.vec("origin", grid->origin, zero);
  esf_params_default(grid, p);
  p->dt = c.f("dt", 0.01);
  p->fluid_density = c.f("fluid density", 1);
  p->fluid_viscosity = c.f("fluid viscocity", 0);
  p->vorticity_eps = c.f("vorticity eps", 2.0);
  p->buoyancy = c.f("buoyancy", 0.1);
  p->gravity = c.f("gravity", 0);
  p->rayleigh_alpha = c.f("rayleigh alpha", 0);
  p->rayleigh_beta = c.f("rayleigh beta", 0);
  p->implicit_solver_eps = c.f("implicit solver eps", 1e-8);
  p->div_free_solver_eps = c.f("div free solver eps", 1e-8);
  p->cr_max_iterations = c.i("cr max iterations", 10);
  p->mass_sample_dh = c.f("mass sample dh", grid->dh / 10);
  p->tight_border = c.i("tight border", 3);
  p->extrapolation_cells = c.i("extrapolation cells", 20);
  p->particles_per_cell = c.i("number of particles per material cell", 8);
  p->flip_alpha = c.f("flip alpha", 0.95);
  p->contact_safe_distance = c.f("contact safe distance", grid->dh * 0.5);
  p->wall_thickness = c.f("wall thickness", grid->dh * 1.5);
  p->contact_spring_stiffness = c.f("contact spring stiffness", 10000);
  p->friction = c.f("friction", 0.5);
  p->flip_cutoff = c.i("flip cutoff", 3);
  p->flow_rate = c.f("flow rate", 0);
  {
    const std::string prec = c.s("precision", "fp64");
    p->precision = prec == "mixed" ? ESF_MIXED : prec == "mixed x64" ? ESF_MIXED_X64 : ESF_FP64;
  }
  p->inner_eps = c.f("inner solver eps", 1e-4);
  int n = c.i("number of solids", 1);
  if (num_solids) *num_solids = n;
  for (int i = 0; i < n && i < max_solids; i++) {
    std::string idx = std::to_string(i);
    if (solid_paths && stride > 0) {
      std::string pth = c.s("solid path " + idx, "") + c.s("solid name " + idx, "");
      strncpy(solid_paths + i * stride, pth.c_str(), stride - 1);
      solid_paths[i * stride + stride - 1] = 0;
    }
    if (solids) {
      esf_solid_desc& d = solids[i];
      memset(&d, 0, sizeof d);
      d.lambda = c.f("material lambda " + idx, 100);
      d.mu = c.f("material mu " + idx, 100);
      d.density = c.f("solid mass density " + idx, 1);
      c.vec("solid translation " + idx, d.translation, zero);
      c.vec("solid scaling " + idx, d.scaling, one);
      c.vec("solid initial velocity " + idx, d.initial_velocity, zero);
      double rot[3];
      c.vec("solid rotation " + idx, rot, zero);
      // R = Rx(a pi) Ry(b pi) Rz(c pi)  (main.cpp:131-136)
      double ca = cos(rot[0] * M_PI), sa = sin(rot[0] * M_PI);
      double cb = cos(rot[1] * M_PI), sb = sin(rot[1] * M_PI);
      double cc = cos(rot[2] * M_PI), scz = sin(rot[2] * M_PI);
      double Rx[9] = {1, 0, 0, 0, ca, -sa, 0, sa, ca};
      double Ry[9] = {cb, 0, sb, 0, 1, 0, -sb, 0, cb};
      double Rz[9] = {cc, -scz, 0, scz, cc, 0, 0, 0, 1};
      double t[9];
      for (int r = 0; r < 3; r++)
        for (int q = 0; q < 3; q++) t[3 * r + q] = Rx[3 * r] * Ry[q] + Rx[3 * r + 1] * Ry[3 + q] + Rx[3 * r + 2] * Ry[6 + q];
      for (int r = 0; r < 3; r++)
        for (int q = 0; q < 3; q++) d.rotation[3 * r + q] = t[3 * r] * Rz[q] + t[3 * r + 1] * Rz[3 + q] + t[3 * r + 2] * Rz[6 + q];
    }
  }
  return ESF_OK;
}
