// Drives one coupled step through the C++ facade (include/eulersf.hpp) the
// way projects/rubberBall/main.cpp drives COUPLED_INTEGRATOR_3D: construct,
// addSolid, setFluidDensity, setFluidViscocity, init, setMaxDt,
// stepImplicit. Inputs are raw files written by tests/test_facade.py:
//   params.bin  the esf_params struct as bytes
//   grid.txt    xRes yRes zRes dh ox oy oz
//   solid.txt   mass_res[3] mass_dh mass_origin[3] lambda mu density
//               translation[3] velocity[3] num_vertices num_triangles
//   rest.f64 verts.f64 tris.i32
// Prints one JSON line; exits 3 with the esf::Error text on failure.
#include <cstdio>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

#include "eulersf.hpp"

template <typename T>
static std::vector<T> read_raw(const std::string& path) {
  std::ifstream f(path, std::ios::binary | std::ios::ate);
  std::vector<T> v((size_t)f.tellg() / sizeof(T));
  f.seekg(0);
  f.read(reinterpret_cast<char*>(v.data()), v.size() * sizeof(T));
  return v;
}

int main(int argc, char** argv) {
  if (argc < 2) {
    std::fprintf(stderr, "usage: facade_step <dir> [max_dt]\n");
    return 2;
  }
  const std::string dir = argv[1];
  esf_params params;
  {
    std::vector<char> raw = read_raw<char>(dir + "/params.bin");
    if (raw.size() != sizeof params) {
      std::fprintf(stderr, "params.bin has %zu bytes, esf_params %zu\n", raw.size(), sizeof params);
      return 2;
    }
    std::memcpy(&params, raw.data(), sizeof params);
  }
  int xRes, yRes, zRes;
  double dh, origin[3];
  std::ifstream g(dir + "/grid.txt");
  g >> xRes >> yRes >> zRes >> dh >> origin[0] >> origin[1] >> origin[2];
  esf_solid_desc s;
  std::memset(&s, 0, sizeof s);
  std::ifstream sd(dir + "/solid.txt");
  sd >> s.mass_res[0] >> s.mass_res[1] >> s.mass_res[2] >> s.mass_dh >> s.mass_origin[0] >>
      s.mass_origin[1] >> s.mass_origin[2] >> s.lambda >> s.mu >> s.density >> s.translation[0] >>
      s.translation[1] >> s.translation[2] >> s.initial_velocity[0] >> s.initial_velocity[1] >>
      s.initial_velocity[2] >> s.num_vertices >> s.num_triangles;
  std::vector<double> rest = read_raw<double>(dir + "/rest.f64");
  std::vector<double> verts = read_raw<double>(dir + "/verts.f64");
  std::vector<int> tris = read_raw<int>(dir + "/tris.i32");
  s.rest_mass = rest.data();
  s.vertices = verts.data();
  s.triangles = tris.data();
  const double rot[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
  std::memcpy(s.rotation, rot, sizeof rot);
  for (int k = 0; k < 3; k++) s.scaling[k] = 1.0;
  try {
    esf::CoupledIntegrator3D integrator(xRes, yRes, zRes, dh, origin, &params);
    integrator.addSolid(s);
    integrator.setFluidDensity(params.fluid_density);
    integrator.setFluidViscocity(0.0);
    integrator.init();
    if (argc > 2) integrator.setMaxDt(std::stod(argv[2]));
    esf_step_report r;
    const double energy = integrator.stepImplicit(&r);
    std::vector<double> v = integrator.get<double>(ESF_F_VELOCITY);
    double vsum = 0;
    for (double x : v) vsum += x < 0 ? -x : x;
    std::printf("{\"energy\": %.17g, \"dt\": %.17g, \"iterations\": [%d, %d, %d], "
                "\"velocity_l1\": %.17g, \"status\": %d}\n",
                energy, integrator.dt(), r.iterations[0], r.iterations[1], r.iterations[2], vsum,
                r.status);
  } catch (const esf::Error& e) {
    std::fprintf(stderr, "esf::Error %s\n", e.what());
    return 3;
  }
  return 0;
}
