// eulersf.hpp - header-only C++ facade over include/eulersf.h with the call
// surface of the reference's COUPLED_INTEGRATOR_3D / DEFOR_SOLID_3D
// (include/integrator/COUPLED_INTEGRATOR_3D.h:29-78,
//  include/integrator/DEFOR_SOLID_3D.h:43-71), so that the driver logic of
// projects/rubberBall/main.cpp can run unchanged on the GPU.
//
//   esf::CoupledIntegrator3D* integrator =
//       new esf::CoupledIntegrator3D(xRes, yRes, zRes, dh, origin, params);
//   integrator->addSolid(solidDesc);           // DEFOR_SOLID_3D set-up
//   integrator->setFluidDensity(rho);
//   integrator->init();
//   integrator->setMaxDt(maxDt);
//   double energy = integrator->stepImplicit();
//
// Errors surface as esf::Error (the reference exits or prints instead).
#ifndef EULERSF_HPP
#define EULERSF_HPP

#include <stdexcept>
#include <string>
#include <vector>

#include "eulersf.h"

namespace esf {

class Error : public std::runtime_error {
 public:
  Error(esf_status s, const std::string& where)
      : std::runtime_error(where + ": status " + std::to_string((int)s) + " " + esf_last_error()),
        status(s) {}
  esf_status status;
};

inline void check(esf_status s, const char* where) {
  if (s != ESF_OK) throw Error(s, where);
}

class CoupledIntegrator3D {
 public:
  CoupledIntegrator3D(int xRes, int yRes, int zRes, double dh, const double origin[3],
                      const esf_params* params = nullptr, void* stream = nullptr) {
    grid_.xRes = xRes;
    grid_.yRes = yRes;
    grid_.zRes = zRes;
    grid_.dh = dh;
    for (int k = 0; k < 3; k++) grid_.origin[k] = origin[k];
    if (params) {
      params_ = *params;
    } else {
      check(esf_params_default(&grid_, &params_), "esf_params_default");
    }
    check(esf_create(&grid_, &params_, stream, &scene_), "esf_create");
  }
  ~CoupledIntegrator3D() { esf_destroy(scene_); }
  CoupledIntegrator3D(const CoupledIntegrator3D&) = delete;
  CoupledIntegrator3D& operator=(const CoupledIntegrator3D&) = delete;

  int xRes() const { return grid_.xRes; }
  int yRes() const { return grid_.yRes; }
  int zRes() const { return grid_.zRes; }
  double dh() const { return grid_.dh; }
  const double* origin() const { return grid_.origin; }

  void addSolid(const esf_solid_desc& solid) { check(esf_add_solid(scene_, &solid), "esf_add_solid"); }
  // DEFOR_SOLID_3D::loadRestSDF of solid i (needed by scenes with several solids)
  void loadRestSDF(int solid, const std::string& svolPath) {
    check(esf_solid_load_rest_sdf(scene_, solid, svolPath.c_str()), "esf_solid_load_rest_sdf");
  }
  void setFluidDensity(double d) {
    density_ = d;
    check(esf_set_fluid(scene_, density_, viscosity_), "esf_set_fluid");
  }
  void setFluidViscocity(double v) {
    viscosity_ = v;
    check(esf_set_fluid(scene_, density_, viscosity_), "esf_set_fluid");
  }
  void init() { check(esf_init(scene_), "esf_init"); }
  void setMaxDt(double dt) { check(esf_set_max_dt(scene_, dt), "esf_set_max_dt"); }
  // returns the energy, like COUPLED_INTEGRATOR_3D::stepImplicit
  double stepImplicit(esf_step_report* report = nullptr) {
    esf_step_report r;
    esf_status s = esf_step(scene_, &r);
    if (s != ESF_OK && s != ESF_ERR_NUMERIC) throw Error(s, "esf_step");
    if (report) *report = r;
    return r.energy;
  }
  double dt() const { return esf_dt(scene_); }
  // COUPLED_INTEGRATOR_3D::writeFrame/readFrame; dataPath is the cfg's
  // "data path" (prefix of "frame.NNNN.*")
  void writeFrame(int frame, bool debug = false, const std::string& dataPath = "") {
    check(esf_write_frame(scene_, dataPath.c_str(), frame, debug ? 1 : 0), "esf_write_frame");
  }
  void readFrame(int frame, bool debug = false, const std::string& dataPath = "") {
    check(esf_read_frame(scene_, dataPath.c_str(), frame, debug ? 1 : 0), "esf_read_frame");
  }

  // FIELD_3Df& intensity() of the reference, as a host copy
  std::vector<double> intensity() { return get<double>(ESF_F_INTENSITY); }
  void setIntensity(const std::vector<double>& v) { set(ESF_F_INTENSITY, v); }

  template <typename T>
  std::vector<T> get(esf_field f, int solid = 0) {
    size_t n = 0, eb = 0;
    check(esf_field_info(scene_, f, solid, &n, &eb), "esf_field_info");
    if (eb != sizeof(T)) throw Error(ESF_ERR_INVALID_ARG, "element size mismatch");
    std::vector<T> out(n);
    check(esf_get_field(scene_, f, solid, out.data(), n * eb), "esf_get_field");
    return out;
  }
  template <typename T>
  void set(esf_field f, const std::vector<T>& v, int solid = 0) {
    check(esf_set_field(scene_, f, solid, v.data(), v.size() * sizeof(T)), "esf_set_field");
  }

  esf_scene* handle() { return scene_; }

 private:
  esf_grid grid_;
  esf_params params_;
  esf_scene* scene_ = nullptr;
  double density_ = 1.0, viscosity_ = 0.0;
};

}  // namespace esf

#endif  // EULERSF_HPP
