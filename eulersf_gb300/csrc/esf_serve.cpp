// Serving: many independent coupled-step scenes on one GPU. Requests arrive
// at any time (esf_server_submit); a request is admitted when its estimated
// device footprint fits the remaining memory budget and a slot is free
// (first fit in arrival order); each admitted scene runs on its own CUDA
// stream, driven by its own host thread, so scenes that arrive while others
// are on the GPU overlap with them on the device; the inner solves of active
// scenes of one grid shape share launches (continuous batching, esf_solver.cu). Results stay readable until
// the client releases the request, which also returns its memory to the
// budget. The reference has no counterpart: it runs one scene per process
// (its function-local statics pin one grid size per process).
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/eulersf.h"

namespace esf {
void set_error(const char* fmt, ...);
struct InnerBatcher;
esf_status batcher_create(int device, InnerBatcher** out, bool autotune);
void batcher_destroy(InnerBatcher* b);
void batcher_stats(InnerBatcher* b, esf_batch_stats* out);
esf_status scene_set_batcher(esf_scene* s, InnerBatcher* b);
}

namespace {

using Clock = std::chrono::steady_clock;

double ms_since(Clock::time_point a, Clock::time_point b) {
  return std::chrono::duration<double, std::milli>(b - a).count();
}

struct SolidCopy {
  esf_solid_desc d;
  std::vector<double> rest, verts;
  std::vector<int> tris;
  std::string sdfPath;  // rest SDF of solid-solid contact, or empty
};

struct Request {
  esf_grid grid;
  esf_params params;
  std::vector<std::unique_ptr<SolidCopy>> solids;
  double density = 1.0, viscosity = 0.0, carpet = 0.0, noiseAmp = 0.0;
  unsigned long long noiseSeed = 0;
  int steps = 0;
  size_t footprint = 0;
  esf_scene* scene = nullptr;
  esf_request_status st;
  Clock::time_point submitted;
};

// U(-a, a) per component at interior nodes; the same splitmix64 mapping as
// eulersf_gb300/scene.py:noise_field, added where the node has no solid mass.
void add_noise(std::vector<double>& v, const std::vector<double>& solidMass, int X, int Y, int Z,
               unsigned long long seed, double a) {
  const unsigned long long base = seed << 40;
  for (long long n = 0; n < (long long)X * Y * Z; n++) {
    const int x = (int)(n % X), y = (int)((n / X) % Y), z = (int)(n / ((long long)X * Y));
    if (!(x > 0 && x < X - 1 && y > 0 && y < Y - 1 && z > 0 && z < Z - 1)) continue;
    if (solidMass[n] != 0.0) continue;
    for (int c = 0; c < 3; c++) {
      unsigned long long q = (unsigned long long)(3 * n + c) + base;
      q += 0x9E3779B97F4A7C15ull;
      q = (q ^ (q >> 30)) * 0xBF58476D1CE4E5B9ull;
      q = (q ^ (q >> 27)) * 0x94D049BB133111EBull;
      q ^= q >> 31;
      const double u = (double)(q >> 11) * (1.0 / 9007199254740992.0);
      v[3 * n + c] += a * (2.0 * u - 1.0);
    }
  }
}

}  // namespace

struct esf_server {
  int device = 0;
  esf::InnerBatcher* batcher = nullptr;  // shared by every scene's inner solves
  size_t budget = 0, inUse = 0;
  int maxActive = 8, active = 0;
  uint64_t next = 1;
  bool stop = false;
  std::mutex m;
  std::condition_variable cv, doneCv;
  std::deque<uint64_t> queue;
  std::map<uint64_t, std::unique_ptr<Request>> reqs;
  std::vector<std::thread> workers;

  // first request in arrival order that fits the remaining budget
  bool pick(uint64_t* t) {
    for (auto it = queue.begin(); it != queue.end(); ++it) {
      Request* r = reqs[*it].get();
      if (inUse + r->footprint <= budget || (active == 0 && inUse == 0)) {
        *t = *it;
        queue.erase(it);
        return true;
      }
    }
    return false;
  }

  esf_status run(Request* r) {
    cudaSetDevice(device);
    esf_status e = esf_create(&r->grid, &r->params, nullptr, &r->scene);
    if (e) return e;
    if (batcher && (e = esf::scene_set_batcher(r->scene, batcher))) return e;
    for (size_t i = 0; i < r->solids.size(); i++) {
      if ((e = esf_add_solid(r->scene, &r->solids[i]->d))) return e;
      if (!r->solids[i]->sdfPath.empty() &&
          (e = esf_solid_load_rest_sdf(r->scene, (int)i, r->solids[i]->sdfPath.c_str())))
        return e;
    }
    if ((e = esf_set_fluid(r->scene, r->density, r->viscosity))) return e;
    if ((e = esf_init(r->scene))) return e;
    const int X = r->grid.xRes, Y = r->grid.yRes, Z = r->grid.zRes;
    const size_t T = (size_t)X * Y * Z;
    if (r->carpet > 0) {
      // smoke carpet (projects/rubberBall/main.cpp:80-90)
      std::vector<double> in(T);
      if ((e = esf_get_field(r->scene, ESF_F_INTENSITY, 0, in.data(), T * 8))) return e;
      const int layers = (int)(r->carpet / r->grid.dh);
      for (int z = 1; z < Z - 1; z++)
        for (int y = 1; y < layers; y++)
          for (int x = 1; x < X - 1; x++) in[x + (size_t)X * (y + (size_t)Y * z)] = (double)0.8f;
      if ((e = esf_set_field(r->scene, ESF_F_INTENSITY, 0, in.data(), T * 8))) return e;
    }
    if (r->noiseAmp > 0) {
      std::vector<double> v(T * 3), sm(T);
      if ((e = esf_get_field(r->scene, ESF_F_VELOCITY, 0, v.data(), T * 24))) return e;
      if ((e = esf_get_field(r->scene, ESF_F_SOLID_MASS, 0, sm.data(), T * 8))) return e;
      add_noise(v, sm, X, Y, Z, r->noiseSeed, r->noiseAmp);
      if ((e = esf_set_field(r->scene, ESF_F_VELOCITY, 0, v.data(), T * 24))) return e;
    }
    for (int k = 0; k < r->steps; k++) {
      esf_step_report rep;
      e = esf_step(r->scene, &rep);
      if (e && e != ESF_ERR_NUMERIC) return e;
      std::lock_guard<std::mutex> g(m);
      r->st.steps_done = k + 1;
      r->st.device_ms += rep.device_ms;
      r->st.last = rep;
      if (e) r->st.status = e;
    }
    return ESF_OK;
  }

  void worker() {
    for (;;) {
      uint64_t t = 0;
      Request* r = nullptr;
      {
        std::unique_lock<std::mutex> g(m);
        cv.wait(g, [&] { return stop || pick(&t); });
        if (stop) return;
        r = reqs[t].get();
        inUse += r->footprint;
        active++;
        r->st.state = ESF_REQ_RUNNING;
        r->st.queued_ms = ms_since(r->submitted, Clock::now());
      }
      const esf_status e = run(r);
      {
        std::lock_guard<std::mutex> g(m);
        active--;
        r->st.latency_ms = ms_since(r->submitted, Clock::now());
        if (e) {
          r->st.state = ESF_REQ_FAILED;
          r->st.status = e;
        } else {
          r->st.state = ESF_REQ_DONE;
        }
      }
      doneCv.notify_all();
      cv.notify_all();
    }
  }
};

extern "C" size_t esf_scene_footprint(const esf_grid* g, const esf_params* p, int ns,
                                      const esf_solid_desc* solids) {
  if (!g || !p) return 0;
  const double T = (double)g->xRes * g->yRes * g->zRes;
  const double R = (double)(g->xRes - 1) * (g->yRes - 1) * (g->zRes - 1);
  // integrator and per-solid node fields, pressure vectors (FP64 + FP32);
  // coefficients fitted to scenes measured on GB300 at 48^3, 96^3 and 160^3
  // (estimate / measured = 1.07, 1.00, 0.99 for a 0.2-radius ball), plus
  // the one-pass FP32 iteration's second set of r, t, q (12 bytes a row)
  double bytes = T * (520.0 + 240.0 * ns) + R * 192.0;
  // ESF_MIXED_X64: the double-float correction and direction (8 bytes each a row)
  if (p->precision == ESF_MIXED_X64) bytes += R * 16.0;
  // scenes with several solids: each further solid's cell -> valid-cell map,
  // and every solid's rest-SDF lattice with its triangle lists (~21 MB for
  // the shipped sphere's volume)
  if (ns > 1) bytes += R * 4.0 * (ns - 1) + ns * 24.0e6;
  for (int i = 0; i < ns && solids; i++) {
    // solid nodes and particles from the scaled mesh's bounding box
    const esf_solid_desc& d = solids[i];
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (int v = 0; v < d.num_vertices; v++)
      for (int q = 0; q < 3; q++) {
        const double c = d.vertices[3 * v + q] * d.scaling[q];
        lo[q] = std::min(lo[q], c);
        hi[q] = std::max(hi[q], c);
      }
    double cells = 1.0;
    for (int q = 0; q < 3; q++) cells *= std::max(0.0, (hi[q] - lo[q]) / g->dh + 2.0);
    const double solidNodes = 0.55 * cells;  // sphere / box volume, plus a margin
    bytes += solidNodes * (27 * 9 * 8 * 1.5 + 27 * 4 + 400) + solidNodes * p->particles_per_cell * 80.0;
  }
  return (size_t)(bytes * 1.1) + (140u << 20);
}

extern "C" esf_status esf_server_create(const esf_server_config* cfg, esf_server** out) {
  if (!out) return ESF_ERR_INVALID_ARG;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    esf::set_error("esf_server_create: no CUDA device");
    return ESF_ERR_NO_DEVICE;
  }
  esf_server* s = new esf_server();
  cudaGetDevice(&s->device);
  size_t freeB = 0, totalB = 0;
  cudaMemGetInfo(&freeB, &totalB);
  s->budget = (cfg && cfg->hbm_budget_bytes) ? cfg->hbm_budget_bytes : (size_t)(0.85 * (double)freeB);
  s->maxActive = (cfg && cfg->max_active > 0) ? cfg->max_active : 8;
  if (!(cfg && cfg->no_batching)) {
    esf_status e = esf::batcher_create(s->device, &s->batcher, cfg && cfg->autotune);
    if (e) {
      delete s;
      return e;
    }
  }
  for (int i = 0; i < s->maxActive; i++) s->workers.emplace_back([s] { s->worker(); });
  *out = s;
  return ESF_OK;
}

extern "C" esf_status esf_server_submit(esf_server* s, const esf_request* q, uint64_t* ticket) {
  if (!s || !q || !ticket || q->steps < 0 || q->num_solids < 1 || q->num_solids > ESF_MAX_SOLIDS ||
      !q->solids) {
    esf::set_error("esf_server_submit: invalid request");
    return ESF_ERR_INVALID_ARG;
  }
  std::unique_ptr<Request> r(new Request());
  r->grid = q->grid;
  r->params = q->params;
  r->density = q->fluid_density;
  r->viscosity = q->fluid_viscosity;
  r->carpet = q->smoke_carpet;
  r->noiseSeed = q->noise_seed;
  r->noiseAmp = q->noise_amplitude;
  r->steps = q->steps;
  for (int i = 0; i < q->num_solids; i++) {
    const esf_solid_desc& d = q->solids[i];
    if (!d.rest_mass || !d.vertices || !d.triangles) {
      esf::set_error("esf_server_submit: solid %d lacks rest mass or mesh", i);
      return ESF_ERR_INVALID_ARG;
    }
    std::unique_ptr<SolidCopy> c(new SolidCopy());
    c->d = d;
    c->rest.assign(d.rest_mass, d.rest_mass + (size_t)d.mass_res[0] * d.mass_res[1] * d.mass_res[2]);
    c->verts.assign(d.vertices, d.vertices + 3 * (size_t)d.num_vertices);
    c->tris.assign(d.triangles, d.triangles + 3 * (size_t)d.num_triangles);
    c->d.rest_mass = c->rest.data();
    c->d.vertices = c->verts.data();
    c->d.triangles = c->tris.data();
    if (q->rest_sdf_paths && q->rest_sdf_paths[i]) c->sdfPath = q->rest_sdf_paths[i];
    if (q->num_solids > 1 && c->sdfPath.empty()) {
      esf::set_error("esf_server_submit: solid %d of a scene with several solids has no rest SDF path", i);
      return ESF_ERR_INVALID_ARG;
    }
    r->solids.push_back(std::move(c));
  }
  r->footprint = esf_scene_footprint(&q->grid, &q->params, q->num_solids, q->solids);
  memset(&r->st, 0, sizeof r->st);
  r->st.state = ESF_REQ_QUEUED;
  r->st.footprint_bytes = r->footprint;
  r->submitted = Clock::now();
  {
    std::lock_guard<std::mutex> g(s->m);
    if (r->footprint > s->budget) {
      esf::set_error("esf_server_submit: request needs ~%zu bytes, the budget is %zu", r->footprint,
                     s->budget);
      return ESF_ERR_OOM;
    }
    *ticket = s->next++;
    s->queue.push_back(*ticket);
    s->reqs[*ticket] = std::move(r);
  }
  s->cv.notify_all();
  return ESF_OK;
}

extern "C" esf_status esf_server_poll(esf_server* s, uint64_t ticket, esf_request_status* out) {
  if (!s || !out) return ESF_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> g(s->m);
  auto it = s->reqs.find(ticket);
  if (it == s->reqs.end()) {
    esf::set_error("esf_server_poll: unknown ticket %llu", (unsigned long long)ticket);
    return ESF_ERR_INVALID_ARG;
  }
  *out = it->second->st;
  return ESF_OK;
}

extern "C" esf_status esf_server_wait(esf_server* s, uint64_t ticket, esf_request_status* out) {
  if (!s || !out) return ESF_ERR_INVALID_ARG;
  std::unique_lock<std::mutex> g(s->m);
  auto it = s->reqs.find(ticket);
  if (it == s->reqs.end()) {
    esf::set_error("esf_server_wait: unknown ticket %llu", (unsigned long long)ticket);
    return ESF_ERR_INVALID_ARG;
  }
  Request* r = it->second.get();
  s->doneCv.wait(g, [&] { return r->st.state == ESF_REQ_DONE || r->st.state == ESF_REQ_FAILED; });
  *out = r->st;
  return ESF_OK;
}

extern "C" esf_status esf_server_get_field(esf_server* s, uint64_t ticket, esf_field f, int solid,
                                           void* host, size_t bytes) {
  if (!s) return ESF_ERR_INVALID_ARG;
  esf_scene* sc = nullptr;
  {
    std::lock_guard<std::mutex> g(s->m);
    auto it = s->reqs.find(ticket);
    if (it == s->reqs.end() || it->second->st.state != ESF_REQ_DONE) {
      esf::set_error("esf_server_get_field: ticket %llu is not a finished request",
                     (unsigned long long)ticket);
      return ESF_ERR_STATE;
    }
    sc = it->second->scene;
  }
  cudaSetDevice(s->device);
  return esf_get_field(sc, f, solid, host, bytes);
}

extern "C" esf_status esf_server_release(esf_server* s, uint64_t ticket) {
  if (!s) return ESF_ERR_INVALID_ARG;
  std::unique_ptr<Request> r;
  {
    std::lock_guard<std::mutex> g(s->m);
    auto it = s->reqs.find(ticket);
    if (it == s->reqs.end()) return ESF_ERR_INVALID_ARG;
    const int state = it->second->st.state;
    if (state == ESF_REQ_RUNNING) {
      esf::set_error("esf_server_release: ticket %llu is still running", (unsigned long long)ticket);
      return ESF_ERR_STATE;
    }
    if (state == ESF_REQ_QUEUED) s->queue.erase(std::find(s->queue.begin(), s->queue.end(), ticket));
    else s->inUse -= it->second->footprint;
    r = std::move(it->second);
    s->reqs.erase(it);
  }
  if (r->scene) {
    cudaSetDevice(s->device);
    esf_destroy(r->scene);
  }
  s->cv.notify_all();
  return ESF_OK;
}

extern "C" esf_status esf_server_destroy(esf_server* s) {
  if (!s) return ESF_OK;
  {
    std::lock_guard<std::mutex> g(s->m);
    s->stop = true;
  }
  s->cv.notify_all();
  for (auto& t : s->workers) t.join();  // running requests finish their steps first
  cudaSetDevice(s->device);
  for (auto& kv : s->reqs)
    if (kv.second->scene) esf_destroy(kv.second->scene);
  esf::batcher_destroy(s->batcher);
  delete s;
  return ESF_OK;
}

extern "C" esf_status esf_server_batch_stats(esf_server* s, esf_batch_stats* out) {
  if (!s || !out) return ESF_ERR_INVALID_ARG;
  memset(out, 0, sizeof *out);
  if (s->batcher) esf::batcher_stats(s->batcher, out);
  return ESF_OK;
}
