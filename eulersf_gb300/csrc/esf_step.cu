// Host orchestration of the coupled step and the C ABI of include/eulersf.h.
// The order of operations follows COUPLED_INTEGRATOR_3D::stepImplicit
// (COUPLED_INTEGRATOR_3D.cpp:377-636), pcrImplicitSolve (:662-764) and
// finalizeSolution (:828-917); every array stays resident in HBM and the host
// only reads back a handful of integers per step (bounding boxes, particle
// and solid-node counts, the CFL speed).
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>
#include <chrono>
#include <mutex>
#include <thread>
#include <string>
#include <vector>

#include "esf_contact_host.h"
#include "esf_io.h"
#include "esf_kernels.cuh"

namespace esf {

static thread_local char g_err[1024] = "";
static unsigned long long g_launches = 0;
static thread_local unsigned long long* g_capture = nullptr;
void note_launch() {
  if (g_capture) (*g_capture)++;
  else __atomic_add_fetch(&g_launches, 1ull, __ATOMIC_RELAXED);
}
void note_graph_replay(unsigned long long kernels) { __atomic_add_fetch(&g_launches, kernels, __ATOMIC_RELAXED); }
void set_capturing(bool on, unsigned long long* counter) { g_capture = on ? counter : nullptr; }
void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof g_err, fmt, ap);
  va_end(ap);
}

// ESF_TRACE: host-clock breakdown inside a phase, printed to stderr. Each
// mark synchronises the stream, so traced steps run slower; for finding
// where a phase's time goes.
struct TraceMarks {
  cudaStream_t st;
  bool on;
  std::chrono::steady_clock::time_point t0;
  explicit TraceMarks(cudaStream_t s) : st(s), on(getenv("ESF_TRACE") != nullptr) {
    if (on) {
      cudaStreamSynchronize(st);
      t0 = std::chrono::steady_clock::now();
    }
  }
  void mark(const char* what) {
    if (!on) return;
    cudaStreamSynchronize(st);
    const auto t = std::chrono::steady_clock::now();
    fprintf(stderr, "[esf]   %s %.3f ms\n", what, std::chrono::duration<double, std::milli>(t - t0).count());
    t0 = t;
  }
};

static int kblocks(long long n, int per = KT) {
  long long b = (n + per - 1) / per;
  if (b < 1) b = 1;
  if (b > 152LL * 16) b = 152LL * 16;
  return (int)b;
}

// grow-only device buffer
struct DBuf {
  void* p = nullptr;
  size_t bytes = 0;
  esf_status ensure(size_t b) {
    if (b <= bytes && p) return ESF_OK;
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
    size_t nb = b + b / 4 + 256;
    cudaError_t e = cudaMalloc(&p, nb);
    if (e != cudaSuccess) {
      set_error("cudaMalloc(%zu): %s", nb, cudaGetErrorString(e));
      return ESF_ERR_OOM;
    }
    bytes = nb;
    return ESF_OK;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
  template <typename T>
  T* as() const {
    return (T*)p;
  }
};

struct Solid {
  SolidDev d;
  // host copies of the description
  double rot[9], trans[3], scale[3], v0[3];
  int nv = 0, ntri = 0;
  std::vector<double> restPose;
  std::vector<int> tris;
  double *dRot = nullptr, *dVerts = nullptr, *dRest = nullptr, *dRestMass = nullptr;
  int* dTris = nullptr;
  // boxes (reference members _xmin.._zmax, _tightMin/_tightMax)
  int ex[6];   // xmin ymin zmin xmax ymax zmax
  int tmin[3], tmax[3];
  double safeMin[3], safeMax[3];
  // particles and valid-cell list
  DBuf part, cellList, cellFlag, cellScan;
  // plasticity: FpInv per material cell, per-valid-cell updates, winners
  DBuf fp, fpUpd, fpVal, fpWin;
  long long pn = 0;
  long long np = 0, nValid = 0;
  double pmass = 0;
  // rest SDF of solid-solid contact (esf_solid_load_rest_sdf): lattice
  // values and codes, per-point triangle lists
  DBuf sdfVal, sdfCode, sdfOff, sdfIds;
  RestSdfDev sdf{};
  bool hasSdf = false;
  // cell -> valid-cell ordinal of this solid (scenes with several solids)
  DBuf ord;
};

}  // namespace esf

struct esf_scene {
  GridDev g;
  esf_params p;
  cudaStream_t stream = nullptr;
  bool ownStream = false;
  int device = 0;
  int ns = 0;
  esf::Solid* s[ESF_MAX_SOLIDS] = {};
  bool inited = false;
  bool failed = false;  // a solve met NaN/Inf; cleared by esf_read_frame
  double fluidDensity = 1.0, defaultDt = 0.01, dt = 0.01, vortEps = 0.0;
  // node fields
  double *vel = nullptr, *vws = nullptr, *vort = nullptr, *intensity = nullptr, *ws = nullptr;
  double *solidMass = nullptr, *nodeVF = nullptr, *quarter = nullptr, *minv = nullptr;
  double *uf = nullptr, *mvf = nullptr, *vstar = nullptr, *v1 = nullptr, *pc = nullptr;
  int *sdof = nullptr, *nodeFlag = nullptr, *nodeScan = nullptr;
  // cell fields
  double *lambda = nullptr, *jdiag = nullptr, *rhs = nullptr, *b1 = nullptr;
  int* cellOrd = nullptr;
  // solid unknowns (grow-only)
  long long S = 0;
  esf::DBuf sNode, solidF, solidMv, damped, solidV0, solidPC, solidB1, sysDiag, blocks, nbr, mask;
  esf::DBuf Ke, nf, energy;
  esf::DBuf fbCells, fbSlot;  // mixed: near-degenerate cells for the FP64 stiffness
  esf::DBuf mfCell, mfCorner;  // mixed: per valid cell data of the matrix-free solid operator
  long long mfCells = 0;       // valid cells they hold (0: assembled FP32 blocks)
  long long Sstep = 0;        // solid nodes of the last step's solid system
  // asynchronous frame writing (esf_write_frame_async)
  double* framePinned = nullptr;
  size_t frameWords = 0;
  cudaEvent_t frameEv = nullptr;
  std::thread frameThread;
  int frameStatus = 0;
  long long validCells = 0;
  esf::DBuf contactCount;  // particles that took a solid-solid impulse this step
  // scratch
  esf::DBuf cubTmp, keys, vals, skeys, svals, bstart, bend, mt, pweights;
  long long mtLen = 0;
  int *dInts = nullptr, *hInts = nullptr;
  unsigned long long* dU64 = nullptr;
  unsigned long long* hU64 = nullptr;
  esf::PressureWork* pw = nullptr;
  esf::SolidWork* sw = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaEvent_t ph[14] = {};
  int status = 0;
};

using namespace esf;

#define TRY(x)                   \
  do {                           \
    esf_status _s = (x);         \
    if (_s != ESF_OK) return _s; \
  } while (0)

extern "C" {

int esf_abi_version(void) { return ESF_ABI_VERSION; }
uint64_t esf_kernel_launches(void) { return __atomic_load_n(&esf::g_launches, __ATOMIC_RELAXED); }
const char* esf_last_error(void) { return esf::g_err; }

esf_status esf_params_default(const esf_grid* g, esf_params* p) {
  if (!g || !p) return ESF_ERR_INVALID_ARG;
  memset(p, 0, sizeof *p);
  p->dt = 0.01;
  p->fluid_density = 1.0;
  p->vorticity_eps = 2.0;
  p->buoyancy = 0.1;
  p->gravity = 0.0;
  p->implicit_solver_eps = 1e-8;
  p->div_free_solver_eps = 1e-8;
  p->cr_max_iterations = 10;
  p->mass_sample_dh = g->dh / 10;
  p->tight_border = 3;
  p->extrapolation_cells = 20;
  p->particles_per_cell = 8;
  p->flip_alpha = 0.95;
  p->contact_safe_distance = g->dh * 0.5;
  p->wall_thickness = g->dh * 1.5;
  p->contact_spring_stiffness = 10000;
  p->friction = 0.5;
  p->flip_cutoff = 3;
  p->precision = ESF_FP64;
  p->inner_eps = 1e-4;
  p->max_refinements = 50;
  return ESF_OK;
}

}  // extern "C"

static esf_status dalloc(void** p, size_t bytes) {
  cudaError_t e = cudaMalloc(p, bytes ? bytes : 8);
  if (e != cudaSuccess) {
    set_error("cudaMalloc(%zu): %s", bytes, cudaGetErrorString(e));
    return ESF_ERR_OOM;
  }
  return ESF_OK;
}

extern "C" esf_status esf_create(const esf_grid* g, const esf_params* p, void* stream,
                                 esf_scene** out) {
  if (!g || !p || !out) {
    set_error("esf_create: null argument");
    return ESF_ERR_INVALID_ARG;
  }
  *out = nullptr;
  if (g->xRes < 4 || g->yRes < 4 || g->zRes < 4 || !(g->dh > 0)) {
    set_error("esf_create: grid must have >= 4 nodes per axis and dh > 0");
    return ESF_ERR_INVALID_ARG;
  }
  if ((long long)g->xRes * g->yRes * g->zRes * 8 >= (1LL << 31)) {
    set_error("esf_create: grid too large for 32-bit solid/particle indices");
    return ESF_ERR_UNSUPPORTED;
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    set_error("esf_create: no CUDA device");
    return ESF_ERR_NO_DEVICE;
  }
  esf_scene* s = new esf_scene();
  cudaGetDevice(&s->device);
  GridDev& G = s->g;
  G.X = g->xRes;
  G.Y = g->yRes;
  G.Z = g->zRes;
  G.slab = (long long)G.X * G.Y;
  G.T = G.slab * G.Z;
  G.cX = G.X - 1;
  G.cY = G.Y - 1;
  G.cZ = G.Z - 1;
  G.cslab = (long long)G.cX * G.cY;
  G.R = G.cslab * G.cZ;
  G.dh = g->dh;
  G.dhInv = 1.0 / g->dh;
  for (int k = 0; k < 3; k++) G.o[k] = g->origin[k];
  s->p = *p;
  s->defaultDt = s->dt = p->dt;
  int maxRes = G.X > G.Y ? (G.X > G.Z ? G.X : G.Z) : (G.Y > G.Z ? G.Y : G.Z);
  double scaling = 64.0f / maxRes;
  scaling = (scaling < 1.0f) ? 1.0f : scaling;
  s->vortEps = p->vorticity_eps / scaling;  // COUPLED_INTEGRATOR_3D.cpp:67-71
  if (stream) {
    s->stream = (cudaStream_t)stream;
  } else {
    if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess) {
      delete s;
      set_error("cudaStreamCreate failed");
      return ESF_ERR_CUDA;
    }
    s->ownStream = true;
  }
  const size_t T = G.T, R = G.R;
  esf_status e = ESF_OK;
#define A(ptr, bytes) \
  if (!e) e = dalloc((void**)&s->ptr, bytes)
  A(vel, T * 24);
  A(vws, T * 24);
  A(vort, T * 24);
  A(intensity, T * 8);
  A(ws, T * 8);
  A(solidMass, T * 8);
  A(nodeVF, T * 8);
  A(quarter, T * 64);
  A(minv, T * 8);
  A(uf, T * 24);
  A(mvf, T * 24);
  A(vstar, T * 24);
  A(v1, T * 24);
  A(pc, T * 24);
  A(sdof, T * 4);
  A(nodeFlag, T * 4);
  A(nodeScan, T * 4);
  A(lambda, R * 8);
  A(jdiag, R * 8);
  A(rhs, R * 8);
  A(b1, R * 8);
  A(cellOrd, R * 4);
  A(dInts, 64 * 4);
  A(dU64, 16 * 8);
#undef A
  if (!e && cudaMallocHost(&s->hInts, 64 * 4) != cudaSuccess) e = ESF_ERR_OOM;
  if (!e && cudaMallocHost(&s->hU64, 16 * 8) != cudaSuccess) e = ESF_ERR_OOM;
  if (!e) {
    // zero-initialised like the reference's Eigen/vector fields
    cudaMemsetAsync(s->vel, 0, T * 24, s->stream);
    cudaMemsetAsync(s->vws, 0, T * 24, s->stream);
    cudaMemsetAsync(s->vort, 0, T * 24, s->stream);
    cudaMemsetAsync(s->intensity, 0, T * 8, s->stream);
    cudaMemsetAsync(s->ws, 0, T * 8, s->stream);
    cudaMemsetAsync(s->solidMass, 0, T * 8, s->stream);
    cudaMemsetAsync(s->nodeVF, 0, T * 8, s->stream);
    cudaMemsetAsync(s->uf, 0, T * 24, s->stream);
    cudaMemsetAsync(s->mvf, 0, T * 24, s->stream);
    cudaMemsetAsync(s->vstar, 0, T * 24, s->stream);
    cudaMemsetAsync(s->v1, 0, T * 24, s->stream);
    cudaMemsetAsync(s->pc, 0, T * 24, s->stream);
    cudaMemsetAsync(s->lambda, 0, R * 8, s->stream);
    cudaMemsetAsync(s->jdiag, 0, R * 8, s->stream);
    cudaMemsetAsync(s->rhs, 0, R * 8, s->stream);
    cudaMemsetAsync(s->b1, 0, R * 8, s->stream);
    e = pressure_work_alloc(&s->pw, G, p->precision != ESF_FP64);
  }
  if (!e && cudaEventCreate(&s->e0) != cudaSuccess) e = ESF_ERR_CUDA;
  if (!e && cudaEventCreate(&s->e1) != cudaSuccess) e = ESF_ERR_CUDA;
  for (int i = 0; i < 14 && !e; i++)
    if (cudaEventCreate(&s->ph[i]) != cudaSuccess) e = ESF_ERR_CUDA;
  if (e) {
    esf_destroy(s);
    return e;
  }
  *out = s;
  return ESF_OK;
}

static void free_solid(Solid* d) {
  if (!d) return;
  SolidDev& x = d->d;
  cudaFree(x.X); cudaFree(x.u); cudaFree(x.vel); cudaFree(x.vws); cudaFree(x.tmp3);
  cudaFree(x.mass); cudaFree(x.phi); cudaFree(x.detFInv); cudaFree(x.quarter); cudaFree(x.valid);
  cudaFree(d->dRot); cudaFree(d->dVerts); cudaFree(d->dRest); cudaFree(d->dRestMass); cudaFree(d->dTris);
  d->part.release(); d->cellList.release(); d->cellFlag.release(); d->cellScan.release();
  d->fp.release(); d->fpUpd.release(); d->fpVal.release(); d->fpWin.release();
  d->sdfVal.release(); d->sdfCode.release(); d->sdfOff.release(); d->sdfIds.release(); d->ord.release();
  delete d;
}

extern "C" esf_status esf_frame_wait(esf_scene* s);

extern "C" esf_status esf_destroy(esf_scene* s) {
  if (!s) return ESF_OK;
  esf_frame_wait(s);
  if (s->framePinned) cudaFreeHost(s->framePinned);
  if (s->frameEv) cudaEventDestroy(s->frameEv);
  if (s->stream) cudaStreamSynchronize(s->stream);
  for (int i = 0; i < s->ns; i++) free_solid(s->s[i]);
  double* d64[] = {s->vel, s->vws, s->vort, s->intensity, s->ws, s->solidMass, s->nodeVF, s->quarter,
                   s->minv, s->uf, s->mvf, s->vstar, s->v1, s->pc, s->lambda, s->jdiag, s->rhs, s->b1};
  for (double* p : d64) cudaFree(p);
  cudaFree(s->sdof); cudaFree(s->nodeFlag); cudaFree(s->nodeScan); cudaFree(s->cellOrd);
  cudaFree(s->dInts); cudaFree(s->dU64);
  if (s->hInts) cudaFreeHost(s->hInts);
  if (s->hU64) cudaFreeHost(s->hU64);
  DBuf* bufs[] = {&s->sNode, &s->solidF, &s->solidMv, &s->damped, &s->solidV0, &s->solidPC,
                  &s->solidB1, &s->sysDiag, &s->blocks, &s->nbr, &s->mask, &s->Ke, &s->nf, &s->fbCells, &s->fbSlot, &s->mfCell, &s->mfCorner,
                  &s->energy, &s->cubTmp, &s->keys, &s->vals, &s->skeys, &s->svals, &s->bstart,
                  &s->bend, &s->mt, &s->pweights, &s->contactCount};
  for (DBuf* b : bufs) b->release();
  pressure_work_free(s->pw);
  solid_work_free(s->sw);
  if (s->e0) cudaEventDestroy(s->e0);
  if (s->e1) cudaEventDestroy(s->e1);
  for (int i = 0; i < 14; i++)
    if (s->ph[i]) cudaEventDestroy(s->ph[i]);
  if (s->ownStream && s->stream) cudaStreamDestroy(s->stream);
  delete s;
  return ESF_OK;
}

extern "C" esf_status esf_add_solid(esf_scene* sc, const esf_solid_desc* dd) {
  if (!sc || !dd) {
    set_error("esf_add_solid: null argument");
    return ESF_ERR_INVALID_ARG;
  }
  if (sc->inited || sc->ns >= ESF_MAX_SOLIDS) {
    set_error("esf_add_solid: scene already initialised or too many solids");
    return ESF_ERR_STATE;
  }
  if (!dd->rest_mass || dd->mass_res[0] < 2 || dd->mass_res[1] < 2 || dd->mass_res[2] < 2 ||
      !(dd->mass_dh > 0) || dd->num_vertices <= 0 || !dd->vertices || dd->num_triangles <= 0 ||
      !dd->triangles) {
    set_error("esf_add_solid: invalid rest mass grid or mesh");
    return ESF_ERR_INVALID_ARG;
  }
  for (long long t = 0; t < 3LL * dd->num_triangles; t++)
    if (dd->triangles[t] < 0 || dd->triangles[t] >= dd->num_vertices) {
      set_error("esf_add_solid: triangle index out of range");
      return ESF_ERR_INVALID_ARG;
    }
  const GridDev& G = sc->g;
  Solid* d = new Solid();
  SolidDev& x = d->d;
  memset(&x, 0, sizeof x);
  const size_t T = G.T;
  esf_status e = ESF_OK;
#define A(ptr, bytes) \
  if (!e) e = dalloc((void**)&(ptr), bytes)
  A(x.X, T * 24);
  A(x.u, T * 24);
  A(x.vel, T * 24);
  A(x.vws, T * 24);
  A(x.tmp3, T * 24);
  A(x.mass, T * 8);
  A(x.phi, T * 8);
  A(x.detFInv, T * 8);
  A(x.quarter, T * 64);
  A(x.valid, G.R);
  size_t mn = (size_t)dd->mass_res[0] * dd->mass_res[1] * dd->mass_res[2];
  A(d->dRestMass, mn * 8);
  A(d->dRot, 9 * 8);
  A(d->dVerts, (size_t)dd->num_vertices * 24);
  A(d->dRest, (size_t)dd->num_vertices * 24);
  A(d->dTris, (size_t)dd->num_triangles * 12);
#undef A
  if (e) {
    free_solid(d);
    return e;
  }
  cudaStream_t st = sc->stream;
  for (int k = 0; k < 3; k++) {
    x.mres[k] = dd->mass_res[k];
    x.morig[k] = dd->mass_origin[k];
    d->trans[k] = dd->translation[k];
    d->scale[k] = dd->scaling[k];
    d->v0[k] = dd->initial_velocity[k];
  }
  memcpy(d->rot, dd->rotation, sizeof d->rot);
  x.mdh = dd->mass_dh;
  x.rest = d->dRestMass;
  x.lambda = dd->lambda;
  x.mu = dd->mu;
  x.qcm = dd->density * G.dh * G.dh * G.dh * 0.125;  // setMassDensity (DEFOR_SOLID_3D.h:64-66)
  x.G = 0.25 * G.dhInv;
  x.dt = sc->p.dt;
  d->pmass = (x.qcm / (G.dh * G.dh * G.dh * 0.125)) * (G.dh * G.dh * G.dh / sc->p.particles_per_cell);
  ESF_CUDA(cudaMemcpy(d->dRestMass, dd->rest_mass, mn * 8, cudaMemcpyHostToDevice));
  ESF_CUDA(cudaMemcpy(d->dRot, d->rot, 72, cudaMemcpyHostToDevice));
  d->nv = dd->num_vertices;
  d->ntri = dd->num_triangles;
  d->restPose.assign(dd->vertices, dd->vertices + 3 * d->nv);
  d->tris.assign(dd->triangles, dd->triangles + 3 * d->ntri);
  // current pose: OBJ::scale, transformMesh, translateMesh (main.cpp:150-154)
  std::vector<double> cur(3 * d->nv);
  for (int v = 0; v < d->nv; v++) {
    double pp[3], q[3];
    for (int k = 0; k < 3; k++) pp[k] = d->restPose[3 * v + k] * d->scale[k];
    for (int i = 0; i < 3; i++) q[i] = (d->rot[i * 3 + 0] * pp[0] + d->rot[i * 3 + 1] * pp[1]) + d->rot[i * 3 + 2] * pp[2];
    for (int k = 0; k < 3; k++) cur[3 * v + k] = q[k] + d->trans[k];
  }
  ESF_CUDA(cudaMemcpy(d->dVerts, cur.data(), cur.size() * 8, cudaMemcpyHostToDevice));
  ESF_CUDA(cudaMemcpy(d->dRest, d->restPose.data(), cur.size() * 8, cudaMemcpyHostToDevice));
  ESF_CUDA(cudaMemcpy(d->dTris, d->tris.data(), d->tris.size() * 4, cudaMemcpyHostToDevice));
  for (int k = 0; k < 3; k++) d->safeMin[k] = G.o[k] + 2 * G.dh;
  d->safeMax[0] = G.o[0] + (G.X - 3) * G.dh;
  d->safeMax[1] = G.o[1] + (G.Y - 3) * G.dh;
  d->safeMax[2] = G.o[2] + (G.Z - 3) * G.dh;
  ESF_CUDA(cudaMemsetAsync(x.vws, 0, T * 24, st));
  ESF_CUDA(cudaMemsetAsync(x.tmp3, 0, T * 24, st));
  ESF_CUDA(cudaMemsetAsync(x.mass, 0, T * 8, st));
  ESF_CUDA(cudaMemsetAsync(x.phi, 0, T * 8, st));
  ESF_CUDA(cudaMemsetAsync(x.detFInv, 0, T * 8, st));
  ESF_CUDA(cudaMemsetAsync(x.quarter, 0, T * 64, st));
  ESF_CUDA(cudaMemsetAsync(x.valid, 0, G.R, st));
  // setPlasticYield before loadSurfaceMesh (main.cpp:119-123, 144): FpInv
  // on a grid of half the cell size over the rest mesh's box grown by one
  // cell, identity (DEFOR_SOLID_3D.cpp:158-186)
  if (dd->plastic_yield > 0) {
    x.plastic = 1;
    x.yield = dd->plastic_yield;
    x.flowRate = sc->p.flow_rate;
    double bmin[3] = {1e9, 1e9, 1e9}, bmax[3] = {-1e9, -1e9, -1e9};
    for (int v = 0; v < d->nv; v++)
      for (int k = 0; k < 3; k++) {
        bmin[k] = std::min(bmin[k], d->restPose[3 * v + k]);
        bmax[k] = std::max(bmax[k], d->restPose[3 * v + k]);
      }
    x.pdh = G.dh * .5;
    for (int k = 0; k < 3; k++) {
      bmin[k] -= G.dh;
      bmax[k] += G.dh;
      x.pres[k] = (int)((bmax[k] - bmin[k]) / x.pdh + 1);
      x.porig[k] = bmin[k];
    }
    d->pn = (long long)x.pres[0] * x.pres[1] * x.pres[2];
    std::vector<double> id((size_t)d->pn * 9, 0.0);
    for (long long c = 0; c < d->pn; c++)
      for (int i = 0; i < 3; i++) id[c * 9 + 4 * i] = 1.0;
    esf_status ea = d->fp.ensure(d->pn * 72);
    if (!ea) ea = d->fpWin.ensure(d->pn * 4);
    if (ea) {
      free_solid(d);
      return ea;
    }
    x.FpInv = d->fp.as<double>();
    ESF_CUDA(cudaMemcpy(x.FpInv, id.data(), d->pn * 72, cudaMemcpyHostToDevice));
  }
  ESF_COUNTED k_initial_state<<<kblocks(G.T), KT, 0, st>>>(G, x, d->dRot, d->trans[0], d->trans[1], d->trans[2],
                                               d->scale[0], d->scale[1], d->scale[2], d->v0[0],
                                               d->v0[1], d->v0[2]);
  ESF_LAUNCH_CHECK();
  ESF_CUDA(cudaStreamSynchronize(st));
  sc->s[sc->ns++] = d;
  return ESF_OK;
}

// DEFOR_SOLID_3D::loadRestSDF (DEFOR_SOLID_3D.cpp:210-214): the solid's
// rest SDF from a ".svol" file and the triangle lists of its band points,
// hashed from the rest-pose mesh, on the device.
extern "C" esf_status esf_solid_load_rest_sdf(esf_scene* sc, int solid, const char* path) {
  if (!sc || !path || solid < 0 || solid >= sc->ns) {
    set_error("esf_solid_load_rest_sdf: no such solid or null path");
    return ESF_ERR_INVALID_ARG;
  }
  cudaSetDevice(sc->device);
  Solid* d = sc->s[solid];
  SvolLattice L;
  std::vector<int> off, ids;
  try {  // host allocations of the lattice and the triangle lists
    TRY(svol_read(path, &L));
    if (!svol_hash_triangles(L, d->restPose.data(), d->ntri, d->tris.data(), &off, &ids)) {
      set_error("esf_solid_load_rest_sdf: %s: the mesh's triangle lists on this lattice exceed 2^31 entries",
                path);
      return ESF_ERR_UNSUPPORTED;
    }
  } catch (...) {
    set_error("esf_solid_load_rest_sdf: out of host memory for %s", path);
    return ESF_ERR_OOM;
  }
  TRY(d->sdfVal.ensure(L.val.size() * 4));
  TRY(d->sdfCode.ensure(L.code.size()));
  TRY(d->sdfOff.ensure(off.size() * 4));
  TRY(d->sdfIds.ensure(ids.size() * 4));
  ESF_CUDA(cudaStreamSynchronize(sc->stream));
  ESF_CUDA(cudaMemcpy(d->sdfVal.p, L.val.data(), L.val.size() * 4, cudaMemcpyHostToDevice));
  ESF_CUDA(cudaMemcpy(d->sdfCode.p, L.code.data(), L.code.size(), cudaMemcpyHostToDevice));
  ESF_CUDA(cudaMemcpy(d->sdfOff.p, off.data(), off.size() * 4, cudaMemcpyHostToDevice));
  ESF_CUDA(cudaMemcpy(d->sdfIds.p, ids.data(), ids.size() * 4, cudaMemcpyHostToDevice));
  RestSdfDev& r = d->sdf;
  r.val = d->sdfVal.as<float>();
  r.code = d->sdfCode.as<signed char>();
  r.triOff = d->sdfOff.as<int>();
  r.triIds = d->sdfIds.as<int>();
  for (int k = 0; k < 3; k++) {
    r.lo[k] = L.lo[k];
    r.n[k] = L.n[k];
  }
  r.nxy = (long long)L.n[0] * L.n[1];
  r.dx = L.dx;
  r.inv = 1.0 / L.dx;
  for (int k = 0; k < 3; k++) r.off[k] = (-L.t[k]) * r.inv;
  r.inC = L.inC;
  r.outC = L.outC;
  r.rest = d->dRest;
  r.cur = d->dVerts;
  r.tris = d->dTris;
  d->hasSdf = true;
  return ESF_OK;
}

// SPARSE_SDF::signedDistAndCurrentNormal of solid `solid` at n rest-space
// points (host arrays), with the solid's current mesh as the step left it.
extern "C" esf_status esf_rest_sdf_query(esf_scene* sc, int solid, int n, const double* points, double safe_dist,
                                         double* sd, double* normals) {
  if (!sc || solid < 0 || solid >= sc->ns || n < 0 || (n > 0 && (!points || !sd || !normals))) {
    set_error("esf_rest_sdf_query: invalid argument");
    return ESF_ERR_INVALID_ARG;
  }
  Solid* d = sc->s[solid];
  if (!d->hasSdf) {
    set_error("esf_rest_sdf_query: solid %d has no rest SDF", solid);
    return ESF_ERR_STATE;
  }
  if (n == 0) return ESF_OK;
  cudaSetDevice(sc->device);
  double *dp = nullptr, *dsd = nullptr, *dn = nullptr;
  esf_status e = dalloc((void**)&dp, (size_t)n * 24);
  if (!e) e = dalloc((void**)&dsd, (size_t)n * 8);
  if (!e) e = dalloc((void**)&dn, (size_t)n * 24);
  cudaStream_t st = sc->stream;
  if (!e && cudaMemcpyAsync(dp, points, (size_t)n * 24, cudaMemcpyHostToDevice, st) != cudaSuccess) e = ESF_ERR_CUDA;
  if (!e) {
    ESF_COUNTED k_rest_sdf_query<<<kblocks(n), KT, 0, st>>>(d->sdf, n, dp, safe_dist, dsd, dn);
    if (cudaGetLastError() != cudaSuccess) e = ESF_ERR_CUDA;
  }
  if (!e && (cudaMemcpyAsync(sd, dsd, (size_t)n * 8, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
             cudaMemcpyAsync(normals, dn, (size_t)n * 24, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
             cudaStreamSynchronize(st) != cudaSuccess))
    e = ESF_ERR_CUDA;
  if (e == ESF_ERR_CUDA) set_error("esf_rest_sdf_query: %s", cudaGetErrorString(cudaGetLastError()));
  cudaFree(dp);
  cudaFree(dsd);
  cudaFree(dn);
  return e;
}

extern "C" esf_status esf_set_fluid(esf_scene* s, double density, double viscosity) {
  if (!s) return ESF_ERR_INVALID_ARG;
  (void)viscosity;  // stored but unused by the reference (COUPLED_INTEGRATOR_3D.cpp:46)
  s->fluidDensity = density;
  return ESF_OK;
}
extern "C" esf_status esf_set_max_dt(esf_scene* s, double max_dt) {
  if (!s) return ESF_ERR_INVALID_ARG;
  s->defaultDt = max_dt;
  return ESF_OK;
}
extern "C" double esf_dt(const esf_scene* s) { return s ? s->dt : 0.0; }

// ------------------------------------------------------------ step pieces
static Box mkbox(int x0, int y0, int z0, int x1, int y1, int z1) {
  Box b;
  b.lo[0] = x0;
  b.lo[1] = y0;
  b.lo[2] = z0;
  b.hi[0] = x1;
  b.hi[1] = y1;
  b.hi[2] = z1;
  return b;
}
static long long boxn(const Box& b) {
  long long n = 1;
  for (int k = 0; k < 3; k++) n *= (b.hi[k] > b.lo[k]) ? (b.hi[k] - b.lo[k]) : 0;
  return n;
}

// computeSolidMass (DEFOR_SOLID_3D.cpp:576-669)
static esf_status compute_solid_mass(esf_scene* sc, Solid* d, int usesdf) {
  const GridDev& G = sc->g;
  cudaStream_t st = sc->stream;
  SolidDev& x = d->d;
  ESF_CUDA(cudaMemsetAsync(x.mass, 0, G.T * 8, st));
  ESF_CUDA(cudaMemsetAsync(x.valid, 0, G.R, st));
  ESF_CUDA(cudaMemsetAsync(x.detFInv, 0, G.T * 8, st));
  ESF_CUDA(cudaMemsetAsync(x.quarter, 0, G.T * 64, st));
  Box cells = mkbox(d->tmin[0], d->tmin[1], d->tmin[2], d->tmax[0] - 1, d->tmax[1] - 1, d->tmax[2] - 1);
  Box nodes = mkbox(d->tmin[0], d->tmin[1], d->tmin[2], d->tmax[0], d->tmax[1], d->tmax[2]);
  long long nc = boxn(cells);
  if (nc <= 0) return ESF_OK;
  const double subDh = sc->p.mass_sample_dh;
  const int res = (int)(G.dh / subDh);
  ESF_COUNTED k_det_finv<<<kblocks(nc), KT, 0, st>>>(G, x, cells);
  ESF_COUNTED k_mass_subsample<<<kblocks(nc, 128), 128, 0, st>>>(G, x, cells, usesdf, subDh, res);
  ESF_COUNTED k_mass_gather<<<kblocks(boxn(nodes)), KT, 0, st>>>(G, x, cells, nodes);
  ESF_LAUNCH_CHECK();
  return ESF_OK;
}

// One Gauss-Seidel sweep pass (sweepPhi when !VEC, sweepOnePass of the
// velocity when VEC): the cooperative hyperplane wave (k_sweep_wave, one
// launch per pass, sweepPhi) or the tile wavefront (k_sweep_tile, ~3n/8
// launches, the velocity passes, and sweepPhi where the device has no
// cooperative launch); ESF_SWEEP=wave or =tiles forces one for both. Both
// give the bits of the sequential loop. A wave whose
// grid barrier timed out raises the scene's sweep error word (dInts[42]),
// checked when the step or init ends.
constexpr int kSweepBar = 40, kSweepErr = 42;
constexpr int kFallbackCount = 44;  // mixed: cells of the FP32 stiffness evaluated again in FP64 (one per solid)
constexpr int kOverlap = 52;        // broad phase: two solids' meshes overlap
template <bool VEC>
static esf_status sweep_pass(esf_scene* sc, Solid* d, const Sweep& w, const unsigned long long* ranks) {
  cudaStream_t st = sc->stream;
  static const int coopBlocks = [] {
    int dev = 0, coop = 0, sms = 0, per = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (!coop || cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_sweep_wave<VEC>, SWEEP_THREADS, 0) !=
                     cudaSuccess)
      return 0;
    return sms * per;
  }();
  // sweepPhi's per-node work (FP64 square roots and divisions) makes its
  // critical path the cost: the wave (3n steps) beats the tiles (~9n
  // sub-plane steps), 23.3 against 37.6 ms for 2 x 8 passes per 256^3 step
  // (blocks of 32, 64 or 128 threads: the same). The velocity pass is a
  // blend of three values: there the wave's ~5 us per plane (grid barrier,
  // L2 round trips) costs more than the tiles' extra sub-planes in shared
  // memory, 37.6 against 21.1 ms for 4 x 8 passes. One cluster of 8 blocks
  // of 1024 threads with the hardware cluster barrier measured 82 ms for
  // sweepPhi: FP64 work of a plane on 8 SMs.
  const char* pick = getenv("ESF_SWEEP");
  const bool wave = pick ? strcmp(pick, "wave") == 0 : !VEC;
  double* f = VEC ? d->d.vel : nullptr;
  double* ph = d->d.phi;
  const double* ms = d->d.mass;
  if (coopBlocks > 0 && wave) {
    const long long nij = (long long)w.ni * w.nj;
    const int blocks = (int)std::min<long long>(coopBlocks, (nij + SWEEP_THREADS - 1) / SWEEP_THREADS);
    unsigned* bar = reinterpret_cast<unsigned*>(sc->dInts + kSweepBar);
    int* err = sc->dInts + kSweepErr;
    ESF_CUDA(cudaMemsetAsync(bar, 0, 2 * sizeof(unsigned), st));
    GridDev g = sc->g;
    Sweep ww = w;
    void* args[] = {&g, &f, &ph, (void*)&ms, &ww, (void*)&ranks, &bar, &err};
    note_launch();
    ESF_CUDA(cudaLaunchCooperativeKernel((const void*)k_sweep_wave<VEC>, dim3(blocks), dim3(SWEEP_THREADS),
                                         args, 0, st));
    return ESF_OK;
  }
  const int launches = sweep_tile_launches(w), blocks = sweep_tile_blocks(w);
  for (int P = 0; P < launches; P++)
    ESF_COUNTED k_sweep_tile<VEC><<<blocks, TILE_THREADS, 0, st>>>(sc->g, f, ph, ms, w, P, ranks);
  ESF_LAUNCH_CHECK();
  return ESF_OK;
}
// Reads the sweep error word (after the stream has been synchronised).
static esf_status check_sweeps(esf_scene* sc) {
  int e = 0;
  ESF_CUDA(cudaMemcpy(&e, sc->dInts + kSweepErr, sizeof e, cudaMemcpyDeviceToHost));
  if (e) {
    set_error("a sweep's grid barrier timed out");
    return ESF_ERR_CUDA;
  }
  return ESF_OK;
}

// computeSDF (DEFOR_SOLID_3D.cpp:216-268): phi, the boxes, 2 x sweepPhi.
static esf_status compute_sdf(esf_scene* sc, Solid* d) {
  const GridDev& G = sc->g;
  cudaStream_t st = sc->stream;
  int init[6] = {G.X, G.Y, G.Z, 0, 0, 0};
  memcpy(sc->hInts, init, sizeof init);
  ESF_CUDA(cudaMemcpyAsync(sc->dInts, sc->hInts, sizeof init, cudaMemcpyHostToDevice, st));
  double large = G.X + G.Y + G.Z + 2;
  TraceMarks tm(st);
  ESF_COUNTED k_phi_init<<<kblocks(G.T), 256, 0, st>>>(G, d->d, large, sc->dInts);
  ESF_LAUNCH_CHECK();
  ESF_CUDA(cudaMemcpyAsync(sc->hInts, sc->dInts, sizeof init, cudaMemcpyDeviceToHost, st));
  ESF_CUDA(cudaStreamSynchronize(st));
  tm.mark("sdf: phi and box");
  int xmin = sc->hInts[0], ymin = sc->hInts[1], zmin = sc->hInts[2];
  int xmax = sc->hInts[3], ymax = sc->hInts[4], zmax = sc->hInts[5];
  int tb = sc->p.tight_border, exn = sc->p.extrapolation_cells;
  d->tmin[0] = std::max(xmin - tb, 0);
  d->tmin[1] = std::max(ymin - tb, 0);
  d->tmin[2] = std::max(zmin - tb, 0);
  d->tmax[0] = std::min(xmax + tb, G.X);
  d->tmax[1] = std::min(ymax + tb, G.Y);
  d->tmax[2] = std::min(zmax + tb, G.Z);
  d->ex[0] = std::max(xmin - exn, 0);
  d->ex[1] = std::max(ymin - exn, 0);
  d->ex[2] = std::max(zmin - exn, 0);
  d->ex[3] = std::min(xmax + exn, G.X);
  d->ex[4] = std::min(ymax + exn, G.Y);
  d->ex[5] = std::min(zmax + exn, G.Z);
  Box ex = mkbox(d->ex[0], d->ex[1], d->ex[2], d->ex[3], d->ex[4], d->ex[5]);
  // 2 x sweepPhi: 8 passes each, every pass a wavefront of 8^3 tiles
  for (int rep = 0; rep < 2; rep++)
    for (int dir = 0; dir < 8; dir++) {
      Sweep w;
      w.dj = (dir & 1) ? -1 : 1;
      w.di = (dir & 2) ? -1 : 1;
      w.dk = (dir & 4) ? -1 : 1;
      w.i0 = w.di > 0 ? ex.lo[0] + 1 : ex.hi[0] - 2;
      w.j0 = w.dj > 0 ? ex.lo[1] + 1 : ex.hi[1] - 2;
      w.k0 = w.dk > 0 ? ex.lo[2] + 1 : ex.hi[2] - 2;
      w.ni = ex.hi[0] - ex.lo[0] - 1;
      w.nj = ex.hi[1] - ex.lo[1] - 1;
      w.nk = ex.hi[2] - ex.lo[2] - 1;
      if (w.ni <= 0 || w.nj <= 0 || w.nk <= 0) continue;
      TRY(sweep_pass<false>(sc, d, w, nullptr));
    }
  ESF_LAUNCH_CHECK();
  tm.mark("sdf: 2 x sweepPhi");
  return ESF_OK;
}

// MT19937 stream shared by every initMaterialParticles call (the reference
// re-seeds a fresh MERSENNETWISTER with 123456 each time, MERSENNETWISTER.h:259-262).
static esf_status ensure_mt(esf_scene* sc, long long need) {
  if (need <= sc->mtLen) return ESF_OK;
  long long len = need + need / 2 + 1024;
  std::vector<uint32_t> h(len);
  uint32_t mt[624];
  mt[0] = 123456u;
  for (int i = 1; i < 624; i++) mt[i] = 1812433253u * (mt[i - 1] ^ (mt[i - 1] >> 30)) + (uint32_t)i;
  int idx = 624;
  for (long long k = 0; k < len; k++) {
    if (idx >= 624) {
      for (int i = 0; i < 624; i++) {
        uint32_t y = (mt[i] & 0x80000000u) | (mt[(i + 1) % 624] & 0x7fffffffu);
        mt[i] = mt[(i + 397) % 624] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
      }
      idx = 0;
    }
    uint32_t y = mt[idx++];
    y ^= y >> 11;
    y ^= (y << 7) & 0x9d2c5680u;
    y ^= (y << 15) & 0xefc60000u;
    y ^= y >> 18;
    h[k] = y;
  }
  TRY(sc->mt.ensure(len * 4));
  ESF_CUDA(cudaMemcpyAsync(sc->mt.p, h.data(), len * 4, cudaMemcpyHostToDevice, sc->stream));
  ESF_CUDA(cudaStreamSynchronize(sc->stream));
  sc->mtLen = len;
  return ESF_OK;
}

// valid==1 cells of the tight box in z,y,x order (list + per-cell ordinal)
static esf_status collect_valid_cells(esf_scene* sc, Solid* d) {
  const GridDev& G = sc->g;
  cudaStream_t st = sc->stream;
  Box cells = mkbox(d->tmin[0], d->tmin[1], d->tmin[2], d->tmax[0] - 1, d->tmax[1] - 1, d->tmax[2] - 1);
  long long nc = boxn(cells);
  d->nValid = 0;
  if (nc <= 0) return ESF_OK;
  TRY(d->cellFlag.ensure(nc * 4));
  TRY(d->cellScan.ensure((nc + 1) * 4));
  ESF_COUNTED k_flag_valid_cells<<<kblocks(nc), KT, 0, st>>>(G, d->d, cells, d->cellFlag.as<int>());
  size_t tb = 0;
  cub::DeviceScan::ExclusiveSum(nullptr, tb, d->cellFlag.as<int>(), d->cellScan.as<int>(), (int)nc, st);
  TRY(sc->cubTmp.ensure(tb));
  cub::DeviceScan::ExclusiveSum(sc->cubTmp.p, tb, d->cellFlag.as<int>(), d->cellScan.as<int>(), (int)nc, st);
  ESF_CUDA(cudaMemcpyAsync(&sc->hInts[0], d->cellScan.as<int>() + nc - 1, 4, cudaMemcpyDeviceToHost, st));
  ESF_CUDA(cudaMemcpyAsync(&sc->hInts[1], d->cellFlag.as<int>() + nc - 1, 4, cudaMemcpyDeviceToHost, st));
  ESF_CUDA(cudaStreamSynchronize(st));
  d->nValid = (long long)sc->hInts[0] + sc->hInts[1];
  TRY(d->cellList.ensure((d->nValid + 1) * 8));
  ESF_COUNTED k_collect_valid_cells<<<kblocks(nc), KT, 0, st>>>(G, cells, d->cellFlag.as<int>(), d->cellScan.as<int>(),
                                                    d->cellList.as<long long>());
  ESF_LAUNCH_CHECK();
  return ESF_OK;
}

// initMaterialParticles (DEFOR_SOLID_3D.cpp:333-367)
static esf_status init_particles(esf_scene* sc, Solid* d) {
  TRY(collect_valid_cells(sc, d));
  const int ppc = sc->p.particles_per_cell;
  d->np = d->nValid * ppc;
  if (d->np == 0) return ESF_OK;
  TRY(ensure_mt(sc, 3 * d->np));
  TRY(d->part.ensure(d->np * 80));
  ESF_COUNTED k_seed_particles<<<kblocks(d->np), KT, 0, sc->stream>>>(sc->g, d->d, d->cellList.as<long long>(),
                                                           d->nValid, ppc, sc->mt.as<uint32_t>(),
                                                           d->pmass, d->part.as<double>());
  ESF_LAUNCH_CHECK();
  return ESF_OK;
}

static esf_status advect_mesh(esf_scene* sc, Solid* d) {
  ESF_COUNTED k_advect_mesh<<<kblocks(d->nv), KT, 0, sc->stream>>>(sc->g, d->d, d->nv, d->dVerts, d->dRest);
  ESF_LAUNCH_CHECK();
  return ESF_OK;
}

// gatherSolidMasses (COUPLED_INTEGRATOR_3D.cpp:327-375)
static esf_status gather_solid_masses(esf_scene* sc) {
  const GridDev& G = sc->g;
  cudaStream_t st = sc->stream;
  for (int i = 0; i < sc->ns; i++)
    ESF_COUNTED k_gather_accumulate<<<kblocks(G.T), KT, 0, st>>>(G, sc->s[i]->d, i == 0, sc->solidMass, sc->quarter);
  ESF_COUNTED k_node_vf<<<kblocks(G.T), KT, 0, st>>>(G, sc->quarter, sc->solidMass, sc->nodeVF, sc->nodeFlag);
  size_t tb = 0;
  cub::DeviceScan::ExclusiveSum(nullptr, tb, sc->nodeFlag, sc->nodeScan, (int)G.T, st);
  TRY(sc->cubTmp.ensure(tb));
  cub::DeviceScan::ExclusiveSum(sc->cubTmp.p, tb, sc->nodeFlag, sc->nodeScan, (int)G.T, st);
  ESF_CUDA(cudaMemcpyAsync(&sc->hInts[0], sc->nodeScan + G.T - 1, 4, cudaMemcpyDeviceToHost, st));
  ESF_CUDA(cudaMemcpyAsync(&sc->hInts[1], sc->nodeFlag + G.T - 1, 4, cudaMemcpyDeviceToHost, st));
  ESF_CUDA(cudaStreamSynchronize(st));
  long long S = (long long)sc->hInts[0] + sc->hInts[1];
  TRY(sc->sNode.ensure((S + 1) * 8));
  ESF_COUNTED k_sdof<<<kblocks(G.T), KT, 0, st>>>(G, sc->nodeFlag, sc->nodeScan, sc->sdof, sc->sNode.as<long long>());
  ESF_LAUNCH_CHECK();
  sc->S = S;
  return ESF_OK;
}

static esf_status recover_velocity(esf_scene* sc) {
  for (int i = 0; i < sc->ns; i++) {
    Solid* d = sc->s[i];
    Box b = mkbox(d->ex[0], d->ex[1], d->ex[2], d->ex[3] - 1, d->ex[4] - 1, d->ex[5] - 1);
    if (boxn(b) > 0)
      ESF_COUNTED k_recover_velocity<<<kblocks(boxn(b)), KT, 0, sc->stream>>>(sc->g, d->d, b, sc->vel);
  }
  ESF_LAUNCH_CHECK();
  return ESF_OK;
}

extern "C" esf_status esf_init(esf_scene* sc) {
  if (!sc) return ESF_ERR_INVALID_ARG;
  if (sc->inited || sc->ns == 0) {
    set_error("esf_init: needs at least one solid and may run once");
    return ESF_ERR_STATE;
  }
  if (!(sc->p.mass_sample_dh > 0) || (int)(sc->g.dh / sc->p.mass_sample_dh) < 1 ||
      sc->p.particles_per_cell < 1) {
    set_error("esf_init: invalid mass sample dh or particle count");
    return ESF_ERR_INVALID_ARG;
  }
  cudaSetDevice(sc->device);
  const GridDev& G = sc->g;
  ESF_CUDA(cudaMemsetAsync(sc->dInts + kSweepErr, 0, sizeof(int), sc->stream));
  // DEFOR_SOLID_3D::init (DEFOR_SOLID_3D.cpp:269-331)
  for (int i = 0; i < sc->ns; i++) {
    Solid* d = sc->s[i];
    d->ex[0] = d->ex[1] = d->ex[2] = 0;
    d->ex[3] = G.X;
    d->ex[4] = G.Y;
    d->ex[5] = G.Z;
    d->tmin[0] = d->tmin[1] = d->tmin[2] = 0;
    d->tmax[0] = G.X;
    d->tmax[1] = G.Y;
    d->tmax[2] = G.Z;
    TRY(compute_solid_mass(sc, d, 0));
    TRY(compute_sdf(sc, d));
    TRY(init_particles(sc, d));
    TRY(advect_mesh(sc, d));
  }
  TRY(gather_solid_masses(sc));
  TRY(recover_velocity(sc));
  ESF_CUDA(cudaStreamSynchronize(sc->stream));
  TRY(check_sweeps(sc));
  sc->inited = true;
  return ESF_OK;
}

static double u64_to_double(unsigned long long b) {
  b = (b >> 63) ? (b & 0x7fffffffffffffffull) : ~b;
  double d;
  memcpy(&d, &b, 8);
  return d;
}

// cell -> valid-cell ordinal map of solid i (solid 0 uses the scene's)
static int* solid_ord(esf_scene* sc, int i) {
  if (i == 0) return sc->cellOrd;
  Solid* d = sc->s[i];
  if (d->ord.ensure((size_t)sc->g.R * 4) != ESF_OK) return nullptr;
  return d->ord.as<int>();
}

// stiffness + computeMV + assembly (DEFOR_SOLID_3D.cpp:697-889;
// COUPLED_INTEGRATOR_3D.cpp:432-437, 609-620 for the assembly)
static esf_status solid_system(esf_scene* sc, double* energyOut) {
  const GridDev& G = sc->g;
  cudaStream_t st = sc->stream;
  const long long S = sc->S;
  sc->Sstep = S;
  TRY(sc->solidF.ensure((3 * S + 1) * 8));
  TRY(sc->solidMv.ensure((3 * S + 1) * 8));
  TRY(sc->damped.ensure((3 * S + 1) * 8));
  TRY(sc->solidV0.ensure((3 * S + 1) * 8));
  TRY(sc->solidPC.ensure((3 * S + 1) * 8));
  TRY(sc->solidB1.ensure((3 * S + 1) * 8));
  TRY(sc->sysDiag.ensure((3 * S + 1) * 8));
  TRY(sc->blocks.ensure((243 * rows32(S) + 1) * 8));
  TRY(sc->nbr.ensure((27 * rows32(S) + 1) * 4));
  TRY(sc->mask.ensure((S + 1) * 4));
  ESF_CUDA(cudaMemsetAsync(sc->solidF.p, 0, 3 * S * 8 + 8, st));
  ESF_CUDA(cudaMemsetAsync(sc->solidMv.p, 0, 3 * S * 8 + 8, st));
  ESF_CUDA(cudaMemsetAsync(sc->damped.p, 0, 3 * S * 8 + 8, st));
  ESF_CUDA(cudaMemsetAsync(sc->mask.p, 0, S * 4 + 4, st));
  const int EB = 4096;
  // energy partials, 4 x EB per solid: stiffness, mass-weighted velocity,
  // body forces (solid 0's region only), FP64 fallback cells of the mixed
  // path's FP32 stiffness
  TRY(sc->energy.ensure((size_t)EB * 4 * 8 * (sc->ns > 0 ? sc->ns : 1)));
  ESF_CUDA(cudaMemsetAsync(sc->energy.p, 0, (size_t)EB * 4 * 8 * (sc->ns > 0 ? sc->ns : 1), st));
  // element matrices and forces of all solids, concatenated in solid order
  long long totalCells = 0;
  for (int i = 0; i < sc->ns; i++) totalCells += sc->s[i]->nValid;
  TRY(sc->Ke.ensure((576 * totalCells + 1) * 8));
  TRY(sc->nf.ensure((24 * totalCells + 1) * 8));
  sc->validCells = totalCells;
  sc->mfCells = 0;
  long long keBase = 0;
  for (int i = 0; i < sc->ns; i++) {
    Solid* d = sc->s[i];
    double* ePart = sc->energy.as<double>() + (size_t)4 * EB * i;
    int* ord = solid_ord(sc, i);
    if (!ord) return ESF_ERR_OOM;
    ESF_CUDA(cudaMemsetAsync(ord, 0xff, G.R * 4, st));
    const long long nc = d->nValid;
    sc->hInts[kFallbackCount + i] = 0;
    double* Ke = sc->Ke.as<double>() + 576 * keBase;
    double* nf = sc->nf.as<double>() + 24 * keBase;
    // mixed precision, elastic, one solid: record the matrix-free operator's
    // per-cell data (ESF_SOLID_ASSEMBLED=1 keeps the FP32 copy of the
    // assembled blocks, as scenes with several solids do)
    const bool mf = sc->ns == 1 && nc > 0 && sc->p.precision != ESF_FP64 && !d->d.plastic &&
                    !getenv("ESF_SOLID_ASSEMBLED");
    d->d.mf = nullptr;
    d->d.mfCells = 0;
    if (mf) {
      TRY(sc->mfCell.ensure((size_t)MF_PLANES * nc * 4));
      TRY(sc->mfCorner.ensure((size_t)8 * nc * 4));
      d->d.mf = sc->mfCell.as<float>();
      d->d.mfCells = nc;
      sc->mfCells = nc;
      ESF_COUNTED k_mf_corners<<<kblocks(nc), KT, 0, st>>>(G, d->cellList.as<long long>(), nc, sc->sdof,
                                                          sc->mfCorner.as<int>());
    }
    if (nc > 0 && d->d.plastic) {
      TRY(d->fpUpd.ensure(nc * 4));
      TRY(d->fpVal.ensure(nc * 72));
      d->d.updIdx = d->fpUpd.as<int>();
      d->d.updVal = d->fpVal.as<double>();
    }
    if (nc > 0 && sc->p.precision != ESF_FP64 && !d->d.plastic) {
      // stress and stiffness in FP32; near-degenerate cells again in FP64
      TRY(sc->fbCells.ensure(nc * 8));
      TRY(sc->fbSlot.ensure(nc * 8));
      ESF_CUDA(cudaMemsetAsync(sc->dInts + kFallbackCount, 0, sizeof(int), st));
      unsigned* fbCount = reinterpret_cast<unsigned*>(sc->dInts + kFallbackCount);
      ESF_COUNTED k_element_stiffness_f32<<<kblocks(nc, 128), 128, 0, st>>>(
          G, d->d, d->cellList.as<long long>(), nc, Ke, nf, ePart, sc->fbCells.as<long long>(),
          sc->fbSlot.as<long long>(), fbCount);
      ESF_COUNTED k_element_stiffness<<<kblocks(nc, 128), 128, 0, st>>>(
          G, d->d, sc->fbCells.as<long long>(), nc, Ke, nf, ePart + 3 * EB, sc->fbSlot.as<long long>(), fbCount);
      ESF_CUDA(cudaMemcpyAsync(&sc->hInts[kFallbackCount + i], fbCount, sizeof(int), cudaMemcpyDeviceToHost, st));
    } else if (nc > 0) {
      ESF_COUNTED k_element_stiffness<<<kblocks(nc, 128), 128, 0, st>>>(G, d->d, d->cellList.as<long long>(), nc,
                                                             Ke, nf, ePart, nullptr, nullptr);
    }
    if (nc > 0) {
      if (d->d.plastic) {
        ESF_CUDA(cudaMemsetAsync(d->fpWin.p, 0xff, d->pn * 4, st));
        ESF_COUNTED k_fp_winner<<<kblocks(nc), KT, 0, st>>>(d->d.updIdx, nc, d->fpWin.as<int>());
        ESF_COUNTED k_fp_apply<<<kblocks(nc), KT, 0, st>>>(d->d.updIdx, d->d.updVal, nc, d->fpWin.as<int>(),
                                                           d->d.FpInv);
      }
      // cell -> ordinal in the valid list
      ESF_COUNTED k_cell_ord_fill<<<kblocks(nc), KT, 0, st>>>(G, d->cellList.as<long long>(), nc, ord);
    }
    Box b = mkbox(d->ex[0], d->ex[1], d->ex[2], d->ex[3] - 1, d->ex[4] - 1, d->ex[5] - 1);
    if (boxn(b) > 0 && S > 0)
      ESF_COUNTED k_compute_mv<<<std::min(kblocks(boxn(b)), EB), KT, 0, st>>>(G, d->d, b, sc->sdof,
                                                                  sc->solidMv.as<double>(), ePart + EB);
    ESF_LAUNCH_CHECK();
    keBase += nc;
  }
  *energyOut = 0;
  return ESF_OK;
}

static double sum_partials(esf_scene* sc, int n) {
  std::vector<double> h(n);
  // the scene stream is non-blocking: copy on it, then wait for it
  cudaMemcpyAsync(h.data(), sc->energy.p, n * 8, cudaMemcpyDeviceToHost, sc->stream);
  cudaStreamSynchronize(sc->stream);
  double a = 0;
  for (double v : h) a += v;
  return a;
}

extern "C" esf_status esf_step(esf_scene* sc, esf_step_report* rep) {
  if (!sc) return ESF_ERR_INVALID_ARG;
  if (!sc->inited) {
    set_error("esf_step: call esf_init first");
    return ESF_ERR_STATE;
  }
  if (sc->failed) {
    set_error("esf_step: a solve of an earlier step met NaN/Inf; restore a state with esf_read_frame first");
    return ESF_ERR_STATE;
  }
  for (int i = 0; i < sc->ns && sc->ns > 1; i++)
    if (!sc->s[i]->hasSdf) {
      set_error("esf_step: solid %d has no rest SDF; scenes with several solids need one per solid for "
                "solid-solid contact (esf_solid_load_rest_sdf)", i);
      return ESF_ERR_STATE;
    }
  cudaSetDevice(sc->device);
  const GridDev& G = sc->g;
  cudaStream_t st = sc->stream;
  sc->status = ESF_OK;
  ESF_CUDA(cudaMemsetAsync(sc->dInts + kSweepErr, 0, sizeof(int), st));
  ESF_CUDA(cudaEventRecord(sc->e0, st));
  ESF_CUDA(cudaEventRecord(sc->ph[0], st));
  // ---- broad phase (COUPLED_INTEGRATOR_3D.cpp:378-411)
  int prone = 0;
  for (int i = 0; i < sc->ns && !prone; i++) {
    Solid* d = sc->s[i];
    unsigned long long init[6] = {~0ull, ~0ull, ~0ull, 0, 0, 0};
    memcpy(sc->hU64, init, sizeof init);
    ESF_CUDA(cudaMemcpyAsync(sc->dU64, sc->hU64, sizeof init, cudaMemcpyHostToDevice, st));
    ESF_COUNTED k_mesh_aabb<<<kblocks(3LL * d->ntri), KT, 0, st>>>(d->ntri, d->dTris, d->dVerts, sc->dU64);
    ESF_CUDA(cudaMemcpyAsync(sc->hU64, sc->dU64, sizeof init, cudaMemcpyDeviceToHost, st));
    ESF_CUDA(cudaStreamSynchronize(st));
    double mn[3], mx[3];
    for (int k = 0; k < 3; k++) {
      mn[k] = u64_to_double(sc->hU64[k]);
      mx[k] = u64_to_double(sc->hU64[3 + k]);
    }
    bool inside = true;
    for (int k = 0; k < 3; k++)
      if (mn[k] < d->safeMin[k] || mn[k] > d->safeMax[k] || mx[k] < d->safeMin[k] || mx[k] > d->safeMax[k])
        inside = false;
    if (!inside) prone = 1;
  }
  // solids close to one another (:394-404): the first pair whose meshes'
  // triangle boxes overlap
  for (int i = 0; i + 1 < sc->ns && !prone; i++)
    for (int j = i + 1; j < sc->ns && !prone; j++) {
      Solid *a = sc->s[i], *b = sc->s[j];
      int* hit = sc->dInts + kOverlap;
      ESF_CUDA(cudaMemsetAsync(hit, 0, sizeof(int), st));
      const long long pairs = (long long)a->ntri * b->ntri;
      ESF_COUNTED k_mesh_pair_overlap<<<kblocks(pairs), KT, 0, st>>>(a->ntri, a->dTris, a->dVerts, b->ntri,
                                                                     b->dTris, b->dVerts, hit);
      ESF_LAUNCH_CHECK();
      ESF_CUDA(cudaMemcpyAsync(&sc->hInts[kOverlap], hit, sizeof(int), cudaMemcpyDeviceToHost, st));
      ESF_CUDA(cudaStreamSynchronize(st));
      if (sc->hInts[kOverlap]) prone = 1;
    }
  // CFL (:88-102)
  sc->hU64[0] = 0;
  ESF_CUDA(cudaMemcpyAsync(sc->dU64, sc->hU64, 8, cudaMemcpyHostToDevice, st));
  ESF_COUNTED k_cfl_vmax<<<kblocks(G.T), KT, 0, st>>>(G, sc->vel, sc->solidMass, sc->dU64);
  ESF_CUDA(cudaMemcpyAsync(sc->hU64, sc->dU64, 8, cudaMemcpyDeviceToHost, st));
  ESF_CUDA(cudaStreamSynchronize(st));
  {
    double vm;
    memcpy(&vm, sc->hU64, 8);
    double alpha = prone ? 0.6 : 1.8;
    double dt = 1e9;
    if (sc->S > 0) {
      double vmax = vm * G.dhInv;
      double c = alpha / vmax;
      dt = (c < dt) ? c : dt;
    }
    sc->dt = (sc->defaultDt < dt) ? sc->defaultDt : dt;
  }
  const double dt = sc->dt;
  const long long S = sc->S;
  ESF_CUDA(cudaEventRecord(sc->ph[1], st));
  // ---- solid forces, stiffness, mv
  double e_unused;
  TRY(solid_system(sc, &e_unused));
  const int EB = 4096;
  double* ePart = sc->energy.as<double>();
  // ---- vorticity + body forces (:442-606)
  ESF_CUDA(cudaMemsetAsync(sc->ws, 0, G.T * 8, st));
  if (sc->vortEps > 0) ESF_COUNTED k_vorticity<<<kblocks(G.T), KT, 0, st>>>(G, sc->nodeVF, sc->vel, sc->vort, sc->ws);
  // The reference adds the stiffness forces before the body forces, so the
  // block/force gather runs first; the damped mass it needs for the diagonal
  // comes from the body-force kernel and is added afterwards.
  BodyParams bp;
  bp.fluidDensity = sc->fluidDensity;
  bp.gravity = sc->p.gravity;
  bp.buoyancy = sc->p.buoyancy;
  bp.damp = 1 + dt * sc->p.rayleigh_alpha;
  bp.vortEps = sc->vortEps;
  bp.dt = dt;
  const double scale = dt * dt + sc->p.rayleigh_beta * dt;
  if (S > 0) {
    // forces + blocks (diagonal mass added in a second pass, below)
    SolidSet ss;
    memset(&ss, 0, sizeof ss);
    ss.n = sc->ns;
    long long base = 0;
    for (int i = 0; i < sc->ns; i++) {
      ss.mass[i] = sc->s[i]->d.mass;
      ss.ord[i] = solid_ord(sc, i);
      ss.keBase[i] = base;
      base += sc->s[i]->nValid;
    }
    ESF_COUNTED k_assemble<<<kblocks(S * 27), KT, 0, st>>>(G, ss, sc->sdof, sc->sNode.as<long long>(), S,
                                                sc->Ke.as<double>(), sc->nf.as<double>(), scale,
                                                sc->blocks.as<double>(),
                                                sc->nbr.as<int>(), sc->mask.as<int>(), sc->solidF.as<double>());
  }
  ESF_CUDA(cudaEventRecord(sc->ph[2], st));
  ESF_COUNTED k_body_forces<<<EB, KT, 0, st>>>(G, bp, sc->nodeVF, sc->solidMass, sc->vel, sc->intensity, sc->vort,
                                   sc->ws, sc->sdof, sc->uf, sc->mvf, sc->minv, sc->damped.as<double>(),
                                   sc->solidMv.as<double>(), sc->solidF.as<double>(), ePart + 2 * EB);
  ESF_LAUNCH_CHECK();
  if (S > 0) {
    ESF_COUNTED k_add_diag<<<kblocks(S), KT, 0, st>>>(S, sc->damped.as<double>(), sc->blocks.as<double>(),
                                          sc->sysDiag.as<double>());
    ESF_LAUNCH_CHECK();
  }
  double energy = sum_partials(sc, 4 * EB * (sc->ns > 0 ? sc->ns : 1));
  // ---- pcrImplicitSolve (:662-764)
  int it[3] = {0, 0, 0}, cv[3] = {0, 0, 0}, rf[3] = {0, 0, 0}, it64 = 0;
  double rr[3] = {0, 0, 0};
  const int prec = sc->p.precision;
  if (!sc->sw || solid_work_capacity(sc->sw) < S) {
    solid_work_free(sc->sw);
    sc->sw = nullptr;
    TRY(solid_work_alloc(&sc->sw, S + S / 4 + 16, prec != ESF_FP64));
  }
  TRY(solid_work_set_matrix_free(sc->sw, G, sc->mfCells, sc->mfCells ? sc->mfCell.as<float>() : nullptr,
                                 sc->mfCorner.as<int>(), sc->sNode.as<long long>(), sc->cellOrd,
                                 sc->ns ? sc->s[0]->d.mu : 0.0, sc->ns ? sc->s[0]->d.lambda : 0.0, scale));
  esf_status es = ESF_OK;
  // A solve that met NaN/Inf ends the step there: nothing downstream (the
  // velocity update, particles, advection) runs on non-finite values. The
  // report carries what was done; the scene refuses further steps until a
  // state is restored (esf_read_frame).
  auto numeric_stop = [&]() -> esf_status {
    cudaStreamSynchronize(st);
    sc->failed = true;
    if (rep) {
      memset(rep, 0, sizeof *rep);
      rep->dt = dt;
      rep->energy = energy;
      for (int k = 0; k < 3; k++) {
        rep->iterations[k] = it[k];
        rep->converged[k] = cv[k];
        rep->rel_residual[k] = rr[k];
        rep->refinements[k] = rf[k];
      }
      rep->prone_to_contact = prone;
      rep->fp64_iterations = it64;
      rep->status = ESF_ERR_NUMERIC;
    }
    set_error("esf_step: NaN/Inf met in a solve; the step stopped after it");
    return ESF_ERR_NUMERIC;
  };
  ESF_CUDA(cudaEventRecord(sc->ph[3], st));
  if (S > 0) {
    es = solid_solve(sc->sw, S, sc->blocks.as<double>(), sc->nbr.as<int>(), sc->sysDiag.as<double>(),
                     sc->solidF.as<double>(), sc->solidV0.as<double>(), sc->p.implicit_solver_eps,
                     sc->p.cr_max_iterations, prec, sc->p.inner_eps, sc->p.max_refinements, &it[0],
                     &rr[0], &rf[0], &cv[0], st, sc->damped.as<double>());
    if (es == ESF_ERR_NUMERIC) return numeric_stop();
    if (es) return es;
  }
  ESF_CUDA(cudaEventRecord(sc->ph[4], st));
  ESF_COUNTED k_vstar<<<kblocks(G.T), KT, 0, st>>>(G, sc->sdof, sc->uf, sc->minv, sc->solidV0.as<double>(), sc->vstar);
  ESF_COUNTED k_cell_rhs<<<kblocks(G.R), KT, 0, st>>>(G, sc->vel, sc->vstar, sc->minv, sc->rhs, sc->jdiag, sc->b1);
  ESF_LAUNCH_CHECK();
  es = pressure_solve(sc->pw, G, sc->minv, sc->jdiag, sc->b1, sc->lambda, sc->p.div_free_solver_eps,
                      sc->p.cr_max_iterations, prec, sc->p.inner_eps, sc->p.max_refinements, &it[1],
                      &rr[1], &rf[1], &cv[1], st, &it64);
  if (es == ESF_ERR_NUMERIC) return numeric_stop();
  if (es) return es;
  ESF_CUDA(cudaEventRecord(sc->ph[5], st));
  if (S > 0) {
    ESF_COUNTED k_solid_b1<<<kblocks(S), KT, 0, st>>>(G, sc->sNode.as<long long>(), S, sc->lambda, sc->solidB1.as<double>());
    ESF_LAUNCH_CHECK();
    es = solid_solve(sc->sw, S, sc->blocks.as<double>(), sc->nbr.as<int>(), sc->sysDiag.as<double>(),
                     sc->solidB1.as<double>(), sc->solidPC.as<double>(), sc->p.implicit_solver_eps,
                     sc->p.cr_max_iterations, prec, sc->p.inner_eps, sc->p.max_refinements, &it[2],
                     &rr[2], &rf[2], &cv[2], st, sc->damped.as<double>());
    if (es == ESF_ERR_NUMERIC) return numeric_stop();
    if (es) return es;
  }
  ESF_COUNTED k_velocity_update<<<kblocks(G.T), KT, 0, st>>>(G, sc->sdof, sc->lambda, sc->minv, sc->solidPC.as<double>(),
                                                 sc->vstar, sc->pc, sc->v1, sc->vel);
  ESF_LAUNCH_CHECK();
  ESF_CUDA(cudaEventRecord(sc->ph[6], st));
  // ---- finalizeSolution (:828-917)
  ContactParams cp;
  cp.wallThickness = sc->p.wall_thickness;
  cp.spring = sc->p.contact_spring_stiffness;
  cp.friction = sc->p.friction;
  cp.alpha = sc->p.flip_alpha;
  cp.bnd[0] = G.o[0];
  cp.bnd[1] = G.o[1];
  cp.bnd[2] = G.o[2];
  cp.bnd[3] = G.o[0] + G.dh * (G.X - 1);
  cp.bnd[4] = G.o[1] + G.dh * (G.Y - 1);
  cp.bnd[5] = G.o[2] + G.dh * (G.Z - 1);
  for (int i = 0; i < sc->ns; i++) {  // DEFOR_SOLID_3D::finalizeSolution(v, dt) (:1182-1197)
    Solid* d = sc->s[i];
    Box ex = mkbox(d->ex[0], d->ex[1], d->ex[2], d->ex[3], d->ex[4], d->ex[5]);
    if (boxn(ex) > 0) ESF_COUNTED k_copy_grid_velocity<<<kblocks(boxn(ex)), KT, 0, st>>>(G, d->d, ex, sc->vel);
    d->d.dt = dt;
  }
  TRY(sc->contactCount.ensure(8));
  ESF_CUDA(cudaMemsetAsync(sc->contactCount.p, 0, 8, st));
  for (int i = 0; i < sc->ns; i++) {  // gridToParticle, with the other solids as contact neighbours
    Solid* d = sc->s[i];
    ContactSet cs;
    memset(&cs, 0, sizeof cs);
    cs.thickness = sc->p.contact_safe_distance;
    cs.contacts = sc->contactCount.as<unsigned long long>();
    for (int j = 0; j < sc->ns; j++) {
      if (j == i) continue;
      Solid* o = sc->s[j];
      if (!o->hasSdf) {
        set_error("esf_step: solid %d has no rest SDF; scenes with several solids need one per solid "
                  "(esf_solid_load_rest_sdf)", j);
        return ESF_ERR_STATE;
      }
      ContactNeighbor& nb = cs.nb[cs.n++];
      nb.phi = o->d.phi;
      nb.X = o->d.X;
      nb.vel = o->d.vel;
      nb.sdf = o->sdf;
    }
    if (d->np > 0)
      ESF_COUNTED k_grid_to_particle<<<kblocks(d->np), KT, 0, st>>>(G, d->d, d->np, d->part.as<double>(), cp, cs);
  }
  ESF_CUDA(cudaEventRecord(sc->ph[7], st));
  for (int i = 0; i < sc->ns; i++) {  // particleToGrid
    Solid* d = sc->s[i];
    TraceMarks tm(st);
    ESF_CUDA(cudaMemsetAsync(d->d.mass, 0, G.T * 8, st));
    if (d->np == 0) continue;
    const long long np = d->np;
    const unsigned int nkeys = (unsigned int)((long long)(G.X + 3) * (G.Y + 3) * (G.Z + 3));
    TRY(sc->keys.ensure(np * 4));
    TRY(sc->vals.ensure(np * 4));
    TRY(sc->skeys.ensure(np * 4));
    TRY(sc->svals.ensure(np * 4));
    TRY(sc->bstart.ensure((size_t)nkeys * 4));
    TRY(sc->bend.ensure((size_t)nkeys * 4));
    TRY(sc->pweights.ensure((size_t)np * 96));
    int pinit[6] = {1 << 30, 1 << 30, 1 << 30, -(1 << 30), -(1 << 30), -(1 << 30)};
    memcpy(sc->hInts, pinit, sizeof pinit);
    ESF_CUDA(cudaMemcpyAsync(sc->dInts, sc->hInts, sizeof pinit, cudaMemcpyHostToDevice, st));
    ESF_COUNTED k_p2g_keys<<<kblocks(np), 256, 0, st>>>(G, np, d->part.as<double>(), sc->keys.as<unsigned int>(),
                                           sc->vals.as<unsigned int>(), sc->dInts, sc->pweights.as<double>());
    tm.mark("p2g: keys and weights");
    int bits = 1;
    while (bits < 32 && (1ull << bits) <= nkeys) bits++;
    size_t tb = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, tb, sc->keys.as<unsigned int>(), sc->skeys.as<unsigned int>(),
                                    sc->vals.as<unsigned int>(), sc->svals.as<unsigned int>(), (int)np, 0, bits, st);
    TRY(sc->cubTmp.ensure(tb));
    cub::DeviceRadixSort::SortPairs(sc->cubTmp.p, tb, sc->keys.as<unsigned int>(), sc->skeys.as<unsigned int>(),
                                    sc->vals.as<unsigned int>(), sc->svals.as<unsigned int>(), (int)np, 0, bits, st);
    tm.mark("p2g: sort");
    ESF_CUDA(cudaMemsetAsync(sc->bstart.p, 0, (size_t)nkeys * 4, st));
    ESF_CUDA(cudaMemsetAsync(sc->bend.p, 0, (size_t)nkeys * 4, st));
    ESF_COUNTED k_bucket_bounds<<<kblocks(np), KT, 0, st>>>(np, sc->skeys.as<unsigned int>(), sc->bstart.as<int>(),
                                                sc->bend.as<int>(), nkeys);
    ESF_CUDA(cudaMemcpyAsync(sc->hInts, sc->dInts, sizeof pinit, cudaMemcpyDeviceToHost, st));
    ESF_CUDA(cudaStreamSynchronize(st));
    Box nb = mkbox(std::max(sc->hInts[0], 0), std::max(sc->hInts[1], 0), std::max(sc->hInts[2], 0),
                   std::min(sc->hInts[3] + 4, G.X), std::min(sc->hInts[4] + 4, G.Y), std::min(sc->hInts[5] + 4, G.Z));
    tm.mark("p2g: bucket bounds");
    if (boxn(nb) > 0)
      ESF_COUNTED k_p2g_gather<<<kblocks(boxn(nb)), KT, 0, st>>>(G, d->d, nb, d->part.as<double>(), sc->pweights.as<double>(), sc->svals.as<unsigned int>(),
                                                     sc->bstart.as<int>(), sc->bend.as<int>(), sc->p.flip_cutoff);
    ESF_LAUNCH_CHECK();
    tm.mark("p2g: gather");
  }
  ESF_CUDA(cudaEventRecord(sc->ph[8], st));
  for (int i = 0; i < sc->ns; i++) {  // extendVectorField = 4 x sweepVectorField
    Solid* d = sc->s[i];
    Box ex = mkbox(d->ex[0], d->ex[1], d->ex[2], d->ex[3], d->ex[4], d->ex[5]);
    if (ex.hi[0] - ex.lo[0] < 3 || ex.hi[1] - ex.lo[1] < 3 || ex.hi[2] - ex.lo[2] < 3) continue;
    unsigned long long* ranks = sc->dU64 + 8;
    for (int rep = 0; rep < 4; rep++) {
      for (int dir = 0; dir < 8; dir++) {
        Sweep w;
        w.dj = (dir & 1) ? -1 : 1;
        w.di = (dir & 2) ? -1 : 1;
        w.dk = (dir & 4) ? -1 : 1;
        w.i0 = w.di > 0 ? ex.lo[0] + 1 : ex.hi[0] - 2;
        w.j0 = w.dj > 0 ? ex.lo[1] + 1 : ex.hi[1] - 2;
        w.k0 = w.dk > 0 ? ex.lo[2] + 1 : ex.hi[2] - 2;
        w.ni = ex.hi[0] - ex.lo[0] - 2;
        w.nj = ex.hi[1] - ex.lo[1] - 2;
        w.nk = ex.hi[2] - ex.lo[2] - 2;
        if (w.ni <= 0 || w.nj <= 0 || w.nk <= 0) continue;
        ESF_CUDA(cudaMemsetAsync(ranks, 0xff, 3 * 8, st));
        const long long total = (long long)w.ni * w.nj * w.nk;
        ESF_COUNTED k_sweep_vec_ranks<<<kblocks(total), KT, 0, st>>>(G, d->d.phi, d->d.mass, w, ranks);
        TRY(sweep_pass<true>(sc, d, w, ranks));
      }
      for (int axis = 2; axis >= 0; axis--) {
        const long long nf = boxn(ex) / (ex.hi[axis] - ex.lo[axis]);
        ESF_COUNTED k_extend_faces<<<kblocks(nf), KT, 0, st>>>(G, d->d.vel, d->d.mass, ex, axis);
      }
    }
    ESF_LAUNCH_CHECK();
  }
  ESF_CUDA(cudaEventRecord(sc->ph[9], st));
  for (int i = 0; i < sc->ns; i++) {  // DEFOR_SOLID_3D::finalizeSolution() (:1198-1233)
    Solid* d = sc->s[i];
    ESF_COUNTED k_u_add<<<kblocks(3 * G.T), KT, 0, st>>>(G, d->d);
    ESF_COUNTED k_u_advect<<<kblocks(G.T), KT, 0, st>>>(G, d->d);
    std::swap(d->d.u, d->d.tmp3);
    Box ex = mkbox(d->ex[0], d->ex[1], d->ex[2], d->ex[3], d->ex[4], d->ex[5]);
    // the face extrapolation reads two layers inward: boxes thinner than 3
    // nodes (a vanished solid) are left as advected
    if (ex.hi[0] - ex.lo[0] >= 3 && ex.hi[1] - ex.lo[1] >= 3 && ex.hi[2] - ex.lo[2] >= 3)
      for (int axis = 2; axis >= 0; axis--)
        ESF_COUNTED k_u_extrapolate<<<kblocks(boxn(ex)), KT, 0, st>>>(G, d->d.u, ex, axis);
    ESF_COUNTED k_recover_X<<<kblocks(G.T), KT, 0, st>>>(G, d->d);
    ESF_LAUNCH_CHECK();
  }
  ESF_CUDA(cudaEventRecord(sc->ph[10], st));
  for (int i = 0; i < sc->ns; i++) TRY(compute_solid_mass(sc, sc->s[i], 1));
  ESF_CUDA(cudaEventRecord(sc->ph[11], st));
  {
    TraceMarks tm(st);
    for (int i = 0; i < sc->ns; i++) TRY(advect_mesh(sc, sc->s[i]));
    tm.mark("mesh advection");
    for (int i = 0; i < sc->ns; i++) {
      TRY(compute_sdf(sc, sc->s[i]));
      tm.mark("sdf");
      TRY(init_particles(sc, sc->s[i]));
      tm.mark("particles");
    }
    TRY(gather_solid_masses(sc));
    tm.mark("gather solid masses");
  }
  ESF_CUDA(cudaEventRecord(sc->ph[12], st));
  // fluid velocity and intensity: FP32 arithmetic in mixed precision (the
  // solid's material coordinates, which decide its cell flags, stay FP64)
  if (prec != ESF_FP64) {
    ESF_COUNTED k_advect_velocity_f32<<<kblocks(G.T), KT, 0, st>>>(G, sc->solidMass, sc->vel, sc->vws, dt);
    std::swap(sc->vel, sc->vws);
    ESF_COUNTED k_advect_scalar_f32<<<kblocks(G.T), KT, 0, st>>>(G, sc->solidMass, sc->vel, sc->intensity, sc->ws, dt);
  } else {
    ESF_COUNTED k_advect_velocity<<<kblocks(G.T), KT, 0, st>>>(G, sc->solidMass, sc->vel, sc->vws, dt);
    std::swap(sc->vel, sc->vws);
    ESF_COUNTED k_advect_scalar<<<kblocks(G.T), KT, 0, st>>>(G, sc->solidMass, sc->vel, sc->intensity, sc->ws, dt);
  }
  std::swap(sc->intensity, sc->ws);
  TRY(recover_velocity(sc));
  ESF_COUNTED k_dirichlet<<<kblocks(G.T), KT, 0, st>>>(G, sc->vel, sc->intensity);
  ESF_LAUNCH_CHECK();
  ESF_CUDA(cudaEventRecord(sc->ph[13], st));
  ESF_CUDA(cudaEventRecord(sc->e1, st));
  ESF_CUDA(cudaStreamSynchronize(st));
  TRY(check_sweeps(sc));
  if (rep) {
    memset(rep, 0, sizeof *rep);
    rep->dt = dt;
    rep->energy = energy;
    for (int k = 0; k < 3; k++) {
      rep->iterations[k] = it[k];
      rep->converged[k] = cv[k];
      rep->rel_residual[k] = rr[k];
      rep->refinements[k] = rf[k];
    }
    rep->prone_to_contact = prone;
    rep->fp64_iterations = it64;
    int fb = 0;
    for (int i = 0; i < sc->ns; i++) fb += sc->hInts[kFallbackCount + i];
    rep->fp64_stress_cells = prec != ESF_FP64 ? fb : (int)sc->validCells;
    rep->valid_cells = (int)sc->validCells;
    unsigned long long contacts = 0;
    ESF_CUDA(cudaMemcpy(&contacts, sc->contactCount.p, 8, cudaMemcpyDeviceToHost));
    rep->solid_contacts = (int)contacts;
    long long np = 0;
    for (int i = 0; i < sc->ns; i++) np += sc->s[i]->np;
    rep->num_particles = (int)np;
    rep->status = sc->status;
    float ms = 0;
    cudaEventElapsedTime(&ms, sc->e0, sc->e1);
    rep->device_ms = ms;
    for (int i = 0; i < 13; i++) {
      float t = 0;
      cudaEventElapsedTime(&t, sc->ph[i], sc->ph[i + 1]);
      rep->phase_ms[i] = t;
    }
  }
  return (esf_status)sc->status;
}

// ------------------------------------------------------------ field access
namespace {
struct FieldRef {
  void* dev = nullptr;     // device source (node/cell/solid layouts)
  size_t count = 0;        // elements exposed
  size_t eb = 8;
  int kind = 0;            // 0 direct, 1 node3->dof3, 2 node1->dof3, 3 host ints, 4 dof map,
                           // 5 system blocks, 6 plastic material grid header
  bool writable = false;
};
}  // namespace

static esf_status field_ref(esf_scene* s, int f, int si, FieldRef& r) {
  const GridDev& G = s->g;
  const size_t T = G.T, R = G.R, D = 3ull * (G.X - 2) * (G.Y - 2) * (G.Z - 2);
  // the solid system of the last step is sized by the solid nodes it was
  // assembled for (the step's closing mass update can change their count)
  const size_t S3 = 3ull * s->Sstep;
  Solid* d = (si >= 0 && si < s->ns) ? s->s[si] : nullptr;
  switch (f) {
    case ESF_F_VELOCITY: r = {s->vel, T * 3, 8, 0, true}; return ESF_OK;
    case ESF_F_INTENSITY: r = {s->intensity, T, 8, 0, true}; return ESF_OK;
    case ESF_F_SOLID_MASS: r = {s->solidMass, T, 8, 0, false}; return ESF_OK;
    case ESF_F_NODE_SOLID_VF: r = {s->nodeVF, T, 8, 0, false}; return ESF_OK;
    case ESF_F_DOF_MAP: r = {nullptr, T, 4, 4, false}; return ESF_OK;
    case ESF_F_SOLID_DOF_MAP: r = {s->sdof, T, 4, 0, false}; return ESF_OK;
    case ESF_F_PRESSURE: r = {s->lambda, R, 8, 0, true}; return ESF_OK;
    case ESF_F_JMINVJT_DIAG: r = {s->jdiag, R, 8, 0, false}; return ESF_OK;
    case ESF_F_DIV_RHS: r = {s->rhs, R, 8, 0, false}; return ESF_OK;
    case ESF_F_B1: r = {s->b1, R, 8, 0, false}; return ESF_OK;
    case ESF_F_NZ_MASS_INV: r = {s->minv, D, 8, 2, false}; return ESF_OK;
    case ESF_F_VELOCITY_DT0: r = {s->vstar, D, 8, 1, false}; return ESF_OK;
    case ESF_F_VELOCITY_DT1: r = {s->v1, D, 8, 1, false}; return ESF_OK;
    case ESF_F_UNIT_FORCE: r = {s->uf, D, 8, 1, false}; return ESF_OK;
    case ESF_F_SOLID_UNIT_FORCE: r = {s->solidF.p, S3, 8, 0, false}; return ESF_OK;
    case ESF_F_SOLID_VELOCITY_DT0: r = {s->solidV0.p, S3, 8, 0, false}; return ESF_OK;
    case ESF_F_SOLID_PRESSURE_CORRECTION: r = {s->solidPC.p, S3, 8, 0, false}; return ESF_OK;
    case ESF_F_DAMPED_SOLID_MASS: r = {s->damped.p, S3, 8, 0, false}; return ESF_OK;
    case ESF_F_SYSTEM_DIAG: r = {s->sysDiag.p, S3, 8, 0, false}; return ESF_OK;
    case ESF_F_SYSTEM_BLOCKS: r = {s->blocks.p, 243ull * s->Sstep, 8, 5, false}; return ESF_OK;
    case ESF_F_SYSTEM_MASK: r = {s->mask.p, (size_t)s->Sstep, 4, 0, false}; return ESF_OK;
    default: break;
  }
  if (!d) {
    set_error("field %d: invalid solid index %d", f, si);
    return ESF_ERR_INVALID_ARG;
  }
  switch (f) {
    case ESF_F_S_U: r = {d->d.u, T * 3, 8, 0, true}; return ESF_OK;
    case ESF_F_S_X: r = {d->d.X, T * 3, 8, 0, true}; return ESF_OK;
    case ESF_F_S_VELOCITY: r = {d->d.vel, T * 3, 8, 0, true}; return ESF_OK;
    case ESF_F_S_VEC_WORKSPACE: r = {d->d.vws, T * 3, 8, 0, true}; return ESF_OK;
    case ESF_F_S_MASS: r = {d->d.mass, T, 8, 0, true}; return ESF_OK;
    case ESF_F_S_PHI: r = {d->d.phi, T, 8, 0, true}; return ESF_OK;
    case ESF_F_S_DET_FINV: r = {d->d.detFInv, T, 8, 0, false}; return ESF_OK;
    case ESF_F_S_VALID: r = {d->d.valid, R, 1, 0, false}; return ESF_OK;
    case ESF_F_S_QUARTER_FRACTIONS: r = {d->d.quarter, T * 8, 8, 0, false}; return ESF_OK;
    case ESF_F_S_PARTICLES: r = {d->part.p, (size_t)d->np * 10, 8, 0, false}; return ESF_OK;
    case ESF_F_S_MESH_VERTICES: r = {d->dVerts, (size_t)d->nv * 3, 8, 0, false}; return ESF_OK;
    case ESF_F_S_BOXES: r = {nullptr, 12, 4, 3, false}; return ESF_OK;
    case ESF_F_S_FPINV:
      if (!d->d.plastic) break;
      r = {d->d.FpInv, (size_t)d->pn * 9, 8, 0, true};
      return ESF_OK;
    case ESF_F_S_FPINV_GRID:
      if (!d->d.plastic) break;
      r = {nullptr, 7, 8, 6, false};
      return ESF_OK;
    default: break;
  }
  set_error("unknown field id %d", f);
  return ESF_ERR_INVALID_ARG;
}

extern "C" esf_status esf_field_info(const esf_scene* s, esf_field f, int si, size_t* count,
                                     size_t* eb) {
  if (!s || !count || !eb) return ESF_ERR_INVALID_ARG;
  FieldRef r;
  TRY(field_ref((esf_scene*)s, f, si, r));
  *count = r.count;
  *eb = r.eb;
  return ESF_OK;
}

extern "C" esf_status esf_get_field(esf_scene* s, esf_field f, int si, void* host, size_t bytes) {
  if (!s || (!host && bytes)) return ESF_ERR_INVALID_ARG;
  FieldRef r;
  TRY(field_ref(s, f, si, r));
  if (bytes != r.count * r.eb) {
    set_error("esf_get_field(%d): %zu bytes given, %zu expected", (int)f, bytes, r.count * r.eb);
    return ESF_ERR_INVALID_ARG;
  }
  const GridDev& G = s->g;
  ESF_CUDA(cudaStreamSynchronize(s->stream));
  if (r.kind == 0) {
    if (bytes) ESF_CUDA(cudaMemcpy(host, r.dev, bytes, cudaMemcpyDeviceToHost));
    return ESF_OK;
  }
  if (r.kind == 3) {
    Solid* d = s->s[si];
    int b[12] = {d->ex[0], d->ex[1], d->ex[2], d->ex[3], d->ex[4], d->ex[5],
                 d->tmin[0], d->tmin[1], d->tmin[2], d->tmax[0], d->tmax[1], d->tmax[2]};
    memcpy(host, b, 48);
    return ESF_OK;
  }
  if (r.kind == 6) {  // material grid of FpInv: xRes, yRes, zRes, dh, origin
    const SolidDev& x = s->s[si]->d;
    const double h[7] = {(double)x.pres[0], (double)x.pres[1], (double)x.pres[2], x.pdh,
                         x.porig[0], x.porig[1], x.porig[2]};
    memcpy(host, h, sizeof h);
    return ESF_OK;
  }
  if (r.kind == 5) {  // system blocks: device entry-major -> [node][27][3][3]
    const long long S = s->Sstep;
    std::vector<double> tmp(243 * rows32(S));
    if (S) ESF_CUDA(cudaMemcpy(tmp.data(), r.dev, tmp.size() * 8, cudaMemcpyDeviceToHost));
    double* o = (double*)host;
    for (long long a = 0; a < S; a++)
      for (int je = 0; je < 243; je++) o[243 * a + je] = tmp[blk_at(a, je)];
    return ESF_OK;
  }
  if (r.kind == 4) {  // _gridIdxToSolutionIdx (COUPLED_INTEGRATOR_3D.cpp:123-131)
    int* o = (int*)host;
    int idx = 0;
    for (long long n = 0; n < G.T; n++) o[n] = -1;
    for (int z = 1; z < G.Z - 1; z++)
      for (int y = 1; y < G.Y - 1; y++)
        for (int x = 1; x < G.X - 1; x++) o[x + (long long)y * G.X + z * G.slab] = idx++;
    return ESF_OK;
  }
  // node-indexed -> compacted DOF order
  const int comp = (r.kind == 1) ? 3 : 1;
  std::vector<double> tmp(G.T * comp);
  ESF_CUDA(cudaMemcpy(tmp.data(), r.dev, tmp.size() * 8, cudaMemcpyDeviceToHost));
  double* o = (double*)host;
  long long k = 0;
  for (int z = 1; z < G.Z - 1; z++)
    for (int y = 1; y < G.Y - 1; y++)
      for (int x = 1; x < G.X - 1; x++, k++) {
        long long n = x + (long long)y * G.X + z * G.slab;
        for (int q = 0; q < 3; q++) o[3 * k + q] = (comp == 3) ? tmp[3 * n + q] : tmp[n];
      }
  return ESF_OK;
}

extern "C" esf_status esf_set_field(esf_scene* s, esf_field f, int si, const void* host,
                                    size_t bytes) {
  if (!s || (!host && bytes)) return ESF_ERR_INVALID_ARG;
  FieldRef r;
  TRY(field_ref(s, f, si, r));
  if (!r.writable || r.kind != 0) {
    set_error("esf_set_field(%d): field is read-only", (int)f);
    return ESF_ERR_INVALID_ARG;
  }
  if (bytes != r.count * r.eb) {
    set_error("esf_set_field(%d): %zu bytes given, %zu expected", (int)f, bytes, r.count * r.eb);
    return ESF_ERR_INVALID_ARG;
  }
  ESF_CUDA(cudaStreamSynchronize(s->stream));
  if (bytes) ESF_CUDA(cudaMemcpy(r.dev, host, bytes, cudaMemcpyHostToDevice));
  return ESF_OK;
}

// ------------------------------------------------------- operator seam
static GridDev grid_dev(const esf_grid* g) {
  GridDev G;
  G.X = g->xRes;
  G.Y = g->yRes;
  G.Z = g->zRes;
  G.slab = (long long)G.X * G.Y;
  G.T = G.slab * G.Z;
  G.cX = G.X - 1;
  G.cY = G.Y - 1;
  G.cZ = G.Z - 1;
  G.cslab = (long long)G.cX * G.cY;
  G.R = G.cslab * G.cZ;
  G.dh = g->dh;
  G.dhInv = 1.0 / g->dh;
  for (int k = 0; k < 3; k++) G.o[k] = g->origin[k];
  return G;
}

extern "C" esf_status esf_pressure_apply(const esf_grid* g, const double* minv, const double* in,
                                         double* out, void* stream) {
  if (!g || !minv || !in || !out || g->xRes < 3 || g->yRes < 3 || g->zRes < 3) {
    set_error("esf_pressure_apply: invalid argument");
    return ESF_ERR_INVALID_ARG;
  }
  GridDev G = grid_dev(g);
  return pressure_apply<double>(G, minv, in, out, (cudaStream_t)stream);
}

extern "C" esf_status esf_pressure_solve(const esf_grid* g, const double* minv, const double* diag,
                                         const double* b, double* x, double eps, int maxIt,
                                         int precision, int* iters, double* relres, void* stream) {
  if (!g || !minv || !diag || !b || !x || g->xRes < 3 || g->yRes < 3 || g->zRes < 3 || maxIt < 0 ||
      (precision != ESF_FP64 && precision != ESF_MIXED && precision != ESF_MIXED_X64)) {
    set_error("esf_pressure_solve: invalid argument");
    return ESF_ERR_INVALID_ARG;
  }
  GridDev G = grid_dev(g);
  PressureWork* w = nullptr;
  TRY(pressure_work_alloc(&w, G, precision != ESF_FP64));
  int it = 0, rf = 0, cv = 0;
  double rr = 0;
  esf_status e = pressure_solve(w, G, minv, diag, b, x, eps, maxIt, precision, 1e-4, 50, &it, &rr, &rf,
                                &cv, (cudaStream_t)stream);
  cudaStreamSynchronize((cudaStream_t)stream);
  pressure_work_free(w);
  if (iters) *iters = it;
  if (relres) *relres = rr;
  return e;
}

namespace esf {
// Serving: hand this scene's mixed inner solves to a batcher shared with
// other scenes (nullptr: solve them on the scene's own stream).
esf_status scene_set_batcher(esf_scene* s, InnerBatcher* b) {
  if (!s || !s->pw) return ESF_ERR_STATE;
  return pressure_work_set_batcher(s->pw, b);
}
}  // namespace esf

extern "C" esf_status esf_pressure_solve_batch(int n, const esf_grid* grids, const double* const* minv,
                                               const double* const* diag, const double* const* b,
                                               double* const* x, double eps, int maxIt, int precision,
                                               int autotune, int* iters, double* relres,
                                               esf_batch_stats* stats, void* stream) {
  if (n < 1 || !grids || !minv || !diag || !b || !x || maxIt < 0 ||
      (precision != ESF_FP64 && precision != ESF_MIXED && precision != ESF_MIXED_X64)) {
    set_error("esf_pressure_solve_batch: invalid argument");
    return ESF_ERR_INVALID_ARG;
  }
  for (int i = 0; i < n; i++)
    if (!minv[i] || !diag[i] || !b[i] || !x[i] || grids[i].xRes < 3 || grids[i].yRes < 3 ||
        grids[i].zRes < 3) {
      set_error("esf_pressure_solve_batch: invalid system %d", i);
      return ESF_ERR_INVALID_ARG;
    }
  int dev = 0;
  ESF_CUDA(cudaGetDevice(&dev));
  InnerBatcher* batcher = nullptr;
  if (precision == ESF_MIXED) TRY(batcher_create(dev, &batcher, autotune != 0));
  cudaEvent_t start = nullptr;
  ESF_CUDA(cudaEventCreateWithFlags(&start, cudaEventDisableTiming));
  ESF_CUDA(cudaEventRecord(start, (cudaStream_t)stream));
  std::vector<esf_status> st(n, ESF_OK);
  std::vector<int> it(n, 0);
  std::vector<double> rr(n, 0.0);
  // every system's work is attached before any solve starts, so systems of
  // one grid shape find each other in the batcher from their first inner solve
  std::vector<PressureWork*> works(n, nullptr);
  std::vector<cudaStream_t> streams(n, nullptr);
  esf_status e = ESF_OK;
  for (int i = 0; i < n && !e; i++) {
    if (cudaStreamCreateWithFlags(&streams[i], cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamWaitEvent(streams[i], start, 0) != cudaSuccess) {
      set_error("esf_pressure_solve_batch: %s", cudaGetErrorString(cudaGetLastError()));
      e = ESF_ERR_CUDA;
      break;
    }
    e = pressure_work_alloc(&works[i], grid_dev(&grids[i]), precision != ESF_FP64);
    if (!e && batcher) e = pressure_work_set_batcher(works[i], batcher);
  }
  if (!e) {
    // one host thread per system drives its FP64 refinement loop on its own
    // stream; the inner iterations of systems of one grid shape share the
    // batcher's launches
    std::vector<std::thread> threads;
    for (int i = 0; i < n; i++)
      threads.emplace_back([&, i] {
        cudaSetDevice(dev);
        int rf = 0, cv = 0;
        st[i] = pressure_solve(works[i], grid_dev(&grids[i]), minv[i], diag[i], b[i], x[i], eps, maxIt,
                               precision, 1e-4, 50, &it[i], &rr[i], &rf, &cv, streams[i]);
        cudaStreamSynchronize(streams[i]);
      });
    for (auto& t : threads) t.join();
  }
  for (int i = 0; i < n; i++) {
    pressure_work_free(works[i]);
    if (streams[i]) cudaStreamDestroy(streams[i]);
  }
  if (stats) {
    memset(stats, 0, sizeof *stats);
    if (batcher) batcher_stats(batcher, stats);
  }
  batcher_destroy(batcher);
  cudaEventDestroy(start);
  for (int i = 0; i < n; i++) {
    if (iters) iters[i] = it[i];
    if (relres) relres[i] = rr[i];
    if (st[i] && !e) e = st[i];
  }
  return e;
}

extern "C" esf_status esf_pressure_solve_static(const esf_grid* g, const double* minv,
                                                const double* diag, const double* b, double* x,
                                                double eps, int maxIt, int* iters, double* relres,
                                                void* stream) {
  if (!g || !minv || !diag || !b || !x || g->xRes < 3 || g->yRes < 3 || g->zRes < 3 || maxIt < 0) {
    set_error("esf_pressure_solve_static: invalid argument");
    return ESF_ERR_INVALID_ARG;
  }
  const long long cells = (long long)(g->xRes - 1) * (g->yRes - 1) * (g->zRes - 1);
  if (cells > ESF_STATIC_SOLVE_MAX_CELLS) {
    set_error("esf_pressure_solve_static: grid has %lld cells, the static scratch holds at most %d",
              cells, ESF_STATIC_SOLVE_MAX_CELLS);
    return ESF_ERR_UNSUPPORTED;
  }
  void* scratch = nullptr;
  TRY(static_scratch_address(&scratch));
  GridDev G = grid_dev(g);
  int it = 0, cv = 0;
  double rr = 0;
  esf_status e = pressure_solve_static(scratch, G, minv, diag, b, x, eps, maxIt, &it, &rr, &cv,
                                       (cudaStream_t)stream);
  if (iters) *iters = it;
  if (relres) *relres = rr;
  return e;
}

// One block arrives at a grid barrier that expects a second block, which is
// never launched, and waits with wave_barrier, the wave sweep's bounded wait
// (WAVE_WAIT_LIMIT polls): the wait runs out, the block sets *err and returns.
__global__ void k_selftest_wave_barrier(unsigned* count, int* err) { wave_barrier(count, 2, err); }

extern "C" esf_status esf_selftest_bounded_wait(int kind, int* gave_up, double* elapsed_ms) {
  if ((kind != 0 && kind != 1) || !gave_up) {
    set_error("esf_selftest_bounded_wait: kind must be 0 or 1 and gave_up non-NULL");
    return ESF_ERR_INVALID_ARG;
  }
  int* d = nullptr;
  ESF_CUDA(cudaMalloc(&d, 16));
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  esf_status e = ESF_OK;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) e = ESF_ERR_CUDA;
  if (!e && cudaMemset(d, 0, 16) != cudaSuccess) e = ESF_ERR_CUDA;
  if (!e) {
    cudaEventRecord(e0, 0);
    if (kind == 0) {
      e = selftest_mbar_wait(d, 0);
    } else {
      ESF_COUNTED k_selftest_wave_barrier<<<1, 32>>>(reinterpret_cast<unsigned*>(d + 1), d);
      if (cudaGetLastError() != cudaSuccess) e = ESF_ERR_CUDA;
    }
    cudaEventRecord(e1, 0);
  }
  int h = -1;
  if (!e && cudaMemcpy(&h, d, sizeof h, cudaMemcpyDeviceToHost) != cudaSuccess) e = ESF_ERR_CUDA;
  float ms = 0;
  if (!e) cudaEventElapsedTime(&ms, e0, e1);
  if (e == ESF_ERR_CUDA) set_error("esf_selftest_bounded_wait: %s", cudaGetErrorString(cudaGetLastError()));
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaFree(d);
  *gave_up = h;
  if (elapsed_ms) *elapsed_ms = ms;
  return e;
}

// COUPLED_INTEGRATOR_3D::writeFrame (COUPLED_INTEGRATOR_3D.cpp:997-1012) with
// DEFOR_SOLID_3D::writeFrame (DEFOR_SOLID_3D.cpp:1362-1370): per solid i
// "frame.NNNN.solid.i" + .displacement/.velocity/.phi (every 10th frame or
// debug) and .obj (always); the fluid .velocity (every 10th frame or debug)
// and .intensity (always). The .pbrt render export is not written.
// A frame's content in host memory: per solid its displacement, velocity,
// phi, FpInv (row-major, plastic solids) and mesh vertices; the grid velocity,
// the pressure warm start and the intensity. Fields a partial frame (not
// every 10th, not debug) does not write may be null.
namespace {
struct FrameSnap {
  bool full = false;
  std::vector<const double*> u, vel, phi, fp, verts;
  const double *gridVel = nullptr, *lambda = nullptr, *intensity = nullptr;
};
}  // namespace

// The files of COUPLED_INTEGRATOR_3D::writeFrame (COUPLED_INTEGRATOR_3D.cpp:
// 997-1012) and DEFOR_SOLID_3D::writeFrame (DEFOR_SOLID_3D.cpp:1362-1370)
// from a snapshot.
static esf_status write_frame_files(esf_scene* s, const FrameSnap& f, const std::string& base) {
  const GridDev& G = s->g;
  const int res[3] = {G.X, G.Y, G.Z};
  for (int i = 0; i < s->ns; i++) {
    Solid* d = s->s[i];
    const std::string fn = base + ".solid." + std::to_string(i);
    if (f.full) {
      TRY(write_field_gz(fn + ".displacement", res, G.dh, G.o, f.u[i], G.T * 3));
      TRY(write_field_gz(fn + ".velocity", res, G.dh, G.o, f.vel[i], G.T * 3));
      TRY(write_field_gz(fn + ".phi", res, G.dh, G.o, f.phi[i], G.T));
      if (d->d.plastic) {
        // MATRIX3_FIELD_3D::writeGz: 9 doubles per cell, column-major
        std::vector<double> cm((size_t)d->pn * 9);
        const double* fp = f.fp[i];
        for (long long c = 0; c < d->pn; c++)
          for (int a = 0; a < 3; a++)
            for (int b = 0; b < 3; b++) cm[9 * c + 3 * b + a] = fp[9 * c + 3 * a + b];
        TRY(write_field_gz(fn + ".plasticdefor", d->d.pres, d->d.pdh, d->d.porig, cm.data(), cm.size()));
      }
    }
    TRY(write_obj(fn + ".obj", f.verts[i], d->nv, d->tris.data(), d->ntri));
  }
  if (f.full) {
    TRY(write_field_gz(base + ".velocity", res, G.dh, G.o, f.gridVel, G.T * 3));
    // extension: the pressure warm start, which the reference keeps in a
    // function-local static and never writes; a cell field (cell centres)
    const int cres[3] = {G.cX, G.cY, G.cZ};
    const double corig[3] = {G.o[0] + 0.5 * G.dh, G.o[1] + 0.5 * G.dh, G.o[2] + 0.5 * G.dh};
    TRY(write_field_gz(base + ".lambda1", cres, G.dh, corig, f.lambda, G.R));
  }
  TRY(write_field_gz(base + ".intensity", res, G.dh, G.o, f.intensity, G.T));
  return ESF_OK;
}

extern "C" esf_status esf_frame_wait(esf_scene* s);

extern "C" esf_status esf_write_frame(esf_scene* s, const char* path, int frame, int debug) {
  if (!s || !path) {
    set_error("esf_write_frame: invalid argument");
    return ESF_ERR_INVALID_ARG;
  }
  if (!s->inited) {
    set_error("esf_write_frame: scene not initialised");
    return ESF_ERR_STATE;
  }
  TRY(esf_frame_wait(s));  // an asynchronous frame still being written goes first
  const GridDev& G = s->g;
  FrameSnap f;
  f.full = debug || (frame % 10 == 0);
  std::vector<std::vector<double>> keep;
  auto get = [&](esf_field id, int si, size_t n) -> const double* {
    keep.emplace_back(n);
    return esf_get_field(s, id, si, keep.back().data(), n * 8) == ESF_OK ? keep.back().data() : nullptr;
  };
  keep.reserve(8 + 6 * s->ns);
  for (int i = 0; i < s->ns; i++) {
    Solid* d = s->s[i];
    f.u.push_back(f.full ? get(ESF_F_S_U, i, G.T * 3) : nullptr);
    f.vel.push_back(f.full ? get(ESF_F_S_VELOCITY, i, G.T * 3) : nullptr);
    f.phi.push_back(f.full ? get(ESF_F_S_PHI, i, G.T) : nullptr);
    f.fp.push_back(f.full && d->d.plastic ? get(ESF_F_S_FPINV, i, (size_t)d->pn * 9) : nullptr);
    f.verts.push_back(get(ESF_F_S_MESH_VERTICES, i, (size_t)d->nv * 3));
    if ((f.full && (!f.u.back() || !f.vel.back() || !f.phi.back() || (d->d.plastic && !f.fp.back()))) ||
        !f.verts.back())
      return ESF_ERR_CUDA;
  }
  if (f.full && (!(f.gridVel = get(ESF_F_VELOCITY, 0, G.T * 3)) || !(f.lambda = get(ESF_F_PRESSURE, 0, G.R))))
    return ESF_ERR_CUDA;
  if (!(f.intensity = get(ESF_F_INTENSITY, 0, G.T))) return ESF_ERR_CUDA;
  return write_frame_files(s, f, frame_prefix(path, frame));
}

// Asynchronous frame: the fields are copied on the scene's stream into pinned
// host memory, behind the work queued so far, and a host thread compresses
// and writes the files once the copies have landed, while the caller goes on
// stepping. One frame is in flight per scene: the next call (or
// esf_write_frame, esf_read_frame, esf_destroy) first waits for it;
// esf_frame_wait returns its status.
extern "C" esf_status esf_write_frame_async(esf_scene* s, const char* path, int frame, int debug) {
  if (!s || !path) {
    set_error("esf_write_frame_async: invalid argument");
    return ESF_ERR_INVALID_ARG;
  }
  if (!s->inited) {
    set_error("esf_write_frame_async: scene not initialised");
    return ESF_ERR_STATE;
  }
  TRY(esf_frame_wait(s));
  cudaSetDevice(s->device);
  const GridDev& G = s->g;
  const bool full = debug || (frame % 10 == 0);
  // pinned snapshot: [grid velocity | lambda | intensity | per solid u, vel, phi, FpInv, vertices]
  size_t words = (full ? G.T * 3 + G.R : 0) + G.T;
  for (int i = 0; i < s->ns; i++) {
    Solid* d = s->s[i];
    words += (full ? G.T * 7 + (d->d.plastic ? (size_t)d->pn * 9 : 0) : 0) + (size_t)d->nv * 3;
  }
  if (s->frameWords < words) {
    if (s->framePinned) cudaFreeHost(s->framePinned);
    s->framePinned = nullptr;
    s->frameWords = 0;
    ESF_CUDA(cudaMallocHost(&s->framePinned, words * 8));
    s->frameWords = words;
  }
  if (!s->frameEv) ESF_CUDA(cudaEventCreateWithFlags(&s->frameEv, cudaEventDisableTiming));
  cudaStream_t st = s->stream;
  double* h = s->framePinned;
  auto copy = [&](const double* dev, size_t n) -> const double* {
    const double* at = h;
    if (cudaMemcpyAsync(h, dev, n * 8, cudaMemcpyDeviceToHost, st) != cudaSuccess) return nullptr;
    h += n;
    return at;
  };
  FrameSnap f;
  f.full = full;
  bool ok = true;
  if (full) {
    ok = ok && (f.gridVel = copy(s->vel, G.T * 3)) && (f.lambda = copy(s->lambda, G.R));
  }
  ok = ok && (f.intensity = copy(s->intensity, G.T));
  for (int i = 0; i < s->ns && ok; i++) {
    Solid* d = s->s[i];
    const double *u = nullptr, *v = nullptr, *ph = nullptr, *fp = nullptr, *vx = nullptr;
    if (full) {
      ok = (u = copy(d->d.u, G.T * 3)) && (v = copy(d->d.vel, G.T * 3)) && (ph = copy(d->d.phi, G.T));
      if (ok && d->d.plastic) ok = (fp = copy(d->d.FpInv, (size_t)d->pn * 9)) != nullptr;
    }
    ok = ok && (vx = copy(d->dVerts, (size_t)d->nv * 3));
    f.u.push_back(u);
    f.vel.push_back(v);
    f.phi.push_back(ph);
    f.fp.push_back(fp);
    f.verts.push_back(vx);
  }
  if (!ok || cudaEventRecord(s->frameEv, st) != cudaSuccess) {
    set_error("esf_write_frame_async: %s", cudaGetErrorString(cudaGetLastError()));
    cudaStreamSynchronize(st);
    return ESF_ERR_CUDA;
  }
  const std::string base = frame_prefix(path, frame);
  const int dev = s->device;
  s->frameStatus = ESF_OK;
  s->frameThread = std::thread([s, f, base, dev] {
    cudaSetDevice(dev);
    s->frameStatus = cudaEventSynchronize(s->frameEv) == cudaSuccess ? write_frame_files(s, f, base)
                                                                      : ESF_ERR_CUDA;
  });
  return ESF_OK;
}

extern "C" esf_status esf_frame_wait(esf_scene* s) {
  if (!s) return ESF_ERR_INVALID_ARG;
  if (s->frameThread.joinable()) s->frameThread.join();
  const esf_status e = (esf_status)s->frameStatus;
  s->frameStatus = ESF_OK;
  return e;
}

// COUPLED_INTEGRATOR_3D::readFrame (COUPLED_INTEGRATOR_3D.cpp:977-996) with
// DEFOR_SOLID_3D::readFrame (DEFOR_SOLID_3D.cpp:1299-1361): the fields above,
// then per solid X from u, the mesh from its OBJ, the boxes from the mesh's
// vertex bounds, computeSolidMass(true) and initMaterialParticles; then
// gatherSolidMasses and recoverVelocityField. dt is not part of a frame (it
// is recomputed from the CFL condition each step); the pressure warm start is
// read from the ".lambda1" extension file where present. A successful read
// also lifts the stop left by a step whose solve met NaN/Inf.
extern "C" esf_status esf_read_frame(esf_scene* s, const char* path, int frame, int debug) {
  if (!s || !path) {
    set_error("esf_read_frame: invalid argument");
    return ESF_ERR_INVALID_ARG;
  }
  if (!s->inited) {
    set_error("esf_read_frame: scene not initialised");
    return ESF_ERR_STATE;
  }
  TRY(esf_frame_wait(s));
  cudaSetDevice(s->device);
  const GridDev& G = s->g;
  cudaStream_t st = s->stream;
  const int res[3] = {G.X, G.Y, G.Z};
  const bool full = debug || (frame % 10 == 0);
  const std::string base = frame_prefix(path, frame);
  std::vector<double> buf((size_t)G.T * 3);
  for (int i = 0; i < s->ns; i++) {
    Solid* d = s->s[i];
    const std::string fn = base + ".solid." + std::to_string(i);
    if (full) {
      TRY(read_field_gz(fn + ".displacement", res, G.T * 3, buf.data()));
      TRY(esf_set_field(s, ESF_F_S_U, i, buf.data(), G.T * 24));
      TRY(read_field_gz(fn + ".velocity", res, G.T * 3, buf.data()));
      TRY(esf_set_field(s, ESF_F_S_VELOCITY, i, buf.data(), G.T * 24));
      TRY(read_field_gz(fn + ".phi", res, G.T, buf.data()));
      TRY(esf_set_field(s, ESF_F_S_PHI, i, buf.data(), G.T * 8));
      if (d->d.plastic) {
        std::vector<double> fp((size_t)d->pn * 9), cm((size_t)d->pn * 9);
        TRY(read_field_gz(fn + ".plasticdefor", d->d.pres, cm.size(), cm.data()));
        for (long long c = 0; c < d->pn; c++)
          for (int a = 0; a < 3; a++)
            for (int b = 0; b < 3; b++) fp[9 * c + 3 * a + b] = cm[9 * c + 3 * b + a];
        TRY(esf_set_field(s, ESF_F_S_FPINV, i, fp.data(), fp.size() * 8));
      }
    }
    ESF_COUNTED k_frame_X<<<kblocks(G.T), KT, 0, st>>>(G, d->d);
    ESF_LAUNCH_CHECK();
    std::vector<double> v((size_t)d->nv * 3);
    TRY(read_obj_vertices(fn + ".obj", d->nv, v.data()));
    ESF_CUDA(cudaMemcpyAsync(d->dVerts, v.data(), v.size() * 8, cudaMemcpyHostToDevice, st));
    double mn[3] = {1e9, 1e9, 1e9}, mx[3] = {-1e9, -1e9, -1e9};
    for (int k = 0; k < d->nv; k++)
      for (int q = 0; q < 3; q++) {
        mn[q] = std::min(mn[q], v[3 * k + q]);
        mx[q] = std::max(mx[q], v[3 * k + q]);
      }
    int lo[3], hi[3];
    for (int q = 0; q < 3; q++) {
      lo[q] = (int)((mn[q] - G.o[q]) / G.dh);
      hi[q] = (int)((mx[q] - G.o[q]) / G.dh);
    }
    const int tb = s->p.tight_border, exn = s->p.extrapolation_cells;
    for (int q = 0; q < 3; q++) {
      d->tmin[q] = std::max(lo[q] - tb, 0);
      d->tmax[q] = std::min(hi[q] + tb, res[q]);
      d->ex[q] = std::max(lo[q] - exn, 0);
      d->ex[3 + q] = std::min(hi[q] + exn, res[q]);
    }
    TRY(compute_solid_mass(s, d, 1));
    TRY(init_particles(s, d));
  }
  if (full) {
    TRY(read_field_gz(base + ".velocity", res, G.T * 3, buf.data()));
    TRY(esf_set_field(s, ESF_F_VELOCITY, 0, buf.data(), G.T * 24));
  }
  // the pressure warm start, where the frame has it (our extension); a frame
  // written by the reference has none, and the warm start is kept, as the
  // reference keeps its static one, unless a failed solve left it non-finite
  {
    const int cres[3] = {G.cX, G.cY, G.cZ};
    const std::string lf = base + ".lambda1";
    FILE* probe = full ? fopen(lf.c_str(), "rb") : nullptr;
    if (probe) {
      fclose(probe);
      TRY(read_field_gz(lf, cres, G.R, buf.data()));
      TRY(esf_set_field(s, ESF_F_PRESSURE, 0, buf.data(), G.R * 8));
    } else if (s->failed) {
      ESF_CUDA(cudaMemsetAsync(s->lambda, 0, G.R * 8, st));
    }
  }
  TRY(read_field_gz(base + ".intensity", res, G.T, buf.data()));
  TRY(esf_set_field(s, ESF_F_INTENSITY, 0, buf.data(), G.T * 8));
  TRY(gather_solid_masses(s));
  TRY(recover_velocity(s));
  ESF_CUDA(cudaStreamSynchronize(st));
  s->failed = false;
  return ESF_OK;
}

extern "C" esf_status esf_time_pressure_kernels(esf_scene* s, int reps, double* update_ms,
                                                double* axpy_ms) {
  if (!s || reps < 1) return ESF_ERR_INVALID_ARG;
  if (!s->inited) return ESF_ERR_STATE;
  double u = 0, a = 0;
  TRY(pressure_time_kernels(s->pw, s->g, s->minv, s->jdiag, s->b1, s->lambda, s->p.precision, reps,
                            &u, &a, s->stream));
  if (update_ms) *update_ms = u;
  if (axpy_ms) *axpy_ms = a;
  return ESF_OK;
}
