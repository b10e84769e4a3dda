// Shared declarations of the GB300 coupled-step library.
//
// Device data layout (all in HBM, FP64 unless stated):
//   node fields    T = X*Y*Z entries, index x + y*X + z*X*Y; 3-vectors are
//                  interleaved (x,y,z) per node like VEC3F_FIELD_3D.
//   cell fields    R = (X-1)(Y-1)(Z-1) entries, index x + y*(X-1) + z*(X-1)(Y-1):
//                  pressure rows, the Jacobi diagonal, b1, the PCR vectors.
//   solid unknowns 3*S (S = nodes with solid mass), solid index from the
//                  prefix scan of COUPLED_INTEGRATOR_3D::gatherSolidMasses.
// The velocity unknowns of the reference (3 per interior node, compacted in
// z,y,x order) are kept node-indexed on the device; the compaction is only
// done when a caller reads them through esf_get_field.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <math.h>

#include "../../include/eulersf.h"

#define ESF_HD __host__ __device__ __forceinline__

struct GridDev {
  int X, Y, Z;       // nodes per axis
  long long slab;    // X*Y
  long long T;       // nodes
  int cX, cY, cZ;    // cells per axis
  long long cslab;   // cX*cY
  long long R;       // cells
  double dh, dhInv;
  double o[3];
};

// ------------------------------------------------------------ interpolation
// FIELD_3D::get_barycentric (include/geometry/FIELD_3D.h:368-382).
ESF_HD void bary(double x, double dh, int ihigh, int& i, double& f) {
  x /= dh;
  double s = floor(x);
  int ii = (int)s;
  if (ii < 0) {
    i = 0;
    f = 0.5;
  } else if (ii > ihigh) {
    i = ihigh;
    f = 0.5;
  } else {
    i = ii;
    f = x - s;
  }
}
ESF_HD double lerpd(double a, double b, double f) { return (1 - f) * a + f * b; }

// FIELD_3D::interpolate_value (FIELD_3D.h:198-216) on a scalar grid.
ESF_HD double interp1(const double* __restrict__ d, int X, int Y, int Z, double dh,
                      const double* o, const double* p) {
  int i, j, k;
  double fx, fy, fz;
  bary(p[0] - o[0], dh, X - 2, i, fx);
  bary(p[1] - o[1], dh, Y - 2, j, fy);
  bary(p[2] - o[2], dh, Z - 2, k, fz);
  long long sl = (long long)X * Y;
  long long b = i + (long long)j * X + k * sl;
  double a0 = lerpd(lerpd(d[b], d[b + 1], fx), lerpd(d[b + X], d[b + X + 1], fx), fy);
  double a1 = lerpd(lerpd(d[b + sl], d[b + sl + 1], fx), lerpd(d[b + sl + X], d[b + sl + X + 1], fx), fy);
  return lerpd(a0, a1, fz);
}
// VEC3F_FIELD_3D::interpolate_value (VEC3F_FIELD_3D.h:179-197).
ESF_HD void interp3(const double* __restrict__ d, int X, int Y, int Z, double dh, const double* o,
                    const double* p, double* out) {
  int i, j, k;
  double fx, fy, fz;
  bary(p[0] - o[0], dh, X - 2, i, fx);
  bary(p[1] - o[1], dh, Y - 2, j, fy);
  bary(p[2] - o[2], dh, Z - 2, k, fz);
  long long sl = (long long)X * Y;
  long long b = i + (long long)j * X + k * sl;
#pragma unroll
  for (int c = 0; c < 3; c++) {
    const double* e = d + c;
    double a0 = lerpd(lerpd(e[3 * b], e[3 * (b + 1)], fx), lerpd(e[3 * (b + X)], e[3 * (b + X + 1)], fx), fy);
    double a1 = lerpd(lerpd(e[3 * (b + sl)], e[3 * (b + sl + 1)], fx),
                      lerpd(e[3 * (b + sl + X)], e[3 * (b + sl + X + 1)], fx), fy);
    out[c] = lerpd(a0, a1, fz);
  }
}

// corner i of a cell: x + (i&1), y + ((i>>1)&1), z + ((i>>2)&1); J sign
// pattern of COUPLED_INTEGRATOR_3D.cpp:241-243.
ESF_HD double sgnx(int i) { return (i % 2 == 0) ? -1.0 : 1.0; }
ESF_HD double sgny(int i) { return (i % 4 <= 1) ? -1.0 : 1.0; }
ESF_HD double sgnz(int i) { return (i < 4) ? -1.0 : 1.0; }

// ------------------------------------------------------------- solver state
// Device-resident scalars of one Conjugate Residual solve
// (CONJUGATE_RESIDUAL.inl:109-192). Written only by the last block of a
// kernel (ticket pattern), read by every block of the next kernel.
struct PcrState {
  double delta;      // r.s of the current iterate
  double alpha, beta;
  double bnorm2;     // ||b||^2
  double resid2;     // last ||Ax-b||^2
  double eps;
  int iter;          // current iteration i
  int maxIt;
  int done;          // 1: converged or stopped
  int converged;
  int setup;         // 1: next phase-B reduction initialises delta
  int status;        // 0 ok, 6 numeric (NaN met)
  int inner;         // 1: inner solve of a refinement, stops on delta/delta0
  double delta0;     // delta after set-up or after the last residual replacement
  int rebase;        // 1: next update reduction replaces the residual (keeps d)
  int iter0;         // iteration of the last replacement
  int cap;           // inner mode: iterations between replacements (0 = none)
  int pp;            // one-pass FP32 iteration: which buffer set holds r, t, q
  unsigned int ticket[4];
  double deltaPrev;  // one-pass double-float run: r.s of the iterate before the current one
};

// Solid system layout ("sliced"): the 27 neighbour 3x3 blocks of solid node a,
// entry je = 9 j + e, live at ((a / 32) * 243 + je) * 32 + a % 32, and the
// neighbour index of block j at ((a / 32) * 27 + j) * 32 + a % 32, so a warp's
// 32 rows read one contiguous region. Arrays hold S rounded up to 32 rows.
ESF_HD long long blk_at(long long a, int je) { return (((a >> 5) * 243 + je) << 5) + (a & 31); }
ESF_HD long long nbr_at(long long a, int j) { return (((a >> 5) * 27 + j) << 5) + (a & 31); }
ESF_HD long long rows32(long long S) { return (S + 31) & ~31LL; }

// Block partial sums live in a scratch array sized for the largest grid; the
// last block of each kernel folds them in block order (deterministic).
#define ESF_MAX_PARTIALS 65536

// ------------------------------------------------------------- host helpers
namespace esf {
void set_error(const char* fmt, ...);
const char* cuda_err(cudaError_t e);
// kernel-launch accounting: direct launches count once; launches made while
// a graph is being captured are counted per replay instead
void note_launch();
void note_graph_replay(unsigned long long kernels);
void set_capturing(bool on, unsigned long long* counter);
}  // namespace esf
#define ESF_COUNTED esf::note_launch(),

#define ESF_CUDA(call)                                                                  \
  do {                                                                                  \
    cudaError_t _e = (call);                                                            \
    if (_e != cudaSuccess) {                                                            \
      esf::set_error("%s:%d %s: %s", __FILE__, __LINE__, #call, cudaGetErrorString(_e)); \
      return (_e == cudaErrorMemoryAllocation) ? ESF_ERR_OOM : ESF_ERR_CUDA;            \
    }                                                                                   \
  } while (0)

#define ESF_LAUNCH_CHECK()                                                                  \
  do {                                                                                      \
    cudaError_t _e = cudaGetLastError();                                                    \
    if (_e != cudaSuccess) {                                                                \
      esf::set_error("%s:%d kernel launch: %s", __FILE__, __LINE__, cudaGetErrorString(_e)); \
      return ESF_ERR_CUDA;                                                                  \
    }                                                                                       \
  } while (0)

// ------------------------------------------------------------ solver API
namespace esf {
// Pressure operator J diag(minv) J^T (matrix-free; minv per node, zero on the
// boundary nodes). T = double or float.
template <typename T>
esf_status pressure_apply(const GridDev& g, const T* minv, const T* in, T* out, cudaStream_t st);

struct PressureWork;  // device work arrays of one pressure solve
esf_status pressure_work_alloc(PressureWork** w, const GridDev& g, int mixed);
void pressure_work_free(PressureWork* w);
// Full pressure solve; x is the warm start / result. minv64 per node.
esf_status pressure_solve(PressureWork* w, const GridDev& g, const double* minv64,
                          const double* diag64, const double* b, double* x, double eps, int maxIt,
                          int precision, double innerEps, int maxRefine, int* iters,
                          double* relres, int* refinements, int* converged, cudaStream_t st,
                          int* fp64Iters = nullptr);
// continuous batching of the mixed inner solves of several scenes (serving,
// batched solves): scenes whose pressure work is attached to a batcher hand
// their inner solves over to its thread and streams (esf_solver.cu)
struct InnerBatcher;
esf_status batcher_create(int device, InnerBatcher** out, bool autotune);
void batcher_destroy(InnerBatcher* b);
void batcher_stats(InnerBatcher* b, esf_batch_stats* out);
esf_status pressure_work_set_batcher(PressureWork* w, InnerBatcher* b);
// self-test of the TMA kernels' bounded mbarrier wait (esf_solver.cu)
esf_status selftest_mbar_wait(int* gaveUp, cudaStream_t st);
// allocation-free FP64 solve on the module's static scratch (esf_solver.cu)
esf_status static_scratch_address(void** out);
esf_status pressure_solve_static(void* scratch, const GridDev& g, const double* minv,
                                 const double* diag, const double* b, double* x, double eps,
                                 int maxIt, int* iters, double* relres, int* converged,
                                 cudaStream_t st);

// Average device time of the fused update kernel and of the axpy+norm kernel
// on scratch copies of the pressure problem (state untouched).
esf_status pressure_time_kernels(PressureWork* w, const GridDev& g, const double* minv64,
                                 const double* diag64, const double* b, const double* x,
                                 int precision, int reps, double* update_ms, double* axpy_ms,
                                 cudaStream_t st);

// Solid system in node-block form: for solid node a, 27 neighbour blocks of
// 3x3 (neighbour j = (dx+1) + 3(dy+1) + 9(dz+1)), nbr[a*27+j] = solid index
// or -1.
struct SolidWork;
esf_status solid_work_alloc(SolidWork** w, long long S, int mixed);
void solid_work_free(SolidWork* w);
long long solid_work_capacity(const SolidWork* w);
esf_status solid_solve(SolidWork* w, long long S, const double* blocks, const int* nbr,
                       const double* diag, const double* b, double* x, double eps, int maxIt,
                       int precision, double innerEps, int maxRefine, int* iters, double* relres,
                       int* refinements, int* converged, cudaStream_t st, const double* damped = nullptr);
// Mixed precision: the inner solves apply the stiffness matrix-free from the
// valid cells' recorded corotation data (cell: 43 planes of nc floats;
// corner: 8 planes of nc corner solid DOFs) instead of FP32 blocks; cell =
// NULL turns it off. damped (the assembled diagonal's mass part) is then
// passed to solid_solve.
esf_status solid_work_set_matrix_free(SolidWork* w, const GridDev& g, long long nc, const float* cell,
                                      const int* corner, const long long* sNode, const int* cellOrd,
                                      double mu, double lambda, double scale);
}  // namespace esf
