// Device kernels of the coupled step other than the linear solvers.
// Included only by esf_step.cu, which is compiled with -fmad=false so that
// cell flags, DOF maps, mass fractions and particle seeding reproduce the
// reference's (non-FMA, x86-64) arithmetic bit for bit.
#pragma once
#include <climits>

#include "esf_common.cuh"
#include "esf_contact.cuh"

namespace esf {

constexpr int KT = 256;
__device__ __forceinline__ double fmax_ref(double a, double b) { return (a < b) ? b : a; }

struct Box {
  int lo[3], hi[3];  // half-open
};
__device__ __forceinline__ long long box_count(const Box& b) {
  return (long long)max(0, b.hi[0] - b.lo[0]) * max(0, b.hi[1] - b.lo[1]) * max(0, b.hi[2] - b.lo[2]);
}
__device__ __forceinline__ void box_xyz(const Box& b, long long t, int& x, int& y, int& z) {
  int nx = b.hi[0] - b.lo[0], ny = b.hi[1] - b.lo[1];
  x = b.lo[0] + (int)(t % nx);
  y = b.lo[1] + (int)((t / nx) % ny);
  z = b.lo[2] + (int)(t / ((long long)nx * ny));
}
#define FOR_BOX(b, x, y, z)                                                                 \
  for (long long _t = blockIdx.x * (long long)blockDim.x + threadIdx.x, _n = box_count(b); \
       _t < _n; _t += (long long)gridDim.x * blockDim.x)                                    \
    if (int x, y, z; (box_xyz(b, _t, x, y, z), true))

#define FOR_N(n, i) \
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < (n); i += (long long)gridDim.x * blockDim.x)

__device__ __forceinline__ long long nidx(const GridDev& g, int x, int y, int z) {
  return x + (long long)y * g.X + (long long)z * g.slab;
}
__device__ __forceinline__ long long cidx(const GridDev& g, int x, int y, int z) {
  return x + (long long)y * g.cX + (long long)z * g.cslab;
}

struct SolidDev {
  double* X;
  double* u;
  double* vel;
  double* vws;
  double* tmp3;
  double* mass;
  double* phi;
  double* detFInv;
  double* quarter;  // 8 per node
  signed char* valid;  // per cell
  const double* rest;
  int mres[3];
  double mdh, morig[3];
  double lambda, mu, qcm;
  double G;  // 0.25 / dh
  double dt;
  // plasticity (setPlasticYield; material grid of loadSurfaceMesh)
  int plastic;
  double yield, flowRate;
  int pres[3];
  double pdh, porig[3];
  double* FpInv;    // 9 per material cell, row-major
  int* updIdx;      // per valid cell: material cell it updates, or -1
  double* updVal;   // per valid cell: the updated FpInv
  // mixed precision: per valid cell, the data of the matrix-free FP32
  // stiffness (MF_PLANES planes of nc floats: R, L, GF, Jinv dh^3), or null
  float* mf;
  long long mfCells;
};
// planes of the per-cell matrix-free data: R (row-major) 0-8, L 9-17, the
// F-weighted corner gradients GF 18-41 (corner i, component b at 18+3i+b),
// Jinv dh^3 at 42
constexpr int MF_PLANES = 43;

// --------------------------------------------------------- 3x3 helpers
// Templated on the arithmetic type: double everywhere on the reference's
// path; float for the stress evaluation of the mixed-precision path
// (k_element_stiffness_f32). The double instantiations are the reference's
// operation order.
template <class T>
struct M3T {
  T m[3][3];
};
using M3 = M3T<double>;
template <class T = double>
__device__ __forceinline__ M3T<T> m3_id() {
  M3T<T> r;
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) r.m[i][j] = (i == j) ? T(1) : T(0);
  return r;
}
template <class T>
__device__ __forceinline__ M3T<T> m3_mul(const M3T<T>& a, const M3T<T>& b) {
  M3T<T> r;
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) r.m[i][j] = (a.m[i][0] * b.m[0][j] + a.m[i][1] * b.m[1][j]) + a.m[i][2] * b.m[2][j];
  return r;
}
template <class T>
__device__ __forceinline__ M3T<T> m3_mul_bt(const M3T<T>& a, const M3T<T>& b) {
  M3T<T> r;
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) r.m[i][j] = (a.m[i][0] * b.m[j][0] + a.m[i][1] * b.m[j][1]) + a.m[i][2] * b.m[j][2];
  return r;
}
template <class T>
__device__ __forceinline__ M3T<T> m3_mul_at(const M3T<T>& a, const M3T<T>& b) {
  M3T<T> r;
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) r.m[i][j] = (a.m[0][i] * b.m[0][j] + a.m[1][i] * b.m[1][j]) + a.m[2][i] * b.m[2][j];
  return r;
}
// MatrixBase::determinant, 3x3 (Eigen/src/LU/Determinant.h:18-23, 61-68)
template <class T>
__device__ __forceinline__ T m3_det(const M3T<T>& a) {
  T h0 = a.m[0][0] * (a.m[1][1] * a.m[2][2] - a.m[1][2] * a.m[2][1]);
  T h1 = a.m[0][1] * (a.m[1][0] * a.m[2][2] - a.m[1][2] * a.m[2][0]);
  T h2 = a.m[0][2] * (a.m[1][0] * a.m[2][1] - a.m[1][1] * a.m[2][0]);
  return (h0 - h1) + h2;
}
template <class T>
__device__ __forceinline__ T cof3(const M3T<T>& a, int i, int j) {
  int i1 = (i + 1) % 3, i2 = (i + 2) % 3, j1 = (j + 1) % 3, j2 = (j + 2) % 3;
  return a.m[i1][j1] * a.m[i2][j2] - a.m[i1][j2] * a.m[i2][j1];
}
// compute_inverse<...,3> (Eigen/src/LU/Inverse.h:130-158)
template <class T>
__device__ __forceinline__ M3T<T> m3_inv(const M3T<T>& a) {
  T c0 = cof3(a, 0, 0), c1 = cof3(a, 1, 0), c2 = cof3(a, 2, 0);
  T det = c0 * a.m[0][0] + (c1 * a.m[1][0] + c2 * a.m[2][0]);
  T iv = T(1) / det;
  M3T<T> r;
  r.m[0][0] = c0 * iv;
  r.m[0][1] = c1 * iv;
  r.m[0][2] = c2 * iv;
#pragma unroll
  for (int i = 1; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) r.m[i][j] = cof3(a, j, i) * iv;
  return r;
}
__device__ __forceinline__ double sum3(double a, double b, double c) { return a + (b + c); }
__device__ __forceinline__ float sum3(float a, float b, float c) { return a + (b + c); }

// DEFOR_SOLID_3D::computeF (DEFOR_SOLID_3D.cpp:671-682) on the 8 corner
// displacements of the cell whose corner 0 is node `base`.
__device__ double compute_F(const GridDev& g, const double* __restrict__ u, long long base,
                            double Gs, M3& F) {
  double c[8][3];
  const long long off[8] = {0, 1, g.X, g.X + 1, g.slab, g.slab + 1, g.slab + g.X, g.slab + g.X + 1};
#pragma unroll
  for (int i = 0; i < 8; i++)
#pragma unroll
    for (int k = 0; k < 3; k++) c[i][k] = u[3 * (base + off[i]) + k];
  M3 Fi;
#pragma unroll
  for (int r = 0; r < 3; r++)
#pragma unroll
    for (int cc = 0; cc < 3; cc++) {
      double acc = c[0][r] * (Gs * (cc == 0 ? sgnx(0) : cc == 1 ? sgny(0) : sgnz(0)));
#pragma unroll
      for (int k = 1; k < 8; k++)
        acc += c[k][r] * (Gs * (cc == 0 ? sgnx(k) : cc == 1 ? sgny(k) : sgnz(k)));
      Fi.m[r][cc] = (r == cc ? 1.0 : 0.0) - acc;
    }
  double Jinv = m3_det(Fi);
  if (fabs(Jinv) > 1e-4) {
    F = m3_inv(Fi);
  } else {
    F = m3_id();
    Jinv = 1;
  }
  return 1.0 / Jinv;
}

// --------------------------------------------------------- initial state
// DEFOR_SOLID_3D::setInitialState + setInitialVelocity (DEFOR_SOLID_3D.cpp:126-155)
__global__ void k_initial_state(GridDev g, SolidDev s, const double* rot, double tx, double ty,
                                double tz, double sx, double sy, double sz, double vx, double vy,
                                double vz) {
  FOR_N(g.T, n) {
    int x = (int)(n % g.X), y = (int)((n / g.X) % g.Y), z = (int)(n / g.slab);
    double pt[3] = {(double)x, (double)y, (double)z};
    double tr[3] = {tx, ty, tz}, sc[3] = {sx, sy, sz};
#pragma unroll
    for (int k = 0; k < 3; k++) {
      pt[k] *= g.dh;
      pt[k] += g.o[k];
      pt[k] -= tr[k];
    }
    double q[3];
#pragma unroll
    for (int i = 0; i < 3; i++) q[i] = (rot[0 * 3 + i] * pt[0] + rot[1 * 3 + i] * pt[1]) + rot[2 * 3 + i] * pt[2];
    double pos[3] = {x * g.dh, y * g.dh, z * g.dh};
#pragma unroll
    for (int k = 0; k < 3; k++) {
      double X = q[k] / sc[k];
      s.X[3 * n + k] = X;
      s.u[3 * n + k] = (pos[k] + g.o[k]) - X;
    }
    s.vel[3 * n] = vx;
    s.vel[3 * n + 1] = vy;
    s.vel[3 * n + 2] = vz;
  }
}

// ----------------------------------------------------- solid mass (a17)
// DEFOR_SOLID_3D::computeSolidMass (DEFOR_SOLID_3D.cpp:576-669), first loop.
__global__ void k_det_finv(GridDev g, SolidDev s, Box cells) {
  FOR_BOX(cells, x, y, z) {
    long long n = nidx(g, x, y, z);
    M3 F;
    s.detFInv[n] = fabs(1.0 / compute_F(g, s.u, n, s.G, F));
  }
}

// Subsample loop: per-octant counts, then the reference's sequential sums of
// `fraction`, the 0.5 threshold and the valid flag (1 full, 2 partial).
__global__ void k_mass_subsample(GridDev g, SolidDev s, Box cells, int usesdf, double subDh,
                                 int res) {
  const double subVol = subDh * subDh * subDh;
  const int half = res >> 1;
  const double fraction = 1.0 / (double)(res * res * res);
  FOR_BOX(cells, x, y, z) {
    long long n = nidx(g, x, y, z);
    if (usesdf && s.phi[n] > 2) continue;
    double node[3] = {x * g.dh + g.o[0], y * g.dh + g.o[1], z * g.dh + g.o[2]};
    int cnt[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int p = 0; p < res; p++)
      for (int q = 0; q < res; q++)
        for (int r = 0; r < res; r++) {
          double pos[3] = {node[0] + (p + 0.5) * subDh, node[1] + (q + 0.5) * subDh,
                           node[2] + (r + 0.5) * subDh};
          double rp[3];
          interp3(s.X, g.X, g.Y, g.Z, g.dh, g.o, pos, rp);
          double d = interp1(s.rest, s.mres[0], s.mres[1], s.mres[2], s.mdh, s.morig, rp) * subVol;
          if (d < 1e-6) continue;
          int o = (p < half ? 0 : 1) + (q < half ? 0 : 2) + (r < half ? 0 : 4);
          cnt[o]++;
        }
    double qv[8];
    double sum = 0;
#pragma unroll
    for (int i = 0; i < 8; i++) {
      double a = 0;
      for (int k = 0; k < cnt[i]; k++) a += fraction;
      qv[i] = a;
    }
#pragma unroll
    for (int i = 0; i < 8; i++) sum += qv[i];
    signed char v = 0;
    if (sum > 0.5) {
#pragma unroll
      for (int i = 0; i < 8; i++) qv[i] = 1;
      v = 1;
    } else {
      if (sum > 0) v = 2;
#pragma unroll
      for (int i = 0; i < 8; i++) qv[i] = 0;
    }
    s.valid[cidx(g, x, y, z)] = v;
#pragma unroll
    for (int i = 0; i < 8; i++) s.quarter[8 * n + i] = qv[i];
  }
}

// Nodal mass: sum over the node's 8 cells in corner order i = 0..7 of the
// valid cells of the tight box (DEFOR_SOLID_3D.cpp:655-667).
__global__ void k_mass_gather(GridDev g, SolidDev s, Box cells, Box nodes) {
  FOR_BOX(nodes, x, y, z) {
    double m = 0;
#pragma unroll
    for (int i = 0; i < 8; i++) {
      int cx = x - (i & 1), cy = y - ((i >> 1) & 1), cz = z - ((i >> 2) & 1);
      if (cx < cells.lo[0] || cx >= cells.hi[0] || cy < cells.lo[1] || cy >= cells.hi[1] ||
          cz < cells.lo[2] || cz >= cells.hi[2])
        continue;
      if (!s.valid[cidx(g, cx, cy, cz)]) continue;
      long long c = nidx(g, cx, cy, cz);
      m += s.quarter[8 * c + i] * s.detFInv[c] * s.qcm;
    }
    s.mass[nidx(g, x, y, z)] = m;
  }
}

// ------------------------------------------------------------- SDF (a18)
// DEFOR_SOLID_3D::computeSDF (DEFOR_SOLID_3D.cpp:216-241): phi and the
// bounding box of the massive nodes (ints: xmin ymin zmin xmax ymax zmax).
// The box is reduced per warp and per block first: one atomic per block and
// bound instead of one per massive node (~237k nodes at 256^3 all hitting
// the same six words).
__global__ void __launch_bounds__(256) k_phi_init(GridDev g, SolidDev s, double large, int* bbox) {
  __shared__ int sb[6];
  if (threadIdx.x < 6) sb[threadIdx.x] = threadIdx.x < 3 ? INT_MAX : INT_MIN;
  __syncthreads();
  int lo[3] = {INT_MAX, INT_MAX, INT_MAX}, hi[3] = {INT_MIN, INT_MIN, INT_MIN};
  FOR_N(g.T, n) {
    if (s.mass[n] > 0) {
      s.phi[n] = -0.5;
      const int c[3] = {(int)(n % g.X), (int)((n / g.X) % g.Y), (int)(n / g.slab)};
#pragma unroll
      for (int q = 0; q < 3; q++) {
        lo[q] = min(lo[q], c[q]);
        hi[q] = max(hi[q], c[q]);
      }
    } else {
      s.phi[n] = large;
    }
  }
#pragma unroll
  for (int q = 0; q < 3; q++) {
    for (int o = 16; o > 0; o >>= 1) {
      lo[q] = min(lo[q], __shfl_down_sync(0xffffffffu, lo[q], o));
      hi[q] = max(hi[q], __shfl_down_sync(0xffffffffu, hi[q], o));
    }
  }
  if ((threadIdx.x & 31) == 0 && lo[0] != INT_MAX) {
#pragma unroll
    for (int q = 0; q < 3; q++) {
      atomicMin(&sb[q], lo[q]);
      atomicMax(&sb[3 + q], hi[q]);
    }
  }
  __syncthreads();
  if (threadIdx.x < 6 && sb[0] != INT_MAX) {
    if (threadIdx.x < 3) atomicMin(&bbox[threadIdx.x], sb[threadIdx.x]);
    else atomicMax(&bbox[threadIdx.x], sb[threadIdx.x]);
  }
}

// solveDistance (DEFOR_SOLID_3D.cpp:369-394)
__device__ __forceinline__ void solve_distance(double p, double q, double r, double* v) {
  // std::min / std::max semantics: (b < a) ? b : a
  double ds[3];
  double mqr = (r < q) ? r : q, Mqr = (q < r) ? r : q;
  ds[0] = (mqr < p) ? mqr : p;
  ds[2] = (p < Mqr) ? Mqr : p;
  ds[1] = p + q + r - ds[0] - ds[2];
  double b[3], c[3];
  b[0] = ds[0];
  c[0] = ds[0] * ds[0] - 1.0f;
  for (int x = 1; x < 3; x++) {
    b[x] = ds[x] + b[x - 1];
    c[x] = ds[x] * ds[x] + c[x - 1];
  }
  int i = 2;
  double discrim = b[i] * b[i] - (double)(i + 1) * c[i];
  double nd = (b[i] + sqrt(discrim)) / (double)(i + 1);
  while ((discrim < 0.0f || nd < ds[i]) && i != -1) {
    i--;
    if (i < 0) break;
    discrim = b[i] * b[i] - (double)(i + 1) * c[i];
    if (discrim > 0.0f) nd = (b[i] + sqrt(discrim)) / (double)(i + 1);
  }
  if (nd < *v) *v = nd;
}

// A Gauss-Seidel sweep pass (sweepPhi, sweepOnePass): node (i,j,k) reads
// its three upwind neighbours as updated in the same pass, so every order in
// which each node comes after its three upwind neighbours gives the
// sequential loop's result bit for bit. The pass runs as a wavefront of
// tiles (k_sweep_tile below).
struct Sweep {
  int i0, j0, k0;   // first index in sweep order
  int di, dj, dk;   // +1 / -1
  int ni, nj, nk;   // counts
};

// ---------------------------------------------- velocity extension (a19)
// DEFOR_SOLID_3D::sweepOnePass (DEFOR_SOLID_3D.cpp:457-519). Its
// solvableX/Y/Z flags live for the whole pass and, once cleared, stay
// cleared: a node sees a flag cleared iff some node at or before it in loop
// order triggered it. Triggers depend on phi and mass only (constant during
// the pass), so the first trigger rank of each flag is found by a min
// reduction before the wavefront runs.

// First trigger rank of the three pass-long flags of sweepOnePass, by
// atomicMin over all nodes of the pass (ranks: long long loop order).
__global__ void k_sweep_vec_ranks(GridDev g, const double* ph, const double* ms, Sweep w,
                                  unsigned long long* ranks) {
  __shared__ unsigned long long sm[3];
  if (threadIdx.x < 3) sm[threadIdx.x] = ~0ull;
  __syncthreads();
  unsigned long long r0 = ~0ull, r1 = ~0ull, r2 = ~0ull;
  const long long nij = (long long)w.ni * w.nj, total = nij * w.nk;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    int a = (int)(t % w.ni), b = (int)((t / w.ni) % w.nj), c = (int)(t / nij);
    int i = w.i0 + a * w.di, j = w.j0 + b * w.dj, k = w.k0 + c * w.dk;
    long long n = nidx(g, i, j, k);
    if (ms[n] != 0) continue;
    double pn = ph[n];
    double dp = pn - ph[nidx(g, i - w.di, j, k)], dpn = pn - ph[nidx(g, i + w.di, j, k)];
    if (dp < 0 && dpn >= 0) continue;
    if (dp < 0 && dpn < 0 && (unsigned long long)t < r0) r0 = t;
    double dq = pn - ph[nidx(g, i, j - w.dj, k)], dqn = pn - ph[nidx(g, i, j + w.dj, k)];
    if (dq < 0 && dqn >= 0) continue;
    if (dq < 0 && dqn < 0 && (unsigned long long)t < r1) r1 = t;
    double dr = pn - ph[nidx(g, i, j, k - w.dk)], drn = pn - ph[nidx(g, i, j, k + w.dk)];
    if (dr < 0 && drn >= 0) continue;
    if (dr < 0 && drn < 0 && (unsigned long long)t < r2) r2 = t;
  }
  // one shared-memory and one global atomic per block and flag
  if (r0 != ~0ull) atomicMin(&sm[0], r0);
  if (r1 != ~0ull) atomicMin(&sm[1], r1);
  if (r2 != ~0ull) atomicMin(&sm[2], r2);
  __syncthreads();
  if (threadIdx.x < 3 && sm[threadIdx.x] != ~0ull) atomicMin(&ranks[threadIdx.x], sm[threadIdx.x]);
}
// One launch of a sweep pass as a tile wavefront: the pass's nodes in
// sweep coordinates (a, b, c) are cut into ST^3 tiles, and launch P runs
// every tile (I, J, K) with I + J + K = P, whose three upwind tiles ran in
// launch P - 1. A block copies its tile and the upwind layer of each axis
// into shared memory, settles for each of its nodes what does not change
// during the pass (all nodes at once), sweeps the tile's sub-planes
// a'+b'+c' = q in order in shared memory (a barrier between sub-planes), and
// writes the tile back. PHI: the distance update of sweepPhi
// (DEFOR_SOLID_3D.cpp:397-455) on phi, for nodes without solid mass. VEC:
// the sweepOnePass update (DEFOR_SOLID_3D.cpp:457-519) of the three velocity
// components; its skip tests and blend weights depend on phi, the mass and
// the pass-long flags (resolved from the ranks of k_sweep_vec_ranks) only,
// none of which change during the pass, so they are formed up front.
constexpr int ST = 8;           // tile edge
constexpr int SP = ST + 1;      // tile plus the upwind layer
constexpr int SWEEP_THREADS = 128;  // blocks of the wave kernel
constexpr int TILE_THREADS = ST * ST * ST;  // one thread per node of a tile
static_assert(ST * ST <= TILE_THREADS, "one thread per (a', b') of a tile");
template <bool VEC>
__global__ void __launch_bounds__(TILE_THREADS) k_sweep_tile(GridDev g, double* f, double* ph,
                                                              const double* ms, Sweep w, int P,
                                                              const unsigned long long* ranks) {
  constexpr int NC = VEC ? 3 : 1;
  __shared__ double sv[NC * SP * SP * SP];
  __shared__ double sAlpha[VEC ? ST * ST * ST : 1], sBeta[VEC ? ST * ST * ST : 1];
  __shared__ unsigned char sUpd[ST * ST * ST];
  const int nti = (w.ni + ST - 1) / ST, ntj = (w.nj + ST - 1) / ST, ntk = (w.nk + ST - 1) / ST;
  const int I = blockIdx.x % nti, J = blockIdx.x / nti, K = P - I - J;
  if (J >= ntj || K < 0 || K >= ntk) return;
  const int a0 = I * ST, b0 = J * ST, c0 = K * ST;
  const int na = min(ST, w.ni - a0), nb = min(ST, w.nj - b0), nc = min(ST, w.nk - c0);
  double* const src = VEC ? f : ph;
  // tile and upwind layers: local -1 .. n-1 on each axis (local -1 of the
  // first tile is the node before the pass's first, inside the box)
  for (int t = threadIdx.x; t < SP * SP * SP; t += TILE_THREADS) {
    const int la = t % SP - 1, lb = (t / SP) % SP - 1, lc = t / (SP * SP) - 1;
    if (la >= na || lb >= nb || lc >= nc) continue;
    const long long n = nidx(g, w.i0 + (a0 + la) * w.di, w.j0 + (b0 + lb) * w.dj, w.k0 + (c0 + lc) * w.dk);
#pragma unroll
    for (int q = 0; q < NC; q++) sv[NC * t + q] = src[NC * n + q];
  }
  // per node of the tile: update or not, and (VEC) the blend weights
  const long long nij = (long long)w.ni * w.nj;
  for (int t = threadIdx.x; t < ST * ST * ST; t += TILE_THREADS) {
    const int la = t % ST, lb = (t / ST) % ST, lc = t / (ST * ST);
    unsigned char upd = 0;
    if (la < na && lb < nb && lc < nc) {
      const int a = a0 + la, b = b0 + lb, c = c0 + lc;
      const int i = w.i0 + a * w.di, j = w.j0 + b * w.dj, k = w.k0 + c * w.dk;
      const long long n = nidx(g, i, j, k);
      if (ms[n] == 0) {
        if (!VEC) {
          upd = 1;
        } else {
          const unsigned long long rank = (unsigned long long)(a + (long long)b * w.ni + (long long)c * nij);
          const double pn = ph[n];
          double dp = pn - ph[nidx(g, i - w.di, j, k)], dpn = pn - ph[nidx(g, i + w.di, j, k)];
          bool skip = dp < 0 && dpn >= 0;
          double dq = 0, dqn = 0, dr = 0, drn = 0;
          if (!skip) {
            dq = pn - ph[nidx(g, i, j - w.dj, k)];
            dqn = pn - ph[nidx(g, i, j + w.dj, k)];
            skip = dq < 0 && dqn >= 0;
          }
          if (!skip) {
            dr = pn - ph[nidx(g, i, j, k - w.dk)];
            drn = pn - ph[nidx(g, i, j, k + w.dk)];
            skip = dr < 0 && drn >= 0;
          }
          if (!skip) {
            if (rank >= ranks[0]) dp = 0;
            if (rank >= ranks[1]) dq = 0;
            if (rank >= ranks[2]) dr = 0;
            double alpha, beta;
            if (dp + dq + dr < 1e-3) {
              alpha = 0.333;
              beta = 0.333;
            } else {
              alpha = dp / (dp + dq + dr);
              beta = dq / (dp + dq + dr);
            }
            sAlpha[t] = alpha;
            sBeta[t] = beta;
            upd = 1;
          }
        }
      }
    }
    sUpd[t] = upd;
  }
  __syncthreads();
  const int la = threadIdx.x % ST, lb = threadIdx.x / ST;
  const bool mine = threadIdx.x < ST * ST && la < na && lb < nb;
  for (int q = 0; q <= (na - 1) + (nb - 1) + (nc - 1); q++) {
    const int lc = q - la - lb;
    if (mine && lc >= 0 && lc < nc) {
      const int u = la + lb * ST + lc * ST * ST;
      if (sUpd[u]) {
        const int s = (la + 1) + (lb + 1) * SP + (lc + 1) * SP * SP;
        const int sa = s - 1, sb = s - SP, sc = s - SP * SP;  // upwind in a, b, c
        if (!VEC) {
          solve_distance(sv[sa], sv[sb], sv[sc], &sv[s]);
        } else {
          const double alpha = sAlpha[u], beta = sBeta[u];
#pragma unroll
          for (int e = 0; e < 3; e++)
            sv[3 * s + e] = (alpha * sv[3 * sa + e] + beta * sv[3 * sb + e]) + (1 - alpha - beta) * sv[3 * sc + e];
        }
      }
    }
    __syncthreads();
  }
  for (int t = threadIdx.x; t < SP * SP * SP; t += TILE_THREADS) {
    const int ta = t % SP - 1, tb = (t / SP) % SP - 1, tc = t / (SP * SP) - 1;
    if (ta < 0 || tb < 0 || tc < 0 || ta >= na || tb >= nb || tc >= nc) continue;
    const long long n = nidx(g, w.i0 + (a0 + ta) * w.di, w.j0 + (b0 + tb) * w.dj, w.k0 + (c0 + tc) * w.dk);
#pragma unroll
    for (int e = 0; e < NC; e++) src[NC * n + e] = sv[NC * t + e];
  }
}
// A whole sweep pass in one cooperative launch: the blocks walk the pass's
// hyperplanes a + b + c = p in order, each plane split over all threads, with
// a grid-wide barrier between planes. Values written in this pass by other
// blocks are read through L2 (ld.cg); the barrier is one growing counter in
// global memory, its wait bounded (a block that gives up sets *err and
// carries on, so the launch always ends; the host reports it).
// Same per-node operations as k_sweep_tile, each node after its three
// upwind neighbours, so the same bits; the critical path is the 3n planes
// rather than the tile wavefront's ~9n sub-planes.
constexpr unsigned WAVE_WAIT_LIMIT = 1u << 22;
// Arrival p of every block: a release add on a counter that only grows (the
// host zeroes it before the launch), then acquire loads until it reaches
// (p + 1) x blocks.
__device__ __forceinline__ void wave_barrier(unsigned* count, unsigned target, int* err) {
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned cur;
    asm volatile("atom.add.release.gpu.global.u32 %0, [%1], 1;" : "=r"(cur) : "l"(count) : "memory");
    cur += 1;
    unsigned it = 0;
    while (cur < target && ++it < WAVE_WAIT_LIMIT)
      asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(cur) : "l"(count) : "memory");
    if (cur < target) *err = 1;
  }
  __syncthreads();
}
template <bool VEC>
__global__ void __launch_bounds__(SWEEP_THREADS) k_sweep_wave(GridDev g, double* f, double* ph,
                                                              const double* ms, Sweep w,
                                                              const unsigned long long* ranks,
                                                              unsigned* bar, int* err) {
  const long long nij = (long long)w.ni * w.nj;
  const int planes = w.ni + w.nj + w.nk - 2;
  unsigned long long rx = 0, ry = 0, rz = 0;
  if (VEC) {
    rx = ranks[0];
    ry = ranks[1];
    rz = ranks[2];
  }
  for (int p = 0; p < planes; p++) {
    for (long long t = blockIdx.x * (long long)SWEEP_THREADS + threadIdx.x; t < nij;
         t += (long long)gridDim.x * SWEEP_THREADS) {
      const int a = (int)(t % w.ni), b = (int)(t / w.ni);
      const int c = p - a - b;
      if (c < 0 || c >= w.nk) continue;
      const int i = w.i0 + a * w.di, j = w.j0 + b * w.dj, k = w.k0 + c * w.dk;
      const long long n = nidx(g, i, j, k);
      if (ms[n] != 0) continue;
      const long long ea = nidx(g, i - w.di, j, k), eb = nidx(g, i, j - w.dj, k), ec = nidx(g, i, j, k - w.dk);
      if (!VEC) {
        double v = __ldcg(ph + n);
        solve_distance(__ldcg(ph + ea), __ldcg(ph + eb), __ldcg(ph + ec), &v);
        ph[n] = v;
        continue;
      }
      const unsigned long long rank = (unsigned long long)(a + (long long)b * w.ni + (long long)c * nij);
      const double pn = ph[n];
      double dp = pn - ph[ea], dpn = pn - ph[nidx(g, i + w.di, j, k)];
      if (dp < 0 && dpn >= 0) continue;
      double dq = pn - ph[eb], dqn = pn - ph[nidx(g, i, j + w.dj, k)];
      if (dq < 0 && dqn >= 0) continue;
      double dr = pn - ph[ec], drn = pn - ph[nidx(g, i, j, k + w.dk)];
      if (dr < 0 && drn >= 0) continue;
      if (rank >= rx) dp = 0;
      if (rank >= ry) dq = 0;
      if (rank >= rz) dr = 0;
      double alpha, beta;
      if (dp + dq + dr < 1e-3) {
        alpha = 0.333;
        beta = 0.333;
      } else {
        alpha = dp / (dp + dq + dr);
        beta = dq / (dp + dq + dr);
      }
#pragma unroll
      for (int e = 0; e < 3; e++)
        f[3 * n + e] = (alpha * __ldcg(f + 3 * ea + e) + beta * __ldcg(f + 3 * eb + e)) +
                       (1 - alpha - beta) * __ldcg(f + 3 * ec + e);
    }
    wave_barrier(bar, (unsigned)(p + 1) * gridDim.x, err);
  }
}

// Launches of one sweep pass as a tile wavefront.
inline int sweep_tile_launches(const Sweep& w) {
  return (w.ni + ST - 1) / ST + (w.nj + ST - 1) / ST + (w.nk + ST - 1) / ST - 2;
}
inline int sweep_tile_blocks(const Sweep& w) {
  return ((w.ni + ST - 1) / ST) * ((w.nj + ST - 1) / ST);
}

// Face copies of sweepVectorField (DEFOR_SOLID_3D.cpp:544-563), one axis
// per launch, in the order z, y, x.
__global__ void k_extend_faces(GridDev g, double* f, const double* ms, Box ex, int axis) {
  int a0, a1;
  if (axis == 2) {
    a0 = 0;
    a1 = 1;
  } else if (axis == 1) {
    a0 = 0;
    a1 = 2;
  } else {
    a0 = 1;
    a1 = 2;
  }
  const long long n0 = ex.hi[a0] - ex.lo[a0], n1 = ex.hi[a1] - ex.lo[a1];
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n0 * n1;
       t += (long long)gridDim.x * blockDim.x) {
    int c[3];
    c[a0] = ex.lo[a0] + (int)(t % n0);
    c[a1] = ex.lo[a1] + (int)(t / n0);
    int cc[3] = {c[0], c[1], c[2]};
    cc[axis] = ex.lo[axis];
    long long A = nidx(g, cc[0], cc[1], cc[2]);
    cc[axis] = ex.lo[axis] + 1;
    long long B = nidx(g, cc[0], cc[1], cc[2]);
    if (ms[A] == 0)
      for (int q = 0; q < 3; q++) f[3 * A + q] = f[3 * B + q];
    cc[axis] = ex.hi[axis] - 1;
    A = nidx(g, cc[0], cc[1], cc[2]);
    cc[axis] = ex.hi[axis] - 2;
    B = nidx(g, cc[0], cc[1], cc[2]);
    if (ms[A] == 0)
      for (int q = 0; q < 3; q++) f[3 * A + q] = f[3 * B + q];
  }
}

// -------------------------------------------------- particles (a20-a22)
// DEFOR_SOLID_3D::initMaterialParticles (DEFOR_SOLID_3D.cpp:333-367): the
// v-th valid cell of the tight box (z, y, x order) seeds particles
// v*ppc .. v*ppc+ppc-1; particle p consumes MT19937 outputs 3p..3p+2 as the
// z, y, x offsets (the argument order in which the reference's x86-64 build
// evaluates VEC3F(rand, rand, rand)).
__global__ void k_flag_valid_cells(GridDev g, SolidDev s, Box cells, int* flag) {
  FOR_BOX(cells, x, y, z) {
    long long t = (x - cells.lo[0]) + (long long)(cells.hi[0] - cells.lo[0]) *
                                          ((y - cells.lo[1]) + (long long)(cells.hi[1] - cells.lo[1]) * (z - cells.lo[2]));
    flag[t] = (s.valid[cidx(g, x, y, z)] == 1) ? 1 : 0;
  }
}
__global__ void k_collect_valid_cells(GridDev g, Box cells, const int* flag, const int* scan,
                                      long long* list) {
  FOR_BOX(cells, x, y, z) {
    long long t = (x - cells.lo[0]) + (long long)(cells.hi[0] - cells.lo[0]) *
                                          ((y - cells.lo[1]) + (long long)(cells.hi[1] - cells.lo[1]) * (z - cells.lo[2]));
    if (flag[t]) list[scan[t]] = nidx(g, x, y, z);
  }
}
__global__ void k_seed_particles(GridDev g, SolidDev s, const long long* cellList, long long nCells,
                                 int ppc, const uint32_t* mt, double pmass, double* part) {
  FOR_N(nCells * ppc, p) {
    long long n = cellList[p / ppc];
    int x = (int)(n % g.X), y = (int)((n / g.X) % g.Y), z = (int)(n / g.slab);
    double grid[3] = {g.o[0] + x * g.dh, g.o[1] + y * g.dh, g.o[2] + z * g.dh};
    double r2 = ((double)mt[3 * p] * (1.0 / 4294967295.0)) * g.dh;
    double r1 = ((double)mt[3 * p + 1] * (1.0 / 4294967295.0)) * g.dh;
    double r0 = ((double)mt[3 * p + 2] * (1.0 / 4294967295.0)) * g.dh;
    double* P = part + 10 * p;
    double pos[3] = {grid[0] + r0, grid[1] + r1, grid[2] + r2};
    P[0] = pos[0];
    P[1] = pos[1];
    P[2] = pos[2];
    double rp[3], v[3];
    interp3(s.X, g.X, g.Y, g.Z, g.dh, g.o, pos, rp);
    interp3(s.vel, g.X, g.Y, g.Z, g.dh, g.o, pos, v);
    P[3] = v[0];
    P[4] = v[1];
    P[5] = v[2];
    P[6] = rp[0];
    P[7] = rp[1];
    P[8] = rp[2];
    P[9] = pmass;
  }
}

// cubic B-spline weight of gridToParticle/particleToGrid
// (DEFOR_SOLID_3D.cpp:928-935); |d|^3 as a product (the reference's
// pow(d, 3) agrees to an ulp).
__device__ __forceinline__ double bspline(double d) {
  double a = fabs(d);
  double c = a * a * a;
  if (a < 1) return 0.5 * c - d * d + 2.0 / 3;
  if (a < 2) return -1.0 / 6 * c + d * d - 2 * a + 4.0 / 3;
  return 0;
}
// The 4 weights per axis of a particle's 4^3 stencil, whose first node is
// floor((p - o)/dh) - 1 on each axis: w[4*axis + k] for node base + k.
__device__ __forceinline__ void stencil_weights(const GridDev& g, const double* pos, int base[3],
                                                double w[12]) {
#pragma unroll
  for (int q = 0; q < 3; q++) {
    base[q] = (int)floor((pos[q] - g.o[q]) / g.dh) - 1;
    const double f = g.dhInv * (pos[q] - g.o[q]);
#pragma unroll
    for (int k = 0; k < 4; k++) w[4 * q + k] = bspline(f - (base[q] + k));
  }
}

struct ContactParams {
  double wallThickness, spring, friction, alpha;
  double bnd[6];
};

// DEFOR_SOLID_3D::gridToParticle (DEFOR_SOLID_3D.cpp:891-1034): FLIP/PIC
// blend, one solid-solid contact impulse (the first neighbour the particle
// touches), one wall contact impulse, then p += v dt.
__global__ void k_grid_to_particle(GridDev g, SolidDev s, long long np, double* part,
                                   ContactParams cp, const ContactSet cs) {
  FOR_N(np, c) {
    double* P = part + 10 * c;
    double pos[3] = {P[0], P[1], P[2]};
    int i = (int)floor((pos[0] - g.o[0]) / g.dh) - 1;
    int j = (int)floor((pos[1] - g.o[1]) / g.dh) - 1;
    int k = (int)floor((pos[2] - g.o[2]) / g.dh) - 1;
    double pic[3] = {0, 0, 0}, flip[3] = {0, 0, 0};
    int bb[3];
    double wt[12];
    stencil_weights(g, pos, bb, wt);
    // (offsets as compile-time indices keep the weights in registers)
#pragma unroll
    for (int dr = 0; dr < 4; dr++)
#pragma unroll
      for (int dt = 0; dt < 4; dt++)
#pragma unroll
        for (int ds = 0; ds < 4; ds++) {
          const int r = k + dr, t = j + dt, sx = i + ds;
          if (sx < 0 || t < 0 || r < 0 || sx > g.X - 1 || t > g.Y - 1 || r > g.Z - 1) continue;
          long long n = nidx(g, sx, t, r);
          if (s.mass[n] == 0) continue;
          double w = wt[ds] * wt[4 + dt] * wt[8 + dr];
          for (int q = 0; q < 3; q++) {
            double v = s.vel[3 * n + q];
            pic[q] += v * w;
            flip[q] += (v - s.vws[3 * n + q]) * w;
          }
        }
    double pv[3];
    for (int q = 0; q < 3; q++) {
      flip[q] += P[3 + q];
      pv[q] = (1 - cp.alpha) * pic[q] + cp.alpha * flip[q];
    }
    int ci = (int)floor((pos[0] - g.o[0]) / g.dh), cj = (int)floor((pos[1] - g.o[1]) / g.dh),
        ck = (int)floor((pos[2] - g.o[2]) / g.dh);
    ci = min(max(ci, 0), g.X - 2);
    cj = min(max(cj, 0), g.Y - 2);
    ck = min(max(ck, 0), g.Z - 2);
    // collision with the other solids (:967-995): B's rest SDF at the
    // particle's position in B's rest space
    for (int y = 0; y < cs.n; y++) {
      const ContactNeighbor& B = cs.nb[y];
      if (interp1(B.phi, g.X, g.Y, g.Z, g.dh, g.o, pos) > 2) continue;
      double restPos[3], normal[3] = {0.0, 0.0, 0.0};
      interp3(B.X, g.X, g.Y, g.Z, g.dh, g.o, pos, restPos);
      const double sdf = sdf_contact(B.sdf, restPos, cs.thickness, normal);
      if (sdf > cs.thickness) continue;
      const double overlap = cs.thickness - sdf;
      double vo[3];
      interp3(B.vel, g.X, g.Y, g.Z, g.dh, g.o, pos, vo);
      double vrel[3] = {pv[0] - vo[0], pv[1] - vo[1], pv[2] - vo[2]};
      const double vn = (vrel[0] * normal[0] + vrel[1] * normal[1]) + vrel[2] * normal[2];
      if (vn <= 0 || sdf <= 0) {
        const double A = s.dt * cp.spring * overlap, Bv = P[9] * (0.1 * overlap / s.dt - vn);
        const double impulse = -((Bv < A) ? Bv : A);
        const double dvn = -impulse / P[9];
        double vt[3];
        for (int q = 0; q < 3; q++) vt[q] = vrel[q] - vn * normal[q];
        const double vtn = sqrt(vt[0] * vt[0] + (vt[1] * vt[1] + vt[2] * vt[2]));  // as the wall's vt.norm()
        double sc = 1 - cp.friction * dvn / vtn;
        sc = (sc < 0.0) ? 0.0 : sc;  // std::max(sc, 0.0)
        for (int q = 0; q < 3; q++) pv[q] = ((vn + dvn) * normal[q] + sc * vt[q]) + vo[q];
        if (cs.contacts) atomicAdd(cs.contacts, 1ull);
        break;
      }
    }
    for (int b = 0; b < 6; b++) {
      // wall normal b: +x, +y, +z, -x, -y, -z (the values, not a table, so
      // nothing is indexed at run time)
      double N[3];
      for (int q = 0; q < 3; q++) N[q] = (q == b % 3) ? (b < 3 ? 1.0 : -1.0) : 0.0;
      double dist = fabs(pos[b % 3] - cp.bnd[b]);
      if (dist < cp.wallThickness) {
        double overlap = cp.wallThickness - dist;
        int xi = ci, yi = cj, zi = ck;
        if (b == 0) xi = 0;
        else if (b == 3) xi = g.X - 1;
        if (b == 1) yi = 0;
        else if (b == 4) yi = g.Y - 1;
        if (b == 2) zi = 0;
        else if (b == 5) zi = g.Z - 1;
        const double* vo = s.vel + 3 * nidx(g, xi, yi, zi);
        double vrel[3] = {pv[0] - vo[0], pv[1] - vo[1], pv[2] - vo[2]};
        double vn = (vrel[0] * N[0] + vrel[1] * N[1]) + vrel[2] * N[2];
        if (vn <= 0) {
          double A = s.dt * cp.spring * overlap, B = P[9] * (0.1 * overlap / s.dt - vn);
          double impulse = -((B < A) ? B : A);
          double dvn = -impulse / P[9];
          double vt[3];
          for (int q = 0; q < 3; q++) vt[q] = vrel[q] - vn * N[q];
          double vtn = sqrt(vt[0] * vt[0] + (vt[1] * vt[1] + vt[2] * vt[2]));
          double sc = 0.1 - cp.friction * dvn / vtn;
          sc = (sc < 0.0) ? 0.0 : sc;
          for (int q = 0; q < 3; q++) pv[q] = ((vn + dvn) * N[q] + sc * vt[q]) + vo[q];
          break;
        }
      }
    }
    for (int q = 0; q < 3; q++) {
      P[3 + q] = pv[q];
      P[q] = pos[q] + pv[q] * s.dt;
    }
  }
}

// P2G binning: key = stencil base node shifted by +3 per axis on an
// (X+3)(Y+3)(Z+3) lattice; particles whose stencil misses the grid get the
// key `nkeys` (sorted last, never gathered).
// Keys, stencil weights and the particles' index box (reduced per warp and
// block, one atomic per block and bound; the box words start at
// +/- 2^30 on the host).
__global__ void __launch_bounds__(256) k_p2g_keys(GridDev g, long long np, const double* part, unsigned int* keys,
                                                  unsigned int* vals, int* pbox, double* pw) {
  __shared__ int sb[6];
  if (threadIdx.x < 6) sb[threadIdx.x] = threadIdx.x < 3 ? INT_MAX : INT_MIN;
  __syncthreads();
  int lo[3] = {INT_MAX, INT_MAX, INT_MAX}, hi[3] = {INT_MIN, INT_MIN, INT_MIN};
  const long long KX = g.X + 3, KY = g.Y + 3, KZ = g.Z + 3;
  FOR_N(np, c) {
    const double* P = part + 10 * c;
    int bb[3];
    double wt[12];
    stencil_weights(g, P, bb, wt);
    for (int q = 0; q < 12; q++) pw[12 * c + q] = wt[q];
    int i = bb[0], j = bb[1], k = bb[2];
    unsigned int key = (unsigned int)(KX * KY * KZ);
    if (i >= -3 && i <= g.X - 1 && j >= -3 && j <= g.Y - 1 && k >= -3 && k <= g.Z - 1) {
      key = (unsigned int)((i + 3) + KX * ((j + 3) + KY * (k + 3)));
      lo[0] = min(lo[0], i);
      lo[1] = min(lo[1], j);
      lo[2] = min(lo[2], k);
      hi[0] = max(hi[0], i);
      hi[1] = max(hi[1], j);
      hi[2] = max(hi[2], k);
    }
    keys[c] = key;
    vals[c] = (unsigned int)c;
  }
#pragma unroll
  for (int q = 0; q < 3; q++) {
    for (int o = 16; o > 0; o >>= 1) {
      lo[q] = min(lo[q], __shfl_down_sync(0xffffffffu, lo[q], o));
      hi[q] = max(hi[q], __shfl_down_sync(0xffffffffu, hi[q], o));
    }
  }
  if ((threadIdx.x & 31) == 0 && lo[0] != INT_MAX) {
#pragma unroll
    for (int q = 0; q < 3; q++) {
      atomicMin(&sb[q], lo[q]);
      atomicMax(&sb[3 + q], hi[q]);
    }
  }
  __syncthreads();
  if (threadIdx.x < 6 && sb[0] != INT_MAX) {
    if (threadIdx.x < 3) atomicMin(&pbox[threadIdx.x], sb[threadIdx.x]);
    else atomicMax(&pbox[threadIdx.x], sb[threadIdx.x]);
  }
}
__global__ void k_bucket_bounds(long long np, const unsigned int* skeys, int* bstart, int* bend,
                                unsigned int nkeys) {
  FOR_N(np, c) {
    unsigned int k = skeys[c];
    if (k >= nkeys) continue;
    if (c == 0 || skeys[c - 1] != k) bstart[k] = (int)c;
    if (c == np - 1 || skeys[c + 1] != k) bend[k] = (int)c + 1;
  }
}
// DEFOR_SOLID_3D::particleToGrid (DEFOR_SOLID_3D.cpp:1036-1107) as a
// per-node gather over the 4^3 buckets whose stencils reach the node, in
// bucket order then particle order (deterministic).
__global__ void k_p2g_gather(GridDev g, SolidDev s, Box nodes, const double* part,
                             const double* pw, const unsigned int* sval, const int* bstart,
                             const int* bend, int cutoff) {
  const long long KX = g.X + 3, KY = g.Y + 3;
  FOR_BOX(nodes, x, y, z) {
    double acc[4] = {0, 0, 0, 0};
    bool touched = false;
    for (int bz = z - 3; bz <= z; bz++)
      for (int by = y - 3; by <= y; by++)
        for (int bx = x - 3; bx <= x; bx++) {
          if (bx < -3 || by < -3 || bz < -3) continue;
          long long key = (bx + 3) + KX * ((by + 3) + KY * (long long)(bz + 3));
          int b0 = bstart[key], b1 = bend[key];
          const int ox = x - bx, oy = 4 + y - by, oz = 8 + z - bz;
          for (int e = b0; e < b1; e++) {
            const long long pi = sval[e];
            const double* P = part + 10 * pi;
            const double* W = pw + 12 * pi;
            double w = W[ox] * W[oy] * W[oz];
            touched = true;
            acc[0] += w * P[3];
            acc[1] += w * P[4];
            acc[2] += w * P[5];
            acc[3] += w;
          }
        }
    long long n = nidx(g, x, y, z);
    if (touched && !(acc[3] < (double)cutoff)) {
      for (int q = 0; q < 3; q++) s.vel[3 * n + q] = acc[q] / acc[3];
      s.mass[n] = 1;
    }
  }
}

// ------------------------------------------------ solid advection (a16)
__global__ void k_copy_grid_velocity(GridDev g, SolidDev s, Box ex, const double* vel) {
  FOR_BOX(ex, x, y, z) {
    long long n = nidx(g, x, y, z);
    for (int q = 0; q < 3; q++) s.vel[3 * n + q] = vel[3 * n + q];
  }
}
// u += v dt; u_new(x) = I(u)(x - v(x) dt)  (DEFOR_SOLID_3D.cpp:1200-1203, 1108-1123)
__global__ void k_u_add(GridDev g, SolidDev s) {
  FOR_N(3 * g.T, i) s.u[i] += s.vel[i] * s.dt;
}
__global__ void k_u_advect(GridDev g, SolidDev s) {
  FOR_N(g.T, n) {
    int x = (int)(n % g.X), y = (int)((n / g.X) % g.Y), z = (int)(n / g.slab);
    double node[3] = {(double)x, (double)y, (double)z};
    double p[3];
    for (int q = 0; q < 3; q++) {
      node[q] = node[q] * g.dh + g.o[q];
      p[q] = node[q] - s.vel[3 * n + q] * s.dt;
    }
    interp3(s.u, g.X, g.Y, g.Z, g.dh, g.o, p, s.tmp3 + 3 * n);
  }
}
// bbox face extrapolation, one axis per launch (DEFOR_SOLID_3D.cpp:1206-1220)
__global__ void k_u_extrapolate(GridDev g, double* u, Box ex, int axis) {
  int a0, a1;
  if (axis == 2) {
    a0 = 0;
    a1 = 1;
  } else if (axis == 1) {
    a0 = 0;
    a1 = 2;
  } else {
    a0 = 1;
    a1 = 2;
  }
  long long n0 = ex.hi[a0] - ex.lo[a0], n1 = ex.hi[a1] - ex.lo[a1];
  FOR_N(n0 * n1, t) {
    int c[3];
    c[a0] = ex.lo[a0] + (int)(t % n0);
    c[a1] = ex.lo[a1] + (int)(t / n0);
    int lo = ex.lo[axis], hi = ex.hi[axis];
    int cc[3] = {c[0], c[1], c[2]};
    cc[axis] = lo;
    long long A = nidx(g, cc[0], cc[1], cc[2]);
    cc[axis] = lo + 1;
    long long B = nidx(g, cc[0], cc[1], cc[2]);
    cc[axis] = lo + 2;
    long long C = nidx(g, cc[0], cc[1], cc[2]);
    for (int q = 0; q < 3; q++) u[3 * A + q] = 2 * u[3 * B + q] - u[3 * C + q];
    cc[axis] = hi - 1;
    A = nidx(g, cc[0], cc[1], cc[2]);
    cc[axis] = hi - 2;
    B = nidx(g, cc[0], cc[1], cc[2]);
    cc[axis] = hi - 3;
    C = nidx(g, cc[0], cc[1], cc[2]);
    for (int q = 0; q < 3; q++) u[3 * A + q] = 2 * u[3 * B + q] - u[3 * C + q];
  }
}
// X = x - u; vecWorkspace = velocity (DEFOR_SOLID_3D.cpp:1222-1232)
__global__ void k_recover_X(GridDev g, SolidDev s) {
  FOR_N(g.T, n) {
    int x = (int)(n % g.X), y = (int)((n / g.X) % g.Y), z = (int)(n / g.slab);
    double pos[3] = {x * g.dh, y * g.dh, z * g.dh};
    for (int q = 0; q < 3; q++) {
      s.X[3 * n + q] = pos[q] + (g.o[q] - s.u[3 * n + q]);
      s.vws[3 * n + q] = s.vel[3 * n + q];
    }
  }
}

// DEFOR_SOLID_3D::readFrame (DEFOR_SOLID_3D.cpp:1305-1316): workspace =
// velocity, X = (node position + origin) - u
__global__ void k_frame_X(GridDev g, SolidDev s) {
  FOR_N(g.T, n) {
    int x = (int)(n % g.X), y = (int)((n / g.X) % g.Y), z = (int)(n / g.slab);
    double pos[3] = {x * g.dh, y * g.dh, z * g.dh};
    for (int q = 0; q < 3; q++) {
      s.vws[3 * n + q] = s.vel[3 * n + q];
      s.X[3 * n + q] = (pos[q] + g.o[q]) - s.u[3 * n + q];
    }
  }
}

// --------------------------------------------------- surface mesh (a24)
// DEFOR_SOLID_3D::advectSurfaceMesh (DEFOR_SOLID_3D.cpp:1125-1180)
__global__ void k_advect_mesh(GridDev g, SolidDev s, int nv, double* verts, const double* rest) {
  FOR_N(nv, v) {
    double* vx = verts + 3 * v;
    double p[3] = {vx[0], vx[1], vx[2]};
    double vel[3];
    interp3(s.vel, g.X, g.Y, g.Z, g.dh, g.o, p, vel);
    for (int q = 0; q < 3; q++) p[q] += vel[q] * s.dt;
    double residual = 1;
    int count = 0;
    while (residual > 1e-4 && count++ < 10) {
      double uu[3], diff[3];
      interp3(s.u, g.X, g.Y, g.Z, g.dh, g.o, p, uu);
      for (int q = 0; q < 3; q++) diff[q] = (p[q] - uu[q]) - rest[3 * v + q];
      residual = sqrt(diff[0] * diff[0] + (diff[1] * diff[1] + diff[2] * diff[2]));
      int i = (int)((p[0] - g.o[0]) / g.dh);
      i = i < 0 ? 0 : (i > g.X - 2 ? g.X - 2 : i);
      int j = (int)((p[1] - g.o[1]) / g.dh);
      j = j < 0 ? 0 : (j > g.Y - 2 ? g.Y - 2 : j);
      int k = (int)((p[2] - g.o[2]) / g.dh);
      k = k < 0 ? 0 : (k > g.Z - 2 ? g.Z - 2 : k);
      M3 F;
      compute_F(g, s.u, nidx(g, i, j, k), s.G, F);
      for (int r = 0; r < 3; r++) p[r] -= (F.m[r][0] * diff[0] + F.m[r][1] * diff[1]) + F.m[r][2] * diff[2];
    }
    double hi[3] = {g.o[0] + g.dh * (g.X - 1), g.o[1] + g.dh * (g.Y - 1), g.o[2] + g.dh * (g.Z - 1)};
    for (int q = 0; q < 3; q++) {
      double a = (p[q] < g.o[q]) ? g.o[q] : p[q];
      vx[q] = (hi[q] < a) ? hi[q] : a;
    }
  }
}
// vertex AABB of the triangle vertices (TRIANGLE_BVH::refit root box)
__global__ void k_mesh_aabb(int ntri, const int* tris, const double* verts, unsigned long long* box) {
  FOR_N(3LL * ntri, t) {
    const double* v = verts + 3 * tris[t];
    for (int q = 0; q < 3; q++) {
      // order-preserving map of doubles onto unsigned 64-bit integers
      unsigned long long b = (unsigned long long)__double_as_longlong(v[q]);
      b = (b >> 63) ? ~b : (b | 0x8000000000000000ull);
      atomicMin(&box[q], b);
      atomicMax(&box[3 + q], b);
    }
  }
}

// TRIANGLE_BVH::collide (TRIANGLE_BVH.cpp:187-200) without the tree: two
// meshes collide when a triangle of one and a triangle of the other have
// overlapping bounding boxes (aabb::overlaps, closed intervals). A node's box
// holds its leaves' boxes, so the tree walk reports exactly these pairs.
__global__ void k_mesh_pair_overlap(int na, const int* ta, const double* va, int nb, const int* tb,
                                    const double* vb, int* hit) {
  FOR_N((long long)na * nb, t) {
    if (*(volatile int*)hit) return;
    const int i = (int)(t / nb), j = (int)(t % nb);
    double amin[3], amax[3], bmin[3], bmax[3];
    for (int k = 0; k < 3; k++) {
      amin[k] = amax[k] = va[3 * ta[3 * i] + k];
      bmin[k] = bmax[k] = vb[3 * tb[3 * j] + k];
    }
    for (int c = 1; c < 3; c++)
      for (int k = 0; k < 3; k++) {
        const double x = va[3 * ta[3 * i + c] + k], y = vb[3 * tb[3 * j + c] + k];
        amin[k] = fmin(amin[k], x);
        amax[k] = fmax(amax[k], x);
        bmin[k] = fmin(bmin[k], y);
        bmax[k] = fmax(bmax[k], y);
      }
    bool overlap = true;
    for (int k = 0; k < 3; k++)
      if (amin[k] > bmax[k] || amax[k] < bmin[k]) overlap = false;
    if (overlap) atomicExch(hit, 1);
  }
}

// SPARSE_SDF::signedDistAndCurrentNormal at given rest points (the contact
// query alone, for checking it against the reference's).
__global__ void k_rest_sdf_query(RestSdfDev s, int n, const double* pts, double safe, double* sd, double* normal) {
  FOR_N(n, i) {
    double nrm[3] = {0.0, 0.0, 0.0};
    sd[i] = sdf_contact(s, pts + 3 * i, safe, nrm);
    for (int k = 0; k < 3; k++) normal[3 * i + k] = nrm[k];
  }
}

// ------------------------------------------- integrator node kernels
// gatherSolidMasses (COUPLED_INTEGRATOR_3D.cpp:327-375) for solid `si`:
// accumulate its mass and quarter fractions (si == 0 initialises).
__global__ void k_gather_accumulate(GridDev g, const SolidDev s, int first, double* solidMass,
                                    double* quarter) {
  FOR_N(g.T, n) {
    solidMass[n] = first ? (0.0 + s.mass[n]) : solidMass[n] + s.mass[n];
    for (int i = 0; i < 8; i++)
      quarter[8 * n + i] = first ? (0.0 + s.quarter[8 * n + i]) : quarter[8 * n + i] + s.quarter[8 * n + i];
  }
}
// node volume fraction: cells with corner 0 in the interior, i = 0..7 order,
// times 0.125; solid-node flags for the DOF scan.
__global__ void k_node_vf(GridDev g, const double* quarter, const double* solidMass, double* vf,
                          int* flag) {
  FOR_N(g.T, n) {
    int x = (int)(n % g.X), y = (int)((n / g.X) % g.Y), z = (int)(n / g.slab);
    double a = 0;
#pragma unroll
    for (int i = 0; i < 8; i++) {
      int cx = x - (i & 1), cy = y - ((i >> 1) & 1), cz = z - ((i >> 2) & 1);
      if (cx < 1 || cx > g.X - 2 || cy < 1 || cy > g.Y - 2 || cz < 1 || cz > g.Z - 2) continue;
      a += quarter[8 * nidx(g, cx, cy, cz) + i];
    }
    vf[n] = a * 0.125;
    bool interior = x > 0 && x < g.X - 1 && y > 0 && y < g.Y - 1 && z > 0 && z < g.Z - 1;
    flag[n] = (interior && solidMass[n] > 0) ? 1 : 0;
  }
}
__global__ void k_sdof(GridDev g, const int* flag, const int* scan, int* sdof, long long* sNode) {
  FOR_N(g.T, n) {
    if (flag[n]) {
      sdof[n] = scan[n];
      sNode[scan[n]] = n;
    } else {
      sdof[n] = -1;
    }
  }
}
// DEFOR_SOLID_3D::recoverVelocityField (DEFOR_SOLID_3D.cpp:1235-1241)
__global__ void k_recover_velocity(GridDev g, SolidDev s, Box b, double* vel) {
  FOR_BOX(b, x, y, z) {
    long long n = nidx(g, x, y, z);
    if (s.mass[n] > 0)
      for (int q = 0; q < 3; q++) vel[3 * n + q] = s.vel[3 * n + q];
  }
}

// max_k |v_k| over interior nodes with solid mass (COUPLED_INTEGRATOR_3D::CFL :88-102)
__global__ void k_cfl_vmax(GridDev g, const double* vel, const double* solidMass,
                           unsigned long long* out) {
  FOR_N(g.T, n) {
    int x = (int)(n % g.X), y = (int)((n / g.X) % g.Y), z = (int)(n / g.slab);
    if (x < 1 || x > g.X - 2 || y < 1 || y > g.Y - 2 || z < 1 || z > g.Z - 2) continue;
    if (!(solidMass[n] > 0)) continue;
    double m = fmax(fmax(fabs(vel[3 * n]), fabs(vel[3 * n + 1])), fabs(vel[3 * n + 2]));
    atomicMax(out, (unsigned long long)__double_as_longlong(m));
  }
}


// ----------------------------------------------------- material (a5-a8)
// Cyclic Jacobi eigen-decomposition of the symmetric F^T F (stands in for
// Eigen::JacobiSVD in COROTATION::svd, COROTATION.cpp:239; R, S and L are
// invariant to its sign and order choices). Sweeps stop when the
// off-diagonal mass falls to the type's rounding level.
template <class T>
struct JacobiTol;
template <>
struct JacobiTol<double> {
  static constexpr double tiny = 1e-300, rel = 1e-18;
};
template <>
struct JacobiTol<float> {
  static constexpr float tiny = 1e-30f, rel = 1e-7f;
};
template <class T>
__device__ void sym_eig3(const M3T<T>& A, T w[3], M3T<T>& V) {
  T a[3][3];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) a[i][j] = A.m[i][j];
  M3T<T> v = m3_id<T>();
  for (int sweep = 0; sweep < 50; sweep++) {
    T off = fabs(a[0][1]) + fabs(a[0][2]) + fabs(a[1][2]);
    T scale = fabs(a[0][0]) + fabs(a[1][1]) + fabs(a[2][2]);
    if (off == T(0) || off <= JacobiTol<T>::tiny + JacobiTol<T>::rel * scale) break;
    for (int p = 0; p < 2; p++)
      for (int q = p + 1; q < 3; q++) {
        T apq = a[p][q];
        if (apq == T(0)) continue;
        T theta = (a[q][q] - a[p][p]) / (T(2) * apq);
        T t = (theta >= T(0) ? T(1) : T(-1)) / (fabs(theta) + sqrt(theta * theta + T(1)));
        T c = T(1) / sqrt(t * t + T(1)), s = t * c;
        for (int k = 0; k < 3; k++) {
          T akp = a[k][p], akq = a[k][q];
          a[k][p] = c * akp - s * akq;
          a[k][q] = s * akp + c * akq;
        }
        for (int k = 0; k < 3; k++) {
          T apk = a[p][k], aqk = a[q][k];
          a[p][k] = c * apk - s * aqk;
          a[q][k] = s * apk + c * aqk;
        }
        for (int k = 0; k < 3; k++) {
          T vkp = v.m[k][p], vkq = v.m[k][q];
          v.m[k][p] = c * vkp - s * vkq;
          v.m[k][q] = s * vkp + c * vkq;
        }
      }
  }
  int ord[3] = {0, 1, 2};
  T d[3] = {a[0][0], a[1][1], a[2][2]};
  for (int i = 0; i < 3; i++)
    for (int j = i + 1; j < 3; j++)
      if (d[ord[j]] > d[ord[i]]) {
        int t = ord[i];
        ord[i] = ord[j];
        ord[j] = t;
      }
  for (int c = 0; c < 3; c++) {
    w[c] = d[ord[c]] < T(0) ? T(0) : d[ord[c]];
    for (int r = 0; r < 3; r++) V.m[r][c] = v.m[r][ord[c]];
  }
}

template <class T>
struct CorotT {
  T lambda, mu;
  M3T<T> R, S, L;
  M3T<T> V, Fh;  // of the decomposition (COROTATION::V(), Fhat())
  T w[3];        // eigenvalues of F^T F, descending
};
using Corot = CorotT<double>;

// COROTATION::orthogonalizeU (COROTATION.cpp:127-230)
template <class T>
__device__ void orthogonalize_u(M3T<T>& U, const M3T<T>& Fh) {
  T signU = (m3_det(U) >= T(0)) ? T(1) : T(-1);
  int inv[3] = {0, 0, 0}, total = 0;
  for (int x = 0; x < 3; x++)
    if (Fh.m[x][x] < T(1e-4)) {
      inv[x] = 1;
      total++;
    }
  if (total == 0) return;
  if (total == 1) {
    int w = inv[2] ? 2 : (inv[1] ? 1 : 0);
    T c0[3], c1[3], c2[3];
    for (int r = 0; r < 3; r++) {
      c0[r] = U.m[r][(w + 1) % 3];
      c1[r] = U.m[r][(w + 2) % 3];
    }
    c2[0] = c0[1] * c1[2] - c0[2] * c1[1];
    c2[1] = c0[2] * c1[0] - c0[0] * c1[2];
    c2[2] = c0[0] * c1[1] - c0[1] * c1[0];
    T n = sqrt(c2[0] * c2[0] + (c2[1] * c2[1] + c2[2] * c2[2]));
    if (n > T(0))
      for (int r = 0; r < 3; r++) c2[r] /= n;
    for (int r = 0; r < 3; r++) U.m[r][w] = c2[r];
    if (signU * m3_det(U) < T(0))
      for (int r = 0; r < 3; r++) U.m[r][w] = -c2[r];
    return;
  }
  if (total == 2) {
    int wv = !inv[2] ? 2 : (!inv[1] ? 1 : 0);
    T v[3] = {U.m[0][wv], U.m[1][wv], U.m[2][wv]};
    int sm = (fabs(v[0]) < fabs(v[1])) ? 0 : 1;
    sm = (fabs(v[2]) < fabs(v[sm])) ? 2 : sm;
    T sv[3];
    int nx = (sm + 1) % 3, nn = (sm + 2) % 3;
    sv[sm] = T(0);
    sv[nx] = -v[nn];
    sv[nn] = v[nx];
    T tv[3] = {v[1] * sv[2] - v[2] * sv[1], v[2] * sv[0] - v[0] * sv[2], v[0] * sv[1] - v[1] * sv[0]};
    T n = sqrt(tv[0] * tv[0] + (tv[1] * tv[1] + tv[2] * tv[2]));
    if (n > T(0))
      for (int r = 0; r < 3; r++) tv[r] /= n;
    nx = (wv + 1) % 3;
    nn = (wv + 2) % 3;
    for (int r = 0; r < 3; r++) {
      U.m[r][nx] = sv[r];
      U.m[r][nn] = tv[r];
    }
    if (signU * m3_det(U) < T(0)) {
      if (Fh.m[nx][nx] < Fh.m[nn][nn])
        for (int r = 0; r < 3; r++) U.m[r][nx] = -sv[r];
      else
        for (int r = 0; r < 3; r++) U.m[r][nn] = -tv[r];
    }
    return;
  }
  U = m3_id<T>();
}

// COROTATION::init -> decomposeF -> svd (COROTATION.cpp:37-39, 91-107, 235-280)
template <class T>
__device__ void corot_init(CorotT<T>& c, const M3T<T>& F) {
  M3T<T> FtF = m3_mul_at(F, F);
  M3T<T> V;
  sym_eig3(FtF, c.w, V);
  M3T<T> Fh;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) Fh.m[i][j] = T(0);
  for (int i = 0; i < 3; i++) {
    Fh.m[i][i] = sqrt(c.w[i]);
    if (isnan(Fh.m[i][i])) Fh.m[i][i] = T(0);
  }
  if (m3_det(V) < T(0))
    for (int r = 0; r < 3; r++) V.m[r][0] *= T(-1);
  M3T<T> D;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) D.m[i][j] = T(0);
  for (int i = 0; i < 3; i++) D.m[i][i] = (Fh.m[i][i] > T(0)) ? T(1) / Fh.m[i][i] : T(0);
  M3T<T> U = m3_mul(m3_mul(F, V), D);
  orthogonalize_u(U, Fh);
  if (m3_det(F) < T(0)) {
    int sm = (Fh.m[0][0] < Fh.m[1][1]) ? 0 : 1;
    sm = (Fh.m[sm][sm] < Fh.m[2][2]) ? sm : 2;
    Fh.m[sm][sm] *= T(-1);
    for (int r = 0; r < 3; r++) U.m[r][sm] *= T(-1);
  }
  c.R = m3_mul_bt(U, V);
  c.S = m3_mul_bt(m3_mul(V, Fh), V);
  c.V = V;
  c.Fh = Fh;
  T trF = sum3(Fh.m[0][0], Fh.m[1][1], Fh.m[2][2]);
  T trFm1 = sum3(Fh.m[0][0] - T(1), Fh.m[1][1] - T(1), Fh.m[2][2] - T(1));
  M3T<T> Tm;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) Tm.m[i][j] = (i == j ? trF : T(0)) - Fh.m[i][j];
  M3T<T> Ti = m3_inv(Tm);
  T k = c.lambda * trFm1 - T(2) * c.mu;
  M3T<T> Ld;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) Ld.m[i][j] = (i == j ? c.mu : T(0)) + k * Ti.m[i][j];
  for (int i = 0; i < 3; i++) Ld.m[i][i] = Ld.m[i][i] > T(0) ? Ld.m[i][i] : T(0);
  c.L = m3_mul_bt(m3_mul(V, Ld), V);
}

// COROTATION::firstPKDifferential (COROTATION.cpp:64-84) for dF = e_j (x) gf
// (row j of dF is gf): the 24 columns of the element stiffness
// (DEFOR_SOLID_3D.cpp:805-827).
template <class T>
__device__ M3T<T> corot_dpk_row(const CorotT<T>& c, int j, const T* gf) {
  M3T<T> dFh;  // R^T dF
  for (int a = 0; a < 3; a++)
    for (int b = 0; b < 3; b++) dFh.m[a][b] = c.R.m[j][a] * gf[b];
  M3T<T> sym, skew;
  for (int a = 0; a < 3; a++)
    for (int b = 0; b < 3; b++) {
      sym.m[a][b] = T(0.5) * (dFh.m[a][b] + dFh.m[b][a]);
      skew.m[a][b] = T(0.5) * (dFh.m[a][b] - dFh.m[b][a]);
    }
  T trs = sum3(sym.m[0][0], sym.m[1][1], sym.m[2][2]);
  M3T<T> dP;
  for (int a = 0; a < 3; a++)
    for (int b = 0; b < 3; b++) dP.m[a][b] = (T(2) * c.mu * sym.m[a][b]) + (a == b ? c.lambda * trs : T(0));
  T f[3] = {-skew.m[1][2] + skew.m[2][1], -skew.m[2][0] + skew.m[0][2], -skew.m[0][1] + skew.m[1][0]};
  T tr = c.lambda * sum3(dFh.m[0][0], dFh.m[1][1], dFh.m[2][2]);
  for (int a = 0; a < 3; a++) dP.m[a][a] += tr;
  T Lf[3];
  for (int a = 0; a < 3; a++) Lf[a] = (c.L.m[a][0] * f[0] + c.L.m[a][1] * f[1]) + c.L.m[a][2] * f[2];
  dP.m[0][1] += -Lf[2];
  dP.m[0][2] += Lf[1];
  dP.m[1][0] += Lf[2];
  dP.m[1][2] += -Lf[0];
  dP.m[2][0] += -Lf[1];
  dP.m[2][1] += Lf[0];
  return m3_mul(c.R, dP);
}

// DEFOR_SOLID_3D::computeStiffnessMatrixAndMaterialForce
// (DEFOR_SOLID_3D.cpp:697-871), one thread per valid cell: stores the
// cell's 24x24 stiffness (row k, column i) and its 3x8 nodal forces.
// ||A|| (Eigen's norm()): squares in column-major order, summed as two-lane
// packets ((a0,a1)+(a2,a3)) + ((a4,a5)+(a6,a7)), lanes added, then the ninth
__device__ double m3_norm(const M3& a) {
  double q[9];
  for (int j = 0; j < 3; j++)
    for (int i = 0; i < 3; i++) q[j * 3 + i] = a.m[i][j] * a.m[i][j];
  const double l0 = (q[0] + q[2]) + (q[4] + q[6]);
  const double l1 = (q[1] + q[3]) + (q[5] + q[7]);
  return sqrt((l0 + l1) + q[8]);
}

// FpInv write-back after the stiffness sweep: per material cell the update
// of the last valid cell in sweep order (z, y, x) wins, as the reference's
// serial map assignment does (DEFOR_SOLID_3D.cpp:862-868)
__global__ void k_fp_winner(const int* upd, long long nc, int* winner) {
  FOR_N(nc, t) {
    const int m = upd[t];
    if (m >= 0) atomicMax(&winner[m], (int)t);
  }
}
__global__ void k_fp_apply(const int* upd, const double* val, long long nc, const int* winner,
                           double* FpInv) {
  FOR_N(nc, t) {
    const int m = upd[t];
    if (m >= 0 && winner[m] == (int)t)
      for (int q = 0; q < 9; q++) FpInv[9 * m + q] = val[9 * t + q];
  }
}

// slotOf/ncDev (both NULL on the reference's path): entry t of `cells` is
// the valid cell of ordinal slotOf[t], and only the first *ncDev entries are
// used (the FP32 kernel's FP64 fallback list, below).
__global__ void k_element_stiffness(GridDev g, SolidDev s, const long long* cells, long long nc,
                                    double* Ke, double* nf, double* energyPart,
                                    const long long* slotOf, const unsigned* ncDev) {
  double dh = g.dh;
  double e = 0;
  const long long off[8] = {0, 1, g.X, g.X + 1, g.slab, g.slab + 1, g.slab + g.X, g.slab + g.X + 1};
  if (ncDev) nc = *ncDev;
  FOR_N(nc, tt) {
    const long long t = slotOf ? slotOf[tt] : tt;
    long long n = cells[tt];
    M3 F;
    double Jinv = 1.0 / compute_F(g, s.u, n, s.G, F);
    Corot c;
    c.lambda = s.lambda;
    c.mu = s.mu;
    M3 E, cs;
    double trE;
    // P = R (2 mu E + lambda tr(E) I), E = S - I  (COROTATION.cpp:53-62);
    // cauchy = Jinv P F^T
    auto stress = [&]() {
      corot_init(c, F);
      E = c.S;
      for (int i = 0; i < 3; i++) E.m[i][i] -= 1.0;
      M3 tmp;
      for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) tmp.m[i][j] = 2.0 * c.mu * E.m[i][j];
      trE = sum3(E.m[0][0], E.m[1][1], E.m[2][2]);
      for (int i = 0; i < 3; i++) tmp.m[i][i] += c.lambda * trE;
      M3 P = m3_mul(c.R, tmp);
      M3 JP;
      for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) JP.m[i][j] = Jinv * P.m[i][j];
      cs = m3_mul_bt(JP, F);
    };
    stress();
    // plasticity (DEFOR_SOLID_3D.cpp:765-791): above the yield stress the
    // elastic part F FpInv is used and a flow step on the singular values
    // gives the cell's FpInv update, written after the sweep (k_fp_apply)
    if (s.plastic) {
      int upd = -1;
      if (m3_norm(cs) > s.yield) {
        double rp[3] = {0, 0, 0};
        for (int i = 0; i < 8; i++)
          for (int k = 0; k < 3; k++) rp[k] += s.X[3 * (n + off[i]) + k];
        for (int k = 0; k < 3; k++) rp[k] /= 8;
        int ci[3];
        for (int k = 0; k < 3; k++) {
          int i = (int)floor((rp[k] - s.porig[k]) / s.pdh);
          ci[k] = i <= 0 ? 0 : (i >= s.pres[k] - 1 ? s.pres[k] - 1 : i);
        }
        const int mc = (ci[2] * s.pres[1] + ci[1]) * s.pres[0] + ci[0];
        M3 Fp;
        for (int i = 0; i < 3; i++)
          for (int j = 0; j < 3; j++) Fp.m[i][j] = s.FpInv[9 * mc + 3 * i + j];
        F = m3_mul(F, Fp);
        stress();
        const double cN = m3_norm(cs);
        if (cN > s.yield) {
          const double gamma = s.flowRate * (cN - s.yield) / cN;
          const double cr = cbrt(1.0 / fmax(fabs(Jinv), 1e-3));
          M3 Fh = c.Fh;
          for (int i = 0; i < 3; i++) Fh.m[i][i] = pow(Fh.m[i][i] / cr, -gamma);
          const M3 nFp = m3_mul(m3_mul_bt(m3_mul(c.V, Fh), c.V), Fp);
          bool bad = false;
          for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) bad |= nFp.m[i][j] != nFp.m[i][j];
          if (!bad) {
            upd = mc;
            for (int i = 0; i < 3; i++)
              for (int j = 0; j < 3; j++) s.updVal[9 * t + 3 * i + j] = nFp.m[i][j];
          }
        }
      }
      s.updIdx[t] = upd;
    }
    double GF[8][3];
    for (int i = 0; i < 8; i++) {
      double gi[3] = {sgnx(i) * s.G, sgny(i) * s.G, sgnz(i) * s.G};
      for (int j = 0; j < 3; j++) GF[i][j] = (gi[0] * F.m[0][j] + gi[1] * F.m[1][j]) + gi[2] * F.m[2][j];
    }
    if (s.mf) {
      float* q = s.mf + t;
      const long long P = s.mfCells;
      for (int i = 0; i < 9; i++) {
        q[i * P] = (float)c.R.m[i / 3][i % 3];
        q[(9 + i) * P] = (float)c.L.m[i / 3][i % 3];
      }
      for (int i = 0; i < 8; i++)
        for (int b = 0; b < 3; b++) q[(18 + 3 * i + b) * P] = (float)GF[i][b];
      q[42 * P] = (float)(((Jinv * dh) * dh) * dh);
    }
    double* nft = nf + 24 * t;
    for (int r = 0; r < 3; r++)
      for (int m = 0; m < 8; m++) {
        double gm[3] = {sgnx(m) * s.G, sgny(m) * s.G, sgnz(m) * s.G};
        double v = (cs.m[r][0] * gm[0] + cs.m[r][1] * gm[1]) + cs.m[r][2] * gm[2];
        nft[r * 8 + m] = 0.0 - ((v * dh) * dh) * dh;
      }
    // strainEnergy (COROTATION.cpp:42-49)
    M3 EtE = m3_mul_at(E, E);
    e += (c.mu * sum3(EtE.m[0][0], EtE.m[1][1], EtE.m[2][2]) + 0.5 * c.lambda * (trE * trE)) * dh * dh * dh;
    double* K = Ke + 576 * t;
    for (int k = 0; k < 24; k++) {
      int ci = k / 3, cj = k % 3;
      bool on = s.mass[n + off[ci]] != 0;
      M3 dP;
      if (on) dP = corot_dpk_row(c, cj, GF[ci]);
      for (int m = 0; m < 8; m++)
        for (int r = 0; r < 3; r++) {
          double v = 0;
          if (on) {
            double t2 = (dP.m[r][0] * GF[m][0] + dP.m[r][1] * GF[m][1]) + dP.m[r][2] * GF[m][2];
            v = 0.0 + (((t2 * Jinv) * dh) * dh) * dh;
          }
          K[(m * 3 + r) * 24 + k] = v;
        }
    }
  }
  __shared__ double sh[32];
  // per-block energy (deterministic order) -> energyPart[block]
  for (int o = 16; o > 0; o >>= 1) e += __shfl_down_sync(0xffffffffu, e, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = e;
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0;
    for (int w = 0; w < (int)blockDim.x / 32; w++) a += sh[w];
    energyPart[blockIdx.x] = a;
  }
}


// Mixed precision: the stress evaluation and element stiffness of
// k_element_stiffness in FP32 (F from the displacements in FP64, then the
// polar decomposition, PK1, forces, energy and the 24x24 stiffness in FP32).
// A cell whose F is near-degenerate (cond(F) = sqrt(w_max / w_min) > 1e3 from
// the eigenvalues w of F^T F, or w_min = 0) is not evaluated here: it is
// appended to a list that k_element_stiffness then evaluates in FP64, the
// reference's arithmetic. Elastic solids only (plastic ones use the FP64
// kernel throughout).
__global__ void k_element_stiffness_f32(GridDev g, SolidDev s, const long long* cells, long long nc,
                                        double* Ke, double* nf, double* energyPart, long long* fbCells,
                                        long long* fbSlot, unsigned* fbCount) {
  const float dh = (float)g.dh;
  double e = 0;
  const long long off[8] = {0, 1, g.X, g.X + 1, g.slab, g.slab + 1, g.slab + g.X, g.slab + g.X + 1};
  FOR_N(nc, t) {
    long long n = cells[t];
    M3 Fd;
    const double Jinvd = 1.0 / compute_F(g, s.u, n, s.G, Fd);
    M3T<float> F;
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) F.m[i][j] = (float)Fd.m[i][j];
    const float Jinv = (float)Jinvd;
    CorotT<float> c;
    c.lambda = (float)s.lambda;
    c.mu = (float)s.mu;
    corot_init(c, F);
    if (!(c.w[2] > 0.0f) || c.w[0] > 1e6f * c.w[2]) {
      const unsigned k = atomicAdd(fbCount, 1u);
      fbCells[k] = n;
      fbSlot[k] = t;
      continue;
    }
    M3T<float> E = c.S;
    for (int i = 0; i < 3; i++) E.m[i][i] -= 1.0f;
    M3T<float> tmp;
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) tmp.m[i][j] = 2.0f * c.mu * E.m[i][j];
    const float trE = sum3(E.m[0][0], E.m[1][1], E.m[2][2]);
    for (int i = 0; i < 3; i++) tmp.m[i][i] += c.lambda * trE;
    const M3T<float> P = m3_mul(c.R, tmp);
    M3T<float> JP;
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) JP.m[i][j] = Jinv * P.m[i][j];
    const M3T<float> cs = m3_mul_bt(JP, F);
    const float G = (float)s.G;
    float GF[8][3];
    for (int i = 0; i < 8; i++) {
      const float gi[3] = {(float)sgnx(i) * G, (float)sgny(i) * G, (float)sgnz(i) * G};
      for (int j = 0; j < 3; j++) GF[i][j] = (gi[0] * F.m[0][j] + gi[1] * F.m[1][j]) + gi[2] * F.m[2][j];
    }
    const float dh3 = dh * dh * dh;
    if (s.mf) {
      float* q = s.mf + t;
      const long long P = s.mfCells;
      for (int i = 0; i < 9; i++) {
        q[i * P] = c.R.m[i / 3][i % 3];
        q[(9 + i) * P] = c.L.m[i / 3][i % 3];
      }
      for (int i = 0; i < 8; i++)
        for (int b = 0; b < 3; b++) q[(18 + 3 * i + b) * P] = GF[i][b];
      q[42 * P] = Jinv * dh3;
    }
    double* nft = nf + 24 * t;
    for (int r = 0; r < 3; r++)
      for (int m = 0; m < 8; m++) {
        const float gm[3] = {(float)sgnx(m) * G, (float)sgny(m) * G, (float)sgnz(m) * G};
        const float v = (cs.m[r][0] * gm[0] + cs.m[r][1] * gm[1]) + cs.m[r][2] * gm[2];
        nft[r * 8 + m] = (double)(-(v * dh3));
      }
    const M3T<float> EtE = m3_mul_at(E, E);
    e += (double)((c.mu * sum3(EtE.m[0][0], EtE.m[1][1], EtE.m[2][2]) + 0.5f * c.lambda * (trE * trE)) * dh3);
    double* K = Ke + 576 * t;
    const float scale = Jinv * dh3;
    for (int k = 0; k < 24; k++) {
      const int ci = k / 3, cj = k % 3;
      const bool on = s.mass[n + off[ci]] != 0;
      M3T<float> dP;
      if (on) dP = corot_dpk_row(c, cj, GF[ci]);
      for (int m = 0; m < 8; m++)
        for (int r = 0; r < 3; r++) {
          float v = 0.0f;
          if (on) v = ((dP.m[r][0] * GF[m][0] + dP.m[r][1] * GF[m][1]) + dP.m[r][2] * GF[m][2]) * scale;
          K[(m * 3 + r) * 24 + k] = (double)v;
        }
    }
  }
  __shared__ double sh[32];
  for (int o = 16; o > 0; o >>= 1) e += __shfl_down_sync(0xffffffffu, e, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = e;
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0;
    for (int w = 0; w < (int)blockDim.x / 32; w++) a += sh[w];
    energyPart[blockIdx.x] = a;
  }
}

// Mixed precision: semi-Lagrangian advection of the fluid velocity and of the
// scalar intensity (k_advect_velocity / k_advect_scalar) in FP32 arithmetic
// on the FP64 fields: the same backtrace, bisection into the fluid and
// trilinear interpolation (FIELD_3D::get_barycentric's clamping).
__device__ __forceinline__ void bary_f(float x, float dhInv, int ihigh, int& i, float& f) {
  x *= dhInv;
  const float s = floorf(x);
  const int ii = (int)s;
  if (ii < 0) {
    i = 0;
    f = 0.5f;
  } else if (ii > ihigh) {
    i = ihigh;
    f = 0.5f;
  } else {
    i = ii;
    f = x - s;
  }
}
__device__ __forceinline__ float lerp_f(float a, float b, float f) { return (1.0f - f) * a + f * b; }
__device__ __forceinline__ long long cell_f(const GridDev& g, const float* p, float o[3], float dhInv,
                                            float fr[3]) {
  int i, j, k;
  bary_f(p[0] - o[0], dhInv, g.X - 2, i, fr[0]);
  bary_f(p[1] - o[1], dhInv, g.Y - 2, j, fr[1]);
  bary_f(p[2] - o[2], dhInv, g.Z - 2, k, fr[2]);
  return i + (long long)j * g.X + k * g.slab;
}
__device__ __forceinline__ float interp1_f(const GridDev& g, const double* __restrict__ d, const float* p,
                                           float o[3], float dhInv) {
  float f[3];
  const long long b = cell_f(g, p, o, dhInv, f), X = g.X, sl = g.slab;
  const float a0 = lerp_f(lerp_f((float)d[b], (float)d[b + 1], f[0]),
                          lerp_f((float)d[b + X], (float)d[b + X + 1], f[0]), f[1]);
  const float a1 = lerp_f(lerp_f((float)d[b + sl], (float)d[b + sl + 1], f[0]),
                          lerp_f((float)d[b + sl + X], (float)d[b + sl + X + 1], f[0]), f[1]);
  return lerp_f(a0, a1, f[2]);
}
__device__ __forceinline__ void interp3_f(const GridDev& g, const double* __restrict__ d, const float* p,
                                          float o[3], float dhInv, float out[3]) {
  float f[3];
  const long long b = cell_f(g, p, o, dhInv, f), X = g.X, sl = g.slab;
#pragma unroll
  for (int c = 0; c < 3; c++) {
    const double* e = d + c;
    const float a0 = lerp_f(lerp_f((float)e[3 * b], (float)e[3 * (b + 1)], f[0]),
                            lerp_f((float)e[3 * (b + X)], (float)e[3 * (b + X + 1)], f[0]), f[1]);
    const float a1 = lerp_f(lerp_f((float)e[3 * (b + sl)], (float)e[3 * (b + sl + 1)], f[0]),
                            lerp_f((float)e[3 * (b + sl + X)], (float)e[3 * (b + sl + X + 1)], f[0]), f[1]);
    out[c] = lerp_f(a0, a1, f[2]);
  }
}
__global__ void k_advect_velocity_f32(GridDev g, const double* solidMass, const double* vel, double* out,
                                      double dtd) {
  float o[3] = {(float)g.o[0], (float)g.o[1], (float)g.o[2]};
  const float dh = (float)g.dh, dhInv = (float)g.dhInv, dt = (float)dtd;
  FOR_N(g.T, n) {
    int x = (int)(n % g.X), y = (int)((n / g.X) % g.Y), z = (int)(n / g.slab);
    if (x < 1 || x > g.X - 2 || y < 1 || y > g.Y - 2 || z < 1 || z > g.Z - 2) continue;
    if (solidMass[n] > 0) continue;
    const float node[3] = {x * dh + o[0], y * dh + o[1], z * dh + o[2]};
    float p[3], v[3], np[3], r[3];
    for (int q = 0; q < 3; q++) p[q] = node[q] - 0.5f * (float)vel[3 * n + q] * dt;
    interp3_f(g, vel, p, o, dhInv, v);
    for (int q = 0; q < 3; q++) np[q] = node[q] - v[q] * dt;
    float mass = interp1_f(g, solidMass, np, o, dhInv);
    float newdt = dt / 2;
    while (mass > 0.0f && newdt > dt / 16) {
      for (int q = 0; q < 3; q++) np[q] += v[q] * newdt;
      newdt /= 2;
      mass = interp1_f(g, solidMass, np, o, dhInv);
    }
    interp3_f(g, vel, np, o, dhInv, r);
    for (int q = 0; q < 3; q++) out[3 * n + q] = (double)r[q];
  }
}
__global__ void k_advect_scalar_f32(GridDev g, const double* solidMass, const double* vel,
                                    const double* field, double* out, double dtd) {
  float o[3] = {(float)g.o[0], (float)g.o[1], (float)g.o[2]};
  const float dh = (float)g.dh, dhInv = (float)g.dhInv, dt = (float)dtd;
  FOR_N(g.T, n) {
    int x = (int)(n % g.X), y = (int)((n / g.X) % g.Y), z = (int)(n / g.slab);
    if (solidMass[n] > 0) {
      out[n] = 0.0;
      continue;
    }
    const float node[3] = {x * dh + o[0], y * dh + o[1], z * dh + o[2]};
    float np[3], v[3];
    for (int q = 0; q < 3; q++) {
      v[q] = (float)vel[3 * n + q];
      np[q] = node[q] - v[q] * dt;
    }
    float mass = interp1_f(g, solidMass, np, o, dhInv);
    float newdt = dt / 2;
    while (mass > 0.0f && newdt > dt / 16) {
      for (int q = 0; q < 3; q++) np[q] += v[q] * newdt;
      newdt /= 2;
      mass = interp1_f(g, solidMass, np, o, dhInv);
    }
    out[n] = (double)interp1_f(g, field, np, o, dhInv);
  }
}

// Per solid node: the 27 neighbour blocks of sum_cells K_e (cells in
// increasing index, as Eigen's setFromTriplets sums them), scaled by
// dt^2 + beta dt, plus the damped mass on the diagonal entries; the
// structural mask; and the stiffness force sum in the same cell order.
// The solids of a scene as the assembly sees them: each one's mass and its
// cell -> valid-cell ordinal map; the element matrices and forces of solid i
// start at valid cell keBase[i] of the concatenated arrays.
struct SolidSet {
  int n;
  const double* mass[ESF_MAX_SOLIDS];
  const int* ord[ESF_MAX_SOLIDS];
  long long keBase[ESF_MAX_SOLIDS];
};

// _systemMatrix from the triplets of every solid's
// computeStiffnessMatrixAndMaterialForce (DEFOR_SOLID_3D.cpp:697-871): a
// solid contributes between two nodes that both carry its mass; Eigen's
// setFromTriplets sums the duplicates in list order (solid 0's cells in
// index order, then solid 1's), and the force vector takes each solid's
// own sum (its local force) in turn.
__global__ void k_assemble(GridDev g, SolidSet ss, const int* sdof, const long long* sNode, long long S,
                           const double* Ke, const double* nf, double scale,
                           double* blocks, int* nbr, int* mask, double* force) {
  FOR_N(S * 27, t) {
    long long a = t / 27;
    int j = (int)(t % 27);
    long long n = sNode[a];
    int nx = (int)(n % g.X), ny = (int)((n / g.X) % g.Y), nz = (int)(n / g.slab);
    int dx = j % 3 - 1, dy = (j / 3) % 3 - 1, dz = j / 9 - 1;
    int mx = nx + dx, my = ny + dy, mz = nz + dz;
    double blk[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    bool present = false;
    int mdof = -1;
    if (mx >= 0 && mx < g.X && my >= 0 && my < g.Y && mz >= 0 && mz < g.Z) {
      long long m = nidx(g, mx, my, mz);
      mdof = sdof[m];
      for (int si = 0; si < ss.n && mdof >= 0; si++) {
        if (ss.mass[si][n] == 0 || ss.mass[si][m] == 0) continue;
        for (int ia = 7; ia >= 0; ia--) {  // cells containing n, increasing index
          int cx = nx - (ia & 1), cy = ny - ((ia >> 1) & 1), cz = nz - ((ia >> 2) & 1);
          if (cx < 0 || cy < 0 || cz < 0 || cx > g.X - 2 || cy > g.Y - 2 || cz > g.Z - 2) continue;
          int bx = mx - cx, by = my - cy, bz = mz - cz;
          if (bx < 0 || bx > 1 || by < 0 || by > 1 || bz < 0 || bz > 1) continue;
          int ord = ss.ord[si][cidx(g, cx, cy, cz)];
          if (ord < 0) continue;
          int ib = bx + 2 * by + 4 * bz;
          const double* K = Ke + 576LL * (ss.keBase[si] + ord);
          for (int r = 0; r < 3; r++)
            for (int q = 0; q < 3; q++) blk[r * 3 + q] += K[(ia * 3 + r) * 24 + ib * 3 + q];
          present = true;
        }
      }
    }
    for (int e = 0; e < 9; e++) blocks[blk_at(a, 9 * j + e)] = present ? blk[e] * scale : 0.0;
    if (j == 13) {
      present = true;  // coeffRef(i, i) creates the diagonal entries
      // force: per solid, cells containing n in increasing index, corner ia
      double f[3] = {0, 0, 0};
      for (int si = 0; si < ss.n; si++) {
        double fs[3] = {0, 0, 0};
        for (int ia = 7; ia >= 0; ia--) {
          int cx = nx - (ia & 1), cy = ny - ((ia >> 1) & 1), cz = nz - ((ia >> 2) & 1);
          if (cx < 0 || cy < 0 || cz < 0 || cx > g.X - 2 || cy > g.Y - 2 || cz > g.Z - 2) continue;
          int ord = ss.ord[si][cidx(g, cx, cy, cz)];
          if (ord < 0) continue;
          for (int r = 0; r < 3; r++) fs[r] += nf[24LL * (ss.keBase[si] + ord) + r * 8 + ia];
        }
        for (int r = 0; r < 3; r++) f[r] = si == 0 ? fs[r] : f[r] + fs[r];
      }
      for (int r = 0; r < 3; r++) force[3 * a + r] = f[r];
    }
    nbr[nbr_at(a, j)] = present ? mdof : -1;
    unsigned int bit = present ? (1u << j) : 0u;
    if (bit) atomicOr((unsigned int*)&mask[a], bit);
  }
}

// cell index -> position in the valid-cell list
__global__ void k_cell_ord_fill(GridDev g, const long long* cells, long long nc, int* ord) {
  FOR_N(nc, t) {
    long long n = cells[t];
    int x = (int)(n % g.X), y = (int)((n / g.X) % g.Y), z = (int)(n / g.slab);
    ord[cidx(g, x, y, z)] = (int)t;
  }
}
// _systemMatrix.coeffRef(i, i) += damped[i]; diagonal for the preconditioner
// (COUPLED_INTEGRATOR_3D.cpp:615-617, 663)
__global__ void k_add_diag(long long S, const double* damped, double* blocks, double* diag) {
  FOR_N(3 * S, i) {
    long long a = i / 3;
    int r = (int)(i % 3);
    double* e = blocks + blk_at(a, 13 * 9 + 4 * r);
    *e = *e + damped[i];
    diag[i] = *e;
  }
}

// DEFOR_SOLID_3D::computeMV (DEFOR_SOLID_3D.cpp:873-889) for one solid.
__global__ void k_compute_mv(GridDev g, SolidDev s, Box b, const int* sdof, double* mv,
                             double* energyPart) {
  double e = 0;
  FOR_BOX(b, x, y, z) {
    long long n = nidx(g, x, y, z);
    int a = sdof[n];
    if (a < 0) continue;
    const double* v = s.vel + 3 * n;
    for (int q = 0; q < 3; q++) mv[3 * a + q] += s.mass[n] * v[q];
    e += 0.5 * s.mass[n] * (v[0] * v[0] + (v[1] * v[1] + v[2] * v[2]));
  }
  __shared__ double sh[32];
  for (int o = 16; o > 0; o >>= 1) e += __shfl_down_sync(0xffffffffu, e, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = e;
  __syncthreads();
  if (threadIdx.x == 0) {
    double acc = 0;
    for (int w = 0; w < (int)blockDim.x / 32; w++) acc += sh[w];
    energyPart[blockIdx.x] += acc;
  }
}

// Vorticity (COUPLED_INTEGRATOR_3D.cpp:451-497).
__global__ void k_vorticity(GridDev g, const double* VF, const double* v, double* vort, double* ws) {
  FOR_N(g.T, n) {
    int x = (int)(n % g.X), y = (int)((n / g.X) % g.Y), z = (int)(n / g.slab);
    if (x < 1 || x > g.X - 2 || y < 1 || y > g.Y - 2 || z < 1 || z > g.Z - 2) continue;
    if (VF[n] >= 1) continue;
    const double gs = 0.5 / g.dh;
    long long up = (VF[n + g.X] >= 1 || y == g.Y - 2) ? n : n + g.X;
    long long down = (VF[n - g.X] >= 1 || y == 1) ? n : n - g.X;
    double ddy = (up == n || down == n) ? g.dhInv : gs;
    long long out = (VF[n + g.slab] >= 1 || z == g.Z - 2) ? n : n + g.slab;
    long long in = (VF[n - g.slab] >= 1 || z == 1) ? n : n - g.slab;
    double ddz = (out == n || in == n) ? g.dhInv : gs;
    long long right = (VF[n + 1] >= 1 || x == g.X - 2) ? n : n + 1;
    long long left = (VF[n - 1] >= 1 || x == 1) ? n : n - 1;
    double ddx = (right == n || left == n) ? g.dhInv : gs;
    double w0 = ((v[3 * up + 2] - v[3 * down + 2]) + (-v[3 * out + 1] + v[3 * in + 1])) * ddz;
    double w1 = ((v[3 * out + 0] - v[3 * in + 0]) + (-v[3 * right + 2] + v[3 * left + 2])) * ddx;
    double w2 = ((v[3 * right + 1] - v[3 * left + 1]) + (-v[3 * up + 0] + v[3 * down + 0])) * ddy;
    vort[3 * n] = w0;
    vort[3 * n + 1] = w1;
    vort[3 * n + 2] = w2;
    ws[n] = sqrt(w0 * w0 + (w1 * w1 + w2 * w2));
  }
}

struct BodyParams {
  double fluidDensity, gravity, buoyancy, damp, vortEps, dt;
};

// Body forces, masses and energy per interior node (COUPLED_INTEGRATOR_3D.cpp:503-606);
// also m^-1 per node (zero on the boundary) for the pressure operator.
__global__ void k_body_forces(GridDev g, BodyParams bp, const double* VF, const double* solidMass,
                              const double* v, const double* intensity, const double* vort,
                              const double* ws, const int* sdof, double* uf, double* mvf,
                              double* minv, double* damped, double* solidMv, double* solidF,
                              double* energyPart) {
  double e = 0;
  FOR_N(g.T, n) {
    int x = (int)(n % g.X), y = (int)((n / g.X) % g.Y), z = (int)(n / g.slab);
    if (x < 1 || x > g.X - 2 || y < 1 || y > g.Y - 2 || z < 1 || z > g.Z - 2) {
      minv[n] = 0.0;
      continue;
    }
    int a = sdof[n];
    double dh = g.dh;
    double fm = fmax_ref(1.0 - VF[n], 0.0) * bp.fluidDensity * dh * dh * dh;
    double mass = fm + solidMass[n];
    double h = dh * y + g.o[1];
    e += mass * bp.gravity * h;
    const double* vn = v + 3 * n;
    if (a < 0) {
      double mg = mass * bp.gravity;
      double f0 = 0.0 + mg * 0.0, f1 = 0.0 + mg * -1.0, f2 = 0.0 + mg * 0.0;
      f1 += bp.buoyancy * fm * intensity[n];
      if (bp.vortEps > 0) {
        if (VF[n + g.X] == 0 && VF[n - g.X] == 0 && VF[n + 1] == 0 && VF[n - 1] == 0 &&
            VF[n + g.slab] == 0 && VF[n - g.slab] == 0) {
          const double gs = 0.5 / g.dh;
          long long up = (y == g.Y - 2) ? n : n + g.X;
          long long down = (VF[n - g.X] >= 1 || y == 1) ? n : n - g.X;
          double ddy = (up == n || down == n) ? g.dhInv : gs;
          long long out = (VF[n + g.slab] >= 1 || z == g.Z - 2) ? n : n + g.slab;
          long long in = (VF[n - g.slab] >= 1 || z == 1) ? n : n - g.slab;
          double ddz = (out == n || in == n) ? g.dhInv : gs;
          long long right = (VF[n + 1] >= 1 || x == g.X - 2) ? n : n + 1;
          long long left = (VF[n - 1] >= 1 || x == 1) ? n : n - 1;
          double ddx = (right == n || left == n) ? g.dhInv : gs;
          double N0 = (ws[right] - ws[left]) * ddx;
          double N1 = (ws[up] - ws[down]) * ddy;
          double N2 = (ws[out] - ws[in]) * ddz;
          double mag = sqrt(N0 * N0 + N1 * N1 + N2 * N2);
          if (mag > 0.0f) {
            mag = 1.0 / mag;
            N0 *= mag;
            N1 *= mag;
            N2 *= mag;
            const double* w = vort + 3 * n;
            f0 += (N1 * w[2] - N2 * w[1]) * dh * bp.vortEps * fm;
            f1 -= (N0 * w[2] - N2 * w[0]) * dh * bp.vortEps * fm;
            f2 += (N0 * w[1] - N1 * w[0]) * dh * bp.vortEps * fm;
          }
        }
      }
      // _unitForce *= dt; += mv  (pcrImplicitSolve :669-670)
      uf[3 * n] = f0 * bp.dt + fm * vn[0];
      uf[3 * n + 1] = f1 * bp.dt + fm * vn[1];
      uf[3 * n + 2] = f2 * bp.dt + fm * vn[2];
      mvf[3 * n] = fm * vn[0];
      mvf[3 * n + 1] = fm * vn[1];
      mvf[3 * n + 2] = fm * vn[2];
    } else {
      double dm = solidMass[n] * bp.damp + fm;
      for (int q = 0; q < 3; q++) {
        damped[3 * a + q] = dm;
        solidMv[3 * a + q] += fm * vn[q];
      }
      double mg = mass * bp.gravity;
      solidF[3 * a] += mg * 0.0;
      solidF[3 * a + 1] += mg * -1.0;
      solidF[3 * a + 2] += mg * 0.0;
      solidF[3 * a + 1] += bp.buoyancy * fm * intensity[n];
      // _solidUnitForce *= dt; += _solidMv  (:664-665)
      for (int q = 0; q < 3; q++) solidF[3 * a + q] = solidF[3 * a + q] * bp.dt + solidMv[3 * a + q];
    }
    minv[n] = 1.0 / mass;
    e += 0.5 * fm * (vn[0] * vn[0] + (vn[1] * vn[1] + vn[2] * vn[2]));
  }
  __shared__ double sh[32];
  for (int o = 16; o > 0; o >>= 1) e += __shfl_down_sync(0xffffffffu, e, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = e;
  __syncthreads();
  if (threadIdx.x == 0) {
    double acc = 0;
    for (int w = 0; w < (int)blockDim.x / 32; w++) acc += sh[w];
    energyPart[blockIdx.x] = acc;
  }
}

// v* per interior node (pcrImplicitSolve :678-692): fluid (dt f + m v)/m,
// solid: the first solid solve.
__global__ void k_vstar(GridDev g, const int* sdof, const double* uf, const double* minv,
                        const double* solidV0, double* vstar) {
  FOR_N(g.T, n) {
    int x = (int)(n % g.X), y = (int)((n / g.X) % g.Y), z = (int)(n / g.slab);
    if (x < 1 || x > g.X - 2 || y < 1 || y > g.Y - 2 || z < 1 || z > g.Z - 2) {
      vstar[3 * n] = vstar[3 * n + 1] = vstar[3 * n + 2] = 0.0;
      continue;
    }
    int a = sdof[n];
    for (int q = 0; q < 3; q++) vstar[3 * n + q] = (a < 0) ? uf[3 * n + q] * minv[n] : solidV0[3 * a + q];
  }
}

// Per cell: rhs (computeDivergenceConstraintRHS :286-325), the Jacobi
// diagonal of J M^-1 J^T (:694-705) and b1 = J v* - rhs (:708-709).
__global__ void k_cell_rhs(GridDev g, const double* v, const double* vstar, const double* minv,
                           double* rhs, double* jdiag, double* b1) {
  FOR_N(g.R, c) {
    int x = (int)(c % g.cX), y = (int)((c / g.cX) % g.cY), z = (int)(c / g.cslab);
    double r = 0, jd = 0, jv = 0;
    for (int i = 0; i < 8; i++) {
      int nx = x + (i & 1), ny = y + ((i >> 1) & 1), nz = z + ((i >> 2) & 1);
      long long n = nidx(g, nx, ny, nz);
      bool dof = nx > 0 && nx < g.X - 1 && ny > 0 && ny < g.Y - 1 && nz > 0 && nz < g.Z - 1;
      double sg[3] = {sgnx(i), sgny(i), sgnz(i)};
      if (!dof) {
        r -= sg[0] * v[3 * n];
        r -= sg[1] * v[3 * n + 1];
        r -= sg[2] * v[3 * n + 2];
      } else {
        for (int q = 0; q < 3; q++) {
          jd += minv[n] * 1.0;
          jv += sg[q] * vstar[3 * n + q];
        }
      }
    }
    rhs[c] = r;
    jdiag[c] = jd;
    b1[c] = jv - r;
  }
}

// -J^T lambda per interior node (:719): cells in increasing index.
__device__ __forceinline__ void jt_lambda(const GridDev& g, const double* lam, int x, int y, int z,
                                          double* m) {
  m[0] = m[1] = m[2] = 0;
  for (int i = 7; i >= 0; i--) {
    int cx = x - (i & 1), cy = y - ((i >> 1) & 1), cz = z - ((i >> 2) & 1);
    double l = lam[cidx(g, cx, cy, cz)];
    m[0] += sgnx(i) * l;
    m[1] += sgny(i) * l;
    m[2] += sgnz(i) * l;
  }
}
// solid right-hand side of the second solid solve (:720-729)
__global__ void k_solid_b1(GridDev g, const long long* sNode, long long S, const double* lam,
                           double* sb1) {
  FOR_N(S, a) {
    long long n = sNode[a];
    int x = (int)(n % g.X), y = (int)((n / g.X) % g.Y), z = (int)(n / g.slab);
    double m[3];
    jt_lambda(g, lam, x, y, z, m);
    for (int q = 0; q < 3; q++) sb1[3 * a + q] = -m[q];
  }
}
// pressure correction and v = v* + dv into the grid velocity (:737-763)
__global__ void k_velocity_update(GridDev g, const int* sdof, const double* lam, const double* minv,
                                  const double* solidPC, const double* vstar, double* pc, double* v1,
                                  double* vel) {
  FOR_N(g.T, n) {
    int x = (int)(n % g.X), y = (int)((n / g.X) % g.Y), z = (int)(n / g.slab);
    if (x < 1 || x > g.X - 2 || y < 1 || y > g.Y - 2 || z < 1 || z > g.Z - 2) continue;
    int a = sdof[n];
    double m[3];
    if (a < 0) jt_lambda(g, lam, x, y, z, m);
    for (int q = 0; q < 3; q++) {
      double p = (a < 0) ? (-m[q]) * minv[n] : solidPC[3 * a + q];
      pc[3 * n + q] = p;
      double w = vstar[3 * n + q] + p;
      v1[3 * n + q] = w;
      vel[3 * n + q] = w;
    }
  }
}

// ------------------------------------------------ fluid advection (a14, a15)
__global__ void k_advect_velocity(GridDev g, const double* solidMass, const double* vel, double* out,
                                  double dt) {
  FOR_N(g.T, n) {
    int x = (int)(n % g.X), y = (int)((n / g.X) % g.Y), z = (int)(n / g.slab);
    if (x < 1 || x > g.X - 2 || y < 1 || y > g.Y - 2 || z < 1 || z > g.Z - 2) continue;
    if (solidMass[n] > 0) continue;
    double node[3] = {x * g.dh + g.o[0], y * g.dh + g.o[1], z * g.dh + g.o[2]};
    double p[3], v[3], np[3];
    for (int q = 0; q < 3; q++) p[q] = node[q] - 0.5 * vel[3 * n + q] * dt;
    interp3(vel, g.X, g.Y, g.Z, g.dh, g.o, p, v);
    for (int q = 0; q < 3; q++) np[q] = node[q] - v[q] * dt;
    double mass = interp1(solidMass, g.X, g.Y, g.Z, g.dh, g.o, np);
    double newdt = dt / 2;
    while (mass > 0 && newdt > dt / 16) {
      for (int q = 0; q < 3; q++) np[q] += v[q] * newdt;
      newdt /= 2;
      mass = interp1(solidMass, g.X, g.Y, g.Z, g.dh, g.o, np);
    }
    interp3(vel, g.X, g.Y, g.Z, g.dh, g.o, np, out + 3 * n);
  }
}
__global__ void k_advect_scalar(GridDev g, const double* solidMass, const double* vel,
                                const double* field, double* out, double dt) {
  FOR_N(g.T, n) {
    int x = (int)(n % g.X), y = (int)((n / g.X) % g.Y), z = (int)(n / g.slab);
    if (solidMass[n] > 0) {
      out[n] = 0.0;
      continue;
    }
    double node[3] = {x * g.dh + g.o[0], y * g.dh + g.o[1], z * g.dh + g.o[2]};
    double np[3];
    for (int q = 0; q < 3; q++) np[q] = node[q] - vel[3 * n + q] * dt;
    double mass = interp1(solidMass, g.X, g.Y, g.Z, g.dh, g.o, np);
    double newdt = dt / 2;
    while (mass > 0 && newdt > dt / 16) {
      for (int q = 0; q < 3; q++) np[q] += vel[3 * n + q] * newdt;
      newdt /= 2;
      mass = interp1(solidMass, g.X, g.Y, g.Z, g.dh, g.o, np);
    }
    out[n] = interp1(field, g.X, g.Y, g.Z, g.dh, g.o, np);
  }
}
// Dirichlet walls (:900-916)
__global__ void k_dirichlet(GridDev g, double* vel, double* intensity) {
  FOR_N(g.T, n) {
    int x = (int)(n % g.X), y = (int)((n / g.X) % g.Y), z = (int)(n / g.slab);
    bool face = x == 0 || x == g.X - 1 || y == 0 || y == g.Y - 1 || z == 0 || z == g.Z - 1;
    if (face) vel[3 * n] = vel[3 * n + 1] = vel[3 * n + 2] = 0.0;
    if (y == 0) intensity[n] = 0.0;
  }
}

}  // namespace esf

// ------------------------------------- matrix-free FP32 solid stiffness
// The solid DOF of each corner of each valid cell (-1: not a solid node),
// 8 planes of nc ints, for the matrix-free apply.
__global__ void k_mf_corners(GridDev g, const long long* cells, long long nc, const int* sdof, int* ci) {
  const long long off[8] = {0, 1, g.X, g.X + 1, g.slab, g.slab + 1, g.slab + g.X, g.slab + g.X + 1};
  FOR_N(nc, t) {
    const long long n = cells[t];
    for (int i = 0; i < 8; i++) ci[i * nc + t] = sdof[n + off[i]];
  }
}
