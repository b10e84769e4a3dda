// Solid-solid contact of the particle update (DEFOR_SOLID_3D.cpp:953-995).
//
// A particle of solid A that comes within `contact safe distance` of solid B
// is pushed out along B's surface normal. B's side of the test is its
// rest-pose signed distance: the particle's position is taken to B's rest
// space through B's material coordinates X, and the rest SDF tells how deep
// it is and which surface point is closest (SPARSE_SDF, src/dtgrid/
// SPARSE_SDF.cpp:98-157, over the DT-Grid narrow band of a ".svol" file).
//
// The narrow band is held as a dense lattice over its bounding box (one
// point of margin): a float per point where the band stores a value, and a
// code that says which constant stands in elsewhere. That is the value the
// DT-Grid's random access returns for every lattice point of a closed level
// set (DTGrid_Impl.h operator()(x,y,z): the band value; the inside constant
// in a gap between two z-runs whose next run starts inside; the outside
// constant everywhere else). The lattice also carries, per band point, the
// surface triangles whose rest bounding box (grown by one lattice cell)
// covers it, in increasing triangle order (SPARSE_SDF::initHashSurface,
// :37-75), so the triangle under a surface point is found without a BVH.
//
// Arithmetic follows the reference's operation order with no fused
// multiply-adds (the file is compiled with -fmad=false and the transforms
// use explicit rounding): the contact decision is a threshold test, and a
// different rounding can flip it for a particle at the threshold.
#pragma once
#include "esf_common.cuh"

struct RestSdfDev {
  const float* val;          // band value per lattice point (0 elsewhere)
  const signed char* code;   // 1 band, -1 inside constant, 0 outside constant
  const int* triOff;         // per lattice point: first entry in triIds (points + 1 entries)
  const int* triIds;         // triangles hashed at each lattice point
  int lo[3], n[3];           // lattice index range [lo, lo + n) per axis
  long long nxy;             // n[0] * n[1]
  double inv;                // 1 / dx
  double off[3];             // -translation * inv
  double dx;
  double inC, outC;          // insideConstant, outsideConstant
  const double* rest;        // rest vertex positions, 3 per vertex
  const double* cur;         // current vertex positions, 3 per vertex
  const int* tris;           // 3 vertex indices per triangle
};

// DTGrid worldToGrid (scale(1/dx) * rotation^T * translation(-t), with no
// rotation): g = p * (1/dx) + (-t * (1/dx)), evaluated as Matrix4x4 *
// Vector4(p, 1) does.
__device__ __forceinline__ void sdf_to_grid(const RestSdfDev& s, const double* p, double* g) {
#pragma unroll
  for (int k = 0; k < 3; k++) g[k] = __dadd_rn(__dmul_rn(p[k], s.inv), s.off[k]);
}

__device__ __forceinline__ long long sdf_point(const RestSdfDev& s, int x, int y, int z) {
  const int i = x - s.lo[0], j = y - s.lo[1], k = z - s.lo[2];
  if (i < 0 || j < 0 || k < 0 || i >= s.n[0] || j >= s.n[1] || k >= s.n[2]) return -1;
  return i + (long long)j * s.n[0] + (long long)k * s.nxy;
}

// DTGrid::operator()(x, y, z): the value at a lattice point
__device__ __forceinline__ double sdf_value(const RestSdfDev& s, int x, int y, int z) {
  const long long q = sdf_point(s, x, y, z);
  if (q < 0) return s.outC;
  const signed char c = s.code[q];
  return c > 0 ? (double)s.val[q] : (c < 0 ? s.inC : s.outC);
}

// DTGrid::operator()(Vector3): trilinear interpolation of the 8 lattice
// values around p (TrilinearInterpolator::interp, its term order)
__device__ inline double sdf_trilinear(const RestSdfDev& s, const double* p) {
  double g[3];
  sdf_to_grid(s, p, g);
  const double fx = floor(g[0]), fy = floor(g[1]), fz = floor(g[2]);
  const int x = (int)fx, y = (int)fy, z = (int)fz;
  const double u = __dsub_rn(g[0], fx), v = __dsub_rn(g[1], fy), w = __dsub_rn(g[2], fz);
  const double v0 = sdf_value(s, x, y, z), v1 = sdf_value(s, x, y, z + 1);
  const double v2 = sdf_value(s, x, y + 1, z), v3 = sdf_value(s, x, y + 1, z + 1);
  const double v4 = sdf_value(s, x + 1, y, z), v5 = sdf_value(s, x + 1, y, z + 1);
  const double v6 = sdf_value(s, x + 1, y + 1, z), v7 = sdf_value(s, x + 1, y + 1, z + 1);
  const double iu = 1.0 - u, iv = 1.0 - v, iw = 1.0 - w;
  double r = __dmul_rn(__dmul_rn(__dmul_rn(v0, iu), iv), iw);
  r = __dadd_rn(r, __dmul_rn(__dmul_rn(__dmul_rn(v4, u), iv), iw));
  r = __dadd_rn(r, __dmul_rn(__dmul_rn(__dmul_rn(v2, iu), v), iw));
  r = __dadd_rn(r, __dmul_rn(__dmul_rn(__dmul_rn(v1, iu), iv), w));
  r = __dadd_rn(r, __dmul_rn(__dmul_rn(__dmul_rn(v5, u), iv), w));
  r = __dadd_rn(r, __dmul_rn(__dmul_rn(__dmul_rn(v3, iu), v), w));
  r = __dadd_rn(r, __dmul_rn(__dmul_rn(__dmul_rn(v6, u), v), iw));
  r = __dadd_rn(r, __dmul_rn(__dmul_rn(__dmul_rn(v7, u), v), w));
  return r;
}

// Vector3::normalize: divide by the length unless it is zero
__device__ __forceinline__ void sdf_normalize(double* n) {
  const double len = sqrt(__dadd_rn(__dadd_rn(__dmul_rn(n[0], n[0]), __dmul_rn(n[1], n[1])), __dmul_rn(n[2], n[2])));
  if (len != 0) {
    n[0] /= len;
    n[1] /= len;
    n[2] /= len;
  }
}

// DTGrid::lookupDistanceAndNormalFast (DTGrid_Impl.h): the lattice point
// nearest p (round half away from zero); in the band its value and the
// normalised central-difference gradient (closestPoint, computeGradient),
// else the inside or outside constant and no normal. Returns in-band.
__device__ inline bool sdf_lookup_fast(const RestSdfDev& s, const double* p, double* dist, double* n) {
  double g[3];
  sdf_to_grid(s, p, g);
  const int x = (int)round(g[0]), y = (int)round(g[1]), z = (int)round(g[2]);
  const long long q = sdf_point(s, x, y, z);
  const signed char c = q < 0 ? 0 : s.code[q];
  if (c <= 0) {
    *dist = c < 0 ? s.inC : s.outC;
    return false;
  }
  *dist = (double)s.val[q];
  const double h = 2 * s.dx;
  n[0] = (sdf_value(s, x + 1, y, z) - sdf_value(s, x - 1, y, z)) / h;
  n[1] = (sdf_value(s, x, y + 1, z) - sdf_value(s, x, y - 1, z)) / h;
  n[2] = (sdf_value(s, x, y, z + 1) - sdf_value(s, x, y, z - 1)) / h;
  sdf_normalize(n);
  return true;
}

// SPARSE_SDF::nearestSurfacePoint (SPARSE_SDF.cpp:119-145): from the fast
// lookup, walk along the (fixed) normal by the interpolated distance until
// it is below 1e-9 or 100 steps; returns the distance, surf the point.
__device__ inline double sdf_nearest_surface(const RestSdfDev& s, const double* p, double safe, double* surf) {
  double sdf, n[3] = {0.0, 0.0, 0.0};
  sdf_lookup_fast(s, p, &sdf, n);
  surf[0] = p[0];
  surf[1] = p[1];
  surf[2] = p[2];
  if (sdf >= safe) return sdf;
  const bool moves = n[0] != 0 || n[1] != 0 || n[2] != 0;
  for (int it = 0; fabs(sdf) > 1e-9 && it < 100; it++) {
#pragma unroll
    for (int k = 0; k < 3; k++) surf[k] = __dadd_rn(surf[k], __dmul_rn(-sdf, n[k]));
    const double next = sdf_trilinear(s, surf);
    if (!moves) {  // a zero normal leaves the point, and so the value, where it is
      sdf = next;
      break;
    }
    sdf = next;
  }
  return sdf;
}

__device__ __forceinline__ void sdf_cross(const double* a, const double* b, double* r) {
  r[0] = __dsub_rn(__dmul_rn(a[1], b[2]), __dmul_rn(a[2], b[1]));
  r[1] = __dsub_rn(__dmul_rn(a[2], b[0]), __dmul_rn(a[0], b[2]));
  r[2] = __dsub_rn(__dmul_rn(a[0], b[1]), __dmul_rn(a[1], b[0]));
}
__device__ __forceinline__ double sdf_dot(const double* a, const double* b) {
  return __dadd_rn(__dadd_rn(__dmul_rn(a[0], b[0]), __dmul_rn(a[1], b[1])), __dmul_rn(a[2], b[2]));
}

// TRIANGLE::baryCenter(point, lambda, rest = true) (TRIANGLE.cpp:109-136):
// the three sub-triangle normals agree in direction with the triangle's and
// the sub-areas sum to the area within 10%.
__device__ inline bool sdf_bary_rest(const RestSdfDev& s, int t, const double* p) {
  const double* a = s.rest + 3 * (long long)s.tris[3 * t];
  const double* b = s.rest + 3 * (long long)s.tris[3 * t + 1];
  const double* c = s.rest + 3 * (long long)s.tris[3 * t + 2];
  double ba[3], ca[3], bp[3], cp[3], pa[3];
#pragma unroll
  for (int k = 0; k < 3; k++) {
    ba[k] = b[k] - a[k];
    ca[k] = c[k] - a[k];
    bp[k] = b[k] - p[k];
    cp[k] = c[k] - p[k];
    pa[k] = p[k] - a[k];
  }
  double A[3], Aa[3], Ab[3], Ac[3];
  sdf_cross(ba, ca, A);
  sdf_cross(bp, cp, Aa);
  sdf_cross(pa, ca, Ab);
  sdf_cross(ba, pa, Ac);
  if (sdf_dot(Aa, A) < 0 || sdf_dot(Ab, A) < 0 || sdf_dot(Ac, A) < 0) return false;
  const double nA = sqrt(sdf_dot(A, A)), na = sqrt(sdf_dot(Aa, Aa)), nb = sqrt(sdf_dot(Ab, Ab)),
               nc = sqrt(sdf_dot(Ac, Ac));
  const double length = __dadd_rn(__dadd_rn(na / nA, nb / nA), nc / nA);
  return fabs(length - 1) <= 0.1;
}

// TRIANGLE::normal (TRIANGLE.h:51-55): unit normal of the current triangle
__device__ inline void sdf_current_normal(const RestSdfDev& s, int t, double* n) {
  const double* a = s.cur + 3 * (long long)s.tris[3 * t];
  const double* b = s.cur + 3 * (long long)s.tris[3 * t + 1];
  const double* c = s.cur + 3 * (long long)s.tris[3 * t + 2];
  double ba[3], ca[3];
#pragma unroll
  for (int k = 0; k < 3; k++) {
    ba[k] = b[k] - a[k];
    ca[k] = c[k] - a[k];
  }
  sdf_cross(ba, ca, n);
  const double z = sdf_dot(n, n);
  if (z > 0) {
    const double len = sqrt(z);
    n[0] /= len;
    n[1] /= len;
    n[2] /= len;
  }
}

// SPARSE_SDF::signedDistAndCurrentNormal (SPARSE_SDF.cpp:98-117): the
// distance of rest point p and the current normal of the triangle under its
// nearest surface point; 1 when p is farther than safe or no hashed
// triangle contains that point.
__device__ inline double sdf_contact(const RestSdfDev& s, const double* p, double safe, double* normal) {
  double surf[3];
  const double sd = sdf_nearest_surface(s, p, safe, surf);
  if (sd > safe) return 1;
  double g[3];
  sdf_to_grid(s, surf, g);  // SPARSE_SDF::trianglesAt: DTGrid::getLocator(pos) floors
  const long long q = sdf_point(s, (int)floor(g[0]), (int)floor(g[1]), (int)floor(g[2]));
  if (q < 0 || s.code[q] <= 0) return 1;
  for (int e = s.triOff[q]; e < s.triOff[q + 1]; e++) {
    const int t = s.triIds[e];
    if (sdf_bary_rest(s, t, surf)) {
      sdf_current_normal(s, t, normal);
      return sd;
    }
  }
  return 1;
}

// The other solids a particle can touch, for k_grid_to_particle.
struct ContactNeighbor {
  const double* phi;  // level set (DEFOR_SOLID_3D::_phi)
  const double* X;    // material coordinates
  const double* vel;  // grid velocity
  RestSdfDev sdf;
};
struct ContactSet {
  int n;
  double thickness;  // "contact safe distance"
  unsigned long long* contacts;  // particles that took a solid-solid impulse
  ContactNeighbor nb[ESF_MAX_SOLIDS - 1];
};
