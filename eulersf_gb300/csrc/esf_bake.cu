// Offline mass baking on the GPU: the rest-pose mass grid of a solid from
// its closed triangle mesh, the job of the reference's rasterizeSolid tool
// (projects/rasterizeSolid/main.cpp:20-80). The grid is the mesh's bounding
// box grown by 10 cells on every side, `int` resolution (box extent / dh,
// truncated), node (x, y, z) at box_min + (x, y, z) * dh; a node carries the
// density where the signed distance to the surface is at most dh / 2.
//
// The reference evaluates the distance from a narrow-band DT-Grid SDF of the
// mesh (SPARSE_SDF::signedDist on the .svol file); here it is the exact
// distance to the triangles, signed by the generalised winding number
// (inside where the solid angle the surface subtends sums to 4 pi). The two
// agree away from the threshold; nodes whose distance lies within the SDF
// grid's interpolation error of dh / 2 can fall either side.
//
// One thread per node; the triangles are staged through shared memory in
// tiles, every thread testing every triangle (a closed mesh of a few thousand
// triangles and a 220^3 grid is ~2e10 point-triangle tests, tens of ms).
// Distances and solid angles are evaluated in FP32 relative to the node
// (coordinates of a few tenths, thresholds of 5e-4), the mass written in FP64.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <vector>

#include "esf_common.cuh"

namespace esf {
namespace {

constexpr int BT = 256;        // threads per block
constexpr int TILE = 256;      // triangles per shared-memory tile

// Squared distance from p to triangle (a, b, c), by the region of the
// triangle's plane the closest point falls in (vertex, edge or face
// region; the standard Voronoi-region construction of the closest point).
__device__ float tri_dist2(const float3 p, const float3 a, const float3 b, const float3 c) {
  const float3 ab = make_float3(b.x - a.x, b.y - a.y, b.z - a.z);
  const float3 ac = make_float3(c.x - a.x, c.y - a.y, c.z - a.z);
  const float3 ap = make_float3(p.x - a.x, p.y - a.y, p.z - a.z);
  auto dot = [](float3 u, float3 v) { return u.x * v.x + u.y * v.y + u.z * v.z; };
  auto d2 = [](float3 u) { return u.x * u.x + u.y * u.y + u.z * u.z; };
  const float d1 = dot(ab, ap), d2v = dot(ac, ap);
  if (d1 <= 0.0f && d2v <= 0.0f) return d2(ap);  // vertex a
  const float3 bp = make_float3(p.x - b.x, p.y - b.y, p.z - b.z);
  const float d3 = dot(ab, bp), d4 = dot(ac, bp);
  if (d3 >= 0.0f && d4 <= d3) return d2(bp);  // vertex b
  const float vc = d1 * d4 - d3 * d2v;
  if (vc <= 0.0f && d1 >= 0.0f && d3 <= 0.0f) {  // edge ab
    const float t = d1 / (d1 - d3);
    return d2(make_float3(ap.x - t * ab.x, ap.y - t * ab.y, ap.z - t * ab.z));
  }
  const float3 cp = make_float3(p.x - c.x, p.y - c.y, p.z - c.z);
  const float d5 = dot(ab, cp), d6 = dot(ac, cp);
  if (d6 >= 0.0f && d5 <= d6) return d2(cp);  // vertex c
  const float vb = d5 * d2v - d1 * d6;
  if (vb <= 0.0f && d2v >= 0.0f && d6 <= 0.0f) {  // edge ac
    const float t = d2v / (d2v - d6);
    return d2(make_float3(ap.x - t * ac.x, ap.y - t * ac.y, ap.z - t * ac.z));
  }
  const float va = d3 * d6 - d5 * d4;
  if (va <= 0.0f && (d4 - d3) >= 0.0f && (d5 - d6) >= 0.0f) {  // edge bc
    const float t = (d4 - d3) / ((d4 - d3) + (d5 - d6));
    const float3 bc = make_float3(c.x - b.x, c.y - b.y, c.z - b.z);
    return d2(make_float3(bp.x - t * bc.x, bp.y - t * bc.y, bp.z - t * bc.z));
  }
  // face: p minus its projection onto the plane
  const float denom = 1.0f / (va + vb + vc);
  const float v = vb * denom, w = vc * denom;
  return d2(make_float3(ap.x - ab.x * v - ac.x * w, ap.y - ab.y * v - ac.y * w,
                        ap.z - ab.z * v - ac.z * w));
}

// Signed solid angle of triangle (a, b, c) seen from p (Van Oosterom and
// Strackee's formula, tan(Omega / 2) = det / (|a||b||c| + ...)): the
// winding number is the sum over a closed surface / 4 pi.
__device__ float tri_solid_angle(const float3 p, const float3 a, const float3 b, const float3 c) {
  const float3 x = make_float3(a.x - p.x, a.y - p.y, a.z - p.z);
  const float3 y = make_float3(b.x - p.x, b.y - p.y, b.z - p.z);
  const float3 z = make_float3(c.x - p.x, c.y - p.y, c.z - p.z);
  const float lx = sqrtf(x.x * x.x + x.y * x.y + x.z * x.z);
  const float ly = sqrtf(y.x * y.x + y.y * y.y + y.z * y.z);
  const float lz = sqrtf(z.x * z.x + z.y * z.y + z.z * z.z);
  const float det = x.x * (y.y * z.z - y.z * z.y) - x.y * (y.x * z.z - y.z * z.x) + x.z * (y.x * z.y - y.y * z.x);
  const float dxy = x.x * y.x + x.y * y.y + x.z * y.z;
  const float dyz = y.x * z.x + y.y * z.y + y.z * z.z;
  const float dzx = z.x * x.x + z.y * x.y + z.z * x.z;
  const float den = lx * ly * lz + dxy * lz + dyz * lx + dzx * ly;
  return 2.0f * atan2f(det, den);
}

__global__ void k_bake_mass(int X, int Y, int Z, double dh, double ox, double oy, double oz,
                            const float* __restrict__ tri, int ntri, double rx, double ry, double rz,
                            double density,
                            double* __restrict__ mass, unsigned long long* __restrict__ count) {
  __shared__ float st[TILE * 9];
  const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long total = (long long)X * Y * Z;
  const bool live = n < total;
  const int x = live ? (int)(n % X) : 0, y = live ? (int)((n / X) % Y) : 0;
  const int z = live ? (int)(n / ((long long)X * Y)) : 0;
  // node position (the reference's pos = (x, y, z) dh + box_min, in FP64),
  // then relative to the mesh's reference point in FP32
  const float3 p = make_float3((float)(x * dh + ox - rx), (float)(y * dh + oy - ry),
                               (float)(z * dh + oz - rz));
  float best = 3.4e38f, angle = 0.0f;
  for (int t0 = 0; t0 < ntri; t0 += TILE) {
    const int nt = min(TILE, ntri - t0);
    __syncthreads();
    for (int i = threadIdx.x; i < nt * 9; i += blockDim.x) st[i] = tri[(long long)t0 * 9 + i];
    __syncthreads();
    for (int k = 0; k < nt; k++) {
      const float* q = st + 9 * k;
      const float3 a = make_float3(q[0], q[1], q[2]), b = make_float3(q[3], q[4], q[5]),
                   c = make_float3(q[6], q[7], q[8]);
      best = fminf(best, tri_dist2(p, a, b, c));
      angle += tri_solid_angle(p, a, b, c);
    }
  }
  if (!live) return;
  // winding number angle / 4 pi: ~1 inside a closed outward-oriented mesh,
  // ~0 outside
  const bool inside = fabsf(angle) > 6.2831853f;
  const float sd = inside ? -sqrtf(best) : sqrtf(best);
  const bool solid = sd <= (float)(0.5 * dh);
  mass[n] = solid ? density : 0.0;
  if (solid) atomicAdd(count, 1ull);
}

}  // namespace
}  // namespace esf

using namespace esf;

extern "C" esf_status esf_rasterize_solid(const double* vertices, int num_vertices, const int* triangles,
                                          int num_triangles, double mass_dh, double density, int res[3],
                                          double origin[3], double* mass, size_t capacity,
                                          double* total_mass) {
  if (!vertices || num_vertices < 3 || !triangles || num_triangles < 1 || !(mass_dh > 0) || !res ||
      !origin) {
    set_error("esf_rasterize_solid: invalid argument");
    return ESF_ERR_INVALID_ARG;
  }
  // OBJ::BoundingBox, grown by 10 cells (rasterizeSolid/main.cpp:44-53)
  double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
  for (int v = 0; v < num_vertices; v++)
    for (int k = 0; k < 3; k++) {
      lo[k] = vertices[3 * v + k] < lo[k] ? vertices[3 * v + k] : lo[k];
      hi[k] = vertices[3 * v + k] > hi[k] ? vertices[3 * v + k] : hi[k];
    }
  for (int k = 0; k < 3; k++) {
    lo[k] -= mass_dh * 10;
    hi[k] += mass_dh * 10;
    res[k] = (int)((hi[k] - lo[k]) / mass_dh);
    origin[k] = lo[k];
  }
  const long long total = (long long)res[0] * res[1] * res[2];
  if (!mass) return ESF_OK;  // size query
  if (capacity < (size_t)total) {
    set_error("esf_rasterize_solid: the grid has %lld nodes, the buffer holds %zu", total, capacity);
    return ESF_ERR_INVALID_ARG;
  }
  for (int t = 0; t < 3 * num_triangles; t++)
    if (triangles[t] < 0 || triangles[t] >= num_vertices) {
      set_error("esf_rasterize_solid: triangle %d names vertex %d of %d", t / 3, triangles[t], num_vertices);
      return ESF_ERR_INVALID_ARG;
    }
  // triangles as FP32 corner coordinates relative to the box centre
  float ref[3];
  for (int k = 0; k < 3; k++) ref[k] = (float)(0.5 * (lo[k] + hi[k]));
  std::vector<float> tri((size_t)num_triangles * 9);
  for (int t = 0; t < num_triangles; t++)
    for (int c = 0; c < 3; c++)
      for (int k = 0; k < 3; k++)
        tri[9 * t + 3 * c + k] = (float)(vertices[3 * triangles[3 * t + c] + k] - (double)ref[k]);
  float* dTri = nullptr;
  double* dMass = nullptr;
  unsigned long long* dCount = nullptr;
  esf_status e = ESF_OK;
  if (cudaMalloc(&dTri, tri.size() * 4) != cudaSuccess || cudaMalloc(&dMass, total * 8) != cudaSuccess ||
      cudaMalloc(&dCount, 8) != cudaSuccess) {
    set_error("esf_rasterize_solid: device allocation failed");
    e = ESF_ERR_OOM;
  }
  if (!e && (cudaMemcpy(dTri, tri.data(), tri.size() * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
             cudaMemset(dCount, 0, 8) != cudaSuccess))
    e = ESF_ERR_CUDA;
  if (!e) {
    const int blocks = (int)((total + BT - 1) / BT);
    ESF_COUNTED k_bake_mass<<<blocks, BT>>>(res[0], res[1], res[2], mass_dh, origin[0], origin[1], origin[2],
                                            dTri, num_triangles, (double)ref[0], (double)ref[1],
                                            (double)ref[2], density, dMass, dCount);
    if (cudaGetLastError() != cudaSuccess) e = ESF_ERR_CUDA;
  }
  unsigned long long cnt = 0;
  if (!e && (cudaMemcpy(mass, dMass, total * 8, cudaMemcpyDeviceToHost) != cudaSuccess ||
             cudaMemcpy(&cnt, dCount, 8, cudaMemcpyDeviceToHost) != cudaSuccess))
    e = ESF_ERR_CUDA;
  if (e == ESF_ERR_CUDA) set_error("esf_rasterize_solid: %s", cudaGetErrorString(cudaGetLastError()));
  cudaFree(dTri);
  cudaFree(dMass);
  cudaFree(dCount);
  if (!e && total_mass) *total_mass = (double)cnt * density * mass_dh * mass_dh * mass_dh;
  return e;
}
