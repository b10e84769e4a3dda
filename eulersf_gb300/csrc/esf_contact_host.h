// Host declarations of the rest-SDF reader and triangle hash (esf_contact.cu).
#pragma once
#include <vector>

#include "../../include/eulersf.h"

namespace esf {

// The DT-Grid narrow band of a ".svol" file on a dense lattice over its
// bounding box plus one point of margin: index (x, y, z) at
// (x - lo[0]) + (y - lo[1]) n[0] + (z - lo[2]) n[0] n[1].
struct SvolLattice {
  int lo[3] = {0, 0, 0}, n[3] = {0, 0, 0};
  double dx = 0, t[3] = {0, 0, 0};
  double inC = 0, outC = 0;     // insideConstant, outsideConstant
  std::vector<float> val;       // band value (0 elsewhere)
  std::vector<signed char> code;  // 1 band, -1 inside constant, 0 outside constant
};

esf_status svol_read(const char* path, SvolLattice* L);
// lattice coordinates of a rest-space point (DTGrid worldToGrid)
void svol_to_grid(const SvolLattice& L, const double* p, double* g);
// per lattice point, the triangles whose rest bounding box covers it, in
// triangle order: CSR offsets (points + 1) and ids; false when the lists
// would hold 2^31 entries or more
bool svol_hash_triangles(const SvolLattice& L, const double* rest, int ntri, const int* tris,
                         std::vector<int>* off, std::vector<int>* ids);

}  // namespace esf
