// Host side of solid-solid contact: the rest SDF of a solid from its ".svol"
// file (SPARSE_SDF::load -> DTGrid::loadSparseVolume, the "DTG v1.0" format
// of SvolLoader_DTTop1.0.h) turned into the dense lattice the device reads,
// and the per-lattice-point triangle lists of SPARSE_SDF::initHashSurface
// (SPARSE_SDF.cpp:37-75).
//
// The file holds a DT-Grid: runs of x; per x the runs of y; per (x, y) the
// runs of z; then the band values in (x, y, z) order, z fastest. Text lines
// give the index, integer and real sizes, the endianness and, after the
// topology, the constants dx, gamma, beta, insideConstant, outsideConstant.
// The run-start offsets ("aa" arrays) are not stored; they are the running
// sums of the run lengths (SvolLoaderDTTop1::buildAAData).
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <fstream>
#include <string>
#include <vector>

#include "esf_common.cuh"
#include "esf_contact_host.h"

namespace esf {
namespace {

bool host_little_endian() {
  const uint16_t w = 1;
  unsigned char b;
  memcpy(&b, &w, 1);
  return b == 1;
}

// n integers of `size` bytes (1, 2, 4 or 8), signed, byte-swapped if asked
bool read_ints(std::istream& is, int size, bool swap, long long* out, size_t n) {
  if (size != 1 && size != 2 && size != 4 && size != 8) return false;
  unsigned char b[8];
  for (size_t i = 0; i < n; i++) {
    if (!is.read(reinterpret_cast<char*>(b), size)) return false;
    if (swap)
      for (int l = 0, r = size - 1; l < r; l++, r--) {
        unsigned char t = b[l];
        b[l] = b[r];
        b[r] = t;
      }
    if (size == 1) {
      int8_t v;
      memcpy(&v, b, 1);
      out[i] = v;
    } else if (size == 2) {
      int16_t v;
      memcpy(&v, b, 2);
      out[i] = v;
    } else if (size == 4) {
      int32_t v;
      memcpy(&v, b, 4);
      out[i] = v;
    } else {
      int64_t v;
      memcpy(&v, b, 8);
      out[i] = v;
    }
  }
  return true;
}

// the counts and offsets are unsigned ints in the file
bool read_uints(std::istream& is, int size, bool swap, long long* out, size_t n) {
  if (!read_ints(is, size, swap, out, n)) return false;
  if (size == 4)
    for (size_t i = 0; i < n; i++) out[i] &= 0xffffffffLL;
  return true;
}

bool read_reals(std::istream& is, int size, bool swap, double* out, size_t n) {
  if (size != 4 && size != 8) return false;
  unsigned char b[8];
  for (size_t i = 0; i < n; i++) {
    if (!is.read(reinterpret_cast<char*>(b), size)) return false;
    if (swap)
      for (int l = 0, r = size - 1; l < r; l++, r--) {
        unsigned char t = b[l];
        b[l] = b[r];
        b[r] = t;
      }
    if (size == 4) {
      float f;
      memcpy(&f, b, 4);
      out[i] = f;
    } else {
      memcpy(&out[i], b, 8);
    }
  }
  return true;
}

bool swap_for(const std::string& endian) {
  return (endian == "LittleEndian") != host_little_endian();
}

// bytes left in the stream (a malformed count must not size an allocation
// beyond the file)
long long remaining(std::istream& is) {
  const std::streampos here = is.tellg();
  if (here < 0) return 0;
  is.seekg(0, std::ios_base::end);
  const std::streampos end = is.tellg();
  is.seekg(here);
  return end < here ? 0 : (long long)(end - here);
}

// running run-length sums: aa[j] = values before run j
std::vector<long long> build_aa(const std::vector<long long>& idx) {
  std::vector<long long> aa(idx.size() / 2 + 1);
  long long count = 0;
  for (size_t i = 0, j = 0; i + 1 < idx.size(); i += 2, j++) {
    aa[j] = count;
    count += idx[i + 1] - idx[i] + 1;
  }
  aa[idx.size() / 2] = count;
  return aa;
}

}  // namespace

esf_status svol_read(const char* path, SvolLattice* L) {
  std::ifstream is(path, std::ios_base::binary);
  if (!is) {
    set_error("svol_read: cannot open %s", path);
    return ESF_ERR_IO;
  }
  char header[11] = {0};
  is.read(header, 10);
  if (!is || strcmp(header, "DTG v1.0  ") != 0) {
    set_error("svol_read: %s: unknown header format", path);
    return ESF_ERR_IO;
  }
  // topology header: the same sequence of line and word reads as the loader
  std::string line, word, endian;
  int indexSize = 0, intSize = 0, realSize = 0;
  std::getline(is, line);
  is >> word >> indexSize;
  std::getline(is, line);
  std::getline(is, line);
  is >> word >> intSize;
  std::getline(is, line);
  std::getline(is, line);
  is >> word >> realSize;
  std::getline(is, line);
  is >> word >> endian;
  std::getline(is, line);
  if (!is) {
    set_error("svol_read: %s: truncated header", path);
    return ESF_ERR_IO;
  }
  const bool swap = swap_for(endian);
  long long bbox[6];
  double tr[3], rot[3];
  bool ok = read_ints(is, indexSize, swap, bbox, 6) && read_reals(is, realSize, swap, tr, 3) &&
            read_reals(is, realSize, swap, rot, 3);
  std::vector<long long> idx[3], va[3];
  long long numVa3D = 0;
  for (int lev = 0; lev < 3 && ok; lev++) {
    long long num = 0;
    ok = read_uints(is, intSize, swap, &num, 1) && num >= 0 && num < (1LL << 31) && num % 2 == 0 &&
         num * indexSize <= remaining(is);
    if (!ok) break;
    idx[lev].resize((size_t)num);
    ok = read_ints(is, indexSize, swap, idx[lev].data(), (size_t)num);
    long long nva = 0;
    ok = ok && read_uints(is, intSize, swap, &nva, 1) && nva >= 0 && nva < (1LL << 31) &&
         (lev == 2 || nva * intSize <= remaining(is));
    if (!ok) break;
    if (lev < 2) {
      va[lev].resize((size_t)nva);
      ok = read_uints(is, intSize, swap, va[lev].data(), (size_t)nva);
    } else {
      numVa3D = nva;
    }
  }
  if (!ok) {
    set_error("svol_read: %s: truncated or malformed topology", path);
    return ESF_ERR_IO;
  }
  // auxiliary field header, then the constants and the values
  std::getline(is, line);
  if (line != "Auxiliary Fields v1.0") {
    set_error("svol_read: %s: unknown auxiliary fields format: %s", path, line.c_str());
    return ESF_ERR_IO;
  }
  int nfields = 0, dataSize = 0, nconst = 0;
  is >> word >> nfields;
  std::getline(is, line);
  std::getline(is, line);
  std::getline(is, line);
  if (line != "DataTextDescription SignedDistanceField") {
    set_error("svol_read: %s: the first field is not a signed distance field", path);
    return ESF_ERR_IO;
  }
  std::string endian2;
  is >> word >> endian2;
  std::getline(is, line);
  std::getline(is, line);
  is >> word >> dataSize;
  std::getline(is, line);
  std::getline(is, line);
  is >> word >> nconst;
  double dx = 0, inC = 0, outC = 0;
  for (int j = 0; j < nconst && is; j++) {
    std::string name;
    is >> word >> name;
    double v = 0;
    if (name == "dx" || name == "gamma" || name == "beta" || name == "insideConstant" ||
        name == "outsideConstant")
      is >> v;
    if (name == "dx") dx = v;
    if (name == "insideConstant") inC = v;
    if (name == "outsideConstant") outC = v;
    std::getline(is, line);
  }
  if (!is || (dataSize != 4 && dataSize != 8) || numVa3D * dataSize > remaining(is)) {
    set_error("svol_read: %s: truncated values", path);
    return ESF_ERR_IO;
  }
  std::vector<double> values((size_t)numVa3D);
  if (!is || !read_reals(is, dataSize, swap_for(endian2), values.data(), values.size()) || !(dx > 0)) {
    set_error("svol_read: %s: truncated values or no dx", path);
    return ESF_ERR_IO;
  }
  if (rot[0] != 0 || rot[1] != 0 || rot[2] != 0) {
    set_error("svol_read: %s: rotated sparse volumes are not supported", path);
    return ESF_ERR_UNSUPPORTED;
  }
  // structure checks: every offset the decode follows stays in its array
  const std::vector<long long> aa0 = build_aa(idx[0]), aa1 = build_aa(idx[1]), aa2 = build_aa(idx[2]);
  if ((long long)va[0].size() != aa0.back() || (long long)va[1].size() != aa1.back() || numVa3D != aa2.back()) {
    set_error("svol_read: %s: run lengths do not match the value counts", path);
    return ESF_ERR_IO;
  }
  if (idx[0].empty()) {
    set_error("svol_read: %s: empty narrow band", path);
    return ESF_ERR_IO;
  }
  auto in_range = [](const std::vector<long long>& v) {
    for (size_t i = 0; i + 1 < v.size(); i += 2)
      if (v[i + 1] < v[i]) return false;
    return true;
  };
  if (!in_range(idx[0]) || !in_range(idx[1]) || !in_range(idx[2])) {
    set_error("svol_read: %s: a run ends before it starts", path);
    return ESF_ERR_IO;
  }
  long long lo[3], hi[3];
  for (int k = 0; k < 3; k++) {
    lo[k] = 1LL << 40;
    hi[k] = -(1LL << 40);
    for (long long v : idx[k]) {
      lo[k] = v < lo[k] ? v : lo[k];
      hi[k] = v > hi[k] ? v : hi[k];
    }
    if (idx[k].empty()) lo[k] = hi[k] = 0;
    // one point of margin, so neighbour and corner reads stay on the lattice
    L->lo[k] = (int)(lo[k] - 1);
    L->n[k] = (int)(hi[k] - lo[k] + 3);
  }
  const long long nxy = (long long)L->n[0] * L->n[1];
  const long long total = nxy * L->n[2];
  if (total > (1LL << 31)) {
    set_error("svol_read: %s: lattice of %lld points is too large", path, total);
    return ESF_ERR_UNSUPPORTED;
  }
  L->val.assign((size_t)total, 0.0f);
  L->code.assign((size_t)total, 0);
  auto at = [&](long long x, long long y, long long z) {
    return (x - L->lo[0]) + (y - L->lo[1]) * L->n[0] + (z - L->lo[2]) * nxy;
  };
  const long long nY = (long long)idx[1].size(), nZ = (long long)idx[2].size();
  for (size_t r = 0; r + 1 < idx[0].size(); r += 2)
    for (long long x = idx[0][r]; x <= idx[0][r + 1]; x++) {
      const long long iv1 = aa0[r / 2] + x - idx[0][r];
      const long long ya = va[0][(size_t)iv1];
      const long long yb = iv1 + 1 < (long long)va[0].size() ? va[0][(size_t)iv1 + 1] : nY;
      if (ya < 0 || yb > nY || ya > yb || (ya & 1)) {
        set_error("svol_read: %s: bad y-run offsets", path);
        return ESF_ERR_IO;
      }
      for (long long ry = ya; ry + 1 < yb; ry += 2)
        for (long long y = idx[1][ry]; y <= idx[1][ry + 1]; y++) {
          const long long iv2 = aa1[ry / 2] + y - idx[1][ry];
          const long long za = va[1][(size_t)iv2];
          const long long zb = iv2 + 1 < (long long)va[1].size() ? va[1][(size_t)iv2 + 1] : nZ;
          if (za < 0 || zb > nZ || za > zb || (za & 1)) {
            set_error("svol_read: %s: bad z-run offsets", path);
            return ESF_ERR_IO;
          }
          for (long long rz = za; rz + 1 < zb; rz += 2) {
            for (long long z = idx[2][rz]; z <= idx[2][rz + 1]; z++) {
              const long long q = at(x, y, z);
              L->val[(size_t)q] = (float)values[(size_t)(aa2[rz / 2] + z - idx[2][rz])];
              L->code[(size_t)q] = 1;
            }
            // a gap before the next run of the column takes the sign of
            // that run's first value (DTGrid operator(), get)
            if (rz + 3 < zb) {
              const signed char c = values[(size_t)aa2[(rz + 2) / 2]] < 0 ? -1 : 0;
              for (long long z = idx[2][rz + 1] + 1; z < idx[2][rz + 2]; z++) L->code[(size_t)at(x, y, z)] = c;
            }
          }
        }
    }
  L->dx = dx;
  L->inC = inC;
  L->outC = outC;
  for (int k = 0; k < 3; k++) L->t[k] = tr[k];
  return ESF_OK;
}

void svol_to_grid(const SvolLattice& L, const double* p, double* g) {
  const double inv = 1.0 / L.dx;
  for (int k = 0; k < 3; k++) g[k] = p[k] * inv + (-L.t[k]) * inv;
}

// SPARSE_SDF::hashTriangle over all triangles in order: each triangle's
// rest bounding box (TRIANGLE::boundingBox) in lattice indices, grown by one
// (DTGrid::boundingBoxIndices: floor - 1 .. ceil + 1); band points in it
// list the triangle.
bool svol_hash_triangles(const SvolLattice& L, const double* rest, int ntri, const int* tris,
                         std::vector<int>* off, std::vector<int>* ids) {
  const long long nxy = (long long)L.n[0] * L.n[1];
  const long long total = nxy * L.n[2];
  std::vector<int> count((size_t)total + 1, 0);
  auto for_points = [&](int t, auto&& fn) {
    const double* v0 = rest + 3 * (long long)tris[3 * t];
    double mins[3] = {v0[0], v0[1], v0[2]}, maxs[3] = {v0[0], v0[1], v0[2]};
    for (int c = 1; c < 3; c++) {
      const double* v = rest + 3 * (long long)tris[3 * t + c];
      for (int k = 0; k < 3; k++) {
        mins[k] = v[k] < mins[k] ? v[k] : mins[k];
        maxs[k] = v[k] > maxs[k] ? v[k] : maxs[k];
      }
    }
    double gmin[3], gmax[3];
    svol_to_grid(L, mins, gmin);
    svol_to_grid(L, maxs, gmax);
    long long a[3], b[3];
    for (int k = 0; k < 3; k++) {
      a[k] = (long long)floor(gmin[k]) - 1 - L.lo[k];
      b[k] = (long long)ceil(gmax[k]) + 1 - L.lo[k];
      a[k] = a[k] < 0 ? 0 : a[k];
      b[k] = b[k] > L.n[k] - 1 ? L.n[k] - 1 : b[k];
    }
    for (long long z = a[2]; z <= b[2]; z++)
      for (long long y = a[1]; y <= b[1]; y++)
        for (long long x = a[0]; x <= b[0]; x++) {
          const long long q = x + y * L.n[0] + z * nxy;
          if (L.code[(size_t)q] == 1) fn(q);
        }
  };
  long long entries = 0;
  for (int t = 0; t < ntri; t++)
    for_points(t, [&](long long q) {
      count[(size_t)q + 1]++;
      entries++;
    });
  if (entries >= (1LL << 31) - 1) return false;  // offsets are 32-bit
  off->assign((size_t)total + 1, 0);
  for (long long q = 0; q < total; q++) (*off)[(size_t)q + 1] = (*off)[(size_t)q] + count[(size_t)q + 1];
  ids->assign((size_t)(*off)[(size_t)total] + 1, 0);
  std::vector<int> fill(off->begin(), off->end() - 1);
  for (int t = 0; t < ntri; t++) for_points(t, [&](long long q) { (*ids)[(size_t)fill[(size_t)q]++] = t; });
  return true;
}

}  // namespace esf

// Host-only reader of a ".svol" rest SDF into its dense lattice, for callers
// and tests that want the values without a scene. values/codes NULL: size
// query (lo, n, dx, translation, constants filled).
extern "C" esf_status esf_svol_read(const char* path, int lo[3], int n[3], double* dx, double translation[3],
                                    double constants[2], float* values, signed char* codes, size_t capacity) {
  if (!path || !lo || !n) {
    esf::set_error("esf_svol_read: null argument");
    return ESF_ERR_INVALID_ARG;
  }
  esf::SvolLattice L;
  esf_status e;
  try {
    e = esf::svol_read(path, &L);
  } catch (...) {  // host allocation of a very large lattice
    esf::set_error("esf_svol_read: out of host memory for %s", path);
    return ESF_ERR_OOM;
  }
  if (e) return e;
  for (int k = 0; k < 3; k++) {
    lo[k] = L.lo[k];
    n[k] = L.n[k];
    if (translation) translation[k] = L.t[k];
  }
  if (dx) *dx = L.dx;
  if (constants) {
    constants[0] = L.inC;
    constants[1] = L.outC;
  }
  if (!values && !codes) return ESF_OK;
  if (capacity < L.val.size()) {
    esf::set_error("esf_svol_read: the lattice has %zu points, the buffers hold %zu", L.val.size(), capacity);
    return ESF_ERR_INVALID_ARG;
  }
  if (values) memcpy(values, L.val.data(), L.val.size() * sizeof(float));
  if (codes) memcpy(codes, L.code.data(), L.code.size());
  return ESF_OK;
}
