// Frame files of COUPLED_INTEGRATOR_3D::writeFrame/readFrame
// (src/integrator/COUPLED_INTEGRATOR_3D.cpp:977-1012) and
// DEFOR_SOLID_3D::writeFrame/readFrame (src/integrator/DEFOR_SOLID_3D.cpp:1299-1370):
//   * gz fields in the FIELD_3D / VEC3F_FIELD_3D layout
//     (include/geometry/FIELD_3D.h:286-365, VEC3F_FIELD_3D.h:199-267): three
//     int32 resolutions, dh and the origin as float64, then float64 data, x
//     fastest, vectors interleaved xyz; written with gzip level 1 ("wb1");
//   * the surface mesh as OBJ text in OBJ::Save's format
//     (src/geometry/OBJ.cpp:336-375): "v x y z" with the iostream default of
//     6 significant digits, "f a/t b/t c/t " with 1-based indices (t = 0 for a
//     mesh without texture coordinates);
//   * file names "frame." + the frame number zero-padded to 4 digits
//     (include/util/IO.h:27-37).
// zlib is loaded at run time (libz.so.1) so that the library builds and loads
// where zlib's headers are absent; without it, frame I/O reports an error.
#include <dlfcn.h>
#include <stdio.h>
#include <string.h>

#include <mutex>
#include <string>
#include <vector>

#include "esf_io.h"

namespace esf {

namespace {
struct Zlib {
  void* (*open)(const char*, const char*) = nullptr;
  int (*write)(void*, const void*, unsigned) = nullptr;
  int (*read)(void*, void*, unsigned) = nullptr;
  int (*close)(void*) = nullptr;
  bool ok = false;
};

const Zlib& zlib() {
  static Zlib z;
  static std::once_flag once;
  std::call_once(once, [] {
    void* h = dlopen("libz.so.1", RTLD_NOW | RTLD_LOCAL);
    if (!h) h = dlopen("libz.so", RTLD_NOW | RTLD_LOCAL);
    if (!h) return;
    z.open = reinterpret_cast<void* (*)(const char*, const char*)>(dlsym(h, "gzopen"));
    z.write = reinterpret_cast<int (*)(void*, const void*, unsigned)>(dlsym(h, "gzwrite"));
    z.read = reinterpret_cast<int (*)(void*, void*, unsigned)>(dlsym(h, "gzread"));
    z.close = reinterpret_cast<int (*)(void*)>(dlsym(h, "gzclose"));
    z.ok = z.open && z.write && z.read && z.close;
  });
  return z;
}

// gzwrite/gzread take unsigned counts: move large arrays in 1 GiB pieces
bool gz_put(const Zlib& z, void* f, const void* p, size_t n) {
  const char* c = static_cast<const char*>(p);
  while (n > 0) {
    unsigned k = (unsigned)(n < (1u << 30) ? n : (1u << 30));
    if (z.write(f, c, k) != (int)k) return false;
    c += k;
    n -= k;
  }
  return true;
}
bool gz_get(const Zlib& z, void* f, void* p, size_t n) {
  char* c = static_cast<char*>(p);
  while (n > 0) {
    unsigned k = (unsigned)(n < (1u << 30) ? n : (1u << 30));
    if (z.read(f, c, k) != (int)k) return false;
    c += k;
    n -= k;
  }
  return true;
}
}  // namespace

std::string frame_prefix(const char* dataPath, int frame) {
  char num[32];
  snprintf(num, sizeof num, "%i", frame);
  std::string s(num);
  if (frame < 10) s = "0" + s;
  if (frame < 100) s = "0" + s;
  if (frame < 1000) s = "0" + s;
  return std::string(dataPath ? dataPath : "") + "frame." + s;
}

esf_status write_field_gz(const std::string& path, const int res[3], double dh, const double origin[3],
                          const double* data, size_t count) {
  const Zlib& z = zlib();
  if (!z.ok) {
    set_error("frame I/O needs zlib (libz.so.1), which could not be loaded");
    return ESF_ERR_UNSUPPORTED;
  }
  void* f = z.open(path.c_str(), "wb1");
  if (!f) {
    set_error("could not open %s for writing", path.c_str());
    return ESF_ERR_IO;
  }
  bool ok = gz_put(z, f, res, 3 * sizeof(int)) && gz_put(z, f, &dh, sizeof(double)) &&
            gz_put(z, f, origin, 3 * sizeof(double)) && gz_put(z, f, data, count * sizeof(double));
  ok = (z.close(f) == 0) && ok;
  if (!ok) {
    set_error("writing %s failed", path.c_str());
    return ESF_ERR_IO;
  }
  return ESF_OK;
}

esf_status read_field_gz(const std::string& path, const int res[3], size_t count, double* data) {
  const Zlib& z = zlib();
  if (!z.ok) {
    set_error("frame I/O needs zlib (libz.so.1), which could not be loaded");
    return ESF_ERR_UNSUPPORTED;
  }
  void* f = z.open(path.c_str(), "rb");
  if (!f) {
    set_error("could not open %s", path.c_str());
    return ESF_ERR_IO;
  }
  int r[3];
  double hdr[4];
  bool ok = gz_get(z, f, r, sizeof r) && gz_get(z, f, hdr, sizeof hdr);
  if (ok && (r[0] != res[0] || r[1] != res[1] || r[2] != res[2])) {
    z.close(f);
    set_error("%s holds a %dx%dx%d field, the scene needs %dx%dx%d", path.c_str(), r[0], r[1], r[2],
              res[0], res[1], res[2]);
    return ESF_ERR_IO;
  }
  ok = ok && gz_get(z, f, data, count * sizeof(double));
  z.close(f);
  if (!ok) {
    set_error("%s is truncated or unreadable", path.c_str());
    return ESF_ERR_IO;
  }
  return ESF_OK;
}

esf_status write_obj(const std::string& path, const double* verts, int nv, const int* tris, int ntri) {
  FILE* f = fopen(path.c_str(), "w");
  if (!f) {
    set_error("could not open %s for writing", path.c_str());
    return ESF_ERR_IO;
  }
  for (int i = 0; i < nv; i++)
    fprintf(f, "v %g %g %g\n", verts[3 * i], verts[3 * i + 1], verts[3 * i + 2]);
  for (int t = 0; t < ntri; t++)
    fprintf(f, "f %d/0 %d/0 %d/0 \n", tris[3 * t] + 1, tris[3 * t + 1] + 1, tris[3 * t + 2] + 1);
  const bool bad = ferror(f) != 0;
  if (fclose(f) != 0 || bad) {
    set_error("writing %s failed", path.c_str());
    return ESF_ERR_IO;
  }
  return ESF_OK;
}

esf_status read_obj_vertices(const std::string& path, int nv, double* verts) {
  FILE* f = fopen(path.c_str(), "r");
  if (!f) {
    set_error("could not open %s", path.c_str());
    return ESF_ERR_IO;
  }
  char line[512];
  int n = 0;
  while (fgets(line, sizeof line, f)) {
    if (line[0] != 'v' || (line[1] != ' ' && line[1] != '\t')) continue;
    double a, b, c;
    if (sscanf(line + 2, "%lf %lf %lf", &a, &b, &c) != 3) continue;
    if (n < nv) {
      verts[3 * n] = a;
      verts[3 * n + 1] = b;
      verts[3 * n + 2] = c;
    }
    n++;
  }
  fclose(f);
  if (n != nv) {
    set_error("%s has %d vertices, the solid's mesh %d", path.c_str(), n, nv);
    return ESF_ERR_IO;
  }
  return ESF_OK;
}

}  // namespace esf
