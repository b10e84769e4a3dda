// Frame-file helpers (esf_io.cpp): gz fields in the reference's FIELD_3D
// layout, OBJ meshes, frame file names. Host code only.
#pragma once

#include <stddef.h>

#include <string>

#include "../../include/eulersf.h"

namespace esf {

void set_error(const char* fmt, ...);

// "<dataPath>frame.NNNN" (IO::itoPaddedString, include/util/IO.h:27-37)
std::string frame_prefix(const char* dataPath, int frame);
// FIELD_3D::writeGz layout; count = doubles of data (x3 for vector fields)
esf_status write_field_gz(const std::string& path, const int res[3], double dh, const double origin[3],
                          const double* data, size_t count);
// FIELD_3D::readGz; the file's resolution must equal res
esf_status read_field_gz(const std::string& path, const int res[3], size_t count, double* data);
// OBJ::Save format
esf_status write_obj(const std::string& path, const double* verts, int nv, const int* tris, int ntri);
// vertex positions of an OBJ written for a mesh of nv vertices
esf_status read_obj_vertices(const std::string& path, int nv, double* verts);

}  // namespace esf
