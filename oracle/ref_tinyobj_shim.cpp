// TEST INFRASTRUCTURE: a C entry point over the reference's own OBJ reader
// (thirdparty/tinyobjloader/tiny_obj_loader.cpp of joshbainbridge/msc-project),
// compiled from the reference sources where they lie by oracle/build.py into
// oracle/_ref/.  Tests use it to pin the OBJ readers of the oracle and of the
// product against the reference on the same files.
#include <cstdint>
#include <cstring>
#include <string>

#include "tinyobjloader/tiny_obj_loader.h"

extern "C" int ref_obj_load(const char* path, float* positions, float* texcoords, uint32_t* indices, int64_t* sizes) {
  tinyobj::shape_t shape;
  std::string err = tinyobj::LoadObj(shape, path);
  if (!err.empty()) return -1;
  sizes[0] = (int64_t)shape.mesh.positions.size();
  sizes[1] = (int64_t)shape.mesh.texcoords.size();
  sizes[2] = (int64_t)shape.mesh.indices.size();
  if (positions) memcpy(positions, shape.mesh.positions.data(), shape.mesh.positions.size() * 4);
  if (texcoords) memcpy(texcoords, shape.mesh.texcoords.data(), shape.mesh.texcoords.size() * 4);
  if (indices) memcpy(indices, shape.mesh.indices.data(), shape.mesh.indices.size() * 4);
  return 0;
}
