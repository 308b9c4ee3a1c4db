// Device LBVH over the flattened scene triangles (see bvh.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <string>

namespace mscg {

struct DeviceBvh {
  float4* nodes = nullptr;     // binary: 4 float4 per internal node (layout in trace.cuh)
  uint4* wnodes = nullptr;     // 8-wide: 5 uint4 per node (layout in trace.cuh), null for the binary form
  float4* tris = nullptr;      // 3 float4 per triangle in leaf order
  int* tri_orig = nullptr;     // leaf order -> global triangle index (geomID-major)
  float* bounds_dev = nullptr; // scene box: lo.xyz, hi.xyz
  int num_tris = 0;
  int num_nodes = 0;
  int num_wnodes = 0;
};

// d_v: 9 floats per triangle (v0, v1, v2) in global order; d_geom: geomID per
// triangle; d_light: 1 for emitter triangles.  wide: collapse the binary LBVH
// into 8-wide nodes with quantised child boxes (leaves of up to 3 triangles).
// Returns the number of kernel launches, or -1 with *err set.
int bvh_build(const float* d_v, const int* d_geom, const uint8_t* d_light, int n, bool wide, DeviceBvh* out,
              cudaStream_t stream, std::string* err);
void bvh_free(DeviceBvh* b);

}  // namespace mscg
