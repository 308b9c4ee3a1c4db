// Device records and stage launchers of the wavefront render loop.
//
// A ray record (the reference's RayCompressed, include/core/RayCompressed.h:14-23)
// is three float4 in structure-of-arrays form:
//   o = (org.xyz, lastPdf), d = (dir.xyz, rayDepth as int; < 0 = dead),
//   w = (weight.rgb, sampleID as int).
// A shadow ray is o = (org.xyz, tmax), d = (dir.xyz, sampleID), c = (weighted contribution.rgb, 0).
// A hit is (t, u, v, leaf-order triangle or -1).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "scene.h"

namespace mscg {

struct RayBuf {
  float4* o = nullptr;
  float4* d = nullptr;
  float4* w = nullptr;
};

struct ShadowBuf {
  float4* o = nullptr;
  float4* d = nullptr;
  float4* c = nullptr;
};

struct DevScene {
  const float4* nodes;   // binary BVH (null when the 8-wide form is used)
  const uint4* wnodes;   // 8-wide BVH (null for the binary form)
  int num_wnodes;
  const float4* tris;
  const int* tri_orig;
  int num_tris;
  const ShaderRec* shaders;
  const GeomRec* geoms;
  const LightRec* lights;
  int num_lights;
  float light_pick;  // 1 / num_lights (Integrator.cpp:22)
};

struct DevFrame {
  CameraRec cam;
  int width, height, spp;
  int grid_x, grid_y;  // stratification cells (base x base in the reference)
  int sampler;
  int min_depth, max_depth;
  float threshold;
  int mis_power;
  uint32_t iter_seed;
  float4* sample_rgb;  // per-sample radiance (Image::samples r,g,b)
  float2* sample_pos;  // per-sample film position (Image::samples x,y)
};

// Error bits reported through the engine's device flag word.
enum : int { ERR_BIN_OVERFLOW = 1, ERR_STACK_OVERFLOW = 2, ERR_TRAVERSAL_CAP = 4, ERR_BVH_INDEX = 8 };

constexpr int kMaxBins = 8;  // 6 cardinal bins + the dead bucket, rounded up

// Each launcher returns the number of kernels it enqueued.
int launch_raygen(const DevFrame& f, uint32_t first, int n, RayBuf out, cudaStream_t s);

struct BinPool {
  RayBuf rays;       // kMaxBins-1 bins of `cap` rays each, bin b at [b*cap, (b+1)*cap)
  int cap = 0;
  int* count = nullptr;      // device: rays held per bin
  uint32_t* tile_counts = nullptr;  // scratch for the partition (kMaxBins * tiles)
  int max_tiles = 0;
  int* err = nullptr;
};
constexpr int kPartTile = 2048;
// Stable partition of src[0, n) by cardinal bin, appended behind each bin's
// current content; dead rays (d.w < 0) are dropped.
int launch_bin_partition(const RayBuf& src, int n, BinPool& pool, cudaStream_t s);

// Per-ray cardinal bin only (stage test).
int launch_cardinal(const float4* d, int n, int* out, cudaStream_t s);

// Origin box of rays [0, n) into box6 (ordered-int min xyz, max xyz; caller initialises).
int launch_origin_box(const float4* o, int n, uint32_t* box6, cudaStream_t s);
int launch_ray_keys(const float4* o, const float4* d, int n, const uint32_t* box6, uint32_t* keys, cudaStream_t s);
int launch_gather(const RayBuf& src, const uint32_t* perm, int n, RayBuf dst, cudaStream_t s);

int launch_trace_closest(const DevScene& sc, const float4* o, const float4* d, int n, float4* hits, int* err,
                         cudaStream_t s);
int launch_hit_keys(const DevScene& sc, const float4* hits, int n, uint32_t* keys, cudaStream_t s);
int launch_shade(const DevScene& sc, const DevFrame& f, const RayBuf& batch, const float4* hits, const uint32_t* order,
                 int n, RayBuf next, ShadowBuf sh, int* sh_count, cudaStream_t s);
int launch_trace_shadow(const DevScene& sc, const ShadowBuf& sh, const int* sh_count, int max_n, float4* sample_rgb,
                        int* err, cudaStream_t s);
// Occlusion for explicit rays (stage test): occluded[i] = 1 if blocked in (tnear, tmax).
int launch_occluded(const DevScene& sc, const float4* o, const float4* d, int n, int* occluded, int* err, cudaStream_t s);
int launch_filter(const DevFrame& f, int filter, float* pixels, cudaStream_t s);

}  // namespace mscg
