// Device records and stage launchers of the wavefront render loop.
//
// A ray record (the reference's RayCompressed, include/core/RayCompressed.h:14-23)
// is three float4 in structure-of-arrays form:
//   o = (org.xyz, lastPdf)
//   d = (dir.xyz, info)   info = job << 16 | scene << 8 | rayDepth as int; < 0 = dead
//   w = (weight.rgb, sampleID within its job, as int)
// A shadow ray is o = (org.xyz, tmax), d = (dir.xyz, global sample index),
// c = (weighted contribution.rgb, scene as int).  A hit is (t, u, v, triangle or -1).
//
// Scenes and jobs live in device tables indexed by the ray's info word, so one
// batch can hold rays of many jobs over many scenes.
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

constexpr int kMaxJobs = 1 << 15;
constexpr int kMaxScenes = 256;
constexpr int kMaxDepth = 255;

__host__ __device__ __forceinline__ int ray_info(int job, int scene, int depth) {
  return (job << 16) | (scene << 8) | depth;
}
__host__ __device__ __forceinline__ int info_job(int info) { return info >> 16; }
__host__ __device__ __forceinline__ int info_scene(int info) { return (info >> 8) & 0xff; }
__host__ __device__ __forceinline__ int info_depth(int info) { return info & 0xff; }

struct SceneRec {        // one resident scene
  const uint4* wnodes;   // 8-wide BVH (null for the binary form)
  const float4* nodes;   // binary BVH (null for the wide form)
  const float4* tris;
  const int* tri_orig;
  int num_wnodes;
  int num_tris;
  const ShaderRec* shaders;
  const GeomRec* geoms;
  const LightRec* lights;
  int num_lights;
  float light_pick;      // 1 / num_lights (Integrator.cpp:22)
  uint32_t tri_base;     // offset of this scene's triangles in the hit-key space
  int hit_key_bits;      // 32 or 64 (single-scene runs)
  const float4* spheres; // sphere lights (extension): centre, radius
  const int* sphere_light;  // light index of each sphere
  int num_spheres;
  int texel_res;         // face texels per side (0: none)
  const unsigned short* texels;  // FP16 bits, [face][j][i][rgb], face = original triangle index
  // image textures (Standard / Layered): post-order programs of (op, node),
  // op 0 constant, 1 image, 2 layer; images as (first texel, width, height)
  const TexNode* tex_nodes;
  const int2* tex_ops;
  const int4* tex_images;
  const float4* tex_texels;
  const float* tri_uv;   // 6 per original triangle: uv of v0, v1, v2
  float4 key_lo;         // ray sort key: the scene box's low corner
  float4 key_scale;      // and 64 / its extent per axis (0 for a flat axis)
  // 64-bit hit key scenes: 1 + the rank of each triangle (BVH leaf order) in
  // the order of the key's (shader id, face id) fields, so that a sort of
  // shade_rank_bits bits groups hits as the key's top 35 bits do
  const uint32_t* shade_rank;
  int shade_rank_bits;
};

// Texture coordinate of a hit (PolygonObject::texture, src/core/PolygonObject.cpp:45-63).
__host__ __device__ __forceinline__ float uv_interp(float a0, float a1, float a2, float s, float t) {
  return (((1.f - s) - t) * a0 + s * a1) + t * a2;
}

// A closest hit on sphere light s is recorded as triangle -2 - s.
__host__ __device__ __forceinline__ int sphere_hit_code(int s) { return -2 - s; }

struct JobRec {          // one render job: a scene seen through one camera
  CameraRec cam;
  int width, height, spp;
  int grid_x, grid_y;    // stratification cells (base x base in the reference)
  int sampler;
  int filter;
  int min_depth, max_depth;
  float threshold;
  int mis_power;
  uint32_t iter_seed;
  int scene;
  uint32_t sample_base;  // first entry of this job in the sample arrays
  float* pixels;         // W*H*3 accumulated image, row-major
};

struct Film {            // per-sample radiance and film position, all jobs (Image::samples)
  float4* rgb = nullptr;
  float2* pos = nullptr;
};

// Error bits reported through the engine's device flag word.
enum : int {
  ERR_BIN_OVERFLOW = 1,
  ERR_STACK_OVERFLOW = 2,
  ERR_TRAVERSAL_CAP = 4,
  ERR_BVH_INDEX = 8,
  ERR_APPEND_WAIT = 16  // a bin append waited past its cap for a chunk another lane was taking
};

// Direction bins: the reference's 6 cardinal bins (dominant axis and sign),
// or the 26 / 98 surface cells of a 3^3 / 5^3 direction cube (extension).
constexpr int kMaxBins = 98;
constexpr int kBinRadix = 128;  // partition digits: bins + the dead bucket, rounded up
// Bin pool chunks: a bin is a list of whole chunks of the pool (a chunk table
// row), so any number of bins share one pool of about one generation of rays.
constexpr int kChunkShift = 12;
constexpr int kChunk = 1 << kChunkShift;

__host__ __device__ __forceinline__ int bin_bits(int nbins) { return nbins <= 8 ? 3 : (nbins <= 32 ? 5 : 7); }

// Where the rays of one batch sit: up to kMaxBins (bin, first position) runs.
struct Segments {
  int count;
  int prefix[kMaxBins + 1];  // prefix[k] = rays in runs before k; prefix[count] = total
  int bin[kMaxBins];
  int start[kMaxBins];       // first position within the bin
};

// One batch as the device chose it (k_plan): the runs of the bin pool it
// takes, its size and the key prefix width.  Kernels after the plan read it
// from device memory, so a batch body needs no host decision and can be
// replayed from a CUDA graph.
struct BatchPlan {
  int nb;
  int prefix_bits;
  int bin_bits;
  int pad;
  Segments seg;
};

// Device counters of the wavefront, read back in one copy.
struct Counters {
  int bin_count[kBinRadix];  // rays held per bin
  int shadow_count[2];       // shadow rays of the current batch, per shadow queue
  int err;                   // error bits
  int in_bins;               // rays held in all bins
  int pad[4];
  unsigned long long closest, shadow, batches;
};

// Each launcher returns the number of kernels it enqueued.

struct BinPool {
  RayBuf rays;               // num_chunks * kChunk rays
  int nbins = 6;             // the bin function new rays are sorted by (6, 26 or 98)
  int num_chunks = 0;
  int max_chunks = 0;        // chunk-table row length
  int* count = nullptr;      // device [kMaxBins]: rays held per bin
  int* held = nullptr;       // device [kMaxBins]: chunks in each bin's row
  int* table = nullptr;      // device [kMaxBins * max_chunks]: pool chunk of a bin's k-th chunk
  int* free_stack = nullptr; // device [num_chunks]
  int* free_top = nullptr;   // device: entries on the free stack
  int* in_bins = nullptr;    // device: rays held in all bins
  uint32_t* keys = nullptr;  // device [num_chunks * kChunk]: ray sort key of each held ray
                             // (top 24 bits of ray_sort_key, the ray's scene in the low byte)
  uint32_t* tile_counts = nullptr;  // partition scratch ((kMaxBins + 1) * tiles)
  int max_tiles = 0;
  int* err = nullptr;
  // Direct binning (shading appends continuing rays into the bins; batches of
  // at least kDirectMin rays): each bin's append cursor, the chunks taken for
  // the appends past the bin's held chunks (pend_cols per bin; -1 not taken
  // yet, -2 a failed take; the chunk table itself still maps the batch's own
  // rays while they are read) and the chunks of the batch in flight, returned
  // to the free stack after its shading.
  int* cursor = nullptr;     // device [kMaxBins]
  int* pend = nullptr;       // device [kMaxBins * pend_cols]
  int pend_cols = 0;
  int* retired = nullptr;    // device [retire_cap]
  int* n_retired = nullptr;  // device
  int retire_cap = 0;
};
// Smallest batch whose plan keeps each touched bin chunk-aligned (direct binning).
constexpr int kDirectMin = 2 * kChunk;
__host__ __device__ __forceinline__ int pool_index(const int* table, int max_chunks, int bin, int pos) {
  return table[bin * max_chunks + (pos >> kChunkShift)] * kChunk + (pos & (kChunk - 1));
}
// Chunks a pool needs so that `rays_in_flight` rays fit in any split over
// the bins (each bin holds at most one partial chunk), with room for the
// chunks of one batch of `batch` rays held back while its shading appends.
inline size_t bin_pool_chunks(size_t rays_in_flight, size_t batch = 0) {
  return (rays_in_flight + kChunk - 1) / kChunk + (batch + kChunk - 1) / kChunk + 3 * (size_t)kMaxBins;
}
// Empties the pool: every chunk free (stream-ordered).
int launch_pool_reset(BinPool& pool, cudaStream_t s);
constexpr int kPartTile = 2048;
// Stable partition of src[0, n) by direction bin, appended behind each bin's
// current content; dead rays (info < 0) are dropped.
// n_dev (optional): the count is read on the device, n is then its upper bound.
// scenes (optional): also store each ray's sort key (pool.keys) for the ray sort.
int launch_bin_partition(const RayBuf& src, int n, BinPool& pool, cudaStream_t s, const int* n_dev = nullptr,
                         const SceneRec* scenes = nullptr);
// Camera rays of samples [first, first + n) of a job straight into their
// direction bins in sample order (a stable partition whose rays are made
// twice instead of staged), their film samples zeroed and positioned;
// key_scenes (optional): also store each ray's sort key; digits: scratch of
// n bytes (each ray's bin between the two kernels).
int launch_camera_rays(const JobRec& job, int job_index, uint32_t first, int n, Film film, BinPool& pool,
                       const SceneRec* key_scenes, uint8_t* digits, cudaStream_t s);

// The next batch from the bins: the fullest bin's top, topped up from the
// next fullest while merge is set (the order of the host's choice before).
// Also opens the batch: shadow count zeroed, counters.  direct: the batch's
// shading appends into the bins (launch_shade with the pool), so each bin the
// batch takes from is left chunk-aligned, the batch's chunks are held back
// until launch_append_commit and the append cursors are set.
int launch_plan(BinPool& pool, int batch_cap, int merge, int scene_bits, BatchPlan* plan, Counters* ctr,
                cudaStream_t s, bool direct = false);
// After a direct-binning shade: the appended rays join their bins and the
// batch's chunks return to the free stack.
int launch_append_commit(BinPool& pool, cudaStream_t s);
// Direction bin of each direction (6, 26 or 98 bins).
int launch_ray_bins(const float4* d, int n, int nbins, int* out, cudaStream_t s);

// Per-ray cardinal bin only (stage test).
int launch_cardinal(const float4* d, int n, int* out, cudaStream_t s);

// Sort keys of the batch rays from pool.keys: (scene, direction bin) above the
// key when prefix_bits > 0; only the top key_bits bits are kept (shifted down).
// where (optional): each batch ray's pool index, which sorted beside the keys
// gives the rays' slots in sorted order.  hist (optional, with where; key_bits
// a multiple of 8): the 8-bit digit counts of every pass of the keys are
// added into it (zeroed beforehand), as an 8-bit-digit sort with hist_ready
// takes them.
int launch_ray_keys(const BinPool& pool, const BatchPlan* plan, int n_max, int key_bits, uint32_t* keys,
                    cudaStream_t s, uint32_t* where = nullptr, uint32_t* hist = nullptr);
// ray_sort_key of n rays (o, d as float4) in the origin box lo + [0, 64 / scale).
int launch_ray_keys_direct(const float4* o, const float4* d, int n, float3 lo, float3 scale, uint32_t* keys,
                           cudaStream_t s);
// Pool index of each batch ray in sorted order (perm optional) into slots.
int launch_batch_slots(const BinPool& pool, const BatchPlan* plan, int n_max, const uint32_t* perm, int* slots,
                       cudaStream_t s);

// slots (optional): ray i is (o, d)[slots[i]] (the batch read in place from
// the bin pool); hits are indexed by i.
int launch_trace_closest(const SceneRec* scenes, int num_scenes, const SceneRec& scene0, const float4* o,
                         const float4* d, const int* slots, int n, float4* hits, int* err, cudaStream_t s,
                         const int* n_dev = nullptr, int block = 128, int* counter = nullptr);
int launch_hit_keys(const SceneRec* scenes, const float4* d, const int* slots, const float4* hits, int n,
                    uint32_t* keys, cudaStream_t s, const int* n_dev = nullptr);
// The 64-bit hit key of one scene (shader id 12 b, face 23 b, quantised u 15 b, v 14 b; misses and
// sphere-light hits 0) as low and high words.
int launch_hit_keys64(const SceneRec* scenes, const float4* hits, int n, uint32_t* lo, uint32_t* hi,
                      cudaStream_t s, const int* n_dev = nullptr);
// Hit keys from the (shader, face) rank table of a 64-bit-key scene (misses 0).
int launch_hit_keys_rank(const SceneRec* scenes, const float4* hits, int n, uint32_t* keys, cudaStream_t s,
                         const int* n_dev = nullptr);
int launch_gather_u32(const uint32_t* src, const uint32_t* idx, int n, uint32_t* dst, cudaStream_t s,
                      const int* n_dev = nullptr);
// Fills the scene's face texels from their seed (FP16 bits of k / 1024).
int launch_face_texels(unsigned short* texels, int64_t faces, int res, uint32_t seed, cudaStream_t s);
// Continuing rays go to `next` (one record per hit, ended paths dead), or
// with `direct` straight into the pool's bins (plan made with direct set);
// key_scenes (direct only, optional): also store each ray's sort key.
int launch_shade(const SceneRec* scenes, const JobRec* jobs, Film film, const RayBuf& batch, const int* slots,
                 const float4* hits, const uint32_t* order, int n, RayBuf next, ShadowBuf sh, int* sh_count,
                 uint32_t* job_done, cudaStream_t s, const int* n_dev = nullptr, const BinPool* direct = nullptr,
                 const SceneRec* key_scenes = nullptr);
// shadow_total (optional): the batch's shadow count is added to it.
int launch_trace_shadow(const SceneRec* scenes, int num_scenes, const SceneRec& scene0, const ShadowBuf& sh,
                        const int* sh_count, int max_n, float4* sample_rgb, int* err, cudaStream_t s,
                        unsigned long long* shadow_total = nullptr, int block = 128, int* counter = nullptr);
// Sizes the persistent traversal grids (call before any stream capture).
void persistent_grids_init();
// counter (optional, 8-wide BVH only): a device int for the persistent
// traversal with per-lane ray refill; null selects one thread per ray.
// Occlusion for explicit rays of scene 0 (stage test): occluded[i] = 1 if blocked in (tnear, tmax).
int launch_occluded(const SceneRec& scene, const float4* o, const float4* d, int n, int* occluded, int* err,
                    cudaStream_t s);
int launch_filter(const JobRec& job, Film film, cudaStream_t s);

}  // namespace mscg
