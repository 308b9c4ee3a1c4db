/*
 * CPU oracle of the sorted deferred-shading path tracer - TEST INFRASTRUCTURE.
 *
 * A plain C++ restatement of the reference renderer (joshbainbridge/msc-project)
 * used only by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg
 * as the checker; the product never links or calls it.  Each function cites
 * the reference code it follows in oracle.cpp.
 *
 * Parity pinning: the reference ships no tests, golden images or example
 * scenes, and cannot be built here (Embree 2.6.1, TBB, Boost, yaml-cpp, Eigen,
 * OpenImageIO and OpenEXR are absent).  Only its OBJ reader
 * (thirdparty/tinyobjloader) compiles from its own sources, and it is used to
 * pin this oracle's OBJ reader.  Everything else is parity unpinned against
 * the reference itself; it is checked by analytic known-answer tests instead.
 *
 * The float instantiation follows the exact arithmetic order documented for
 * the device stages (explicit fused multiply-adds in dot/cross/affine maps,
 * correctly rounded division and square root), so it can be compared with the
 * GPU bit for bit; the double instantiation is the converged reference.
 */
#ifndef MSC_ORACLE_H_
#define MSC_ORACLE_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle_scene oracle_scene;

oracle_scene* oracle_load(const char* yaml_path, char* err, int errcap);
void oracle_free(oracle_scene* s);
/* World-space triangles (9 floats each, geomID order) and their geomIDs. */
void oracle_triangles(const oracle_scene* s, float* v9, int32_t* geom);
/* Per-job overrides (values <= 0 / < 0 / NULL keep the scene's): resolution,
 * sample count (grid split as for non-square counts), depth limits, a pinhole
 * camera (translation, rotation in degrees, focal length) and the seed. */
int oracle_set_job(oracle_scene* s, int width, int height, int spp, int min_depth, int max_depth, const float* cam_t,
                   const float* cam_r, float focal, uint32_t seed);
/* w, h, spp, triangles, lights */
void oracle_info(const oracle_scene* s, int* out5);

/* One render iteration (iteration index `iteration`, 0-based) of every path
 * with `threads` worker threads.  sample_rgb (3*P), sample_xy (2*P) may be
 * NULL; pixels (3*W*H, row-major) is accumulated into (pixels += filtered).
 * counts[0] = closest-hit queries, counts[1] = occlusion queries. */
int oracle_render_f32(oracle_scene* s, int iteration, int threads, float* sample_rgb, float* sample_xy, float* pixels,
                      uint64_t* counts);
int oracle_render_f64(oracle_scene* s, int iteration, int threads, double* sample_rgb, double* sample_xy,
                      double* pixels, uint64_t* counts);
/* Paths [first, first+n) only, no film output: the timed CPU baseline. */
int oracle_render_range_f32(oracle_scene* s, int iteration, int threads, uint64_t first, uint64_t n, uint64_t* counts);
/* Paths [first, first+n) with their radiance (3*n floats) and film positions
 * (2*n floats, may be NULL), indexed from `first`: spot checks of full-size scenes. */
int oracle_render_range_rgb_f32(oracle_scene* s, int iteration, int threads, uint64_t first, uint64_t n, float* rgb,
                                float* xy, uint64_t* counts);

/* Closest hit (geom/prim = reference geomID/primID, -1 for a miss) and occlusion. */
int oracle_trace_f32(const oracle_scene* s, const float* org, const float* dir, int n, float* t, float* u, float* v,
                     int32_t* geom, int32_t* prim);
int oracle_occluded_f32(const oracle_scene* s, const float* org, const float* dir, const float* tmax, int n,
                        int32_t* occluded);

/* Stage restatements on plain arrays. */
void oracle_cardinal(const float* dirs, int n, int32_t* bins);
void oracle_ray_keys(const float* org, const float* dir, int n, uint32_t* keys);
void oracle_stable_sort_pairs(uint32_t* keys, uint32_t* vals, int n, int bits);
/* The reference's median-split ray order of a batch (RaySort.cpp:7-118): order[i]
 * = index of the i-th ray; for coherence comparisons with the project's key. */
void oracle_median_split_order(const float* org, const float* dir, int n, uint32_t* order);
void oracle_bin_partition(const float* rays, int n, int cap, float* out, int32_t* counts);
void oracle_ray_bins(const float* dirs, int n, int nbins, int32_t* bins);
// Periodic bilinear lookups of a PFM / PPM image at (s[i], t[i]); -1 if unreadable.
int oracle_image_lookup(const char* path, int n, const float* s, const float* t, float* rgb);
void oracle_bin_partition_n(const float* rays, int n, int nbins, int cap, float* out, int32_t* counts);
void oracle_tent_filter(const float* sample_rgb, const float* sample_xy, int w, int h, int spp, float* pixels);

/* OBJ reading with tinyobjloader's rules: sizes[0..2] = #positions floats,
 * #texcoord floats, #indices; arrays may be NULL to query sizes. */
int oracle_obj_load(const char* path, float* positions, float* texcoords, uint32_t* indices, int64_t* sizes);

#ifdef __cplusplus
}
#endif

#endif
