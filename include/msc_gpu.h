/*
 * msc_gpu.h - C ABI of the GB300 (sm_103a) sorted deferred-shading path tracer.
 *
 * The render-loop entry points replace the public interface of the
 * reference's engine class, msc::Pathtracer (include/core/Pathtracer.h:36-110
 * of joshbainbridge/msc-project).  Every function returns MSC_OK (0) or a
 * negative status; msc_last_error() gives the message.  No C++ exception
 * crosses this boundary.  Pointers are plain host pointers unless a name ends
 * in _device.  A handle is used by one render thread; msc_terminate() and
 * msc_image() may be called from another thread.
 */
#ifndef MSC_GPU_H_
#define MSC_GPU_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MSC_OK 0
#define MSC_ERR_ARG (-1)       /* bad argument or null handle */
#define MSC_ERR_SCENE (-2)     /* scene file could not be read or is malformed */
#define MSC_ERR_CUDA (-3)      /* a CUDA call failed (no device, out of memory, launch error) */
#define MSC_ERR_DEVICE (-4)    /* a device stage reported an error flag (bin overflow, stack overflow) */
#define MSC_ERR_BUSY (-5)      /* the handle is rendering on another thread */

typedef struct msc_handle msc_handle;

/* Pathtracer::Pathtracer(const std::string&) - include/core/Pathtracer.h:44,
 * src/core/Pathtracer.cpp:369-379.  Loads the two-document YAML scene (and the
 * OBJ files it names), builds the device BVH and allocates the render buffers
 * on the current CUDA device. */
int msc_create(const char* yaml_path, msc_handle** out);

/* Pathtracer::~Pathtracer() - include/core/Pathtracer.h:49, src/core/Pathtracer.cpp:381-392. */
int msc_destroy(msc_handle* h);

/* int Pathtracer::process() - include/core/Pathtracer.h:82, src/core/Pathtracer.cpp:425-493.
 * Renders one iteration (every pixel x sample), adds the filtered result to
 * the accumulated image and copies it to the host mirror.  *iteration gets
 * the new iteration count, or 0 when msc_terminate() stopped the pass. */
int msc_process(msc_handle* h, int* iteration);

/* Same as msc_process without the device-to-host copy of the image; the
 * host mirror is refreshed by the next msc_image() call. */
int msc_process_device(msc_handle* h, int* iteration);

/* void Pathtracer::image(float**, int*, int*) - include/core/Pathtracer.h:58,
 * src/core/Pathtracer.cpp:394-400.  Row-major y*W+x, 3 floats per pixel, the
 * sum over iterations (divide by the iteration count to display).  The
 * buffer is owned by the handle and valid until the next process/clear/destroy. */
int msc_image(msc_handle* h, const float** rgb, int* width, int* height);

/* void Pathtracer::clear() - include/core/Pathtracer.h:63, src/core/Pathtracer.cpp:402-413. */
int msc_clear(msc_handle* h);

/* bool Pathtracer::active() - include/core/Pathtracer.h:70, src/core/Pathtracer.cpp:415-418. */
int msc_active(msc_handle* h, int* active);

/* void Pathtracer::terminate() - include/core/Pathtracer.h:75, src/core/Pathtracer.cpp:420-423.
 * Thread-safe; a running msc_process stops at its next batch boundary. */
int msc_terminate(msc_handle* h);

/* Writes the accumulated image: ".exr" gives RGBA half-float OpenEXR with alpha 1 as the
 * reference's batch mode writes it (src/main.cpp:199-213); ".pfm" a float portable map.
 * divide_by_iterations != 0 writes pixels / iteration (the display scaling of main.cpp:169-174). */
int msc_save_image(msc_handle* h, const char* path, int divide_by_iterations);

/* Host-only form of the writer above for any row-major RGB float image. */
int msc_write_image_file(const char* path, int width, int height, const float* rgb);

/* Message of the last failing call on this handle (or of the last failed msc_create when h is NULL). */
const char* msc_last_error(msc_handle* h);

/* ---- introspection (no reference counterpart beyond the batch loop's stdout progress,
 *      src/core/Pathtracer.cpp:435-438,453) ---- */
typedef struct msc_stats {
  uint64_t closest_queries;   /* closest-hit ray queries in the last process() */
  uint64_t shadow_queries;    /* occlusion ray queries in the last process() */
  uint64_t batches;           /* ray batches processed */
  uint64_t kernel_launches;   /* kernels enqueued by the last process() */
  double process_ms;          /* device time of the last process(), CUDA events */
  double stage_ms[12];        /* per-stage device time when profiling is on (see MSC_STAGE_*) */
  uint64_t stage_launches[12];
  int width, height, spp, triangles, lights, iteration;
  double load_ms;             /* msc_create: host wall time of the YAML + OBJ parse */
  double bvh_ms;              /* msc_create: host wall time of the device BVH build and scene upload */
  double gpu_busy_ms;         /* device time of the enqueued work between host waits (the rest of the
                                 wall time the GPU sat idle waiting for the host) */
} msc_stats;

enum {
  MSC_STAGE_RAYGEN = 0, MSC_STAGE_BINS = 1, MSC_STAGE_RAYKEYS = 2, MSC_STAGE_RAYSORT = 3,
  MSC_STAGE_GATHER = 4, MSC_STAGE_TRACE = 5, MSC_STAGE_HITSORT = 6, MSC_STAGE_SHADE = 7,
  MSC_STAGE_SHADOW = 8, MSC_STAGE_FILTER = 9, MSC_STAGE_OTHER = 10, MSC_STAGE_COUNT = 11
};

int msc_get_stats(msc_handle* h, msc_stats* out);
/* 1: bracket every stage with CUDA events (adds host syncs; for measurement runs only). */
int msc_set_profiling(msc_handle* h, int on);

/* Per-sample radiance and film position of the last iteration (Image::samples,
 * include/core/Image.h:15-19): rgb gets 3*N floats, xy 2*N floats, N = W*H*spp,
 * in sampleID order x*H*spp + y*spp + i. */
int msc_get_samples(msc_handle* h, float* rgb, float* xy);

/* ---- stage entry points on host arrays (one call = upload, kernel, download) ---- */

/* Cardinal direction bin of each direction (src/core/Camera.cpp:42-44,
 * src/core/Integrator.cpp:240-242).  dirs: 3*n floats. */
int msc_stage_cardinal(const float* dirs, int n, int32_t* bins);

/* Stable partition of rays into the six cardinal bins (DirectionalBins::add,
 * src/core/DirectionalBins.cpp:37-73).  rays: 12 floats per ray
 * (org.xyz, lastPdf, dir.xyz, depth-as-int, weight.rgb, sampleID-as-int);
 * a ray whose depth word is negative is dropped.  out: 6*cap*12 floats,
 * bin b at [b*cap, (b+1)*cap); counts: 6 ints. */
int msc_stage_bin_partition(const float* rays, int n, int cap, float* out, int32_t* counts);
/* The same stable partition into 6, 26 or 98 direction bins (out holds
 * nbins * cap rays; counts: nbins ints).  26/98 bins have no reference
 * counterpart: they are the surface cells of a 3^3 / 5^3 direction cube. */
int msc_stage_bin_partition_n(const float* rays, int n, int nbins, int cap, float* out, int32_t* counts);
/* Direction bin of each of n directions (3 floats each) among 6, 26 or 98. */
int msc_stage_ray_bins(const float* dirs, int n, int nbins, int32_t* bins);

/* 32-bit ray sort keys in the origin box of the given rays (replaces the
 * median split of RaySort, src/core/RaySort.cpp:7-118). org, dir: 3*n floats. */
int msc_stage_ray_keys(const float* org, const float* dir, int n, uint32_t* keys);

/* Stable LSD radix sort of (keys, vals) on bits [0, bits); sorted in place. */
int msc_sort_pairs(uint32_t* keys, uint32_t* vals, int n, int bits);
/* The same with 4-, 8- or 11-bit digits (the autotuner's digit widths). */
int msc_stage_sort_pairs_digits(uint32_t* keys, uint32_t* vals, int n, int bits, int digit_bits);

/* The stable order of 64-bit keys as the hit sort takes it for a 64-bit hit
 * key (stable by the low word, then stably by the high word): perm[i] = index
 * of the i-th smallest key.  No reference counterpart: the reference sorts
 * hits by (geomID, primID) with tbb::parallel_sort (Pathtracer.cpp:335-339). */
int msc_stage_sort_keys64(const uint64_t* keys, int n, uint32_t* perm);

/* Test hook of the sort's bounded waits (no reference counterpart): sorts host
 * arrays on the device with the look-back spin cap set to spin_cap; with
 * withhold_first_tile != 0 the first tile never posts its digit counts, so every
 * later tile's look-back gives up after spin_cap rounds.  Returns MSC_ERR_DEVICE
 * (message in msc_last_error(NULL)) when a wait ran out; the output pairs are then
 * not sorted.  Every wait is bounded, so the call always returns. */
int msc_stage_sort_lookback_check(uint32_t* keys, uint32_t* vals, int n, int bits, int spin_cap,
                                  int withhold_first_tile);

/* Device-pointer form of msc_sort_pairs on the given CUDA stream (0 = default).
 * Scratch is allocated per call.  A look-back wait that runs out of its spin cap
 * (which only a scheduling failure of the GPU could cause) is not reported by
 * this form; msc_stage_sort_lookback_check shows the cap at work. */
int msc_sort_pairs_device(uint32_t* keys, uint32_t* vals, int n, int bits, void* stream);

/* Same sort as msc_sort_pairs_device (a look-back time-out is likewise not reported),
 * for callers that cannot allocate device memory
 * while they run (a host that reserves its whole device budget up front, or a
 * latency-critical loop that cannot take cudaFree's device synchronisation).
 * No counterpart in the reference.  Allocates nothing: its scratch is a static
 * device array sized for at most 1,048,576 pairs, held by every GPU that loads
 * the library; larger n returns MSC_ERR_ARG with a message in msc_last_error(NULL).
 * The first call on a device looks up that array's address (make it before any
 * stream capture); calls that overlap on the GPU share the array and race. */
int msc_sort_pairs_device_noalloc(uint32_t* keys, uint32_t* vals, int n, int bits, void* stream);

/* Closest hit against the handle's scene (rtcIntersect, src/core/RayIntersect.cpp:7-12)
 * on [0.001, 1e5].  geom/prim are the reference's geomID/primID, -1 for a miss. */
int msc_trace_closest(msc_handle* h, const float* org, const float* dir, int n, float* t, float* u, float* v,
                      int32_t* geom, int32_t* prim);

/* Occlusion against non-emitter geometry on (0.001, tmax) (rtcOccluded with mask
 * 0x0FFFFFFF, src/core/Integrator.cpp:153-174).  occluded[i] = 1 when blocked. */
int msc_trace_occluded(msc_handle* h, const float* org, const float* dir, const float* tmax, int n,
                       int32_t* occluded);

/* ---- batched form: many resident scenes and jobs in one wavefront ----
 * No counterpart in the reference, which renders one scene per process.  A
 * job is a resident scene seen through one camera at one resolution and
 * sample count; the rays of all submitted jobs share bins, sorted batches and
 * kernels.  Each job's image equals the image it gets when rendered alone. */
typedef struct msc_batch msc_batch;

typedef struct msc_job_desc {
  int scene;                  /* id from msc_batch_add_scene */
  int width, height, spp;     /* 0: the scene's own (spp other than base^2 allowed) */
  int min_depth, max_depth;   /* -1: the scene's own */
  int use_camera;             /* 1: the pinhole camera below replaces the scene's */
  float translation[3], rotation[3], focal_length;  /* PinHoleCamera fields (PinHoleCamera.h:98-113) */
  uint32_t seed;              /* 0: the scene's */
} msc_job_desc;

/* batch_exponent: rays per sorted batch (2^e); film_samples: capacity of the
 * shared per-sample film (sum of width*height*spp over jobs in flight). */
int msc_batch_create(int batch_exponent, int64_t film_samples, msc_batch** out);
int msc_batch_destroy(msc_batch* b);
const char* msc_batch_last_error(msc_batch* b);
int msc_batch_add_scene(msc_batch* b, const char* yaml_path, int* scene_id);
/* The resident scene's triangle box (lo.xyz, hi.xyz) and triangle count, for
   placing job cameras.  No reference counterpart. */
int msc_batch_scene_info(msc_batch* b, int scene, float lo[3], float hi[3], int64_t* triangles);
/* MSC_ERR_BUSY when the job's film does not fit in the free film capacity, or
 * its image does not fit in the device-memory budget. */
int msc_batch_submit(msc_batch* b, const msc_job_desc* desc, int* job_id);
/* A device-memory budget in bytes for the batch object (0, the default: none).
 * What counts: the fixed buffers taken at msc_batch_create (film pool, ray
 * pools, batch buffers), every resident scene (BVH, triangles, tables, texels,
 * as measured when it was built) and the images of admitted jobs.
 * msc_batch_add_scene returns MSC_ERR_BUSY when a scene (estimated before it is
 * built) would not fit; msc_batch_submit and the served form's admission treat
 * a job whose image would not fit like a full film pool.  No reference
 * counterpart. */
int msc_batch_set_memory_budget(msc_batch* b, int64_t bytes);
/* Bytes counted against the budget: all of them, the fixed buffers and
 * scenes, and the admitted jobs' images (any pointer may be NULL). */
int msc_batch_memory(msc_batch* b, int64_t* in_use, int64_t* fixed_bytes, int64_t* job_bytes);
/* The batch loop's tuning point.  No choice changes a result. */
typedef struct msc_tuning {
  int batch_exponent; /* rays per batch = 2^batch_exponent (at most the capacity given at create) */
  int trace_block;    /* traversal block size: 64, 128 or 256 */
  int ray_sort;       /* 1: each batch sorted on the origin/direction key (RaySort.cpp:7-118) */
  int hit_sort;       /* 1: each batch's hits sorted by (geomID, primID) (Pathtracer.cpp:335-339) */
  int bins;           /* direction bins: 6 (DirectionalBins.cpp:37-115) or 26 / 98 (cube surface cells) */
  int persistent;     /* 1: persistent traversal kernels with per-lane ray refill (8-wide BVH) */
  int digit_bits;     /* radix sort digit width: 4, 8 or 11 */
  int tuning;         /* read only: 1 while the autotuner is still sampling */
  int samples;        /* read only: candidate samples booked by the autotuner */
  int ray_key_bits;   /* top bits of the 32-bit ray key that the ray sort orders: 8, 16, 24 or 32;
                         0 = 16 for one scene, 24 (scene and bin above the key) for several */
} msc_tuning;
typedef struct msc_tune_sample {
  int batch_exponent, trace_block, ray_sort, hit_sort, bins, persistent, digit_bits;
  double mrays_per_s; /* device-timed rays per second over the candidate's windows */
  int ray_key_bits;   /* 0: the default width */
} msc_tune_sample;
/* Starts the online autotuner: each following msc_batch_run (each pass of
   the plain engine) renders with the next candidate choice (direction bins,
   traversal block and form, sort digit width, the two sorts) and is timed;
   every candidate gets `windows` runs (0: 1), and the fastest is kept.  No reference
   counterpart. */
int msc_batch_autotune(msc_batch* b, int windows);
int msc_batch_get_tuning(msc_batch* b, msc_tuning* out);
/* The plain engine's tuning point (it tunes itself during its first passes
   unless the scene's extensions say `autotune: 0`). */
int msc_get_tuning(msc_handle* h, msc_tuning* out);
/* Applies a tuning point to the plain engine (stops its autotuner). */
int msc_set_tuning(msc_handle* h, const msc_tuning* in);
/* Applies a choice (the read-only fields are ignored); stops a running autotuner. */
int msc_batch_set_tuning(msc_batch* b, const msc_tuning* in);
/* The autotuner's booked samples, at most cap; *n = how many exist. */
int msc_batch_tune_log(msc_batch* b, msc_tune_sample* out, int cap, int* n);
/* Renders every submitted job to completion in one merged wavefront. */
int msc_batch_run(msc_batch* b);
int msc_batch_job_image(msc_batch* b, int job, const float** rgb, int* width, int* height);
/* Frees a finished job's film for new submissions. */
int msc_batch_release_job(msc_batch* b, int job);
int msc_batch_get_stats(msc_batch* b, msc_stats* out);
int msc_batch_set_profiling(msc_batch* b, int on);
/* At most n jobs admitted at once (0 = no limit).  n = 1 renders one job at a
 * time: the plain per-job loop the batched and served forms are compared with. */
int msc_batch_set_max_active(msc_batch* b, int n);

/* ---- served form: requests admitted as they arrive and as film frees up ---- */
typedef struct msc_request {
  double arrival_s;           /* seconds after the call starts */
  msc_job_desc job;
} msc_request;

typedef struct msc_request_result {
  int job_id;
  int status;                 /* 0 done, negative: the submit error */
  double admit_s, done_s, latency_s;  /* latency = done - arrival */
} msc_request_result;

typedef struct msc_serve_stats {
  int completed;
  double wall_s, p50_s, p99_s, p999_s, mrays_per_s;
  uint64_t closest_queries, shadow_queries;
  int64_t peak_film_samples;
  double gpu_busy_s;          /* device time of the enqueued work between host waits */
  int not_admitted;           /* requests still waiting when admission closed (msc_serve_window) */
} msc_serve_stats;

/* Runs the request stream in real time on the batch object's resident scenes:
 * arrived requests are admitted in arrival order whenever their film fits;
 * admitted jobs share the wavefront; a finished job's image is copied to the
 * host and its film released.  Images stay readable with msc_batch_job_image. */
int msc_serve(msc_batch* b, const msc_request* reqs, int n, msc_request_result* results, msc_serve_stats* stats);

/* msc_serve with admission open only for window_s seconds: requests that have
 * not been admitted by then are not served (status MSC_ERR_BUSY, counted in
 * stats->not_admitted); the admitted ones run to completion.  Measures an
 * overloaded request stream over a fixed window. */
int msc_serve_window(msc_batch* b, const msc_request* reqs, int n, double window_s, msc_request_result* results,
                     msc_serve_stats* stats);

/* ---- host-only scene input (no GPU needed) ---- */

/* OBJ reading with tinyobjloader's rules (thirdparty/tinyobjloader/tiny_obj_loader.cpp:309-412,
 * 643-891, as PolygonObject::construct calls it, src/core/PolygonObject.cpp:7-8).
 * sizes[0..2] = float count of positions, float count of texcoords, index count;
 * pass NULL arrays to query the sizes first. */
int msc_obj_load(const char* path, float* positions, float* texcoords, uint32_t* indices, int64_t* sizes);

/* Parses a scene YAML and its OBJ files on the host only (Pathtracer::construct,
 * src/core/Pathtracer.cpp:32-275).  info[0..7] = width, height, spp, triangles,
 * lights, shaders, geometries, camera type.  tri_v (9 floats per triangle, world
 * space, geomID order) and tri_geom may be NULL. */
int msc_scene_load_host(const char* yaml_path, int32_t* info, float* tri_v, int32_t* tri_geom);

/* Writes a seeded synthetic scene (YAML + OBJ files) into out_dir.
 * config 0: the Cornell-style box; config 1: the terrain + icospheres scene;
 * config 100: a tiny test scene.  scale in (0, 1] shrinks geometry, image and
 * sample counts for tests.  The YAML path is written to yaml_path (size cap). */
int msc_generate_scene(int config, uint32_t seed, double scale, const char* out_dir, char* yaml_path, int cap);

#ifdef __cplusplus
}
#endif

#endif /* MSC_GPU_H_ */
