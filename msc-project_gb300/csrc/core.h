// The render core shared by the plain, batched and served forms.
//
// Resident scenes (BVH + tables) and jobs (a scene seen through one camera at
// one resolution and sample count) live in device tables.  The core runs one
// wavefront over the rays of every admitted job:
//   top up: camera rays of admitted jobs are generated while fewer than one
//           generation of paths is in flight, and partitioned into the six
//           cardinal bins (the reference's DirectionalBins)
//   batch:  up to 2^bin_exponent rays from the fullest bins -> origin box ->
//           ray keys -> radix sort -> gather -> closest hit -> hit keys ->
//           hit sort -> shade -> occlusion + accumulate -> partition into bins
//   finish: a job whose paths are all generated and ended is filtered into
//           its image (pixels += tent/box filter of its samples)
// step() performs one top-up or one batch; the drivers in engine.cu loop it.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <memory>
#include <string>
#include <vector>

#include "../../include/msc_gpu.h"
#include "bvh.h"
#include "radix.cuh"
#include "render.h"
#include "scene.h"

namespace mscg {

struct SceneGPU {
  SceneDesc desc;
  DeviceBvh bvh;
  ShaderRec* d_shaders = nullptr;
  GeomRec* d_geoms = nullptr;
  LightRec* d_lights = nullptr;
  float4* d_spheres = nullptr;        // sphere lights: centre, radius
  int* d_sphere_light = nullptr;
  unsigned short* d_texels = nullptr; // face texels (FP16 bits)
  TexNode* d_tex_nodes = nullptr;     // image textures
  int2* d_tex_ops = nullptr;
  int4* d_tex_images = nullptr;
  float4* d_tex_texels = nullptr;
  float* d_tri_uv = nullptr;
  uint32_t* d_shade_rank = nullptr;  // 64-bit hit key scenes: (shader, face) rank + 1 per leaf-order triangle
  std::vector<int> h_tri_orig;  // leaf order -> global triangle index
  int64_t bytes = 0;            // device bytes the resident scene holds
  SceneRec rec;
  ~SceneGPU();
};

struct JobSpec {          // what a caller asks for; the scene's own setup fills the rest
  int scene = 0;
  int width = 0, height = 0, spp = 0;  // 0: the scene's
  int min_depth = -1, max_depth = -1;  // -1: the scene's
  int use_camera = 0;                  // 1: pinhole camera below instead of the scene's
  float cam_translation[3] = {0, 0, 0};
  float cam_rotation[3] = {0, 0, 0};
  float cam_focal = 0.f;
  uint32_t seed = 0;                   // 0: the scene's extension seed
  int iteration = 0;
};

struct JobState {
  JobRec rec;
  int slot = -1;
  uint64_t paths = 0, generated = 0, done = 0;
  size_t sample_off = 0, sample_len = 0;
  float* d_pixels = nullptr;
  std::vector<float> h_pixels;
  bool complete = false;
  bool image_on_host = false;
  double t_submit = 0, t_admit = 0, t_done = 0;
};

// One point of the tuning space of the batch loop.  None of these changes a
// result: every path draws its own random sequence and adds to its own sample
// in bounce order, whatever batch it rides in.
struct TuneChoice {
  int batch_exp = 20;   // rays per batch = 2^batch_exp (at most the allocated capacity)
  int block = 128;      // traversal block size: 64, 128 or 256
  bool ray_sort = true; // origin/direction key sort of each batch
  bool hit_sort = true; // (geomID, primID) sort of each batch's hits
  int bins = 6;         // direction bins: 6, 26 or 98
  bool persistent = false;  // persistent traversal with per-lane ray refill
  int digit_bits = 8;       // radix sort digit width: 4, 8 or 11
  int ray_key_bits = 0;     // top bits of the ray key sorted: 16, 24 or 32 (0: 16, or 24 with several scenes)
};

struct TuneSample {
  TuneChoice choice;
  double rays = 0, ms = 0;  // rays traced and device time over the sample windows
};

struct CoreStats {
  uint64_t closest = 0, shadow = 0, batches = 0, launches = 0, generations = 0, graph_replays = 0;
  double busy_ms = 0;  // device time from the first enqueue after a host wait to the next host wait
  double stage_ms[12] = {0};
  uint64_t stage_launches[12] = {0};
};

class Core {
 public:
  std::string err;
  CoreStats stats;
  bool profiling = false;
  bool ray_sort = true, hit_sort = true;
  bool merge_bins = true;  // let a batch take rays of several bins when the fullest is short
  int max_active = 0;      // jobs admitted at once (0 = no limit); 1 gives the one-job-at-a-time loop
  // Device-memory budget (0: none): the fixed buffers and the resident scenes
  // (mem_fixed) plus the admitted jobs' images (mem_jobs) must stay within it.
  int64_t mem_budget = 0, mem_fixed = 0, mem_jobs = 0;
  bool use_graph = true;   // replay the batch body from a captured CUDA graph (eager launches when profiling)
  int max_batches_per_step = 16;  // batch bodies enqueued between two host looks at the counters
  int trace_block = 128;          // traversal block size
  bool persistent_trace = false;  // persistent traversal kernels (8-wide BVH)
  int sort_digits = 8;            // radix sort digit width (4, 8 or 11)
  int ray_key_bits = 0;           // ray key bits sorted (0: the default for the scene count)

  // Online autotuner: while on, each run_all (a render pass or a batched
  // run) is one timed sample of the next candidate choice (coordinate
  // descent: direction bins, traversal block and form, sort digit width,
  // then the two sorts);
  // the fastest in rays per ms is kept.  Results are the same under any choice.
  void start_autotune(int runs_per_candidate = 1);
  void stop_autotune() { tune_active_ = false; }
  bool tuning() const { return tune_active_; }
  TuneChoice choice() const;
  void apply(const TuneChoice& c);
  std::vector<TuneSample> tune_log;

  ~Core();
  // batch_exponent: rays per batch (2^e); generation: paths in flight; samples: film capacity.
  int init(int batch_exponent, int generation, size_t sample_capacity, bool wide);
  int add_scene(const SceneDesc& d, int* id);
  int scene_bounds(int id, float lo[3], float hi[3]);  // the device BVH's root box
  // Admits a job if its film fits; returns MSC_ERR_BUSY when it does not (yet).
  int add_job(const JobSpec& spec, int* id);
  // Starts the next iteration of a finished job (same film, next random sequence).
  int restart_job(int id);
  int remove_job(int id);
  // One top-up or one batch; *idle = true when no work was left.
  int step(bool* idle);
  // Steps until every admitted job is complete (or `stop` becomes true).
  int run_all(const volatile bool* stop = nullptr);
  // Zeroes the statistics and the device ray counters (stream-ordered).
  void reset_stats();
  int copy_image(int id);
  cudaStream_t stream() const { return stream_; }
  JobState* job(int id) { return (id >= 0 && id < (int)jobs_.size()) ? jobs_[id].get() : nullptr; }
  SceneGPU* scene(int id) { return (id >= 0 && id < (int)scenes_.size()) ? scenes_[id].get() : nullptr; }
  int num_scenes() const { return (int)scenes_.size(); }
  size_t samples_free() const;
  size_t sample_capacity() const { return sample_cap_; }
  Film film() const { return film_; }
  int batch_cap() const { return batch_cap_; }
  int64_t scene_bytes(int id) const { return id >= 0 && id < (int)scenes_.size() ? scenes_[id]->bytes : 0; }
  int ray_key_bits_used() const;
  int batch_size() const { return batch_size_; }
  double now() const;
  // Host wait for the core's stream that keeps the busy accounting right.
  cudaError_t sync_stream();
  // Closest hit / occlusion of explicit rays against scene 0 (stage entry points).
  int trace_closest(const float* org, const float* dir, int n, float4* hits_host);
  int trace_occluded(const float* org, const float* dir, const float* tmax, int n, int* occluded);

 private:
  // One batch body: plan, sort, trace, shade, shadow, re-bin.  In a captured
  // graph of several bodies (`overlap`), body i's occlusion runs on the side
  // stream beside body i+1's plan, gather and closest-hit traversal; body
  // i+1's shading waits for it, so every path still adds to its sample in
  // bounce order.
  int enqueue_batch(int index, bool overlap);
  // k batch bodies (graph replays or eager); drain: the bins hold at most
  // kDrainBatch rays, so the smaller drain graph serves
  int run_batches(int k, bool drain = false);
  int ensure_graph();
  int capture_graph(cudaGraphExec_t* exec, uint64_t* exec_key, int* exec_launches);
  void drop_graph();
  int finish_job(JobState& j);
  int generate(bool* did);
  bool alloc_samples(size_t n, size_t* off);
  void free_samples(size_t off, size_t n);
  void harvest();

  cudaStream_t stream_ = nullptr;
  bool wide_ = true;
  int batch_cap_ = 0, generation_ = 0, staging_cap_ = 0;
  int batch_size_ = 0;  // rays per batch now (<= batch_cap_)
  // autotuner state
  bool tune_active_ = false;
  int tune_dim_ = 0, tune_windows_ = 2;
  std::vector<TuneSample> tune_cands_;
  int tune_next_ = 0;           // candidate of the next run
  cudaEvent_t tune_ev_[2] = {nullptr, nullptr};
  // GPU busy accounting: an event at the first enqueue after each host wait
  // and one before the next wait; the stretches between are the GPU's busy time
  cudaEvent_t busy_ev_[2] = {nullptr, nullptr};
  bool busy_open_ = false;
  void mark_busy();
  void close_busy();   // before a host wait on stream_
  void settle_busy();  // after it
  void tune_begin_dim();
  void tune_sample_done();
  std::vector<std::unique_ptr<SceneGPU>> scenes_;
  std::vector<std::unique_ptr<JobState>> jobs_;
  std::vector<int> free_slots_;
  int max_slot_ = -1;
  uint32_t total_tris_ = 0;
  int hit_bits_ = 1;
  SceneRec* d_scenes_ = nullptr;
  SceneRec* h_scenes_ = nullptr;  // pinned mirror
  JobRec* d_jobs_ = nullptr;
  JobRec* h_jobs_ = nullptr;      // pinned mirror
  uint32_t* d_job_done_ = nullptr;
  uint32_t* h_job_done_ = nullptr;
  // film pool
  Film film_;
  size_t sample_cap_ = 0;
  std::vector<std::pair<size_t, size_t>> free_ranges_;  // (offset, length), sorted
  // wavefront buffers
  char* arena_ = nullptr;
  BinPool bins_;
  RayBuf staging_;
  uint32_t *keys_ = nullptr, *keys_sorted_ = nullptr, *perm_ = nullptr, *hkeys_ = nullptr, *hkeys_sorted_ = nullptr,
           *hperm_ = nullptr, *hhi_ = nullptr, *hhi_g_ = nullptr, *hperm1_ = nullptr;
  SortScratch ss_;
  float4* hits_ = nullptr;
  int* slots_ = nullptr;  // pool index of each batch ray (sorted order)
  uint8_t* cam_digits_ = nullptr;  // direction bin of each camera ray of a top-up
  ShadowBuf shadow_[2];          // shadow queues, alternating between batches
  cudaStream_t side_ = nullptr;  // occlusion of batch k runs here beside batch k+1's front part
  static constexpr int kGraphBodies = 4;
  static constexpr int kDrainBatch = 1 << 20;  // batch capacity of the drain graph
  cudaEvent_t fork_ev_[kGraphBodies] = {}, join_ev_[kGraphBodies] = {};
  Counters* ctr_ = nullptr;    // device counters
  int* trace_counter_ = nullptr;  // ray counters of the persistent traversal (closest, shadow)
  Counters* h_ctr_ = nullptr;  // pinned copy
  BatchPlan* plan_ = nullptr;
  cudaGraphExec_t graph_ = nullptr;
  uint64_t graph_key_ = 0;
  cudaGraphExec_t drain_graph_ = nullptr;  // the bodies sized for kDrainBatch rays
  uint64_t drain_key_ = 0;
  int drain_launches_ = 0;
  int graph_launches_ = 0;     // kernels in one replay
  uint64_t graph_key() const;
  std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> stage_events_;
  std::vector<cudaEvent_t> event_pool_;
  size_t event_used_ = 0;
  friend struct StageClock;
  cudaEvent_t pool_event();
};

// Device job record for a scene's own setup document (PinHole/ThinLens camera,
// sampler, filter, depth limits) overridden by the spec.
JobRec job_record(const SceneDesc& d, const JobSpec& spec, int scene_id);

}  // namespace mscg
