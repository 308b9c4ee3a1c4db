// Render core: see core.h.  Restates Pathtracer::process
// (src/core/Pathtracer.cpp:425-493) as a device-resident wavefront over the
// rays of any number of jobs.
#include "core.h"

#include <algorithm>
#include <chrono>
#include <cstring>

namespace mscg {

namespace {

size_t al256(size_t x) { return (x + 255) & ~(size_t)255; }

struct Arena {  // one cudaMalloc carved into aligned pieces
  char* base = nullptr;
  size_t used = 0;
  template <class T>
  T* take(size_t count) {
    T* p = (T*)(base + used);
    used += al256(count * sizeof(T));
    return p;
  }
};

void grid_of(int spp, int base, bool square, int* gx, int* gy) {
  if (square) {
    *gx = base;
    *gy = base;
    return;
  }
  int a = 1;
  for (int d = 1; d * d <= spp; ++d)
    if (spp % d == 0) a = d;
  *gx = a;
  *gy = spp / a;
}

}  // namespace

#define CK(call)                                                   \
  do {                                                             \
    cudaError_t e_ = (call);                                       \
    if (e_ != cudaSuccess) {                                       \
      err = std::string(#call) + ": " + cudaGetErrorString(e_);    \
      return MSC_ERR_CUDA;                                         \
    }                                                              \
  } while (0)

SceneGPU::~SceneGPU() {
  bvh_free(&bvh);
  if (d_shaders) cudaFree(d_shaders);
  if (d_geoms) cudaFree(d_geoms);
  if (d_lights) cudaFree(d_lights);
}

JobRec job_record(const SceneDesc& d, const JobSpec& spec, int scene_id) {
  JobRec f;
  memset(&f, 0, sizeof(f));
  f.cam = d.camera;
  if (spec.use_camera) {
    f.cam.type = CAMERA_PINHOLE;
    f.cam.xf = make_tr_yxz(spec.cam_translation, spec.cam_rotation);
    normal_of_x_axis(f.cam.xf, f.cam.normal);
    for (int i = 0; i < 3; ++i) f.cam.translation[i] = spec.cam_translation[i];
    f.cam.focal_length = spec.cam_focal;
  }
  f.width = spec.width > 0 ? spec.width : d.width;
  f.height = spec.height > 0 ? spec.height : d.height;
  const bool own_spp = spec.spp <= 0;
  f.spp = own_spp ? d.spp() : spec.spp;
  const bool square = own_spp ? d.ext.spp == 0 : false;
  grid_of(f.spp, d.base, square, &f.grid_x, &f.grid_y);
  f.sampler = d.sampler;
  f.filter = d.filter;
  f.min_depth = spec.min_depth >= 0 ? spec.min_depth : d.settings.min_depth;
  f.max_depth = std::min(kMaxDepth - 1, spec.max_depth >= 0 ? spec.max_depth : d.settings.max_depth);
  f.threshold = d.settings.threshold;
  f.mis_power = d.ext.mis_power;
  const uint32_t seed = spec.seed ? spec.seed : d.ext.seed;
  f.iter_seed = iteration_seed(seed, (uint32_t)spec.iteration);
  f.scene = scene_id;
  return f;
}

Core::~Core() {
  if (stream_) cudaStreamSynchronize(stream_);
  for (auto& j : jobs_)
    if (j && j->d_pixels) cudaFree(j->d_pixels);
  scenes_.clear();
  if (arena_) cudaFree(arena_);
  if (d_scenes_) cudaFree(d_scenes_);
  if (d_jobs_) cudaFree(d_jobs_);
  if (d_job_done_) cudaFree(d_job_done_);
  if (film_.rgb) cudaFree(film_.rgb);
  if (film_.pos) cudaFree(film_.pos);
  if (h_scenes_) cudaFreeHost(h_scenes_);
  if (h_jobs_) cudaFreeHost(h_jobs_);
  if (h_job_done_) cudaFreeHost(h_job_done_);
  if (h_small_) cudaFreeHost(h_small_);
  if (h_counts_up_) cudaFreeHost(h_counts_up_);
  for (auto e : event_pool_) cudaEventDestroy(e);
  if (stream_) cudaStreamDestroy(stream_);
}

double Core::now() const {
  using namespace std::chrono;
  return duration<double>(steady_clock::now().time_since_epoch()).count();
}

int Core::init(int batch_exponent, int generation, size_t sample_capacity, bool wide) {
  wide_ = wide;
  batch_exponent = std::max(6, std::min(batch_exponent, 24));
  batch_cap_ = 1 << batch_exponent;
  generation_ = std::max(generation, batch_cap_);
  staging_cap_ = std::max(batch_cap_, std::min(generation_, 4 * batch_cap_));
  sample_cap_ = std::max<size_t>(sample_capacity, 1);
  if (sample_cap_ >= (1ull << 31)) {
    err = "the film pool holds at most 2^31 - 1 samples";
    return MSC_ERR_ARG;
  }
  CK(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
  CK(cudaMalloc(&d_scenes_, kMaxScenes * sizeof(SceneRec)));
  CK(cudaMallocHost(&h_scenes_, kMaxScenes * sizeof(SceneRec)));
  CK(cudaMalloc(&d_jobs_, (size_t)kMaxJobs * sizeof(JobRec)));
  CK(cudaMallocHost(&h_jobs_, (size_t)kMaxJobs * sizeof(JobRec)));
  CK(cudaMalloc(&d_job_done_, (size_t)kMaxJobs * sizeof(uint32_t)));
  CK(cudaMallocHost(&h_job_done_, (size_t)kMaxJobs * sizeof(uint32_t)));
  CK(cudaMemset(d_job_done_, 0, (size_t)kMaxJobs * sizeof(uint32_t)));
  CK(cudaMalloc(&film_.rgb, sample_cap_ * sizeof(float4)));
  CK(cudaMalloc(&film_.pos, sample_cap_ * sizeof(float2)));
  free_ranges_.assign(1, std::make_pair((size_t)0, sample_cap_));
  const int B = batch_cap_, G = generation_, S = staging_cap_;
  const int part_tiles = (std::max(S, B) + kPartTile - 1) / kPartTile;
  size_t bytes = 3 * al256((size_t)6 * G * sizeof(float4)) + 3 * al256((size_t)S * sizeof(float4)) +
                 3 * al256((size_t)B * sizeof(float4)) + 6 * al256((size_t)B * 4) + 2 * al256(8 * 4) +
                 sort_scratch_bytes(B) + al256((size_t)B * sizeof(float4)) + 3 * al256((size_t)B * sizeof(float4)) +
                 al256((size_t)kMaxBins * part_tiles * 4) + 4096;
  CK(cudaMalloc(&arena_, bytes));
  Arena A{arena_, 0};
  bins_.rays.o = A.take<float4>((size_t)6 * G);
  bins_.rays.d = A.take<float4>((size_t)6 * G);
  bins_.rays.w = A.take<float4>((size_t)6 * G);
  bins_.cap = G;
  staging_.o = A.take<float4>(S);
  staging_.d = A.take<float4>(S);
  staging_.w = A.take<float4>(S);
  batch_.o = A.take<float4>(B);
  batch_.d = A.take<float4>(B);
  batch_.w = A.take<float4>(B);
  keys_ = A.take<uint32_t>(B);
  keys_sorted_ = A.take<uint32_t>(B);
  perm_ = A.take<uint32_t>(B);
  hkeys_ = A.take<uint32_t>(B);
  hkeys_sorted_ = A.take<uint32_t>(B);
  hperm_ = A.take<uint32_t>(B);
  small_ = A.take<int>(8);
  box6_ = A.take<uint32_t>(8);
  sort_scratch_bind(&ss_, A.take<char>(sort_scratch_bytes(B)), B);
  hits_ = A.take<float4>(B);
  shadow_.o = A.take<float4>(B);
  shadow_.d = A.take<float4>(B);
  shadow_.c = A.take<float4>(B);
  bins_.tile_counts = A.take<uint32_t>((size_t)kMaxBins * part_tiles);
  bins_.max_tiles = part_tiles;
  bins_.count = small_;
  bins_.err = small_ + 7;
  if (A.used > bytes) {
    err = "internal: device arena overflow";
    return MSC_ERR_CUDA;
  }
  CK(cudaMemset(small_, 0, 8 * sizeof(int)));
  CK(cudaMallocHost(&h_small_, 8 * sizeof(int)));
  CK(cudaMallocHost(&h_counts_up_, 8 * sizeof(int)));
  return MSC_OK;
}

int Core::add_scene(const SceneDesc& d_in, int* id) {
  if ((int)scenes_.size() >= kMaxScenes) {
    err = "at most 256 resident scenes";
    return MSC_ERR_ARG;
  }
  std::unique_ptr<SceneGPU> sg(new SceneGPU());
  sg->desc = d_in;
  SceneDesc& d = sg->desc;
  std::vector<float> tv = d.tri_v;
  std::vector<int> tg = d.tri_geom;
  std::vector<uint8_t> tl = d.tri_is_light;
  std::vector<GeomRec> geoms = d.geoms;
  const int real_tris = (int)tg.size();
  while ((int)tg.size() < 2) {  // the LBVH needs two leaves: pad with a point triangle that no ray hits
    for (int k = 0; k < 9; ++k) tv.push_back(0.f);
    tg.push_back((int)geoms.size());
    tl.push_back(0);
  }
  if ((int)geoms.size() <= *std::max_element(tg.begin(), tg.end())) {
    GeomRec pad = {0, real_tris, 0, -1};
    if (d.shaders.empty()) {
      ShaderRec ns;
      memset(&ns, 0, sizeof(ns));
      ns.type = SHADER_NULL;
      ns.light = -1;
      d.shaders.push_back(ns);
    }
    geoms.push_back(pad);
  }
  const int T = (int)tg.size();
  float* d_v = nullptr;
  int* d_g = nullptr;
  uint8_t* d_l = nullptr;
  CK(cudaMalloc(&d_v, tv.size() * sizeof(float)));
  CK(cudaMalloc(&d_g, tg.size() * sizeof(int)));
  CK(cudaMalloc(&d_l, tl.size()));
  CK(cudaMemcpy(d_v, tv.data(), tv.size() * sizeof(float), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(d_g, tg.data(), tg.size() * sizeof(int), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(d_l, tl.data(), tl.size(), cudaMemcpyHostToDevice));
  std::string berr;
  int bl = bvh_build(d_v, d_g, d_l, T, wide_, &sg->bvh, stream_, &berr);
  cudaFree(d_v);
  cudaFree(d_g);
  cudaFree(d_l);
  if (bl < 0) {
    err = berr;
    return MSC_ERR_CUDA;
  }
  sg->h_tri_orig.resize(T);
  CK(cudaMemcpy(sg->h_tri_orig.data(), sg->bvh.tri_orig, T * sizeof(int), cudaMemcpyDeviceToHost));
  CK(cudaMalloc(&sg->d_shaders, std::max<size_t>(1, d.shaders.size()) * sizeof(ShaderRec)));
  CK(cudaMalloc(&sg->d_geoms, std::max<size_t>(1, geoms.size()) * sizeof(GeomRec)));
  CK(cudaMalloc(&sg->d_lights, std::max<size_t>(1, d.lights.size()) * sizeof(LightRec)));
  if (!d.shaders.empty())
    CK(cudaMemcpy(sg->d_shaders, d.shaders.data(), d.shaders.size() * sizeof(ShaderRec), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(sg->d_geoms, geoms.data(), geoms.size() * sizeof(GeomRec), cudaMemcpyHostToDevice));
  if (!d.lights.empty())
    CK(cudaMemcpy(sg->d_lights, d.lights.data(), d.lights.size() * sizeof(LightRec), cudaMemcpyHostToDevice));
  SceneRec& r = sg->rec;
  memset(&r, 0, sizeof(r));
  r.wnodes = sg->bvh.wnodes;
  r.nodes = sg->bvh.nodes;
  r.tris = sg->bvh.tris;
  r.tri_orig = sg->bvh.tri_orig;
  r.num_wnodes = sg->bvh.num_wnodes;
  r.num_tris = sg->bvh.num_tris;
  r.shaders = sg->d_shaders;
  r.geoms = sg->d_geoms;
  r.lights = sg->d_lights;
  r.num_lights = (int)d.lights.size();
  r.light_pick = r.num_lights > 0 ? 1.f / (float)r.num_lights : 0.f;
  r.tri_base = total_tris_;
  if ((uint64_t)total_tris_ + (uint64_t)T + 1 >= (1ull << 32)) {
    err = "too many triangles across resident scenes";
    return MSC_ERR_ARG;
  }
  total_tris_ += (uint32_t)T;
  hit_bits_ = 32 - __builtin_clz(total_tris_);  // keys lie in [0, total_tris_]
  const int sid = (int)scenes_.size();
  h_scenes_[sid] = r;
  CK(cudaMemcpy(d_scenes_ + sid, &h_scenes_[sid], sizeof(SceneRec), cudaMemcpyHostToDevice));
  scenes_.push_back(std::move(sg));
  *id = sid;
  return MSC_OK;
}

size_t Core::samples_free() const {
  size_t best = 0;
  for (auto& r : free_ranges_) best = std::max(best, r.second);
  return best;
}

bool Core::alloc_samples(size_t n, size_t* off) {
  for (size_t i = 0; i < free_ranges_.size(); ++i) {
    if (free_ranges_[i].second >= n) {
      *off = free_ranges_[i].first;
      free_ranges_[i].first += n;
      free_ranges_[i].second -= n;
      if (free_ranges_[i].second == 0) free_ranges_.erase(free_ranges_.begin() + i);
      return true;
    }
  }
  return false;
}

void Core::free_samples(size_t off, size_t n) {
  free_ranges_.push_back(std::make_pair(off, n));
  std::sort(free_ranges_.begin(), free_ranges_.end());
  std::vector<std::pair<size_t, size_t>> merged;
  for (auto& r : free_ranges_) {
    if (!merged.empty() && merged.back().first + merged.back().second == r.first) merged.back().second += r.second;
    else merged.push_back(r);
  }
  free_ranges_.swap(merged);
}

int Core::add_job(const JobSpec& spec, int* id) {
  if (spec.scene < 0 || spec.scene >= (int)scenes_.size()) {
    err = "job names a scene that is not resident";
    return MSC_ERR_ARG;
  }
  JobRec rec = job_record(scenes_[spec.scene]->desc, spec, spec.scene);
  if (rec.width <= 0 || rec.height <= 0 || rec.spp <= 0) {
    err = "job sizes must be positive";
    return MSC_ERR_ARG;
  }
  const uint64_t paths = (uint64_t)rec.width * rec.height * rec.spp;
  if (paths >= (1ull << 31)) {
    err = "width * height * samples must stay below 2^31";
    return MSC_ERR_ARG;
  }
  if (paths > sample_cap_) {  // would never fit: refuse rather than wait
    err = "the job needs more film samples than the film pool holds";
    return MSC_ERR_ARG;
  }
  if (max_active > 0) {
    int active = 0;
    for (auto& jp : jobs_)
      if (jp->slot >= 0 && !jp->complete) ++active;
    if (active >= max_active) {
      err = "the admitted-job limit is reached";
      return MSC_ERR_BUSY;
    }
  }
  int slot = -1;
  if (!free_slots_.empty()) {
    slot = free_slots_.back();
    free_slots_.pop_back();
  } else if (max_slot_ + 1 < kMaxJobs) {
    slot = max_slot_ + 1;
  } else {
    err = "too many jobs in flight";
    return MSC_ERR_BUSY;
  }
  size_t off = 0;
  if (!alloc_samples(paths, &off)) {
    free_slots_.push_back(slot);
    err = "the film pool has no room for this job yet";
    return MSC_ERR_BUSY;
  }
  std::unique_ptr<JobState> js(new JobState());
  const size_t px = (size_t)3 * rec.width * rec.height;
  if (cudaMallocAsync(&js->d_pixels, px * sizeof(float), stream_) != cudaSuccess) {
    free_samples(off, paths);
    free_slots_.push_back(slot);
    err = "out of device memory for the job image";
    return MSC_ERR_BUSY;
  }
  CK(cudaMemsetAsync(js->d_pixels, 0, px * sizeof(float), stream_));
  max_slot_ = std::max(max_slot_, slot);
  rec.sample_base = (uint32_t)off;
  rec.pixels = js->d_pixels;
  js->rec = rec;
  js->slot = slot;
  js->paths = paths;
  js->sample_off = off;
  js->sample_len = paths;
  js->t_submit = js->t_admit = now();
  h_jobs_[slot] = rec;
  CK(cudaMemcpyAsync(d_jobs_ + slot, &h_jobs_[slot], sizeof(JobRec), cudaMemcpyHostToDevice, stream_));
  CK(cudaMemsetAsync(d_job_done_ + slot, 0, sizeof(uint32_t), stream_));
  // the info word holds the slot; job ids index jobs_
  *id = (int)jobs_.size();
  jobs_.push_back(std::move(js));
  return MSC_OK;
}

int Core::restart_job(int id) {
  JobState* j = job(id);
  if (!j || !j->complete) {
    err = "restart of a job that is not complete";
    return MSC_ERR_ARG;
  }
  // the slot may have been freed when the job completed: take one again
  if (j->slot < 0) {
    if (!free_slots_.empty()) {
      j->slot = free_slots_.back();
      free_slots_.pop_back();
    } else if (max_slot_ + 1 < kMaxJobs) {
      j->slot = ++max_slot_;
    } else {
      err = "too many jobs in flight";
      return MSC_ERR_BUSY;
    }
  }
  j->generated = 0;
  j->done = 0;
  j->complete = false;
  j->image_on_host = false;
  j->t_admit = now();
  h_jobs_[j->slot] = j->rec;
  CK(cudaMemcpyAsync(d_jobs_ + j->slot, &h_jobs_[j->slot], sizeof(JobRec), cudaMemcpyHostToDevice, stream_));
  CK(cudaMemsetAsync(d_job_done_ + j->slot, 0, sizeof(uint32_t), stream_));
  return MSC_OK;
}

int Core::remove_job(int id) {
  JobState* j = job(id);
  if (!j) return MSC_ERR_ARG;
  if (!j->complete && j->generated > 0) {
    err = "a job with rays in flight cannot be removed";
    return MSC_ERR_BUSY;
  }
  if (j->d_pixels) cudaFreeAsync(j->d_pixels, stream_);
  j->d_pixels = nullptr;
  if (j->sample_len) free_samples(j->sample_off, j->sample_len);
  j->sample_len = 0;
  if (j->slot >= 0) free_slots_.push_back(j->slot);
  j->slot = -1;
  return MSC_OK;
}

cudaEvent_t Core::pool_event() {
  if (event_used_ == event_pool_.size()) {
    cudaEvent_t e;
    cudaEventCreate(&e);
    event_pool_.push_back(e);
  }
  return event_pool_[event_used_++];
}

struct StageClock {
  Core* c;
  int stage;
  cudaEvent_t a = nullptr;
  StageClock(Core* core, int s) : c(core), stage(s) {
    if (c->profiling) {
      a = c->pool_event();
      cudaEventRecord(a, c->stream_);
    }
  }
  void done(int launches) {
    c->stats.stage_launches[stage] += (uint64_t)launches;
    c->stats.launches += (uint64_t)launches;
    if (c->profiling) {
      cudaEvent_t b = c->pool_event();
      cudaEventRecord(b, c->stream_);
      c->stage_events_.push_back({stage, {a, b}});
    }
  }
};

void Core::harvest() {
  for (auto& se : stage_events_) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, se.second.first, se.second.second) == cudaSuccess) stats.stage_ms[se.first] += ms;
  }
  stage_events_.clear();
  event_used_ = 0;
}

int Core::finish_job(JobState& j) {
  {
    StageClock t(this, MSC_STAGE_FILTER);
    t.done(launch_filter(j.rec, film_, stream_));
  }
  j.complete = true;
  j.t_done = now();
  return MSC_OK;
}

int Core::copy_image(int id) {
  JobState* j = job(id);
  if (!j || !j->d_pixels) return MSC_ERR_ARG;
  j->h_pixels.resize((size_t)3 * j->rec.width * j->rec.height);
  CK(cudaMemcpyAsync(j->h_pixels.data(), j->d_pixels, j->h_pixels.size() * sizeof(float), cudaMemcpyDeviceToHost,
                     stream_));
  CK(cudaStreamSynchronize(stream_));
  j->image_on_host = true;
  return MSC_OK;
}

// Camera rays of admitted jobs (in submission order) while fewer than one
// generation of paths is in flight, partitioned into the bins.
int Core::generate(bool* did) {
  *did = false;
  uint64_t inflight = 0;
  bool pending = false;
  for (auto& jp : jobs_) {
    JobState& j = *jp;
    if (j.slot < 0 || j.complete) continue;
    inflight += j.generated - j.done;
    if (j.generated < j.paths) pending = true;
  }
  if (!pending) return MSC_OK;
  const uint64_t room = (uint64_t)generation_ > inflight ? (uint64_t)generation_ - inflight : 0;
  // top up in pieces of at least one batch (or whatever is left)
  uint64_t left_total = 0;
  for (auto& jp : jobs_)
    if (jp->slot >= 0 && !jp->complete) left_total += jp->paths - jp->generated;
  const uint64_t want = std::min<uint64_t>((uint64_t)staging_cap_, room);
  if (want < std::min<uint64_t>((uint64_t)batch_cap_, left_total)) return MSC_OK;
  uint64_t filled = 0;
  StageClock t(this, MSC_STAGE_RAYGEN);
  int launches = 0;
  for (auto& jp : jobs_) {
    JobState& j = *jp;
    if (j.slot < 0 || j.complete || j.generated >= j.paths) continue;
    const uint64_t n = std::min<uint64_t>(want - filled, j.paths - j.generated);
    if (n == 0) break;
    RayBuf out{staging_.o + filled, staging_.d + filled, staging_.w + filled};
    launches += launch_raygen(j.rec, j.slot, (uint32_t)j.generated, (int)n, out, film_, stream_);
    j.generated += n;
    filled += n;
    if (filled >= want) break;
  }
  t.done(launches);
  if (filled > 0) {
    StageClock tb(this, MSC_STAGE_BINS);
    tb.done(launch_bin_partition(staging_, (int)filled, bins_, stream_));
    stats.generations += 1;
    *did = true;
  }
  return MSC_OK;
}

int Core::run_batch(const Segments& seg, int nb, int prefix_bits) {
  cudaStream_t st = stream_;
  const SceneRec& s0 = scenes_[0]->rec;
  const int ns = (int)scenes_.size();
  const uint32_t* perm = nullptr;
  if (ray_sort) {
    {
      StageClock t(this, MSC_STAGE_RAYKEYS);
      cudaMemsetAsync(box6_, 0xff, 12, st);
      cudaMemsetAsync(box6_ + 3, 0x00, 12, st);
      int l = launch_origin_box(bins_.rays.o, seg, box6_, st);
      l += launch_ray_keys(bins_.rays.o, bins_.rays.d, seg, box6_, prefix_bits, keys_, st);
      t.done(l);
    }
    StageClock t(this, MSC_STAGE_RAYSORT);
    t.done(sort_pairs(keys_, nullptr, keys_sorted_, perm_, nb, 32, ss_, st, small_ + 7));
    perm = perm_;
  }
  {
    StageClock t(this, MSC_STAGE_GATHER);
    t.done(launch_gather(bins_.rays, seg, perm, batch_, st));
  }
  {
    StageClock t(this, MSC_STAGE_TRACE);
    t.done(launch_trace_closest(d_scenes_, ns, s0, batch_.o, batch_.d, nb, hits_, small_ + 7, st));
  }
  const uint32_t* order = nullptr;
  if (hit_sort) {
    StageClock t(this, MSC_STAGE_HITSORT);
    int l = launch_hit_keys(d_scenes_, batch_.d, hits_, nb, hkeys_, st);
    l += sort_pairs(hkeys_, nullptr, hkeys_sorted_, hperm_, nb, hit_bits_, ss_, st, small_ + 7);
    t.done(l);
    order = hperm_;
  }
  {
    StageClock t(this, MSC_STAGE_SHADE);
    cudaMemsetAsync(small_ + 6, 0, sizeof(int), st);
    t.done(launch_shade(d_scenes_, d_jobs_, film_, batch_, hits_, order, nb, staging_, shadow_, small_ + 6,
                        d_job_done_, st));
  }
  {
    StageClock t(this, MSC_STAGE_SHADOW);
    t.done(launch_trace_shadow(d_scenes_, ns, s0, shadow_, small_ + 6, nb, film_.rgb, small_ + 7, st));
  }
  {
    StageClock t(this, MSC_STAGE_BINS);
    t.done(launch_bin_partition(staging_, nb, bins_, st));
  }
  return MSC_OK;
}

int Core::step(bool* idle) {
  *idle = false;
  cudaStream_t st = stream_;
  CK(cudaMemcpyAsync(h_small_, small_, 8 * sizeof(int), cudaMemcpyDeviceToHost, st));
  if (max_slot_ >= 0)
    CK(cudaMemcpyAsync(h_job_done_, d_job_done_, (size_t)(max_slot_ + 1) * sizeof(uint32_t), cudaMemcpyDeviceToHost,
                       st));
  CK(cudaStreamSynchronize(st));
  if (profiling) harvest();
  if (last_was_batch_) stats.shadow += (uint64_t)h_small_[6];
  last_was_batch_ = false;
  if (h_small_[7] != 0) {
    const int e = h_small_[7];
    err = (e & ERR_BIN_OVERFLOW)    ? "a direction bin overflowed"
          : (e & ERR_TRAVERSAL_CAP) ? "BVH traversal exceeded its step cap"
          : (e & kSortErrLookback)  ? "radix sort look-back exceeded its spin cap"
          : (e & ERR_BVH_INDEX)     ? "BVH traversal met an out-of-range node or triangle index"
                                    : "BVH traversal stack overflowed";
    return MSC_ERR_DEVICE;
  }
  // jobs whose paths have all ended
  for (auto& jp : jobs_) {
    JobState& j = *jp;
    if (j.slot < 0 || j.complete) continue;
    j.done = h_job_done_[j.slot];
    if (j.generated == j.paths && j.done == j.paths) {
      int rc = finish_job(j);
      if (rc != MSC_OK) return rc;
    }
  }
  bool did = false;
  int rc = generate(&did);
  if (rc != MSC_OK) return rc;
  if (did) return MSC_OK;
  // the next batch: the top of the fullest bin, topped up from the next
  // fullest when merging is on and the fullest is short
  int order[6] = {0, 1, 2, 3, 4, 5};
  std::stable_sort(order, order + 6, [&](int a, int b) { return h_small_[a] > h_small_[b]; });
  if (h_small_[order[0]] == 0) {
    *idle = true;
    return MSC_OK;
  }
  Segments seg;
  memset(&seg, 0, sizeof(seg));
  int nb = 0;
  for (int k = 0; k < 6 && nb < batch_cap_; ++k) {
    const int b = order[k];
    const int cnt = h_small_[b];
    if (cnt == 0) break;
    if (k > 0 && !merge_bins) break;
    const int take = std::min(batch_cap_ - nb, cnt);
    seg.start[seg.count] = b * generation_ + cnt - take;
    seg.prefix[seg.count] = nb;
    seg.count += 1;
    nb += take;
    h_small_[b] = cnt - take;
  }
  seg.prefix[seg.count] = nb;
  for (int k = 0; k < 6; ++k) h_counts_up_[k] = h_small_[k];
  CK(cudaMemcpyAsync(small_, h_counts_up_, 6 * sizeof(int), cudaMemcpyHostToDevice, st));
  int scene_bits = 0;
  while ((1 << scene_bits) < (int)scenes_.size()) ++scene_bits;
  const int prefix_bits = (seg.count > 1 || scene_bits > 0) ? scene_bits + 3 : 0;
  rc = run_batch(seg, nb, prefix_bits);
  if (rc != MSC_OK) return rc;
  stats.closest += (uint64_t)nb;
  stats.batches += 1;
  last_was_batch_ = true;
  return MSC_OK;
}

int Core::run_all(const volatile bool* stop) {
  while (true) {
    if (stop && *stop) return MSC_OK;
    bool idle = false;
    int rc = step(&idle);
    if (rc != MSC_OK) return rc;
    if (idle) {
      bool open = false;
      for (auto& jp : jobs_)
        if (jp->slot >= 0 && !jp->complete) open = true;
      if (!open) break;
    }
  }
  CK(cudaStreamSynchronize(stream_));
  CK(cudaGetLastError());
  return MSC_OK;
}

int Core::trace_closest(const float* org, const float* dir, int n, float4* hits_host) {
  std::vector<float4> o((size_t)n), d((size_t)n);
  for (int i = 0; i < n; ++i) {
    o[i] = make_float4(org[3 * i], org[3 * i + 1], org[3 * i + 2], 0.f);
    d[i] = make_float4(dir[3 * i], dir[3 * i + 1], dir[3 * i + 2], 0.f);  // info 0: scene 0
  }
  float4 *dev = nullptr;
  int* e = nullptr;
  CK(cudaMalloc(&dev, (size_t)n * 3 * sizeof(float4)));
  CK(cudaMalloc(&e, sizeof(int)));
  CK(cudaMemset(e, 0, sizeof(int)));
  CK(cudaMemcpy(dev, o.data(), (size_t)n * sizeof(float4), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(dev + n, d.data(), (size_t)n * sizeof(float4), cudaMemcpyHostToDevice));
  launch_trace_closest(d_scenes_, 1, scenes_[0]->rec, dev, dev + n, n, dev + 2 * n, e, 0);
  int he = 0;
  CK(cudaMemcpy(hits_host, dev + 2 * n, (size_t)n * sizeof(float4), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(&he, e, sizeof(int), cudaMemcpyDeviceToHost));
  cudaFree(dev);
  cudaFree(e);
  if (he != 0) {
    err = "BVH traversal reported an error";
    return MSC_ERR_DEVICE;
  }
  return MSC_OK;
}

int Core::trace_occluded(const float* org, const float* dir, const float* tmax, int n, int* occluded) {
  std::vector<float4> o((size_t)n), d((size_t)n);
  for (int i = 0; i < n; ++i) {
    o[i] = make_float4(org[3 * i], org[3 * i + 1], org[3 * i + 2], tmax[i]);
    d[i] = make_float4(dir[3 * i], dir[3 * i + 1], dir[3 * i + 2], 0.f);
  }
  float4* dev = nullptr;
  int* res = nullptr;
  CK(cudaMalloc(&dev, (size_t)n * 2 * sizeof(float4)));
  CK(cudaMalloc(&res, ((size_t)n + 1) * sizeof(int)));
  CK(cudaMemset(res + n, 0, sizeof(int)));
  CK(cudaMemcpy(dev, o.data(), (size_t)n * sizeof(float4), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(dev + n, d.data(), (size_t)n * sizeof(float4), cudaMemcpyHostToDevice));
  launch_occluded(scenes_[0]->rec, dev, dev + n, n, res, res + n, 0);
  int he = 0;
  CK(cudaMemcpy(occluded, res, (size_t)n * sizeof(int), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(&he, res + n, sizeof(int), cudaMemcpyDeviceToHost));
  cudaFree(dev);
  cudaFree(res);
  if (he != 0) {
    err = "BVH traversal reported an error";
    return MSC_ERR_DEVICE;
  }
  return MSC_OK;
}

}  // namespace mscg
