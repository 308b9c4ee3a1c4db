// Render engine behind the C ABI of include/msc_gpu.h.
//
// msc_process() restates Pathtracer::process (src/core/Pathtracer.cpp:425-493)
// as a device-resident batch loop:
//   camera generation -> stable partition into the six cardinal bins
//   while any bin holds rays:
//     take up to 2^bin_exponent rays from the fullest bin (DirectionalBins::flush)
//     origin box -> 32-bit origin/direction key -> radix sort -> gather
//     closest-hit traversal -> (geomID, primID) hit sort -> shade
//     occlusion traversal + accumulate -> partition continuation rays into bins
//   tent (or box) filter: pixels += filtered samples
// The loop's only host synchronisation is the read-back of the per-bin counts
// that picks the next batch.  Paths are generated in bounded generations so the
// bins never hold more rays than one generation.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "../../include/msc_gpu.h"
#include "bvh.h"
#include "radix.cuh"
#include "render.h"
#include "scene.h"

namespace mscg {
bool generate_scene(int config, uint32_t seed, double scale, const std::string& dir, std::string* yaml,
                    std::string* err);
bool write_exr_rgba_half(const std::string& path, int w, int h, const float* rgb, std::string* err);
bool write_pfm(const std::string& path, int w, int h, const float* rgb, std::string* err);
}

using namespace mscg;

namespace {
thread_local std::string g_create_error;
}

namespace mscg {
// Message returned by msc_last_error(NULL) on this thread.
void set_global_error(const std::string& msg) { g_create_error = msg; }
}  // namespace mscg

namespace {

size_t al256(size_t x) { return (x + 255) & ~(size_t)255; }

struct DeviceArena {  // one cudaMalloc carved into aligned pieces
  char* base = nullptr;
  size_t size = 0, used = 0;
  template <class T>
  T* take(size_t count) {
    size_t b = al256(count * sizeof(T));
    T* p = (T*)(base + used);
    used += b;
    return p;
  }
};

}  // namespace

struct msc_handle {
  SceneDesc desc;
  std::string err;
  std::mutex busy;
  std::atomic<bool> terminate{false};
  cudaStream_t stream = nullptr;
  // scene on the device
  DeviceBvh bvh;
  ShaderRec* d_shaders = nullptr;
  GeomRec* d_geoms = nullptr;
  LightRec* d_lights = nullptr;
  std::vector<int> h_tri_orig;  // leaf order -> global triangle
  // sizes
  uint64_t paths = 0;  // W * H * spp
  int batch_cap = 0;   // 2^bin_exponent (capped)
  int generation = 0;  // paths per camera generation (= bin capacity)
  int hit_bits = 0;
  // buffers
  char* arena = nullptr;
  BinPool bins;
  RayBuf staging, batch;
  uint32_t *keys = nullptr, *keys_sorted = nullptr, *perm = nullptr, *hkeys = nullptr, *hkeys_sorted = nullptr,
           *hperm = nullptr;
  uint32_t* box6 = nullptr;
  SortScratch ss;
  float4* hits = nullptr;
  ShadowBuf shadow;
  int* small = nullptr;  // [0..5] bin counts, [6] shadow count, [7] error bits
  float4* sample_rgb = nullptr;
  float2* sample_pos = nullptr;
  float* d_pixels = nullptr;
  std::vector<float> h_pixels;
  bool host_stale = false;
  int* h_small = nullptr;     // pinned read-back
  int* h_counts_up = nullptr; // pinned upload
  int iteration = 0;
  // stats
  msc_stats stats;
  bool profiling = false;
  cudaEvent_t ev_begin = nullptr, ev_end = nullptr;
  std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> stage_events;
  std::vector<cudaEvent_t> event_pool;
  size_t event_used = 0;
};

namespace {

#define CK(call)                                                                      \
  do {                                                                                \
    cudaError_t e_ = (call);                                                          \
    if (e_ != cudaSuccess) {                                                          \
      h->err = std::string(#call) + ": " + cudaGetErrorString(e_);                    \
      return MSC_ERR_CUDA;                                                            \
    }                                                                                 \
  } while (0)

cudaEvent_t pool_event(msc_handle* h) {
  if (h->event_used == h->event_pool.size()) {
    cudaEvent_t e;
    cudaEventCreate(&e);
    h->event_pool.push_back(e);
  }
  return h->event_pool[h->event_used++];
}

struct StageTimer {
  msc_handle* h;
  int stage;
  cudaEvent_t a = nullptr;
  StageTimer(msc_handle* hh, int s) : h(hh), stage(s) {
    if (h->profiling) {
      a = pool_event(h);
      cudaEventRecord(a, h->stream);
    }
  }
  void done(int launches) {
    h->stats.stage_launches[stage] += (uint64_t)launches;
    h->stats.kernel_launches += (uint64_t)launches;
    if (h->profiling) {
      cudaEvent_t b = pool_event(h);
      cudaEventRecord(b, h->stream);
      h->stage_events.push_back({stage, {a, b}});
    }
  }
};

void harvest_stage_events(msc_handle* h) {
  for (auto& se : h->stage_events) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, se.second.first, se.second.second) == cudaSuccess) h->stats.stage_ms[se.first] += ms;
  }
  h->stage_events.clear();
  h->event_used = 0;
}

DevScene dev_scene(msc_handle* h) {
  DevScene s;
  s.nodes = h->bvh.nodes;
  s.wnodes = h->bvh.wnodes;
  s.num_wnodes = h->bvh.num_wnodes;
  s.tris = h->bvh.tris;
  s.tri_orig = h->bvh.tri_orig;
  s.num_tris = h->bvh.num_tris;
  s.shaders = h->d_shaders;
  s.geoms = h->d_geoms;
  s.lights = h->d_lights;
  s.num_lights = (int)h->desc.lights.size();
  s.light_pick = s.num_lights > 0 ? 1.f / (float)s.num_lights : 0.f;
  return s;
}

void grid_of(int spp, int base, bool square, int* gx, int* gy) {
  if (square) { *gx = base; *gy = base; return; }
  int a = 1;
  for (int d = 1; d * d <= spp; ++d)
    if (spp % d == 0) a = d;
  *gx = a;
  *gy = spp / a;
}

DevFrame dev_frame(msc_handle* h) {
  DevFrame f;
  const SceneDesc& d = h->desc;
  f.cam = d.camera;
  f.width = d.width;
  f.height = d.height;
  f.spp = d.spp();
  grid_of(f.spp, d.base, d.ext.spp == 0, &f.grid_x, &f.grid_y);
  f.sampler = d.sampler;
  f.min_depth = d.settings.min_depth;
  f.max_depth = d.settings.max_depth;
  f.threshold = d.settings.threshold;
  f.mis_power = d.ext.mis_power;
  f.iter_seed = iteration_seed(d.ext.seed, (uint32_t)h->iteration);
  f.sample_rgb = h->sample_rgb;
  f.sample_pos = h->sample_pos;
  return f;
}

int setup(msc_handle* h) {
  SceneDesc& d = h->desc;
  CK(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
  CK(cudaEventCreate(&h->ev_begin));
  CK(cudaEventCreate(&h->ev_end));
  // ---- scene tables
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
  int bl = bvh_build(d_v, d_g, d_l, T, d.ext.wide_bvh != 0, &h->bvh, h->stream, &berr);
  cudaFree(d_v);
  cudaFree(d_g);
  cudaFree(d_l);
  if (bl < 0) { h->err = berr; return MSC_ERR_CUDA; }
  h->h_tri_orig.resize(T);
  CK(cudaMemcpy(h->h_tri_orig.data(), h->bvh.tri_orig, T * sizeof(int), cudaMemcpyDeviceToHost));
  CK(cudaMalloc(&h->d_shaders, std::max<size_t>(1, d.shaders.size()) * sizeof(ShaderRec)));
  CK(cudaMalloc(&h->d_geoms, std::max<size_t>(1, geoms.size()) * sizeof(GeomRec)));
  CK(cudaMalloc(&h->d_lights, std::max<size_t>(1, d.lights.size()) * sizeof(LightRec)));
  if (!d.shaders.empty()) CK(cudaMemcpy(h->d_shaders, d.shaders.data(), d.shaders.size() * sizeof(ShaderRec), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(h->d_geoms, geoms.data(), geoms.size() * sizeof(GeomRec), cudaMemcpyHostToDevice));
  if (!d.lights.empty()) CK(cudaMemcpy(h->d_lights, d.lights.data(), d.lights.size() * sizeof(LightRec), cudaMemcpyHostToDevice));
  h->hit_bits = 32 - __builtin_clz((unsigned)T);  // keys lie in [0, T]

  // ---- render buffers
  h->paths = (uint64_t)d.width * (uint64_t)d.height * (uint64_t)d.spp();
  if (h->paths >= (1ull << 31)) { h->err = "width * height * samples must stay below 2^31"; return MSC_ERR_ARG; }
  int e = std::min(d.settings.bin_exponent, 24);
  h->batch_cap = 1 << e;
  uint64_t gen = d.ext.generation > 0 ? (uint64_t)d.ext.generation : std::max<uint64_t>(4ull << e, 1ull << 22);
  gen = std::min<uint64_t>(gen, h->paths);
  gen = std::max<uint64_t>(gen, 1);
  h->generation = (int)gen;
  const int B = h->batch_cap, G = h->generation, S = std::max(G, B);
  const int part_tiles = (S + kPartTile - 1) / kPartTile;
  size_t bytes = 0;
  bytes += 3 * al256((size_t)6 * G * sizeof(float4));  // bins
  bytes += 3 * al256((size_t)S * sizeof(float4));      // staging
  bytes += 3 * al256((size_t)B * sizeof(float4));      // batch
  bytes += 6 * al256((size_t)B * 4);                   // keys
  bytes += al256(8 * 4) + al256(8 * 4);
  bytes += sort_scratch_bytes(B);
  bytes += al256((size_t)B * sizeof(float4));           // hits
  bytes += 3 * al256((size_t)B * sizeof(float4));       // shadow
  bytes += al256((size_t)kMaxBins * part_tiles * 4);    // partition tiles
  bytes += al256(h->paths * sizeof(float4)) + al256(h->paths * sizeof(float2));
  bytes += al256((size_t)3 * d.width * d.height * sizeof(float));
  bytes += 4096;
  CK(cudaMalloc(&h->arena, bytes));
  DeviceArena A{h->arena, bytes, 0};
  h->bins.rays.o = A.take<float4>((size_t)6 * G);
  h->bins.rays.d = A.take<float4>((size_t)6 * G);
  h->bins.rays.w = A.take<float4>((size_t)6 * G);
  h->bins.cap = G;
  h->staging.o = A.take<float4>(S);
  h->staging.d = A.take<float4>(S);
  h->staging.w = A.take<float4>(S);
  h->batch.o = A.take<float4>(B);
  h->batch.d = A.take<float4>(B);
  h->batch.w = A.take<float4>(B);
  h->keys = A.take<uint32_t>(B);
  h->keys_sorted = A.take<uint32_t>(B);
  h->perm = A.take<uint32_t>(B);
  h->hkeys = A.take<uint32_t>(B);
  h->hkeys_sorted = A.take<uint32_t>(B);
  h->hperm = A.take<uint32_t>(B);
  h->small = A.take<int>(8);
  h->box6 = A.take<uint32_t>(8);
  sort_scratch_bind(&h->ss, A.take<char>(sort_scratch_bytes(B)), B);
  h->hits = A.take<float4>(B);
  h->shadow.o = A.take<float4>(B);
  h->shadow.d = A.take<float4>(B);
  h->shadow.c = A.take<float4>(B);
  h->bins.tile_counts = A.take<uint32_t>((size_t)kMaxBins * part_tiles);
  h->bins.max_tiles = part_tiles;
  h->sample_rgb = A.take<float4>(h->paths);
  h->sample_pos = A.take<float2>(h->paths);
  h->d_pixels = A.take<float>((size_t)3 * d.width * d.height);
  h->bins.count = h->small;
  h->bins.err = h->small + 7;
  if (A.used > bytes) { h->err = "internal: device arena overflow"; return MSC_ERR_CUDA; }
  CK(cudaMemset(h->d_pixels, 0, (size_t)3 * d.width * d.height * sizeof(float)));
  CK(cudaMemset(h->small, 0, 8 * sizeof(int)));
  CK(cudaMallocHost(&h->h_small, 8 * sizeof(int)));
  CK(cudaMallocHost(&h->h_counts_up, 8 * sizeof(int)));
  h->h_pixels.assign((size_t)3 * d.width * d.height, 0.f);
  memset(&h->stats, 0, sizeof(h->stats));
  return MSC_OK;
}

void release(msc_handle* h) {
  if (h->stream) cudaStreamSynchronize(h->stream);
  bvh_free(&h->bvh);
  if (h->d_shaders) cudaFree(h->d_shaders);
  if (h->d_geoms) cudaFree(h->d_geoms);
  if (h->d_lights) cudaFree(h->d_lights);
  if (h->arena) cudaFree(h->arena);
  if (h->h_small) cudaFreeHost(h->h_small);
  if (h->h_counts_up) cudaFreeHost(h->h_counts_up);
  for (auto e : h->event_pool) cudaEventDestroy(e);
  if (h->ev_begin) cudaEventDestroy(h->ev_begin);
  if (h->ev_end) cudaEventDestroy(h->ev_end);
  if (h->stream) cudaStreamDestroy(h->stream);
}

// One batch of nb rays at bins[base, base+nb).
int run_batch(msc_handle* h, const DevScene& sc, const DevFrame& fr, int base, int nb) {
  cudaStream_t st = h->stream;
  RayBuf src{h->bins.rays.o + base, h->bins.rays.d + base, h->bins.rays.w + base};
  if (h->desc.ext.ray_sort) {
    {
      StageTimer t(h, MSC_STAGE_RAYKEYS);
      cudaMemsetAsync(h->box6, 0xff, 12, st);
      cudaMemsetAsync(h->box6 + 3, 0x00, 12, st);
      int l = launch_origin_box(src.o, nb, h->box6, st);
      l += launch_ray_keys(src.o, src.d, nb, h->box6, h->keys, st);
      t.done(l);
    }
    {
      StageTimer t(h, MSC_STAGE_RAYSORT);
      t.done(sort_pairs(h->keys, nullptr, h->keys_sorted, h->perm, nb, 32, h->ss, st, h->small + 7));
    }
    StageTimer t(h, MSC_STAGE_GATHER);
    t.done(launch_gather(src, h->perm, nb, h->batch, st));
  } else {
    StageTimer t(h, MSC_STAGE_GATHER);
    t.done(launch_gather(src, nullptr, nb, h->batch, st));
  }
  {
    StageTimer t(h, MSC_STAGE_TRACE);
    t.done(launch_trace_closest(sc, h->batch.o, h->batch.d, nb, h->hits, h->small + 7, st));
  }
  const uint32_t* order = nullptr;
  if (h->desc.ext.hit_sort) {
    StageTimer t(h, MSC_STAGE_HITSORT);
    int l = launch_hit_keys(sc, h->hits, nb, h->hkeys, st);
    l += sort_pairs(h->hkeys, nullptr, h->hkeys_sorted, h->hperm, nb, h->hit_bits, h->ss, st, h->small + 7);
    t.done(l);
    order = h->hperm;
  }
  {
    StageTimer t(h, MSC_STAGE_SHADE);
    cudaMemsetAsync(h->small + 6, 0, sizeof(int), st);
    t.done(launch_shade(sc, fr, h->batch, h->hits, order, nb, h->staging, h->shadow, h->small + 6, st));
  }
  {
    StageTimer t(h, MSC_STAGE_SHADOW);
    t.done(launch_trace_shadow(sc, h->shadow, h->small + 6, nb, h->sample_rgb, h->small + 7, st));
  }
  {
    StageTimer t(h, MSC_STAGE_BINS);
    t.done(launch_bin_partition(h->staging, nb, h->bins, st));
  }
  return MSC_OK;
}

int process_impl(msc_handle* h, int* iteration, bool copy_image) {
  if (!h || !iteration) return MSC_ERR_ARG;
  std::unique_lock<std::mutex> lock(h->busy, std::try_to_lock);
  if (!lock.owns_lock()) { h->err = "msc_process: the handle is rendering on another thread"; return MSC_ERR_BUSY; }
  *iteration = 0;
  h->stats.closest_queries = 0;
  h->stats.shadow_queries = 0;
  h->stats.batches = 0;
  h->stats.kernel_launches = 0;
  for (int s = 0; s < 12; ++s) { h->stats.stage_ms[s] = 0; h->stats.stage_launches[s] = 0; }
  if (h->terminate.load()) return MSC_OK;  // the reference's loop does not start (Pathtracer.cpp:449)
  cudaStream_t st = h->stream;
  const DevScene sc = dev_scene(h);
  const DevFrame fr = dev_frame(h);
  CK(cudaEventRecord(h->ev_begin, st));
  CK(cudaMemsetAsync(h->small, 0, 8 * sizeof(int), st));
  bool aborted = false;
  uint64_t shadow_total = 0;
  for (uint64_t first = 0; first < h->paths && !aborted; first += (uint64_t)h->generation) {
    const int n = (int)std::min<uint64_t>((uint64_t)h->generation, h->paths - first);
    {
      StageTimer t(h, MSC_STAGE_RAYGEN);
      t.done(launch_raygen(fr, (uint32_t)first, n, h->staging, st));
    }
    {
      StageTimer t(h, MSC_STAGE_BINS);
      t.done(launch_bin_partition(h->staging, n, h->bins, st));
    }
    bool first_read = true;
    while (true) {
      CK(cudaMemcpyAsync(h->h_small, h->small, 8 * sizeof(int), cudaMemcpyDeviceToHost, st));
      CK(cudaStreamSynchronize(st));
      if (h->profiling) harvest_stage_events(h);
      if (!first_read) shadow_total += (uint64_t)h->h_small[6];
      first_read = false;
      if (h->h_small[7] != 0) {
        const int e = h->h_small[7];
        h->err = (e & ERR_BIN_OVERFLOW)    ? "a direction bin overflowed"
                 : (e & ERR_TRAVERSAL_CAP) ? "BVH traversal exceeded its step cap"
                 : (e & kSortErrLookback)  ? "radix sort look-back exceeded its spin cap"
                 : (e & ERR_BVH_INDEX)     ? "BVH traversal met an out-of-range node or triangle index"
                                           : "BVH traversal stack overflowed";
        return MSC_ERR_DEVICE;
      }
      if (h->terminate.load()) { aborted = true; break; }
      int b = 0;
      for (int k = 1; k < 6; ++k)
        if (h->h_small[k] > h->h_small[b]) b = k;
      const int cnt = h->h_small[b];
      if (cnt == 0) break;
      const int nb = std::min(h->batch_cap, cnt);
      for (int k = 0; k < 6; ++k) h->h_counts_up[k] = h->h_small[k];
      h->h_counts_up[b] = cnt - nb;
      CK(cudaMemcpyAsync(h->small, h->h_counts_up, 6 * sizeof(int), cudaMemcpyHostToDevice, st));
      int rc = run_batch(h, sc, fr, b * h->generation + cnt - nb, nb);
      if (rc != MSC_OK) return rc;
      h->stats.closest_queries += (uint64_t)nb;
      h->stats.batches += 1;
    }
  }
  if (aborted) {
    CK(cudaStreamSynchronize(st));
    return MSC_OK;  // Pathtracer.cpp:486-487: a terminated pass returns 0 and leaves the image alone
  }
  {
    StageTimer t(h, MSC_STAGE_FILTER);
    t.done(launch_filter(fr, h->desc.filter, h->d_pixels, st));
  }
  CK(cudaEventRecord(h->ev_end, st));
  if (copy_image) {
    CK(cudaMemcpyAsync(h->h_pixels.data(), h->d_pixels, h->h_pixels.size() * sizeof(float), cudaMemcpyDeviceToHost, st));
  }
  CK(cudaStreamSynchronize(st));
  CK(cudaGetLastError());
  if (h->profiling) harvest_stage_events(h);
  h->host_stale = !copy_image;
  float ms = 0.f;
  cudaEventElapsedTime(&ms, h->ev_begin, h->ev_end);
  h->stats.process_ms = ms;
  h->stats.shadow_queries = shadow_total;
  h->iteration += 1;
  h->stats.iteration = h->iteration;
  *iteration = h->iteration;
  return MSC_OK;
}

template <class F>
int guarded(msc_handle* h, F&& f) {
  try {
    return f();
  } catch (const std::bad_alloc&) {
    if (h) h->err = "host out of memory";
    return MSC_ERR_CUDA;
  } catch (const std::exception& e) {
    if (h) h->err = e.what();
    return MSC_ERR_ARG;
  } catch (...) {
    if (h) h->err = "unknown error";
    return MSC_ERR_ARG;
  }
}

int upload_f4(const float* src, int n, int stride, int comps, float4** dst, float wval) {
  std::vector<float4> tmp((size_t)n);
  for (int i = 0; i < n; ++i) {
    float c[4] = {0.f, 0.f, 0.f, wval};
    for (int k = 0; k < comps; ++k) c[k] = src[(size_t)i * stride + k];
    tmp[i] = make_float4(c[0], c[1], c[2], c[3]);
  }
  if (cudaMalloc(dst, std::max<size_t>(1, (size_t)n) * sizeof(float4)) != cudaSuccess) return MSC_ERR_CUDA;
  if (n > 0 && cudaMemcpy(*dst, tmp.data(), (size_t)n * sizeof(float4), cudaMemcpyHostToDevice) != cudaSuccess)
    return MSC_ERR_CUDA;
  return MSC_OK;
}

}  // namespace

// ============================================================== C ABI

extern "C" {

int msc_create(const char* yaml_path, msc_handle** out) {
  if (!yaml_path || !out) { g_create_error = "msc_create: null argument"; return MSC_ERR_ARG; }
  *out = nullptr;
  msc_handle* h = nullptr;
  try {
    h = new msc_handle();
  } catch (...) {
    g_create_error = "host out of memory";
    return MSC_ERR_CUDA;
  }
  std::string err;
  bool ok = false;
  try {
    ok = load_scene(yaml_path, &h->desc, &err);
  } catch (const std::exception& e) {
    err = e.what();
  }
  if (!ok) {
    g_create_error = err;
    delete h;
    return MSC_ERR_SCENE;
  }
  int rc = guarded(h, [&] { return setup(h); });
  if (rc != MSC_OK) {
    g_create_error = h->err;
    release(h);
    delete h;
    return rc;
  }
  *out = h;
  return MSC_OK;
}

int msc_destroy(msc_handle* h) {
  if (!h) return MSC_ERR_ARG;
  {
    std::lock_guard<std::mutex> lock(h->busy);
    release(h);
  }
  delete h;
  return MSC_OK;
}

int msc_process(msc_handle* h, int* iteration) {
  return guarded(h, [&] { return process_impl(h, iteration, true); });
}

int msc_process_device(msc_handle* h, int* iteration) {
  return guarded(h, [&] { return process_impl(h, iteration, false); });
}

int msc_image(msc_handle* h, const float** rgb, int* width, int* height) {
  if (!h || !rgb || !width || !height) return MSC_ERR_ARG;
  if (h->host_stale) {
    std::unique_lock<std::mutex> lock(h->busy, std::try_to_lock);
    if (lock.owns_lock()) {
      if (cudaMemcpy(h->h_pixels.data(), h->d_pixels, h->h_pixels.size() * sizeof(float), cudaMemcpyDeviceToHost) !=
          cudaSuccess) {
        h->err = "msc_image: device copy failed";
        return MSC_ERR_CUDA;
      }
      h->host_stale = false;
    }
  }
  *rgb = h->h_pixels.data();
  *width = h->desc.width;
  *height = h->desc.height;
  return MSC_OK;
}

int msc_clear(msc_handle* h) {
  if (!h) return MSC_ERR_ARG;
  std::unique_lock<std::mutex> lock(h->busy, std::try_to_lock);
  if (!lock.owns_lock()) { h->err = "msc_clear: the handle is rendering on another thread"; return MSC_ERR_BUSY; }
  CK(cudaMemsetAsync(h->d_pixels, 0, h->h_pixels.size() * sizeof(float), h->stream));
  CK(cudaStreamSynchronize(h->stream));
  std::fill(h->h_pixels.begin(), h->h_pixels.end(), 0.f);
  h->host_stale = false;
  h->iteration = 0;
  return MSC_OK;
}

int msc_active(msc_handle* h, int* active) {
  if (!h || !active) return MSC_ERR_ARG;
  *active = h->terminate.load() ? 0 : 1;
  return MSC_OK;
}

int msc_terminate(msc_handle* h) {
  if (!h) return MSC_ERR_ARG;
  h->terminate.store(true);
  return MSC_OK;
}

int msc_save_image(msc_handle* h, const char* path, int divide_by_iterations) {
  if (!h || !path) return MSC_ERR_ARG;
  const float* px = nullptr;
  int w = 0, ht = 0;
  int rc = msc_image(h, &px, &w, &ht);
  if (rc != MSC_OK) return rc;
  std::vector<float> buf(px, px + (size_t)3 * w * ht);
  if (divide_by_iterations && h->iteration > 0)
    for (float& v : buf) v /= (float)h->iteration;
  std::string p(path), err;
  bool ok = false;
  try {
    if (p.size() >= 4 && p.compare(p.size() - 4, 4, ".pfm") == 0) ok = write_pfm(p, w, ht, buf.data(), &err);
    else ok = write_exr_rgba_half(p, w, ht, buf.data(), &err);
  } catch (const std::exception& e) {
    err = e.what();
  }
  if (!ok) { h->err = err; return MSC_ERR_ARG; }
  return MSC_OK;
}

int msc_write_image_file(const char* path, int width, int height, const float* rgb) {
  if (!path || !rgb || width <= 0 || height <= 0) return MSC_ERR_ARG;
  std::string p(path), err;
  bool ok = false;
  try {
    if (p.size() >= 4 && p.compare(p.size() - 4, 4, ".pfm") == 0) ok = write_pfm(p, width, height, rgb, &err);
    else ok = write_exr_rgba_half(p, width, height, rgb, &err);
  } catch (const std::exception& e) {
    err = e.what();
  }
  if (!ok) { g_create_error = err; return MSC_ERR_ARG; }
  return MSC_OK;
}

const char* msc_last_error(msc_handle* h) {
  if (!h) return g_create_error.c_str();
  return h->err.c_str();
}

int msc_get_stats(msc_handle* h, msc_stats* out) {
  if (!h || !out) return MSC_ERR_ARG;
  *out = h->stats;
  out->width = h->desc.width;
  out->height = h->desc.height;
  out->spp = h->desc.spp();
  out->triangles = (int)h->desc.tri_geom.size();
  out->lights = (int)h->desc.lights.size();
  out->iteration = h->iteration;
  return MSC_OK;
}

int msc_set_profiling(msc_handle* h, int on) {
  if (!h) return MSC_ERR_ARG;
  h->profiling = on != 0;
  return MSC_OK;
}

int msc_get_samples(msc_handle* h, float* rgb, float* xy) {
  if (!h || !rgb || !xy) return MSC_ERR_ARG;
  std::vector<float4> c(h->paths);
  std::vector<float2> p(h->paths);
  CK(cudaMemcpy(c.data(), h->sample_rgb, h->paths * sizeof(float4), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(p.data(), h->sample_pos, h->paths * sizeof(float2), cudaMemcpyDeviceToHost));
  for (uint64_t i = 0; i < h->paths; ++i) {
    rgb[3 * i + 0] = c[i].x;
    rgb[3 * i + 1] = c[i].y;
    rgb[3 * i + 2] = c[i].z;
    xy[2 * i + 0] = p[i].x;
    xy[2 * i + 1] = p[i].y;
  }
  return MSC_OK;
}

int msc_stage_cardinal(const float* dirs, int n, int32_t* bins) {
  if (n < 0 || (n > 0 && (!dirs || !bins))) return MSC_ERR_ARG;
  if (n == 0) return MSC_OK;
  float4* d = nullptr;
  int* o = nullptr;
  if (upload_f4(dirs, n, 3, 3, &d, 0.f) != MSC_OK) return MSC_ERR_CUDA;
  int rc = MSC_OK;
  if (cudaMalloc(&o, (size_t)n * 4) != cudaSuccess) rc = MSC_ERR_CUDA;
  if (rc == MSC_OK) {
    launch_cardinal(d, n, o, 0);
    if (cudaMemcpy(bins, o, (size_t)n * 4, cudaMemcpyDeviceToHost) != cudaSuccess) rc = MSC_ERR_CUDA;
  }
  cudaFree(d);
  if (o) cudaFree(o);
  return rc;
}

int msc_stage_bin_partition(const float* rays, int n, int cap, float* out, int32_t* counts) {
  if (n < 0 || cap <= 0 || !out || !counts || (n > 0 && !rays)) return MSC_ERR_ARG;
  RayBuf src;
  float4 *o = nullptr, *d = nullptr, *w = nullptr;
  int rc = MSC_OK;
  if (upload_f4(rays, n, 12, 4, &o, 0.f) || upload_f4(rays + 4, n, 12, 4, &d, 0.f) ||
      upload_f4(rays + 8, n, 12, 4, &w, 0.f))
    rc = MSC_ERR_CUDA;
  src.o = o; src.d = d; src.w = w;
  BinPool pool;
  char* mem = nullptr;
  const int tiles = std::max(1, (n + kPartTile - 1) / kPartTile);
  size_t bytes = 3 * al256((size_t)6 * cap * sizeof(float4)) + al256((size_t)kMaxBins * tiles * 4) + al256(8 * 4);
  if (rc == MSC_OK && cudaMalloc(&mem, bytes) != cudaSuccess) rc = MSC_ERR_CUDA;
  if (rc == MSC_OK) {
    DeviceArena A{mem, bytes, 0};
    pool.rays.o = A.take<float4>((size_t)6 * cap);
    pool.rays.d = A.take<float4>((size_t)6 * cap);
    pool.rays.w = A.take<float4>((size_t)6 * cap);
    pool.cap = cap;
    pool.tile_counts = A.take<uint32_t>((size_t)kMaxBins * tiles);
    pool.max_tiles = tiles;
    pool.count = A.take<int>(8);
    pool.err = pool.count + 7;
    cudaMemset(pool.count, 0, 8 * 4);
    cudaMemset(pool.rays.o, 0, 3 * al256((size_t)6 * cap * sizeof(float4)));
    launch_bin_partition(src, n, pool, 0);
    std::vector<float4> ho((size_t)6 * cap), hd((size_t)6 * cap), hw((size_t)6 * cap);
    int hc[8];
    if (cudaMemcpy(ho.data(), pool.rays.o, ho.size() * 16, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(hd.data(), pool.rays.d, hd.size() * 16, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(hw.data(), pool.rays.w, hw.size() * 16, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(hc, pool.count, 8 * 4, cudaMemcpyDeviceToHost) != cudaSuccess) {
      rc = MSC_ERR_CUDA;
    } else {
      for (size_t i = 0; i < ho.size(); ++i) {
        const float4 a = ho[i], b = hd[i], c = hw[i];
        float* r = out + 12 * i;
        r[0] = a.x; r[1] = a.y; r[2] = a.z; r[3] = a.w;
        r[4] = b.x; r[5] = b.y; r[6] = b.z; r[7] = b.w;
        r[8] = c.x; r[9] = c.y; r[10] = c.z; r[11] = c.w;
      }
      for (int k = 0; k < 6; ++k) counts[k] = hc[k];
      if (hc[7] != 0) rc = MSC_ERR_DEVICE;
    }
  }
  if (mem) cudaFree(mem);
  if (o) cudaFree(o);
  if (d) cudaFree(d);
  if (w) cudaFree(w);
  return rc;
}

int msc_stage_ray_keys(const float* org, const float* dir, int n, uint32_t* keys) {
  if (n < 0 || (n > 0 && (!org || !dir || !keys))) return MSC_ERR_ARG;
  if (n == 0) return MSC_OK;
  float4 *o = nullptr, *d = nullptr;
  uint32_t* mem = nullptr;
  int rc = MSC_OK;
  if (upload_f4(org, n, 3, 3, &o, 0.f) || upload_f4(dir, n, 3, 3, &d, 0.f)) rc = MSC_ERR_CUDA;
  if (rc == MSC_OK && cudaMalloc(&mem, (size_t)(n + 8) * 4) != cudaSuccess) rc = MSC_ERR_CUDA;
  if (rc == MSC_OK) {
    uint32_t* box = mem + n;
    cudaMemset(box, 0xff, 12);
    cudaMemset(box + 3, 0, 12);
    launch_origin_box(o, n, box, 0);
    launch_ray_keys(o, d, n, box, mem, 0);
    if (cudaMemcpy(keys, mem, (size_t)n * 4, cudaMemcpyDeviceToHost) != cudaSuccess) rc = MSC_ERR_CUDA;
  }
  if (o) cudaFree(o);
  if (d) cudaFree(d);
  if (mem) cudaFree(mem);
  return rc;
}

int msc_sort_pairs_device(uint32_t* keys, uint32_t* vals, int n, int bits, void* stream) {
  if (n < 0 || bits < 0 || bits > 32 || (n > 0 && (!keys || !vals))) return MSC_ERR_ARG;
  if (n == 0) return MSC_OK;
  cudaStream_t st = (cudaStream_t)stream;
  char* mem = nullptr;
  size_t bytes = sort_scratch_bytes(n);
  if (cudaMallocAsync(&mem, bytes, st) != cudaSuccess) return MSC_ERR_CUDA;
  SortScratch ss;
  sort_scratch_bind(&ss, mem, n);
  sort_pairs(keys, vals, keys, vals, n, bits, ss, st);
  cudaFreeAsync(mem, st);
  return cudaGetLastError() == cudaSuccess ? MSC_OK : MSC_ERR_CUDA;
}

int msc_sort_pairs(uint32_t* keys, uint32_t* vals, int n, int bits) {
  if (n < 0 || bits < 0 || bits > 32 || (n > 0 && (!keys || !vals))) return MSC_ERR_ARG;
  if (n == 0) return MSC_OK;
  uint32_t* d = nullptr;
  if (cudaMalloc(&d, (size_t)n * 8) != cudaSuccess) return MSC_ERR_CUDA;
  int rc = MSC_OK;
  if (cudaMemcpy(d, keys, (size_t)n * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(d + n, vals, (size_t)n * 4, cudaMemcpyHostToDevice) != cudaSuccess)
    rc = MSC_ERR_CUDA;
  if (rc == MSC_OK) rc = msc_sort_pairs_device(d, d + n, n, bits, nullptr);
  if (rc == MSC_OK && (cudaMemcpy(keys, d, (size_t)n * 4, cudaMemcpyDeviceToHost) != cudaSuccess ||
                       cudaMemcpy(vals, d + n, (size_t)n * 4, cudaMemcpyDeviceToHost) != cudaSuccess))
    rc = MSC_ERR_CUDA;
  cudaFree(d);
  return rc;
}

int msc_trace_closest(msc_handle* h, const float* org, const float* dir, int n, float* t, float* u, float* v,
                      int32_t* geom, int32_t* prim) {
  if (!h || n < 0 || (n > 0 && (!org || !dir || !t || !u || !v || !geom || !prim))) return MSC_ERR_ARG;
  if (n == 0) return MSC_OK;
  float4 *o = nullptr, *d = nullptr, *hits = nullptr;
  int* err = nullptr;
  int rc = MSC_OK;
  if (upload_f4(org, n, 3, 3, &o, 0.f) || upload_f4(dir, n, 3, 3, &d, 0.f)) rc = MSC_ERR_CUDA;
  if (rc == MSC_OK && (cudaMalloc(&hits, (size_t)n * 16) != cudaSuccess || cudaMalloc(&err, 4) != cudaSuccess))
    rc = MSC_ERR_CUDA;
  if (rc == MSC_OK) {
    cudaMemset(err, 0, 4);
    DevScene sc = dev_scene(h);
    launch_trace_closest(sc, o, d, n, hits, err, 0);
    std::vector<float4> hh((size_t)n);
    int he = 0;
    if (cudaMemcpy(hh.data(), hits, (size_t)n * 16, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(&he, err, 4, cudaMemcpyDeviceToHost) != cudaSuccess) {
      rc = MSC_ERR_CUDA;
    } else {
      for (int i = 0; i < n; ++i) {
        int k;
        memcpy(&k, &hh[i].w, 4);
        t[i] = hh[i].x;
        u[i] = hh[i].y;
        v[i] = hh[i].z;
        if (k < 0) {
          geom[i] = -1;
          prim[i] = -1;
          t[i] = MSC_TFAR;
        } else {
          int g = h->h_tri_orig[k];
          int gid = h->desc.tri_geom[g];
          geom[i] = gid;
          prim[i] = g - h->desc.geoms[gid].first_prim;
        }
      }
      if (he != 0) { h->err = "BVH traversal stack overflowed"; rc = MSC_ERR_DEVICE; }
    }
  }
  if (o) cudaFree(o);
  if (d) cudaFree(d);
  if (hits) cudaFree(hits);
  if (err) cudaFree(err);
  return rc;
}

int msc_trace_occluded(msc_handle* h, const float* org, const float* dir, const float* tmax, int n,
                       int32_t* occluded) {
  if (!h || n < 0 || (n > 0 && (!org || !dir || !tmax || !occluded))) return MSC_ERR_ARG;
  if (n == 0) return MSC_OK;
  std::vector<float> o4((size_t)n * 4);
  for (int i = 0; i < n; ++i) {
    o4[4 * i + 0] = org[3 * i + 0];
    o4[4 * i + 1] = org[3 * i + 1];
    o4[4 * i + 2] = org[3 * i + 2];
    o4[4 * i + 3] = tmax[i];
  }
  float4 *o = nullptr, *d = nullptr;
  int *res = nullptr, *err = nullptr;
  int rc = MSC_OK;
  if (upload_f4(o4.data(), n, 4, 4, &o, 0.f) || upload_f4(dir, n, 3, 3, &d, 0.f)) rc = MSC_ERR_CUDA;
  if (rc == MSC_OK && (cudaMalloc(&res, (size_t)n * 4) != cudaSuccess || cudaMalloc(&err, 4) != cudaSuccess))
    rc = MSC_ERR_CUDA;
  if (rc == MSC_OK) {
    cudaMemset(err, 0, 4);
    launch_occluded(dev_scene(h), o, d, n, res, err, 0);
    int he = 0;
    if (cudaMemcpy(occluded, res, (size_t)n * 4, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(&he, err, 4, cudaMemcpyDeviceToHost) != cudaSuccess)
      rc = MSC_ERR_CUDA;
    else if (he != 0) { h->err = "BVH traversal stack overflowed"; rc = MSC_ERR_DEVICE; }
  }
  if (o) cudaFree(o);
  if (d) cudaFree(d);
  if (res) cudaFree(res);
  if (err) cudaFree(err);
  return rc;
}

int msc_obj_load(const char* path, float* positions, float* texcoords, uint32_t* indices, int64_t* sizes) {
  if (!path || !sizes) return MSC_ERR_ARG;
  ObjMesh m;
  std::string err;
  try {
    if (!obj_load_file(path, &m, &err)) { g_create_error = err; return MSC_ERR_SCENE; }
  } catch (const std::exception& e) {
    g_create_error = e.what();
    return MSC_ERR_SCENE;
  }
  sizes[0] = (int64_t)m.positions.size();
  sizes[1] = (int64_t)m.texcoords.size();
  sizes[2] = (int64_t)m.indices.size();
  if (positions) memcpy(positions, m.positions.data(), m.positions.size() * 4);
  if (texcoords) memcpy(texcoords, m.texcoords.data(), m.texcoords.size() * 4);
  if (indices) memcpy(indices, m.indices.data(), m.indices.size() * 4);
  return MSC_OK;
}

int msc_scene_load_host(const char* yaml_path, int32_t* info, float* tri_v, int32_t* tri_geom) {
  if (!yaml_path || !info) return MSC_ERR_ARG;
  SceneDesc d;
  std::string err;
  try {
    if (!load_scene(yaml_path, &d, &err)) { g_create_error = err; return MSC_ERR_SCENE; }
  } catch (const std::exception& e) {
    g_create_error = e.what();
    return MSC_ERR_SCENE;
  }
  info[0] = d.width;
  info[1] = d.height;
  info[2] = d.spp();
  info[3] = (int32_t)d.tri_geom.size();
  info[4] = (int32_t)d.lights.size();
  info[5] = (int32_t)d.shaders.size();
  info[6] = (int32_t)d.geoms.size();
  info[7] = d.camera.type;
  if (tri_v) memcpy(tri_v, d.tri_v.data(), d.tri_v.size() * sizeof(float));
  if (tri_geom) memcpy(tri_geom, d.tri_geom.data(), d.tri_geom.size() * sizeof(int32_t));
  return MSC_OK;
}

int msc_generate_scene(int config, uint32_t seed, double scale, const char* out_dir, char* yaml_path, int cap) {
  if (!out_dir || !yaml_path || cap <= 0) return MSC_ERR_ARG;
  std::string yaml, err;
  bool ok = false;
  try {
    ok = generate_scene(config, seed, scale, out_dir, &yaml, &err);
  } catch (const std::exception& e) {
    err = e.what();
  }
  if (!ok) {
    g_create_error = err;
    return MSC_ERR_SCENE;
  }
  if ((int)yaml.size() + 1 > cap) return MSC_ERR_ARG;
  memcpy(yaml_path, yaml.c_str(), yaml.size() + 1);
  return MSC_OK;
}

}  // extern "C"
