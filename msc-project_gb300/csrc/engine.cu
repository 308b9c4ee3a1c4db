// The C ABI of include/msc_gpu.h over the render core (core.h).
//
//   msc_*        the reference engine's interface (msc::Pathtracer,
//                include/core/Pathtracer.h:36-110): one scene, one job whose
//                image accumulates over process() calls
//   msc_batch_*  many resident scenes and jobs of uneven size in one wavefront
//   msc_serve    a request loop that admits jobs as they arrive and as film
//                memory frees up, and reports per-job latency
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "../../include/msc_gpu.h"
#include "core.h"

namespace mscg {
bool generate_scene(int config, uint32_t seed, double scale, const std::string& dir, std::string* yaml,
                    std::string* err);
bool write_exr_rgba_half(const std::string& path, int w, int h, const float* rgb, std::string* err);
bool write_pfm(const std::string& path, int w, int h, const float* rgb, std::string* err);
}  // namespace mscg

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

template <class F>
int guarded(std::string* err, F&& f) {
  try {
    return f();
  } catch (const std::bad_alloc&) {
    if (err) *err = "host out of memory";
    return MSC_ERR_CUDA;
  } catch (const std::exception& e) {
    if (err) *err = e.what();
    return MSC_ERR_ARG;
  } catch (...) {
    if (err) *err = "unknown error";
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

void fill_stats(const CoreStats& cs, double ms, msc_stats* out) {
  out->closest_queries = cs.closest;
  out->shadow_queries = cs.shadow;
  out->batches = cs.batches;
  out->kernel_launches = cs.launches;
  out->process_ms = ms;
  out->gpu_busy_ms = cs.busy_ms;
  for (int s = 0; s < 12; ++s) {
    out->stage_ms[s] = cs.stage_ms[s];
    out->stage_launches[s] = cs.stage_launches[s];
  }
}

JobSpec spec_of(const msc_job_desc& d) {
  JobSpec s;
  s.scene = d.scene;
  s.width = d.width;
  s.height = d.height;
  s.spp = d.spp;
  s.min_depth = d.min_depth;
  s.max_depth = d.max_depth;
  s.use_camera = d.use_camera;
  for (int i = 0; i < 3; ++i) {
    s.cam_translation[i] = d.translation[i];
    s.cam_rotation[i] = d.rotation[i];
  }
  s.cam_focal = d.focal_length;
  s.seed = d.seed;
  s.iteration = 0;
  return s;
}

}  // namespace

// ================================================================ plain form

// The host image of a plain handle: allocated page-locked by the driver
// (cudaMallocHost), so the copy after every pass runs at the host link's
// speed; an ordinary allocation when that fails (pageable copies still work).
struct HostImage {
  float* p = nullptr;
  size_t n = 0;
  bool pinned = false;
  std::vector<float> fallback;
  float* data() { return p; }
  size_t size() const { return n; }
  float* begin() { return p; }
  float* end() { return p + n; }
  void assign(size_t count, float v) {
    release();
    n = count;
    pinned = cudaMallocHost(reinterpret_cast<void**>(&p), std::max<size_t>(n, 1) * sizeof(float)) == cudaSuccess;
    if (!pinned) {
      cudaGetLastError();
      fallback.assign(std::max<size_t>(n, 1), v);
      p = fallback.data();
    }
    std::fill(p, p + n, v);
  }
  void release() {
    if (pinned && p) cudaFreeHost(p);
    p = nullptr;
    pinned = false;
    fallback.clear();
  }
  ~HostImage() { release(); }
};

struct msc_handle {
  Core core;
  SceneDesc desc;
  std::string err;
  std::mutex busy;
  std::atomic<bool> terminate{false};
  volatile bool stop_flag = false;
  int job = -1;
  int iteration = 0;
  bool host_stale = false;
  HostImage h_pixels;
  msc_stats stats;
  double load_ms = 0, bvh_ms = 0;  // msc_create's scene parse and device BVH build, wall clock
  cudaEvent_t ev_begin = nullptr, ev_end = nullptr;
};

namespace {

int plain_setup(msc_handle* h) {
  const SceneDesc& d = h->desc;
  const uint64_t paths = (uint64_t)d.width * (uint64_t)d.height * (uint64_t)d.spp();
  if (paths >= (1ull << 31)) {
    h->err = "width * height * samples must stay below 2^31";
    return MSC_ERR_ARG;
  }
  const int e = std::min(d.settings.bin_exponent, 24);
  // paths in flight: 64 times the scene's batch (fuller bins, so the batches
  // stay full for more of the pass)
  uint64_t gen = d.ext.generation > 0 ? (uint64_t)d.ext.generation : std::max<uint64_t>(64ull << e, 1ull << 22);
  gen = std::max<uint64_t>(std::min<uint64_t>(gen, paths), 1);
  // capacity for sixteen times the scene's batch so the autotuner can also try larger ones
  int rc = h->core.init(std::min(e + 4, 24), (int)gen, paths, d.ext.wide_bvh != 0);
  if (rc != MSC_OK) {
    h->err = h->core.err;
    return rc;
  }
  h->core.ray_sort = d.ext.ray_sort != 0;
  h->core.hit_sort = d.ext.hit_sort != 0;
  {
    TuneChoice c = h->core.choice();
    // sixteen times the scene's batch (2^bin exponent, Settings.h:16-24):
    // larger traversal grids amortise the kernels' tails and larger sorted
    // batches trace more coherently
    c.batch_exp = std::min(e + 4, 24);
    c.bins = d.ext.bins;
    h->core.apply(c);
  }
  if (d.ext.autotune) h->core.start_autotune();
  int sid = 0;
  const auto t0 = std::chrono::steady_clock::now();
  rc = h->core.add_scene(d, &sid);
  if (rc != MSC_OK) {
    h->err = h->core.err;
    return rc;
  }
  if (cudaDeviceSynchronize() != cudaSuccess) {
    h->err = "device BVH build failed";
    return MSC_ERR_CUDA;
  }
  h->bvh_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  JobSpec spec;
  spec.scene = sid;
  rc = h->core.add_job(spec, &h->job);
  if (rc != MSC_OK) {
    h->err = h->core.err;
    return rc;
  }
  h->h_pixels.assign((size_t)3 * d.width * d.height, 0.f);
  if (cudaEventCreate(&h->ev_begin) != cudaSuccess || cudaEventCreate(&h->ev_end) != cudaSuccess) {
    h->err = "cannot create CUDA events";
    return MSC_ERR_CUDA;
  }
  memset(&h->stats, 0, sizeof(h->stats));
  return MSC_OK;
}

int process_impl(msc_handle* h, int* iteration, bool copy_image) {
  if (!h || !iteration) return MSC_ERR_ARG;
  std::unique_lock<std::mutex> lock(h->busy, std::try_to_lock);
  if (!lock.owns_lock()) {
    h->err = "msc_process: the handle is rendering on another thread";
    return MSC_ERR_BUSY;
  }
  *iteration = 0;
  if (h->terminate.load()) return MSC_OK;  // the reference's loop does not start (Pathtracer.cpp:449)
  Core& c = h->core;
  JobState* j = c.job(h->job);
  if (h->iteration > 0 || j->complete) {
    JobSpec spec;
    spec.iteration = h->iteration;
    j->rec.iter_seed = job_record(h->desc, spec, 0).iter_seed;
    int rc = c.restart_job(h->job);
    if (rc != MSC_OK) {
      h->err = c.err;
      return rc;
    }
  }
  c.reset_stats();
  cudaEventRecord(h->ev_begin, c.stream());
  struct Watch {  // mirror terminate() into the core's stop flag while running
    msc_handle* h;
    std::atomic<bool> on{true};
    std::thread t;
    explicit Watch(msc_handle* hh) : h(hh) {
      t = std::thread([this] {
        while (on.load()) {
          if (h->terminate.load()) h->stop_flag = true;
          std::this_thread::sleep_for(std::chrono::microseconds(200));
        }
      });
    }
    ~Watch() {
      on.store(false);
      t.join();
    }
  };
  int rc;
  {
    Watch w(h);
    rc = c.run_all(&h->stop_flag);
  }
  if (rc != MSC_OK) {
    h->err = c.err;
    return rc;
  }
  if (h->terminate.load() || !j->complete) {
    c.sync_stream();
    return MSC_OK;  // Pathtracer.cpp:486-487: a terminated pass returns 0 and leaves the image alone
  }
  cudaEventRecord(h->ev_end, c.stream());
  if (copy_image) {
    if (cudaMemcpyAsync(h->h_pixels.data(), j->d_pixels, h->h_pixels.size() * sizeof(float), cudaMemcpyDeviceToHost,
                        c.stream()) != cudaSuccess) {
      h->err = "msc_process: image copy failed";
      return MSC_ERR_CUDA;
    }
  }
  if (c.sync_stream() != cudaSuccess) {
    h->err = "msc_process: device error";
    return MSC_ERR_CUDA;
  }
  h->host_stale = !copy_image;
  float ms = 0.f;
  cudaEventElapsedTime(&ms, h->ev_begin, h->ev_end);
  fill_stats(c.stats, ms, &h->stats);
  h->iteration += 1;
  h->stats.iteration = h->iteration;
  *iteration = h->iteration;
  return MSC_OK;
}

}  // namespace

// ============================================================ batched form

struct msc_batch {
  Core core;
  std::string err;
  std::vector<std::string> scene_paths;
  bool initialised = false;
  int batch_exponent = 20;
  int64_t film_samples = 0;
  double last_ms = 0.0;
};

extern "C" {

// ------------------------------------------------------------------ plain

int msc_create(const char* yaml_path, msc_handle** out) {
  if (!yaml_path || !out) {
    g_create_error = "msc_create: null argument";
    return MSC_ERR_ARG;
  }
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
  const auto t0 = std::chrono::steady_clock::now();
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
  h->load_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  int rc = guarded(&h->err, [&] { return plain_setup(h); });
  if (rc != MSC_OK) {
    g_create_error = h->err;
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
    if (h->ev_begin) cudaEventDestroy(h->ev_begin);
    if (h->ev_end) cudaEventDestroy(h->ev_end);
  }
  delete h;
  return MSC_OK;
}

int msc_process(msc_handle* h, int* iteration) {
  if (!h) return MSC_ERR_ARG;
  return guarded(&h->err, [&] { return process_impl(h, iteration, true); });
}

int msc_process_device(msc_handle* h, int* iteration) {
  if (!h) return MSC_ERR_ARG;
  return guarded(&h->err, [&] { return process_impl(h, iteration, false); });
}

int msc_image(msc_handle* h, const float** rgb, int* width, int* height) {
  if (!h || !rgb || !width || !height) return MSC_ERR_ARG;
  if (h->host_stale) {
    std::unique_lock<std::mutex> lock(h->busy, std::try_to_lock);
    if (lock.owns_lock()) {
      JobState* j = h->core.job(h->job);
      if (cudaMemcpy(h->h_pixels.data(), j->d_pixels, h->h_pixels.size() * sizeof(float), cudaMemcpyDeviceToHost) !=
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
  if (!lock.owns_lock()) {
    h->err = "msc_clear: the handle is rendering on another thread";
    return MSC_ERR_BUSY;
  }
  JobState* j = h->core.job(h->job);
  if (cudaMemsetAsync(j->d_pixels, 0, h->h_pixels.size() * sizeof(float), h->core.stream()) != cudaSuccess ||
      cudaStreamSynchronize(h->core.stream()) != cudaSuccess) {
    h->err = "msc_clear: device error";
    return MSC_ERR_CUDA;
  }
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
  h->stop_flag = true;
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
  rc = msc_write_image_file(path, w, ht, buf.data());
  if (rc != MSC_OK) h->err = g_create_error;
  return rc;
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
  if (!ok) {
    g_create_error = err;
    return MSC_ERR_ARG;
  }
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
  out->load_ms = h->load_ms;
  out->bvh_ms = h->bvh_ms;
  return MSC_OK;
}

int msc_set_profiling(msc_handle* h, int on) {
  if (!h) return MSC_ERR_ARG;
  h->core.profiling = on != 0;
  return MSC_OK;
}

int msc_get_samples(msc_handle* h, float* rgb, float* xy) {
  if (!h || !rgb || !xy) return MSC_ERR_ARG;
  JobState* j = h->core.job(h->job);
  const size_t n = j->paths;
  std::vector<float4> c(n);
  std::vector<float2> p(n);
  const Film f = h->core.film();
  if (cudaMemcpy(c.data(), f.rgb + j->sample_off, n * sizeof(float4), cudaMemcpyDeviceToHost) != cudaSuccess ||
      cudaMemcpy(p.data(), f.pos + j->sample_off, n * sizeof(float2), cudaMemcpyDeviceToHost) != cudaSuccess) {
    h->err = "msc_get_samples: device copy failed";
    return MSC_ERR_CUDA;
  }
  for (size_t i = 0; i < n; ++i) {
    rgb[3 * i + 0] = c[i].x;
    rgb[3 * i + 1] = c[i].y;
    rgb[3 * i + 2] = c[i].z;
    xy[2 * i + 0] = p[i].x;
    xy[2 * i + 1] = p[i].y;
  }
  return MSC_OK;
}

// ------------------------------------------------------------------ stages

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

int msc_stage_bin_partition_n(const float* rays, int n, int nbins, int cap, float* out, int32_t* counts) {
  if (n < 0 || cap <= 0 || !out || !counts || (n > 0 && !rays) || (nbins != 6 && nbins != 26 && nbins != 98))
    return MSC_ERR_ARG;
  RayBuf src;
  float4 *o = nullptr, *d = nullptr, *w = nullptr;
  int rc = MSC_OK;
  if (upload_f4(rays, n, 12, 4, &o, 0.f) || upload_f4(rays + 4, n, 12, 4, &d, 0.f) ||
      upload_f4(rays + 8, n, 12, 4, &w, 0.f))
    rc = MSC_ERR_CUDA;
  src.o = o;
  src.d = d;
  src.w = w;
  // a chunked pool sized for the rays, as the render loop uses it
  BinPool pool;
  pool.nbins = nbins;
  const size_t chunks = bin_pool_chunks((size_t)std::max(n, 1));
  pool.num_chunks = (int)chunks;
  pool.max_chunks = (std::max(n, 1) + kChunk - 1) / kChunk + 1;
  char* mem = nullptr;
  const int tiles = std::max(1, (n + kPartTile - 1) / kPartTile);
  const size_t ray_bytes = al256(chunks * kChunk * sizeof(float4));
  const size_t table_bytes = al256((size_t)kMaxBins * pool.max_chunks * 4);
  size_t bytes = 3 * ray_bytes + al256((size_t)(kMaxBins + 1) * tiles * 4) + table_bytes + al256(chunks * 4) +
                 al256(sizeof(Counters)) + al256((size_t)kMaxBins * 4) + al256(4);
  if (rc == MSC_OK && cudaMalloc(&mem, bytes) != cudaSuccess) rc = MSC_ERR_CUDA;
  if (rc == MSC_OK) {
    char* p = mem;
    pool.rays.o = (float4*)p;
    p += ray_bytes;
    pool.rays.d = (float4*)p;
    p += ray_bytes;
    pool.rays.w = (float4*)p;
    p += ray_bytes;
    pool.tile_counts = (uint32_t*)p;
    p += al256((size_t)(kMaxBins + 1) * tiles * 4);
    pool.max_tiles = tiles;
    pool.table = (int*)p;
    p += table_bytes;
    pool.free_stack = (int*)p;
    p += al256(chunks * 4);
    Counters* ctr = (Counters*)p;
    p += al256(sizeof(Counters));
    pool.held = (int*)p;
    p += al256((size_t)kMaxBins * 4);
    pool.free_top = (int*)p;
    pool.count = ctr->bin_count;
    pool.in_bins = &ctr->in_bins;
    pool.err = &ctr->err;
    cudaMemset(ctr, 0, sizeof(Counters));
    launch_pool_reset(pool, 0);
    launch_bin_partition(src, n, pool, 0);
    Counters hc;
    std::vector<int> table((size_t)kMaxBins * pool.max_chunks);
    std::vector<float4> ho(chunks * kChunk), hd(chunks * kChunk), hw(chunks * kChunk);
    if (cudaMemcpy(&hc, ctr, sizeof(hc), cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(table.data(), pool.table, table.size() * 4, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(ho.data(), pool.rays.o, ho.size() * 16, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(hd.data(), pool.rays.d, hd.size() * 16, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(hw.data(), pool.rays.w, hw.size() * 16, cudaMemcpyDeviceToHost) != cudaSuccess) {
      rc = MSC_ERR_CUDA;
    } else if (hc.err != 0) {
      rc = MSC_ERR_DEVICE;
    } else {
      // bin b's rays in bin order at out[(b * cap + i) * 12]
      memset(out, 0, sizeof(float) * 12 * (size_t)nbins * cap);
      for (int bb = 0; bb < nbins; ++bb) {
        counts[bb] = hc.bin_count[bb];
        for (int i = 0; i < hc.bin_count[bb] && i < cap; ++i) {
          const int q = pool_index(table.data(), pool.max_chunks, bb, i);
          const float4 a4 = ho[q], b4 = hd[q], c4 = hw[q];
          float* r = out + 12 * ((size_t)bb * cap + i);
          r[0] = a4.x; r[1] = a4.y; r[2] = a4.z; r[3] = a4.w;
          r[4] = b4.x; r[5] = b4.y; r[6] = b4.z; r[7] = b4.w;
          r[8] = c4.x; r[9] = c4.y; r[10] = c4.z; r[11] = c4.w;
        }
      }
    }
  }
  if (mem) cudaFree(mem);
  if (o) cudaFree(o);
  if (d) cudaFree(d);
  if (w) cudaFree(w);
  return rc;
}

int msc_stage_bin_partition(const float* rays, int n, int cap, float* out, int32_t* counts) {
  return msc_stage_bin_partition_n(rays, n, 6, cap, out, counts);
}

int msc_stage_ray_bins(const float* dirs, int n, int nbins, int32_t* bins) {
  if (n < 0 || (n > 0 && (!dirs || !bins)) || (nbins != 6 && nbins != 26 && nbins != 98)) return MSC_ERR_ARG;
  if (n == 0) return MSC_OK;
  float4* d = nullptr;
  int* out = nullptr;
  int rc = MSC_OK;
  if (upload_f4(dirs, n, 3, 3, &d, 0.f)) rc = MSC_ERR_CUDA;
  if (rc == MSC_OK && cudaMalloc(&out, (size_t)n * 4) != cudaSuccess) rc = MSC_ERR_CUDA;
  if (rc == MSC_OK) {
    launch_ray_bins(d, n, nbins, out, 0);
    if (cudaMemcpy(bins, out, (size_t)n * 4, cudaMemcpyDeviceToHost) != cudaSuccess) rc = MSC_ERR_CUDA;
  }
  if (d) cudaFree(d);
  if (out) cudaFree(out);
  return rc;
}

int msc_stage_ray_keys(const float* org, const float* dir, int n, uint32_t* keys) {
  if (n < 0 || (n > 0 && (!org || !dir || !keys))) return MSC_ERR_ARG;
  if (n == 0) return MSC_OK;
  // the origin box of the given rays (RayBoundingbox.cpp:10-35)
  float lo[3] = {org[0], org[1], org[2]}, hi[3] = {org[0], org[1], org[2]};
  for (int i = 0; i < n; ++i)
    for (int a = 0; a < 3; ++a) {
      lo[a] = std::min(lo[a], org[3 * i + a]);
      hi[a] = std::max(hi[a], org[3 * i + a]);
    }
  float sc[3];
  for (int a = 0; a < 3; ++a) {
    const float e = hi[a] - lo[a];
    sc[a] = e > 0.f ? 64.0f / e : 0.f;
  }
  float4 *o = nullptr, *d = nullptr;
  uint32_t* mem = nullptr;
  int rc = MSC_OK;
  if (upload_f4(org, n, 3, 3, &o, 0.f) || upload_f4(dir, n, 3, 3, &d, 0.f)) rc = MSC_ERR_CUDA;
  if (rc == MSC_OK && cudaMalloc(&mem, (size_t)n * 4) != cudaSuccess) rc = MSC_ERR_CUDA;
  if (rc == MSC_OK) {
    launch_ray_keys_direct(o, d, n, make_float3(lo[0], lo[1], lo[2]), make_float3(sc[0], sc[1], sc[2]), mem, 0);
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

int msc_stage_sort_pairs_digits(uint32_t* keys, uint32_t* vals, int n, int bits, int digit_bits) {
  if (n < 0 || bits < 0 || bits > 32 || (n > 0 && (!keys || !vals)) ||
      (digit_bits != 4 && digit_bits != 8 && digit_bits != 11))
    return MSC_ERR_ARG;
  if (n == 0) return MSC_OK;
  uint32_t* d = nullptr;
  char* scratch = nullptr;
  const size_t sb = sort_scratch_bytes(n, 11);
  int rc = MSC_OK;
  if (cudaMalloc(&d, (size_t)n * 16) != cudaSuccess || cudaMalloc(&scratch, sb) != cudaSuccess) rc = MSC_ERR_CUDA;
  if (rc == MSC_OK && (cudaMemcpy(d, keys, (size_t)n * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
                       cudaMemcpy(d + n, vals, (size_t)n * 4, cudaMemcpyHostToDevice) != cudaSuccess))
    rc = MSC_ERR_CUDA;
  if (rc == MSC_OK) {
    SortScratch ss;
    sort_scratch_bind(&ss, scratch, n, 11);
    sort_pairs(d, d + n, d + 2 * (size_t)n, d + 3 * (size_t)n, n, bits, ss, 0, nullptr, nullptr, digit_bits);
    if (cudaMemcpy(keys, d + 2 * (size_t)n, (size_t)n * 4, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(vals, d + 3 * (size_t)n, (size_t)n * 4, cudaMemcpyDeviceToHost) != cudaSuccess)
      rc = MSC_ERR_CUDA;
  }
  if (d) cudaFree(d);
  if (scratch) cudaFree(scratch);
  return rc;
}

int msc_stage_sort_lookback_check(uint32_t* keys, uint32_t* vals, int n, int bits, int spin_cap,
                                  int withhold_first_tile) {
  if (n <= 0 || bits < 1 || bits > 32 || !keys || !vals || spin_cap < 1) return MSC_ERR_ARG;
  uint32_t* d = nullptr;
  char* scratch = nullptr;
  int* d_err = nullptr;
  const size_t sb = sort_scratch_bytes(n);
  int rc = MSC_OK;
  if (cudaMalloc(&d, (size_t)n * 16) != cudaSuccess || cudaMalloc(&scratch, sb) != cudaSuccess ||
      cudaMalloc(&d_err, sizeof(int)) != cudaSuccess || cudaMemset(d_err, 0, sizeof(int)) != cudaSuccess)
    rc = MSC_ERR_CUDA;
  if (rc == MSC_OK && (cudaMemcpy(d, keys, (size_t)n * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
                       cudaMemcpy(d + n, vals, (size_t)n * 4, cudaMemcpyHostToDevice) != cudaSuccess))
    rc = MSC_ERR_CUDA;
  int h_err = 0;
  if (rc == MSC_OK) {
    SortScratch ss;
    sort_scratch_bind(&ss, scratch, n);
    SortTestHook hook;
    hook.spin_cap = spin_cap;
    hook.withhold_first_tile = withhold_first_tile != 0;
    sort_pairs(d, d + n, d + 2 * (size_t)n, d + 3 * (size_t)n, n, bits, ss, 0, d_err, nullptr, 8, &hook);
    if (cudaMemcpy(keys, d + 2 * (size_t)n, (size_t)n * 4, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(vals, d + 3 * (size_t)n, (size_t)n * 4, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(&h_err, d_err, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
      rc = MSC_ERR_CUDA;
  }
  if (d) cudaFree(d);
  if (scratch) cudaFree(scratch);
  if (d_err) cudaFree(d_err);
  if (rc == MSC_OK && (h_err & kSortErrLookback)) {
    set_global_error("sort: a look-back wait ran out of its spin cap (a predecessor tile never posted its counts)");
    return MSC_ERR_DEVICE;
  }
  return rc;
}

int msc_stage_sort_keys64(const uint64_t* keys, int n, uint32_t* perm) {
  if (n < 0 || (n > 0 && (!keys || !perm))) return MSC_ERR_ARG;
  if (n == 0) return MSC_OK;
  std::vector<uint32_t> lo((size_t)n), hi((size_t)n);
  for (int i = 0; i < n; ++i) {
    lo[i] = (uint32_t)keys[i];
    hi[i] = (uint32_t)(keys[i] >> 32);
  }
  uint32_t* d = nullptr;
  char* scratch = nullptr;
  const size_t sb = sort_scratch_bytes(n);
  int rc = MSC_OK;
  if (cudaMalloc(&d, (size_t)n * 4 * 6) != cudaSuccess || cudaMalloc(&scratch, sb) != cudaSuccess) rc = MSC_ERR_CUDA;
  if (rc == MSC_OK) {
    uint32_t *d_lo = d, *d_hi = d + n, *lo_s = d + 2 * (size_t)n, *perm1 = d + 3 * (size_t)n,
             *hi_g = d + 4 * (size_t)n, *d_perm = d + 5 * (size_t)n;
    SortScratch ss;
    sort_scratch_bind(&ss, scratch, n);
    if (cudaMemcpy(d_lo, lo.data(), (size_t)n * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(d_hi, hi.data(), (size_t)n * 4, cudaMemcpyHostToDevice) != cudaSuccess)
      rc = MSC_ERR_CUDA;
    if (rc == MSC_OK) {
      sort_pairs(d_lo, nullptr, lo_s, perm1, n, 32, ss, 0);
      launch_gather_u32(d_hi, perm1, n, hi_g, 0);
      sort_pairs(hi_g, perm1, d_hi, d_perm, n, 32, ss, 0);
      if (cudaMemcpy(perm, d_perm, (size_t)n * 4, cudaMemcpyDeviceToHost) != cudaSuccess) rc = MSC_ERR_CUDA;
    }
  }
  if (d) cudaFree(d);
  if (scratch) cudaFree(scratch);
  return rc;
}

int msc_trace_closest(msc_handle* h, const float* org, const float* dir, int n, float* t, float* u, float* v,
                      int32_t* geom, int32_t* prim) {
  if (!h || n < 0 || (n > 0 && (!org || !dir || !t || !u || !v || !geom || !prim))) return MSC_ERR_ARG;
  if (n == 0) return MSC_OK;
  std::vector<float4> hh((size_t)n);
  int rc = h->core.trace_closest(org, dir, n, hh.data());
  if (rc != MSC_OK) {
    h->err = h->core.err;
    return rc;
  }
  SceneGPU* sg = h->core.scene(0);
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
      const int g = sg->h_tri_orig[k];
      const int gid = sg->desc.tri_geom[g];
      geom[i] = gid;
      prim[i] = g - sg->desc.geoms[gid].first_prim;
    }
  }
  return MSC_OK;
}

int msc_trace_occluded(msc_handle* h, const float* org, const float* dir, const float* tmax, int n,
                       int32_t* occluded) {
  if (!h || n < 0 || (n > 0 && (!org || !dir || !tmax || !occluded))) return MSC_ERR_ARG;
  if (n == 0) return MSC_OK;
  int rc = h->core.trace_occluded(org, dir, tmax, n, occluded);
  if (rc != MSC_OK) h->err = h->core.err;
  return rc;
}

// ------------------------------------------------------------------ host-only

int msc_obj_load(const char* path, float* positions, float* texcoords, uint32_t* indices, int64_t* sizes) {
  if (!path || !sizes) return MSC_ERR_ARG;
  ObjMesh m;
  std::string err;
  try {
    if (!obj_load_file(path, &m, &err)) {
      g_create_error = err;
      return MSC_ERR_SCENE;
    }
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
    if (!load_scene(yaml_path, &d, &err)) {
      g_create_error = err;
      return MSC_ERR_SCENE;
    }
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

// ------------------------------------------------------------------ batched

int msc_batch_create(int batch_exponent, int64_t film_samples, msc_batch** out) {
  if (!out || film_samples <= 0 || film_samples >= (1ll << 31)) {
    g_create_error = "msc_batch_create: bad argument";
    return MSC_ERR_ARG;
  }
  *out = nullptr;
  msc_batch* b = nullptr;
  try {
    b = new msc_batch();
  } catch (...) {
    g_create_error = "host out of memory";
    return MSC_ERR_CUDA;
  }
  const int e = std::max(10, std::min(batch_exponent, 24));
  b->batch_exponent = e;
  b->film_samples = film_samples;
  const int gen = (int)std::min<int64_t>(std::max<int64_t>(16ll << e, 1ll << 22), 1ll << 25);
  size_t free0 = 0, free1 = 0, total = 0;
  cudaMemGetInfo(&free0, &total);
  int rc = guarded(&b->err, [&] { return b->core.init(e, gen, (size_t)film_samples, true); });
  if (rc == MSC_OK && cudaMemGetInfo(&free1, &total) == cudaSuccess && free0 > free1)
    b->core.mem_fixed = (int64_t)(free0 - free1);  // film pool, ray pools, batch buffers
  if (rc != MSC_OK) {
    g_create_error = b->core.err.empty() ? b->err : b->core.err;
    delete b;
    return rc;
  }
  *out = b;
  return MSC_OK;
}

int msc_batch_destroy(msc_batch* b) {
  if (!b) return MSC_ERR_ARG;
  delete b;
  return MSC_OK;
}

const char* msc_batch_last_error(msc_batch* b) { return b ? b->err.c_str() : g_create_error.c_str(); }

int msc_batch_add_scene(msc_batch* b, const char* yaml_path, int* scene_id) {
  if (!b || !yaml_path || !scene_id) return MSC_ERR_ARG;
  SceneDesc d;
  std::string err;
  bool ok = false;
  try {
    ok = load_scene(yaml_path, &d, &err);
  } catch (const std::exception& e) {
    err = e.what();
  }
  if (!ok) {
    b->err = err;
    return MSC_ERR_SCENE;
  }
  if (b->core.mem_budget > 0) {
    // a scene's device bytes, estimated before it is built: triangles, BVH
    // nodes, index tables and texcoords (~160 B per triangle), face texels
    const int64_t T = (int64_t)d.tri_geom.size();
    const int64_t est = 160 * T + (int64_t)6 * d.texels.res * d.texels.res * T;
    if (b->core.mem_fixed + b->core.mem_jobs + est > b->core.mem_budget) {
      b->err = "the device-memory budget has no room for this scene";
      return MSC_ERR_BUSY;
    }
  }
  int rc = guarded(&b->err, [&] { return b->core.add_scene(d, scene_id); });
  if (rc != MSC_OK && b->err.empty()) b->err = b->core.err;
  if (rc != MSC_OK) b->err = b->core.err;
  if (rc == MSC_OK) b->core.mem_fixed += b->core.scene_bytes(*scene_id);  // the scene as built
  return rc;
}

int msc_batch_set_memory_budget(msc_batch* b, int64_t bytes) {
  if (!b || bytes < 0) return MSC_ERR_ARG;
  b->core.mem_budget = bytes;
  return MSC_OK;
}

int msc_batch_memory(msc_batch* b, int64_t* in_use, int64_t* fixed_bytes, int64_t* job_bytes) {
  if (!b) return MSC_ERR_ARG;
  if (in_use) *in_use = b->core.mem_fixed + b->core.mem_jobs;
  if (fixed_bytes) *fixed_bytes = b->core.mem_fixed;
  if (job_bytes) *job_bytes = b->core.mem_jobs;
  return MSC_OK;
}

int msc_batch_scene_info(msc_batch* b, int scene, float lo[3], float hi[3], int64_t* triangles) {
  if (!b || !lo || !hi) return MSC_ERR_ARG;
  int rc = guarded(&b->err, [&] { return b->core.scene_bounds(scene, lo, hi); });
  if (rc != MSC_OK) {
    b->err = b->core.err;
    return rc;
  }
  if (triangles) *triangles = (int64_t)b->core.scene(scene)->bvh.num_tris;
  return MSC_OK;
}

int msc_batch_submit(msc_batch* b, const msc_job_desc* desc, int* job_id) {
  if (!b || !desc || !job_id) return MSC_ERR_ARG;
  int rc = guarded(&b->err, [&] { return b->core.add_job(spec_of(*desc), job_id); });
  if (rc != MSC_OK) b->err = b->core.err;
  return rc;
}

int msc_batch_run(msc_batch* b) {
  if (!b) return MSC_ERR_ARG;
  b->core.reset_stats();
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, b->core.stream());
  int rc = guarded(&b->err, [&] { return b->core.run_all(nullptr); });
  cudaEventRecord(e1, b->core.stream());
  cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  b->last_ms = ms;
  if (rc != MSC_OK) b->err = b->core.err;
  return rc;
}

int msc_batch_job_image(msc_batch* b, int job, const float** rgb, int* width, int* height) {
  if (!b || !rgb || !width || !height) return MSC_ERR_ARG;
  JobState* j = b->core.job(job);
  if (!j || !j->complete) {
    b->err = "msc_batch_job_image: the job is not complete";
    return MSC_ERR_ARG;
  }
  if (!j->image_on_host) {
    int rc = b->core.copy_image(job);
    if (rc != MSC_OK) {
      b->err = b->core.err;
      return rc;
    }
  }
  *rgb = j->h_pixels.data();
  *width = j->rec.width;
  *height = j->rec.height;
  return MSC_OK;
}

int msc_batch_release_job(msc_batch* b, int job) {
  if (!b) return MSC_ERR_ARG;
  int rc = b->core.remove_job(job);
  if (rc != MSC_OK) b->err = b->core.err;
  return rc;
}

int msc_batch_get_stats(msc_batch* b, msc_stats* out) {
  if (!b || !out) return MSC_ERR_ARG;
  memset(out, 0, sizeof(*out));
  fill_stats(b->core.stats, b->last_ms, out);
  return MSC_OK;
}

int msc_batch_autotune(msc_batch* b, int windows) {
  if (!b || windows < 0) return MSC_ERR_ARG;
  b->core.start_autotune(windows == 0 ? 1 : windows);
  return MSC_OK;
}

static void tuning_of(Core& c, msc_tuning* out) {
  const TuneChoice t = c.choice();
  out->batch_exponent = t.batch_exp;
  out->trace_block = t.block;
  out->ray_sort = t.ray_sort ? 1 : 0;
  out->hit_sort = t.hit_sort ? 1 : 0;
  out->bins = t.bins;
  out->persistent = t.persistent ? 1 : 0;
  out->digit_bits = t.digit_bits;
  out->tuning = c.tuning() ? 1 : 0;
  out->samples = (int)c.tune_log.size();
  out->ray_key_bits = t.ray_key_bits;
}

int msc_batch_get_tuning(msc_batch* b, msc_tuning* out) {
  if (!b || !out) return MSC_ERR_ARG;
  tuning_of(b->core, out);
  return MSC_OK;
}

int msc_get_tuning(msc_handle* h, msc_tuning* out) {
  if (!h || !out) return MSC_ERR_ARG;
  std::lock_guard<std::mutex> lock(h->busy);
  tuning_of(h->core, out);
  return MSC_OK;
}

static int set_tuning(Core& core, std::string* err, const msc_tuning* in) {
  if (in->batch_exponent < 6 || (1 << std::min(in->batch_exponent, 30)) > core.batch_cap() ||
      (in->trace_block != 64 && in->trace_block != 128 && in->trace_block != 256) ||
      (in->bins != 6 && in->bins != 26 && in->bins != 98) ||
      (in->digit_bits != 4 && in->digit_bits != 8 && in->digit_bits != 11) ||
      (in->ray_key_bits != 0 && in->ray_key_bits != 8 && in->ray_key_bits != 16 && in->ray_key_bits != 24 &&
       in->ray_key_bits != 32)) {
    *err = "tuning: batch exponent above the capacity, block size not 64, 128 or 256, bins not 6, 26 or 98, "
           "digit width not 4, 8 or 11, or ray key bits not 0, 8, 16, 24 or 32";
    return MSC_ERR_ARG;
  }
  TuneChoice c;
  c.batch_exp = in->batch_exponent;
  c.block = in->trace_block;
  c.ray_sort = in->ray_sort != 0;
  c.hit_sort = in->hit_sort != 0;
  c.bins = in->bins;
  c.persistent = in->persistent != 0;
  c.digit_bits = in->digit_bits;
  c.ray_key_bits = in->ray_key_bits;
  core.stop_autotune();
  core.apply(c);
  return MSC_OK;
}

int msc_batch_set_tuning(msc_batch* b, const msc_tuning* in) {
  if (!b || !in) return MSC_ERR_ARG;
  return set_tuning(b->core, &b->err, in);
}

int msc_set_tuning(msc_handle* h, const msc_tuning* in) {
  if (!h || !in) return MSC_ERR_ARG;
  std::lock_guard<std::mutex> lock(h->busy);
  return set_tuning(h->core, &h->err, in);
}

int msc_batch_tune_log(msc_batch* b, msc_tune_sample* out, int cap, int* n) {
  if (!b || !n || cap < 0 || (cap > 0 && !out)) return MSC_ERR_ARG;
  const auto& log = b->core.tune_log;
  *n = (int)log.size();
  for (int i = 0; i < cap && i < (int)log.size(); ++i) {
    out[i].batch_exponent = log[i].choice.batch_exp;
    out[i].trace_block = log[i].choice.block;
    out[i].ray_sort = log[i].choice.ray_sort ? 1 : 0;
    out[i].hit_sort = log[i].choice.hit_sort ? 1 : 0;
    out[i].bins = log[i].choice.bins;
    out[i].persistent = log[i].choice.persistent ? 1 : 0;
    out[i].digit_bits = log[i].choice.digit_bits;
    out[i].ray_key_bits = log[i].choice.ray_key_bits;
    out[i].mrays_per_s = log[i].ms > 0 ? log[i].rays / log[i].ms / 1e3 : 0.0;
  }
  return MSC_OK;
}

int msc_batch_set_profiling(msc_batch* b, int on) {
  if (!b) return MSC_ERR_ARG;
  b->core.profiling = on != 0;
  return MSC_OK;
}

int msc_batch_set_max_active(msc_batch* b, int n) {
  if (!b || n < 0) return MSC_ERR_ARG;
  b->core.max_active = n;
  return MSC_OK;
}

// ------------------------------------------------------------------ served

int msc_serve(msc_batch* b, const msc_request* reqs, int n, msc_request_result* results, msc_serve_stats* stats) {
  return msc_serve_window(b, reqs, n, -1.0, results, stats);
}

int msc_serve_window(msc_batch* b, const msc_request* reqs, int n, double window_s, msc_request_result* results,
                     msc_serve_stats* stats) {
  if (!b || n < 0 || (n > 0 && (!reqs || !results)) || !stats) return MSC_ERR_ARG;
  return guarded(&b->err, [&]() -> int {
    Core& c = b->core;
    c.reset_stats();
    std::vector<int> order((size_t)n);
    for (int i = 0; i < n; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int a, int x) { return reqs[a].arrival_s < reqs[x].arrival_s; });
    std::vector<int> job_of((size_t)n, -1);
    size_t next = 0;
    int finished = 0;
    uint64_t peak_samples = 0;
    const double t0 = c.now();
    for (int i = 0; i < n; ++i) {
      memset(&results[i], 0, sizeof(results[i]));
      results[i].job_id = -1;
      results[i].status = 1;  // pending
    }
    std::vector<int> live;  // request indices admitted and not finished
    int not_admitted = 0;
    while (finished < n) {
      const double t = c.now() - t0;
      if (window_s >= 0.0 && t >= window_s && next < order.size()) {
        // admission has closed: what has not been admitted is not served
        for (; next < order.size(); ++next) {
          const int r = order[next];
          results[r].status = MSC_ERR_BUSY;
          results[r].done_s = t;
          ++finished;
          ++not_admitted;
        }
        if (finished >= n) break;
      }
      // admit arrived requests in arrival order while their film fits
      while (next < order.size() && reqs[order[next]].arrival_s <= t) {
        const int r = order[next];
        int jid = -1;
        int rc = c.add_job(spec_of(reqs[r].job), &jid);
        if (rc == MSC_ERR_BUSY) break;  // wait for memory to free up
        if (rc != MSC_OK) {
          results[r].status = rc;
          results[r].done_s = t;
          ++finished;
          ++next;
          continue;
        }
        job_of[r] = jid;
        results[r].job_id = jid;
        results[r].admit_s = t;
        live.push_back(r);
        ++next;
      }
      peak_samples = std::max<uint64_t>(peak_samples, c.sample_capacity() - c.samples_free());
      bool idle = false;
      int rc = c.step(&idle);
      if (rc != MSC_OK) {
        b->err = c.err;
        return rc;
      }
      // hand back finished jobs: image to host, film released for new admissions
      for (size_t k = 0; k < live.size();) {
        const int r = live[k];
        JobState* j = c.job(job_of[r]);
        if (j->complete) {
          rc = c.copy_image(job_of[r]);
          if (rc != MSC_OK) {
            b->err = c.err;
            return rc;
          }
          c.remove_job(job_of[r]);
          const double td = c.now() - t0;
          results[r].done_s = td;
          results[r].latency_s = td - reqs[r].arrival_s;
          results[r].status = 0;
          ++finished;
          live[k] = live.back();
          live.pop_back();
        } else {
          ++k;
        }
      }
      if (idle && live.empty() && next < order.size()) {
        const double wait = reqs[order[next]].arrival_s - (c.now() - t0);
        if (wait > 0) std::this_thread::sleep_for(std::chrono::duration<double>(std::min(wait, 0.002)));
      }
    }
    c.sync_stream();
    const double makespan = c.now() - t0;
    std::vector<double> lat;
    for (int i = 0; i < n; ++i)
      if (results[i].status == 0) lat.push_back(results[i].latency_s);
    std::sort(lat.begin(), lat.end());
    auto pct = [&](double p) {
      if (lat.empty()) return 0.0;
      size_t k = (size_t)std::min<double>((double)lat.size() - 1, std::ceil(p * lat.size()) - 1);
      return lat[k];
    };
    memset(stats, 0, sizeof(*stats));
    stats->completed = (int)lat.size();
    stats->wall_s = makespan;
    stats->p50_s = pct(0.50);
    stats->p99_s = pct(0.99);
    stats->p999_s = pct(0.999);
    stats->closest_queries = c.stats.closest;
    stats->shadow_queries = c.stats.shadow;
    stats->mrays_per_s = makespan > 0 ? (double)(c.stats.closest + c.stats.shadow) / makespan / 1e6 : 0.0;
    stats->peak_film_samples = (int64_t)peak_samples;
    stats->gpu_busy_s = c.stats.busy_ms / 1e3;
    stats->not_admitted = not_admitted;
    return MSC_OK;
  });
}

}  // extern "C"
