// Render core: see core.h.  Restates Pathtracer::process
// (src/core/Pathtracer.cpp:425-493) as a device-resident wavefront over the
// rays of any number of jobs.
#include "core.h"

#include <algorithm>
#include <chrono>
#include <cstring>

namespace mscg {

namespace {

// Bits of the ray sort key the batch sort orders by (the top ones): a ray's
// order within a batch only shapes traversal coherence, and the top 16 bits
// of the interleaved key (three levels of origin and direction under the
// bin) carry nearly all of it in two sort passes instead of four.  With
// several resident scenes the (scene, bin) prefix takes more of the key, so
// the sort keeps 24 bits.
constexpr int kRayKeyBits = 16;
constexpr int kRayKeyBitsScenes = 24;

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
  if (d_spheres) cudaFree(d_spheres);
  if (d_sphere_light) cudaFree(d_sphere_light);
  if (d_texels) cudaFree(d_texels);
  if (d_tex_nodes) cudaFree(d_tex_nodes);
  if (d_tex_ops) cudaFree(d_tex_ops);
  if (d_tex_images) cudaFree(d_tex_images);
  if (d_tex_texels) cudaFree(d_tex_texels);
  if (d_tri_uv) cudaFree(d_tri_uv);
  if (d_shade_rank) cudaFree(d_shade_rank);
}

namespace {
// Post-order program of the texture tree rooted at `node`.
void emit_tex_program(const std::vector<TexNode>& nodes, int node, std::vector<int2>* ops) {
  const TexNode& t = nodes[node];
  if (t.type == TEXNODE_LAYERED) {
    emit_tex_program(nodes, t.upper, ops);
    emit_tex_program(nodes, t.lower, ops);
    emit_tex_program(nodes, t.mask, ops);
    ops->push_back(make_int2(2, node));
  } else {
    ops->push_back(make_int2(t.type == TEXNODE_STANDARD ? 1 : 0, node));
  }
}
}  // namespace

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
  if (graph_) cudaGraphExecDestroy(graph_);
  if (drain_graph_) cudaGraphExecDestroy(drain_graph_);
  if (h_ctr_) cudaFreeHost(h_ctr_);
  for (auto e : busy_ev_)
    if (e) cudaEventDestroy(e);
  for (auto e : tune_ev_)
    if (e) cudaEventDestroy(e);
  for (int i = 0; i < kGraphBodies; ++i) {
    if (fork_ev_[i]) cudaEventDestroy(fork_ev_[i]);
    if (join_ev_[i]) cudaEventDestroy(join_ev_[i]);
  }
  if (side_) cudaStreamDestroy(side_);
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
  batch_size_ = batch_cap_;
  generation_ = std::max(generation, batch_cap_);
  staging_cap_ = std::max(batch_cap_, std::min(generation_, 4 * batch_cap_));
  sample_cap_ = std::max<size_t>(sample_capacity, 1);
  if (sample_cap_ >= (1ull << 31)) {
    err = "the film pool holds at most 2^31 - 1 samples";
    return MSC_ERR_ARG;
  }
  CK(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
  CK(cudaStreamCreateWithFlags(&side_, cudaStreamNonBlocking));
  for (int i = 0; i < kGraphBodies; ++i) {
    CK(cudaEventCreateWithFlags(&fork_ev_[i], cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&join_ev_[i], cudaEventDisableTiming));
  }
  CK(cudaEventCreate(&tune_ev_[0]));
  CK(cudaEventCreate(&tune_ev_[1]));
  CK(cudaEventCreate(&busy_ev_[0]));
  CK(cudaEventCreate(&busy_ev_[1]));
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
  const size_t chunks = bin_pool_chunks((size_t)G, (size_t)B);
  const int max_chunks = (int)(((size_t)G + kChunk - 1) / kChunk) + 1;
  const size_t pool_rays = chunks * (size_t)kChunk;
  const int pend_cols = B / kChunk + 2;              // new chunks one batch's appends can take per bin
  const int retire_cap = B / kChunk + kMaxBins + 1;  // chunks one batch can hold back
  size_t bytes = 3 * al256(pool_rays * sizeof(float4)) + 3 * al256((size_t)B * sizeof(float4)) +
                 2 * al256((size_t)kMaxBins * 4) + al256((size_t)kMaxBins * max_chunks * 4) + al256(chunks * 4) +
                 al256(4) +
                 10 * al256((size_t)B * 4) + al256(sizeof(Counters)) +
                 al256(pool_rays * 4) + al256(sizeof(BatchPlan)) +
                 sort_scratch_bytes(B, 11) + al256((size_t)B * sizeof(float4)) + 6 * al256((size_t)B * sizeof(float4)) +
                 al256((size_t)(kMaxBins + 1) * part_tiles * 4) + al256((size_t)kMaxBins * 4) +
                 al256((size_t)kMaxBins * pend_cols * 4) + al256((size_t)retire_cap * 4) + al256(4) + al256((size_t)S) +
                 4096;
  CK(cudaMalloc(&arena_, bytes));
  Arena A{arena_, 0};
  bins_.rays.o = A.take<float4>(pool_rays);
  bins_.rays.d = A.take<float4>(pool_rays);
  bins_.rays.w = A.take<float4>(pool_rays);
  bins_.keys = A.take<uint32_t>(pool_rays);
  bins_.num_chunks = (int)chunks;
  bins_.max_chunks = max_chunks;
  bins_.held = A.take<int>(kMaxBins);
  bins_.table = A.take<int>((size_t)kMaxBins * max_chunks);
  bins_.free_stack = A.take<int>(chunks);
  bins_.free_top = A.take<int>(1);
  A.take<int>(kMaxBins);  // spare
  // continuing rays of batches too small for direct binning
  staging_.o = A.take<float4>(B);
  staging_.d = A.take<float4>(B);
  staging_.w = A.take<float4>(B);
  slots_ = A.take<int>(B);
  keys_ = A.take<uint32_t>(B);
  keys_sorted_ = A.take<uint32_t>(B);
  perm_ = A.take<uint32_t>(B);
  hkeys_ = A.take<uint32_t>(B);
  hkeys_sorted_ = A.take<uint32_t>(B);
  hperm_ = A.take<uint32_t>(B);
  hhi_ = A.take<uint32_t>(B);
  hhi_g_ = A.take<uint32_t>(B);
  hperm1_ = A.take<uint32_t>(B);
  ctr_ = A.take<Counters>(1);
  trace_counter_ = A.take<int>(2);
  plan_ = A.take<BatchPlan>(1);
  sort_scratch_bind(&ss_, A.take<char>(sort_scratch_bytes(B, 11)), B, 11);
  hits_ = A.take<float4>(B);
  for (int q = 0; q < 2; ++q) {
    shadow_[q].o = A.take<float4>(B);
    shadow_[q].d = A.take<float4>(B);
    shadow_[q].c = A.take<float4>(B);
  }
  bins_.tile_counts = A.take<uint32_t>((size_t)(kMaxBins + 1) * part_tiles);
  bins_.max_tiles = part_tiles;
  bins_.cursor = A.take<int>(kMaxBins);
  bins_.pend = A.take<int>((size_t)kMaxBins * pend_cols);
  bins_.pend_cols = pend_cols;
  bins_.retired = A.take<int>(retire_cap);
  bins_.retire_cap = retire_cap;
  bins_.n_retired = A.take<int>(1);
  cam_digits_ = A.take<uint8_t>(S);
  bins_.count = ctr_->bin_count;
  bins_.in_bins = &ctr_->in_bins;
  bins_.err = &ctr_->err;
  if (A.used > bytes) {
    err = "internal: device arena overflow";
    return MSC_ERR_CUDA;
  }
  CK(cudaMemset(ctr_, 0, sizeof(Counters)));
  CK(cudaMemset(plan_, 0, sizeof(BatchPlan)));
  persistent_grids_init();
  sort_init();
  launch_pool_reset(bins_, stream_);
  CK(cudaMemsetAsync(bins_.keys, 0, (size_t)bins_.num_chunks * kChunk * 4, stream_));
  // every pool record starts as a well-formed ray (job, scene and sample 0),
  // so that no position ever reads as out-of-range indices
  CK(cudaMemsetAsync(bins_.rays.o, 0, pool_rays * sizeof(float4), stream_));
  CK(cudaMemsetAsync(bins_.rays.d, 0, pool_rays * sizeof(float4), stream_));
  CK(cudaMemsetAsync(bins_.rays.w, 0, pool_rays * sizeof(float4), stream_));
  CK(cudaStreamSynchronize(stream_));
  CK(cudaMallocHost(&h_ctr_, sizeof(Counters)));
  memset(h_ctr_, 0, sizeof(Counters));
  return MSC_OK;
}

int Core::scene_bounds(int id, float lo[3], float hi[3]) {
  SceneGPU* sg = scene(id);
  if (!sg) {
    err = "no such scene";
    return MSC_ERR_ARG;
  }
  float b[8];
  CK(cudaMemcpyAsync(b, sg->bvh.bounds_dev, sizeof(b), cudaMemcpyDeviceToHost, stream_));
  CK(cudaStreamSynchronize(stream_));
  for (int i = 0; i < 3; ++i) {
    lo[i] = b[i];
    hi[i] = b[3 + i];
  }
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
  // image textures: programs into the shader records, nodes, images, texcoords
  std::vector<int2> tex_ops;
  for (auto& sh : d.shaders) {
    if (sh.texture != TEXTURE_TREE) continue;
    sh.tex_prog = (int)tex_ops.size();
    emit_tex_program(d.tex_nodes, sh.tex_root, &tex_ops);
    sh.tex_len = (int)tex_ops.size() - sh.tex_prog;
  }
  if (!tex_ops.empty()) {
    std::vector<int4> ims;
    std::vector<float4> tx;
    for (const auto& im : d.images) {
      ims.push_back(make_int4((int)tx.size(), im.width, im.height, 0));
      for (size_t i = 0; i < (size_t)im.width * im.height; ++i)
        tx.push_back(make_float4(im.rgb[3 * i], im.rgb[3 * i + 1], im.rgb[3 * i + 2], 0.f));
    }
    if (ims.empty()) ims.push_back(make_int4(0, 1, 1, 0));
    if (tx.empty()) tx.push_back(make_float4(0.f, 0.f, 0.f, 0.f));
    std::vector<float> uv(d.tri_uv);
    uv.resize((size_t)6 * T, 0.f);
    CK(cudaMalloc(&sg->d_tex_nodes, d.tex_nodes.size() * sizeof(TexNode)));
    CK(cudaMalloc(&sg->d_tex_ops, tex_ops.size() * sizeof(int2)));
    CK(cudaMalloc(&sg->d_tex_images, ims.size() * sizeof(int4)));
    CK(cudaMalloc(&sg->d_tex_texels, tx.size() * sizeof(float4)));
    CK(cudaMalloc(&sg->d_tri_uv, uv.size() * sizeof(float)));
    CK(cudaMemcpy(sg->d_tex_nodes, d.tex_nodes.data(), d.tex_nodes.size() * sizeof(TexNode), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(sg->d_tex_ops, tex_ops.data(), tex_ops.size() * sizeof(int2), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(sg->d_tex_images, ims.data(), ims.size() * sizeof(int4), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(sg->d_tex_texels, tx.data(), tx.size() * sizeof(float4), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(sg->d_tri_uv, uv.data(), uv.size() * sizeof(float), cudaMemcpyHostToDevice));
  }
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
  r.hit_key_bits = d.ext.hit_key_bits;
  r.tex_nodes = sg->d_tex_nodes;
  r.tex_ops = sg->d_tex_ops;
  r.tex_images = sg->d_tex_images;
  r.tex_texels = sg->d_tex_texels;
  r.tri_uv = sg->d_tri_uv;
  {  // the ray sort key quantises origins in the scene box
    float b[8];
    CK(cudaMemcpy(b, sg->bvh.bounds_dev, sizeof(b), cudaMemcpyDeviceToHost));
    float sc[3];
    for (int a = 0; a < 3; ++a) {
      const float e = b[3 + a] - b[a];
      sc[a] = e > 0.f ? 64.0f / e : 0.f;
    }
    r.key_lo = make_float4(b[0], b[1], b[2], 0.f);
    r.key_scale = make_float4(sc[0], sc[1], sc[2], 0.f);
  }
  if (!d.sphere_lights.empty()) {
    std::vector<float4> sp;
    for (int li : d.sphere_lights) {
      const LightRec& L = d.lights[li];
      sp.push_back(make_float4(L.centre[0], L.centre[1], L.centre[2], L.radius));
    }
    CK(cudaMalloc(&sg->d_spheres, sp.size() * sizeof(float4)));
    CK(cudaMalloc(&sg->d_sphere_light, sp.size() * sizeof(int)));
    CK(cudaMemcpy(sg->d_spheres, sp.data(), sp.size() * sizeof(float4), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(sg->d_sphere_light, d.sphere_lights.data(), sp.size() * sizeof(int), cudaMemcpyHostToDevice));
    r.spheres = sg->d_spheres;
    r.sphere_light = sg->d_sphere_light;
    r.num_spheres = (int)sp.size();
  }
  if (d.texels.res > 0) {
    const size_t count = (size_t)T * d.texels.res * d.texels.res * 3;
    CK(cudaMalloc(&sg->d_texels, count * sizeof(unsigned short)));
    launch_face_texels(sg->d_texels, (int64_t)T, d.texels.res, d.texels.seed, stream_);
    CK(cudaStreamSynchronize(stream_));
    CK(cudaGetLastError());
    r.texel_res = d.texels.res;
    r.texels = sg->d_texels;
  }
  if (d.ext.hit_key_bits == 64 && T < (1 << 23)) {
    // The 64-bit hit key is shader id (12 bits) | face id (23 bits) | quantised uv.
    // Its top 35 bits order a batch's hits by (shader, face); the rank of each
    // triangle in that order gives the same grouping from a sort of
    // ceil(log2(T + 1)) bits (three 8-bit digit passes for 8 M triangles)
    // instead of two 32-bit sorts.  Hits on the same face keep their batch
    // order (the uv bits only split such ties).  Counting sort by shader
    // over the faces in original order:
    std::vector<uint32_t> shader_of(T), start(4097, 0), rank(T);
    for (int o = 0; o < T; ++o) {
      const int g = tg[o];
      shader_of[o] = (g >= 0 && g < (int)geoms.size()) ? (uint32_t)(geoms[g].shader & 0xfff) : 0u;
      ++start[shader_of[o] + 1];
    }
    for (int s = 0; s < 4096; ++s) start[s + 1] += start[s];
    for (int o = 0; o < T; ++o) rank[o] = start[shader_of[o]]++;
    std::vector<uint32_t> leaf(T);
    for (int k = 0; k < T; ++k) leaf[k] = rank[sg->h_tri_orig[k]] + 1u;
    CK(cudaMalloc(&sg->d_shade_rank, (size_t)T * sizeof(uint32_t)));
    CK(cudaMemcpy(sg->d_shade_rank, leaf.data(), (size_t)T * sizeof(uint32_t), cudaMemcpyHostToDevice));
    r.shade_rank = sg->d_shade_rank;
    r.shade_rank_bits = 32 - __builtin_clz((uint32_t)T);  // keys lie in [0, T]
  }
  if ((uint64_t)total_tris_ + (uint64_t)T + 1 >= (1ull << 32)) {
    err = "too many triangles across resident scenes";
    return MSC_ERR_ARG;
  }
  {  // what the scene holds on the device, for the batch's memory budget
    int64_t b = (int64_t)T * (3 * sizeof(float4) + sizeof(int)) + 8 * sizeof(float);  // triangles, index, box
    b += sg->bvh.wnodes ? (int64_t)sg->bvh.num_wnodes * 5 * sizeof(uint4)
                        : (int64_t)std::max(T - 1, 0) * 4 * sizeof(float4);
    b += (int64_t)std::max<size_t>(1, d.shaders.size()) * sizeof(ShaderRec) +
         (int64_t)std::max<size_t>(1, geoms.size()) * sizeof(GeomRec) +
         (int64_t)std::max<size_t>(1, d.lights.size()) * sizeof(LightRec);
    b += (int64_t)d.sphere_lights.size() * (sizeof(float4) + sizeof(int));
    if (d.texels.res > 0) b += (int64_t)T * d.texels.res * d.texels.res * 3 * sizeof(unsigned short);
    if (sg->d_tri_uv) {
      b += (int64_t)6 * T * sizeof(float) + (int64_t)d.tex_nodes.size() * sizeof(TexNode) +
           (int64_t)tex_ops.size() * sizeof(int2);
      for (const auto& im : d.images) b += (int64_t)im.width * im.height * sizeof(float4) + sizeof(int4);
    }
    if (sg->d_shade_rank) b += (int64_t)T * sizeof(uint32_t);
    sg->bytes = b;
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
  const int64_t image_bytes = (int64_t)3 * rec.width * rec.height * (int64_t)sizeof(float);
  if (mem_budget > 0 && mem_fixed + mem_jobs + image_bytes > mem_budget) {
    err = "the device-memory budget has no room for this job's image yet";
    return MSC_ERR_BUSY;
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
  mem_jobs += image_bytes;
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
  if (j->d_pixels) {
    cudaFreeAsync(j->d_pixels, stream_);
    mem_jobs -= (int64_t)3 * j->rec.width * j->rec.height * (int64_t)sizeof(float);
  }
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

void Core::mark_busy() {
  if (busy_open_ || !busy_ev_[0]) return;
  if (cudaEventRecord(busy_ev_[0], stream_) == cudaSuccess) busy_open_ = true;
}

void Core::close_busy() {
  if (busy_open_ && cudaEventRecord(busy_ev_[1], stream_) != cudaSuccess) busy_open_ = false;
}

cudaError_t Core::sync_stream() {
  close_busy();
  const cudaError_t e = cudaStreamSynchronize(stream_);
  settle_busy();
  return e;
}

void Core::settle_busy() {
  if (!busy_open_) return;
  float ms = 0.f;
  if (cudaEventElapsedTime(&ms, busy_ev_[0], busy_ev_[1]) == cudaSuccess) stats.busy_ms += ms;
  busy_open_ = false;
}

int Core::finish_job(JobState& j) {
  mark_busy();
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
  mark_busy();
  CK(cudaMemcpyAsync(j->h_pixels.data(), j->d_pixels, j->h_pixels.size() * sizeof(float), cudaMemcpyDeviceToHost,
                     stream_));
  close_busy();
  CK(cudaStreamSynchronize(stream_));
  settle_busy();
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
  if (want < std::min<uint64_t>((uint64_t)batch_size_, left_total)) return MSC_OK;
  uint64_t filled = 0;
  mark_busy();
  StageClock t(this, MSC_STAGE_RAYGEN);
  int launches = 0;
  for (auto& jp : jobs_) {
    JobState& j = *jp;
    if (j.slot < 0 || j.complete || j.generated >= j.paths) continue;
    const uint64_t n = std::min<uint64_t>(want - filled, j.paths - j.generated);
    if (n == 0) break;
    // the camera rays go straight into their bins, in sample order
    // (Camera.cpp:42-44, DirectionalBins::add), made twice instead of staged
    launches += launch_camera_rays(j.rec, j.slot, (uint32_t)j.generated, (int)n, film_, bins_,
                                   ray_sort ? d_scenes_ : nullptr, cam_digits_, stream_);
    j.generated += n;
    filled += n;
    if (filled >= want) break;
  }
  t.done(launches);
  if (filled > 0) {
    stats.generations += 1;
    *did = true;
  }
  return MSC_OK;
}

uint64_t Core::graph_key() const {
  const uint64_t ns = scenes_.size();  // <= 256
  const uint64_t k64 = (ns == 1 && scenes_[0]->rec.hit_key_bits == 64) ? 1 : 0;
  uint64_t bexp = 0;
  while ((1 << (bexp + 1)) <= batch_size_) ++bexp;
  const uint64_t block = trace_block == 64 ? 0 : (trace_block == 128 ? 1 : 2);
  const uint64_t bins = bins_.nbins == 6 ? 0 : (bins_.nbins == 26 ? 1 : 2);
  const uint64_t pers = persistent_trace ? 1 : 0;
  const uint64_t dig = sort_digits == 4 ? 0 : (sort_digits == 8 ? 1 : 2);
  const uint64_t kb = (uint64_t)ray_key_bits_used() / 8;  // 1 to 4
  return ns | (k64 << 9) | ((uint64_t)hit_bits_ << 10) | ((uint64_t)ray_sort << 16) | ((uint64_t)hit_sort << 17) |
         ((uint64_t)merge_bins << 18) | ((uint64_t)wide_ << 19) | (bexp << 20) | (block << 25) | (bins << 27) |
         (pers << 29) | (dig << 30) | (kb << 32) | (1ull << 63);
}

void Core::drop_graph() {
  if (graph_) cudaGraphExecDestroy(graph_);
  graph_ = nullptr;
  graph_key_ = 0;
  if (drain_graph_) cudaGraphExecDestroy(drain_graph_);
  drain_graph_ = nullptr;
  drain_key_ = 0;
}

// One batch body.  Every size is read on the device from the plan, so the
// same launches serve any batch and can be captured once.
int Core::enqueue_batch(int index, bool overlap) {
  cudaStream_t st = stream_;
  const SceneRec& s0 = scenes_[0]->rec;
  const int ns = (int)scenes_.size();
  const int B = batch_size_;
  const int* nb = &plan_->nb;
  int* errw = &ctr_->err;
  const int q = index & 1;
  int* shc = &ctr_->shadow_count[q];
  int scene_bits = 0;
  while ((1 << scene_bits) < ns) ++scene_bits;
  // direct binning: the shading appends the continuing rays into the bins
  const bool direct = B >= kDirectMin;
  {
    StageClock t(this, MSC_STAGE_OTHER);
    t.done(launch_plan(bins_, B, merge_bins ? 1 : 0, scene_bits, plan_, ctr_, st, direct));
  }
  // traversal and shading read the batch's rays where the bins hold them
  // (RayDecompress, RayDecompress.cpp:5-29, needs no copy here), through the
  // pool index of each ray in sorted order: sorted as the values beside the
  // keys, or listed in batch order without the ray sort
  if (ray_sort) {
    // with 8-bit digits (and a key of whole digits) the key kernel also
    // counts the sort's digits
    const bool fused = sort_digits == 8 && ray_key_bits_used() % 8 == 0;
    {
      StageClock t(this, MSC_STAGE_RAYKEYS);
      if (fused) CK(cudaMemsetAsync(ss_.hist, 0, (size_t)kSortHistWords * 4 + 64, st));
      t.done(launch_ray_keys(bins_, plan_, B, ray_key_bits_used(), keys_, st, perm_, fused ? ss_.hist : nullptr));
    }
    StageClock t(this, MSC_STAGE_RAYSORT);
    const int l = sort_pairs(keys_, perm_, keys_sorted_, reinterpret_cast<uint32_t*>(slots_), B, ray_key_bits_used(),
                             ss_, st, errw, nb, sort_digits, nullptr, fused);
    if (l < 0) {
      err = "internal: ray sort without distinct outputs";
      return MSC_ERR_CUDA;
    }
    t.done(l);
  } else {
    StageClock t(this, MSC_STAGE_GATHER);
    t.done(launch_batch_slots(bins_, plan_, B, nullptr, slots_, st));
  }
  const RayBuf& rays = bins_.rays;
  const int* slots = slots_;
  {
    StageClock t(this, MSC_STAGE_TRACE);
    t.done(launch_trace_closest(d_scenes_, ns, s0, rays.o, rays.d, slots, B, hits_, errw, st, nb, trace_block,
                                persistent_trace ? trace_counter_ : nullptr));
  }
  const uint32_t* order = nullptr;
  if (hit_sort && ns == 1 && s0.hit_key_bits == 64 && s0.shade_rank) {
    // 64-bit key scenes: the (shader, face) order from the rank table
    StageClock t(this, MSC_STAGE_HITSORT);
    int l = launch_hit_keys_rank(d_scenes_, hits_, B, hkeys_, st, nb);
    const int ls = sort_pairs(hkeys_, nullptr, hkeys_sorted_, hperm_, B, s0.shade_rank_bits, ss_, st, errw, nb,
                              sort_digits);
    if (ls < 0) {
      err = "internal: hit sort without distinct outputs";
      return MSC_ERR_CUDA;
    }
    t.done(l + ls);
    order = hperm_;
  } else if (hit_sort && ns == 1 && s0.hit_key_bits == 64) {
    // 64-bit key: stable by the low word, then stable by the high word
    StageClock t(this, MSC_STAGE_HITSORT);
    int l = launch_hit_keys64(d_scenes_, hits_, B, hkeys_, hhi_, st, nb);
    const int l1 = sort_pairs(hkeys_, nullptr, hkeys_sorted_, hperm1_, B, 32, ss_, st, errw, nb, sort_digits);
    l += launch_gather_u32(hhi_, hperm1_, B, hhi_g_, st, nb);
    const int l2 = sort_pairs(hhi_g_, hperm1_, hhi_, hperm_, B, 32, ss_, st, errw, nb, sort_digits);
    if (l1 < 0 || l2 < 0) {
      err = "internal: hit sort without distinct outputs";
      return MSC_ERR_CUDA;
    }
    t.done(l + l1 + l2);
    order = hperm_;
  } else if (hit_sort) {
    StageClock t(this, MSC_STAGE_HITSORT);
    int l = launch_hit_keys(d_scenes_, rays.d, slots, hits_, B, hkeys_, st, nb);
    const int ls = sort_pairs(hkeys_, nullptr, hkeys_sorted_, hperm_, B, hit_bits_, ss_, st, errw, nb, sort_digits);
    if (ls < 0) {
      err = "internal: hit sort without distinct outputs";
      return MSC_ERR_CUDA;
    }
    t.done(l + ls);
    order = hperm_;
  }
  if (overlap && index > 0) CK(cudaStreamWaitEvent(st, join_ev_[index - 1], 0));  // the previous occlusion
  {
    StageClock t(this, MSC_STAGE_SHADE);
    CK(cudaMemsetAsync(shc, 0, sizeof(int), st));
    t.done(launch_shade(d_scenes_, d_jobs_, film_, rays, slots, hits_, order, B, staging_, shadow_[q], shc, d_job_done_,
                        st, nb, direct ? &bins_ : nullptr, (direct && ray_sort) ? d_scenes_ : nullptr));
  }
  {
    StageClock t(this, MSC_STAGE_SHADOW);
    cudaStream_t ss = st;
    if (overlap) {
      CK(cudaEventRecord(fork_ev_[index], st));
      CK(cudaStreamWaitEvent(side_, fork_ev_[index], 0));
      ss = side_;
    }
    t.done(launch_trace_shadow(d_scenes_, ns, s0, shadow_[q], shc, B, film_.rgb, errw, ss, &ctr_->shadow,
                               trace_block, persistent_trace ? trace_counter_ + 1 : nullptr));
    if (overlap) CK(cudaEventRecord(join_ev_[index], side_));
  }
  {
    StageClock t(this, MSC_STAGE_BINS);
    if (direct) t.done(launch_append_commit(bins_, st));
    else t.done(launch_bin_partition(staging_, B, bins_, st, nb, ray_sort ? d_scenes_ : nullptr));
  }
  return MSC_OK;
}

// Captures and instantiates the batch graph for the current choice if needed,
// and (for batches above kDrainBatch) the drain graph: the same bodies sized
// for kDrainBatch rays, replayed once the bins hold no more than that, so the
// small batches of a pass's end launch grids 8 or more times smaller.
int Core::ensure_graph() {
  if (profiling || !use_graph) return MSC_OK;
  int rc = capture_graph(&graph_, &graph_key_, &graph_launches_);
  if (rc != MSC_OK || batch_size_ <= kDrainBatch) return rc;
  const int full = batch_size_;
  batch_size_ = kDrainBatch;
  rc = capture_graph(&drain_graph_, &drain_key_, &drain_launches_);
  batch_size_ = full;
  return rc;
}

int Core::capture_graph(cudaGraphExec_t* exec, uint64_t* exec_key, int* exec_launches) {
  const uint64_t key = graph_key();
  if (!*exec || *exec_key != key) {
    if (*exec) cudaGraphExecDestroy(*exec);
    *exec = nullptr;
    *exec_key = 0;
    cudaGraph_t g = nullptr;
    const uint64_t launches0 = stats.launches;
    uint64_t stage0[12];
    memcpy(stage0, stats.stage_launches, sizeof(stage0));
    CK(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal));
    int rc = MSC_OK;
    for (int i = 0; i < kGraphBodies && rc == MSC_OK; ++i) rc = enqueue_batch(i, true);
    if (rc == MSC_OK && cudaStreamWaitEvent(stream_, join_ev_[kGraphBodies - 1], 0) != cudaSuccess) {
      err = "joining the occlusion stream in the batch graph";
      rc = MSC_ERR_CUDA;
    }
    cudaError_t ce = cudaStreamEndCapture(stream_, &g);
    if (rc != MSC_OK) {
      if (g) cudaGraphDestroy(g);
      return rc;
    }
    if (ce != cudaSuccess) {
      err = std::string("capturing the batch body: ") + cudaGetErrorString(ce);
      return MSC_ERR_CUDA;
    }
    ce = cudaGraphInstantiate(exec, g, 0);
    cudaGraphDestroy(g);
    if (ce != cudaSuccess) {
      *exec = nullptr;
      err = std::string("instantiating the batch graph: ") + cudaGetErrorString(ce);
      return MSC_ERR_CUDA;
    }
    *exec_launches = (int)(stats.launches - launches0);
    stats.launches = launches0;  // counted per replay below
    memcpy(stats.stage_launches, stage0, sizeof(stage0));
    *exec_key = key;
  }
  return MSC_OK;
}

int Core::run_batches(int k, bool drain) {
  mark_busy();
  if (profiling || !use_graph) {
    for (int i = 0; i < k; ++i) {
      int rc = enqueue_batch(i, false);
      if (rc != MSC_OK) return rc;
    }
    CK(cudaGetLastError());
    return MSC_OK;
  }
  const int grc = ensure_graph();
  if (grc != MSC_OK) return grc;
  const bool small = drain && drain_graph_ != nullptr;
  const int replays = (k + kGraphBodies - 1) / kGraphBodies;  // bodies past the work plan empty batches
  for (int i = 0; i < replays; ++i) CK(cudaGraphLaunch(small ? drain_graph_ : graph_, stream_));
  stats.launches += (uint64_t)(small ? drain_launches_ : graph_launches_) * (uint64_t)replays;
  stats.graph_replays += (uint64_t)replays;
  return MSC_OK;
}

void Core::reset_stats() {
  stats = CoreStats();
  if (ctr_) {
    cudaMemsetAsync(&ctr_->closest, 0, 3 * sizeof(unsigned long long), stream_);
    h_ctr_->closest = h_ctr_->shadow = h_ctr_->batches = 0;
  }
}

int Core::step(bool* idle) {
  *idle = false;
  cudaStream_t st = stream_;
  CK(cudaMemcpyAsync(h_ctr_, ctr_, sizeof(Counters), cudaMemcpyDeviceToHost, st));
  if (max_slot_ >= 0)
    CK(cudaMemcpyAsync(h_job_done_, d_job_done_, (size_t)(max_slot_ + 1) * sizeof(uint32_t), cudaMemcpyDeviceToHost,
                       st));
  close_busy();
  CK(cudaStreamSynchronize(st));
  settle_busy();
  if (profiling) harvest();
  stats.closest = h_ctr_->closest;
  stats.shadow = h_ctr_->shadow;
  stats.batches = h_ctr_->batches;
  if (h_ctr_->err != 0) {
    const int e = h_ctr_->err;
    err = (e & ERR_BIN_OVERFLOW)    ? "a direction bin overflowed"
          : (e & ERR_APPEND_WAIT)   ? "a bin append waited past its cap for a chunk"
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
  // enough batch bodies to take what the bins hold now (the device plans each one)
  uint64_t total = 0, need = 0;
  const uint64_t bs = (uint64_t)batch_size_;
  for (int b = 0; b < kMaxBins; ++b) {
    const uint64_t c = (uint64_t)std::max(0, h_ctr_->bin_count[b]);
    total += c;
    need += (c + bs - 1) / bs;
  }
  if (total == 0) {
    *idle = true;
    return MSC_OK;
  }
  if (merge_bins) need = (total + bs - 1) / bs;
  const int k = (int)std::min<uint64_t>(std::max<uint64_t>(need, 1), (uint64_t)std::max(1, max_batches_per_step));
  return run_batches(k, merge_bins && total <= (uint64_t)kDrainBatch);
}

TuneChoice Core::choice() const {
  TuneChoice c;
  int e = 0;
  while ((1 << (e + 1)) <= batch_size_) ++e;
  c.batch_exp = e;
  c.block = trace_block;
  c.ray_sort = ray_sort;
  c.hit_sort = hit_sort;
  c.bins = bins_.nbins;
  c.persistent = persistent_trace;
  c.digit_bits = sort_digits;
  c.ray_key_bits = ray_key_bits;
  return c;
}

int Core::ray_key_bits_used() const {
  if (ray_key_bits == 8 || ray_key_bits == 16 || ray_key_bits == 24 || ray_key_bits == 32) return ray_key_bits;
  return scenes_.size() > 1 ? kRayKeyBitsScenes : kRayKeyBits;
}

void Core::apply(const TuneChoice& c) {
  const int e = std::max(6, std::min(c.batch_exp, 24));
  batch_size_ = std::min(1 << e, batch_cap_);
  trace_block = (c.block == 64 || c.block == 256) ? c.block : 128;
  ray_sort = c.ray_sort;
  hit_sort = c.hit_sort;
  bins_.nbins = (c.bins == 26 || c.bins == 98) ? c.bins : 6;
  persistent_trace = c.persistent;
  sort_digits = (c.digit_bits == 4 || c.digit_bits == 11) ? c.digit_bits : 8;
  ray_key_bits = (c.ray_key_bits == 8 || c.ray_key_bits == 16 || c.ray_key_bits == 24 || c.ray_key_bits == 32)
                     ? c.ray_key_bits
                     : 0;
}

void Core::start_autotune(int windows) {
  tune_windows_ = std::max(1, windows);
  tune_active_ = true;
  tune_dim_ = 0;
  tune_log.clear();
  tune_begin_dim();
}

// Candidates along one dimension around the current choice.
void Core::tune_begin_dim() {
  for (;;) {
    const TuneChoice base = choice();
    tune_cands_.clear();
    tune_next_ = 0;
    auto add = [&](TuneChoice c) {
      TuneSample t;
      t.choice = c;
      tune_cands_.push_back(t);
    };
    if (tune_dim_ == 0) {
      // Batch size: the capacity and two smaller powers of two.  Each sample
      // is a whole run (a pass of the plain engine), whose first batches are
      // short for every candidate alike.
      int cap_exp = 0;
      while ((2 << cap_exp) <= batch_cap_) ++cap_exp;
      for (int e = std::max(10, cap_exp - 2); e <= cap_exp; ++e) {
        TuneChoice c = base;
        c.batch_exp = e;
        add(c);
      }
    } else if (tune_dim_ == 1) {
      for (int nb : {6, 26, 98}) {
        TuneChoice c = base;
        c.bins = nb;
        add(c);
      }
    } else if (tune_dim_ == 2) {
      for (int b : {64, 128, 256}) {
        TuneChoice c = base;
        c.block = b;
        add(c);
      }
      if (wide_) {
        TuneChoice c = base;
        c.persistent = true;
        add(c);
      }
    } else if (tune_dim_ == 3) {
      if (base.ray_sort || base.hit_sort)
        for (int db : {4, 8, 11}) {
          TuneChoice c = base;
          c.digit_bits = db;
          add(c);
        }
    } else if (tune_dim_ == 4) {
      for (bool on : {true, false}) {
        TuneChoice c = base;
        c.ray_sort = on;
        add(c);
      }
    } else if (tune_dim_ == 5) {
      for (bool on : {true, false}) {
        TuneChoice c = base;
        c.hit_sort = on;
        add(c);
      }
    } else if (tune_dim_ == 6) {
      // ray key width: the default, one byte less (a coarser order, one sort
      // pass fewer) and one byte more (finer, one pass more)
      if (base.ray_sort) {
        const int def = scenes_.size() > 1 ? kRayKeyBitsScenes : kRayKeyBits;
        for (int kb : {def - 8, def, def + 8}) {
          TuneChoice c = base;
          c.ray_key_bits = kb;
          add(c);
        }
      }
    } else {
      tune_active_ = false;
      return;
    }
    if (tune_cands_.size() > 1) return;
    ++tune_dim_;
  }
}

// After a booked run: when every candidate of the dimension has its runs,
// keep the fastest (rays per device ms) and move to the next dimension.
void Core::tune_sample_done() {
  if (tune_next_ < (int)tune_cands_.size() * tune_windows_) return;
  int best = -1;
  double best_rate = -1.0;
  for (int i = 0; i < (int)tune_cands_.size(); ++i) {
    const TuneSample& t = tune_cands_[i];
    const double rate = t.ms > 0 ? t.rays / t.ms : -1.0;
    if (rate > best_rate) {
      best_rate = rate;
      best = i;
    }
    tune_log.push_back(t);
  }
  if (best >= 0) apply(tune_cands_[best].choice);
  ++tune_dim_;
  tune_begin_dim();
}

int Core::run_all(const volatile bool* stop) {
  // while tuning, the whole run is one sample of the next candidate
  int cand = -1;
  double rays0 = 0;
  if (tune_active_ && !tune_cands_.empty()) {
    cand = tune_next_ % (int)tune_cands_.size();
    apply(tune_cands_[cand].choice);
    const int grc = ensure_graph();  // graph construction stays outside the timed run
    if (grc != MSC_OK) return grc;
    rays0 = (double)(h_ctr_->closest + h_ctr_->shadow);
    CK(cudaEventRecord(tune_ev_[0], stream_));
  }
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
  if (cand >= 0) {
    CK(cudaEventRecord(tune_ev_[1], stream_));
    CK(cudaEventSynchronize(tune_ev_[1]));
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, tune_ev_[0], tune_ev_[1]) == cudaSuccess) {
      TuneSample& t = tune_cands_[cand];
      t.rays += (double)(h_ctr_->closest + h_ctr_->shadow) - rays0;
      t.ms += ms;
    }
    tune_next_ += 1;
    tune_sample_done();
  }
  CK(cudaStreamSynchronize(stream_));
  CK(cudaGetLastError());
  if (profiling) harvest();  // the stages after the last step (the jobs' filters)
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
  launch_trace_closest(d_scenes_, 1, scenes_[0]->rec, dev, dev + n, nullptr, n, dev + 2 * n, e, 0);
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
