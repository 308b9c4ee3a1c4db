// Device stages of the render loop.  Each kernel cites the reference code
// whose arithmetic it restates.  Every ray carries its job and scene in its
// info word, so a batch may mix jobs over several resident scenes.
#include <algorithm>

#include "radix.cuh"
#include "render.h"

#include <cuda_fp16.h>
#include "trace.cuh"

namespace mscg {

namespace {

constexpr int TB = 256;
inline int grid_for(int n, int tb = TB) { return (n + tb - 1) / tb; }

// samples[i].rgb += v (one writer per sample within a batch, so no atomics)
__device__ __forceinline__ void add_rgb(float4* p, float3 v) {
  float4 c = *p;
  c.x += v.x;
  c.y += v.y;
  c.z += v.z;
  *p = c;
}

__device__ __forceinline__ float mis_weight(float a, float b, int power) {
  if (power) {  // power heuristic, beta = 2
    float a2 = a * a;
    return a2 / (a2 + b * b);
  }
  return a / (a + b);  // misBalance, include/core/Common.h:45-48
}

// The plan's runs copied into shared memory by a whole block (only the
// runs in use).  Call from every thread of the block.
__device__ __forceinline__ void load_segments(const BatchPlan* __restrict__ plan, Segments& sm) {
  const int c = plan->seg.count;
  for (int k = threadIdx.x; k <= c; k += blockDim.x) {
    sm.prefix[k] = plan->seg.prefix[k];
    if (k < c) {
      sm.bin[k] = plan->seg.bin[k];
      sm.start[k] = plan->seg.start[k];
    }
  }
  if (threadIdx.x == 0) sm.count = c;
  __syncthreads();
}

// Pool index of batch ray i: its run (binary search on the prefix), then the
// run's bin position through the bin's chunk table.
__device__ __forceinline__ int seg_source(const Segments& seg, const int* table, int max_chunks, int i) {
  int lo = 0, hi = seg.count - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (seg.prefix[mid] <= i) lo = mid;
    else hi = mid - 1;
  }
  return pool_index(table, max_chunks, seg.bin[lo], seg.start[lo] + (i - seg.prefix[lo]));
}

// ------------------------------------------------------------------ raygen
// Camera::operator() (src/core/Camera.cpp:6-59) with StratifiedSampler
// (src/core/StratifiedSampler.cpp:5-17), IndependentSampler, GridSampler and
// PinHoleCamera::sample (src/core/PinHoleCamera.cpp:16-32) /
// ThinLensCamera::sample (src/core/ThinLensCamera.cpp:16-56).
// sampleID = x*H*spp + y*spp + i (Camera.cpp:28), local to the job.
// The camera ray of sample sid and its film position.
__device__ __forceinline__ void camera_ray(const JobRec& f, int job_index, uint32_t sid, float4* ro, float4* rd,
                                           float4* rw, float2* fpos) {
  const uint32_t col = (uint32_t)f.height * (uint32_t)f.spp;
  const uint32_t x = sid / col;
  const uint32_t rem = sid - x * col;
  const uint32_t y = rem / (uint32_t)f.spp;
  const uint32_t i = rem - y * (uint32_t)f.spp;
  const uint4 r = path_draws(sid, f.iter_seed, 0u, 0u);
  float sx, sy;
  const uint32_t ix = i / (uint32_t)f.grid_y, iy = i - ix * (uint32_t)f.grid_y;
  const float cellx = 1.f / (float)f.grid_x, celly = 1.f / (float)f.grid_y;
  if (f.sampler == SAMPLER_INDEPENDENT) {
    sx = u01(r.x);
    sy = u01(r.y);
  } else if (f.sampler == SAMPLER_GRID) {
    sx = (float)ix * cellx + 0.5f * cellx;
    sy = (float)iy * celly + 0.5f * celly;
  } else {
    sx = (float)ix * cellx + u01(r.x) * cellx;
    sy = (float)iy * celly + u01(r.y) * celly;
  }
  const float px = (float)x + sx, py = (float)y + sy;
  *fpos = make_float2(px, py);
  const float W = (float)f.width, H = (float)f.height;
  const float fx = ((px * 2.f - W) / W) * 36.f;
  const float fy = ((py * 2.f - H) / W) * 36.f;
  const CameraRec& c = f.cam;
  const float3 cn = f3(c.normal[0], c.normal[1], c.normal[2]);
  const float3 ct = f3(c.translation[0], c.translation[1], c.translation[2]);
  const float3 nodal = v_add(ct, v_mul(cn, c.focal_length));
  const float3 fp = xf_point(c.xf, f3(0.f, fy, fx));
  float3 org, dir;
  if (c.type == CAMERA_THINLENS) {
    const float ratio = c.focal_distance / c.focal_length;
    const float3 focal = v_add(fp, v_mul(v_sub(nodal, fp), ratio));
    // rejection sampling of the unit-diameter disc: attempt 0 uses draws 2,3
    // of the camera block; attempt k >= 1 uses block 1 + k/2 (draws 0,1 for
    // odd k, 2,3 for even k)
    float ax = 0.f, ay = 0.f;
    uint4 q = r;
    for (int attempt = 0; attempt < 64; ++attempt) {
      uint32_t a, b;
      if (attempt == 0) {
        a = r.z;
        b = r.w;
      } else {
        if (attempt & 1) q = path_draws(sid, f.iter_seed, 0u, 1u + (uint32_t)(attempt >> 1));
        a = (attempt & 1) ? q.x : q.z;
        b = (attempt & 1) ? q.y : q.w;
      }
      const float tx = u01(a) - 0.5f, ty = u01(b) - 0.5f;
      if (sqrtf(tx * tx + ty * ty) < 0.5f) { ax = tx; ay = ty; break; }
    }
    const float scale = c.focal_length / c.aperture;
    const float3 ap = xf_point(c.xf, f3(0.f, ax * scale, ay * scale));
    org = v_add(ap, v_mul(cn, c.focal_length));
    dir = v_normalize(v_sub(focal, org));
  } else {
    org = nodal;
    dir = v_normalize(v_sub(nodal, fp));
  }
  *ro = make_float4(org.x, org.y, org.z, 1.f);
  *rd = make_float4(dir.x, dir.y, dir.z, __int_as_float(ray_info(job_index, f.scene, 0)));
  *rw = make_float4(1.f, 1.f, 1.f, __int_as_float((int)sid));
}

// -------------------------------------------------------- bin partition
// DirectionalBins::add (src/core/DirectionalBins.cpp:37-73) as a stable
// counting partition: count digits per tile, scan, reserve chunks, scatter.
constexpr int PB = 256;
constexpr int PITEMS = kPartTile / PB;
constexpr int PRADIX = kBinRadix;

__device__ __forceinline__ int ray_digit(const float4& d, int nbins) {
  if (__float_as_int(d.w) < 0) return nbins;  // the dead bucket
  return ray_bin(f3(d), nbins);
}

__device__ __forceinline__ int dev_count(int n_max, const int* n_dev) {
  return n_dev ? min(*n_dev, n_max) : n_max;
}

// Per-tile digit counts, digit-major: counts[digit * tiles + tile] for the
// nbins + 1 digits (tiles past the count write zeros).
__global__ void __launch_bounds__(PB) k_part_count(const float4* __restrict__ d, int n_max,
                                                   const int* __restrict__ n_dev, int nbins,
                                                   uint32_t* __restrict__ counts, int tiles) {
  const int n = dev_count(n_max, n_dev);
  __shared__ int hist[PRADIX];
  for (int i = threadIdx.x; i < PRADIX; i += PB) hist[i] = 0;
  __syncthreads();
  const int base = blockIdx.x * kPartTile;
  const int lane = threadIdx.x & 31;
  for (int k = 0; k < PITEMS; ++k) {
    int idx = base + k * PB + threadIdx.x;
    int dg = idx < n ? ray_digit(d[idx], nbins) : -1;
    unsigned peers = __match_any_sync(0xffffffffu, dg);
    if (dg >= 0 && lane == __ffs(peers) - 1) atomicAdd(&hist[dg], __popc(peers));
  }
  __syncthreads();
  for (int g = threadIdx.x; g <= nbins; g += PB) counts[g * tiles + blockIdx.x] = (uint32_t)hist[g];
}

// One block, one thread per bin: each bin's missing chunks, as one
// contiguous run off the top of the free stack (an exclusive scan of the
// needs gives each bin its part).
__global__ void __launch_bounds__(kBinRadix) k_part_reserve(const uint32_t* __restrict__ scanned, int tiles,
                                                            BinPool pool) {
  __shared__ int warp_sum[kBinRadix / 32];
  const int b = threadIdx.x, lane = b & 31, warp = b >> 5;
  int need = 0;
  if (b < pool.nbins) {
    const int added = (int)(scanned[(b + 1) * tiles] - scanned[b * tiles]);
    if (added > 0) {
      int want = (pool.count[b] + added + kChunk - 1) >> kChunkShift;
      if (want > pool.max_chunks) {
        atomicOr(pool.err, ERR_BIN_OVERFLOW);
        want = pool.max_chunks;
      }
      need = max(0, want - pool.held[b]);
    }
  }
  int incl = need;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  if (lane == 31) warp_sum[warp] = incl;
  __syncthreads();
  int before = 0, total = 0;
  for (int w = 0; w < kBinRadix / 32; ++w) {
    if (w < warp) before += warp_sum[w];
    total += warp_sum[w];
  }
  const int ofs = before + incl - need;
  const int top = *pool.free_top;
  const int give = total <= top ? need : max(0, min(need, top - ofs));  // a short stack serves the lower bins
  if (total > top && b == 0) atomicOr(pool.err, ERR_BIN_OVERFLOW);
  const int base = top - min(total, top);
  const int h0 = b < pool.nbins ? pool.held[b] : 0;
  // the chunks handed out form one run [base, base + min(total, top)) of the
  // stack, bin b's part starting at its offset: the whole block copies them
  __shared__ int s_ofs[kBinRadix], s_h0[kBinRadix];
  s_ofs[b] = ofs;
  s_h0[b] = h0;
  __syncthreads();
  const int given = min(total, top);
  for (int x = b; x < given; x += kBinRadix) {
    int lo = 0, hi = kBinRadix - 1;  // the last bin whose offset is <= x
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (s_ofs[mid] <= x) lo = mid;
      else hi = mid - 1;
    }
    pool.table[lo * pool.max_chunks + s_h0[lo] + (x - s_ofs[lo])] = pool.free_stack[base + x];
  }
  if (b < pool.nbins) pool.held[b] = h0 + give;
  __syncthreads();
  if (b == 0) *pool.free_top = base;
}

__global__ void __launch_bounds__(PB) k_part_scatter(RayBuf src, int n_max, const int* __restrict__ n_dev,
                                                     const uint32_t* __restrict__ scanned, int tiles, BinPool pool,
                                                     const SceneRec* __restrict__ scenes) {
  const int n = dev_count(n_max, n_dev);
  __shared__ RankSmem<PB, PRADIX> sm;
  __shared__ uint32_t sidx[kPartTile];
  __shared__ int gofs[PRADIX];
  const int tile = blockIdx.x, base = tile * kPartTile;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nbins = pool.nbins;
  for (int b = threadIdx.x; b < PRADIX; b += PB)
    gofs[b] = (b < nbins) ? pool.count[b] + (int)(scanned[b * tiles + tile] - scanned[b * tiles]) : 0;
  int dig[PITEMS], pos[PITEMS];
#pragma unroll
  for (int k = 0; k < PITEMS; ++k) {
    int idx = base + warp * 32 * PITEMS + k * 32 + lane;
    dig[k] = idx < n ? ray_digit(src.d[idx], nbins) : -1;
  }
  tile_rank<PB, PITEMS, PRADIX>(dig, pos, sm);
#pragma unroll
  for (int k = 0; k < PITEMS; ++k)
    if (pos[k] >= 0) sidx[pos[k]] = (uint32_t)((warp * 32 * PITEMS + k * 32 + lane) | (dig[k] << 16));
  __syncthreads();
  const int count = min(kPartTile, n - base);
  for (int p = threadIdx.x; p < count; p += PB) {
    uint32_t e = sidx[p];
    int b = (int)(e >> 16);
    if (b >= nbins) continue;
    int s = base + (int)(e & 0xffffu);
    const int at = gofs[b] + (p - sm.tile_start[b]);
    if ((at >> kChunkShift) >= pool.held[b]) continue;  // no chunk reserved: reported by k_part_reserve
    const int o = pool_index(pool.table, pool.max_chunks, b, at);
    const float4 ro = __ldg(&src.o[s]), rd = __ldg(&src.d[s]);
    pool.rays.o[o] = ro;
    pool.rays.d[o] = rd;
    pool.rays.w[o] = __ldg(&src.w[s]);
    if (scenes) {  // the ray sort key, in the ray's scene box
      const int sc = info_scene(__float_as_int(rd.w));
      const float4 lo = scenes[sc].key_lo, sca = scenes[sc].key_scale;
      const uint32_t k = ray_sort_key(f3(ro), f3(rd), f3(lo), f3(sca));
      pool.keys[o] = (k & ~0xffu) | (uint32_t)sc;
    }
  }
}

__global__ void k_part_commit(const uint32_t* __restrict__ scanned, int tiles, BinPool pool) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= pool.nbins) return;
  const int added = (int)(scanned[(b + 1) * tiles] - scanned[b * tiles]);
  if (added == 0) return;
  const int c = min(pool.count[b] + added, pool.held[b] << kChunkShift);
  atomicAdd(pool.in_bins, c - pool.count[b]);
  pool.count[b] = c;
}

// ------------------------------------------------- camera rays into the bins
// The camera rays of samples [first, first + n) of a job go into the bins in
// the same stable counting partition as the continuing rays (sample order
// inside each bin), without a staging copy: a counting kernel makes each
// tile's rays for their direction bins (kept, one byte per ray, and the film
// samples written), the partition's scan and reserve hand out the positions,
// and a scatter kernel ranks the kept bins and makes each ray again - the
// same arithmetic, so the same bits - to write it into its position.  Sample
// t of the range is tile t / kPartTile's item.
__global__ void __launch_bounds__(PB) k_cam_count(JobRec f, int job_index, uint32_t first, int n, Film film,
                                                  int nbins, uint32_t* __restrict__ counts, int tiles,
                                                  uint8_t* __restrict__ digits) {
  __shared__ int hist[PRADIX];
  for (int i = threadIdx.x; i < PRADIX; i += PB) hist[i] = 0;
  __syncthreads();
  const int base = blockIdx.x * kPartTile;
  const int lane = threadIdx.x & 31;
  for (int k = 0; k < PITEMS; ++k) {
    const int idx = base + k * PB + threadIdx.x;
    int dg = -1;
    if (idx < n) {
      const uint32_t sid = first + (uint32_t)idx;
      float4 ro, rd, rw;
      float2 fp;
      camera_ray(f, job_index, sid, &ro, &rd, &rw, &fp);
      film.rgb[f.sample_base + sid] = make_float4(0.f, 0.f, 0.f, 0.f);
      film.pos[f.sample_base + sid] = fp;
      dg = ray_bin(f3(rd), nbins);
      digits[idx] = (uint8_t)dg;
    }
    const unsigned peers = __match_any_sync(0xffffffffu, dg);
    if (dg >= 0 && lane == __ffs(peers) - 1) atomicAdd(&hist[dg], __popc(peers));
  }
  __syncthreads();
  for (int g = threadIdx.x; g <= nbins; g += PB) counts[g * tiles + blockIdx.x] = (uint32_t)hist[g];
}

__global__ void __launch_bounds__(PB) k_cam_scatter(JobRec f, int job_index, uint32_t first, int n,
                                                    const uint32_t* __restrict__ scanned, int tiles, BinPool pool,
                                                    const SceneRec* __restrict__ key_scenes,
                                                    const uint8_t* __restrict__ digits) {
  __shared__ RankSmem<PB, PRADIX> sm;
  __shared__ uint32_t sidx[kPartTile];
  __shared__ int gofs[PRADIX];
  const int tile = blockIdx.x, base = tile * kPartTile;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nbins = pool.nbins;
  for (int b = threadIdx.x; b < PRADIX; b += PB)
    gofs[b] = (b < nbins) ? pool.count[b] + (int)(scanned[b * tiles + tile] - scanned[b * tiles]) : 0;
  int dig[PITEMS], pos[PITEMS];
#pragma unroll
  for (int k = 0; k < PITEMS; ++k) {
    const int idx = base + warp * 32 * PITEMS + k * 32 + lane;
    dig[k] = idx < n ? (int)digits[idx] : -1;
  }
  tile_rank<PB, PITEMS, PRADIX>(dig, pos, sm);
#pragma unroll
  for (int k = 0; k < PITEMS; ++k)
    if (pos[k] >= 0) sidx[pos[k]] = (uint32_t)((warp * 32 * PITEMS + k * 32 + lane) | (dig[k] << 16));
  __syncthreads();
  const int count = min(kPartTile, n - base);
  for (int p = threadIdx.x; p < count; p += PB) {
    const uint32_t e = sidx[p];
    const int b = (int)(e >> 16);
    const int at = gofs[b] + (p - sm.tile_start[b]);
    if ((at >> kChunkShift) >= pool.held[b]) continue;  // no chunk reserved: reported by k_part_reserve
    const int o = pool_index(pool.table, pool.max_chunks, b, at);
    float4 ro, rd, rw;
    float2 fp;
    camera_ray(f, job_index, first + (uint32_t)(base + (int)(e & 0xffffu)), &ro, &rd, &rw, &fp);
    pool.rays.o[o] = ro;
    pool.rays.d[o] = rd;
    pool.rays.w[o] = rw;
    if (key_scenes) {  // the ray sort key, in the ray's scene box
      const int sc = f.scene;
      const float4 lo = key_scenes[sc].key_lo, sca = key_scenes[sc].key_scale;
      const uint32_t key = ray_sort_key(f3(ro), f3(rd), f3(lo), f3(sca));
      pool.keys[o] = (key & ~0xffu) | (uint32_t)sc;
    }
  }
}

__global__ void k_pool_reset(BinPool pool) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < pool.num_chunks) pool.free_stack[i] = pool.num_chunks - 1 - i;
  if (i < kMaxBins) {
    pool.count[i] = 0;
    pool.held[i] = 0;
    if (pool.cursor) pool.cursor[i] = 0;
  }
  if (pool.pend && i < kMaxBins * pool.pend_cols) pool.pend[i] = -1;
  if (i == 0) {
    *pool.free_top = pool.num_chunks;
    *pool.in_bins = 0;
    if (pool.n_retired) *pool.n_retired = 0;
  }
}

__global__ void k_ray_bins(const float4* __restrict__ d, int n, int nbins, int* __restrict__ out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = ray_bin(f3(d[i]), nbins);
}

__global__ void k_cardinal(const float4* __restrict__ d, int n, int* __restrict__ out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = cardinal_bin(f3(d[i]));
}

// ------------------------------------------------------------ batch plan
// Pathtracer::batchLoading (src/core/Pathtracer.cpp:294-306) pops the next
// full batch, else flushes the fullest bin.  Here: the fullest bin's top
// (LIFO), topped up from the next fullest bins (ties to the lower bin) while
// `merge` is set and the batch is short.  One thread; the bins are six.
// One block of kBinRadix threads: thread b ranks bin b by count (descending,
// ties to the lower bin), thread 0 then walks the ranks.  Every bin of the
// pool is a candidate, so rays of a bin function used before a retune drain too.
__global__ void __launch_bounds__(kBinRadix) k_plan(BinPool pool, int batch_cap, int merge, int scene_bits,
                                                    BatchPlan* plan, Counters* ctr, int direct) {
  __shared__ int cnt[kMaxBins];
  __shared__ int by_rank[kMaxBins];
  __shared__ int f_bin[kMaxBins], f_keep[kMaxBins], f_held[kMaxBins], f_ofs[kMaxBins + 1];
  __shared__ int nsg_s, top_s;
  const int t = threadIdx.x;
  if (t < kMaxBins) cnt[t] = pool.count[t];
  __syncthreads();
  if (t < kMaxBins) {
    const int c = cnt[t];
    int r = 0;
    for (int o = 0; o < kMaxBins; ++o) r += (cnt[o] > c || (cnt[o] == c && o < t)) ? 1 : 0;
    by_rank[r] = t;
  }
  __syncthreads();
  if (t == 0) {
    int nsg = 0, nb = 0, freed = 0;
    for (int k = 0; k < kMaxBins && nb < batch_cap; ++k) {
      const int b = by_rank[k];
      const int c = cnt[b];
      if (c == 0) break;
      if (k > 0 && !merge) break;
      int take = min(batch_cap - nb, c);
      if (direct && take < c) {
        // leave the bin chunk-aligned, so that its appends start in a fresh
        // chunk and never overwrite a ray of this batch
        take = c - (((c - take) + kChunk - 1) & ~(kChunk - 1));
        if (take <= 0) continue;  // the room left is below this bin's partial chunk
      }
      const int left = c - take;
      plan->seg.bin[nsg] = b;
      plan->seg.start[nsg] = left;
      plan->seg.prefix[nsg] = nb;
      // chunks above the new top go back to the free stack; their rays are
      // gathered before any later partition of this stream can reuse them
      const int keep = (left + kChunk - 1) >> kChunkShift;
      f_bin[nsg] = b;
      f_keep[nsg] = keep;
      f_held[nsg] = pool.held[b];
      f_ofs[nsg] = freed;
      freed += max(0, pool.held[b] - keep);
      ++nsg;
      nb += take;
      pool.count[b] = left;
      pool.held[b] = keep;
    }
    f_ofs[nsg] = freed;
    nsg_s = nsg;
    top_s = *pool.free_top;
    if (direct) *pool.n_retired = freed;  // held back until the append commit
    else *pool.free_top = top_s + freed;
    plan->seg.count = nsg;
    plan->seg.prefix[nsg] = nb;
    plan->nb = nb;
    const int bb = bin_bits(pool.nbins);
    plan->bin_bits = bb;
    plan->prefix_bits = (nsg > 1 || scene_bits > 0) ? scene_bits + bb : 0;
    *pool.in_bins -= nb;
    ctr->closest += (unsigned long long)nb;
    ctr->batches += nb > 0 ? 1ull : 0ull;
  }
  __syncthreads();
  int* dst = direct ? pool.retired : pool.free_stack + top_s;
  for (int k = 0; k < nsg_s; ++k) {
    const int b = f_bin[k], keep = f_keep[k], nfree = f_held[k] - keep;
    // (the entries stay: the batch's ray keys and slots are read through them)
    for (int h = t; h < nfree; h += blockDim.x) dst[f_ofs[k] + h] = pool.table[b * pool.max_chunks + keep + h];
  }
  if (direct && t < kMaxBins) pool.cursor[t] = pool.count[t];
}

// Direct binning, after the appends: bin b's rays [count, cursor) sit in its
// held chunks and the chunks taken for it past them (pending), which join its
// chunk table up to its first failed take (whose rays are dropped, the error
// already set; chunks taken past it go back to the free stack); the batch's
// chunks return to the free stack.  One block.
constexpr int kCommitBlock = 1024;

__device__ __forceinline__ int commit_bin_of(const int* ofs, int e) {
  int lo = 0, hi = kMaxBins - 1;  // the last bin whose offset is <= e
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (ofs[mid] <= e) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

__global__ void __launch_bounds__(kCommitBlock) k_append_commit(BinPool pool) {
  __shared__ int kb_s[kMaxBins], fail_s[kMaxBins], ofs_s[kMaxBins + 1];
  const int t = threadIdx.x;
  if (t < kMaxBins) {
    const int c0 = pool.count[t], cur = pool.cursor[t], kb = pool.held[t];
    kb_s[t] = kb;
    fail_s[t] = cur > c0 ? max(kb, min((cur + kChunk - 1) >> kChunkShift, kb + pool.pend_cols)) : kb;
  }
  if (t == 0 && *pool.free_top < 0) *pool.free_top = 0;  // takes from an empty stack took nothing
  __syncthreads();
  if (t == 0) {  // the pending entries of all bins, as one index space
    int o = 0;
    for (int b = 0; b < kMaxBins; ++b) {
      ofs_s[b] = o;
      o += fail_s[b] - kb_s[b];
    }
    ofs_s[kMaxBins] = o;
  }
  __syncthreads();
  const int total = ofs_s[kMaxBins];
  for (int e = t; e < total; e += kCommitBlock) {  // each bin's first failed take
    const int b = commit_bin_of(ofs_s, e), k = kb_s[b] + (e - ofs_s[b]);
    if (pool.pend[b * pool.pend_cols + (k - kb_s[b])] < 0 || k >= pool.max_chunks) atomicMin(&fail_s[b], k);
  }
  __syncthreads();
  for (int e = t; e < total; e += kCommitBlock) {
    const int b = commit_bin_of(ofs_s, e), k = kb_s[b] + (e - ofs_s[b]);
    int* pe = &pool.pend[b * pool.pend_cols + (k - kb_s[b])];
    const int x = *pe;
    *pe = -1;
    if (k < fail_s[b]) pool.table[b * pool.max_chunks + k] = x;
    else if (x >= 0) pool.free_stack[atomicAdd(pool.free_top, 1)] = x;
  }
  int added = 0;
  if (t < kMaxBins) {
    const int c0 = pool.count[t], cur = pool.cursor[t];
    if (cur > c0) {
      const int nh = fail_s[t];
      const int c = min(cur, nh << kChunkShift);
      pool.count[t] = c;
      pool.held[t] = nh;
      added = c - c0;
    }
  }
  if (added > 0) atomicAdd(pool.in_bins, added);
  __syncthreads();
  const int top = *pool.free_top, nr = *pool.n_retired;
  for (int i = t; i < nr; i += kCommitBlock) pool.free_stack[top + i] = pool.retired[i];
  __syncthreads();
  if (t == 0) {
    *pool.free_top = top + nr;
    *pool.n_retired = 0;
  }
}

// ------------------------------------------------------------ ray keys
// Sort keys of the batch rays: the key each ray got when it was binned (its
// scene's box in place of the reference's per-batch origin box,
// RayBoundingbox.cpp:5-50), under (scene, direction bin) when the batch
// spans several; the bin is the run's, the scene sits in the key's low byte.
// The sort key and pool index of batch ray i (the segments in shared memory).
__device__ __forceinline__ uint32_t batch_ray_key(const uint32_t* __restrict__ pool_keys,
                                                  const int* __restrict__ table, int max_chunks,
                                                  const BatchPlan* __restrict__ plan, const Segments& seg,
                                                  int key_bits, int i, int* where) {
  int lo = 0, hi = seg.count - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (seg.prefix[mid] <= i) lo = mid;
    else hi = mid - 1;
  }
  const int bin = seg.bin[lo];
  const int at = pool_index(table, max_chunks, bin, seg.start[lo] + (i - seg.prefix[lo]));
  *where = at;
  const uint32_t pk = pool_keys[at];
  uint32_t key = pk & ~0xffu;
  const int prefix_bits = plan->prefix_bits;
  if (prefix_bits > 0) {
    const uint32_t prefix = ((pk & 0xffu) << plan->bin_bits) | (uint32_t)bin;
    key = (prefix << (32 - prefix_bits)) | (key >> prefix_bits);
  }
  return key >> (32 - key_bits);
}

__global__ void __launch_bounds__(TB) k_ray_keys(const uint32_t* __restrict__ pool_keys, const int* __restrict__ table,
                                                 int max_chunks, const BatchPlan* __restrict__ plan, int key_bits,
                                                 uint32_t* __restrict__ keys, uint32_t* __restrict__ where) {
  __shared__ Segments seg;
  const int n = plan->nb;
  if ((int)(blockIdx.x * blockDim.x) >= n) return;  // the whole block
  load_segments(plan, seg);
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int at;
  keys[i] = batch_ray_key(pool_keys, table, max_chunks, plan, seg, key_bits, i, &at);
  if (where) where[i] = (uint32_t)at;
}

// The same, with the sort's 8-bit digit counts of every pass taken on the way
// (hist zeroed beforehand; pass p's digit d at p * 256 + d): a grid-stride
// loop over the batch, counts gathered in shared memory per block.
constexpr int kKeyHistBlocks = 4 * 152;
__global__ void __launch_bounds__(TB) k_ray_keys_hist(const uint32_t* __restrict__ pool_keys,
                                                      const int* __restrict__ table, int max_chunks,
                                                      const BatchPlan* __restrict__ plan, int key_bits,
                                                      uint32_t* __restrict__ keys, uint32_t* __restrict__ where,
                                                      uint32_t* __restrict__ hist) {
  __shared__ Segments seg;
  __shared__ uint32_t cnt[4 * 256];
  const int n = plan->nb;
  const int passes = key_bits / 8;
  for (int k = threadIdx.x; k < passes * 256; k += TB) cnt[k] = 0u;
  load_segments(plan, seg);  // (syncs)
  for (int i = blockIdx.x * TB + threadIdx.x; i < n; i += gridDim.x * TB) {
    int at;
    const uint32_t key = batch_ray_key(pool_keys, table, max_chunks, plan, seg, key_bits, i, &at);
    keys[i] = key;
    where[i] = (uint32_t)at;
    for (int p = 0; p < passes; ++p) atomicAdd(&cnt[p * 256 + ((key >> (8 * p)) & 0xffu)], 1u);
  }
  __syncthreads();
  for (int k = threadIdx.x; k < passes * 256; k += TB)
    if (cnt[k]) atomicAdd(&hist[k], cnt[k]);
}

__global__ void __launch_bounds__(TB) k_ray_keys_direct(const float4* __restrict__ o, const float4* __restrict__ d,
                                                        int n, float3 lo, float3 scale, uint32_t* __restrict__ keys) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) keys[i] = ray_sort_key(f3(o[i]), f3(d[i]), lo, scale);
}

// Pool index of each batch ray, in sorted order (perm, when given): the
// traversal and shading read the rays where the bins hold them.
__global__ void __launch_bounds__(TB) k_batch_slots(const int* __restrict__ table, int max_chunks,
                                                    const BatchPlan* __restrict__ plan,
                                                    const uint32_t* __restrict__ perm, int* __restrict__ slots) {
  __shared__ Segments seg;
  const int n = plan->nb;
  if ((int)(blockIdx.x * blockDim.x) >= n) return;  // the whole block
  load_segments(plan, seg);
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  slots[j] = seg_source(seg, table, max_chunks, perm ? (int)perm[j] : j);
}

// -------------------------------------------------------------- traversal
// The BVH one ray reads: the 8-wide quantised nodes (WIDE) or the binary
// node-pair layout.
struct BvhRef {
  const void* nodes;
  const float4* tris;
  int num_nodes;
  int num_tris;
};

__host__ __device__ __forceinline__ BvhRef bvh_of(const SceneRec& sc, bool wide) {
  BvhRef r;
  r.nodes = wide ? (const void*)sc.wnodes : (const void*)sc.nodes;
  r.tris = sc.tris;
  r.num_nodes = sc.num_wnodes;
  r.num_tris = sc.num_tris;
  return r;
}

template <bool WIDE, bool ANY>
__device__ __forceinline__ bool scene_trace(const BvhRef& b, float3 o, float3 d, float tmin, float tmax, TriHit* h,
                                            int* ovf) {
  if (WIDE) return bvh8_trace<ANY>((const uint4*)b.nodes, b.tris, b.num_nodes, b.num_tris, o, d, tmin, tmax, h, ovf);
  return bvh_trace<ANY>((const float4*)b.nodes, b.tris, o, d, tmin, tmax, h, ovf);
}

__device__ __forceinline__ int ovf_bits(int ovf) {
  return ovf == 1 ? ERR_STACK_OVERFLOW : (ovf == 2 ? ERR_TRAVERSAL_CAP : ERR_BVH_INDEX);
}

// ------------------------------------------------------- sphere lights
// First intersection of o + t d with the sphere (centre sp.xyz, radius sp.w)
// in (tmin, tmax), else -1.
__device__ __forceinline__ float sphere_hit_t(float3 o, float3 d, float4 sp, float tmin, float tmax) {
  const float3 oc = v_sub(o, f3(sp.x, sp.y, sp.z));
  const float a = v_dot(d, d);
  const float b = v_dot(oc, d);
  const float c = v_dot(oc, oc) - sp.w * sp.w;
  const float disc = b * b - a * c;
  if (disc < 0.f) return -1.f;
  const float q = sqrtf(disc);
  const float t0 = (-b - q) / a;
  if (t0 > tmin && t0 < tmax) return t0;
  const float t1 = (-b + q) / a;
  if (t1 > tmin && t1 < tmax) return t1;
  return -1.f;
}

// Solid-angle pdf of sampling the sphere's cone of directions uniformly from p
// (0 when p is inside): 1 / (2 pi (1 - cos theta_max)), with
// 1 - cos theta_max = s2 / (1 + sqrt(1 - s2)), s2 = r^2 / |c - p|^2.
__device__ __forceinline__ float sphere_cone_pdf(float3 p, float3 c, float r) {
  const float3 wc = v_sub(c, p);
  const float d2 = v_dot(wc, wc);
  const float r2 = r * r;
  if (!(d2 > r2)) return 0.f;
  const float s2 = r2 / d2;
  const float omc = s2 / (1.f + sqrtf(1.f - s2));
  return 1.f / ((2.f * MSC_PI) * omc);
}

// Closest sphere light hit nearer than h->t (triangles win ties).
__device__ __forceinline__ void trace_spheres(const SceneRec& sr, float3 o, float3 d, TriHit* h) {
  const int ns = sr.num_spheres;
  for (int q = 0; q < ns; ++q) {
    const float t = sphere_hit_t(o, d, __ldg(&sr.spheres[q]), MSC_TNEAR, h->t);
    if (t > 0.f) {
      h->t = t;
      h->u = 0.f;
      h->v = 0.f;
      h->tri = sphere_hit_code(q);
    }
  }
}

// MULTI: look each ray's scene up in the table; else every ray uses scene0.
template <bool WIDE, bool MULTI, int BLOCK>
__global__ void __launch_bounds__(BLOCK) k_trace_closest(const SceneRec* __restrict__ scenes, BvhRef scene0,
                                                       const float4* __restrict__ o, const float4* __restrict__ d,
                                                       const int* __restrict__ slots, int n_max,
                                                       const int* __restrict__ n_dev, float4* __restrict__ hits,
                                                       int* err) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= dev_count(n_max, n_dev)) return;
  const int src = slots ? slots[i] : i;
  float4 ro = o[src], rd = d[src];
  const int sc = MULTI ? info_scene(__float_as_int(rd.w)) : 0;
  const BvhRef b = MULTI ? bvh_of(scenes[sc], WIDE) : scene0;
  TriHit h;
  h.t = MSC_TFAR; h.u = 0.f; h.v = 0.f; h.tri = -1;
  int ovf = 0;
  scene_trace<WIDE, false>(b, f3(ro), f3(rd), MSC_TNEAR, MSC_TFAR, &h, &ovf);
  if (scenes[sc].num_spheres > 0) trace_spheres(scenes[sc], f3(ro), f3(rd), &h);
  if (ovf) atomicOr(err, ovf_bits(ovf));
  hits[i] = make_float4(h.t, h.u, h.v, __int_as_float(h.tri));
}

// CompareHit key (include/core/RayUncompressed.h:63-69): (geomID, primID) with
// misses first.  Triangles are numbered geomID-major within a scene and scenes
// follow each other, so tri_base + global triangle index + 1 orders exactly
// like (scene, geomID, primID), and 0 is a miss.
__global__ void __launch_bounds__(TB) k_hit_keys(const SceneRec* __restrict__ scenes, const float4* __restrict__ d,
                                                 const int* __restrict__ slots, const float4* __restrict__ hits,
                                                 int n_max, const int* __restrict__ n_dev,
                                                 uint32_t* __restrict__ keys) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= dev_count(n_max, n_dev)) return;
  int k = __float_as_int(hits[i].w);
  if (k < 0) {  // misses and sphere-light hits first
    keys[i] = 0u;
    return;
  }
  const SceneRec& sc = scenes[info_scene(__float_as_int(d[slots ? slots[i] : i].w))];
  keys[i] = sc.tri_base + (uint32_t)sc.tri_orig[k] + 1u;
}

// The 64-bit hit key of one scene: shader id (12 bits) | original face index
// (23 bits) | u quantised to 15 bits | v to 14 bits.  Misses and sphere-light
// hits take 0, so they come first as in CompareHit.
__global__ void __launch_bounds__(TB) k_hit_keys64(const SceneRec* __restrict__ scenes, const float4* __restrict__ hits,
                                                   int n_max, const int* __restrict__ n_dev, uint32_t* __restrict__ lo,
                                                   uint32_t* __restrict__ hi) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= dev_count(n_max, n_dev)) return;
  const float4 h = hits[i];
  const int k = __float_as_int(h.w);
  uint64_t key = 0;
  if (k >= 0) {
    const SceneRec& sc = scenes[0];
    const float4 ta = __ldg(&sc.tris[3 * k]);
    const uint64_t shader = (uint64_t)(sc.geoms[__float_as_int(ta.w)].shader & 0xfff);
    const uint64_t face = (uint64_t)(__ldg(&sc.tri_orig[k]) & 0x7fffff);
    const uint64_t uq = (uint64_t)min(32767, max(0, (int)(h.y * 32768.f)));
    const uint64_t vq = (uint64_t)min(16383, max(0, (int)(h.z * 16384.f)));
    key = (shader << 52) | (face << 29) | (uq << 14) | vq;
  }
  lo[i] = (uint32_t)key;
  hi[i] = (uint32_t)(key >> 32);
}

// Rank keys of a 64-bit-key scene: a hit's place in (shader, face) order.
__global__ void __launch_bounds__(TB) k_hit_keys_rank(const SceneRec* __restrict__ scenes,
                                                      const float4* __restrict__ hits, int n_max,
                                                      const int* __restrict__ n_dev, uint32_t* __restrict__ keys) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= dev_count(n_max, n_dev)) return;
  const int k = __float_as_int(hits[i].w);
  keys[i] = k >= 0 ? __ldg(&scenes[0].shade_rank[k]) : 0u;
}

__global__ void __launch_bounds__(TB) k_gather_u32(const uint32_t* __restrict__ src, const uint32_t* __restrict__ idx,
                                                   int n_max, const int* __restrict__ n_dev,
                                                   uint32_t* __restrict__ dst) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= dev_count(n_max, n_dev)) return;
  dst[i] = src[idx[i]];
}

// FP16 bits of k / 1024 for a 10-bit k (exact: k / 1024 has at most 10 significant bits).
__device__ __forceinline__ unsigned short k1024_half_bits(uint32_t k) {
  if (k == 0u) return 0;
  const int e = 31 - __clz((int)k);  // 0..9
  return (unsigned short)(((e + 5) << 10) | ((k << (10 - e)) & 0x3ffu));
}

__global__ void k_face_texels(unsigned short* __restrict__ texels, int64_t total, int res, uint32_t seed) {
  const int per_face = res * res * 3;
  for (int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; x < total;
       x += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t face = (uint32_t)(x / per_face);
    const int r = (int)(x - (int64_t)face * per_face);
    texels[x] = k1024_half_bits(face_texel_code(seed, face, (uint32_t)(r / 3), (uint32_t)(r % 3)));
  }
}

// ------------------------------------------------------------------ shading
struct BsdfEval {
  float3 f;
  float cos_theta;
  float pdf;
};

// LambertShader::evaluate (src/core/LambertShader.cpp:27-47), NullShader::evaluate
// (src/core/NullShader.cpp:25-39) and the Phong extension.
// col: the texture colour at the hit.
__device__ __forceinline__ BsdfEval bsdf_evaluate(const ShaderRec& s, float3 col, float3 wi, float3 wo, float3 n) {
  BsdfEval e;
  const float ci = v_dot(n, wi);
  const float co = v_dot(n, wo);
  if (s.type == SHADER_NULL) {
    e.f = f3(0.f, 0.f, 0.f);
    e.cos_theta = 1.f;
    e.pdf = 1.f * MSC_INV_PI * 0.5f;
    return e;
  }
  if (s.type == SHADER_PHONG) {
    const float3 r = v_sub(v_mul(n, 2.f * co), wo);
    const float ca = fmaxf(0.f, v_dot(r, wi));
    const float lobe = pow_pos(ca, s.exponent);
    if (ci < 0.f || co < 0.f) e.f = f3(0.f, 0.f, 0.f);
    else e.f = v_mul(v_mul(col, s.reflectance), ((s.exponent + 2.f) * MSC_INV_PI * 0.5f) * lobe);
    e.cos_theta = ci < 0.f ? 0.f : ci;
    e.pdf = ((s.exponent + 1.f) * MSC_INV_PI * 0.5f) * lobe;
    return e;
  }
  if (ci < 0.f || co < 0.f) e.f = f3(0.f, 0.f, 0.f);
  else e.f = v_mul(v_mul(col, s.reflectance), MSC_INV_PI);
  e.cos_theta = ci < 0.f ? 0.f : ci;
  e.pdf = e.cos_theta * MSC_INV_PI;
  return e;
}

// ------------------------------------------------------- image textures
// StandardTexture::initialize (src/core/StandardTexture.cpp:11-43) looks the
// image up through OpenImageIO with periodic wrap and zero derivatives; this
// build wraps (s, t) into [0, 1) and interpolates bilinearly between texel
// centres, t = 0 being the image's top row.
__device__ __forceinline__ float3 image_lookup(const float4* __restrict__ texels, int4 im, float s, float t) {
  const int w = im.y, h = im.z;
  s = s - floorf(s);
  t = t - floorf(t);
  const float x = s * (float)w - 0.5f, y = t * (float)h - 0.5f;
  const float fx0 = floorf(x), fy0 = floorf(y);
  const float fx = x - fx0, fy = y - fy0;
  int x0 = (int)fx0, y0 = (int)fy0;
  x0 = x0 < 0 ? x0 + w : (x0 >= w ? x0 - w : x0);
  y0 = y0 < 0 ? y0 + h : (y0 >= h ? y0 - h : y0);
  const int x1 = x0 + 1 == w ? 0 : x0 + 1, y1 = y0 + 1 == h ? 0 : y0 + 1;
  const float4 c00 = __ldg(&texels[im.x + y0 * w + x0]), c10 = __ldg(&texels[im.x + y0 * w + x1]);
  const float4 c01 = __ldg(&texels[im.x + y1 * w + x0]), c11 = __ldg(&texels[im.x + y1 * w + x1]);
  const float gx = 1.f - fx, gy = 1.f - fy;
  return f3((c00.x * gx + c10.x * fx) * gy + (c01.x * gx + c11.x * fx) * fy,
            (c00.y * gx + c10.y * fx) * gy + (c01.y * gx + c11.y * fx) * fy,
            (c00.z * gx + c10.z * fx) * gy + (c01.z * gx + c11.z * fx) * fy);
}

// A texture tree as a post-order program on a small value stack;
// LayeredTexture::initialize (src/core/LayeredTexture.cpp:14-37):
// upper * mask + lower * (1 - mask).
constexpr int kTexStack = 34;
__device__ __noinline__ float3 texture_eval(const SceneRec& sc, int prog, int len, float s, float t) {
  float3 st[kTexStack];
  int sp = 0;
  for (int k = 0; k < len; ++k) {
    const int2 op = __ldg(&sc.tex_ops[prog + k]);
    const TexNode& nd = sc.tex_nodes[op.y];
    if (op.x == 0) {
      if (sp < kTexStack) st[sp++] = f3(nd.colour[0], nd.colour[1], nd.colour[2]);
    } else if (op.x == 1) {
      if (sp < kTexStack) st[sp++] = image_lookup(sc.tex_texels, __ldg(&sc.tex_images[nd.image]), s, t);
    } else if (sp >= 3) {
      const float3 m = st[--sp], lo = st[--sp], up = st[--sp];
      st[sp++] = f3(up.x * m.x + lo.x * (1.f - m.x), up.y * m.y + lo.y * (1.f - m.y), up.z * m.z + lo.z * (1.f - m.z));
    }
  }
  return sp > 0 ? st[sp - 1] : f3(0.f, 0.f, 0.f);
}

// Orthonormal frame around axis a as in LambertShader::sample
// (src/core/LambertShader.cpp:63-65): tmp = a.x > 0.99 ? Y : X, s = |tmp x a|, t = |a x s|.
__device__ __forceinline__ float3 frame_dir(float3 a, float x, float y, float z) {
  const float3 tmp = a.x > 0.99f ? f3(0.f, 1.f, 0.f) : f3(1.f, 0.f, 0.f);
  const float3 s = v_normalize(v_cross(tmp, a));
  const float3 t = v_normalize(v_cross(a, s));
  return v_add(v_add(v_mul(t, x), v_mul(s, y)), v_mul(a, z));
}

// Integrator::operator() (src/core/Integrator.cpp:12-255), one hit per thread.
// job_done[j] counts the finished paths of job j.
constexpr int kShadowGroups = 64;  // two per lane of one warp in the group scan
static_assert(kShadowGroups == 64 && TB >= kShadowGroups, "the shadow group scan takes one warp");

constexpr int kAppendSpinCap = 1 << 20;

__device__ __forceinline__ int ld_volatile_i(const int* p) { return *(const volatile int*)p; }

// Direct binning: the continuing ray (dead when b < 0) joins direction bin b
// at a position from the bin's cursor.  One atomic per bin and block, and the
// block's rays of one bin keep their block order (warps, then lanes), so runs
// of rays that were traced next to each other stay together in the bin: the
// block counts its rays per warp and bin (bin_count), one thread per bin
// scans the warps' counts and takes the block's run from the cursor
// (bin_scan), and each ray then has its position (bin_place).  Positions past
// the chunks the bin held at the plan fall in chunks taken from the free
// stack by the lane that holds the chunk's first position; the others wait
// for it (bounded).
constexpr int kShadeWarps = TB / 32;
struct BinBlock {
  int wcnt[kShadeWarps][kMaxBins];  // per warp and bin: count, then the warp's offset in the block's run
  int bbase[kMaxBins];              // the block's first position in each bin
};

__device__ __forceinline__ void bin_zero(BinBlock& bb, int nbins) {
  for (int i = threadIdx.x; i < kShadeWarps * nbins; i += TB) bb.wcnt[i / nbins][i % nbins] = 0;
}

// All lanes of the warp call this; returns the lanes of the warp in the same bin.
__device__ __forceinline__ unsigned bin_count(BinBlock& bb, int b) {
  const int lane = threadIdx.x & 31;
  const unsigned peers = __match_any_sync(0xffffffffu, b);
  if (b >= 0 && lane == __ffs(peers) - 1) bb.wcnt[threadIdx.x >> 5][b] = __popc(peers);
  return peers;
}

// Thread t of [0, nbins) of the calling threads: bin t's run for the block.
__device__ __forceinline__ void bin_scan(BinBlock& bb, const BinPool& pool, int t) {
  int run = 0;
  for (int w = 0; w < kShadeWarps; ++w) {
    const int c = bb.wcnt[w][t];
    bb.wcnt[w][t] = run;
    run += c;
  }
  bb.bbase[t] = run > 0 ? atomicAdd(&pool.cursor[t], run) : 0;
}

// All lanes of the warp call this (after bin_scan, behind a block barrier).
__device__ __forceinline__ void bin_place(const BinBlock& bb, const BinPool& pool, int b, unsigned peers, float4 no,
                                          float4 nd, float4 nw, const SceneRec* __restrict__ key_scenes) {
  const int lane = threadIdx.x & 31;
  const int pos = b >= 0 ? bb.bbase[b] + bb.wcnt[threadIdx.x >> 5][b] + __popc(peers & ((1u << lane) - 1u)) : 0;
  int chunk = -1;
  int* wait_on = nullptr;
  if (b >= 0) {
    const int k = pos >> kChunkShift, kb = pool.held[b];
    if (k < kb) {
      chunk = pool.table[b * pool.max_chunks + k];  // the bin's partial top chunk
    } else if (k - kb < pool.pend_cols && k < pool.max_chunks) {
      int* e = &pool.pend[b * pool.pend_cols + (k - kb)];
      if ((pos & (kChunk - 1)) == 0) {
        const int top = atomicSub(pool.free_top, 1) - 1;
        chunk = top >= 0 ? pool.free_stack[top] : -2;
        if (chunk < 0) atomicOr(pool.err, ERR_BIN_OVERFLOW);
        *(volatile int*)e = chunk;
        __threadfence();
      } else {
        wait_on = e;
      }
    } else {
      atomicOr(pool.err, ERR_BIN_OVERFLOW);
    }
  }
  __syncwarp();
  if (wait_on) {  // a chunk another lane is taking
    int spins = 0;
    while ((chunk = ld_volatile_i(wait_on)) == -1) {
      if (++spins > kAppendSpinCap) {
        atomicOr(pool.err, ERR_APPEND_WAIT);
        break;
      }
    }
  }
  if (chunk >= 0) {
    const int o = chunk * kChunk + (pos & (kChunk - 1));
    pool.rays.o[o] = no;
    pool.rays.d[o] = nd;
    pool.rays.w[o] = nw;
    if (key_scenes) {  // the ray sort key, in the ray's scene box
      const int sc = info_scene(__float_as_int(nd.w));
      const float4 lo = key_scenes[sc].key_lo, sca = key_scenes[sc].key_scale;
      const uint32_t key = ray_sort_key(f3(no), f3(nd), f3(lo), f3(sca));
      pool.keys[o] = (key & ~0xffu) | (uint32_t)sc;
    }
  }
}

template <bool DIRECT>
__global__ void __launch_bounds__(TB, 4) k_shade(const SceneRec* __restrict__ scenes, const JobRec* __restrict__ jobs,
                                              Film film, RayBuf batch, const int* __restrict__ slots,
                                              const float4* __restrict__ hits,
                                              const uint32_t* __restrict__ order, int n_max,
                                              const int* __restrict__ n_dev, RayBuf next, ShadowBuf sh,
                                              int* sh_count, uint32_t* job_done, BinPool pool,
                                              const SceneRec* __restrict__ key_scenes) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = dev_count(n_max, n_dev);
  if (blockIdx.x * blockDim.x >= n) return;  // whole block past the batch
  const bool live = j < n;
  bool emit = false, cont = false;
  int job = -1, light = 0;
  float4 so = make_float4(0.f, 0.f, 0.f, 0.f), sd = so, scol = so;
  float4 no = so, nd = make_float4(0.f, 0.f, 0.f, __int_as_float(-1)), nw = so;
  if (live) {
    const int i = order ? (int)order[j] : j;
    const int src = slots ? slots[i] : i;
    // the batch's rays are only read here (their chunks are rewritten only
    // after this kernel): the read-only path serves them
    const float4 ro = __ldg(&batch.o[src]), rd = __ldg(&batch.d[src]), rw = __ldg(&batch.w[src]), h = hits[i];
    const int k = __float_as_int(h.w);
    const int info = __float_as_int(rd.w);
    job = info_job(info);
    const int scene = info_scene(info);
    const int depth = info_depth(info);
    const int sid = __float_as_int(rw.w);
    const JobRec& f = jobs[job];
    const uint32_t sample = f.sample_base + (uint32_t)sid;
    const float3 w = f3(rw);
    if (k < -1) {  // a sphere light (extension): uniform radiance on its outside
      const SceneRec& sc = scenes[scene];
      const LightRec& L = sc.lights[sc.sphere_light[-2 - k]];
      const float3 dn = v_normalize(f3(rd));
      const float3 c = f3(L.centre[0], L.centre[1], L.centre[2]);
      const float3 pos = v_add(f3(ro), v_mul(dn, h.x));
      const float3 nl = v_mul(v_sub(pos, c), 1.f / L.radius);
      const float le = v_dot(nl, v_neg(dn)) < 0.f ? 0.f : L.intensity;
      float mis = 1.0f;
      if (depth > 0) mis = mis_weight(ro.w, sphere_cone_pdf(f3(ro), c, L.radius) * sc.light_pick, f.mis_power);
      if (le > MSC_EPSILON) add_rgb(&film.rgb[sample], f3(le * mis * w.x, le * mis * w.y, le * mis * w.z));
    } else if (k >= 0) {  // a miss adds nothing (Integrator.cpp:26-27)
      const SceneRec& sc = scenes[scene];
      const float4 ta = __ldg(&sc.tris[3 * k + 0]);
      const float4 tb = __ldg(&sc.tris[3 * k + 1]);
      const float4 tc = __ldg(&sc.tris[3 * k + 2]);
      const GeomRec g = sc.geoms[__float_as_int(ta.w)];
      const ShaderRec s = sc.shaders[g.shader];
      const float3 dn = v_normalize(f3(rd));
      const float t = h.x;
      if (s.light >= 0) {
        // emitter hit: QuadLight::radiance (src/core/QuadLight.cpp:69-84), Integrator.cpp:37-76
        const LightRec& L = sc.lights[s.light];
        const float3 ln = f3(L.normal[0], L.normal[1], L.normal[2]);
        const float cosl = v_dot(ln, v_neg(dn));
        const float le = cosl < 0.f ? 0.f : L.intensity;
        const float pdfa = 1.f / (L.scale[0] * L.scale[1]);
        float mis = 1.0f;
        if (depth > 0) {
          const float pdfw = pdfa * (t * t) / fabsf(cosl);
          mis = mis_weight(ro.w, pdfw * sc.light_pick, f.mis_power);
        }
        if (le > MSC_EPSILON) add_rgb(&film.rgb[sample], f3(le * mis * w.x, le * mis * w.y, le * mis * w.z));
      } else {
        const float3 nrm = v_normalize(v_cross(f3(tb), f3(tc)));  // = -normalize(Ng) (Integrator.cpp:121-125)
        const float3 pos = v_add(f3(ro), v_mul(dn, t));
        const float3 wo = v_neg(dn);
        // texture colour (ConstantTexture.cpp:22-25; face texels: extension)
        float3 col = f3(s.colour[0], s.colour[1], s.colour[2]);
        if (s.texture == TEXTURE_TREE && sc.tex_ops) {
          const int o = __ldg(&sc.tri_orig[k]);
          const float* uv = sc.tri_uv + 6 * (size_t)o;
          col = texture_eval(sc, s.tex_prog, s.tex_len, uv_interp(uv[0], uv[2], uv[4], h.y, h.z),
                             uv_interp(uv[1], uv[3], uv[5], h.y, h.z));
        } else if (s.texture == TEXTURE_FACE && sc.texel_res > 0) {
          const int res = sc.texel_res;
          const int ti = min(res - 1, max(0, (int)(h.y * (float)res)));
          const int tj = min(res - 1, max(0, (int)(h.z * (float)res)));
          const size_t tx = ((size_t)__ldg(&sc.tri_orig[k]) * (size_t)(res * res) + (size_t)(tj * res + ti)) * 3;
          col = f3(col.x * __half2float(__ushort_as_half(__ldg(&sc.texels[tx + 0]))),
                   col.y * __half2float(__ushort_as_half(__ldg(&sc.texels[tx + 1]))),
                   col.z * __half2float(__ushort_as_half(__ldg(&sc.texels[tx + 2]))));
        }
        const uint4 ra = path_draws((uint32_t)sid, f.iter_seed, (uint32_t)depth + 1u, 0u);
        // next-event estimation (Integrator.cpp:103-178)
        if (sc.num_lights > 0) {
          int li = (int)((float)sc.num_lights * u01(ra.x));
          if (li >= sc.num_lights) li = sc.num_lights - 1;
          const LightRec& L = sc.lights[li];
          float3 wi;
          float dist, pdfw, le;
          if (L.type == LIGHT_SPHERE) {
            // extension: a direction uniform in the sphere's cone, the distance to its near side
            const float3 c = f3(L.centre[0], L.centre[1], L.centre[2]);
            const float3 wc = v_sub(c, pos);
            const float d2 = v_dot(wc, wc);
            const float r2 = L.radius * L.radius;
            le = 0.f;
            dist = 0.f;
            pdfw = 1.f;
            wi = f3(0.f, 0.f, 1.f);
            if (d2 > r2) {
              const float s2 = r2 / d2;
              const float omc = s2 / (1.f + sqrtf(1.f - s2));
              const float ct = 1.f - u01(ra.y) * omc;
              const float st = sqrtf(fmaxf(0.f, 1.f - ct * ct));
              float sp, cp;
              sincos_turns(u01(ra.z), &sp, &cp);
              wi = frame_dir(v_mul(wc, 1.f / sqrtf(d2)), cp * st, sp * st, ct);
              const float b = v_dot(wc, wi);
              const float disc = b * b - (d2 - r2);
              dist = disc > 0.f ? b - sqrtf(disc) : b;
              pdfw = 1.f / ((2.f * MSC_PI) * omc);
              le = dist > 0.f ? L.intensity : 0.f;
            }
          } else {
            // QuadLight::illuminate (src/core/QuadLight.cpp:41-67)
            const float3 smp = xf_point(L.xf, f3(0.f, u01(ra.y) - 0.5f, u01(ra.z) - 0.5f));
            const float3 ln = f3(L.normal[0], L.normal[1], L.normal[2]);
            float cosl = v_dot(v_normalize(v_sub(pos, smp)), ln);
            le = cosl < 0.f ? 0.f : L.intensity;
            cosl = cosl < 0.f ? 0.f : cosl;
            const float3 tol = v_sub(smp, pos);
            wi = v_normalize(tol);
            dist = v_len(tol);
            pdfw = (v_dot(tol, tol) / cosl) / (L.scale[0] * L.scale[1]);
          }
          if (le > MSC_EPSILON) {
            const BsdfEval e = bsdf_evaluate(s, col, wi, wo, nrm);
            if (v_maxc(e.f) > MSC_EPSILON) {
              const float a = pdfw * sc.light_pick;
              const float mis = mis_weight(a, e.pdf, f.mis_power);
              const float k0 = (mis * e.cos_theta) / a;
              const float3 c = f3(k0 * (le * e.f.x), k0 * (le * e.f.y), k0 * (le * e.f.z));
              emit = true;
              light = li;
              so = make_float4(pos.x, pos.y, pos.z, dist);
              sd = make_float4(wi.x, wi.y, wi.z, __int_as_float((int)sample));
              scol = make_float4(c.x * w.x, c.y * w.y, c.z * w.z, __int_as_float(scene));
            }
          }
        }
        // continuation with Russian roulette (Integrator.cpp:181-246)
        if (depth < f.max_depth && s.type != SHADER_NULL) {
          float q = fminf(1.f, s.reflectance / f.threshold);
          if (depth < f.min_depth) q = 1.f;
          if (!(u01(ra.w) > q)) {
            const uint4 rb = path_draws((uint32_t)sid, f.iter_seed, (uint32_t)depth + 1u, 1u);
            float sp, cp;
            sincos_turns(u01(rb.x), &sp, &cp);
            float3 wi;
            BsdfEval e;
            bool ok = true;
            if (s.type == SHADER_PHONG) {
              // cos(alpha) = xi^(1/(e+1)) around the mirror direction
              const float ca = pow_pos(u01(rb.y), 1.f / (s.exponent + 1.f));
              const float sa = sqrtf(fmaxf(0.f, 1.f - ca * ca));
              const float3 r = v_sub(v_mul(nrm, 2.f * v_dot(nrm, wo)), wo);
              wi = frame_dir(v_normalize(r), cp * sa, sp * sa, ca);
              e = bsdf_evaluate(s, col, wi, wo, nrm);
              ok = e.cos_theta > 0.f && e.pdf > 0.f;
            } else {
              // LambertShader::sample (src/core/LambertShader.cpp:49-73) with
              // sin(acos(sqrt(xi))) = sqrt(1 - xi) and cos(acos(sqrt(xi))) = sqrt(xi)
              const float st = sqrtf(1.f - u01(rb.y));
              const float ct = sqrtf(u01(rb.y));
              wi = frame_dir(nrm, cp * st, sp * st, ct);
              e.f = v_mul(v_mul(col, s.reflectance), MSC_INV_PI);
              e.cos_theta = v_dot(nrm, wi);
              e.pdf = e.cos_theta * MSC_INV_PI;
              ok = e.pdf > 0.f;
            }
            if (ok) {
              const float g0 = e.cos_theta / e.pdf;
              cont = true;
              no = make_float4(pos.x, pos.y, pos.z, e.pdf);
              nd = make_float4(wi.x, wi.y, wi.z, __int_as_float(ray_info(job, scene, depth + 1)));
              nw = make_float4(((w.x * e.f.x) * g0) / q, ((w.y * e.f.y) * g0) / q, ((w.z * e.f.z) * g0) / q,
                               __int_as_float(sid));
            }
          }
        }
      }
    }
  }
  const int lane = threadIdx.x & 31;
  // the block's shadow rays are appended grouped by light (a block-wide
  // counting sort on the light index modulo kShadowGroups; the order inside a
  // group does not matter), so the occlusion kernel's warps trace rays from
  // one neighbourhood toward one light; with direct binning the continuing
  // rays are counted per bin under the same block barriers
  __shared__ BinBlock bb;
  const int bin = (DIRECT && cont) ? ray_bin(f3(nd), pool.nbins) : -1;
  unsigned bin_peers = 0u;
  {
    __shared__ int grp[kShadowGroups];
    if (threadIdx.x < kShadowGroups) grp[threadIdx.x] = 0;
    if (DIRECT) bin_zero(bb, pool.nbins);
    __syncthreads();
    const int g = light & (kShadowGroups - 1);
    const int rank = emit ? atomicAdd(&grp[g], 1) : 0;
    if (DIRECT) bin_peers = bin_count(bb, bin);
    __syncthreads();
    if (DIRECT && threadIdx.x >= 32 && threadIdx.x < 32 + pool.nbins) bin_scan(bb, pool, threadIdx.x - 32);
    if (threadIdx.x < 32) {  // exclusive scan of the group counts, two per lane
      const int a = grp[2 * lane], b = grp[2 * lane + 1];
      int incl = a + b;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
      }
      const int total = __shfl_sync(0xffffffffu, incl, 31);
      int base = 0;
      if (lane == 0 && total > 0) base = atomicAdd(sh_count, total);
      base = __shfl_sync(0xffffffffu, base, 0);
      grp[2 * lane] = base + incl - a - b;
      grp[2 * lane + 1] = base + incl - b;
    }
    __syncthreads();
    if (emit) {
      const int slot = grp[g] + rank;
      sh.o[slot] = so;
      sh.d[slot] = sd;
      sh.c[slot] = scol;
    }
  }
  // finished paths per job, aggregated over the lanes of one job
  const int ended = (live && !cont) ? job : -1;
  const unsigned peers = __match_any_sync(0xffffffffu, ended);
  if (ended >= 0 && lane == __ffs(peers) - 1) atomicAdd(&job_done[ended], (uint32_t)__popc(peers));
  if (DIRECT) {
    bin_place(bb, pool, bin, bin_peers, no, nd, nw, key_scenes);
  } else if (live) {
    next.o[j] = no;
    next.d[j] = cont ? nd : make_float4(0.f, 0.f, 0.f, __int_as_float(-1));
    next.w[j] = nw;
  }
}

// rtcOccluded with mask 0x0FFFFFFF (Integrator.cpp:153-174); an unoccluded
// shadow ray adds its weighted contribution to its sample.
template <bool WIDE, bool MULTI, int BLOCK>
__global__ void __launch_bounds__(BLOCK) k_trace_shadow(const SceneRec* __restrict__ scenes, BvhRef scene0, ShadowBuf sh,
                                                      const int* __restrict__ count, float4* sample_rgb, int* err,
                                                      unsigned long long* shadow_total) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (shadow_total && i == 0) *shadow_total += (unsigned long long)*count;
  if (i >= *count) return;
  const float4 o = sh.o[i], d = sh.d[i], c = sh.c[i];
  const BvhRef b = MULTI ? bvh_of(scenes[__float_as_int(c.w)], WIDE) : scene0;
  TriHit h;
  int ovf = 0;
  const bool blocked = scene_trace<WIDE, true>(b, f3(o), f3(d), MSC_TNEAR, o.w, &h, &ovf);
  if (ovf) atomicOr(err, ovf_bits(ovf));
  if (!blocked) add_rgb(&sample_rgb[__float_as_int(d.w)], f3(c));
}

// Persistent traversal with per-lane ray refill (8-wide BVH only): every lane
// holds one ray; when at least kRefill lanes of a warp are idle, the warp
// takes that many new rays from `counter` in one atomic.
constexpr int kRefill = 8;
constexpr int kPersistBlock = 128;

template <bool MULTI>
__global__ void __launch_bounds__(kPersistBlock) k_trace_closest_pt(const SceneRec* __restrict__ scenes,
                                                                    BvhRef scene0, const float4* __restrict__ o,
                                                                    const float4* __restrict__ d,
                                                                    const int* __restrict__ slots, int n_max,
                                                                    const int* __restrict__ n_dev,
                                                                    float4* __restrict__ hits, int* err,
                                                                    int* counter) {
  const int n = dev_count(n_max, n_dev);
  const int lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
  Trav8 st;
  TriHit h;
  uint2 stack[kWideStack];
  BvhRef b = scene0;
  int ray = -1, sc = 0, ovf = 0;
  bool exhausted = false;
  while (true) {
    const unsigned idle = __ballot_sync(0xffffffffu, ray < 0);
    if (!exhausted && __popc(idle) >= kRefill) {
      int base = 0;
      if (lane == 0) base = atomicAdd(counter, __popc(idle));
      base = __shfl_sync(0xffffffffu, base, 0);
      exhausted = base + __popc(idle) >= n;
      if (ray < 0) {
        const int my = base + __popc(idle & lt);
        if (my < n) {
          ray = my;
          const int src = slots ? slots[my] : my;
          const float4 ro = o[src], rd = d[src];
          sc = MULTI ? info_scene(__float_as_int(rd.w)) : 0;
          b = MULTI ? bvh_of(scenes[sc], true) : scene0;
          trav8_init(st, f3(ro), f3(rd), MSC_TNEAR, MSC_TFAR);
          h.t = MSC_TFAR; h.u = 0.f; h.v = 0.f; h.tri = -1;
          ovf = 0;
        }
      }
    }
    if (__ballot_sync(0xffffffffu, ray >= 0) == 0u) {
      if (exhausted) break;
      continue;  // all idle and more rays left: refill on the next turn
    }
    if (ray >= 0 &&
        trav8_step<false>(st, stack, (const uint4*)b.nodes, b.tris, b.num_nodes, b.num_tris, &h, &ovf)) {
      if (scenes[sc].num_spheres > 0) trace_spheres(scenes[sc], st.o, st.d, &h);
      if (ovf) atomicOr(err, ovf_bits(ovf));
      hits[ray] = make_float4(h.t, h.u, h.v, __int_as_float(h.tri));
      ray = -1;
    }
  }
}

template <bool MULTI>
__global__ void __launch_bounds__(kPersistBlock) k_trace_shadow_pt(const SceneRec* __restrict__ scenes,
                                                                   BvhRef scene0, ShadowBuf sh,
                                                                   const int* __restrict__ count, float4* sample_rgb,
                                                                   int* err, unsigned long long* shadow_total,
                                                                   int* counter) {
  const int n = *count;
  if (shadow_total && blockIdx.x == 0 && threadIdx.x == 0) *shadow_total += (unsigned long long)n;
  const int lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
  Trav8 st;
  TriHit h;
  uint2 stack[kWideStack];
  BvhRef b = scene0;
  int ray = -1, ovf = 0;
  float4 col = make_float4(0.f, 0.f, 0.f, 0.f);
  int target = 0;
  bool exhausted = false;
  while (true) {
    const unsigned idle = __ballot_sync(0xffffffffu, ray < 0);
    if (!exhausted && __popc(idle) >= kRefill) {
      int base = 0;
      if (lane == 0) base = atomicAdd(counter, __popc(idle));
      base = __shfl_sync(0xffffffffu, base, 0);
      exhausted = base + __popc(idle) >= n;
      if (ray < 0) {
        const int my = base + __popc(idle & lt);
        if (my < n) {
          ray = my;
          const float4 so = sh.o[my], sd = sh.d[my];
          col = sh.c[my];
          target = __float_as_int(sd.w);
          b = MULTI ? bvh_of(scenes[__float_as_int(col.w)], true) : scene0;
          trav8_init(st, f3(so), f3(sd), MSC_TNEAR, so.w);
          ovf = 0;
        }
      }
    }
    if (__ballot_sync(0xffffffffu, ray >= 0) == 0u) {
      if (exhausted) break;
      continue;
    }
    if (ray >= 0 &&
        trav8_step<true>(st, stack, (const uint4*)b.nodes, b.tris, b.num_nodes, b.num_tris, &h, &ovf)) {
      if (ovf) atomicOr(err, ovf_bits(ovf));
      if (!st.found) add_rgb(&sample_rgb[target], f3(col));
      ray = -1;
    }
  }
}

// Resident blocks of a persistent kernel on this device (cached per kernel).
template <class K>
int persistent_grid(K kernel) {
  static int grid = 0;
  if (grid == 0) {
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kPersistBlock, 0);
    grid = std::max(1, sms * std::max(1, per_sm));
  }
  return grid;
}

template <bool WIDE>
__global__ void __launch_bounds__(128) k_occluded(BvhRef bvh, const float4* __restrict__ o,
                                                  const float4* __restrict__ d, int n, int* out, int* err) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 ro = o[i], rd = d[i];
  TriHit h;
  int ovf = 0;
  out[i] = scene_trace<WIDE, true>(bvh, f3(ro), f3(rd), MSC_TNEAR, ro.w, &h, &ovf) ? 1 : 0;
  if (ovf) atomicOr(err, ovf_bits(ovf));
}

// ------------------------------------------------------------------ filters
// TentFilter::convolve (src/core/TentFilter.cpp:5-63): each pixel's value is
// the tent-weighted mean of the samples of its 3x3 neighbour pixels; samples
// are x-major (x*H*spp + y*spp + i), pixels row-major.
//
// Source-centric tiles, so that every sample leaves HBM once: a block owns an
// output tile of kFtX columns x kFtY rows and the (kFtX+2) x (kFtY+2) source
// pixels around it, one thread per source pixel.  The sources' samples are
// staged kFtChunk at a time by asynchronous copies (cp.async) into two shared
// buffers, so the next chunk streams in while the current one is folded: each
// thread folds every sample of its source pixel, in sample order, into nine
// partial sums - one per target pixel of the 3x3 around it - with exactly the
// reference's per-term weights m = max(0, 1-|x-cx|) * max(0, 1-|y-cy|) (the
// colour terms c*m fused into the running sums).  The partials go through
// shared memory and each output pixel adds its nine partials in the
// reference's neighbour order (mx, then my).  The weights are the reference's;
// the association differs (each neighbour's samples are summed from zero
// before they join the pixel's running sum) and the colour products are not
// rounded apart, a difference of a few float ulps per pixel.
constexpr int kFtX = 8, kFtY = 30;                   // output tile
constexpr int kFsX = kFtX + 2, kFsY = kFtY + 2;      // source pixels with their halo
constexpr int kFsN = kFsX * kFsY;                    // 320 source pixels = block threads
constexpr int kFtChunk = 4;                          // samples per source in one staging buffer
constexpr int kFtStages = 2;                         // staging buffers in the ring
constexpr int kFrgbPitch = kFsN + 1;                 // float4 rows: conflict-free stores and loads
constexpr int kFposPitch = kFsN + 9;                 // float2 rows
struct FilterStage {
  float4 rgb[kFtChunk][kFrgbPitch];
  float2 pos[kFtChunk][kFposPitch];
};
struct FilterSmemPart {
  float4 part[9][kFrgbPitch];  // (r, g, b, weight) of source q for target slot (1+dx)*3 + (1+dy)
};
union FilterSmem {
  FilterStage st[kFtStages];
  FilterSmemPart pa;
};

__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

// This thread's share of the staging: as kFsN is a multiple of kFtChunk, all
// its copies of a chunk are the same sample slot k = thread % kFtChunk, of
// source pixels thread / kFtChunk + j * kFsN / kFtChunk.  gbase is that
// source's sample k (-1: outside the image); srgb / spos are the shared-memory
// byte offsets of the copies within a staging buffer.
static_assert(kFsN % kFtChunk == 0, "each thread stages one sample slot");
struct FilterCopies {  // the film pool indexes samples with 31 bits
  int gbase[kFtChunk];
  uint32_t srgb[kFtChunk], spos[kFtChunk];
  int k;
};

__device__ __forceinline__ FilterCopies filter_copies(const JobRec& f, int x0, int y0) {
  FilterCopies fc;
  const int W = f.width, H = f.height;
  fc.k = (int)threadIdx.x % kFtChunk;
#pragma unroll
  for (int j = 0; j < kFtChunk; ++j) {
    const int src = (int)threadIdx.x / kFtChunk + j * (kFsN / kFtChunk);
    const int sx = x0 - 1 + src / kFsY, sy = y0 - 1 + src % kFsY;
    const bool ok = sx >= 0 && sx < W && sy >= 0 && sy < H;
    fc.gbase[j] = ok ? (int)((int64_t)f.sample_base + ((int64_t)sx * H + sy) * f.spp + fc.k) : -1;
    fc.srgb[j] = (uint32_t)(offsetof(FilterStage, rgb) + ((size_t)fc.k * kFrgbPitch + src) * sizeof(float4));
    fc.spos[j] = (uint32_t)(offsetof(FilterStage, pos) + ((size_t)fc.k * kFposPitch + src) * sizeof(float2));
  }
  return fc;
}

__device__ __forceinline__ void cp_async16_s(uint32_t s, const void* gmem) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async8_s(uint32_t s, const void* gmem) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gmem) : "memory");
}

// Issues the copies of samples [s0, s0 + cs) of every source pixel of the tile
// into the staging buffer at shared address st, as one commit group (an empty
// group when cs <= 0, which keeps the count of groups behind each chunk fixed).
__device__ __forceinline__ void filter_stage(uint32_t st, const FilterCopies& fc, const Film& film, int s0, int cs) {
  if (fc.k < cs) {
#pragma unroll
    for (int j = 0; j < kFtChunk; ++j) {
      if (fc.gbase[j] >= 0) {
        const size_t g = (size_t)(fc.gbase[j] + s0);
        cp_async16_s(st + fc.srgb[j], &film.rgb[g]);
        cp_async8_s(st + fc.spos[j], &film.pos[g]);
      }
    }
  }
  cp_async_commit();
}

// One sample of this thread's source pixel into its nine partial sums.
__device__ __forceinline__ void filter_fold(const FilterStage& st, int k, int q, const float* cxs, const float* cys,
                                            float4* acc) {
  const float2 p = st.pos[k][q];
  const float4 cc = st.rgb[k][q];
  float wx[3], wy[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    wx[a] = fmaxf(0.f, 1.f - fabsf(p.x - cxs[a]));
    wy[a] = fmaxf(0.f, 1.f - fabsf(p.y - cys[a]));
  }
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int b = 0; b < 3; ++b) {
      const float m = wx[a] * wy[b];
      float4& r = acc[a * 3 + b];
      r.w = r.w + m;
      r.x = fmaf(cc.x, m, r.x);
      r.y = fmaf(cc.y, m, r.y);
      r.z = fmaf(cc.z, m, r.z);
    }
}

__global__ void __launch_bounds__(kFsN, 3) k_filter_tent(JobRec f, Film film) {
  extern __shared__ __align__(16) unsigned char filter_smem[];
  FilterSmem& sm = *reinterpret_cast<FilterSmem*>(filter_smem);
  const int W = f.width, H = f.height, spp = f.spp;
  const int x0 = blockIdx.y * kFtX, y0 = blockIdx.x * kFtY;
  const int q = threadIdx.x;
  const int qx = x0 - 1 + q / kFsY, qy = y0 - 1 + q % kFsY;  // this thread's source pixel
  const bool qvalid = qx >= 0 && qx < W && qy >= 0 && qy < H;
  const FilterCopies fc = filter_copies(f, x0, y0);
  float4 acc[9];
#pragma unroll
  for (int t = 0; t < 9; ++t) acc[t] = make_float4(0.f, 0.f, 0.f, 0.f);
  // target pixel centres around the source (the reference's cx, cy of each target)
  float cxs[3], cys[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    cxs[a] = (float)(qx + a - 1) + 0.5f;
    cys[a] = (float)(qy + a - 1) + 0.5f;
  }
  const int chunks = (spp + kFtChunk - 1) / kFtChunk;
  const uint32_t st0 = (uint32_t)__cvta_generic_to_shared(&sm.st[0]);
  // chunks 0 .. kFtStages-2 in flight before the loop
#pragma unroll
  for (int c = 0; c < kFtStages - 1; ++c)
    filter_stage(st0 + c * (uint32_t)sizeof(FilterStage), fc, film, c * kFtChunk, min(kFtChunk, spp - c * kFtChunk));
  for (int c = 0; c < chunks; ++c) {
    const int s0 = c * kFtChunk, cs = min(kFtChunk, spp - s0);
    // this thread's copies of chunk c have landed (the kFtStages-2 groups
    // committed after chunk c's may still be in flight)
    cp_async_wait<kFtStages - 2>();
    // chunk c is visible to all, and every thread is done with chunk c - 1,
    // whose buffer the copies of chunk c + kFtStages - 1 now refill
    __syncthreads();
    {
      const int cn = c + kFtStages - 1;
      filter_stage(st0 + (uint32_t)(cn % kFtStages) * (uint32_t)sizeof(FilterStage), fc, film, cn * kFtChunk,
                   min(kFtChunk, spp - cn * kFtChunk));
    }
    const FilterStage& st = sm.st[c % kFtStages];
    if (qvalid) {
      if (cs == kFtChunk) {  // a full chunk: the folds unrolled
#pragma unroll
        for (int k = 0; k < kFtChunk; ++k) filter_fold(st, k, q, cxs, cys, acc);
      } else {
        for (int k = 0; k < cs; ++k) filter_fold(st, k, q, cxs, cys, acc);
      }
    }
  }
  cp_async_wait<0>();  // only empty groups remain; none may write into the partials
  __syncthreads();     // every thread is done with the staging buffers
#pragma unroll
  for (int t = 0; t < 9; ++t) sm.pa.part[t][q] = acc[t];
  __syncthreads();
  if (threadIdx.x >= kFtX * kFtY) return;
  const int tx = threadIdx.x / kFtY, ty = threadIdx.x - tx * kFtY;
  const int x = x0 + tx, y = y0 + ty;
  if (x >= W || y >= H) return;
  float sr = 0.f, sg = 0.f, sb = 0.f, den = 0.f;
  for (int mx = -1; mx < 2; ++mx) {
    if (x + mx < 0 || x + mx >= W) continue;
    for (int my = -1; my < 2; ++my) {
      if (y + my < 0 || y + my >= H) continue;
      const int src = (tx + 1 + mx) * kFsY + (ty + 1 + my);
      const float4 r = sm.pa.part[(1 - mx) * 3 + (1 - my)][src];
      den = den + r.w;
      sr = sr + r.x;
      sg = sg + r.y;
      sb = sb + r.z;
    }
  }
  float* out = f.pixels + 3 * ((size_t)y * W + x);
  out[0] += sr / den;
  out[1] += sg / den;
  out[2] += sb / den;
}

// BoxFilter::convolve (src/core/BoxFilter.cpp:5-37).
__global__ void __launch_bounds__(TB) k_filter_box(JobRec f, Film film) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= f.width * f.height) return;
  const int x = idx / f.height, y = idx - x * f.height;
  const size_t b = (size_t)f.sample_base + ((size_t)x * f.height + y) * f.spp;
  float sr = 0.f, sg = 0.f, sb = 0.f;
  for (int s = 0; s < f.spp; ++s) {
    const float4 c = film.rgb[b + s];
    sr += c.x;
    sg += c.y;
    sb += c.z;
  }
  const float ns = (float)f.spp;
  float* px = f.pixels + 3 * ((size_t)y * f.width + x);
  px[0] += sr / ns;
  px[1] += sg / ns;
  px[2] += sb / ns;
}

}  // namespace

int launch_camera_rays(const JobRec& job, int job_index, uint32_t first, int n, Film film, BinPool& pool,
                       const SceneRec* key_scenes, uint8_t* digits, cudaStream_t s) {
  if (n <= 0) return 0;
  const int tiles = (n + kPartTile - 1) / kPartTile;
  k_cam_count<<<tiles, PB, 0, s>>>(job, job_index, first, n, film, pool.nbins, pool.tile_counts, tiles, digits);
  k_scan_exclusive<<<1, 1024, 0, s>>>(pool.tile_counts, tiles * (pool.nbins + 1), nullptr);
  k_part_reserve<<<1, kBinRadix, 0, s>>>(pool.tile_counts, tiles, pool);
  k_cam_scatter<<<tiles, PB, 0, s>>>(job, job_index, first, n, pool.tile_counts, tiles, pool,
                                     pool.keys ? key_scenes : nullptr, digits);
  k_part_commit<<<1, kBinRadix, 0, s>>>(pool.tile_counts, tiles, pool);
  return 5;
}

int launch_bin_partition(const RayBuf& src, int n, BinPool& pool, cudaStream_t s, const int* n_dev,
                         const SceneRec* scenes) {
  if (n <= 0) return 0;
  const int tiles = (n + kPartTile - 1) / kPartTile;
  k_part_count<<<tiles, PB, 0, s>>>(src.d, n, n_dev, pool.nbins, pool.tile_counts, tiles);
  // the dead bucket's row follows the bins', so every bin's total is the
  // difference of two scanned row starts
  k_scan_exclusive<<<1, 1024, 0, s>>>(pool.tile_counts, tiles * (pool.nbins + 1), nullptr);
  k_part_reserve<<<1, kBinRadix, 0, s>>>(pool.tile_counts, tiles, pool);
  k_part_scatter<<<tiles, PB, 0, s>>>(src, n, n_dev, pool.tile_counts, tiles, pool, pool.keys ? scenes : nullptr);
  k_part_commit<<<1, kBinRadix, 0, s>>>(pool.tile_counts, tiles, pool);
  return 5;
}

int launch_pool_reset(BinPool& pool, cudaStream_t s) {
  const int n = std::max(std::max(pool.num_chunks, kMaxBins), pool.pend ? kMaxBins * pool.pend_cols : 0);
  k_pool_reset<<<grid_for(n), TB, 0, s>>>(pool);
  return 1;
}

int launch_ray_bins(const float4* d, int n, int nbins, int* out, cudaStream_t s) {
  if (n <= 0) return 0;
  k_ray_bins<<<grid_for(n), TB, 0, s>>>(d, n, nbins, out);
  return 1;
}

int launch_cardinal(const float4* d, int n, int* out, cudaStream_t s) {
  if (n <= 0) return 0;
  k_cardinal<<<grid_for(n), TB, 0, s>>>(d, n, out);
  return 1;
}

int launch_plan(BinPool& pool, int batch_cap, int merge, int scene_bits, BatchPlan* plan, Counters* ctr,
                cudaStream_t s, bool direct) {
  k_plan<<<1, kBinRadix, 0, s>>>(pool, batch_cap, merge, scene_bits, plan, ctr, direct ? 1 : 0);
  return 1;
}

int launch_append_commit(BinPool& pool, cudaStream_t s) {
  k_append_commit<<<1, kCommitBlock, 0, s>>>(pool);
  return 1;
}

int launch_ray_keys(const BinPool& pool, const BatchPlan* plan, int n_max, int key_bits, uint32_t* keys,
                    cudaStream_t s, uint32_t* where, uint32_t* hist) {
  if (n_max <= 0) return 0;
  if (hist && where && key_bits % 8 == 0 && key_bits <= 32) {
    const int blocks = std::min((n_max + TB - 1) / TB, kKeyHistBlocks);
    k_ray_keys_hist<<<blocks, TB, 0, s>>>(pool.keys, pool.table, pool.max_chunks, plan, key_bits, keys, where, hist);
    return 1;
  }
  k_ray_keys<<<grid_for(n_max), TB, 0, s>>>(pool.keys, pool.table, pool.max_chunks, plan, key_bits, keys, where);
  return 1;
}

int launch_ray_keys_direct(const float4* o, const float4* d, int n, float3 lo, float3 scale, uint32_t* keys,
                           cudaStream_t s) {
  if (n <= 0) return 0;
  k_ray_keys_direct<<<grid_for(n), TB, 0, s>>>(o, d, n, lo, scale, keys);
  return 1;
}

int launch_batch_slots(const BinPool& pool, const BatchPlan* plan, int n_max, const uint32_t* perm, int* slots,
                       cudaStream_t s) {
  if (n_max <= 0) return 0;
  k_batch_slots<<<grid_for(n_max), TB, 0, s>>>(pool.table, pool.max_chunks, plan, perm, slots);
  return 1;
}

// Traversal block size: 64, 128 or 256 threads (an autotuner choice).
#define MSC_TRACE_DISPATCH(KERNEL, BLOCK, WIDE, MULTI, GRID_N, S, ...)                                     \
  do {                                                                                                  \
    const int bs_ = (BLOCK) == 64 ? 64 : ((BLOCK) == 256 ? 256 : 128);                                  \
    const int g_ = grid_for(GRID_N, bs_);                                                               \
    if (bs_ == 64) {                                                                                    \
      if (WIDE) { if (MULTI) KERNEL<true, true, 64><<<g_, 64, 0, S>>>(__VA_ARGS__);                     \
                  else KERNEL<true, false, 64><<<g_, 64, 0, S>>>(__VA_ARGS__); }                         \
      else { if (MULTI) KERNEL<false, true, 64><<<g_, 64, 0, S>>>(__VA_ARGS__);                         \
             else KERNEL<false, false, 64><<<g_, 64, 0, S>>>(__VA_ARGS__); }                             \
    } else if (bs_ == 256) {                                                                            \
      if (WIDE) { if (MULTI) KERNEL<true, true, 256><<<g_, 256, 0, S>>>(__VA_ARGS__);                   \
                  else KERNEL<true, false, 256><<<g_, 256, 0, S>>>(__VA_ARGS__); }                       \
      else { if (MULTI) KERNEL<false, true, 256><<<g_, 256, 0, S>>>(__VA_ARGS__);                       \
             else KERNEL<false, false, 256><<<g_, 256, 0, S>>>(__VA_ARGS__); }                           \
    } else {                                                                                            \
      if (WIDE) { if (MULTI) KERNEL<true, true, 128><<<g_, 128, 0, S>>>(__VA_ARGS__);                   \
                  else KERNEL<true, false, 128><<<g_, 128, 0, S>>>(__VA_ARGS__); }                       \
      else { if (MULTI) KERNEL<false, true, 128><<<g_, 128, 0, S>>>(__VA_ARGS__);                       \
             else KERNEL<false, false, 128><<<g_, 128, 0, S>>>(__VA_ARGS__); }                           \
    }                                                                                                   \
  } while (0)

int launch_trace_closest(const SceneRec* scenes, int num_scenes, const SceneRec& scene0, const float4* o,
                         const float4* d, const int* slots, int n, float4* hits, int* err, cudaStream_t s,
                         const int* n_dev, int block, int* counter) {
  if (n <= 0) return 0;
  const bool wide = scene0.wnodes != nullptr;
  const BvhRef b0 = bvh_of(scene0, wide);
  if (counter && wide) {
    cudaMemsetAsync(counter, 0, sizeof(int), s);
    if (num_scenes > 1)
      k_trace_closest_pt<true><<<persistent_grid(k_trace_closest_pt<true>), kPersistBlock, 0, s>>>(
          scenes, b0, o, d, slots, n, n_dev, hits, err, counter);
    else
      k_trace_closest_pt<false><<<persistent_grid(k_trace_closest_pt<false>), kPersistBlock, 0, s>>>(
          scenes, b0, o, d, slots, n, n_dev, hits, err, counter);
    return 1;
  }
  MSC_TRACE_DISPATCH(k_trace_closest, block, wide, num_scenes > 1, n, s, scenes, b0, o, d, slots, n, n_dev, hits,
                     err);
  return 1;
}

void persistent_grids_init() {
  persistent_grid(k_trace_closest_pt<true>);
  persistent_grid(k_trace_closest_pt<false>);
  persistent_grid(k_trace_shadow_pt<true>);
  persistent_grid(k_trace_shadow_pt<false>);
}

int launch_hit_keys(const SceneRec* scenes, const float4* d, const int* slots, const float4* hits, int n,
                    uint32_t* keys, cudaStream_t s, const int* n_dev) {
  if (n <= 0) return 0;
  k_hit_keys<<<grid_for(n), TB, 0, s>>>(scenes, d, slots, hits, n, n_dev, keys);
  return 1;
}

int launch_hit_keys64(const SceneRec* scenes, const float4* hits, int n, uint32_t* lo, uint32_t* hi,
                      cudaStream_t s, const int* n_dev) {
  if (n <= 0) return 0;
  k_hit_keys64<<<grid_for(n), TB, 0, s>>>(scenes, hits, n, n_dev, lo, hi);
  return 1;
}

int launch_hit_keys_rank(const SceneRec* scenes, const float4* hits, int n, uint32_t* keys, cudaStream_t s,
                         const int* n_dev) {
  if (n <= 0) return 0;
  k_hit_keys_rank<<<grid_for(n), TB, 0, s>>>(scenes, hits, n, n_dev, keys);
  return 1;
}

int launch_gather_u32(const uint32_t* src, const uint32_t* idx, int n, uint32_t* dst, cudaStream_t s,
                      const int* n_dev) {
  if (n <= 0) return 0;
  k_gather_u32<<<grid_for(n), TB, 0, s>>>(src, idx, n, n_dev, dst);
  return 1;
}

int launch_face_texels(unsigned short* texels, int64_t faces, int res, uint32_t seed, cudaStream_t s) {
  const int64_t total = faces * (int64_t)res * res * 3;
  if (total <= 0) return 0;
  k_face_texels<<<152 * 8, TB, 0, s>>>(texels, total, res, seed);
  return 1;
}

int launch_shade(const SceneRec* scenes, const JobRec* jobs, Film film, const RayBuf& batch, const int* slots,
                 const float4* hits, const uint32_t* order, int n, RayBuf next, ShadowBuf sh, int* sh_count,
                 uint32_t* job_done, cudaStream_t s, const int* n_dev, const BinPool* direct,
                 const SceneRec* key_scenes) {
  if (n <= 0) return 0;
  if (direct)
    k_shade<true><<<grid_for(n), TB, 0, s>>>(scenes, jobs, film, batch, slots, hits, order, n, n_dev, next, sh,
                                             sh_count, job_done, *direct, key_scenes);
  else
    k_shade<false><<<grid_for(n), TB, 0, s>>>(scenes, jobs, film, batch, slots, hits, order, n, n_dev, next, sh,
                                              sh_count, job_done, BinPool(), nullptr);
  return 1;
}

int launch_trace_shadow(const SceneRec* scenes, int num_scenes, const SceneRec& scene0, const ShadowBuf& sh,
                        const int* sh_count, int max_n, float4* sample_rgb, int* err, cudaStream_t s,
                        unsigned long long* shadow_total, int block, int* counter) {
  if (max_n <= 0) return 0;
  const bool wide = scene0.wnodes != nullptr;
  const BvhRef b0 = bvh_of(scene0, wide);
  if (counter && wide) {
    cudaMemsetAsync(counter, 0, sizeof(int), s);
    if (num_scenes > 1)
      k_trace_shadow_pt<true><<<persistent_grid(k_trace_shadow_pt<true>), kPersistBlock, 0, s>>>(
          scenes, b0, sh, sh_count, sample_rgb, err, shadow_total, counter);
    else
      k_trace_shadow_pt<false><<<persistent_grid(k_trace_shadow_pt<false>), kPersistBlock, 0, s>>>(
          scenes, b0, sh, sh_count, sample_rgb, err, shadow_total, counter);
    return 1;
  }
  MSC_TRACE_DISPATCH(k_trace_shadow, block, wide, num_scenes > 1, max_n, s, scenes, b0, sh, sh_count, sample_rgb,
                     err, shadow_total);
  return 1;
}

int launch_occluded(const SceneRec& scene, const float4* o, const float4* d, int n, int* occluded, int* err,
                    cudaStream_t s) {
  if (n <= 0) return 0;
  const bool wide = scene.wnodes != nullptr;
  if (wide) k_occluded<true><<<grid_for(n, 128), 128, 0, s>>>(bvh_of(scene, true), o, d, n, occluded, err);
  else k_occluded<false><<<grid_for(n, 128), 128, 0, s>>>(bvh_of(scene, false), o, d, n, occluded, err);
  return 1;
}

int launch_filter(const JobRec& job, Film film, cudaStream_t s) {
  const int n = job.width * job.height;
  if (job.filter == FILTER_BOX) k_filter_box<<<grid_for(n), TB, 0, s>>>(job, film);
  else {
    // the tile's shared memory exceeds the 48 KB default: opt in once (a
    // function-local static is initialised once, also across host threads)
    static const bool attr = [] {
      cudaFuncSetAttribute(k_filter_tent, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(FilterSmem));
      return true;
    }();
    (void)attr;
    k_filter_tent<<<dim3((job.height + kFtY - 1) / kFtY, (job.width + kFtX - 1) / kFtX), kFsN, sizeof(FilterSmem),
                    s>>>(job, film);
  }
  return 1;
}

}  // namespace mscg
