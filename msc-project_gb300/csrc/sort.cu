// Stable LSD radix sort of 32-bit keys with 32-bit values (reduce-then-scan
// per 8-bit digit): an upsweep counts digits per tile, one block scans the
// digit-major count table, and a downsweep ranks each tile stably, stages it
// in shared memory in digit order and writes contiguous runs.
//
// It replaces the reference's comparison sorts on the batch
// (tbb::parallel_sort in src/core/RaySort.cpp:17,97 and the hit sort in
// src/core/Pathtracer.cpp:335-339) with a key-based stable order.
#include "radix.cuh"

namespace mscg {

namespace {

constexpr int RADIX = 1 << kSortRadixBits;

__global__ void __launch_bounds__(kSortBlock) k_radix_upsweep(const uint32_t* __restrict__ keys, int n, int shift, uint32_t mask,
                                                              uint32_t* __restrict__ counts, int num_tiles) {
  __shared__ int hist[RADIX];
  for (int i = threadIdx.x; i < RADIX; i += kSortBlock) hist[i] = 0;
  __syncthreads();
  const int base = blockIdx.x * kSortTile;
  const int lane = threadIdx.x & 31;
#pragma unroll 4
  for (int k = 0; k < kSortItems; ++k) {
    int idx = base + k * kSortBlock + threadIdx.x;
    int d = idx < n ? (int)((keys[idx] >> shift) & mask) : -1;
    unsigned peers = __match_any_sync(0xffffffffu, d);
    if (d >= 0 && lane == __ffs(peers) - 1) atomicAdd(&hist[d], __popc(peers));
  }
  __syncthreads();
  for (int d = threadIdx.x; d < RADIX; d += kSortBlock) counts[d * num_tiles + blockIdx.x] = (uint32_t)hist[d];
}

__global__ void __launch_bounds__(kSortBlock) k_radix_downsweep(const uint32_t* __restrict__ keys_in,
                                                                const uint32_t* __restrict__ vals_in,
                                                                uint32_t* __restrict__ keys_out,
                                                                uint32_t* __restrict__ vals_out, int n, int shift, uint32_t mask,
                                                                const uint32_t* __restrict__ offsets, int num_tiles) {
  __shared__ RankSmem<kSortBlock, RADIX> sm;
  __shared__ uint32_t skey[kSortTile];
  __shared__ uint32_t sval[kSortTile];
  __shared__ uint32_t gofs[RADIX];
  const int tile = blockIdx.x;
  const int base = tile * kSortTile;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int d = threadIdx.x; d < RADIX; d += kSortBlock) gofs[d] = offsets[d * num_tiles + tile];
  uint32_t key[kSortItems], val[kSortItems];
  int dig[kSortItems], pos[kSortItems];
#pragma unroll
  for (int k = 0; k < kSortItems; ++k) {
    int idx = base + warp * 32 * kSortItems + k * 32 + lane;
    bool ok = idx < n;
    key[k] = ok ? keys_in[idx] : 0u;
    val[k] = ok ? (vals_in ? vals_in[idx] : (uint32_t)idx) : 0u;
    dig[k] = ok ? (int)((key[k] >> shift) & mask) : -1;
  }
  tile_rank<kSortBlock, kSortItems, RADIX>(dig, pos, sm);
#pragma unroll
  for (int k = 0; k < kSortItems; ++k) {
    if (pos[k] >= 0) {
      skey[pos[k]] = key[k];
      sval[pos[k]] = val[k];
    }
  }
  __syncthreads();
  const int count = min(kSortTile, n - base);
  for (int p = threadIdx.x; p < count; p += kSortBlock) {
    uint32_t k = skey[p];
    int d = (int)((k >> shift) & mask);
    uint32_t o = gofs[d] + (uint32_t)(p - sm.tile_start[d]);
    keys_out[o] = k;
    vals_out[o] = sval[p];
  }
}

__global__ void k_copy_u32(const uint32_t* __restrict__ src, uint32_t* __restrict__ dst, int n, int iota) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = iota ? (uint32_t)i : src[i];
}

}  // namespace

__global__ void __launch_bounds__(1024) k_scan_exclusive(uint32_t* data, int len, uint32_t* total) {
  __shared__ uint32_t warp_sums[32];
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  const int per = (len + 1023) / 1024;
  const int b = t * per;
  const int e = min(len, b + per);
  uint32_t local = 0;
  for (int i = b; i < e; ++i) local += data[i];
  uint32_t incl = local;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  if (lane == 31) warp_sums[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = warp_sums[lane];
    uint32_t wi = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t y = __shfl_up_sync(0xffffffffu, wi, o);
      if (lane >= o) wi += y;
    }
    warp_sums[lane] = wi - w;
    if (lane == 31 && total) *total = wi;
  }
  __syncthreads();
  uint32_t run = warp_sums[warp] + incl - local;
  for (int i = b; i < e; ++i) {
    uint32_t v = data[i];
    data[i] = run;
    run += v;
  }
}

static size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

size_t sort_scratch_bytes(int capacity) {
  size_t tiles = (size_t)(capacity + kSortTile - 1) / kSortTile;
  if (tiles == 0) tiles = 1;
  return align256((size_t)capacity * 4) * 2 + align256(tiles * RADIX * 4);
}

void sort_scratch_bind(SortScratch* s, void* base, int capacity) {
  char* p = (char*)base;
  s->keys_alt = (uint32_t*)p;
  p += align256((size_t)capacity * 4);
  s->vals_alt = (uint32_t*)p;
  p += align256((size_t)capacity * 4);
  s->counts = (uint32_t*)p;
  s->capacity = capacity;
}

int sort_pairs(const uint32_t* keys_in, const uint32_t* vals_in, uint32_t* keys_out, uint32_t* vals_out, int n,
               int bits, SortScratch& s, cudaStream_t stream) {
  if (n <= 0) return 0;
  int passes = (bits + kSortRadixBits - 1) / kSortRadixBits;
  int launches = 0;
  if (passes == 0) {
    const int tb = 256, g = (n + tb - 1) / tb;
    if (keys_in != keys_out) { cudaMemcpyAsync(keys_out, keys_in, (size_t)n * 4, cudaMemcpyDeviceToDevice, stream); }
    if (vals_in == nullptr) { k_copy_u32<<<g, tb, 0, stream>>>(nullptr, vals_out, n, 1); ++launches; }
    else if (vals_in != vals_out) cudaMemcpyAsync(vals_out, vals_in, (size_t)n * 4, cudaMemcpyDeviceToDevice, stream);
    return launches;
  }
  const int tiles = (n + kSortTile - 1) / kSortTile;
  const uint32_t* src_k = keys_in;
  const uint32_t* src_v = vals_in;
  if ((passes % 2) == 1 && (keys_in == keys_out || (vals_in != nullptr && vals_in == vals_out))) {
    // an odd pass count writes the outputs first: move the inputs out of the way
    cudaMemcpyAsync(s.keys_alt, keys_in, (size_t)n * 4, cudaMemcpyDeviceToDevice, stream);
    if (vals_in) cudaMemcpyAsync(s.vals_alt, vals_in, (size_t)n * 4, cudaMemcpyDeviceToDevice, stream);
    src_k = s.keys_alt;
    src_v = vals_in ? s.vals_alt : nullptr;
  }
  for (int p = 0; p < passes; ++p) {
    bool to_out = ((passes - 1 - p) % 2) == 0;
    uint32_t* dst_k = to_out ? keys_out : s.keys_alt;
    uint32_t* dst_v = to_out ? vals_out : s.vals_alt;
    const int shift = p * kSortRadixBits;
    // the last pass only looks at the bits below `bits`
    const int width = bits - shift < kSortRadixBits ? bits - shift : kSortRadixBits;
    const uint32_t mask = (1u << width) - 1u;
    k_radix_upsweep<<<tiles, kSortBlock, 0, stream>>>(src_k, n, shift, mask, s.counts, tiles);
    k_scan_exclusive<<<1, 1024, 0, stream>>>(s.counts, tiles * RADIX, nullptr);
    k_radix_downsweep<<<tiles, kSortBlock, 0, stream>>>(src_k, src_v, dst_k, dst_v, n, shift, mask, s.counts,
                                                         tiles);
    launches += 3;
    src_k = dst_k;
    src_v = dst_v;
  }
  return launches;
}

}  // namespace mscg
