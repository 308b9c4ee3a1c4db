// Stable LSD radix sort of 32-bit keys with 32-bit values, 4-, 8- or 11-bit
// digits.
//
// sort_pairs: one histogram kernel counts the digits of every pass in a
// single read of the keys; then each pass is one kernel.  A block takes the
// next tile from a counter, ranks its keys stably (tile_rank: warp match +
// per-warp counters), publishes its per-digit counts, and sums its
// predecessors' counts by a decoupled look-back (each tile first posts an
// aggregate, then its inclusive prefix).  The tile is staged in shared memory
// in digit order, so the global scatter writes contiguous runs.
//
// It replaces the reference's comparison sorts of a batch (tbb::parallel_sort
// in src/core/RaySort.cpp:17,97 and the hit sort of src/core/Pathtracer.cpp:335-339)
// with a key-based stable order.
#include "radix.cuh"

namespace mscg {

namespace {

constexpr uint32_t kFlagAggregate = 1u;
constexpr uint32_t kFlagPrefix = 2u;
constexpr int kLookbackSpinCap = 1 << 20;
constexpr int kLookbackWindow = 8;

__device__ __forceinline__ uint32_t ld_volatile(const uint32_t* p) { return *(const volatile uint32_t*)p; }
__device__ __forceinline__ void st_volatile(uint32_t* p, uint32_t v) { *(volatile uint32_t*)p = v; }

// ------------------------------------------------------------- onesweep
__device__ __forceinline__ int sort_count(int n_max, const int* n_dev) {
  return n_dev ? min(*n_dev, n_max) : n_max;
}

// Digit width RB (4, 8 or 11 bits): radix, keys per thread, tile and passes.
template <int RB>
struct SortShape {
  static constexpr int RADIX = 1 << RB;
  static constexpr int ITEMS = RB > 8 ? 8 : kSortItems;
  static constexpr int TILE = kSortBlock * ITEMS;
  static constexpr int MAXP = (32 + RB - 1) / RB;
  static constexpr int DPT = RADIX > kSortBlock ? RADIX / kSortBlock : 1;  // digits per thread
};

template <int RB>
__global__ void __launch_bounds__(kSortBlock) k_onesweep_hist(const uint32_t* __restrict__ keys, int n_max,
                                                              const int* __restrict__ n_dev, int passes, int bits,
                                                              uint32_t* __restrict__ hist) {
  using S = SortShape<RB>;
  const int n = sort_count(n_max, n_dev);
  __shared__ uint32_t sh[S::MAXP * S::RADIX];
  for (int i = threadIdx.x; i < S::MAXP * S::RADIX; i += kSortBlock) sh[i] = 0;
  __syncthreads();
  // four keys per thread and step, loaded before any is counted (independent
  // loads in flight); shared-memory atomics are cheaper than grouping equal
  // digits first
  constexpr int U = 4;
  const int stride = gridDim.x * kSortBlock * U;
  for (int base = blockIdx.x * kSortBlock * U; base < n; base += stride) {
    uint32_t key[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int idx = base + u * kSortBlock + threadIdx.x;
      key[u] = idx < n ? keys[idx] : 0u;
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      if (base + u * kSortBlock + (int)threadIdx.x >= n) break;
      for (int p = 0; p < passes; ++p) {
        const int shift = p * RB;
        const int width = bits - shift < RB ? bits - shift : RB;
        atomicAdd(&sh[p * S::RADIX + ((key[u] >> shift) & ((1u << width) - 1u))], 1u);
      }
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < passes * S::RADIX; i += kSortBlock) {
    const uint32_t c = sh[i];
    if (c) atomicAdd(&hist[i], c);
  }
}

// Exclusive scan of one value per thread over a 256-thread block.
__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t* warp_tmp) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t incl = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  if (lane == 31) warp_tmp[warp] = incl;
  __syncthreads();
  uint32_t before = 0;
  for (int w = 0; w < warp; ++w) before += warp_tmp[w];
  __syncthreads();
  return before + incl - v;
}

template <int RB>
struct PassSmem {
  using S = SortShape<RB>;
  RankSmem<kSortBlock, S::RADIX> rank;
  uint32_t skey[S::TILE];
  uint32_t sval[S::TILE];
  uint32_t gofs[S::RADIX];
  uint32_t warp_tmp[kSortBlock / 32];
  int tile;
};

// One pass: thread t owns digits [t*DPT, (t+1)*DPT) (the first RADIX threads
// when the radix is smaller than the block) for the scan and the look-back.
template <int RB>
__global__ void __launch_bounds__(kSortBlock) k_onesweep_pass(const uint32_t* __restrict__ keys_in,
                                                              const uint32_t* __restrict__ vals_in,
                                                              uint32_t* __restrict__ keys_out,
                                                              uint32_t* __restrict__ vals_out, int n_max,
                                                              const int* __restrict__ n_dev, int shift,
                                                              uint32_t mask, int pass,
                                                              const uint32_t* __restrict__ hist, uint32_t* status_cur,
                                                              uint32_t* status_next, uint32_t* ctl, int* err,
                                                              int spin_cap, int withhold_first) {
  using S = SortShape<RB>;
  constexpr int RADIX = S::RADIX, DPT = S::DPT, ITEMS = S::ITEMS, TILE = S::TILE;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  PassSmem<RB>& sm = *reinterpret_cast<PassSmem<RB>*>(smem_raw);
  const int d0 = threadIdx.x * DPT;
  const bool owns = d0 < RADIX;
  if (threadIdx.x == 0) sm.tile = (int)atomicAdd(&ctl[pass], 1u);
  // global start of each owned digit: exclusive scan of the pass histogram
  uint32_t hv[DPT], own = 0;
#pragma unroll
  for (int k = 0; k < DPT; ++k) {
    hv[k] = owns ? hist[pass * RADIX + d0 + k] : 0u;
    own += hv[k];
  }
  uint32_t run = block_excl_scan(own, sm.warp_tmp);  // syncs inside
  uint32_t dstart[DPT];
#pragma unroll
  for (int k = 0; k < DPT; ++k) {
    dstart[k] = run;
    run += hv[k];
  }
  const int tile = sm.tile;
  const int base = tile * TILE;
  const int n = sort_count(n_max, n_dev);
  if (base >= n) return;  // the whole block: past a batch smaller than the launch
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  // the next pass reads status_next from zero; the pass that last used it has finished
  if (status_next && owns)
#pragma unroll
    for (int k = 0; k < DPT; ++k) status_next[tile * RADIX + d0 + k] = 0u;
  uint32_t key[ITEMS], val[ITEMS];
  int dig[ITEMS], pos[ITEMS];
#pragma unroll
  for (int k = 0; k < ITEMS; ++k) {
    const int idx = base + warp * 32 * ITEMS + k * 32 + lane;
    const bool ok = idx < n;
    key[k] = ok ? keys_in[idx] : 0u;
    val[k] = ok ? (vals_in ? vals_in[idx] : (uint32_t)idx) : 0u;
    dig[k] = ok ? (int)((key[k] >> shift) & mask) : -1;
  }
  tile_rank<kSortBlock, ITEMS, RADIX>(dig, pos, sm.rank);
  if (owns) {
    uint32_t cnt[DPT];
    // post every owned aggregate first, so successors can sum past this tile
#pragma unroll
    for (int k = 0; k < DPT; ++k) {
      cnt[k] = (uint32_t)sm.rank.tile_count[d0 + k];
      // (withhold_first: a test of the spin cap - the first tile never posts)
      if (!(withhold_first && tile == 0))
        st_volatile(&status_cur[tile * RADIX + d0 + k], (cnt[k] << 2) | (tile == 0 ? kFlagPrefix : kFlagAggregate));
    }
#pragma unroll
    for (int k = 0; k < DPT; ++k) {
      const int d = d0 + k;
      uint32_t excl = 0;
      if (tile > 0) {
        // Look back a window of kLookbackWindow predecessors per step (independent
        // loads), summing aggregates up to the first inclusive prefix.
        int t = tile - 1;
        int spins = 0;
        while (t >= 0) {
          uint32_t v[kLookbackWindow];
#pragma unroll
          for (int w = 0; w < kLookbackWindow; ++w)
            v[w] = (t - w >= 0) ? ld_volatile(&status_cur[(t - w) * RADIX + d]) : kFlagPrefix;
          int used = 0;
          bool done = false;
#pragma unroll
          for (int w = 0; w < kLookbackWindow; ++w) {
            if (done || used < w) continue;  // stop at the first prefix or the first unposted tile
            const uint32_t f = v[w] & 3u;
            if (f == 0u) continue;           // not posted yet: re-read from here
            excl += v[w] >> 2;
            used = w + 1;
            if (f == kFlagPrefix) done = true;
          }
          if (done) break;
          t -= used;
          if (used < kLookbackWindow) {  // a predecessor has not posted yet; it is running, so this ends
            if (++spins > spin_cap) {
              atomicOr(err, kSortErrLookback);
              break;
            }
          }
        }
        st_volatile(&status_cur[tile * RADIX + d], ((excl + cnt[k]) << 2) | kFlagPrefix);
      }
      sm.gofs[d] = dstart[k] + excl;
    }
  }
#pragma unroll
  for (int k = 0; k < ITEMS; ++k) {
    if (pos[k] >= 0) {
      sm.skey[pos[k]] = key[k];
      sm.sval[pos[k]] = val[k];
    }
  }
  __syncthreads();
  const int count = min(TILE, n - base);
  for (int p = threadIdx.x; p < count; p += kSortBlock) {
    const uint32_t k = sm.skey[p];
    const int d = (int)((k >> shift) & mask);
    const uint32_t o = sm.gofs[d] + (uint32_t)(p - sm.rank.tile_start[d]);
    keys_out[o] = k;
    vals_out[o] = sm.sval[p];
  }
}

__global__ void k_copy_u32(const uint32_t* __restrict__ src, uint32_t* __restrict__ dst, int n, int iota) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = iota ? (uint32_t)i : src[i];
}

// Shared front part of both sorts: the zero-bit case and odd-pass aliasing.
int sort_prologue(const uint32_t*& src_k, const uint32_t*& src_v, const uint32_t* keys_in, const uint32_t* vals_in,
                  uint32_t* keys_out, uint32_t* vals_out, int n, int passes, SortScratch& s, cudaStream_t stream,
                  bool* done) {
  *done = false;
  int launches = 0;
  src_k = keys_in;
  src_v = vals_in;
  if (passes == 0) {
    const int tb = 256, g = (n + tb - 1) / tb;
    if (keys_in != keys_out) cudaMemcpyAsync(keys_out, keys_in, (size_t)n * 4, cudaMemcpyDeviceToDevice, stream);
    if (vals_in == nullptr) {
      k_copy_u32<<<g, tb, 0, stream>>>(nullptr, vals_out, n, 1);
      ++launches;
    } else if (vals_in != vals_out) {
      cudaMemcpyAsync(vals_out, vals_in, (size_t)n * 4, cudaMemcpyDeviceToDevice, stream);
    }
    *done = true;
    return launches;
  }
  if ((passes % 2) == 1 && (keys_in == keys_out || (vals_in != nullptr && vals_in == vals_out))) {
    // an odd pass count writes the outputs first: move the inputs out of the way
    cudaMemcpyAsync(s.keys_alt, keys_in, (size_t)n * 4, cudaMemcpyDeviceToDevice, stream);
    if (vals_in) cudaMemcpyAsync(s.vals_alt, vals_in, (size_t)n * 4, cudaMemcpyDeviceToDevice, stream);
    src_k = s.keys_alt;
    src_v = vals_in ? s.vals_alt : nullptr;
  }
  return launches;
}

}  // namespace

// Chunks of 8 x 1024 words are staged in shared memory with coalesced loads
// (padded one word in 32 against bank conflicts); each thread scans 8
// consecutive words, the block scans the thread sums, and a carry runs
// across chunks.
__global__ void __launch_bounds__(1024) k_scan_exclusive(uint32_t* data, int len, uint32_t* total) {
  constexpr int P = 8, CH = 1024 * P;
  __shared__ uint32_t buf[CH + CH / 32];
  __shared__ uint32_t warp_sums[32];
  __shared__ uint32_t chunk_end;
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  auto at = [](int i) { return i + (i >> 5); };
  uint32_t carry = 0;
  for (int c0 = 0; c0 < len; c0 += CH) {
    const int m = min(CH, len - c0);
    for (int i = t; i < CH; i += 1024) buf[at(i)] = i < m ? data[c0 + i] : 0u;
    __syncthreads();
    uint32_t v[P], local = 0;
#pragma unroll
    for (int k = 0; k < P; ++k) {
      v[k] = buf[at(t * P + k)];
      local += v[k];
    }
    uint32_t incl = local;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += y;
    }
    if (lane == 31) warp_sums[warp] = incl;
    __syncthreads();
    if (warp == 0) {
      const uint32_t w = warp_sums[lane];
      uint32_t wi = w;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, wi, o);
        if (lane >= o) wi += y;
      }
      warp_sums[lane] = wi - w;
    }
    __syncthreads();
    uint32_t run = carry + warp_sums[warp] + incl - local;
#pragma unroll
    for (int k = 0; k < P; ++k) {
      buf[at(t * P + k)] = run;
      run += v[k];
    }
    // the running total after this chunk: thread 1023's sum
    if (t == 1023) chunk_end = run;
    __syncthreads();
    for (int i = t; i < m; i += 1024) data[c0 + i] = buf[at(i)];
    carry = chunk_end;
    __syncthreads();
  }
  if (t == 0 && total) *total = carry;
}

void sort_scratch_bind(SortScratch* s, void* base, int capacity, int max_digit_bits) {
  const size_t cap = (size_t)(capacity > 0 ? capacity : 1);
  char* p = (char*)base;
  s->keys_alt = (uint32_t*)p;
  p += sort_align256(cap * 4);
  s->vals_alt = (uint32_t*)p;
  p += sort_align256(cap * 4);
  s->status = (uint32_t*)p;
  p += sort_align256(2 * sort_status_words(capacity, max_digit_bits) * 4);
  s->hist = (uint32_t*)p;
  s->ctl = s->hist + kSortHistWords;
  s->capacity = capacity;
  s->max_digit_bits = max_digit_bits >= 11 ? 11 : 8;
}

namespace {
template <int RB>
int onesweep(const uint32_t* keys_in, const uint32_t* vals_in, uint32_t* keys_out, uint32_t* vals_out, int n, int bits,
             SortScratch& s, cudaStream_t stream, int* err, const int* n_dev, const SortTestHook* hook,
             bool hist_ready) {
  using S = SortShape<RB>;
  const int passes = (bits + RB - 1) / RB;
  if (n_dev && (passes == 0 || ((passes % 2) == 1 && (keys_in == keys_out || (vals_in && vals_in == vals_out)))))
    return -1;  // a device count needs distinct outputs and at least one pass
  const uint32_t* src_k;
  const uint32_t* src_v;
  bool done;
  int launches = sort_prologue(src_k, src_v, keys_in, vals_in, keys_out, vals_out, n, passes, s, stream, &done);
  if (done) return launches;
  const int tiles = (n + S::TILE - 1) / S::TILE;
  uint32_t* status0 = s.status;
  uint32_t* status1 = s.status + (size_t)tiles * S::RADIX;
  // zero the first look-back array, the histograms, the tile counters and the error word
  cudaMemsetAsync(status0, 0, (size_t)tiles * S::RADIX * 4, stream);
  int* errw = err ? err : (int*)(s.ctl + kSortMaxPassesAny);
  if (!hist_ready || RB != 8 || src_k != keys_in) {
    cudaMemsetAsync(s.hist, 0, (size_t)kSortHistWords * 4 + 64, stream);
    const int hist_blocks = std::min(std::max(1, (n + S::TILE - 1) / S::TILE), 4 * 152);
    k_onesweep_hist<RB><<<hist_blocks, kSortBlock, 0, stream>>>(src_k, n, n_dev, passes, bits, s.hist);
    ++launches;
  }
  for (int p = 0; p < passes; ++p) {
    const bool to_out = ((passes - 1 - p) % 2) == 0;
    uint32_t* dst_k = to_out ? keys_out : s.keys_alt;
    uint32_t* dst_v = to_out ? vals_out : s.vals_alt;
    const int shift = p * RB;
    const int width = bits - shift < RB ? bits - shift : RB;  // the last pass may be narrower
    const uint32_t mask = (1u << width) - 1u;
    uint32_t* cur = (p & 1) ? status1 : status0;
    uint32_t* next = (p + 1 < passes) ? ((p & 1) ? status0 : status1) : nullptr;
    k_onesweep_pass<RB><<<tiles, kSortBlock, sizeof(PassSmem<RB>), stream>>>(
        src_k, src_v, dst_k, dst_v, n, n_dev, shift, mask, p, s.hist, cur, next, s.ctl, errw,
        hook ? hook->spin_cap : kLookbackSpinCap, hook ? hook->withhold_first_tile : 0);
    ++launches;
    src_k = dst_k;
    src_v = dst_v;
  }
  return launches;
}
}  // namespace

void sort_init() {
  static bool done = false;
  if (done) return;
  done = true;
  cudaFuncSetAttribute(k_onesweep_pass<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(PassSmem<4>));
  cudaFuncSetAttribute(k_onesweep_pass<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(PassSmem<8>));
  cudaFuncSetAttribute(k_onesweep_pass<11>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(PassSmem<11>));
}

int sort_pairs(const uint32_t* keys_in, const uint32_t* vals_in, uint32_t* keys_out, uint32_t* vals_out, int n,
               int bits, SortScratch& s, cudaStream_t stream, int* err, const int* n_dev, int digit_bits,
               const SortTestHook* hook, bool hist_ready) {
  if (n <= 0) return 0;
  sort_init();
  if (digit_bits > s.max_digit_bits) digit_bits = 8;  // scratch sized for narrower digits
  if (digit_bits == 4)
    return onesweep<4>(keys_in, vals_in, keys_out, vals_out, n, bits, s, stream, err, n_dev, hook, false);
  if (digit_bits == 11)
    return onesweep<11>(keys_in, vals_in, keys_out, vals_out, n, bits, s, stream, err, n_dev, hook, false);
  return onesweep<8>(keys_in, vals_in, keys_out, vals_out, n, bits, s, stream, err, n_dev, hook, hist_ready);
}

}  // namespace mscg
