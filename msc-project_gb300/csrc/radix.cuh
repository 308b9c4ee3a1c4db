// Tile-local stable ranking and the LSD radix sort of 32-bit key/value pairs.
//
// A tile is BLOCK threads x ITEMS items.  Warp w owns the contiguous
// sub-tile [w*32*ITEMS, (w+1)*32*ITEMS); in round k lane l holds item
// w*32*ITEMS + k*32 + l.  Within a round, lanes holding the same digit find
// each other with __match_any_sync; the lowest such lane bumps a per-warp
// digit counter.  Prefixes over warps then give every item its position in
// the tile sorted stably by digit, which is used to stage the tile in shared
// memory so the global scatter writes contiguous runs per digit.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace mscg {

template <int BLOCK, int RADIX>
struct RankSmem {
  int whist[BLOCK / 32][RADIX];
  int tile_start[RADIX];
  int tile_count[RADIX];
  int scan_tmp[BLOCK / 32 + 1];
};

// Exclusive scan of sm.tile_count[0..RADIX) into sm.tile_start.
template <int BLOCK, int RADIX>
__device__ __forceinline__ void tile_digit_scan(RankSmem<BLOCK, RADIX>& sm) {
  constexpr int PER = (RADIX + BLOCK - 1) / BLOCK;
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  int vals[PER];
  int local = 0;
#pragma unroll
  for (int k = 0; k < PER; ++k) {
    int d = t * PER + k;
    vals[k] = d < RADIX ? sm.tile_count[d] : 0;
    local += vals[k];
  }
  int incl = local;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  if (lane == 31) sm.scan_tmp[warp] = incl;
  __syncthreads();
  if (t == 0) {
    int run = 0;
    for (int w = 0; w < BLOCK / 32; ++w) { int c = sm.scan_tmp[w]; sm.scan_tmp[w] = run; run += c; }
  }
  __syncthreads();
  int excl = sm.scan_tmp[warp] + incl - local;
#pragma unroll
  for (int k = 0; k < PER; ++k) {
    int d = t * PER + k;
    if (d < RADIX) sm.tile_start[d] = excl;
    excl += vals[k];
  }
}

// digit[k] < 0 marks an empty slot.  On return pos[k] is the item's index in
// the tile sorted stably by digit (-1 for empty slots), sm.tile_count holds
// the tile histogram and sm.tile_start its exclusive scan.
template <int BLOCK, int ITEMS, int RADIX>
__device__ __forceinline__ void tile_rank(const int (&digit)[ITEMS], int (&pos)[ITEMS], RankSmem<BLOCK, RADIX>& sm) {
  constexpr int WARPS = BLOCK / 32;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int i = threadIdx.x; i < WARPS * RADIX; i += BLOCK) (&sm.whist[0][0])[i] = 0;
  __syncthreads();
  const unsigned lt = (1u << lane) - 1u;
  int rank[ITEMS];
#pragma unroll
  for (int k = 0; k < ITEMS; ++k) {
    const int d = digit[k];
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    const int leader = __ffs(peers) - 1;
    int old = 0;
    if (d >= 0 && lane == leader) {
      old = sm.whist[warp][d];
      sm.whist[warp][d] = old + __popc(peers);
    }
    old = __shfl_sync(0xffffffffu, old, leader);
    rank[k] = old + __popc(peers & lt);
    __syncwarp();
  }
  __syncthreads();
  for (int d = threadIdx.x; d < RADIX; d += BLOCK) {
    int run = 0;
#pragma unroll
    for (int w = 0; w < WARPS; ++w) { int c = sm.whist[w][d]; sm.whist[w][d] = run; run += c; }
    sm.tile_count[d] = run;
  }
  __syncthreads();
  tile_digit_scan<BLOCK, RADIX>(sm);
  __syncthreads();
#pragma unroll
  for (int k = 0; k < ITEMS; ++k) {
    const int d = digit[k];
    pos[k] = d >= 0 ? sm.tile_start[d] + sm.whist[warp][d] + rank[k] : -1;
  }
}

// Single-block exclusive scan of data[0..len) in place; total written to *total if non-null.
__global__ void k_scan_exclusive(uint32_t* data, int len, uint32_t* total);

constexpr int kSortBlock = 256;
constexpr int kSortItems = 16;
constexpr int kSortTile = kSortBlock * kSortItems;
constexpr int kSortRadixBits = 8;
constexpr int kSortMaxPasses = 4;

// Histogram words for any digit width (4: 8 x 16, 8: 4 x 256, 11: 3 x 2048)
// and tile counters for up to 8 passes.
constexpr int kSortHistWords = 3 * 2048;
constexpr int kSortMaxPassesAny = 8;

struct SortScratch {
  uint32_t* keys_alt = nullptr;
  uint32_t* vals_alt = nullptr;
  uint32_t* status = nullptr;   // look-back words: 2 arrays of RADIX * tiles
  uint32_t* hist = nullptr;     // global digit counts of every pass (kSortHistWords)
  uint32_t* ctl = nullptr;      // kSortMaxPassesAny tile counters, then the error word
  int capacity = 0;
  int max_digit_bits = 8;       // widest digit the status arrays were sized for (8 or 11)
};

constexpr size_t sort_align256(size_t x) { return (x + 255) & ~(size_t)255; }
constexpr size_t sort_tiles(int capacity) {
  return capacity <= 0 ? 1 : ((size_t)capacity + kSortTile - 1) / kSortTile;
}
// Look-back words per status array: tiles x radix, the largest over the digit
// widths up to max_digit_bits (11-bit digits use tiles of 2048 keys).
constexpr size_t sort_status_words(int capacity, int max_digit_bits) {
  return max_digit_bits >= 11 ? ((size_t)(capacity > 0 ? capacity : 1) + 2047) / 2048 * 2048
                              : sort_tiles(capacity) * 256;
}
// Scratch bytes for sorts of up to `capacity` pairs with digits of up to
// max_digit_bits (8 or 11) bits.
constexpr size_t sort_scratch_bytes(int capacity, int max_digit_bits = 8) {
  return 2 * sort_align256((size_t)(capacity > 0 ? capacity : 1) * 4) +
         sort_align256(2 * sort_status_words(capacity, max_digit_bits) * 4) +
         sort_align256((size_t)kSortHistWords * 4 + 64);
}
// Carves the scratch buffers out of `base` (sort_scratch_bytes(capacity, max_digit_bits) bytes, 256-aligned).
void sort_scratch_bind(SortScratch* s, void* base, int capacity, int max_digit_bits = 8);
// Opts the pass kernels into the shared memory they need (idempotent; call
// before any stream capture).
void sort_init();

// Test hook of the look-back's bounded wait: a smaller spin cap, and a first
// tile that never posts its counts, so that every later tile's wait runs out.
struct SortTestHook {
  int spin_cap = 1 << 20;
  int withhold_first_tile = 0;
};

// Stable LSD sort of (keys_in, vals_in) on bits [0, bits) into (keys_out, vals_out).
// vals_in == nullptr means vals_in[i] = i.  Input buffers are left unchanged
// unless they alias the outputs.  One histogram kernel for all passes, then
// one kernel per digit pass with a decoupled look-back across tiles.  Spin
// waits are capped; a cap that runs out sets bit 8 of *err (when err is not
// null).  Returns the number of kernel launches.  n_dev (optional): the pair
// count is read on the device when the kernels run and n is its upper bound
// (sizes the grids); this form needs outputs distinct from the inputs when
// the pass count is odd, and returns -1 otherwise.
// digit_bits: 4, 8 or 11 (an 11-bit sort needs scratch bound for 11 bits,
// else it falls back to 8).  hook (tests only): see SortTestHook.
// hist_ready (8-bit digits only): the caller zeroed s.hist and s.ctl (one
// memset of kSortHistWords * 4 + 64 bytes from s.hist) and then counted the
// keys' digits into s.hist (pass p's digit d at p * 256 + d) while it made
// them, so the sort skips its own counting pass.
int sort_pairs(const uint32_t* keys_in, const uint32_t* vals_in, uint32_t* keys_out, uint32_t* vals_out, int n,
               int bits, SortScratch& s, cudaStream_t stream, int* err = nullptr, const int* n_dev = nullptr,
               int digit_bits = 8, const SortTestHook* hook = nullptr, bool hist_ready = false);

constexpr int kSortErrLookback = 256;

}  // namespace mscg
