// Radix sort of device key/value pairs that performs no device allocation.
//
// Some callers cannot allocate device memory while they run: a host
// application that reserves its whole device-memory budget up front (a render
// server, or a plugin host that owns the device pool) has nothing left for a
// cudaMalloc at run time, and a latency-critical frame loop cannot afford the
// device-wide synchronisation that cudaFree implies.  This entry point serves
// them: its scratch (the ping-pong key/value buffers and the digit-count
// table) is one file-scope __device__ array of kNoAllocBytes bytes, which
// every GPU that loads this library holds until the process exits.
//
// The first call on a device looks up the array's device address with
// cudaGetSymbolAddress while that device is current, so make that first call
// before any stream capture on the device.  All calls share the one array and
// it keeps the previous call's contents; every byte a sort reads is written by
// the same sort first, so nothing needs clearing.  Calls whose work overlaps
// on the GPU (two streams, or two host threads) race on the array and must be
// serialised by the caller.  A look-back wait of the sort that runs out of its
// spin cap (possible only if the GPU failed to schedule a running tile's
// predecessor) sets a word inside the static array that no call reads: such a
// sort returns MSC_OK with unsorted output.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "../../include/msc_gpu.h"
#include "radix.cuh"

namespace mscg {
void set_global_error(const std::string& msg);  // defined in engine.cu
}

namespace {

constexpr int kNoAllocMaxPairs = 1 << 20;
constexpr size_t kNoAllocBytes = mscg::sort_scratch_bytes(kNoAllocMaxPairs);

static __device__ __align__(256) unsigned char g_sort_scratch[kNoAllocBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_scratch_ptr[kMaxDevices] = {nullptr};

int scratch_for_current_device(void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    mscg::set_global_error(std::string("msc_sort_pairs_device_noalloc: cudaGetDevice: ") + cudaGetErrorString(e));
    return MSC_ERR_CUDA;
  }
  if (dev < 0 || dev >= kMaxDevices) {
    mscg::set_global_error("msc_sort_pairs_device_noalloc: device index out of range");
    return MSC_ERR_ARG;
  }
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_sort_scratch);
    if (e != cudaSuccess || p == nullptr) {
      mscg::set_global_error(std::string("msc_sort_pairs_device_noalloc: cudaGetSymbolAddress: ") +
                             cudaGetErrorString(e));
      return MSC_ERR_CUDA;
    }
    g_scratch_ptr[dev] = p;
  }
  *out = g_scratch_ptr[dev];
  return MSC_OK;
}

}  // namespace

extern "C" int msc_sort_pairs_device_noalloc(uint32_t* keys, uint32_t* vals, int n, int bits, void* stream) {
  if (n < 0 || bits < 0 || bits > 32 || (n > 0 && (!keys || !vals))) {
    mscg::set_global_error("msc_sort_pairs_device_noalloc: bad argument");
    return MSC_ERR_ARG;
  }
  if (n > kNoAllocMaxPairs) {
    mscg::set_global_error("msc_sort_pairs_device_noalloc: n = " + std::to_string(n) + " exceeds the maximum of " +
                           std::to_string(kNoAllocMaxPairs) + " pairs of its static scratch");
    return MSC_ERR_ARG;
  }
  if (n == 0) return MSC_OK;
  // an error left by the caller's own earlier work is reported as it is and
  // not cleared, so that the launch check below sees only this call's errors
  cudaError_t pending = cudaPeekAtLastError();
  if (pending != cudaSuccess) {
    mscg::set_global_error(std::string("msc_sort_pairs_device_noalloc: an earlier CUDA error is pending: ") +
                           cudaGetErrorString(pending));
    return MSC_ERR_CUDA;
  }
  void* scratch = nullptr;
  int rc = scratch_for_current_device(&scratch);
  if (rc != MSC_OK) return rc;
  if (mscg::sort_scratch_bytes(n) > kNoAllocBytes) {
    mscg::set_global_error("msc_sort_pairs_device_noalloc: internal scratch size mismatch");
    return MSC_ERR_ARG;
  }
  mscg::SortScratch ss;
  mscg::sort_scratch_bind(&ss, scratch, n);
  mscg::sort_pairs(keys, vals, keys, vals, n, bits, ss, (cudaStream_t)stream);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    mscg::set_global_error(std::string("msc_sort_pairs_device_noalloc: launch failed: ") + cudaGetErrorString(e));
    return MSC_ERR_CUDA;
  }
  return MSC_OK;
}
