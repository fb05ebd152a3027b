// gs_noalloc.cu -- the key/value sort for callers that cannot allocate device memory.
//
// Some callers may not call cudaMalloc/cudaFree at all: a per-frame callback of a host engine that
// owns the whole device-memory budget, or code that runs while other streams are in flight
// (allocation and release can synchronise the device).  This entry point takes only the caller's keys, values and count and runs the same radix sort as
// gs_sorter_sort_key_value_indirect, with all of its scratch in the fixed array below.
//
// The array is a file-scope __device__ variable, so every GPU that loads this library holds it
// (about 8.4 MB) until the process exits.  Host code cannot pass the symbol itself to a kernel (in
// host code it names a host-side stand-in); the device address is fetched once per device with
// cudaGetSymbolAddress on the first call made with that device current.
#include <cuda_runtime.h>

#include <atomic>
#include <mutex>

#include "../../include/vkgs_gb300.h"
#include "gs_internal.h"

namespace gs {
namespace {

constexpr u32 kMaxCount = GS_SORT_NOALLOC_MAX_COUNT;
constexpr size_t kAlignWords = 64;  // 256 bytes

constexpr size_t round_words(size_t w) { return (w + kAlignWords - 1) / kAlignWords * kAlignWords; }

// Layout of the scratch, in 32-bit words: control block | error word | status (u64) | keys_alt | values_alt
constexpr size_t kControlWords = round_words(kRadixControlBytes / sizeof(u32));
constexpr size_t kErrorWords = kAlignWords;
constexpr size_t kStatusWords = round_words(2 * ((size_t)(kMaxCount + kRadixTile - 1) / kRadixTile) * 256);
constexpr size_t kAltWords = round_words(kMaxCount);
constexpr size_t kScratchWords = kControlWords + kErrorWords + kStatusWords + 2 * kAltWords;

__device__ __align__(256) u32 g_sort_scratch[kScratchWords];

constexpr int kMaxDevices = 64;
std::atomic<u32*> g_scratch_ptr[kMaxDevices];
std::atomic<int> g_num_sms[kMaxDevices];
std::mutex g_setup_mutex;

// Device address of g_sort_scratch (and the SM count) for the current device; set up once per device.
gs_status scratch_for_current_device(u32** scratch, int* sms) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return GS_ERROR_CUDA;
  if (dev < 0 || dev >= kMaxDevices) return GS_ERROR_CUDA;
  u32* p = g_scratch_ptr[dev].load(std::memory_order_acquire);
  if (!p) {
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    p = g_scratch_ptr[dev].load(std::memory_order_acquire);
    if (!p) {
      void* addr = nullptr;
      if (cudaGetSymbolAddress(&addr, g_sort_scratch) != cudaSuccess || addr == nullptr) {
        cudaGetLastError();
        return GS_ERROR_CUDA;
      }
      int n = 0;
      if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return GS_ERROR_CUDA;
      g_num_sms[dev].store(n, std::memory_order_relaxed);
      p = static_cast<u32*>(addr);
      g_scratch_ptr[dev].store(p, std::memory_order_release);
    }
  }
  *scratch = p;
  *sms = g_num_sms[dev].load(std::memory_order_relaxed);
  return GS_SUCCESS;
}

}  // namespace
}  // namespace gs

extern "C" gs_status gs_sort_key_value_noalloc(gs_stream stream, uint32_t max_count, const uint32_t* count,
                                              uint32_t* keys, uint32_t* values, uint32_t* device_error) {
  using namespace gs;
  if (!count || !keys || !values) return GS_ERROR_INVALID_ARGUMENT;
  if (max_count > kMaxCount) return GS_ERROR_CAPACITY;
  if (max_count == 0) return GS_SUCCESS;
  u32* scratch = nullptr;
  int sms = 1;
  const gs_status st = scratch_for_current_device(&scratch, &sms);
  if (st != GS_SUCCESS) return st;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  u32* control = scratch;
  u32* err = scratch + kControlWords;
  u64* status = reinterpret_cast<u64*>(err + kErrorWords);
  u32* keys_alt = scratch + kControlWords + kErrorWords + kStatusWords;
  u32* values_alt = keys_alt + kAltWords;
  // The array keeps the previous call's contents: clear the look-back status words this call uses
  // (the control block is cleared by the sort itself).
  const size_t status_words = radix_status_words(max_count);
  if (status_words * 2 > kStatusWords) return GS_ERROR_CAPACITY;
  if (cudaMemsetAsync(status, 0, status_words * sizeof(u64), s) != cudaSuccess) return GS_ERROR_CUDA;
  RadixSortArgs a{};
  a.keys = keys;
  a.values = values;
  a.keys_alt = keys_alt;
  a.values_alt = values_alt;
  a.count = count;
  a.max_count = max_count;
  a.begin_bit = 0;
  a.end_bit = 32;
  a.control = control;
  a.status = status;
  a.epoch = 1;
  a.err = device_error ? device_error : err;
  a.num_sms = sms;
  return radix_sort(a, s) == cudaSuccess ? GS_SUCCESS : GS_ERROR_CUDA;  // 4 passes: result in place
}
