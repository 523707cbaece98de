// rq_sort_pairs_noalloc: the stable radix sort of rq_sort_pairs for callers
// that must not allocate device memory while they run.
//
// Who needs it: a process that sizes all of its device memory up front (a
// serving loop held to a fixed HBM budget), code whose device memory is owned
// and accounted by another allocator, and latency-critical loops, where a
// cudaMalloc or cudaFree would synchronize the device and stall other work.
// Such callers hand in their own device buffers for the keys and values; the
// sort's working memory (ping-pong copies, digit histograms, look-back words)
// comes from one fixed-size array that lives in this file for as long as the
// library is loaded.
#include <cuda_runtime.h>

#include "rq_device.cuh"
#include "rq_internal.hpp"

namespace rq {
namespace {

// Working memory layout, in 32-bit words:
//   [0, N)            keys ping-pong copy        [N, 2N)   values ping-pong copy
//   [2N, 2N+1024)     digit histograms (4 x 256) [+16]     tile counters, one per pass
//   [.., +kStatus)    look-back words            [+16]     error word and padding
constexpr uint32_t kMaxPairs = RQ_SORT_NOALLOC_MAX_PAIRS;
constexpr int kMaxPasses = 4;
constexpr uint32_t kTileKeys = 3840;  // keys per tile of the onesweep kernel
constexpr size_t kMaxTiles = (kMaxPairs + kTileKeys - 1) / kTileKeys;
constexpr size_t kStatusWords = (size_t)kMaxPasses * kMaxTiles * 256;
constexpr size_t kHistOff = 2 * (size_t)kMaxPairs;
constexpr size_t kCounterOff = kHistOff + 1024;
constexpr size_t kStatusOff = kCounterOff + 16;
constexpr size_t kErrOff = kStatusOff + kStatusWords;
constexpr size_t kWords = kErrOff + 16;

// One array per GPU that loads the library (about 9.5 MB), shared by every call.
static __device__ __align__(256) uint32_t g_sort_scratch[kWords];

// Device address of g_sort_scratch on the current device, looked up on every
// call.  Host code must not use the symbol itself as a pointer: on the host it
// names a stand-in, not device memory.  The lookup is not cached: after a
// cudaDeviceReset (or a primary context released and created again) the
// module is loaded anew and the array may sit at another address.  Once the
// module is loaded on a device the lookup is cheap; the first one on a device
// may load the module, which is why that first call must precede any capture.
rq_status_t scratch_for_current_device(uint32_t** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return RQ_ERROR_NO_DEVICE;
  }
  void* p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_sort_scratch);
  if (e != cudaSuccess || !p) {
    cudaGetLastError();
    return RQ_ERROR_CUDA;
  }
  *out = static_cast<uint32_t*>(p);
  return RQ_SUCCESS;
}

}  // namespace
}  // namespace rq

extern "C" rq_status_t rq_sort_pairs_noalloc(uint32_t* keys, uint32_t* values, uint32_t n,
                                             uint32_t key_bits, void* cuda_stream) {
  using namespace rq;
  if (n == 0) return RQ_SUCCESS;
  if (!keys || !values) return RQ_ERROR_INVALID_ARGUMENT;
  if (key_bits == 0 || key_bits > 32) return RQ_ERROR_INVALID_ARGUMENT;
  if (n > kMaxPairs) return RQ_ERROR_INVALID_ARGUMENT;  // beyond the fixed working memory
  uint32_t* base = nullptr;
  rq_status_t st = scratch_for_current_device(&base);
  if (st != RQ_SUCCESS) return st;
  if (n == 1) return RQ_SUCCESS;
  cudaStream_t s = static_cast<cudaStream_t>(cuda_stream);
  if (s) {  // the array's address is the current device's: the stream must belong to it
    int cur = 0, sdev = 0;
    if (cudaGetDevice(&cur) != cudaSuccess || cudaStreamGetDevice(s, &sdev) != cudaSuccess) {
      cudaGetLastError();
      return RQ_ERROR_INVALID_ARGUMENT;
    }
    if (sdev != cur) return RQ_ERROR_INVALID_ARGUMENT;
  }
  const int passes = (int)((key_bits + 7) / 8);
  const size_t status_words = sort_status_words(n, passes);
  if (status_words > kStatusWords) return RQ_ERROR_UNSUPPORTED;  // tile size mismatch
  // Histograms, tile counters, the look-back words of this sort's passes
  // (contiguous from kStatusOff) and the error word must start at zero; the
  // array keeps whatever the previous call left there.
  if (cudaMemsetAsync(base + kHistOff, 0, (kStatusOff - kHistOff + status_words) * sizeof(uint32_t), s) !=
          cudaSuccess ||
      cudaMemsetAsync(base + kErrOff, 0, sizeof(uint32_t), s) != cudaSuccess) {
    cudaGetLastError();
    return RQ_ERROR_CUDA;
  }
  uint32_t* err = base + kErrOff;
  launch_histogram(keys, n, passes, base + kHistOff, s);
  SortScratch sc{base, base + kMaxPairs, base + kHistOff, base + kStatusOff, base + kCounterOff};
  launch_onesweep(keys, values, n, passes, sc, err, s);
  if (cudaGetLastError() != cudaSuccess) return RQ_ERROR_CUDA;
  uint32_t flags = 0;
  if (cudaMemcpyAsync(&flags, err, sizeof(flags), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess) {
    cudaGetLastError();
    return RQ_ERROR_CUDA;
  }
  return flags & kErrTimeout ? RQ_ERROR_TIMEOUT : RQ_SUCCESS;
}
