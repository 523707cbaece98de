// Exclusive prefix sum of 32-bit counts (reduce, scan of block totals, add).
// Used by the level-by-level builders for stable partitions and for
// numbering nodes.
#include "rq_device.cuh"
#include "rq_internal.hpp"

namespace rq {
namespace {

constexpr int kThreads = 256;
constexpr int kItems = 16;
constexpr uint32_t kBlock = kThreads * kItems;  // 4096 elements per block

__device__ __forceinline__ uint32_t block_scan_excl(uint32_t v, uint32_t* s_warp, uint32_t& total) {
  int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) s_warp[warp] = x;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = lane < kThreads / 32 ? s_warp[lane] : 0u;
#pragma unroll
    for (int o = 1; o < kThreads / 32; o <<= 1) {
      uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    if (lane < kThreads / 32) s_warp[lane] = w;
  }
  __syncthreads();
  total = s_warp[kThreads / 32 - 1];
  uint32_t r = (warp > 0 ? s_warp[warp - 1] : 0u) + x - v;
  __syncthreads();
  return r;
}

// Each thread owns kItems consecutive elements.
__global__ void __launch_bounds__(kThreads) k_scan_local(const uint32_t* __restrict__ in, uint32_t* __restrict__ out,
                                                         uint64_t n, uint32_t* __restrict__ block_tot) {
  __shared__ uint32_t s_warp[kThreads / 32];
  const uint64_t base = (uint64_t)blockIdx.x * kBlock + (uint64_t)threadIdx.x * kItems;
  uint32_t v[kItems];
  uint32_t sum = 0;
#pragma unroll
  for (int k = 0; k < kItems; ++k) {
    uint64_t i = base + k;
    v[k] = i < n ? in[i] : 0u;
    sum += v[k];
  }
  uint32_t total;
  uint32_t run = block_scan_excl(sum, s_warp, total);
#pragma unroll
  for (int k = 0; k < kItems; ++k) {
    uint64_t i = base + k;
    if (i < n) out[i] = run;
    run += v[k];
  }
  if (threadIdx.x == 0) block_tot[blockIdx.x] = total;
}

// One block scans up to kBlock block totals in place; writes the grand total.
__global__ void __launch_bounds__(kThreads) k_scan_totals(uint32_t* tot, uint32_t nb, uint32_t* grand) {
  __shared__ uint32_t s_warp[kThreads / 32];
  uint32_t carry = 0;
  for (uint32_t base = 0; base < nb; base += kBlock) {
    uint32_t v[kItems];
    uint32_t sum = 0;
    const uint32_t b0 = base + threadIdx.x * kItems;
#pragma unroll
    for (int k = 0; k < kItems; ++k) {
      v[k] = b0 + k < nb ? tot[b0 + k] : 0u;
      sum += v[k];
    }
    uint32_t total;
    uint32_t run = block_scan_excl(sum, s_warp, total) + carry;
#pragma unroll
    for (int k = 0; k < kItems; ++k) {
      if (b0 + k < nb) tot[b0 + k] = run;
      run += v[k];
    }
    carry += total;
  }
  if (threadIdx.x == 0 && grand) *grand = carry;
}

__global__ void __launch_bounds__(kThreads) k_scan_add(uint32_t* __restrict__ out, uint64_t n,
                                                       const uint32_t* __restrict__ tot) {
  const uint32_t add = tot[blockIdx.x];
  if (add == 0) return;
  const uint64_t base = (uint64_t)blockIdx.x * kBlock;
  for (uint32_t k = threadIdx.x; k < kBlock; k += kThreads) {
    uint64_t i = base + k;
    if (i < n) out[i] += add;
  }
}

}  // namespace

size_t scan_tmp_words(uint64_t n) { return (n + kBlock - 1) / kBlock + 1; }

void launch_scan_excl(const uint32_t* in, uint32_t* out, uint64_t n, uint32_t* tmp, uint32_t* total,
                      cudaStream_t s) {
  if (n == 0) return;
  const uint32_t nb = (uint32_t)((n + kBlock - 1) / kBlock);
  count_launch(nb > 1 ? 3 : 2);
  k_scan_local<<<nb, kThreads, 0, s>>>(in, out, n, tmp);
  k_scan_totals<<<1, kThreads, 0, s>>>(tmp, nb, total);
  if (nb > 1) k_scan_add<<<nb, kThreads, 0, s>>>(out, n, tmp);
}

}  // namespace rq
