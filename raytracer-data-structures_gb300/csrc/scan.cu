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

// Up to two arrays scanned side by side (same length): one set of launches
// for both, and twice the loads in flight.
template <int NA>
struct ScanArgs {
  const uint32_t* in[NA];
  uint32_t* out[NA];
  uint32_t* tot[NA];    // per-block totals, then their exclusive scan
  uint32_t* grand[NA];  // optional grand totals
};

// Each thread owns kItems consecutive elements.
template <int NA>
__global__ void __launch_bounds__(kThreads) k_scan_local(ScanArgs<NA> A, uint64_t n) {
  __shared__ uint32_t s_warp[kThreads / 32];
  const uint64_t base = (uint64_t)blockIdx.x * kBlock + (uint64_t)threadIdx.x * kItems;
  uint32_t v[NA][kItems];
  uint32_t sum[NA];
#pragma unroll
  for (int q = 0; q < NA; ++q) {
    sum[q] = 0;
#pragma unroll
    for (int k = 0; k < kItems; ++k) {
      const uint64_t i = base + k;
      v[q][k] = i < n ? A.in[q][i] : 0u;
      sum[q] += v[q][k];
    }
  }
#pragma unroll
  for (int q = 0; q < NA; ++q) {
    uint32_t total;
    uint32_t run = block_scan_excl(sum[q], s_warp, total);
#pragma unroll
    for (int k = 0; k < kItems; ++k) {
      const uint64_t i = base + k;
      if (i < n) A.out[q][i] = run;
      run += v[q][k];
    }
    if (threadIdx.x == 0) {
      A.tot[q][blockIdx.x] = total;
      if (gridDim.x == 1 && A.grand[q]) *A.grand[q] = total;  // one block: no totals pass
    }
  }
}

// One block scans up to kBlock block totals in place per array; writes the
// grand totals.
template <int NA>
__global__ void __launch_bounds__(kThreads) k_scan_totals(ScanArgs<NA> A, uint32_t nb) {
  __shared__ uint32_t s_warp[kThreads / 32];
  for (int q = 0; q < NA; ++q) {
    uint32_t* tot = A.tot[q];
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
    if (threadIdx.x == 0 && A.grand[q]) *A.grand[q] = carry;
  }
}

template <int NA>
__global__ void __launch_bounds__(kThreads) k_scan_add(ScanArgs<NA> A, uint64_t n) {
  const uint64_t base = (uint64_t)blockIdx.x * kBlock;
#pragma unroll
  for (int q = 0; q < NA; ++q) {
    const uint32_t add = A.tot[q][blockIdx.x];
    if (add == 0) continue;
    for (uint32_t k = threadIdx.x; k < kBlock; k += kThreads) {
      const uint64_t i = base + k;
      if (i < n) A.out[q][i] += add;
    }
  }
}

template <int NA>
void scan_launch(const ScanArgs<NA>& A, uint64_t n, cudaStream_t s) {
  const uint32_t nb = (uint32_t)((n + kBlock - 1) / kBlock);
  count_launch(nb > 1 ? 3 : 1);
  k_scan_local<NA><<<nb, kThreads, 0, s>>>(A, n);
  if (nb > 1) {
    k_scan_totals<NA><<<1, kThreads, 0, s>>>(A, nb);
    k_scan_add<NA><<<nb, kThreads, 0, s>>>(A, n);
  }
}

}  // namespace

size_t scan_tmp_words(uint64_t n) { return (n + kBlock - 1) / kBlock + 1; }

void launch_scan_excl(const uint32_t* in, uint32_t* out, uint64_t n, uint32_t* tmp, uint32_t* total,
                      cudaStream_t s) {
  if (n == 0) return;
  ScanArgs<1> A{{in}, {out}, {tmp}, {total}};
  scan_launch(A, n, s);
}

void launch_scan2_excl(const uint32_t* in0, uint32_t* out0, const uint32_t* in1, uint32_t* out1, uint64_t n,
                       uint32_t* tmp, uint32_t* total0, uint32_t* total1, cudaStream_t s) {
  if (n == 0) return;
  ScanArgs<2> A{{in0, in1}, {out0, out1}, {tmp, tmp + scan_tmp_words(n)}, {total0, total1}};
  scan_launch(A, n, s);
}

}  // namespace rq
