// Stable LSD radix sort of (key, value) pairs, 8-bit digits, one kernel per
// digit pass ("onesweep": local ranking + decoupled look-back across tiles).
// Replaces radixSort (accelerators.h:348-369), which sorts a by-value copy and
// so has no effect: the order produced here is the stable order by key, ties
// in input order, which is what that LSD routine computes.
//
// Per pass and tile of 3,840 keys: keys are ranked stably inside each warp
// with __match_any_sync, warp counts are prefixed per digit, the tile's digit
// counts are published for later tiles, and each digit's global offset is
// found by walking back over earlier tiles (bounded wait; a wait that gives
// up marks the tile as failed and later tiles abort instead of waiting).
// Keys are staged in shared memory in digit order so the global writes are
// contiguous runs.
#include "rq_device.cuh"
#include "rq_internal.hpp"

namespace rq {
namespace {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kItems = 15;
constexpr int kTile = kThreads * kItems;  // 3840
constexpr uint32_t kFlagAgg = 1u << 30;
constexpr uint32_t kFlagPrefix = 2u << 30;
constexpr uint32_t kFlagAbort = 3u << 30;
constexpr uint32_t kValueMask = (1u << 30) - 1;
constexpr uint32_t kSpinLimit = 1u << 20;  // polls of one predecessor word before giving up

__global__ void __launch_bounds__(kThreads) k_histogram(const uint32_t* __restrict__ keys, uint32_t n,
                                                        int passes, uint32_t* __restrict__ hist) {
  __shared__ uint32_t sh[4][256];
  for (int i = threadIdx.x; i < 1024; i += blockDim.x) (&sh[0][0])[i] = 0;
  __syncthreads();
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    uint32_t k = __ldg(keys + i);
    for (int p = 0; p < passes; ++p) atomicAdd(&sh[p][(k >> (8 * p)) & 255u], 1u);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < passes * 256; i += blockDim.x) {
    uint32_t v = (&sh[0][0])[i];
    if (v) atomicAdd(&hist[i], v);
  }
}

// Exclusive scan of one value per thread over the 256-thread block.
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* s_warp) {
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
    uint32_t w = lane < kWarps ? s_warp[lane] : 0u;
#pragma unroll
    for (int o = 1; o < kWarps; o <<= 1) {
      uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    if (lane < kWarps) s_warp[lane] = w;
  }
  __syncthreads();
  uint32_t prefix = warp > 0 ? s_warp[warp - 1] : 0u;
  uint32_t r = prefix + x - v;
  __syncthreads();  // s_warp reusable after return
  return r;
}

struct __align__(16) OnesweepSmem {
  uint32_t warp_hist[kWarps][256];
  uint32_t digit_start[256];
  uint32_t global_base[256];
  uint32_t scan_tmp[kWarps];
  uint32_t keys[kTile];
  uint32_t vals[kTile];
  uint32_t tile;
  int abort;
};

__global__ void __launch_bounds__(kThreads) k_onesweep(const uint32_t* __restrict__ kin,
                                                       const uint32_t* __restrict__ vin,
                                                       uint32_t* __restrict__ kout,
                                                       uint32_t* __restrict__ vout, uint32_t n,
                                                       int shift, const uint32_t* __restrict__ hist,
                                                       uint32_t* status, uint32_t* tile_counter,
                                                       uint32_t* err) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  OnesweepSmem& sm = *reinterpret_cast<OnesweepSmem*>(smem_raw);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

  if (tid == 0) {
    sm.tile = atomicAdd(tile_counter, 1u);
    sm.abort = 0;
  }
  for (int i = tid; i < kWarps * 256; i += kThreads) (&sm.warp_hist[0][0])[i] = 0;
  __syncthreads();
  const uint32_t tile = sm.tile;
  const uint64_t base = (uint64_t)tile * kTile;

  // Warp-striped load: element order (warp, item, lane) = input order.
  uint32_t keys[kItems], vals[kItems], rank[kItems];
#pragma unroll
  for (int k = 0; k < kItems; ++k) {
    uint64_t i = base + (uint64_t)warp * (32 * kItems) + (uint64_t)k * 32 + lane;
    bool ok = i < n;
    keys[k] = ok ? __ldg(kin + i) : 0u;
    vals[k] = ok ? __ldg(vin + i) : 0u;
  }

  // Stable rank within the warp, item by item.
#pragma unroll
  for (int k = 0; k < kItems; ++k) {
    uint64_t i = base + (uint64_t)warp * (32 * kItems) + (uint64_t)k * 32 + lane;
    bool ok = i < n;
    uint32_t d = ok ? ((keys[k] >> shift) & 255u) : 256u;
    uint32_t peers = __match_any_sync(0xffffffffu, d);
    int leader = __ffs(peers) - 1;
    uint32_t below = __popc(peers & ((1u << lane) - 1u));
    uint32_t b = 0;
    if (lane == leader && ok) {
      b = sm.warp_hist[warp][d];
      sm.warp_hist[warp][d] = b + __popc(peers);
    }
    b = __shfl_sync(0xffffffffu, b, leader);
    rank[k] = b + below;
    __syncwarp();
  }
  __syncthreads();

  // Digit t: prefix over warps, tile count.
  const uint32_t t = tid;
  uint32_t count = 0;
#pragma unroll
  for (int w = 0; w < kWarps; ++w) {
    uint32_t c = sm.warp_hist[w][t];
    sm.warp_hist[w][t] = count;
    count += c;
  }
  // Publish this tile's count early so later tiles can proceed.
  volatile uint32_t* st = status;
  if (tile == 0) st[t] = kFlagPrefix | count;
  else st[(size_t)tile * 256 + t] = kFlagAgg | count;

  uint32_t gscan = block_exclusive_scan(__ldg(hist + t), sm.scan_tmp);
  sm.digit_start[t] = block_exclusive_scan(count, sm.scan_tmp);

  // Decoupled look-back for digit t.
  uint32_t excl = 0;
  bool failed = false;
  if (tile > 0) {
    for (int64_t j = (int64_t)tile - 1; j >= 0; --j) {
      uint32_t s = 0;
      bool ok = spin_until([&] { s = st[(size_t)j * 256 + t]; return (s & ~kValueMask) != 0; },
                           kSpinLimit);
      if (!ok || (s & ~kValueMask) == kFlagAbort) {
        failed = true;
        break;
      }
      excl += s & kValueMask;
      if ((s & ~kValueMask) == kFlagPrefix) break;
    }
    if (failed) {
      st[(size_t)tile * 256 + t] = kFlagAbort;
      sm.abort = 1;
      atomicOr(err, kErrTimeout);
    } else {
      st[(size_t)tile * 256 + t] = kFlagPrefix | ((excl + count) & kValueMask);
    }
  }
  sm.global_base[t] = gscan + excl;
  __syncthreads();

  // Scatter into shared memory in digit order.
#pragma unroll
  for (int k = 0; k < kItems; ++k) {
    uint64_t i = base + (uint64_t)warp * (32 * kItems) + (uint64_t)k * 32 + lane;
    if (i < n) {
      uint32_t d = (keys[k] >> shift) & 255u;
      uint32_t pos = sm.digit_start[d] + sm.warp_hist[warp][d] + rank[k];
      sm.keys[pos] = keys[k];
      sm.vals[pos] = vals[k];
    }
  }
  __syncthreads();
  if (sm.abort) return;

  const uint32_t valid = (uint64_t)n - base < (uint64_t)kTile ? (uint32_t)(n - base) : (uint32_t)kTile;
  for (uint32_t i = tid; i < valid; i += kThreads) {
    uint32_t key = sm.keys[i];
    uint32_t d = (key >> shift) & 255u;
    uint32_t gpos = sm.global_base[d] + (i - sm.digit_start[d]);
    if (gpos < n) {
      kout[gpos] = key;
      vout[gpos] = sm.vals[i];
    }
  }
}

}  // namespace

uint32_t sort_tiles(uint32_t n) { return (n + kTile - 1) / kTile; }

size_t sort_status_words(uint32_t n, int passes) {
  return (size_t)passes * sort_tiles(n) * 256;
}

void launch_histogram(const uint32_t* keys, uint32_t n, int passes, uint32_t* hist, cudaStream_t s) {
  if (n == 0) return;
  uint32_t g = (n + kThreads * 8 - 1) / (kThreads * 8);
  if (g > 2048) g = 2048;
  count_launch();
  k_histogram<<<g, kThreads, 0, s>>>(keys, n, passes, hist);
}

void launch_onesweep(uint32_t* keys, uint32_t* vals, uint32_t n, int passes, const SortScratch& sc,
                     uint32_t* err, cudaStream_t s) {
  if (n <= 1) return;
  const size_t smem = sizeof(OnesweepSmem);  // ~40 KB: below the 48 KB default limit
  static_assert(sizeof(OnesweepSmem) <= 48 * 1024, "onesweep shared memory over the default limit");
  const uint32_t tiles = sort_tiles(n);
  uint32_t* src_k = keys;
  uint32_t* src_v = vals;
  uint32_t* dst_k = sc.keys_alt;
  uint32_t* dst_v = sc.vals_alt;
  for (int p = 0; p < passes; ++p) {
    count_launch();
    k_onesweep<<<tiles, kThreads, smem, s>>>(src_k, src_v, dst_k, dst_v, n, 8 * p, sc.hist + 256 * p,
                                             sc.status + (size_t)p * tiles * 256, sc.counters + p, err);
    uint32_t* tk = src_k; src_k = dst_k; dst_k = tk;
    uint32_t* tv = src_v; src_v = dst_v; dst_v = tv;
  }
  if (src_k != keys) {
    cudaMemcpyAsync(keys, src_k, (size_t)n * 4, cudaMemcpyDeviceToDevice, s);
    cudaMemcpyAsync(vals, src_v, (size_t)n * 4, cudaMemcpyDeviceToDevice, s);
  }
}

}  // namespace rq
