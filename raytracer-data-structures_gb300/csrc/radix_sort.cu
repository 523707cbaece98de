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
constexpr uint32_t kFlagAgg = 1u << 30;
constexpr uint32_t kFlagPrefix = 2u << 30;
constexpr uint32_t kFlagAbort = 3u << 30;
constexpr uint32_t kValueMask = (1u << 30) - 1;
constexpr uint32_t kSpinLimit = 1u << 20;  // polls of one predecessor word before giving up
constexpr uint32_t kStallSpin = 256;       // polls of the test hook's never-set word

template <typename K>
__global__ void __launch_bounds__(kThreads) k_histogram(const K* __restrict__ keys, uint32_t n,
                                                        int passes, uint32_t* __restrict__ hist) {
  __shared__ uint32_t sh[sizeof(K)][256];
  for (int i = threadIdx.x; i < (int)sizeof(K) * 256; i += blockDim.x) (&sh[0][0])[i] = 0;
  __syncthreads();
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    K k = __ldg(keys + i);
    for (int p = 0; p < passes; ++p) atomicAdd(&sh[p][(uint32_t)(k >> (8 * p)) & 255u], 1u);
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

template <typename K, int kItems>
struct __align__(16) OnesweepSmem {
  static constexpr int kTile = kThreads * kItems;
  K keys[kTile];
  uint32_t warp_hist[kWarps][256];
  uint32_t digit_start[256];
  uint32_t global_base[256];
  uint32_t scan_tmp[kWarps];
  uint32_t vals[kTile];
  uint32_t tile;
  int abort;
};

template <typename K, int kItems>
__global__ void __launch_bounds__(kThreads) k_onesweep(const K* __restrict__ kin,
                                                       const uint32_t* __restrict__ vin,
                                                       K* __restrict__ kout,
                                                       uint32_t* __restrict__ vout, uint32_t n,
                                                       int shift, const uint32_t* __restrict__ hist,
                                                       uint32_t* status, uint32_t* tile_counter,
                                                       uint32_t* err, const uint32_t* stall) {
  constexpr int kTile = kThreads * kItems;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  OnesweepSmem<K, kItems>& sm = *reinterpret_cast<OnesweepSmem<K, kItems>*>(smem_raw);
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
  K keys[kItems];
  uint32_t vals[kItems], rank[kItems];
#pragma unroll
  for (int k = 0; k < kItems; ++k) {
    uint64_t i = base + (uint64_t)warp * (32 * kItems) + (uint64_t)k * 32 + lane;
    bool ok = i < n;
    keys[k] = ok ? __ldg(kin + i) : K(0);
    vals[k] = ok ? __ldg(vin + i) : 0u;
  }

  // Stable rank within the warp, item by item.
#pragma unroll
  for (int k = 0; k < kItems; ++k) {
    uint64_t i = base + (uint64_t)warp * (32 * kItems) + (uint64_t)k * 32 + lane;
    bool ok = i < n;
    uint32_t d = ok ? ((uint32_t)(keys[k] >> shift) & 255u) : 256u;
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
    // Test hook (stall != null): tile 1 first waits on a word that nothing
    // sets, so its bounded wait gives up as a lost predecessor's would.
    if (stall && tile == 1)
      failed = !spin_until([&] { return *reinterpret_cast<const volatile uint32_t*>(stall) != 0u; }, kStallSpin);
    for (int64_t j = (int64_t)tile - 1; j >= 0 && !failed; --j) {
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
      uint32_t d = (uint32_t)(keys[k] >> shift) & 255u;
      uint32_t pos = sm.digit_start[d] + sm.warp_hist[warp][d] + rank[k];
      sm.keys[pos] = keys[k];
      sm.vals[pos] = vals[k];
    }
  }
  __syncthreads();
  if (sm.abort) return;

  const uint32_t valid = (uint64_t)n - base < (uint64_t)kTile ? (uint32_t)(n - base) : (uint32_t)kTile;
  for (uint32_t i = tid; i < valid; i += kThreads) {
    K key = sm.keys[i];
    uint32_t d = (uint32_t)(key >> shift) & 255u;
    uint32_t gpos = sm.global_base[d] + (i - sm.digit_start[d]);
    if (gpos < n) {
      kout[gpos] = key;
      vout[gpos] = sm.vals[i];
    }
  }
}

constexpr int kItems32 = 15;  // 3,840 keys per tile
constexpr int kItems64 = 10;  // 2,560 keys per tile (64-bit keys)

// Sorted pairs land back in keys / vals, unless vals_out is given: then the
// final pass's buffers are left as they are and *vals_out names the one that
// holds the sorted values (keys end in the matching key buffer).
template <typename K, int ITEMS>
void onesweep_passes(K* keys, uint32_t* vals, uint32_t n, int passes, K* keys_alt, uint32_t* vals_alt,
                     const uint32_t* hist, uint32_t* status, uint32_t* counters, uint32_t* err, cudaStream_t s,
                     uint32_t** vals_out = nullptr, const uint32_t* stall = nullptr) {
  using Smem = OnesweepSmem<K, ITEMS>;
  static_assert(sizeof(Smem) <= 48 * 1024, "onesweep shared memory over the default limit");
  const uint32_t tile = kThreads * ITEMS;
  const uint32_t tiles = (n + tile - 1) / tile;
  K* src_k = keys;
  uint32_t* src_v = vals;
  K* dst_k = keys_alt;
  uint32_t* dst_v = vals_alt;
  for (int p = 0; p < passes; ++p) {
    count_launch();
    k_onesweep<K, ITEMS><<<tiles, kThreads, sizeof(Smem), s>>>(src_k, src_v, dst_k, dst_v, n, 8 * p,
                                                               hist + 256 * p, status + (size_t)p * tiles * 256,
                                                               counters + p, err, p == 0 ? stall : nullptr);
    K* tk = src_k; src_k = dst_k; dst_k = tk;
    uint32_t* tv = src_v; src_v = dst_v; dst_v = tv;
  }
  if (vals_out) {
    *vals_out = src_v;
    return;
  }
  if (src_k != keys) {
    cudaMemcpyAsync(keys, src_k, (size_t)n * sizeof(K), cudaMemcpyDeviceToDevice, s);
    cudaMemcpyAsync(vals, src_v, (size_t)n * 4, cudaMemcpyDeviceToDevice, s);
  }
}

template <typename K>
void histogram(const K* keys, uint32_t n, int passes, uint32_t* hist, cudaStream_t s) {
  if (n == 0) return;
  uint32_t g = (n + kThreads * 8 - 1) / (kThreads * 8);
  if (g > 2048) g = 2048;
  count_launch();
  k_histogram<K><<<g, kThreads, 0, s>>>(keys, n, passes, hist);
}

}  // namespace

uint32_t sort_tiles(uint32_t n) { return (n + kThreads * kItems32 - 1) / (kThreads * kItems32); }

size_t sort_status_words(uint32_t n, int passes) {
  return (size_t)passes * sort_tiles(n) * 256;
}

void launch_histogram(const uint32_t* keys, uint32_t n, int passes, uint32_t* hist, cudaStream_t s) {
  histogram<uint32_t>(keys, n, passes, hist, s);
}

void launch_onesweep(uint32_t* keys, uint32_t* vals, uint32_t n, int passes, const SortScratch& sc,
                     uint32_t* err, cudaStream_t s) {
  if (n <= 1) return;
  onesweep_passes<uint32_t, kItems32>(keys, vals, n, passes, sc.keys_alt, sc.vals_alt, sc.hist, sc.status,
                                      sc.counters, err, s, nullptr, sc.stall);
}

uint32_t* launch_onesweep_vals(uint32_t* keys, uint32_t* vals, uint32_t n, int passes, const SortScratch& sc,
                               uint32_t* err, cudaStream_t s) {
  if (n <= 1) return vals;
  uint32_t* out = vals;
  onesweep_passes<uint32_t, kItems32>(keys, vals, n, passes, sc.keys_alt, sc.vals_alt, sc.hist, sc.status,
                                      sc.counters, err, s, &out, sc.stall);
  return out;
}

size_t sort_status_words64(uint32_t n, int passes) {
  return (size_t)passes * ((n + kThreads * kItems64 - 1) / (kThreads * kItems64)) * 256;
}

void launch_histogram64(const uint64_t* keys, uint32_t n, int passes, uint32_t* hist, cudaStream_t s) {
  histogram<uint64_t>(keys, n, passes, hist, s);
}

void launch_onesweep64(uint64_t* keys, uint32_t* vals, uint32_t n, int passes, uint64_t* keys_alt,
                       uint32_t* vals_alt, const uint32_t* hist, uint32_t* status, uint32_t* counters,
                       uint32_t* err, cudaStream_t s) {
  if (n <= 1) return;
  onesweep_passes<uint64_t, kItems64>(keys, vals, n, passes, keys_alt, vals_alt, hist, status, counters, err, s);
}

}  // namespace rq
