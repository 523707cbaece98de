// Ray traversal of BVH2 structures (LBVH and median BVH) and the brute-force
// NONE path.
//
// FAST (the engine's semantics): near child first, far child pushed on a
// per-thread stack of 64 entries, child boxes clipped to [tmin, closest hit]
// with a rounding-safe far bound, primitives accepted in (tmin, closest).
// Replaces boxIntersect + castRay's candidate loop (accelerators.h:668-690,
// main.cpp:330-358) with a pruned closest-hit walk.
//
// REFERENCE: the reference's own semantics, reproduced exactly: the root box
// and each child box pass the division slab test of accelerators.h:588-626
// with no clipping, candidates are visited in boxIntersect's pre-order (left
// subtree before right) and castRay's strict-< selection keeps the first
// closest.
//
// Any-hit queries stop at the first accepted primitive and write one bit per
// ray (warp ballot).
#include <algorithm>

#include "trace_device.cuh"

namespace rq {
namespace {

constexpr int kThreads = 128;

// perm (may be null): thread i traces ray perm[i] and writes that ray's result
// (a reordering for coherence that leaves every result where the caller
// expects it).  With perm, any-hit bits are set with atomicOr on a zeroed array.
// Both box-test forms are inlined and each ray takes the one it needs
// (rq_device.cuh); the counting walk, the small-stack test hook and callers
// without an exact-ray list use this kernel, FAST queries k_trace_warps.
// At most 48 registers (10 blocks of 128 per SM): measured 3-4% faster on
// the closest-hit triangle walk than the unconstrained 52.
template <int KIND, bool ANY, bool COUNT = false, int STACK = kStackSize>
__global__ void __launch_bounds__(kThreads, 10) k_trace_fast(Bvh2View bvh, const float4* __restrict__ rays,
                                                         uint32_t n, float4* __restrict__ hits,
                                                         uint32_t* __restrict__ occ, uint32_t* err,
                                                         unsigned long long* counters = nullptr,
                                                         const uint32_t* __restrict__ perm = nullptr) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t r = (perm && i < n) ? __ldg(perm + i) : i;
  bool occluded = false;
  uint32_t visits = 0, tests = 0;
  if (i < n) {
    Ray ray = load_ray(rays, r);
    Closest c = {ray.tmax, kMiss, 0.f, 0.f};
    occluded = walk_bvh2<KIND, ANY, COUNT, STACK>(bvh, ray, c, visits, tests, err);
    if (!ANY) hits[r] = make_float4(c.t, __uint_as_float(c.prim), c.u, c.v);
  }
  if (ANY) {
    if (perm) {
      if (occluded) atomicOr(occ + (r >> 5), 1u << (r & 31));
    } else {
      uint32_t bits = __ballot_sync(0xffffffffu, occluded);
      uint32_t w0 = (blockIdx.x * blockDim.x + (threadIdx.x & ~31u));
      if ((threadIdx.x & 31) == 0 && w0 < n) occ[w0 >> 5] = bits;
    }
  }
  if (COUNT) add_counts(counters, visits, tests);
}

// The FAST walk as persistent warps: a grid that fits on the GPU at once,
// each warp taking the next 32 rays from a counter (list[1]) until none are
// left, so no warp idles while the slowest warp of its block finishes.
// Secondary rays of the 998k-triangle terrain: 3.52 ms against 3.72 ms for
// one thread per ray in blocks of 128 (blocks of 64: 3.66 ms).  Rays that
// need the exact box test (a direction component zero or too small for the
// fused form) are not walked here but appended to list[2..] (count in
// list[0]) for k_trace_exact, so this kernel carries only the fused walk.
// UNIT: the LBVH's one-primitive leaves (4-byte stack entries).
template <int KIND, bool ANY, bool UNIT>
__global__ void __launch_bounds__(kThreads, 10) k_trace_warps(Bvh2View bvh, const float4* __restrict__ rays,
                                                          uint32_t n, float4* __restrict__ hits,
                                                          uint32_t* __restrict__ occ, uint32_t* err,
                                                          const uint32_t* __restrict__ perm,
                                                          uint32_t* __restrict__ list) {
  const uint32_t lane = threadIdx.x & 31;
  for (;;) {
    uint32_t base = 0;
    if (lane == 0) base = atomicAdd(list + 1, 32u);
    base = __shfl_sync(0xffffffffu, base, 0);
    if (base >= n) break;
    const uint32_t i = base + lane;
    const uint32_t r = (perm && i < n) ? __ldg(perm + i) : i;
    bool occluded = false;
    uint32_t visits = 0, tests = 0;
    if (i < n) {
      Ray ray = load_ray(rays, r);
      Closest c = {ray.tmax, kMiss, 0.f, 0.f};
      const SlabRay sr = slab_ray(ray.o, ray.d);
      if (zero_dir(sr)) {
        list[2 + atomicAdd(list, 1u)] = r;
      } else {
        occluded = walk_bvh2_form<KIND, ANY, false, kStackSize, false, UNIT>(bvh, ray, sr, c, visits, tests, err);
        if (!ANY) store_hit(hits, r, c);
      }
    }
    if (ANY) {
      if (perm) {
        if (occluded) atomicOr(occ + (r >> 5), 1u << (r & 31));
      } else {
        const uint32_t bits = __ballot_sync(0xffffffffu, occluded);
        if (lane == 0) occ[base >> 5] = bits;
      }
    }
  }
}

// The rays k_trace_warps set aside, walked with the exact box test; a
// fixed grid strides over the list (empty in most queries).  Any-hit bits
// are set with atomicOr over the words k_trace_warps stored before.
constexpr uint32_t kExactBlocks = 304;
template <int KIND, bool ANY>
__global__ void __launch_bounds__(kThreads) k_trace_exact(Bvh2View bvh, const float4* __restrict__ rays,
                                                          const uint32_t* __restrict__ list,
                                                          float4* __restrict__ hits, uint32_t* __restrict__ occ,
                                                          uint32_t* err) {
  const uint32_t count = list[0];
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < count; k += gridDim.x * blockDim.x) {
    const uint32_t r = list[2 + k];
    const Ray ray = load_ray(rays, r);
    Closest c = {ray.tmax, kMiss, 0.f, 0.f};
    uint32_t visits = 0, tests = 0;
    const bool occluded =
        walk_bvh2_form<KIND, ANY, false, kStackSize, true>(bvh, ray, slab_ray(ray.o, ray.d), c, visits, tests, err);
    if (!ANY) hits[r] = make_float4(c.t, __uint_as_float(c.prim), c.u, c.v);
    if (ANY && occluded) atomicOr(occ + (r >> 5), 1u << (r & 31));
  }
}

// Blocks of `k` (kThreads each) resident on the current device at once.
template <typename K>
uint32_t resident_blocks(K k) {
  int per_sm = 0, dev = 0, sms = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, kThreads, 0) != cudaSuccess || per_sm < 1) per_sm = 1;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      sms < 1)
    sms = 1;
  return (uint32_t)(per_sm * sms);
}

// ------------------------------------------------ top levels in shared memory
// RQ_SCHEDULING_SHARED_TOP: the top kTopLevels levels of the binary tree
// (at most 63 nodes, 4 KB), copied breadth first into one small array whose
// internal links inside the copy are renumbered kTopBit | position; every
// block stages that array in shared memory and walks it from there, then
// continues in global memory below it.  Same walk, same results.
constexpr int kTopLevels = 6;
constexpr int kTopNodes = (1 << kTopLevels) - 1;
constexpr int kTopBit = 0x40000000;  // node links are below 2^30

// One warp: breadth-first list of the top levels, then the renumbered copies.
__global__ void __launch_bounds__(32) k_top_copy(const float4* __restrict__ nodes, uint32_t n_internal,
                                                 float4* __restrict__ top) {
  __shared__ int32_t q[kTopNodes];
  const uint32_t lane = threadIdx.x;
  int lo = 0, hi = n_internal ? 1 : 0;
  if (lane == 0) q[0] = 0;
  __syncwarp();
  for (int level = 0; level + 1 < kTopLevels && lo < hi; ++level) {
    const int j = lo + (int)lane;  // a level holds at most 32 nodes
    int4 l = make_int4(-1, -1, 0, 0);
    if (j < hi) l = __ldg(reinterpret_cast<const int4*>(nodes + 4 * (size_t)q[j] + 3));
    const uint32_t c = (l.x >= 0 ? 1u : 0u) + (l.y >= 0 ? 1u : 0u);
    uint32_t incl = c;
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
      if ((int)lane >= o) incl += y;
    }
    const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
    const int at = hi + (int)(incl - c);
    if (l.x >= 0) q[at] = l.x;
    if (l.y >= 0) q[at + (l.x >= 0 ? 1 : 0)] = l.y;
    __syncwarp();
    lo = hi;
    hi += (int)total;
  }
  for (int k = (int)lane; k < hi; k += 32) {
    const float4* nd = nodes + 4 * (size_t)q[k];
    int4 l = __ldg(reinterpret_cast<const int4*>(nd + 3));
    for (int m = 0; m < hi; ++m) {  // children that are in the copy
      if (l.x >= 0 && q[m] == l.x) l.x = kTopBit | m;
      if (l.y >= 0 && q[m] == l.y) l.y = kTopBit | m;
    }
    top[4 * k] = __ldg(nd);
    top[4 * k + 1] = __ldg(nd + 1);
    top[4 * k + 2] = __ldg(nd + 2);
    reinterpret_cast<int4*>(top)[4 * k + 3] = l;
  }
}

template <int KIND, bool ANY>
__device__ __forceinline__ bool walk_bvh2_top(const Bvh2View& bvh, const float4* s_top, const Ray& ray, Closest& c,
                                              uint32_t* err) {
  const SlabRay sr = slab_ray(ray.o, ray.d);
  float tn;
  const float* rb = bvh.root;
  if (!slab_box<false>(sr, ray.o, rb[0], rb[3], rb[1], rb[4], rb[2], rb[5], ray.tmin, ray.tmax, tn)) return false;
  int2 stack[kStackSize];
  int sp = 0;
  int cur = bvh.n_internal ? kTopBit : -1;
  int cnt = bvh.n_internal ? 0 : (int)bvh.n_slots;
  const uint32_t max_steps = 2u * (bvh.n_internal + bvh.n_slots) + 8u;
  uint32_t steps = 0;
  for (;;) {
    if (++steps > max_steps) { atomicOr(err, kErrCorrupt); return false; }
    if (cur >= 0) {
      float4 a, b, z;
      int4 l;
      if (cur & kTopBit) {
        const float4* nd = s_top + 4 * (cur & (kTopBit - 1));
        a = nd[0]; b = nd[1]; z = nd[2];
        l = reinterpret_cast<const int4*>(nd)[3];
      } else {
        load_node(bvh.nodes + 4 * (size_t)cur, a, b, z, l);
      }
      const float tfar = ANY ? ray.tmax : c.t;
      float tl, tr;
      const bool hl = slab_box<false>(sr, ray.o, a.x, a.y, a.z, a.w, z.x, z.y, ray.tmin, tfar, tl);
      const bool hr = slab_box<false>(sr, ray.o, b.x, b.y, b.z, b.w, z.z, z.w, ray.tmin, tfar, tr);
      if (hl && hr) {
        int2 nearE = make_int2(l.x, l.z), farE = make_int2(l.y, l.w);
        if (tr < tl) { int2 t = nearE; nearE = farE; farE = t; }
        if (sp >= kStackSize) { atomicOr(err, kErrStackOverflow); return false; }
        stack[sp++] = farE;
        cur = nearE.x;
        cnt = nearE.y;
        continue;
      }
      if (hl) { cur = l.x; cnt = l.z; continue; }
      if (hr) { cur = l.y; cnt = l.w; continue; }
    } else {
      if (test_leaf<KIND, ANY, false>(bvh.prims, bvh.order, (uint32_t)(~cur), cnt, ray, c)) return true;
    }
    if (sp == 0) return false;
    const int2 e = stack[--sp];
    cur = e.x;
    cnt = e.y;
  }
}

template <int KIND, bool ANY>
__global__ void __launch_bounds__(kThreads, 10) k_trace_top(Bvh2View bvh, const float4* __restrict__ top,
                                                        const float4* __restrict__ rays, uint32_t n,
                                                        float4* __restrict__ hits, uint32_t* __restrict__ occ,
                                                        uint32_t* err, const uint32_t* __restrict__ perm) {
  __shared__ float4 s_top[4 * kTopNodes];
  __shared__ uint32_t s_exact[kThreads];
  __shared__ uint32_t s_n;
  for (int k = threadIdx.x; k < 4 * kTopNodes; k += kThreads) s_top[k] = __ldg(top + k);
  if (threadIdx.x == 0) s_n = 0;
  __syncthreads();
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t r = (perm && i < n) ? __ldg(perm + i) : i;
  bool occluded = false;
  if (i < n) {
    const Ray ray = load_ray(rays, r);
    if (zero_dir(slab_ray(ray.o, ray.d))) {
      s_exact[atomicAdd(&s_n, 1u)] = r;
    } else {
      Closest c = {ray.tmax, kMiss, 0.f, 0.f};
      occluded = walk_bvh2_top<KIND, ANY>(bvh, s_top, ray, c, err);
      if (!ANY) hits[r] = make_float4(c.t, __uint_as_float(c.prim), c.u, c.v);
    }
  }
  if (ANY) {
    if (perm) {
      if (occluded) atomicOr(occ + (r >> 5), 1u << (r & 31));
    } else {
      const uint32_t bits = __ballot_sync(0xffffffffu, occluded);
      const uint32_t w0 = blockIdx.x * blockDim.x + (threadIdx.x & ~31u);
      if ((threadIdx.x & 31) == 0 && w0 < n) occ[w0 >> 5] = bits;
    }
  }
  __syncthreads();
  const uint32_t ne = s_n;
  for (uint32_t k = threadIdx.x; k < ne; k += blockDim.x) {
    // inline: an out-of-line call here has crashed ptxas 13.0
    const uint32_t re = s_exact[k];
    const Ray ray = load_ray(rays, re);
    Closest c = {ray.tmax, kMiss, 0.f, 0.f};
    uint32_t visits = 0, tests = 0;
    const bool occ_e =
        walk_bvh2_form<KIND, ANY, false, kStackSize, true>(bvh, ray, slab_ray(ray.o, ray.d), c, visits, tests, err);
    if (!ANY) hits[re] = make_float4(c.t, __uint_as_float(c.prim), c.u, c.v);
    if (ANY && occ_e) atomicOr(occ + (re >> 5), 1u << (re & 31));
  }
}

template <int KIND, bool ANY, bool COUNT = false>
__global__ void __launch_bounds__(kThreads) k_trace_bvh4(Bvh4View bvh, const float4* __restrict__ rays,
                                                         uint32_t n, float4* __restrict__ hits,
                                                         uint32_t* __restrict__ occ, uint32_t* err,
                                                         const uint32_t* __restrict__ perm,
                                                         unsigned long long* counters) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t r = (perm && i < n) ? __ldg(perm + i) : i;
  bool occluded = false;
  uint32_t visits = 0, tests = 0;
  if (i < n) {
    Ray ray = load_ray(rays, r);
    Closest c = {ray.tmax, kMiss, 0.f, 0.f};
    occluded = walk_bvh4<KIND, ANY, COUNT, kStack4>(bvh, ray, c, visits, tests, err);
    if (!ANY) hits[r] = make_float4(c.t, __uint_as_float(c.prim), c.u, c.v);
  }
  if (ANY) {
    if (perm) {
      if (occluded) atomicOr(occ + (r >> 5), 1u << (r & 31));
    } else {
      uint32_t bits = __ballot_sync(0xffffffffu, occluded);
      uint32_t w0 = (blockIdx.x * blockDim.x + (threadIdx.x & ~31u));
      if ((threadIdx.x & 31) == 0 && w0 < n) occ[w0 >> 5] = bits;
    }
  }
  if (COUNT) add_counts(counters, visits, tests);
}

template <int KIND, bool ANY, bool COUNT = false>
__global__ void __launch_bounds__(kThreads) k_trace_bvh8(Bvh8View bvh, const float4* __restrict__ rays,
                                                         uint32_t n, float4* __restrict__ hits,
                                                         uint32_t* __restrict__ occ, uint32_t* err,
                                                         const uint32_t* __restrict__ perm,
                                                         unsigned long long* counters) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t r = (perm && i < n) ? __ldg(perm + i) : i;
  bool occluded = false;
  uint32_t visits = 0, tests = 0;
  if (i < n) {
    Ray ray = load_ray(rays, r);
    Closest c = {ray.tmax, kMiss, 0.f, 0.f};
    occluded = walk_bvh8<KIND, ANY, COUNT, kStack8>(bvh, ray, c, visits, tests, err);
    if (!ANY) hits[r] = make_float4(c.t, __uint_as_float(c.prim), c.u, c.v);
  }
  if (ANY) {
    if (perm) {
      if (occluded) atomicOr(occ + (r >> 5), 1u << (r & 31));
    } else {
      uint32_t bits = __ballot_sync(0xffffffffu, occluded);
      uint32_t w0 = (blockIdx.x * blockDim.x + (threadIdx.x & ~31u));
      if ((threadIdx.x & 31) == 0 && w0 < n) occ[w0 >> 5] = bits;
    }
  }
  if (COUNT) add_counts(counters, visits, tests);
}

template <int KIND, bool ANY>
void dispatch_bvh8(const Bvh8View& v, const float4* rays, uint32_t n, float4* hits, uint32_t* occ,
                   uint32_t* err, const uint32_t* perm, unsigned long long* counters, cudaStream_t s) {
  uint32_t g = (n + kThreads - 1) / kThreads;
  if (counters)
    k_trace_bvh8<KIND, ANY, true><<<g, kThreads, 0, s>>>(v, rays, n, hits, occ, err, perm, counters);
  else
    k_trace_bvh8<KIND, ANY, false><<<g, kThreads, 0, s>>>(v, rays, n, hits, occ, err, perm, nullptr);
}

template <int KIND, bool ANY>
void dispatch_bvh4(const Bvh4View& v, const float4* rays, uint32_t n, float4* hits, uint32_t* occ,
                   uint32_t* err, const uint32_t* perm, unsigned long long* counters, cudaStream_t s) {
  uint32_t g = (n + kThreads - 1) / kThreads;
  if (counters)
    k_trace_bvh4<KIND, ANY, true><<<g, kThreads, 0, s>>>(v, rays, n, hits, occ, err, perm, counters);
  else
    k_trace_bvh4<KIND, ANY, false><<<g, kThreads, 0, s>>>(v, rays, n, hits, occ, err, perm, nullptr);
}

// Warp-packet walk (RQ_SCHEDULING_WARP_PACKET): the warp walks the tree as
// one, with one stack whose entries carry the mask of lanes whose ray entered
// that child.  Each node is fetched once for the warp (a broadcast load); the
// lanes in the node's mask test its two child boxes against their own
// closest hit, and the warp goes next to the child most of them reach first.
// Every lane tests only nodes its ray entered, so results are those of the
// per-ray walk (the closest-hit rule makes them independent of visit order);
// coherent rays (camera, shadow) trade a few extra visits for full warps.
template <int KIND, bool ANY>
__global__ void __launch_bounds__(kThreads, 10) k_trace_packet(Bvh2View bvh, const float4* __restrict__ rays,
                                                               uint32_t n, float4* __restrict__ hits,
                                                               uint32_t* __restrict__ occ, uint32_t* err,
                                                               const uint32_t* __restrict__ perm) {
  __shared__ int4 stack_s[kThreads / 32][kStackSize];  // (node, count, lane mask, -)
  int4* stack = stack_s[threadIdx.x >> 5];
  const uint32_t lane = threadIdx.x & 31u, bit = 1u << lane;
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  const bool live = i < n;
  const uint32_t r = (perm && live) ? __ldg(perm + i) : i;
  Ray ray = live ? load_ray(rays, r) : Ray{{0.f, 0.f, 0.f}, {0.f, 0.f, 1.f}, 0.f, 0.f};
  Closest c = {ray.tmax, kMiss, 0.f, 0.f};
  const SlabRay sr = slab_ray(ray.o, ray.d);
  const bool ex = zero_dir(sr);
  const float* rb = bvh.root;
  float tn;
  const bool in_root = live && slab_any(ex, sr, ray.o, rb[0], rb[3], rb[1], rb[4], rb[2], rb[5], ray.tmin, ray.tmax, tn);
  uint32_t mask = __ballot_sync(0xffffffffu, in_root);
  uint32_t alive = mask;  // lanes still searching (any hit: not yet occluded)
  bool occluded = false;
  int sp = 0;
  int cur = bvh.n_internal ? 0 : -1;
  int cnt = bvh.n_internal ? 0 : (int)bvh.n_slots;
  const uint32_t max_steps = 2u * (bvh.n_internal + bvh.n_slots) + 8u;
  for (uint32_t steps = 0; mask; ++steps) {  // mask, cur, cnt, sp: uniform across the warp
    if (steps > max_steps) {
      if (lane == 0) atomicOr(err, kErrCorrupt);
      break;
    }
    const bool act = (mask & bit) != 0u;
    if (cur >= 0) {
      const float4* nd = bvh.nodes + 4 * (size_t)cur;
      const float4 a = __ldg(nd), b = __ldg(nd + 1), z = __ldg(nd + 2);
      const int4 l = __ldg(reinterpret_cast<const int4*>(nd + 3));
      bool hl = false, hr = false;
      float tl = 0.f, tr = 0.f;
      if (act) {
        const float tfar = ANY ? ray.tmax : c.t;
        hl = slab_any(ex, sr, ray.o, a.x, a.y, a.z, a.w, z.x, z.y, ray.tmin, tfar, tl);
        hr = slab_any(ex, sr, ray.o, b.x, b.y, b.z, b.w, z.z, z.w, ray.tmin, tfar, tr);
      }
      const uint32_t ml = __ballot_sync(0xffffffffu, hl), mr = __ballot_sync(0xffffffffu, hr);
      if (ml && mr) {
        const uint32_t lfirst = __ballot_sync(0xffffffffu, hl && (!hr || tl <= tr));
        const bool left = 2 * __popc(lfirst) >= __popc(ml | mr);
        if (sp >= kStackSize) {
          if (lane == 0) atomicOr(err, kErrStackOverflow);
          break;
        }
        if (lane == 0) stack[sp] = left ? make_int4(l.y, l.w, (int)mr, 0) : make_int4(l.x, l.z, (int)ml, 0);
        __syncwarp();
        ++sp;
        cur = left ? l.x : l.y;
        cnt = left ? l.z : l.w;
        mask = left ? ml : mr;
        continue;
      }
      if (ml) { cur = l.x; cnt = l.z; mask = ml; continue; }
      if (mr) { cur = l.y; cnt = l.w; mask = mr; continue; }
    } else {
      if (act && test_leaf<KIND, ANY, false>(bvh.prims, bvh.order, (uint32_t)(~cur), cnt, ray, c)) occluded = true;
      if (ANY) alive &= ~__ballot_sync(0xffffffffu, occluded);
    }
    // Next entry that still has a lane to serve.
    mask = 0u;
    while (sp > 0 && !mask) {
      const int4 e = stack[--sp];
      cur = e.x;
      cnt = e.y;
      mask = (uint32_t)e.z & alive;
    }
  }
  if (live && !ANY) hits[r] = make_float4(c.t, __uint_as_float(c.prim), c.u, c.v);
  if (ANY) {
    if (perm) {
      if (live && occluded) atomicOr(occ + (r >> 5), 1u << (r & 31));
    } else {
      const uint32_t bits = __ballot_sync(0xffffffffu, occluded);
      const uint32_t w0 = blockIdx.x * blockDim.x + (threadIdx.x & ~31u);
      if (lane == 0 && w0 < n) occ[w0 >> 5] = bits;
    }
  }
}

// -------------------------------------------------------- speculative walk
// While-while walk with speculative leaf postponement (Aila and Laine 2009,
// "Understanding the Efficiency of Ray Traversal on GPUs"): a lane that meets
// a leaf while its warp still has lanes on internal nodes keeps the leaf
// aside and walks on; the warp tests leaves when every active lane holds
// one, so node visits and leaf tests each run with fuller warps.  Leaves are
// tested later than in the plain walk, which can only widen the boxes a ray
// visits; the closest-hit rule (smallest t, ties to the smallest id) makes
// the result independent of that order.
template <int KIND, bool ANY>
__global__ void __launch_bounds__(kThreads, 10) k_trace_spec(Bvh2View bvh, const float4* __restrict__ rays,
                                                             uint32_t n, float4* __restrict__ hits,
                                                             uint32_t* __restrict__ occ, uint32_t* err,
                                                             const uint32_t* __restrict__ perm) {
  constexpr int kDone = 0x7FFFFFFF;  // no node left (never a valid internal index)
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t r = (perm && i < n) ? __ldg(perm + i) : i;
  bool occluded = false;
  if (i < n) {
    const Ray ray = load_ray(rays, r);
    Closest c = {ray.tmax, kMiss, 0.f, 0.f};
    const SlabRay sr = slab_ray(ray.o, ray.d);
    const bool ex = zero_dir(sr);
    float tn;
    const float* rb = bvh.root;
    if (slab_any(ex, sr, ray.o, rb[0], rb[3], rb[1], rb[4], rb[2], rb[5], ray.tmin, ray.tmax, tn)) {
      int2 stack[kStackSize];
      int sp = 0;
      int cur = bvh.n_internal ? 0 : -1;
      int cnt = bvh.n_internal ? 0 : (int)bvh.n_slots;
      int leaf = 0, lcnt = 0;
      bool has_leaf = false;
      const uint32_t max_steps = 2u * (bvh.n_internal + bvh.n_slots) + 8u;
      uint32_t steps = 0;
      for (;;) {
        // internal nodes, postponing the first leaf met
        while (cur >= 0 && cur != kDone) {
          if (++steps > max_steps) { atomicOr(err, kErrCorrupt); goto finish; }
          const float4* nd = bvh.nodes + 4 * (size_t)cur;
          float4 a = __ldg(nd), b = __ldg(nd + 1), z = __ldg(nd + 2);
          int4 l = __ldg(reinterpret_cast<const int4*>(nd + 3));
          const float tfar = ANY ? ray.tmax : c.t;
          float tl, tr;
          bool hl = slab_any(ex, sr, ray.o, a.x, a.y, a.z, a.w, z.x, z.y, ray.tmin, tfar, tl);
          bool hr = slab_any(ex, sr, ray.o, b.x, b.y, b.z, b.w, z.z, z.w, ray.tmin, tfar, tr);
          if (hl && hr) {
            int2 nearE = make_int2(l.x, l.z), farE = make_int2(l.y, l.w);
            if (tr < tl) { int2 t = nearE; nearE = farE; farE = t; }
            if (sp >= kStackSize) { atomicOr(err, kErrStackOverflow); goto finish; }
            stack[sp++] = farE;
            cur = nearE.x;
            cnt = nearE.y;
          } else if (hl) {
            cur = l.x;
            cnt = l.z;
          } else if (hr) {
            cur = l.y;
            cnt = l.w;
          } else if (sp == 0) {
            cur = kDone;
          } else {
            const int2 e = stack[--sp];
            cur = e.x;
            cnt = e.y;
          }
          if (cur < 0 && !has_leaf) {
            has_leaf = true;
            leaf = cur;
            lcnt = cnt;
            if (sp == 0) {
              cur = kDone;
            } else {
              const int2 e = stack[--sp];
              cur = e.x;
              cnt = e.y;
            }
          }
          if (!__any_sync(__activemask(), !has_leaf)) break;  // every active lane holds a leaf
        }
        // the postponed leaf, then leaves found on top of the stack
        while (has_leaf || cur < 0) {
          if (!has_leaf) {
            leaf = cur;
            lcnt = cnt;
            if (sp == 0) {
              cur = kDone;
            } else {
              const int2 e = stack[--sp];
              cur = e.x;
              cnt = e.y;
            }
          }
          has_leaf = false;
          if (++steps > max_steps) { atomicOr(err, kErrCorrupt); goto finish; }
          if (test_leaf<KIND, ANY, false>(bvh.prims, bvh.order, (uint32_t)(~leaf), lcnt, ray, c)) {
            occluded = true;
            goto finish;
          }
        }
        if (cur == kDone) break;
      }
    }
  finish:
    if (!ANY) hits[r] = make_float4(c.t, __uint_as_float(c.prim), c.u, c.v);
  }
  if (ANY) {
    if (perm) {
      if (occluded) atomicOr(occ + (r >> 5), 1u << (r & 31));
    } else {
      const uint32_t bits = __ballot_sync(0xffffffffu, occluded);
      const uint32_t w0 = (blockIdx.x * blockDim.x + (threadIdx.x & ~31u));
      if ((threadIdx.x & 31) == 0 && w0 < n) occ[w0 >> 5] = bits;
    }
  }
}

// ------------------------------------------------------------ lane refill
// FAST walk with persistent warps that refill finished lanes: a warp takes
// new rays from a global counter for its idle lanes once at least
// kRefillIdle of them are idle, so incoherent batches keep more lanes busy
// than one-ray-per-thread launches, where a warp holds its SIMD slots until
// its longest ray ends.  Each ray still takes exactly walk_bvh2's sequence of
// steps (one node or leaf per loop iteration), so results are identical.
// Any-hit bits are set with atomicOr (occ zeroed by the launcher).
constexpr int kRefillIdle = 8;

template <int KIND, bool ANY>
__global__ void __launch_bounds__(kThreads) k_trace_refill(Bvh2View bvh, const float4* __restrict__ rays, uint32_t n,
                                                           float4* __restrict__ hits, uint32_t* __restrict__ occ,
                                                           uint32_t* err, const uint32_t* __restrict__ perm,
                                                           uint32_t* __restrict__ work) {
  const uint32_t lane = threadIdx.x & 31, below = (1u << lane) - 1u;
  const uint32_t max_steps = 2u * (bvh.n_internal + bvh.n_slots) + 8u;
  int2 stack[kStackSize];
  Ray ray = {{0.f, 0.f, 0.f}, {0.f, 0.f, 1.f}, 0.f, 0.f};
  SlabRay sr = slab_ray(ray.o, ray.d);
  bool ex = false;
  Closest c = {0.f, kMiss, 0.f, 0.f};
  int cur = 0, cnt = 0, sp = 0;
  uint32_t r = 0, steps = 0;
  bool active = false, exhausted = false;
  for (;;) {
    const uint32_t idle = __ballot_sync(0xffffffffu, !active);
    if (!exhausted && __popc(idle) >= kRefillIdle) {
      const uint32_t want = __popc(idle);
      uint32_t base = 0;
      if (lane == 0) base = atomicAdd(work, want);
      base = __shfl_sync(0xffffffffu, base, 0);
      if ((uint64_t)base + want >= n) exhausted = true;
      if (!active) {
        const uint32_t i = base + __popc(idle & below);
        if (i < n) {
          r = perm ? __ldg(perm + i) : i;
          ray = load_ray(rays, r);
          c = {ray.tmax, kMiss, 0.f, 0.f};
          sr = slab_ray(ray.o, ray.d);
          ex = zero_dir(sr);
          float tn;
          const float* rb = bvh.root;
          if (slab_any(ex, sr, ray.o, rb[0], rb[3], rb[1], rb[4], rb[2], rb[5], ray.tmin, ray.tmax, tn)) {
            active = true;
            sp = 0;
            steps = 0;
            cur = bvh.n_internal ? 0 : -1;
            cnt = bvh.n_internal ? 0 : (int)bvh.n_slots;
          } else if (!ANY) {
            hits[r] = make_float4(c.t, __uint_as_float(c.prim), c.u, c.v);
          }
        }
      }
      continue;
    }
    if (idle == 0xffffffffu) break;  // every lane idle and no rays left
    if (!active) continue;
    bool done = false, hit = false;
    if (++steps > max_steps) {
      atomicOr(err, kErrCorrupt);
      done = true;
    } else if (cur >= 0) {
      const float4* nd = bvh.nodes + 4 * (size_t)cur;
      float4 a = __ldg(nd), b = __ldg(nd + 1), z = __ldg(nd + 2);
      int4 l = __ldg(reinterpret_cast<const int4*>(nd + 3));
      const float tfar = ANY ? ray.tmax : c.t;
      float tl, tr;
      bool hl = slab_any(ex, sr, ray.o, a.x, a.y, a.z, a.w, z.x, z.y, ray.tmin, tfar, tl);
      bool hr = slab_any(ex, sr, ray.o, b.x, b.y, b.z, b.w, z.z, z.w, ray.tmin, tfar, tr);
      if (hl && hr) {
        int2 nearE = make_int2(l.x, l.z), farE = make_int2(l.y, l.w);
        if (tr < tl) { int2 t = nearE; nearE = farE; farE = t; }
        if (sp >= kStackSize) {
          atomicOr(err, kErrStackOverflow);
          done = true;
        } else {
          stack[sp++] = farE;
          cur = nearE.x;
          cnt = nearE.y;
          continue;
        }
      } else if (hl) {
        cur = l.x;
        cnt = l.z;
        continue;
      } else if (hr) {
        cur = l.y;
        cnt = l.w;
        continue;
      }
    } else if (test_leaf<KIND, ANY, false>(bvh.prims, bvh.order, (uint32_t)(~cur), cnt, ray, c)) {
      hit = true;
      done = true;
    }
    if (!done) {
      if (sp == 0) {
        done = true;
      } else {
        int2 e = stack[--sp];
        cur = e.x;
        cnt = e.y;
      }
    }
    if (done) {
      if (!ANY) hits[r] = make_float4(c.t, __uint_as_float(c.prim), c.u, c.v);
      else if (hit) atomicOr(occ + (r >> 5), 1u << (r & 31));
      active = false;
    }
  }
}

template <int KIND, bool ANY>
cudaError_t launch_refill_kind(const Bvh2View& v, const float4* rays, uint32_t n, float4* hits, uint32_t* occ,
                               uint32_t* err, const uint32_t* perm, uint32_t* work, cudaStream_t s) {
  auto k = k_trace_refill<KIND, ANY>;
  int per_sm = 0, dev = 0, sms = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, kThreads, 0);
  if (e == cudaSuccess) e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return e;
  uint64_t blocks = (uint64_t)(per_sm > 0 ? per_sm : 1) * (uint64_t)sms;
  const uint64_t enough = ((uint64_t)n + kThreads - 1) / kThreads;
  if (blocks > enough) blocks = enough;
  if ((e = cudaMemsetAsync(work, 0, 4, s)) != cudaSuccess) return e;
  if (ANY && (e = cudaMemsetAsync(occ, 0, (size_t)((n + 31) / 32) * 4, s)) != cudaSuccess) return e;
  k<<<(unsigned)blocks, kThreads, 0, s>>>(v, rays, n, hits, occ, err, perm, work);
  return cudaGetLastError();
}

// Reference semantics: pre-order, unclipped division slab tests.
template <int KIND, bool ANY>
__global__ void __launch_bounds__(kThreads) k_trace_ref(Bvh2View bvh, const float4* __restrict__ rays,
                                                        uint32_t n, float4* __restrict__ hits,
                                                        uint32_t* __restrict__ occ, uint32_t* err) {
  const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  bool occluded = false;
  if (r < n) {
    Ray ray = load_ray(rays, r);
    Closest c = {ray.tmax, kMiss, 0.f, 0.f};
    float a0, a1;
    const float* rb = bvh.root;
    if (box_ref(ray.o, ray.d, rb[0], rb[3], rb[1], rb[4], rb[2], rb[5], a0, a1)) {
      int2 stack[kStackSize];
      int sp = 0;
      int cur = bvh.n_internal ? 0 : -1;
      int cnt = bvh.n_internal ? 0 : (int)bvh.n_slots;
      // A valid walk visits every node at most once.
      const uint32_t max_steps = 2u * (bvh.n_internal + bvh.n_slots) + 8u;
      uint32_t steps = 0;
      for (;;) {
        if (++steps > max_steps) { atomicOr(err, kErrCorrupt); break; }
        if (cur >= 0) {
          const float4* nd = bvh.nodes + 4 * (size_t)cur;
          float4 a = __ldg(nd), b = __ldg(nd + 1), z = __ldg(nd + 2);
          int4 l = __ldg(reinterpret_cast<const int4*>(nd + 3));
          bool hl = box_ref(ray.o, ray.d, a.x, a.y, a.z, a.w, z.x, z.y, a0, a1);
          bool hr = box_ref(ray.o, ray.d, b.x, b.y, b.z, b.w, z.z, z.w, a0, a1);
          if (hr) {
            if (sp >= kStackSize) { atomicOr(err, kErrStackOverflow); break; }
            stack[sp++] = make_int2(l.y, l.w);
          }
          if (hl) { cur = l.x; cnt = l.z; continue; }
        } else {
          if (test_leaf<KIND, ANY, true>(bvh.prims, bvh.order, (uint32_t)(~cur), cnt, ray, c)) {
            occluded = true;
            break;
          }
        }
        if (sp == 0) break;
        int2 e = stack[--sp];
        cur = e.x;
        cnt = e.y;
      }
    }
    if (!ANY) hits[r] = make_float4(c.t, __uint_as_float(c.prim), c.u, c.v);
  }
  if (ANY) {
    uint32_t bits = __ballot_sync(0xffffffffu, occluded);
    uint32_t w0 = (blockIdx.x * blockDim.x + (threadIdx.x & ~31u));
    if ((threadIdx.x & 31) == 0 && w0 < n) occ[w0 >> 5] = bits;
  }
}

// boxIntersect (accelerators.h:668-690): the ids of the primitives in every
// leaf the reference's walk reaches (division slab test, no clipping,
// pre-order: left subtree before right), per ray.  FILL = false counts them;
// FILL = true writes them at offs[r] (the exclusive prefix of the counts).
template <bool FILL>
__global__ void __launch_bounds__(kThreads) k_candidates(Bvh2View bvh, const float4* __restrict__ rays, uint32_t n,
                                                         uint32_t* __restrict__ counts,
                                                         const uint32_t* __restrict__ offs,
                                                         uint32_t* __restrict__ ids,
                                                         unsigned long long* __restrict__ total, uint32_t* err) {
  const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  const Ray ray = load_ray(rays, r);
  uint32_t cnt_out = 0;
  const uint32_t base = FILL ? __ldg(offs + r) : 0u;
  const uint32_t cap = FILL ? __ldg(counts + r) : 0u;
  float a0, a1;
  const float* rb = bvh.root;
  if (box_ref(ray.o, ray.d, rb[0], rb[3], rb[1], rb[4], rb[2], rb[5], a0, a1)) {
    int2 stack[kStackSize];
    int sp = 0;
    int cur = bvh.n_internal ? 0 : -1;
    int cnt = bvh.n_internal ? 0 : (int)bvh.n_slots;
    const uint32_t max_steps = 2u * (bvh.n_internal + bvh.n_slots) + 8u;
    uint32_t steps = 0;
    for (;;) {
      if (++steps > max_steps) { atomicOr(err, kErrCorrupt); break; }
      if (cur >= 0) {
        const float4* nd = bvh.nodes + 4 * (size_t)cur;
        float4 a = __ldg(nd), b = __ldg(nd + 1), z = __ldg(nd + 2);
        int4 l = __ldg(reinterpret_cast<const int4*>(nd + 3));
        bool hl = box_ref(ray.o, ray.d, a.x, a.y, a.z, a.w, z.x, z.y, a0, a1);
        bool hr = box_ref(ray.o, ray.d, b.x, b.y, b.z, b.w, z.z, z.w, a0, a1);
        if (hr) {
          if (sp >= kStackSize) { atomicOr(err, kErrStackOverflow); break; }
          stack[sp++] = make_int2(l.y, l.w);
        }
        if (hl) { cur = l.x; cnt = l.z; continue; }
      } else {
        for (int k = 0; k < cnt; ++k) {
          if (FILL && cnt_out < cap) ids[(size_t)base + cnt_out] = __ldg(bvh.order + (uint32_t)(~cur) + (uint32_t)k);
          ++cnt_out;
        }
      }
      if (sp == 0) break;
      int2 e = stack[--sp];
      cur = e.x;
      cnt = e.y;
    }
  }
  if (!FILL) {
    counts[r] = cnt_out;
    atomicAdd(total, (unsigned long long)cnt_out);  // 64-bit: the 32-bit offsets must not wrap
  } else if (cnt_out != cap) {
    atomicOr(err, kErrCorrupt);  // the fill walk repeats the count walk
  }
}

// NONE: every primitive in id order (main.cpp:373-387), staged through
// shared memory in tiles shared by the block's rays.
constexpr int kBruteTile = 256;

template <int KIND, bool ANY, bool REF>
__global__ void __launch_bounds__(kThreads) k_brute(const float4* __restrict__ prims, uint32_t n_prims,
                                                    const float4* __restrict__ rays, uint32_t n,
                                                    float4* __restrict__ hits, uint32_t* __restrict__ occ) {
  constexpr int W = KIND == kTriangles ? 3 : 1;
  __shared__ float4 tile[kBruteTile * W];
  const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  const bool active = r < n;
  Ray ray = active ? load_ray(rays, r) : Ray{{0, 0, 0}, {0, 0, 1}, 0.f, 0.f};
  Closest c = {ray.tmax, kMiss, 0.f, 0.f};
  bool done = !active;
  for (uint32_t base = 0; base < n_prims; base += kBruteTile) {
    uint32_t cnt = n_prims - base < (uint32_t)kBruteTile ? n_prims - base : (uint32_t)kBruteTile;
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < cnt * W; i += blockDim.x) tile[i] = __ldg(prims + (size_t)base * W + i);
    __syncthreads();
    if (done) continue;
    for (uint32_t k = 0; k < cnt; ++k) {
      if (KIND == kTriangles) {
        float t, u, v;
        if (tri_mt(tile[3 * k], tile[3 * k + 1], tile[3 * k + 2], ray.o, ray.d, ray.tmin,
                   ANY ? ray.tmax : c.t, t, u, v)) {
          if (ANY) { done = true; break; }
          c = {t, base + k, u, v};
        }
      } else {
        if (ANY) {
          float t0, t1, t;
          if (REF ? sphere_ref(tile[k], ray.o, ray.d, t0, t1)
                  : sphere_closest(tile[k], ray.o, ray.d, ray.tmin, ray.tmax, false, t)) {
            done = true;
            break;
          }
        } else {
          float t;
          if (sphere_closest(tile[k], ray.o, ray.d, ray.tmin, c.t, REF, t)) c = {t, base + k, 0.f, 0.f};
        }
      }
    }
  }
  if (!ANY && active) hits[r] = make_float4(c.t, __uint_as_float(c.prim), c.u, c.v);
  if (ANY) {
    bool o = active && done;
    uint32_t bits = __ballot_sync(0xffffffffu, o);
    uint32_t w0 = (blockIdx.x * blockDim.x + (threadIdx.x & ~31u));
    if ((threadIdx.x & 31) == 0 && w0 < n) occ[w0 >> 5] = bits;
  }
}

template <int KIND, bool ANY>
void dispatch_bvh2(int traversal, const Bvh2View& v, const float4* rays, uint32_t n, float4* hits,
                   uint32_t* occ, uint32_t* err, const uint32_t* perm, bool small_stack, uint32_t* exact,
                   cudaStream_t s) {
  uint32_t g = (n + kThreads - 1) / kThreads;
  if (traversal == RQ_TRAVERSAL_REFERENCE) {
    k_trace_ref<KIND, ANY><<<g, kThreads, 0, s>>>(v, rays, n, hits, occ, err);
  } else if (small_stack) {
    k_trace_fast<KIND, ANY, false, kDebugStack><<<g, kThreads, 0, s>>>(v, rays, n, hits, occ, err, nullptr, perm);
  } else if (exact) {
    cudaMemsetAsync(exact, 0, 8, s);  // exact-ray count and work counter
    const auto k = v.unit_leaves ? k_trace_warps<KIND, ANY, true> : k_trace_warps<KIND, ANY, false>;
    k<<<std::min(g, resident_blocks(k)), kThreads, 0, s>>>(v, rays, n, hits, occ, err, perm, exact);
    count_launch();
    k_trace_exact<KIND, ANY><<<kExactBlocks, kThreads, 0, s>>>(v, rays, exact, hits, occ, err);
  } else {
    k_trace_fast<KIND, ANY, false><<<g, kThreads, 0, s>>>(v, rays, n, hits, occ, err, nullptr, perm);
  }
}

template <int KIND, bool ANY>
void dispatch_brute(int traversal, const float4* prims, uint32_t np, const float4* rays, uint32_t n,
                    float4* hits, uint32_t* occ, cudaStream_t s) {
  uint32_t g = (n + kThreads - 1) / kThreads;
  if (traversal == RQ_TRAVERSAL_REFERENCE)
    k_brute<KIND, ANY, true><<<g, kThreads, 0, s>>>(prims, np, rays, n, hits, occ);
  else
    k_brute<KIND, ANY, false><<<g, kThreads, 0, s>>>(prims, np, rays, n, hits, occ);
}

template <int KIND, bool ANY>
void dispatch_count(const Bvh2View& v, const float4* rays, uint32_t n, float4* hits, uint32_t* occ,
                    uint32_t* err, unsigned long long* counters, cudaStream_t s) {
  uint32_t g = (n + kThreads - 1) / kThreads;
  k_trace_fast<KIND, ANY, true><<<g, kThreads, 0, s>>>(v, rays, n, hits, occ, err, counters);
}

}  // namespace

void launch_trace_bvh2_counted(int kind, bool any, const Bvh2View& v, const float4* rays, uint32_t n,
                               float4* hits, uint32_t* occ, uint32_t* err, unsigned long long* counters,
                               cudaStream_t s) {
  if (n == 0) return;
  count_launch();
  if (kind == kTriangles) {
    if (any) dispatch_count<kTriangles, true>(v, rays, n, hits, occ, err, counters, s);
    else dispatch_count<kTriangles, false>(v, rays, n, hits, occ, err, counters, s);
  } else {
    if (any) dispatch_count<kSpheres, true>(v, rays, n, hits, occ, err, counters, s);
    else dispatch_count<kSpheres, false>(v, rays, n, hits, occ, err, counters, s);
  }
}

void launch_trace_bvh2(int kind, int traversal, bool any, const Bvh2View& v, const float4* rays,
                       uint32_t n, float4* hits, uint32_t* occ, uint32_t* err, cudaStream_t s,
                       const uint32_t* perm, bool small_stack, uint32_t* exact) {
  if (n == 0) return;
  count_launch();
  if (traversal == RQ_TRAVERSAL_REFERENCE) perm = nullptr;
  if (any && perm) cudaMemsetAsync(occ, 0, (size_t)((n + 31) / 32) * 4, s);
  if (kind == kTriangles) {
    if (any) dispatch_bvh2<kTriangles, true>(traversal, v, rays, n, hits, occ, err, perm, small_stack, exact, s);
    else dispatch_bvh2<kTriangles, false>(traversal, v, rays, n, hits, occ, err, perm, small_stack, exact, s);
  } else {
    if (any) dispatch_bvh2<kSpheres, true>(traversal, v, rays, n, hits, occ, err, perm, small_stack, exact, s);
    else dispatch_bvh2<kSpheres, false>(traversal, v, rays, n, hits, occ, err, perm, small_stack, exact, s);
  }
}

void launch_trace_bvh4(int kind, bool any, const Bvh4View& v, const float4* rays, uint32_t n, float4* hits,
                       uint32_t* occ, uint32_t* err, cudaStream_t s, const uint32_t* perm,
                       unsigned long long* counters) {
  if (n == 0) return;
  count_launch();
  if (any && perm) cudaMemsetAsync(occ, 0, (size_t)((n + 31) / 32) * 4, s);
  if (kind == kTriangles) {
    if (any) dispatch_bvh4<kTriangles, true>(v, rays, n, hits, occ, err, perm, counters, s);
    else dispatch_bvh4<kTriangles, false>(v, rays, n, hits, occ, err, perm, counters, s);
  } else {
    if (any) dispatch_bvh4<kSpheres, true>(v, rays, n, hits, occ, err, perm, counters, s);
    else dispatch_bvh4<kSpheres, false>(v, rays, n, hits, occ, err, perm, counters, s);
  }
}

void launch_trace_bvh2_top(int kind, bool any, const Bvh2View& v, float4* top, const float4* rays, uint32_t n,
                           float4* hits, uint32_t* occ, uint32_t* err, const uint32_t* perm, cudaStream_t s) {
  if (n == 0) return;
  count_launch(2);
  k_top_copy<<<1, 32, 0, s>>>(v.nodes, v.n_internal, top);
  if (any && perm) cudaMemsetAsync(occ, 0, (size_t)((n + 31) / 32) * 4, s);
  const uint32_t g = (n + kThreads - 1) / kThreads;
  if (kind == kTriangles) {
    if (any) k_trace_top<kTriangles, true><<<g, kThreads, 0, s>>>(v, top, rays, n, hits, occ, err, perm);
    else k_trace_top<kTriangles, false><<<g, kThreads, 0, s>>>(v, top, rays, n, hits, occ, err, perm);
  } else {
    if (any) k_trace_top<kSpheres, true><<<g, kThreads, 0, s>>>(v, top, rays, n, hits, occ, err, perm);
    else k_trace_top<kSpheres, false><<<g, kThreads, 0, s>>>(v, top, rays, n, hits, occ, err, perm);
  }
}

void launch_trace_bvh8(int kind, bool any, const Bvh8View& v, const float4* rays, uint32_t n, float4* hits,
                       uint32_t* occ, uint32_t* err, cudaStream_t s, const uint32_t* perm,
                       unsigned long long* counters) {
  if (n == 0) return;
  count_launch();
  if (any && perm) cudaMemsetAsync(occ, 0, (size_t)((n + 31) / 32) * 4, s);
  if (kind == kTriangles) {
    if (any) dispatch_bvh8<kTriangles, true>(v, rays, n, hits, occ, err, perm, counters, s);
    else dispatch_bvh8<kTriangles, false>(v, rays, n, hits, occ, err, perm, counters, s);
  } else {
    if (any) dispatch_bvh8<kSpheres, true>(v, rays, n, hits, occ, err, perm, counters, s);
    else dispatch_bvh8<kSpheres, false>(v, rays, n, hits, occ, err, perm, counters, s);
  }
}

cudaError_t launch_trace_bvh2_refill(int kind, bool any, const Bvh2View& v, const float4* rays, uint32_t n,
                                     float4* hits, uint32_t* occ, uint32_t* err, const uint32_t* perm,
                                     uint32_t* work, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  count_launch();
  if (kind == kTriangles)
    return any ? launch_refill_kind<kTriangles, true>(v, rays, n, hits, occ, err, perm, work, s)
               : launch_refill_kind<kTriangles, false>(v, rays, n, hits, occ, err, perm, work, s);
  return any ? launch_refill_kind<kSpheres, true>(v, rays, n, hits, occ, err, perm, work, s)
             : launch_refill_kind<kSpheres, false>(v, rays, n, hits, occ, err, perm, work, s);
}

void launch_trace_bvh2_spec(int kind, bool any, const Bvh2View& v, const float4* rays, uint32_t n, float4* hits,
                            uint32_t* occ, uint32_t* err, const uint32_t* perm, cudaStream_t s) {
  if (n == 0) return;
  count_launch();
  if (any && perm) cudaMemsetAsync(occ, 0, (size_t)((n + 31) / 32) * 4, s);
  const uint32_t g = (n + kThreads - 1) / kThreads;
  if (kind == kTriangles) {
    if (any) k_trace_spec<kTriangles, true><<<g, kThreads, 0, s>>>(v, rays, n, hits, occ, err, perm);
    else k_trace_spec<kTriangles, false><<<g, kThreads, 0, s>>>(v, rays, n, hits, occ, err, perm);
  } else {
    if (any) k_trace_spec<kSpheres, true><<<g, kThreads, 0, s>>>(v, rays, n, hits, occ, err, perm);
    else k_trace_spec<kSpheres, false><<<g, kThreads, 0, s>>>(v, rays, n, hits, occ, err, perm);
  }
}

void launch_trace_bvh2_packet(int kind, bool any, const Bvh2View& v, const float4* rays, uint32_t n, float4* hits,
                              uint32_t* occ, uint32_t* err, const uint32_t* perm, cudaStream_t s) {
  if (n == 0) return;
  count_launch();
  if (any && perm) cudaMemsetAsync(occ, 0, (size_t)((n + 31) / 32) * 4, s);
  const uint32_t g = (n + kThreads - 1) / kThreads;
  if (kind == kTriangles) {
    if (any) k_trace_packet<kTriangles, true><<<g, kThreads, 0, s>>>(v, rays, n, hits, occ, err, perm);
    else k_trace_packet<kTriangles, false><<<g, kThreads, 0, s>>>(v, rays, n, hits, occ, err, perm);
  } else {
    if (any) k_trace_packet<kSpheres, true><<<g, kThreads, 0, s>>>(v, rays, n, hits, occ, err, perm);
    else k_trace_packet<kSpheres, false><<<g, kThreads, 0, s>>>(v, rays, n, hits, occ, err, perm);
  }
}

void launch_candidates(const Bvh2View& v, const float4* rays, uint32_t n, uint32_t* counts, const uint32_t* offs,
                       uint32_t* ids, unsigned long long* total, uint32_t* err, cudaStream_t s) {
  if (n == 0) return;
  count_launch();
  const uint32_t g = (n + kThreads - 1) / kThreads;
  if (ids) k_candidates<true><<<g, kThreads, 0, s>>>(v, rays, n, counts, offs, ids, nullptr, err);
  else k_candidates<false><<<g, kThreads, 0, s>>>(v, rays, n, counts, nullptr, nullptr, total, err);
}

// Sort keys of rays for coherent tracing (30 bits, direction octant on top):
//   RQ_RAY_SORT_OCTANT_MORTON    octant | 27-bit Morton code of the origin
//   RQ_RAY_SORT_ORIGIN_DIRECTION octant | 15-bit origin Morton | 12-bit direction
//   RQ_RAY_SORT_DIRECTION_ORIGIN octant | 12-bit direction | 15-bit origin Morton
//   RQ_RAY_SORT_OCTANT_MORTON12  octant | 12-bit origin Morton (15 bits: a 2-pass sort)
//   RQ_RAY_SORT_OCTANT_MORTON3   octant | 3-bit origin Morton (6 bits: one pass)
//   RQ_RAY_SORT_OCTANT           octant (3 bits: one pass)
// The origin is quantised in the root box; the direction by |dx|, |dy| of the
// unit direction, 6 bits each (|dz| follows within the octant).
__device__ __forceinline__ uint32_t spread_bits(uint32_t v) {  // 10 bits -> every third bit
  v = (v | (v << 16)) & 0x030000FFu;
  v = (v | (v << 8)) & 0x0300F00Fu;
  v = (v | (v << 4)) & 0x030C30C3u;
  v = (v | (v << 2)) & 0x09249249u;
  return v;
}

// The sort key of ray i under `mode` (the table above).
__device__ __forceinline__ uint32_t ray_sort_key(const float4* __restrict__ rays, uint32_t i,
                                                 const float* __restrict__ root, int mode) {
  uint32_t key = 0;
  const float4 b = __ldg(rays + 2 * (size_t)i + 1);
  const uint32_t oct = (b.x < 0.f ? 4u : 0u) | (b.y < 0.f ? 2u : 0u) | (b.z < 0.f ? 1u : 0u);
  if (mode == RQ_RAY_SORT_OCTANT) {
    key = oct;
  } else {
    const float4 a = __ldg(rays + 2 * (size_t)i);
    const float o[3] = {a.x, a.y, a.z};
    const int obits = mode == RQ_RAY_SORT_OCTANT_MORTON ? 9 : mode == RQ_RAY_SORT_OCTANT_MORTON12 ? 4
                      : mode == RQ_RAY_SORT_OCTANT_MORTON3 ? 1 : 5;
    const float cells = (float)(1u << obits);
    uint32_t q[3];
    for (int k = 0; k < 3; ++k) {
      float lo = root[k], ext = root[3 + k] - root[k];
      float u = ext > 0.f ? (o[k] - lo) / ext : 0.f;
      u = fminf(fmaxf(u * cells, 0.f), cells - 1.f);
      q[k] = (uint32_t)u;
    }
    const uint32_t morton = (spread_bits(q[0]) << 2) | (spread_bits(q[1]) << 1) | spread_bits(q[2]);
    if (mode == RQ_RAY_SORT_OCTANT_MORTON) {
      key = (oct << 27) | morton;
    } else if (mode == RQ_RAY_SORT_OCTANT_MORTON12) {
      key = (oct << 12) | morton;
    } else if (mode == RQ_RAY_SORT_OCTANT_MORTON3) {
      key = (oct << 3) | morton;
    } else {
      const float len = sqrtf(b.x * b.x + b.y * b.y + b.z * b.z);
      const float inv = len > 0.f ? 1.0f / len : 0.f;
      const uint32_t dx = (uint32_t)fminf(fabsf(b.x) * inv * 64.f, 63.f);
      const uint32_t dy = (uint32_t)fminf(fabsf(b.y) * inv * 64.f, 63.f);
      const uint32_t dir = (dx << 6) | dy;
      key = mode == RQ_RAY_SORT_ORIGIN_DIRECTION ? (oct << 27) | (morton << 12) | dir
                                                 : (oct << 27) | (dir << 15) | morton;
    }
  }
  return key;
}

// Sort keys of the optional ray order, and (when hist is given) the digit
// histogram of the sort's `passes` 8-bit digits in the same read: a block
// of 256 threads strides over the rays, counts in shared memory with one
// atomic per distinct digit in a warp, and adds its counts to hist once.
// The octant-only key reads just the direction.
__global__ void __launch_bounds__(256) k_ray_keys(const float4* __restrict__ rays, uint32_t n,
                                                  const float* __restrict__ root, int mode,
                                                  uint32_t* __restrict__ keys, uint32_t* __restrict__ vals,
                                                  uint32_t* __restrict__ hist, int passes) {
  __shared__ uint32_t sh[4][256];
  if (hist) {
    for (int k = threadIdx.x; k < 4 * 256; k += blockDim.x) (&sh[0][0])[k] = 0u;
    __syncthreads();
  }
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t stride = gridDim.x * blockDim.x;
  const uint32_t end = (n + 31u) & ~31u;  // whole warps take part in the histogram
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < end; i += stride) {
    const bool live = i < n;
    uint32_t key = 0;
    if (live) {
      key = ray_sort_key(rays, i, root, mode);
      keys[i] = key;
      vals[i] = i;
    }
    if (hist) {
      const uint32_t lanes = __ballot_sync(0xffffffffu, live);
      if (live) {
        for (int p = 0; p < passes; ++p) {
          const uint32_t d = (key >> (8 * p)) & 255u;
          const uint32_t same = __match_any_sync(lanes, d);
          if ((same & ((1u << lane) - 1u)) == 0u) atomicAdd(&sh[p][d], (uint32_t)__popc(same));
        }
      }
    }
  }
  if (hist) {
    __syncthreads();
    for (int k = threadIdx.x; k < passes * 256; k += blockDim.x) {
      const uint32_t v = (&sh[0][0])[k];
      if (v) atomicAdd(hist + k, v);
    }
  }
}

// Ray orders of at most 6 key bits (RQ_RAY_SORT_OCTANT, RQ_RAY_SORT_OCTANT_MORTON3)
// by a stable counting sort instead of a radix pass (whose decoupled look-back
// runs across thousands of tiles): per block of kOrderSpan rays the key bytes
// and the keys' counts (one shared atomic per distinct key in a warp), an
// exclusive scan of the counts in bucket-major order (one block), then each
// block places its rays -- a ray's position is its bucket's offset for the
// block plus the same-key rays before it in the block (earlier rounds, earlier
// warps of its round, earlier lanes of its warp).  The permutation is the
// stable sort's.
constexpr uint32_t kOrderThreads = 256, kOrderRounds = 16, kOrderSpan = kOrderThreads * kOrderRounds;
constexpr uint32_t kOrderWarps = kOrderThreads / 32, kOrderMaxBuckets = 64, kOrderNone = 64;

__global__ void __launch_bounds__(kOrderThreads) k_order_count(const float4* __restrict__ rays, uint32_t n,
                                                               const float* __restrict__ root, int mode,
                                                               uint32_t buckets, uint8_t* __restrict__ key8,
                                                               uint32_t* __restrict__ counts) {
  __shared__ uint32_t sh[kOrderMaxBuckets];
  const uint32_t lane = threadIdx.x & 31u;
  if (threadIdx.x < kOrderMaxBuckets) sh[threadIdx.x] = 0u;
  __syncthreads();
  const uint32_t base = blockIdx.x * kOrderSpan;
  for (uint32_t r = 0; r < kOrderRounds; ++r) {
    const uint32_t i = base + r * kOrderThreads + threadIdx.x;
    uint32_t k = kOrderNone;
    if (i < n) {
      k = ray_sort_key(rays, i, root, mode);
      key8[i] = (uint8_t)k;
    }
    const uint32_t peers = __match_any_sync(0xffffffffu, k);
    if (k < kOrderNone && lane == (uint32_t)(__ffs(peers) - 1)) atomicAdd(&sh[k], (uint32_t)__popc(peers));
  }
  __syncthreads();
  for (uint32_t k = threadIdx.x; k < buckets; k += blockDim.x) counts[(size_t)k * gridDim.x + blockIdx.x] = sh[k];
}

// Exclusive scan of m words in place, one block of 1024 threads (each a
// contiguous run of the words, read with its loads in flight together).
__global__ void __launch_bounds__(1024) k_order_scan(uint32_t* __restrict__ counts, uint32_t m) {
  __shared__ uint32_t part[1024];
  const uint32_t per = (m + blockDim.x - 1) / blockDim.x;
  const uint32_t b = min(threadIdx.x * per, m), e = min(b + per, m);
  uint32_t sum = 0;
#pragma unroll 16
  for (uint32_t k = b; k < e; ++k) sum += __ldcg(counts + k);
  part[threadIdx.x] = sum;
  __syncthreads();
  for (uint32_t off = 1; off < blockDim.x; off <<= 1) {
    const uint32_t v = threadIdx.x >= off ? part[threadIdx.x - off] : 0u;
    __syncthreads();
    part[threadIdx.x] += v;
    __syncthreads();
  }
  uint32_t run = part[threadIdx.x] - sum;
#pragma unroll 16
  for (uint32_t k = b; k < e; ++k) {
    const uint32_t c = __ldcg(counts + k);
    counts[k] = run;
    run += c;
  }
}

__global__ void __launch_bounds__(kOrderThreads) k_order_scatter(const uint8_t* __restrict__ key8, uint32_t n,
                                                                 uint32_t buckets,
                                                                 const uint32_t* __restrict__ offsets,
                                                                 uint32_t* __restrict__ perm) {
  __shared__ uint32_t run[kOrderMaxBuckets];
  __shared__ uint32_t wcnt[kOrderRounds][kOrderWarps][kOrderMaxBuckets];
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  for (uint32_t k = threadIdx.x; k < buckets; k += blockDim.x) run[k] = offsets[(size_t)k * gridDim.x + blockIdx.x];
  for (uint32_t k = threadIdx.x; k < kOrderRounds * kOrderWarps * kOrderMaxBuckets; k += blockDim.x)
    (&wcnt[0][0][0])[k] = 0u;
  const uint32_t base = blockIdx.x * kOrderSpan;
  uint32_t key[kOrderRounds], peers[kOrderRounds];
#pragma unroll
  for (uint32_t r = 0; r < kOrderRounds; ++r) {
    const uint32_t i = base + r * kOrderThreads + threadIdx.x;
    key[r] = i < n ? (uint32_t)key8[i] : kOrderNone;
  }
  __syncthreads();
  // every round's per-warp counts at once, then one pass of placements
#pragma unroll
  for (uint32_t r = 0; r < kOrderRounds; ++r) {
    peers[r] = __match_any_sync(0xffffffffu, key[r]);
    if (key[r] < kOrderNone && lane == (uint32_t)(__ffs(peers[r]) - 1)) wcnt[r][warp][key[r]] = __popc(peers[r]);
  }
  __syncthreads();
  // prefix over (round, warp) per bucket, in place: wcnt[r][w][b] becomes the
  // count of bucket b in earlier rounds and earlier warps of round r
  for (uint32_t b = threadIdx.x; b < buckets; b += blockDim.x) {
    uint32_t acc = run[b];
    for (uint32_t r = 0; r < kOrderRounds; ++r)
      for (uint32_t w = 0; w < kOrderWarps; ++w) {
        const uint32_t c = wcnt[r][w][b];
        wcnt[r][w][b] = acc;
        acc += c;
      }
  }
  __syncthreads();
#pragma unroll
  for (uint32_t r = 0; r < kOrderRounds; ++r) {
    const uint32_t k = key[r];
    if (k < kOrderNone)
      perm[wcnt[r][warp][k] + (uint32_t)__popc(peers[r] & ((1u << lane) - 1u))] = base + r * kOrderThreads + threadIdx.x;
  }
}

size_t ray_order_small_bytes(uint32_t n, int mode) {
  const size_t buckets = mode == RQ_RAY_SORT_OCTANT ? 8 : 64;
  const size_t blocks = (n + kOrderSpan - 1) / kOrderSpan;
  return (((size_t)n + 15) & ~(size_t)15) + 4 * buckets * blocks;
}

void launch_ray_order_small(const float4* rays, uint32_t n, const float* root, int mode, void* scratch,
                            uint32_t* perm, cudaStream_t s) {
  if (n == 0) return;
  const uint32_t buckets = mode == RQ_RAY_SORT_OCTANT ? 8u : 64u;
  const uint32_t blocks = (n + kOrderSpan - 1) / kOrderSpan;
  uint8_t* key8 = static_cast<uint8_t*>(scratch);
  uint32_t* counts = reinterpret_cast<uint32_t*>(key8 + (((size_t)n + 15) & ~(size_t)15));
  count_launch(3);
  k_order_count<<<blocks, kOrderThreads, 0, s>>>(rays, n, root, mode, buckets, key8, counts);
  k_order_scan<<<1, 1024, 0, s>>>(counts, buckets * blocks);
  k_order_scatter<<<blocks, kOrderThreads, 0, s>>>(key8, n, buckets, counts, perm);
}

void launch_ray_keys(const float4* rays, uint32_t n, const float* root, int mode, uint32_t* keys, uint32_t* vals,
                     cudaStream_t s, uint32_t* hist, int passes) {
  if (n == 0) return;
  count_launch();
  uint32_t g = (n + 255) / 256;
  if (hist) {
    const uint32_t cap = 4u * (uint32_t)device_sm_count();  // few blocks: few global histogram atomics
    if (g > cap) g = cap;
  }
  k_ray_keys<<<g, 256, 0, s>>>(rays, n, root, mode, keys, vals, hist, passes);
}

void launch_trace_brute(int kind, int traversal, bool any, const float4* prims, uint32_t n_prims,
                        const float4* rays, uint32_t n, float4* hits, uint32_t* occ,
                        cudaStream_t s) {
  if (n == 0) return;
  count_launch();
  if (kind == kTriangles) {
    if (any) dispatch_brute<kTriangles, true>(traversal, prims, n_prims, rays, n, hits, occ, s);
    else dispatch_brute<kTriangles, false>(traversal, prims, n_prims, rays, n, hits, occ, s);
  } else {
    if (any) dispatch_brute<kSpheres, true>(traversal, prims, n_prims, rays, n, hits, occ, s);
    else dispatch_brute<kSpheres, false>(traversal, prims, n_prims, rays, n, hits, occ, s);
  }
}

}  // namespace rq
