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
#include "trace_device.cuh"

namespace rq {
namespace {

constexpr int kThreads = 128;

// perm (may be null): thread i traces ray perm[i] and writes that ray's result
// (a reordering for coherence that leaves every result where the caller
// expects it).  With perm, any-hit bits are set with atomicOr on a zeroed array.
template <int KIND, bool ANY, bool COUNT = false>
__global__ void __launch_bounds__(kThreads) k_trace_fast(Bvh2View bvh, const float4* __restrict__ rays,
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
    occluded = walk_bvh2<KIND, ANY, COUNT, kStackSize>(bvh, ray, c, visits, tests, err);
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

template <int KIND, bool ANY>
void dispatch_bvh4(const Bvh4View& v, const float4* rays, uint32_t n, float4* hits, uint32_t* occ,
                   uint32_t* err, const uint32_t* perm, unsigned long long* counters, cudaStream_t s) {
  uint32_t g = (n + kThreads - 1) / kThreads;
  if (counters)
    k_trace_bvh4<KIND, ANY, true><<<g, kThreads, 0, s>>>(v, rays, n, hits, occ, err, perm, counters);
  else
    k_trace_bvh4<KIND, ANY, false><<<g, kThreads, 0, s>>>(v, rays, n, hits, occ, err, perm, nullptr);
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
                   uint32_t* occ, uint32_t* err, const uint32_t* perm, cudaStream_t s) {
  uint32_t g = (n + kThreads - 1) / kThreads;
  if (traversal == RQ_TRAVERSAL_REFERENCE)
    k_trace_ref<KIND, ANY><<<g, kThreads, 0, s>>>(v, rays, n, hits, occ, err);
  else
    k_trace_fast<KIND, ANY, false><<<g, kThreads, 0, s>>>(v, rays, n, hits, occ, err, nullptr, perm);
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
                       const uint32_t* perm) {
  if (n == 0) return;
  count_launch();
  if (traversal == RQ_TRAVERSAL_REFERENCE) perm = nullptr;
  if (any && perm) cudaMemsetAsync(occ, 0, (size_t)((n + 31) / 32) * 4, s);
  if (kind == kTriangles) {
    if (any) dispatch_bvh2<kTriangles, true>(traversal, v, rays, n, hits, occ, err, perm, s);
    else dispatch_bvh2<kTriangles, false>(traversal, v, rays, n, hits, occ, err, perm, s);
  } else {
    if (any) dispatch_bvh2<kSpheres, true>(traversal, v, rays, n, hits, occ, err, perm, s);
    else dispatch_bvh2<kSpheres, false>(traversal, v, rays, n, hits, occ, err, perm, s);
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

// Sort key of a ray for coherent tracing: the direction octant in the top
// three bits, then a 27-bit Morton code of the origin inside the scene box.
__global__ void __launch_bounds__(256) k_ray_keys(const float4* __restrict__ rays, uint32_t n,
                                                  const float* __restrict__ root, uint32_t* __restrict__ keys,
                                                  uint32_t* __restrict__ vals) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float4 a = __ldg(rays + 2 * (size_t)i), b = __ldg(rays + 2 * (size_t)i + 1);
  const float o[3] = {a.x, a.y, a.z};
  uint32_t q[3];
  for (int k = 0; k < 3; ++k) {
    float lo = root[k], ext = root[3 + k] - root[k];
    float u = ext > 0.f ? (o[k] - lo) / ext : 0.f;
    u = fminf(fmaxf(u * 512.f, 0.f), 511.f);
    q[k] = (uint32_t)u;
  }
  auto spread = [](uint32_t v) {  // 9 bits -> every third bit
    v = (v | (v << 16)) & 0x030000FFu;
    v = (v | (v << 8)) & 0x0300F00Fu;
    v = (v | (v << 4)) & 0x030C30C3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
  };
  const uint32_t oct = (b.x < 0.f ? 4u : 0u) | (b.y < 0.f ? 2u : 0u) | (b.z < 0.f ? 1u : 0u);
  keys[i] = (oct << 27) | (spread(q[0]) << 2) | (spread(q[1]) << 1) | spread(q[2]);
  vals[i] = i;
}

void launch_ray_keys(const float4* rays, uint32_t n, const float* root, uint32_t* keys, uint32_t* vals,
                     cudaStream_t s) {
  if (n == 0) return;
  count_launch();
  k_ray_keys<<<(n + 255) / 256, 256, 0, s>>>(rays, n, root, keys, vals);
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
