// Per-ray traversal device code shared by the one-structure kernels
// (trace.cu) and the persistent many-structure kernel (trace_batched.cu).
#pragma once
#include <type_traits>

#include "rq_device.cuh"
#include "rq_internal.hpp"

namespace rq {

struct Ray {
  F3 o, d;
  float tmin, tmax;
};

// Rays are read once: streaming loads (evict first), which leave L1 and L2
// to the tree's nodes and primitives.
__device__ __forceinline__ Ray load_ray(const float4* __restrict__ rays, uint32_t r) {
  float4 a = __ldcs(rays + 2 * (size_t)r), b = __ldcs(rays + 2 * (size_t)r + 1);
  return {{a.x, a.y, a.z}, {b.x, b.y, b.z}, a.w, b.w};
}

struct Closest {
  float t;
  uint32_t prim;
  float u, v;
};
// Hits are written once: a streaming store.
__device__ __forceinline__ void store_hit(float4* __restrict__ hits, uint32_t r, const Closest& c) {
  __stcs(hits + r, make_float4(c.t, __uint_as_float(c.prim), c.u, c.v));
}

// Test the primitives of one leaf.  Returns true when an any-hit query is done.
// FAST closest hit (REF = false) keeps the smallest t and, among primitives
// hit at exactly that t, the smallest primitive id, so the result does not
// depend on the order in which a walk meets the primitives.  REF keeps the
// reference's first closest (strict <, castRay main.cpp:343-358).
template <int KIND, bool ANY, bool REF>
__device__ __forceinline__ bool test_leaf(const float4* __restrict__ prims,
                                          const uint32_t* __restrict__ order, uint32_t first,
                                          int count, const Ray& ray, Closest& c) {
  for (int k = 0; k < count; ++k) {
    uint32_t slot = first + (uint32_t)k;
    // closest hit: accept t <= c.t once something is hit (ties go to the smaller id)
    const float bound = (ANY || REF || c.prim == kMiss) ? c.t : nextafterf(c.t, __int_as_float(0x7F800000));
    if (KIND == kTriangles) {
      float4 p0 = __ldg(prims + 3 * (size_t)slot), p1 = __ldg(prims + 3 * (size_t)slot + 1),
             p2 = __ldg(prims + 3 * (size_t)slot + 2);
      float t, u, v;
      if (tri_mt(p0, p1, p2, ray.o, ray.d, ray.tmin, ANY ? ray.tmax : bound, t, u, v)) {
        if (ANY) return true;
        const uint32_t id = __float_as_uint(p0.w);
        if (REF || t < c.t || id < c.prim) c = {t, id, u, v};
      }
    } else {
      float4 s = __ldg(prims + slot);
      if (ANY) {
        float t0, t1, t;
        if (REF ? sphere_ref(s, ray.o, ray.d, t0, t1)
                : sphere_closest(s, ray.o, ray.d, ray.tmin, ray.tmax, false, t))
          return true;
      } else {
        float t;
        if (sphere_closest(s, ray.o, ray.d, ray.tmin, bound, REF, t)) {
          const uint32_t id = __ldg(order + slot);
          if (REF || t < c.t || id < c.prim) c = {t, id, 0.f, 0.f};
        }
      }
    }
  }
  return false;
}

// Primitive tests one leaf visit performs: every primitive for closest hit;
// up to and including the first accepted one for any hit (the oracle's count).
template <int KIND, bool ANY>
__device__ __forceinline__ uint32_t test_count(const float4* __restrict__ prims, uint32_t first, int count,
                                               const Ray& ray) {
  if (!ANY) return (uint32_t)count;
  Closest dummy = {ray.tmax, kMiss, 0.f, 0.f};
  for (int k = 0; k < count; ++k)
    if (test_leaf<KIND, true, false>(prims, nullptr, first + (uint32_t)k, 1, ray, dummy)) return (uint32_t)k + 1;
  return (uint32_t)count;
}

// One 64-byte BVH2 node as two 256-bit loads (nodes are 64-byte aligned).
__device__ __forceinline__ void load_node(const float4* nd, float4& a, float4& b, float4& z, int4& l) {
  uint32_t r[16];
  asm("ld.global.nc.v8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
      : "l"(nd));
  asm("ld.global.nc.v8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
      : "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "l"(nd + 2));
  a = make_float4(__uint_as_float(r[0]), __uint_as_float(r[1]), __uint_as_float(r[2]), __uint_as_float(r[3]));
  b = make_float4(__uint_as_float(r[4]), __uint_as_float(r[5]), __uint_as_float(r[6]), __uint_as_float(r[7]));
  z = make_float4(__uint_as_float(r[8]), __uint_as_float(r[9]), __uint_as_float(r[10]), __uint_as_float(r[11]));
  l = make_int4((int)r[12], (int)r[13], (int)r[14], (int)r[15]);
}

// FAST walk of one ray through a BVH2: near child first, far child on a
// per-thread stack of STACK entries, boxes clipped to [tmin, closest hit].
// EXACT: the exact-sign box test (rays with a zero direction component).
// Returns true when an any-hit query found a hit.
// UNIT: every leaf holds one primitive (LBVH), so a stack entry is the
// 4-byte link alone: half the local-memory footprint, which shares L1 with
// the nodes the walk fetches.
template <int KIND, bool ANY, bool COUNT, int STACK, bool EXACT, bool UNIT = false>
__device__ __forceinline__ bool walk_bvh2_form(const Bvh2View& bvh, const Ray& ray, const SlabRay& sr, Closest& c,
                                               uint32_t& visits, uint32_t& tests, uint32_t* err) {
  float tn;
  const float* rb = bvh.root;
  if (!slab_box<EXACT>(sr, ray.o, rb[0], rb[3], rb[1], rb[4], rb[2], rb[5], ray.tmin, ray.tmax, tn)) return false;
  typename std::conditional<UNIT, int, int2>::type stack[STACK];
  int sp = 0;
  int cur = bvh.n_internal ? 0 : -1;
  int cnt = bvh.n_internal ? 0 : (int)bvh.n_slots;
  // A valid walk visits every node at most once.
  const uint32_t max_steps = 2u * (bvh.n_internal + bvh.n_slots) + 8u;
  uint32_t steps = 0;
  for (;;) {
    if (++steps > max_steps) { atomicOr(err, kErrCorrupt); return false; }
    if (cur >= 0) {
      float4 a, b, z;
      int4 l;
      const float4* nd = bvh.nodes + 4 * (size_t)cur;
      if (ANY) {  // any hit measured 1% faster with four 128-bit loads, closest hit 2% slower
        a = __ldg(nd); b = __ldg(nd + 1); z = __ldg(nd + 2);
        l = __ldg(reinterpret_cast<const int4*>(nd + 3));
      } else {
        load_node(nd, a, b, z, l);
      }
      if (COUNT) ++visits;
      const float tfar = ANY ? ray.tmax : c.t;
      float tl, tr;
      bool hl = slab_box<EXACT>(sr, ray.o, a.x, a.y, a.z, a.w, z.x, z.y, ray.tmin, tfar, tl);
      bool hr = slab_box<EXACT>(sr, ray.o, b.x, b.y, b.z, b.w, z.z, z.w, ray.tmin, tfar, tr);
      if (hl && hr) {
        int2 nearE = make_int2(l.x, l.z), farE = make_int2(l.y, l.w);
        if (tr < tl) { int2 t = nearE; nearE = farE; farE = t; }
        if (sp >= STACK) { atomicOr(err, kErrStackOverflow); return false; }
        if constexpr (UNIT) stack[sp++] = farE.x;
        else stack[sp++] = farE;
        cur = nearE.x;
        cnt = nearE.y;
        continue;
      }
      if (hl) { cur = l.x; cnt = l.z; continue; }
      if (hr) { cur = l.y; cnt = l.w; continue; }
    } else {
      if (UNIT) cnt = 1;
      if (COUNT) tests += test_count<KIND, ANY>(bvh.prims, (uint32_t)(~cur), cnt, ray);
      if (test_leaf<KIND, ANY, false>(bvh.prims, bvh.order, (uint32_t)(~cur), cnt, ray, c)) return true;
    }
    if (sp == 0) return false;
    if constexpr (UNIT) {
      cur = stack[--sp];
    } else {
      const int2 e = stack[--sp];
      cur = e.x;
      cnt = e.y;
    }
  }
}

// walk_bvh2_form with the box test each ray needs.
template <int KIND, bool ANY, bool COUNT, int STACK, bool UNIT = false>
__device__ __forceinline__ bool walk_bvh2(const Bvh2View& bvh, const Ray& ray, Closest& c, uint32_t& visits,
                                          uint32_t& tests, uint32_t* err) {
  const SlabRay sr = slab_ray(ray.o, ray.d);
  return zero_dir(sr) ? walk_bvh2_form<KIND, ANY, COUNT, STACK, true, UNIT>(bvh, ray, sr, c, visits, tests, err)
                      : walk_bvh2_form<KIND, ANY, COUNT, STACK, false, UNIT>(bvh, ray, sr, c, visits, tests, err);
}

// Sum the per-thread visit / test counts of a warp into counters[0..1].
__device__ __forceinline__ void add_counts(unsigned long long* counters, uint32_t visits, uint32_t tests) {
  unsigned long long v = visits, t = tests;
  for (int o = 16; o > 0; o >>= 1) {
    v += __shfl_down_sync(0xffffffffu, v, o);
    t += __shfl_down_sync(0xffffffffu, t, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(counters, v);
    atomicAdd(counters + 1, t);
  }
}

// ---------------------------------------------------------------- 4-wide
// FAST traversal of the collapsed 4-wide BVH: one 128-byte node fetch tests
// up to four child boxes.  The hit children are ordered by a 32-bit key, the
// order-preserving bits of the entry distance with the low two bits replaced
// by the slot (unique keys, so a sorting network gives the same order as any
// sort); the nearest is visited next and the others pushed farthest first.
// Three entries per level at most: 96 stack entries cover trees 64 binary
// levels deep, like the binary walk's 64.
constexpr int kStack4 = 96;

__device__ __forceinline__ uint32_t order_key(float f) {
  uint32_t u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

__device__ __forceinline__ void cswap(uint32_t& a, uint32_t& b) {
  uint32_t lo = min(a, b), hi = max(a, b);
  a = lo;
  b = hi;
}

__device__ __forceinline__ int pick(const int4& v, uint32_t k) {
  return k == 0 ? v.x : k == 1 ? v.y : k == 2 ? v.z : v.w;
}

// FAST walk of one ray through the collapsed 4-wide BVH.  Returns true when
// an any-hit query found a hit.
template <int KIND, bool ANY, bool COUNT, int STACK, bool EXACT>
__device__ __forceinline__ bool walk_bvh4_form(const Bvh4View& bvh, const Ray& ray, Closest& c, uint32_t& visits,
                                               uint32_t& tests, uint32_t* err) {
  const SlabRay sr = slab_ray(ray.o, ray.d);
  float tn;
  const float* rb = bvh.root;
  if (!slab_box<EXACT>(sr, ray.o, rb[0], rb[3], rb[1], rb[4], rb[2], rb[5], ray.tmin, ray.tmax, tn)) return false;
  int2 stack[STACK];
  int sp = 0;
  int cur = bvh.n_binary ? 0 : -1;
  int cnt = bvh.n_binary ? 0 : (int)bvh.n_slots;
  // A valid walk visits every node and leaf at most once.
  const uint32_t max_steps = 2u * (bvh.n_binary + bvh.n_slots) + 8u;
  uint32_t steps = 0;
  for (;;) {
    if (++steps > max_steps) { atomicOr(err, kErrCorrupt); return false; }
    if (cur >= 0) {
      const float4* nd = bvh.nodes + 8 * (size_t)cur;
      const float4 lx = __ldg(nd), hx = __ldg(nd + 1), ly = __ldg(nd + 2), hy = __ldg(nd + 3);
      const float4 lz = __ldg(nd + 4), hz = __ldg(nd + 5);
      const int4 lk = __ldg(reinterpret_cast<const int4*>(nd + 6));
      const int4 ct = __ldg(reinterpret_cast<const int4*>(nd + 7));
      if (COUNT) ++visits;
      const float tfar = ANY ? ray.tmax : c.t;
      float t0, t1, t2, t3;
      uint32_t k0 = 0xFFFFFFFFu, k1 = 0xFFFFFFFFu, k2 = 0xFFFFFFFFu, k3 = 0xFFFFFFFFu;
      if (ct.x >= 0 && slab_box<EXACT>(sr, ray.o, lx.x, hx.x, ly.x, hy.x, lz.x, hz.x, ray.tmin, tfar, t0))
        k0 = (order_key(t0) & ~3u) | 0u;
      if (ct.y >= 0 && slab_box<EXACT>(sr, ray.o, lx.y, hx.y, ly.y, hy.y, lz.y, hz.y, ray.tmin, tfar, t1))
        k1 = (order_key(t1) & ~3u) | 1u;
      if (ct.z >= 0 && slab_box<EXACT>(sr, ray.o, lx.z, hx.z, ly.z, hy.z, lz.z, hz.z, ray.tmin, tfar, t2))
        k2 = (order_key(t2) & ~3u) | 2u;
      if (ct.w >= 0 && slab_box<EXACT>(sr, ray.o, lx.w, hx.w, ly.w, hy.w, lz.w, hz.w, ray.tmin, tfar, t3))
        k3 = (order_key(t3) & ~3u) | 3u;
      // A hit key is at most order_key(+inf) | 3 < 0xFFFFFFFF, so misses sort last.
      const int m = (k0 != 0xFFFFFFFFu) + (k1 != 0xFFFFFFFFu) + (k2 != 0xFFFFFFFFu) + (k3 != 0xFFFFFFFFu);
      if (m > 0) {
        cswap(k0, k1);
        cswap(k2, k3);
        cswap(k0, k2);
        cswap(k1, k3);
        cswap(k1, k2);
        if (sp + m - 1 > STACK) { atomicOr(err, kErrStackOverflow); return false; }
        if (m >= 4) stack[sp++] = make_int2(pick(lk, k3 & 3u), pick(ct, k3 & 3u));
        if (m >= 3) stack[sp++] = make_int2(pick(lk, k2 & 3u), pick(ct, k2 & 3u));
        if (m >= 2) stack[sp++] = make_int2(pick(lk, k1 & 3u), pick(ct, k1 & 3u));
        cur = pick(lk, k0 & 3u);
        cnt = pick(ct, k0 & 3u);
        continue;
      }
    } else {
      if (COUNT) tests += test_count<KIND, ANY>(bvh.prims, (uint32_t)(~cur), cnt, ray);
      if (test_leaf<KIND, ANY, false>(bvh.prims, bvh.order, (uint32_t)(~cur), cnt, ray, c)) return true;
    }
    if (sp == 0) return false;
    int2 e = stack[--sp];
    cur = e.x;
    cnt = e.y;
  }
}

template <int KIND, bool ANY, bool COUNT, int STACK>
__device__ __forceinline__ bool walk_bvh4(const Bvh4View& bvh, const Ray& ray, Closest& c, uint32_t& visits,
                                          uint32_t& tests, uint32_t* err) {
  return zero_dir(slab_ray(ray.o, ray.d)) ? walk_bvh4_form<KIND, ANY, COUNT, STACK, true>(bvh, ray, c, visits, tests, err)
                         : walk_bvh4_form<KIND, ANY, COUNT, STACK, false>(bvh, ray, c, visits, tests, err);
}

// ---------------------------------------------------------------- 8-wide
// FAST traversal of the compressed 8-wide BVH (layout in bvh8.cu).  A node
// visit decodes and tests its (up to) eight child boxes and keeps the hit
// ones as a bit mask in the ray's visiting order (bit k = slot k ^ oct); the
// walk takes children from the mask lowest bit first, and when it descends
// it pushes the node with its remaining mask (one stack entry per level, at
// most 22 for a tree 64 binary levels deep).
constexpr int kStack8 = 32;

// One child plane: fma(S, F(q), pm), F(q) = 1 + q * 2^-15 built by one byte
// permute from byte k of `word` (the builder decodes with these operations).
__device__ __forceinline__ float q8(uint32_t word, int k, float S, float pm) {
  return __fmaf_rn(S, __uint_as_float(__byte_perm(word, 0x3F800000u, 0x7604u | (k << 4))), pm);
}

template <bool EXACT>
__device__ __forceinline__ uint32_t node8_hits(const float4* nd, const SlabRay& sr, F3 o, float tmin, float tfar,
                                               uint32_t oct) {
  uint32_t r[16];
  asm("ld.global.nc.v8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
      : "l"(nd));
  asm("ld.global.nc.v8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
      : "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "l"(nd + 2));
  const float pmx = __uint_as_float(r[0]), pmy = __uint_as_float(r[1]), pmz = __uint_as_float(r[2]);
  const uint32_t hb = r[3];
  const float Sx = __uint_as_float((hb & 0xFFu) << 23), Sy = __uint_as_float((hb & 0xFF00u) << 15),
              Sz = __uint_as_float((hb & 0xFF0000u) << 7);
  const uint32_t valid = hb >> 24;
  uint32_t mask = 0;
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const int k = i & 3, h = i >> 2;
    const float lx = q8(r[4 + h], k, Sx, pmx), hx = q8(r[6 + h], k, Sx, pmx);
    const float ly = q8(r[8 + h], k, Sy, pmy), hy = q8(r[10 + h], k, Sy, pmy);
    const float lz = q8(r[12 + h], k, Sz, pmz), hz = q8(r[14 + h], k, Sz, pmz);
    float tn;
    const bool hit = slab_box<EXACT>(sr, o, lx, hx, ly, hy, lz, hz, tmin, tfar, tn);
    mask |= (hit && (valid >> i & 1u)) ? 1u << (i ^ oct) : 0u;
  }
  return mask;
}

template <int KIND, bool ANY, bool COUNT, int STACK, bool EXACT>
__device__ __forceinline__ bool walk_bvh8_form(const Bvh8View& bvh, const Ray& ray, Closest& c, uint32_t& visits,
                                               uint32_t& tests, uint32_t* err) {
  const SlabRay sr = slab_ray(ray.o, ray.d);
  float tn;
  const float* rb = bvh.root;
  if (!slab_box<EXACT>(sr, ray.o, rb[0], rb[3], rb[1], rb[4], rb[2], rb[5], ray.tmin, ray.tmax, tn)) return false;
  if (bvh.n_binary == 0) {  // the root is one leaf
    if (COUNT) tests += test_count<KIND, ANY>(bvh.prims, 0u, (int)bvh.n_slots, ray);
    return test_leaf<KIND, ANY, false>(bvh.prims, bvh.order, 0u, (int)bvh.n_slots, ray, c);
  }
  const uint32_t oct = (ray.d.x < 0.f ? 1u : 0u) | (ray.d.y < 0.f ? 2u : 0u) | (ray.d.z < 0.f ? 4u : 0u);
  uint2 stack[STACK];
  int sp = 0;
  uint32_t node = 0;
  if (COUNT) ++visits;
  uint32_t mask = node8_hits<EXACT>(bvh.nodes, sr, ray.o, ray.tmin, ANY ? ray.tmax : c.t, oct);
  // A valid walk takes every child (node or leaf) at most once.
  const uint32_t max_steps = 2u * (bvh.n_binary + bvh.n_slots) + 8u;
  uint32_t steps = 0;
  for (;;) {
    if (mask == 0u) {
      if (sp == 0) return false;
      const uint2 e = stack[--sp];
      node = e.x;
      mask = e.y;
    }
    if (++steps > max_steps) { atomicOr(err, kErrCorrupt); return false; }
    const uint32_t k = (uint32_t)__ffs(mask) - 1u;
    mask &= mask - 1u;
    const int2 lc = __ldg(reinterpret_cast<const int2*>(bvh.nodes + 8 * (size_t)node + 4) + (k ^ oct));
    if (lc.y == 0) {
      if (mask) {
        if (sp >= STACK) { atomicOr(err, kErrStackOverflow); return false; }
        stack[sp++] = make_uint2(node, mask);
      }
      node = (uint32_t)lc.x;
      if (COUNT) ++visits;
      mask = node8_hits<EXACT>(bvh.nodes + 8 * (size_t)node, sr, ray.o, ray.tmin, ANY ? ray.tmax : c.t, oct);
    } else {
      if (COUNT) tests += test_count<KIND, ANY>(bvh.prims, (uint32_t)lc.x, lc.y, ray);
      if (test_leaf<KIND, ANY, false>(bvh.prims, bvh.order, (uint32_t)lc.x, lc.y, ray, c)) return true;
    }
  }
}

template <int KIND, bool ANY, bool COUNT, int STACK>
__device__ __forceinline__ bool walk_bvh8(const Bvh8View& bvh, const Ray& ray, Closest& c, uint32_t& visits,
                                          uint32_t& tests, uint32_t* err) {
  return zero_dir(slab_ray(ray.o, ray.d)) ? walk_bvh8_form<KIND, ANY, COUNT, STACK, true>(bvh, ray, c, visits, tests, err)
                                          : walk_bvh8_form<KIND, ANY, COUNT, STACK, false>(bvh, ray, c, visits, tests, err);
}

}  // namespace rq
