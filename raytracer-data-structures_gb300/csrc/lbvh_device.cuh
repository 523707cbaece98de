// Device helpers shared by the single-scene LBVH kernels (morton.cu,
// lbvh.cu) and the batched ones (batch.cu), so that a batched build performs
// exactly the operations of a single build.
#pragma once
#include "rq_device.cuh"
#include "rq_internal.hpp"

namespace rq {

// Scene box from the ordered-int accumulators: lo and extent per axis.
__device__ __forceinline__ void bounds_from(const int32_t* lohi, float* lo, float* ext) {
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    lo[k] = ordered_to_float(lohi[k]);
    float hi = ordered_to_float(lohi[3 + k]);
    ext[k] = __fsub_rn(hi, lo[k]);
  }
}

// Cube normalisation (RQ_MORTON_SCENE_CUBE): every axis scaled by the
// largest extent of the scene box, so the curve splits space evenly on flat
// or elongated scenes.
__device__ __forceinline__ void cube_extent(float* ext) {
  const float e = fmaxf(fmaxf(ext[0], ext[1]), ext[2]);
  ext[0] = ext[1] = ext[2] = e;
}

// (c - lo) / ext per axis, 0 where the extent is 0.
__device__ __forceinline__ uint32_t code_scene(F3 c, const float* lo, const float* ext) {
  float q0 = ext[0] > 0.f ? __fdiv_rn(__fsub_rn(c.x, lo[0]), ext[0]) : 0.f;
  float q1 = ext[1] > 0.f ? __fdiv_rn(__fsub_rn(c.y, lo[1]), ext[1]) : 0.f;
  float q2 = ext[2] > 0.f ? __fdiv_rn(__fsub_rn(c.z, lo[2]), ext[2]) : 0.f;
  return morton3d(q0, q1, q2);
}

// Triangle centroid ((v0 + v1) + v2) / 3 per axis.
__device__ __forceinline__ F3 tri_centroid(const float* __restrict__ verts, const uint32_t* __restrict__ idx,
                                           uint32_t i) {
  uint32_t i0 = __ldg(idx + 3 * (size_t)i), i1 = __ldg(idx + 3 * (size_t)i + 1), i2 = __ldg(idx + 3 * (size_t)i + 2);
  const float* a = verts + 3 * (size_t)i0;
  const float* b = verts + 3 * (size_t)i1;
  const float* c = verts + 3 * (size_t)i2;
  F3 cen;
  cen.x = __fdiv_rn(__fadd_rn(__fadd_rn(__ldg(a), __ldg(b)), __ldg(c)), 3.0f);
  cen.y = __fdiv_rn(__fadd_rn(__fadd_rn(__ldg(a + 1), __ldg(b + 1)), __ldg(c + 1)), 3.0f);
  cen.z = __fdiv_rn(__fadd_rn(__fadd_rn(__ldg(a + 2), __ldg(b + 2)), __ldg(c + 2)), 3.0f);
  return cen;
}

// The same from the packed copies (one 16-byte load per triangle and per
// vertex instead of twelve scattered 4-byte loads).
__device__ __forceinline__ F3 tri_centroid(const float4* __restrict__ verts4, const uint4* __restrict__ idx4,
                                           uint32_t i) {
  const uint4 t = __ldg(idx4 + i);
  const float4 a = __ldg(verts4 + t.x), b = __ldg(verts4 + t.y), c = __ldg(verts4 + t.z);
  F3 cen;
  cen.x = __fdiv_rn(__fadd_rn(__fadd_rn(a.x, b.x), c.x), 3.0f);
  cen.y = __fdiv_rn(__fadd_rn(__fadd_rn(a.y, b.y), c.y), 3.0f);
  cen.z = __fdiv_rn(__fadd_rn(__fadd_rn(a.z, b.z), c.z), 3.0f);
  return cen;
}

// Karras 2012 prefix length between sorted codes i and j with the index
// tiebreak; -1 outside the keys.  32-bit indices: scenes hold fewer than
// 2^30 primitives.
__device__ __forceinline__ int delta32(const uint32_t* __restrict__ k, int n, int i, int j, uint32_t ki) {
  if (j < 0 || j >= n) return -1;
  const uint32_t kj = __ldg(k + j);
  return ki != kj ? __clz(ki ^ kj) : 32 + __clz((uint32_t)i ^ (uint32_t)j);
}

// Largest x in [lo, hi) with delta(i, i + x * d) > bound, given that it
// holds at lo and fails at hi (the common prefix of sorted keys shrinks with
// distance, so the predicate is monotone).  The whole warp tests 32 points
// per round: ranges of a million keys take four rounds instead of the
// twenty dependent loads of a binary search.
__device__ __forceinline__ int warp_search(const uint32_t* __restrict__ codes, int n, int i, uint32_t ki, int d,
                                           int bound, int lo, int hi) {
  const int lane = threadIdx.x & 31;
  for (int round = 0; round < 16 && hi - lo > 1; ++round) {
    const int span = hi - lo, q = span / 33, r = span % 33;
    const int p = lo + q * (lane + 1) + (r * (lane + 1)) / 33;  // lo + floor(span * (lane + 1) / 33)
    const bool t = p <= lo ? true : p >= hi ? false : delta32(codes, n, i, i + p * d, ki) > bound;
    const uint32_t yes = __ballot_sync(0xffffffffu, t);  // a prefix of the lanes
    if (yes == 0u) {  // the answer lies below lane 0's point
      hi = __shfl_sync(0xffffffffu, p, 0);
      continue;
    }
    const int last = 31 - __clz(yes);
    const int nlo = __shfl_sync(0xffffffffu, p, last);
    const int nhi = __shfl_sync(0xffffffffu, p, last < 31 ? last + 1 : 31);
    lo = nlo;
    if (last < 31) hi = nhi;
  }
  return lo;
}

constexpr int kSoloSpan = 64;  // longer ranges are searched by the warp

// Internal node i (0 <= i < n - 1) of the radix tree over the n sorted codes
// at `codes` (Karras 2012), given the neighbour deltas: (left, right, first
// leaf, last leaf), children encoded as ~slot for leaves.  A lane searches
// ranges and splits of up to kSoloSpan keys alone; longer ones are searched
// by the whole warp, one lane at a time, with that lane's code array and key
// count broadcast (lanes of one warp may belong to different key sets).  All
// 32 lanes must call it; inactive lanes only take part in the searches.
__device__ __forceinline__ int4 karras_node_warp(const uint32_t* __restrict__ codes, int n, int i, uint32_t ki,
                                                 int dprev, int dnext, bool active) {
  const int lane = threadIdx.x & 31;
  int d = 1, dmin = 0, l = 0;
  bool wide = false;
  if (active) {
    d = (dnext - dprev) > 0 ? 1 : -1;
    dmin = d > 0 ? dprev : dnext;
    int lmax = 2;
    while (delta32(codes, n, i, i + lmax * d, ki) > dmin) {
      lmax *= 2;
      if (lmax > kSoloSpan) { wide = true; break; }
    }
    if (!wide)
      for (int t = lmax / 2; t >= 1; t /= 2)
        if (delta32(codes, n, i, i + (l + t) * d, ki) > dmin) l += t;
  }
  const unsigned long long cw = reinterpret_cast<unsigned long long>(codes);
  // Range end of the wide lanes, one lane at a time, by the whole warp.
  for (uint32_t pend = __ballot_sync(0xffffffffu, wide); pend; pend &= pend - 1) {
    const int src = __ffs(pend) - 1;
    const uint32_t* sc = reinterpret_cast<const uint32_t*>(__shfl_sync(0xffffffffu, cw, src));
    const int sn = __shfl_sync(0xffffffffu, n, src);
    const int si = __shfl_sync(0xffffffffu, i, src);
    const uint32_t sk = __shfl_sync(0xffffffffu, ki, src);
    const int sd = __shfl_sync(0xffffffffu, d, src);
    const int sb = __shfl_sync(0xffffffffu, dmin, src);
    const int lim = (sd > 0 ? sn - 1 - si : si) + 1;  // first distance outside the keys
    const int r = warp_search(sc, sn, si, sk, sd, sb, kSoloSpan, lim);
    if (lane == src) l = r;
  }
  const int j = i + l * d;
  const int dnode = active ? delta32(codes, n, i, j, ki) : 0;
  // Split: the largest s < l with delta(i, i + s d) > dnode.
  int sp = 0;
  const bool wide_split = active && l > kSoloSpan;
  if (active && !wide_split) {
    int t = l;
    do {
      t = (t + 1) >> 1;
      if (delta32(codes, n, i, i + (sp + t) * d, ki) > dnode) sp += t;
    } while (t > 1);
  }
  for (uint32_t pend = __ballot_sync(0xffffffffu, wide_split); pend; pend &= pend - 1) {
    const int src = __ffs(pend) - 1;
    const uint32_t* sc = reinterpret_cast<const uint32_t*>(__shfl_sync(0xffffffffu, cw, src));
    const int sn = __shfl_sync(0xffffffffu, n, src);
    const int si = __shfl_sync(0xffffffffu, i, src);
    const uint32_t sk = __shfl_sync(0xffffffffu, ki, src);
    const int sd = __shfl_sync(0xffffffffu, d, src);
    const int sb = __shfl_sync(0xffffffffu, dnode, src);
    const int sl = __shfl_sync(0xffffffffu, l, src);
    const int r = warp_search(sc, sn, si, sk, sd, sb, 0, sl);
    if (lane == src) sp = r;
  }
  const int gamma = i + sp * d + (d < 0 ? -1 : 0);
  const int lo = i < j ? i : j, hi = i < j ? j : i;
  const int32_t lc = (lo == gamma) ? ~gamma : gamma;
  const int32_t rc = (hi == gamma + 1) ? ~(gamma + 1) : gamma + 1;
  return make_int4(lc, rc, lo, hi);
}

// Refit decomposition of an LBVH: treelets are the maximal subtrees of at
// most kTreeletSpan leaves (each a contiguous slot range), refitted one per
// block in shared memory; the nodes above them (top nodes, more than
// kTreeletSpan leaves: about 2n / kTreeletSpan of them) are refitted by one
// block when there are at most kRefitTopCap, else by device-scope climbing.
constexpr uint32_t kTreeletSpan = 2048;
constexpr uint32_t kTreeletThreads = 1024;
constexpr uint32_t kTreeletBlocksPerSM = 2;  // 2 x 112 KB of shared memory, 32 registers per thread
constexpr uint32_t kRefitTopCap = 2048;
constexpr uint32_t kRefitTopThreads = 1024;
constexpr uint32_t kTopMark = 0x80000000u;
constexpr uint32_t kSlotMask = 0x7FFFFFFFu;
constexpr uint32_t kTreeletRight = 0x80000000u;  // treelet record: the subtree is a right child

// Atomic add with acquire-release semantics at device scope: the adding
// thread's earlier stores are visible to a thread whose own add observes
// this one, and that thread's later loads see them (one round trip instead
// of fence + add + fence).
__device__ __forceinline__ uint32_t atomic_add_acq_rel(uint32_t* p, uint32_t v) {
  uint32_t old;
  asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
  return old;
}

struct Box6 {
  float lo[3], hi[3];
};

__device__ __forceinline__ void write_child(float4* nodes, uint32_t node, uint32_t side, const Box6& b) {
  nodes[4 * (size_t)node + side] = make_float4(b.lo[0], b.hi[0], b.lo[1], b.hi[1]);
  reinterpret_cast<float2*>(nodes + 4 * (size_t)node + 2)[side] = make_float2(b.lo[2], b.hi[2]);
}

// Payload of triangle p in slot `slot` (3 float4: (v0, id), (v1 - v0, 0),
// (v2 - v0, 0)) and its box.
__device__ __forceinline__ Box6 emit_tri(F3 a, F3 c1, F3 c2, uint32_t p, float4* __restrict__ prims,
                                         uint32_t slot) {
  Box6 b;
  F3 e1 = sub_rn(c1, a), e2 = sub_rn(c2, a);
  float4* q = prims + 3 * (size_t)slot;
  q[0] = make_float4(a.x, a.y, a.z, __uint_as_float(p));
  q[1] = make_float4(e1.x, e1.y, e1.z, 0.f);
  q[2] = make_float4(e2.x, e2.y, e2.z, 0.f);
  b.lo[0] = fminf(fminf(a.x, c1.x), c2.x); b.hi[0] = fmaxf(fmaxf(a.x, c1.x), c2.x);
  b.lo[1] = fminf(fminf(a.y, c1.y), c2.y); b.hi[1] = fmaxf(fmaxf(a.y, c1.y), c2.y);
  b.lo[2] = fminf(fminf(a.z, c1.z), c2.z); b.hi[2] = fmaxf(fmaxf(a.z, c1.z), c2.z);
  return b;
}

// Sphere p into slot `slot` (1 float4) and its box: centre -/+ radius
// (main.cpp:686-688).
__device__ __forceinline__ Box6 emit_sphere(const float4* __restrict__ sph, uint32_t p, float4* __restrict__ prims,
                                            uint32_t slot) {
  Box6 b;
  float4 s = __ldg(sph + p);
  prims[slot] = s;
  b.lo[0] = __fsub_rn(s.x, s.w); b.lo[1] = __fsub_rn(s.y, s.w); b.lo[2] = __fsub_rn(s.z, s.w);
  b.hi[0] = __fadd_rn(s.x, s.w); b.hi[1] = __fadd_rn(s.y, s.w); b.hi[2] = __fadd_rn(s.z, s.w);
  return b;
}

// Gather primitive `p` into payload slot `slot` and return its box.
__device__ __forceinline__ Box6 emit_prim(int kind, const float* __restrict__ verts,
                                          const uint32_t* __restrict__ idx,
                                          const float4* __restrict__ sph, uint32_t p,
                                          float4* __restrict__ prims, uint32_t slot) {
  if (kind != kTriangles) return emit_sphere(sph, p, prims, slot);
  uint32_t i0 = __ldg(idx + 3 * (size_t)p), i1 = __ldg(idx + 3 * (size_t)p + 1), i2 = __ldg(idx + 3 * (size_t)p + 2);
  F3 a = {__ldg(verts + 3 * (size_t)i0), __ldg(verts + 3 * (size_t)i0 + 1), __ldg(verts + 3 * (size_t)i0 + 2)};
  F3 c1 = {__ldg(verts + 3 * (size_t)i1), __ldg(verts + 3 * (size_t)i1 + 1), __ldg(verts + 3 * (size_t)i1 + 2)};
  F3 c2 = {__ldg(verts + 3 * (size_t)i2), __ldg(verts + 3 * (size_t)i2 + 1), __ldg(verts + 3 * (size_t)i2 + 2)};
  return emit_tri(a, c1, c2, p, prims, slot);
}

// The same from the packed copies.
__device__ __forceinline__ Box6 emit_prim(int kind, const float4* __restrict__ verts4,
                                          const uint4* __restrict__ idx4,
                                          const float4* __restrict__ sph, uint32_t p,
                                          float4* __restrict__ prims, uint32_t slot) {
  if (kind != kTriangles) return emit_sphere(sph, p, prims, slot);
  const uint4 t = __ldg(idx4 + p);
  const float4 a = __ldg(verts4 + t.x), c1 = __ldg(verts4 + t.y), c2 = __ldg(verts4 + t.z);
  return emit_tri({a.x, a.y, a.z}, {c1.x, c1.y, c1.z}, {c2.x, c2.y, c2.z}, p, prims, slot);
}

// Bottom-up refit from leaf slot j: write the leaf box into its parent, then
// climb while this thread is the second to arrive at a node (atomic count per
// node), computing the node's box from its two children.  Writes the root
// box when it reaches node 0.  parent: internal nodes [0, n-1), leaves at
// (n - 1) + j, each (node << 1) | side.
__device__ __forceinline__ void refit_climb(uint32_t n, uint32_t j, Box6 b, float4* nodes,
                                            const uint32_t* __restrict__ parent, uint32_t* flags,
                                            float* __restrict__ root_out, uint32_t* err) {
  if (n == 1) {
    for (int k = 0; k < 3; ++k) { root_out[k] = b.lo[k]; root_out[3 + k] = b.hi[k]; }
    return;
  }
  uint32_t pw = __ldg(parent + (n - 1) + j);
  for (int level = 0;; ++level) {
    if (level >= 128) { atomicOr(err, kErrCorrupt); return; }  // Karras trees are at most 64 deep
    uint32_t node = pw >> 1, side = pw & 1u;
    const uint32_t up = node ? __ldg(parent + node) : 0u;  // read-only here: fetch beside the add
    write_child(nodes, node, side, b);
    if (atomic_add_acq_rel(flags + node, 1u) == 0u) return;  // the sibling's thread finishes this node
    float4 a = __ldcg(nodes + 4 * (size_t)node);
    float4 c = __ldcg(nodes + 4 * (size_t)node + 1);
    float4 z = __ldcg(nodes + 4 * (size_t)node + 2);
    b.lo[0] = fminf(a.x, c.x); b.hi[0] = fmaxf(a.y, c.y);
    b.lo[1] = fminf(a.z, c.z); b.hi[1] = fmaxf(a.w, c.w);
    b.lo[2] = fminf(z.x, z.z); b.hi[2] = fmaxf(z.y, z.w);
    if (node == 0) {
      for (int k = 0; k < 3; ++k) { root_out[k] = b.lo[k]; root_out[3 + k] = b.hi[k]; }
      return;
    }
    pw = up;
  }
}

}  // namespace rq
