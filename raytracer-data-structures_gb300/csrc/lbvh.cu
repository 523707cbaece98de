// LBVH topology and bottom-up refit.
//
// The reference cites Karras' construction (accelerators.h:371,568) but its
// findSplit (accelerators.h:397-449) is discarded and no refit exists; this
// file implements the cited method: Karras 2012, "Maximizing Parallelism in
// the Construction of BVHs, Octrees, and k-d Trees", one thread per internal
// node, then one thread per leaf climbing to the root, the second thread to
// reach a node computing its box.
//
// BVH2 node (64 B, 4 x float4):
//   [0] left  child box (lo.x, hi.x, lo.y, hi.y)
//   [1] right child box (lo.x, hi.x, lo.y, hi.y)
//   [2] (left lo.z, left hi.z, right lo.z, right hi.z)
//   [3] int (left, right, left count, right count); child >= 0 internal,
//       child < 0 leaf holding slots [~child, ~child + count)
#include "rq_device.cuh"
#include "rq_internal.hpp"

namespace rq {
namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ int delta(const uint32_t* __restrict__ k, int64_t n, int64_t i, int64_t j,
                                     uint32_t ki) {
  if (j < 0 || j >= n) return -1;
  uint32_t kj = __ldg(k + j);
  if (ki != kj) return __clz(ki ^ kj);
  return 32 + __clz((uint32_t)i ^ (uint32_t)j);
}

__global__ void __launch_bounds__(kThreads) k_karras(const uint32_t* __restrict__ codes, uint32_t n,
                                                     float4* __restrict__ nodes,
                                                     uint32_t* __restrict__ parent) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t N = n;
  // Neighbour deltas from warp shuffles where the neighbour is in the warp.
  uint32_t ki = i < N ? __ldg(codes + i) : 0u;
  uint32_t kprev = __shfl_up_sync(0xffffffffu, ki, 1);
  uint32_t knext = __shfl_down_sync(0xffffffffu, ki, 1);
  if (i + 1 >= N) return;
  int lane = threadIdx.x & 31;
  if (lane == 0 && i > 0) kprev = __ldg(codes + i - 1);
  if (lane == 31) knext = __ldg(codes + i + 1);
  int dnext = ki != knext ? __clz(ki ^ knext) : 32 + __clz((uint32_t)i ^ (uint32_t)(i + 1));
  int dprev = i == 0 ? -1 : (ki != kprev ? __clz(ki ^ kprev) : 32 + __clz((uint32_t)i ^ (uint32_t)(i - 1)));
  int d = (dnext - dprev) > 0 ? 1 : -1;
  int dmin = d > 0 ? dprev : dnext;
  int64_t lmax = 2;
  while (delta(codes, N, i, i + lmax * d, ki) > dmin) lmax *= 2;
  int64_t l = 0;
  for (int64_t t = lmax / 2; t >= 1; t /= 2)
    if (delta(codes, N, i, i + (l + t) * d, ki) > dmin) l += t;
  int64_t j = i + l * d;
  int dnode = delta(codes, N, i, j, ki);
  int64_t s = 0, t = l;
  do {
    t = (t + 1) >> 1;
    if (delta(codes, N, i, i + (s + t) * d, ki) > dnode) s += t;
  } while (t > 1);
  int64_t gamma = i + s * d + (d < 0 ? -1 : 0);
  int64_t lo = i < j ? i : j, hi = i < j ? j : i;
  int32_t lc = (lo == gamma) ? ~(int32_t)gamma : (int32_t)gamma;
  int32_t rc = (hi == gamma + 1) ? ~(int32_t)(gamma + 1) : (int32_t)(gamma + 1);
  reinterpret_cast<int4*>(nodes)[4 * i + 3] = make_int4(lc, rc, lc < 0 ? 1 : 0, rc < 0 ? 1 : 0);
  parent[lc >= 0 ? lc : (N - 1 + ~lc)] = ((uint32_t)i << 1) | 0u;
  parent[rc >= 0 ? rc : (N - 1 + ~rc)] = ((uint32_t)i << 1) | 1u;
}

struct Box6 {
  float lo[3], hi[3];
};

__device__ __forceinline__ void write_child(float4* nodes, uint32_t node, uint32_t side, const Box6& b) {
  nodes[4 * (size_t)node + side] = make_float4(b.lo[0], b.hi[0], b.lo[1], b.hi[1]);
  reinterpret_cast<float2*>(nodes + 4 * (size_t)node + 2)[side] = make_float2(b.lo[2], b.hi[2]);
}

// Gather primitive `p` into payload slot `slot` (3 float4 per triangle:
// (v0, id), (v1 - v0, 0), (v2 - v0, 0); 1 float4 per sphere) and return its box.
__device__ __forceinline__ Box6 emit_prim(int kind, const float* __restrict__ verts,
                                          const uint32_t* __restrict__ idx,
                                          const float4* __restrict__ sph, uint32_t p,
                                          float4* __restrict__ prims, uint32_t slot) {
  Box6 b;
  if (kind == kTriangles) {
    uint32_t i0 = __ldg(idx + 3 * (size_t)p), i1 = __ldg(idx + 3 * (size_t)p + 1),
             i2 = __ldg(idx + 3 * (size_t)p + 2);
    F3 a = {__ldg(verts + 3 * (size_t)i0), __ldg(verts + 3 * (size_t)i0 + 1), __ldg(verts + 3 * (size_t)i0 + 2)};
    F3 c1 = {__ldg(verts + 3 * (size_t)i1), __ldg(verts + 3 * (size_t)i1 + 1), __ldg(verts + 3 * (size_t)i1 + 2)};
    F3 c2 = {__ldg(verts + 3 * (size_t)i2), __ldg(verts + 3 * (size_t)i2 + 1), __ldg(verts + 3 * (size_t)i2 + 2)};
    F3 e1 = sub_rn(c1, a), e2 = sub_rn(c2, a);
    float4* q = prims + 3 * (size_t)slot;
    q[0] = make_float4(a.x, a.y, a.z, __uint_as_float(p));
    q[1] = make_float4(e1.x, e1.y, e1.z, 0.f);
    q[2] = make_float4(e2.x, e2.y, e2.z, 0.f);
    b.lo[0] = fminf(fminf(a.x, c1.x), c2.x); b.hi[0] = fmaxf(fmaxf(a.x, c1.x), c2.x);
    b.lo[1] = fminf(fminf(a.y, c1.y), c2.y); b.hi[1] = fmaxf(fmaxf(a.y, c1.y), c2.y);
    b.lo[2] = fminf(fminf(a.z, c1.z), c2.z); b.hi[2] = fmaxf(fmaxf(a.z, c1.z), c2.z);
  } else {
    float4 s = __ldg(sph + p);
    prims[slot] = s;
    // centre -/+ radius, main.cpp:686-688
    b.lo[0] = __fsub_rn(s.x, s.w); b.lo[1] = __fsub_rn(s.y, s.w); b.lo[2] = __fsub_rn(s.z, s.w);
    b.hi[0] = __fadd_rn(s.x, s.w); b.hi[1] = __fadd_rn(s.y, s.w); b.hi[2] = __fadd_rn(s.z, s.w);
  }
  return b;
}

__global__ void __launch_bounds__(kThreads) k_refit(int kind, const float* __restrict__ verts,
                                                    const uint32_t* __restrict__ idx,
                                                    const float4* __restrict__ sph,
                                                    const uint32_t* __restrict__ order, uint32_t n,
                                                    float4* nodes, const uint32_t* __restrict__ parent,
                                                    uint32_t* flags, float4* __restrict__ prims,
                                                    float* __restrict__ root_out, uint32_t* err) {
  uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  Box6 b = emit_prim(kind, verts, idx, sph, __ldg(order + j), prims, j);
  if (n == 1) {
    for (int k = 0; k < 3; ++k) { root_out[k] = b.lo[k]; root_out[3 + k] = b.hi[k]; }
    return;
  }
  uint32_t pw = __ldg(parent + (n - 1) + j);
  for (int level = 0;; ++level) {
    if (level >= 128) { atomicOr(err, kErrCorrupt); return; }  // Karras trees are at most 64 deep
    uint32_t node = pw >> 1, side = pw & 1u;
    write_child(nodes, node, side, b);
    __threadfence();
    if (atomicAdd(flags + node, 1u) == 0u) return;  // the sibling's thread finishes this node
    __threadfence();
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
    pw = __ldg(parent + node);
  }
}

__global__ void __launch_bounds__(kThreads) k_prims_by_id(int kind, const float* __restrict__ verts,
                                                          const uint32_t* __restrict__ idx,
                                                          const float4* __restrict__ sph, uint32_t n,
                                                          float4* __restrict__ prims,
                                                          float* __restrict__ aabb6) {
  uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  Box6 b = emit_prim(kind, verts, idx, sph, p, prims, p);
  if (aabb6)
    for (int k = 0; k < 3; ++k) { aabb6[6 * (size_t)p + k] = b.lo[k]; aabb6[6 * (size_t)p + 3 + k] = b.hi[k]; }
}

}  // namespace

void launch_karras(const uint32_t* sorted_codes, uint32_t n, float4* nodes, uint32_t* parent,
                   cudaStream_t s) {
  if (n < 2) return;
  uint32_t g = (n - 1 + kThreads - 1) / kThreads;
  count_launch();
  k_karras<<<g, kThreads, 0, s>>>(sorted_codes, n, nodes, parent);
}

void launch_refit(int kind, const float* verts, const uint32_t* idx, const float4* sph,
                  const uint32_t* order, uint32_t n, float4* nodes, const uint32_t* parent,
                  uint32_t* flags, float4* prims, float* root_out, uint32_t* err, cudaStream_t s) {
  if (n == 0) return;
  count_launch();
  k_refit<<<(n + kThreads - 1) / kThreads, kThreads, 0, s>>>(kind, verts, idx, sph, order, n, nodes,
                                                             parent, flags, prims, root_out, err);
}

void launch_prims_by_id(int kind, const float* verts, const uint32_t* idx, const float4* sph,
                        uint32_t n, float4* prims, float* aabb6, cudaStream_t s) {
  if (n == 0) return;
  count_launch();
  k_prims_by_id<<<(n + kThreads - 1) / kThreads, kThreads, 0, s>>>(kind, verts, idx, sph, n, prims,
                                                                   aabb6);
}

}  // namespace rq

namespace rq {
namespace {

__global__ void __launch_bounds__(kThreads) k_prims_gather(int kind, const float* __restrict__ verts,
                                                           const uint32_t* __restrict__ idx,
                                                           const float4* __restrict__ sph,
                                                           const uint32_t* __restrict__ order, uint32_t n,
                                                           float4* __restrict__ prims) {
  uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  emit_prim(kind, verts, idx, sph, __ldg(order + j), prims, j);
}

}  // namespace

void launch_prims_gather(int kind, const float* verts, const uint32_t* idx, const float4* sph,
                         const uint32_t* order, uint32_t n, float4* prims, cudaStream_t s) {
  if (n == 0) return;
  count_launch();
  k_prims_gather<<<(n + kThreads - 1) / kThreads, kThreads, 0, s>>>(kind, verts, idx, sph, order, n, prims);
}

}  // namespace rq
