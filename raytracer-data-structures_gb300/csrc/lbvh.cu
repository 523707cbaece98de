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
#include "lbvh_device.cuh"

namespace rq {
namespace {

constexpr int kThreads = 256;

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
  const int2 ch = karras_children(codes, N, i, ki, dprev, dnext);
  const int32_t lc = ch.x, rc = ch.y;
  reinterpret_cast<int4*>(nodes)[4 * i + 3] = make_int4(lc, rc, lc < 0 ? 1 : 0, rc < 0 ? 1 : 0);
  parent[lc >= 0 ? lc : (N - 1 + ~lc)] = ((uint32_t)i << 1) | 0u;
  parent[rc >= 0 ? rc : (N - 1 + ~rc)] = ((uint32_t)i << 1) | 1u;
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
  refit_climb(n, j, b, nodes, parent, flags, root_out, err);
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
