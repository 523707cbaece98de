// LBVH topology and bottom-up refit.
//
// The reference cites Karras' construction (accelerators.h:371,568) but its
// findSplit (accelerators.h:397-449) is discarded and no refit exists; this
// file implements the cited method: Karras 2012, "Maximizing Parallelism in
// the Construction of BVHs, Octrees, and k-d Trees", one thread per internal
// node, then a bottom-up refit in which the second of a node's two children
// to finish computes the node's box.  The refit runs by treelets (maximal
// subtrees of at most kTreeletSpan leaves, one block each, in shared memory)
// and then the top nodes above them (one block), so no level of the climb
// waits on device-scope memory unless the top nodes exceed that block.
//
// BVH2 node (64 B, 4 x float4):
//   [0] left  child box (lo.x, hi.x, lo.y, hi.y)
//   [1] right child box (lo.x, hi.x, lo.y, hi.y)
//   [2] (left lo.z, left hi.z, right lo.z, right hi.z)
//   [3] int (left, right, left count, right count); child >= 0 internal,
//       child < 0 leaf holding slots [~child, ~child + count)
#include <atomic>

#include "lbvh_device.cuh"

namespace rq {
namespace {

constexpr int kThreads = 256;
static_assert(kRefitTopCap == kRefitTopCapHost, "top list capacity");


// Internal node i of the radix tree (one thread per node; Karras 2012).
// Also lays out the refit: a node of more than kTreeletSpan leaves is a top
// node (mark[i] = kTopMark | slot, top[slot] = i for slots below
// kRefitTopCap, count[0] = their number, possibly above the cap) and lists
// its children of at most kTreeletSpan leaves as treelets ({first slot,
// leaf count | kTreeletRight for a right child}, count[1] = their number);
// a root of at most kTreeletSpan leaves is the one treelet.
__global__ void __launch_bounds__(kThreads) k_karras(const uint32_t* __restrict__ codes, uint32_t n_,
                                                     float4* __restrict__ nodes,
                                                     uint32_t* __restrict__ parent, uint32_t* __restrict__ mark,
                                                     uint32_t* __restrict__ top, uint32_t* __restrict__ treelets,
                                                     uint32_t* count) {
  const int n = (int)n_;
  const int i = (int)(blockIdx.x * blockDim.x + threadIdx.x);
  // Neighbour deltas from warp shuffles where the neighbour is in the warp.
  const uint32_t ki = i < n ? __ldg(codes + i) : 0u;
  uint32_t kprev = __shfl_up_sync(0xffffffffu, ki, 1);
  uint32_t knext = __shfl_down_sync(0xffffffffu, ki, 1);
  const bool active = i + 1 < n;  // every lane stays for the warp searches
  const int lane = threadIdx.x & 31;
  int dprev = -1, dnext = -1;
  if (active) {
    if (lane == 0 && i > 0) kprev = __ldg(codes + i - 1);
    if (lane == 31) knext = __ldg(codes + i + 1);
    dnext = ki != knext ? __clz(ki ^ knext) : 32 + __clz((uint32_t)i ^ (uint32_t)(i + 1));
    dprev = i == 0 ? -1 : (ki != kprev ? __clz(ki ^ kprev) : 32 + __clz((uint32_t)i ^ (uint32_t)(i - 1)));
  }
  const int4 nd = karras_node_warp(codes, n, i, ki, dprev, dnext, active);
  if (!active) return;
  const int32_t lc = nd.x, rc = nd.y;
  const int lo = nd.z, hi = nd.w;
  const int gamma = lc >= 0 ? lc : ~lc;  // the left child ends at the split
  reinterpret_cast<int4*>(nodes)[4 * (size_t)i + 3] = make_int4(lc, rc, lc < 0 ? 1 : 0, rc < 0 ? 1 : 0);
  parent[lc >= 0 ? lc : (n - 1 + ~lc)] = ((uint32_t)i << 1) | 0u;
  parent[rc >= 0 ? rc : (n - 1 + ~rc)] = ((uint32_t)i << 1) | 1u;
  uint32_t m = 0u;
  const uint32_t span = (uint32_t)(hi - lo) + 1u;
  uint2* tl = reinterpret_cast<uint2*>(treelets);
  if (span > kTreeletSpan) {
    const uint32_t slot = atomicAdd(count, 1u);
    if (slot < kRefitTopCap) top[slot] = (uint32_t)i;
    m = kTopMark | (slot & kSlotMask);
    const uint32_t ls = (uint32_t)(gamma - lo) + 1u, rs = (uint32_t)(hi - gamma);
    if (ls <= kTreeletSpan) tl[atomicAdd(count + 1, 1u)] = make_uint2((uint32_t)lo, ls);
    if (rs <= kTreeletSpan) tl[atomicAdd(count + 1, 1u)] = make_uint2((uint32_t)gamma + 1u, rs | kTreeletRight);
  } else if (i == 0) {
    tl[atomicAdd(count + 1, 1u)] = make_uint2(0u, span | kTreeletRight);  // the root's index is its first slot
  }
  mark[i] = m;
}

struct RefitShared {
  float box[kTreeletSpan][2][6];  // child boxes of the treelet's internal nodes, by index - first slot
  uint32_t up[kTreeletSpan];      // their parent words
  uint32_t arrived[kTreeletSpan]; // children finished (2: the node is finished), + their heights << 8
  uint32_t next;                  // the block's next treelet
};

// Triangle p's payload (3 float4: (v0, id), (v1 - v0, 0), (v2 - v0, 0)) in
// q and its box, from the packed copies.
__device__ __forceinline__ Box6 tri_payload(const float4* __restrict__ verts4, const uint4* __restrict__ idx4,
                                            uint32_t p, float4 q[3]) {
  const uint4 t = __ldg(idx4 + p);
  const float4 a = __ldg(verts4 + t.x), c1 = __ldg(verts4 + t.y), c2 = __ldg(verts4 + t.z);
  const F3 e1 = sub_rn({c1.x, c1.y, c1.z}, {a.x, a.y, a.z}), e2 = sub_rn({c2.x, c2.y, c2.z}, {a.x, a.y, a.z});
  q[0] = make_float4(a.x, a.y, a.z, __uint_as_float(p));
  q[1] = make_float4(e1.x, e1.y, e1.z, 0.f);
  q[2] = make_float4(e2.x, e2.y, e2.z, 0.f);
  Box6 b;
  b.lo[0] = fminf(fminf(a.x, c1.x), c2.x); b.hi[0] = fmaxf(fmaxf(a.x, c1.x), c2.x);
  b.lo[1] = fminf(fminf(a.y, c1.y), c2.y); b.hi[1] = fmaxf(fmaxf(a.y, c1.y), c2.y);
  b.lo[2] = fminf(fminf(a.z, c1.z), c2.z); b.hi[2] = fmaxf(fmaxf(a.z, c1.z), c2.z);
  return b;
}

// The warp's payloads (lane l: slot base + l, for l < nvalid) stored as 96
// consecutive float4s: store k writes float4s 32k .. 32k + 31, each lane one
// (slot m / 3, part m % 3, fetched from its lane), so every store is one
// contiguous 512-byte run.  All 32 lanes take part.
__device__ __forceinline__ void store_payload_warp(float4* __restrict__ out, int nvalid, uint32_t lane,
                                                   const float4 q[3]) {
  for (int k = 0; k < 3; ++k) {
    const int m = 32 * k + (int)lane, src = m / 3, part = m - 3 * src;
    float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int c = 0; c < 3; ++c) {  // every lane shuffles every part and keeps its own
      const float x = __shfl_sync(0xffffffffu, q[c].x, src), y = __shfl_sync(0xffffffffu, q[c].y, src);
      const float z = __shfl_sync(0xffffffffu, q[c].z, src), w = __shfl_sync(0xffffffffu, q[c].w, src);
      if (part == c) v = make_float4(x, y, z, w);
    }
    if (src < nvalid) out[m] = v;
  }
}

// Above a treelet root: its box goes into the parent (a top node).  With
// the top block active that is all; otherwise climb with device-scope
// arrival counts to the root.
__device__ __forceinline__ void climb_top(uint32_t pw, Box6 b, bool top_mode, float4* nodes,
                                          const uint32_t* __restrict__ parent, uint32_t* flags,
                                          float* __restrict__ root_out, uint32_t* err) {
  for (int level = 0;; ++level) {
    if (level >= 128) { atomicOr(err, kErrCorrupt); return; }  // Karras trees are at most 64 deep
    const uint32_t node = pw >> 1, side = pw & 1u;
    const uint32_t up = node ? __ldg(parent + node) : 0u;
    write_child(nodes, node, side, b);
    if (top_mode) return;
    if (atomic_add_acq_rel(flags + node, 1u) == 0u) return;
    const float4 a = __ldcg(nodes + 4 * (size_t)node);
    const float4 c = __ldcg(nodes + 4 * (size_t)node + 1);
    const float4 z = __ldcg(nodes + 4 * (size_t)node + 2);
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

// Persistent blocks over the treelets.  In a treelet of c leaves from slot
// lo, every internal node has its index in [lo, lo + c) and both children in
// the treelet: one block gathers the leaves' primitives, climbs with
// shared-memory boxes and arrival bits (block-scope ordering only) and at
// the end stores the finished nodes' boxes, coalesced.  heights (optional):
// each internal node's height (longest path to a leaf, leaves 0), from the
// children's heights added into the arrival words.
template <bool HEIGHTS>
__global__ void __launch_bounds__(kTreeletThreads, kTreeletBlocksPerSM) k_refit(int kind, const float4* __restrict__ verts,
                                                          const uint4* __restrict__ idx,
                                                          const float4* __restrict__ sph,
                                                          const uint32_t* __restrict__ order, uint32_t n,
                                                          float4* nodes, const uint32_t* __restrict__ parent,
                                                          const uint32_t* __restrict__ treelets,
                                                          uint32_t* count,  // [0] top nodes, [1] treelets, [2] treelet queue
                                                          uint32_t* flags, float4* __restrict__ prims,
                                                          float* __restrict__ root_out, uint32_t* err,
                                                          uint8_t* __restrict__ heights) {
  extern __shared__ __align__(16) unsigned char refit_smem[];
  RefitShared& sh = *reinterpret_cast<RefitShared*>(refit_smem);
  if (n == 1) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      const Box6 b = emit_prim(kind, verts, idx, sph, __ldg(order), prims, 0);
      for (int k = 0; k < 3; ++k) { root_out[k] = b.lo[k]; root_out[3 + k] = b.hi[k]; }
    }
    return;
  }
  const bool top_mode = __ldcg(count) <= kRefitTopCap;
  const uint32_t ntl = __ldcg(count + 1);
  const uint2* tl = reinterpret_cast<const uint2*>(treelets);
  for (;;) {
    if (threadIdx.x == 0) sh.next = atomicAdd(count + 2, 1u);  // treelets are taken in turn (uneven sizes)
    __syncthreads();
    const uint32_t t = sh.next;
    if (t >= ntl) break;  // uniform per block
    const uint2 rec = __ldcg(tl + t);
    const uint32_t lo = rec.x, cnt = rec.y & ~kTreeletRight;
    if (cnt == 0 || cnt > kTreeletSpan || lo + cnt > n) {  // uniform per block
      if (threadIdx.x == 0) atomicOr(err, kErrCorrupt);
      __syncthreads();  // sh.next is rewritten at the top of the loop
      continue;
    }
    const uint32_t root = cnt == 1 ? ~0u : (rec.y & kTreeletRight) ? lo : lo + cnt - 1;
    for (uint32_t w = threadIdx.x; w < cnt; w += blockDim.x) {
      sh.up[w] = __ldg(parent + lo + w);
      sh.arrived[w] = 0u;
    }
    __syncthreads();
    // Every lane of a warp runs each round (the payload store is warp-wide).
    const uint32_t lane = threadIdx.x & 31u, wbase = threadIdx.x & ~31u;
    for (uint32_t w0 = 0; w0 < cnt; w0 += blockDim.x) {
      const uint32_t w = w0 + threadIdx.x;
      const bool live = w < cnt;
      const uint32_t j = lo + w;
      Box6 b;
      if (kind == kTriangles) {
        float4 q[3] = {};
        if (live) b = tri_payload(verts, idx, __ldg(order + j), q);
        const int nvalid = (int)cnt - (int)(w0 + wbase);  // live lanes of this warp: a prefix
        if (nvalid > 0) store_payload_warp(prims + 3 * (size_t)(lo + w0 + wbase), nvalid < 32 ? nvalid : 32, lane, q);
      } else if (live) {
        b = emit_sphere(sph, __ldg(order + j), prims, j);
      }
      if (!live) continue;
      uint32_t pw = __ldg(parent + (n - 1) + j);
      bool at_root = cnt == 1;  // b is the treelet root's box
      uint32_t h = 0;           // height of the subtree whose box is b
      for (uint32_t step = 0; !at_root; ++step) {
        const uint32_t node = pw >> 1, side = pw & 1u;
        const uint32_t x = node - lo;
        if (x >= cnt || step > kTreeletSpan) { atomicOr(err, kErrCorrupt); break; }
        float* mine = sh.box[x][side];
        for (int k = 0; k < 3; ++k) { mine[k] = b.lo[k]; mine[3 + k] = b.hi[k]; }
        __threadfence_block();
        const uint32_t old = atomicAdd(&sh.arrived[x], HEIGHTS ? 1u + (h << 8) : 1u);
        if ((old & 0xFFu) == 1u) {  // second: finish the node
          __threadfence_block();
          const float* L = sh.box[x][0];
          const float* R = sh.box[x][1];
          for (int k = 0; k < 3; ++k) { b.lo[k] = fminf(L[k], R[k]); b.hi[k] = fmaxf(L[3 + k], R[3 + k]); }
          pw = sh.up[x];
          if constexpr (HEIGHTS) {
            h = 1u + max(h, old >> 8);
            sh.up[x] = h;  // nothing reads x's parent word after this climb: it keeps x's height
          }
          at_root = node == root;
        } else {
          break;
        }
      }
      if (at_root) {
        if (cnt == n) {  // the treelet is the whole tree
          for (int k = 0; k < 3; ++k) { root_out[k] = b.lo[k]; root_out[3 + k] = b.hi[k]; }
        } else {
          climb_top(pw, b, top_mode, nodes, parent, flags, root_out, err);
        }
      }
    }
    __syncthreads();
    // The finished nodes' three box float4s (the fourth, the links, stays),
    // consecutive threads on consecutive float4s.
    for (uint32_t f = threadIdx.x; f < 3 * cnt; f += blockDim.x) {
      const uint32_t w = f / 3, c = f - 3 * w;
      if ((sh.arrived[w] & 0xFFu) != 2u) continue;  // not an internal node of this treelet
      if (HEIGHTS && c == 0) heights[lo + w] = (uint8_t)min(sh.up[w], 255u);
      const float* L = sh.box[w][0];
      const float* R = sh.box[w][1];
      nodes[4 * (size_t)(lo + w) + c] = c == 0 ? make_float4(L[0], L[3], L[1], L[4])
                                      : c == 1 ? make_float4(R[0], R[3], R[1], R[4])
                                               : make_float4(L[2], L[5], R[2], R[5]);
    }
    __syncthreads();  // the next treelet reuses the shared arrays
  }
}

// The top nodes, one block: every child box below them is in place (the
// leaf climb wrote it), so the block climbs the top subtree with shared
// memory boxes and arrival counts, writing each finished box into its
// parent node (and the root box).  Nothing to do when the top nodes exceed
// the cap: the leaf climb went to the root.
struct TopShared {
  float box[kRefitTopCap][2][6];
  uint32_t node[kRefitTopCap];
  uint32_t up[kRefitTopCap];       // parent slot << 1 | side; ~0u for the root
  uint32_t arrived[kRefitTopCap];  // children finished
  uint8_t start[kRefitTopCap];     // both children below the top nodes
};

__device__ __forceinline__ void load_child_box(const float4* nodes, uint32_t node, uint32_t side, float* out) {
  const float4 xy = __ldcg(nodes + 4 * (size_t)node + side);
  const float2 z = __ldcg(reinterpret_cast<const float2*>(nodes + 4 * (size_t)node + 2) + side);
  out[0] = xy.x; out[3] = xy.y; out[1] = xy.z; out[4] = xy.w; out[2] = z.x; out[5] = z.y;
}

__global__ void __launch_bounds__(kRefitTopThreads) k_refit_top(float4* nodes, const uint32_t* __restrict__ parent,
                                                              const uint32_t* __restrict__ mark,
                                                              const uint32_t* __restrict__ top,
                                                              const uint32_t* __restrict__ top_count,
                                                              float* __restrict__ root_out, uint32_t* err) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  TopShared& sh = *reinterpret_cast<TopShared*>(smem_raw);
  const uint32_t cnt = __ldg(top_count);
  if (cnt == 0 || cnt > kRefitTopCap) return;
  for (uint32_t k = threadIdx.x; k < cnt; k += blockDim.x) {
    const uint32_t i = __ldg(top + k);
    sh.node[k] = i;
    const int4 l = __ldcg(reinterpret_cast<const int4*>(nodes) + 4 * (size_t)i + 3);
    uint32_t ready = 0;
    const int32_t ch[2] = {l.x, l.y};
    for (uint32_t side = 0; side < 2; ++side) {
      if (ch[side] >= 0 && (__ldg(mark + ch[side]) & kTopMark)) continue;  // a top child: finished here
      load_child_box(nodes, i, side, sh.box[k][side]);
      ++ready;
    }
    sh.arrived[k] = ready;
    sh.start[k] = ready == 2;
    uint32_t up = ~0u;
    if (i != 0) {
      const uint32_t pw = __ldg(parent + i);
      const uint32_t pm = __ldg(mark + (pw >> 1));
      if (!(pm & kTopMark) || (pm & kSlotMask) >= cnt) {
        atomicOr(err, kErrCorrupt);  // a top node's parent covers more leaves, so it is a top node
        sh.start[k] = 0;
      } else {
        up = ((pm & kSlotMask) << 1) | (pw & 1u);
      }
    }
    sh.up[k] = up;
  }
  __syncthreads();
  for (uint32_t k = threadIdx.x; k < cnt; k += blockDim.x) {
    if (!sh.start[k]) continue;
    uint32_t cur = k;
    for (uint32_t step = 0; step <= cnt; ++step) {
      const float* l = sh.box[cur][0];
      const float* r = sh.box[cur][1];
      Box6 b;
      for (int q = 0; q < 3; ++q) { b.lo[q] = fminf(l[q], r[q]); b.hi[q] = fmaxf(l[3 + q], r[3 + q]); }
      const uint32_t up = sh.up[cur];
      if (up == ~0u) {  // the root
        for (int q = 0; q < 3; ++q) { root_out[q] = b.lo[q]; root_out[3 + q] = b.hi[q]; }
        break;
      }
      const uint32_t ps = up >> 1, side = up & 1u;
      write_child(nodes, sh.node[ps], side, b);
      float* dst = sh.box[ps][side];
      for (int q = 0; q < 3; ++q) { dst[q] = b.lo[q]; dst[3 + q] = b.hi[q]; }
      __threadfence_block();
      if (atomicAdd(&sh.arrived[ps], 1u) != 1u) break;  // the other child is not finished yet
      __threadfence_block();
      cur = ps;
    }
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
                   const RefitTop& t, cudaStream_t s) {
  if (n < 2) return;
  uint32_t g = (n - 1 + kThreads - 1) / kThreads;
  count_launch();
  k_karras<<<g, kThreads, 0, s>>>(sorted_codes, n, nodes, parent, t.mark, t.top, t.treelets, t.count);
}

cudaError_t launch_refit(int kind, const float4* verts, const uint4* idx, const float4* sph,
                         const uint32_t* order, uint32_t n, float4* nodes, const uint32_t* parent,
                         const RefitTop& t, uint32_t* flags, float4* prims, float* root_out, uint32_t* err,
                         cudaStream_t s, uint8_t* heights) {
  if (n == 0) return cudaSuccess;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  static std::atomic<uint64_t> attr_set{0};  // devices whose kernels allow their shared memory
  const uint64_t bit = 1ull << (dev & 63);
  if (!(attr_set.load() & bit)) {
    e = cudaFuncSetAttribute(k_refit<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(RefitShared));
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_refit<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(RefitShared));
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_refit_top, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(TopShared));
    if (e != cudaSuccess) return e;
    attr_set.fetch_or(bit);
  }
  // Persistent: kTreeletBlocksPerSM treelet blocks per SM take treelets from a queue.
  const uint32_t blocks = n == 1 ? 1u : kTreeletBlocksPerSM * (uint32_t)device_sm_count();
  count_launch();
  const auto k = heights ? k_refit<true> : k_refit<false>;
  k<<<blocks, kTreeletThreads, sizeof(RefitShared), s>>>(kind, verts, idx, sph, order, n, nodes, parent, t.treelets,
                                                         t.count, flags, prims, root_out, err, heights);
  if (n < 2) return cudaGetLastError();
  count_launch();
  k_refit_top<<<1, kRefitTopThreads, sizeof(TopShared), s>>>(nodes, parent, t.mark, t.top, t.count, root_out, err);
  return cudaGetLastError();
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
