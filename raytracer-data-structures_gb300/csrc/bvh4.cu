// Collapse of a binary BVH (LBVH or median BVH) into a 4-wide BVH.
//
// Every binary node at even depth becomes one 4-wide node holding the boxes
// of its grandchildren: left.left, left.right, right.left, right.right, where
// a leaf child of the binary node stays a single child.  Nodes are numbered
// by an exclusive scan over the even-depth flags in binary-index order, so
// the root stays node 0 and the layout does not depend on thread timing.
//
// 4-wide node, 128 bytes = 8 float4:
//   [lo.x[4]] [hi.x[4]] [lo.y[4]] [hi.y[4]] [lo.z[4]] [hi.z[4]] [link[4]] [count[4]]
// link >= 0: 4-wide node; link < 0: leaf with slots [~link, ~link + count);
// unused children: lo = +inf, hi = -inf, link 0, count -1 (traversal skips
// them by count, since a slab test with min/max ordering accepts some
// inverted boxes).
//
// Pipeline (all on the build stream, no host synchronisation):
//   k_parents   parent of every binary node (root: 0xFFFFFFFF)
//   k_even      depth parity by walking parent links to the root
//   scan        4-wide index of every even-depth node, total -> count word
//   k_fill4     one thread per even-depth node writes its 128-byte node
// The reference's trees are binary only; this is the engine's node-width
// option for FAST traversal.
#include "rq_build.hpp"
#include "rq_device.cuh"

namespace rq {
namespace {

constexpr int kThreads = 256;

__global__ void __launch_bounds__(kThreads) k_parents(const float4* __restrict__ nodes, uint32_t n,
                                                      uint32_t* __restrict__ parent, uint32_t* err) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int4 l = __ldg(reinterpret_cast<const int4*>(nodes + 4 * (size_t)i + 3));
  if (l.x >= 0) {
    if ((uint32_t)l.x < n && l.x != 0) parent[l.x] = i;
    else atomicOr(err, kErrCorrupt);
  }
  if (l.y >= 0) {
    if ((uint32_t)l.y < n && l.y != 0) parent[l.y] = i;
    else atomicOr(err, kErrCorrupt);
  }
}

// flag[i] = 1 when binary node i sits at even depth.  A valid tree reaches
// the root in fewer than n steps; anything else is reported as corrupt.
__global__ void __launch_bounds__(kThreads) k_even(const uint32_t* __restrict__ parent, uint32_t n,
                                                   uint32_t* __restrict__ flag, uint32_t* err) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint32_t j = i, d = 0;
  while (j != 0) {
    if (j >= n || d >= n) {
      atomicOr(err, kErrCorrupt);
      break;
    }
    j = __ldg(parent + j);
    ++d;
  }
  flag[i] = (d & 1u) ? 0u : 1u;
}

struct Child4 {
  float lo[3], hi[3];
  int32_t link, count;
};

__device__ __forceinline__ Child4 child_of(const float4& a, const float4& b, const float4& z, const int4& l,
                                           int side) {
  Child4 c;
  if (side == 0) {
    c.lo[0] = a.x; c.hi[0] = a.y; c.lo[1] = a.z; c.hi[1] = a.w; c.lo[2] = z.x; c.hi[2] = z.y;
    c.link = l.x; c.count = l.z;
  } else {
    c.lo[0] = b.x; c.hi[0] = b.y; c.lo[1] = b.z; c.hi[1] = b.w; c.lo[2] = z.z; c.hi[2] = z.w;
    c.link = l.y; c.count = l.w;
  }
  return c;
}

__global__ void __launch_bounds__(kThreads) k_fill4(const float4* __restrict__ nodes, uint32_t n,
                                                    const uint32_t* __restrict__ flag,
                                                    const uint32_t* __restrict__ idx4, uint32_t n4_cap,
                                                    float4* __restrict__ out, uint32_t* err) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || !__ldg(flag + i)) return;
  const uint32_t o = __ldg(idx4 + i);
  if (o >= n4_cap) {
    atomicOr(err, kErrCorrupt);
    return;
  }
  float lo[3][4], hi[3][4];
  int32_t link[4], count[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    for (int q = 0; q < 3; ++q) {
      lo[q][k] = __int_as_float(0x7F800000);
      hi[q][k] = __int_as_float((int)0xFF800000u);
    }
    link[k] = 0;
    count[k] = -1;
  }
  int slot = 0;
  auto put = [&](const Child4& c) {
    for (int q = 0; q < 3; ++q) {
      lo[q][slot] = c.lo[q];
      hi[q][slot] = c.hi[q];
    }
    link[slot] = c.link;
    count[slot] = c.count;
    ++slot;
  };
  const float4* nd = nodes + 4 * (size_t)i;
  float4 a = __ldg(nd), b = __ldg(nd + 1), z = __ldg(nd + 2);
  int4 l = __ldg(reinterpret_cast<const int4*>(nd + 3));
  for (int side = 0; side < 2; ++side) {
    Child4 c = child_of(a, b, z, l, side);
    if (c.link < 0) {
      put(c);
      continue;
    }
    if ((uint32_t)c.link >= n) {
      atomicOr(err, kErrCorrupt);
      return;
    }
    const float4* cd = nodes + 4 * (size_t)c.link;
    float4 ca = __ldg(cd), cb = __ldg(cd + 1), cz = __ldg(cd + 2);
    int4 cl = __ldg(reinterpret_cast<const int4*>(cd + 3));
    for (int s2 = 0; s2 < 2; ++s2) {
      Child4 g = child_of(ca, cb, cz, cl, s2);
      if (g.link >= 0) {
        if ((uint32_t)g.link >= n) {
          atomicOr(err, kErrCorrupt);
          return;
        }
        g.link = (int32_t)__ldg(idx4 + g.link);
        g.count = 0;
      }
      put(g);
    }
  }
  float4* w = out + 8 * (size_t)o;
  for (int q = 0; q < 3; ++q) {
    w[2 * q] = make_float4(lo[q][0], lo[q][1], lo[q][2], lo[q][3]);
    w[2 * q + 1] = make_float4(hi[q][0], hi[q][1], hi[q][2], hi[q][3]);
  }
  reinterpret_cast<int4*>(w)[6] = make_int4(link[0], link[1], link[2], link[3]);
  reinterpret_cast<int4*>(w)[7] = make_int4(count[0], count[1], count[2], count[3]);
}

#define RQ_B4(call, what)                                            \
  do {                                                               \
    cudaError_t e_ = (call);                                         \
    if (e_ != cudaSuccess) return BuildResult::cuda_error(e_, what); \
  } while (0)

}  // namespace

void launch_parents(const float4* nodes, uint32_t n, uint32_t* parent, uint32_t* err, cudaStream_t st) {
  count_launch();
  k_parents<<<(n + kThreads - 1) / kThreads, kThreads, 0, st>>>(nodes, n, parent, err);
}

// Upper bound of the 4-wide node count: every even-depth node but the root
// has an odd-depth parent with at most two children, so even <= 1 + 2 * odd
// and even <= (2n + 1) / 3.
uint32_t bvh4_node_cap(uint32_t n_internal) { return (2 * n_internal + 1) / 3 + 1; }

BuildResult collapse_bvh4(AccelBuffers& a, BuildScratch& sc, uint32_t* err, cudaStream_t st) {
  const uint32_t n = a.n_nodes;
  a.node_width = 4;
  if (n == 0) {
    RQ_B4(cudaMemsetAsync(a.root.as<uint32_t>() + 6, 0, 4, st), "memset");
    return {};
  }
  const uint32_t cap = bvh4_node_cap(n);
  RQ_B4(a.nodes4.ensure((size_t)cap * 128), "4-wide nodes");
  RQ_B4(sc.m0.ensure((size_t)n * 4), "collapse scratch");
  RQ_B4(sc.m1.ensure((size_t)n * 4), "collapse scratch");
  RQ_B4(sc.m2.ensure((size_t)n * 4), "collapse scratch");
  RQ_B4(sc.m3.ensure(scan_tmp_words(n) * 4), "collapse scratch");
  uint32_t* parent = sc.m0.as<uint32_t>();
  uint32_t* flag = sc.m1.as<uint32_t>();
  uint32_t* idx4 = sc.m2.as<uint32_t>();
  RQ_B4(cudaMemsetAsync(parent, 0xFF, (size_t)n * 4, st), "memset");
  const uint32_t g = (n + kThreads - 1) / kThreads;
  count_launch(3);
  k_parents<<<g, kThreads, 0, st>>>(a.nodes.as<const float4>(), n, parent, err);
  k_even<<<g, kThreads, 0, st>>>(parent, n, flag, err);
  launch_scan_excl(flag, idx4, n, sc.m3.as<uint32_t>(), a.root.as<uint32_t>() + 6, st);
  k_fill4<<<g, kThreads, 0, st>>>(a.nodes.as<const float4>(), n, flag, idx4, cap, a.nodes4.as<float4>(), err);
  RQ_B4(cudaGetLastError(), "collapse launch");
  a.n4_cap = cap;
  return {};
}

}  // namespace rq
