// Median BVH build on the GPU: constructBVHNew (accelerators.h:246-337),
// level by level.
//
// Per node the reference takes the union of the primitive boxes, seeds the
// centroid bounds with it (:275-277), picks the longest axis (:279, GeMaximumAxis
// :190-199), and if the centroids straddle the axis midpoint (:298-311) puts the
// floor(n/2) smallest centroids on the left (std::nth_element, :312-318); a node
// of one primitive is a leaf.  Degenerate nodes (all centroids on one side of
// the midpoint, or a zero-extent axis) become one leaf holding the whole range;
// the reference there keeps a single primitive or recurses without end.  Ties
// at the median are broken by primitive id; the reference leaves them to
// libstdc++'s nth_element.
//
// Method: the primitive ids are sorted once per axis by (centroid, id) with the
// engine's radix sort.  A level is a set of disjoint position ranges
// (segments) shared by the three lists.  Per level: segment boxes (grouped
// reduction), the split decision per segment (the centroid extremes and the
// count below the midpoint come straight from the sorted list of the split
// axis), node numbering by a prefix sum over split flags, and a stable
// partition of all three lists by one prefix sum over their left flags.  The
// leaves end up as position ranges of the x-sorted list, which becomes the
// slot order.  Internal nodes are numbered breadth-first, left before right.
// The level counts stay on the device (no host round trip per level), and
// once every segment holds at most kFinishSpan primitives the remaining
// levels of each run inside one block (k_finish, in shared memory; two
// passes so that breadth-first numbering spans all subtrees).
#include <algorithm>
#include <atomic>
#include <vector>

#include "rq_build.hpp"
#include "rq_device.cuh"

namespace rq {
namespace {

constexpr int kThreads = 256;
constexpr uint32_t kRoot = 0xFFFFFFFFu;

// Ascending float order as unsigned keys; -0 and +0 map to the same key.
__device__ __forceinline__ uint32_t float_key(float f) {
  uint32_t b = __float_as_uint(__fadd_rn(f, 0.0f));
  return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}

__global__ void __launch_bounds__(kThreads) k_prim_info(int kind, const float* __restrict__ verts,
                                                        const uint32_t* __restrict__ idx,
                                                        const float4* __restrict__ sph, uint32_t n,
                                                        float* __restrict__ aabb, float* __restrict__ cen,
                                                        uint32_t* __restrict__ keys, uint32_t* __restrict__ vals) {
  uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  float lo[3], hi[3], c[3];
  if (kind == kTriangles) {
    const float* a = verts + 3 * (size_t)__ldg(idx + 3 * (size_t)p);
    const float* b = verts + 3 * (size_t)__ldg(idx + 3 * (size_t)p + 1);
    const float* d = verts + 3 * (size_t)__ldg(idx + 3 * (size_t)p + 2);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      float x = __ldg(a + k), y = __ldg(b + k), z = __ldg(d + k);
      lo[k] = fminf(fminf(x, y), z);
      hi[k] = fmaxf(fmaxf(x, y), z);
      c[k] = __fdiv_rn(__fadd_rn(__fadd_rn(x, y), z), 3.0f);
    }
  } else {
    float4 s = __ldg(sph + p);
    float sc[3] = {s.x, s.y, s.z};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      lo[k] = __fsub_rn(sc[k], s.w);
      hi[k] = __fadd_rn(sc[k], s.w);
      c[k] = sc[k];
    }
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    aabb[6 * (size_t)p + k] = lo[k];
    aabb[6 * (size_t)p + 3 + k] = hi[k];
    cen[3 * (size_t)p + k] = c[k];
    keys[(size_t)k * n + p] = float_key(c[k]);
    vals[(size_t)k * n + p] = p;
  }
}

// Segment of every list position (-1 for positions already in a leaf).
__global__ void __launch_bounds__(kThreads) k_seg_id(const uint32_t* __restrict__ start,
                                                     const uint32_t* __restrict__ end, const uint32_t* S_dev,
                                                     uint32_t n, int32_t* __restrict__ seg_id) {
  uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const uint32_t S = *S_dev;
  uint32_t lo = 0, hi = S;  // first segment with start > p
  while (lo < hi) {
    uint32_t m = (lo + hi) >> 1;
    if (__ldg(start + m) <= p) lo = m + 1;
    else hi = m;
  }
  int32_t k = (int32_t)lo - 1;
  seg_id[p] = (k >= 0 && p < __ldg(end + k)) ? k : -1;
}

// Segment boxes: groups of G threads reduce one slice of G*8 positions of a
// segment; one slice per segment stores directly, several use atomics.
template <int G>
__global__ void __launch_bounds__(kThreads) k_seg_bounds(const uint32_t* __restrict__ list0,
                                                         const float* __restrict__ aabb,
                                                         const uint32_t* __restrict__ start,
                                                         const uint32_t* __restrict__ end, const uint32_t* S_dev,
                                                         uint32_t slices, int32_t* __restrict__ box) {
  constexpr int kPer = 8;
  const uint32_t group = (blockIdx.x * kThreads + threadIdx.x) / G;
  const uint32_t t = threadIdx.x % G;
  const uint32_t seg = group / slices, slice = group % slices;
  const bool live = seg < *S_dev;
  float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  if (live) {
    const uint32_t s = __ldg(start + seg), e = __ldg(end + seg);
    const uint32_t b = s + slice * (uint32_t)(G * kPer);
#pragma unroll
    for (int k = 0; k < kPer; ++k) {
      uint32_t p = b + t + (uint32_t)(G * k);
      if (p < e) {
        const float* q = aabb + 6 * (size_t)__ldg(list0 + p);
        for (int a = 0; a < 3; ++a) {
          lo[a] = fminf(lo[a], __ldg(q + a));
          hi[a] = fmaxf(hi[a], __ldg(q + 3 + a));
        }
      }
    }
  }
  if (G <= 32) {
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1)
      for (int a = 0; a < 3; ++a) {
        lo[a] = fminf(lo[a], __shfl_xor_sync(0xffffffffu, lo[a], o, G));
        hi[a] = fmaxf(hi[a], __shfl_xor_sync(0xffffffffu, hi[a], o, G));
      }
  } else {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
      for (int a = 0; a < 3; ++a) {
        lo[a] = fminf(lo[a], __shfl_xor_sync(0xffffffffu, lo[a], o));
        hi[a] = fmaxf(hi[a], __shfl_xor_sync(0xffffffffu, hi[a], o));
      }
    __shared__ float sm[kThreads / 32][6];
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0)
      for (int a = 0; a < 3; ++a) { sm[w][a] = lo[a]; sm[w][3 + a] = hi[a]; }
    __syncthreads();
    if (t == 0) {
      const int w0 = w, nw = G / 32;
      for (int q = 1; q < nw; ++q)
        for (int a = 0; a < 3; ++a) {
          lo[a] = fminf(lo[a], sm[w0 + q][a]);
          hi[a] = fmaxf(hi[a], sm[w0 + q][3 + a]);
        }
    }
  }
  if (!live || t != 0) return;
  int32_t* bx = box + 6 * (size_t)seg;
  if (slices == 1) {
    for (int a = 0; a < 3; ++a) { bx[a] = float_to_ordered(lo[a]); bx[3 + a] = float_to_ordered(hi[a]); }
  } else {
    for (int a = 0; a < 3; ++a) {
      atomicMin(bx + a, float_to_ordered(lo[a]));
      atomicMax(bx + 3 + a, float_to_ordered(hi[a]));
    }
  }
}

__global__ void k_box_init(int32_t* box, uint32_t S) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 6 * S) return;
  box[i] = (i % 6) < 3 ? ordered_pos_inf() : ordered_neg_inf();
}

struct Segs {
  uint32_t* start;
  uint32_t* end;
  uint32_t* parent;  // node << 1 | side, kRoot for the root
  int32_t* box;      // 6 ordered ints
  uint32_t* split;   // 1 when the segment becomes an internal node
  uint32_t* mid;
  uint32_t* dim;
  uint32_t* rank;    // exclusive prefix of split
};

// The split decision of one segment (constructBVHNew's rules), given its
// box and the centroids of its first and last element along each axis (the
// segment's range of that axis' sorted list) and a way to count the
// elements whose centroid along an axis lies below a value (`below(dim,
// pmid)`, over that axis' list).  Shared by the level kernels and the
// in-block subtree builder so both decide with the same operations.
struct SplitDecision {
  uint32_t split, half, dim;  // half: elements on the left (m / 2) when split
};
template <typename Below>
__device__ __forceinline__ SplitDecision decide_split(const float* box_lo, const float* box_hi, const float* cfirst,
                                                      const float* clast, uint32_t m, Below below) {
  SplitDecision d{0u, 0u, 0u};
  if (m <= 1) return d;
  float lo[3], hi[3];
  for (int a = 0; a < 3; ++a) {
    // centroid bounds seeded with the node bounds (:275-277); the extremes of
    // the centroids along axis a are the ends of that axis' sorted list
    lo[a] = cfirst[a] < box_lo[a] ? cfirst[a] : box_lo[a];
    hi[a] = clast[a] > box_hi[a] ? clast[a] : box_hi[a];
  }
  float ax = __fsub_rn(hi[0], lo[0]), ay = __fsub_rn(hi[1], lo[1]), az = __fsub_rn(hi[2], lo[2]);
  d.dim = (ax > ay && ax > az) ? 0u : (ay > az ? 1u : 2u);
  if (hi[d.dim] != lo[d.dim]) {
    const float pmid = __fdiv_rn(__fadd_rn(lo[d.dim], hi[d.dim]), 2.0f);
    const uint32_t less = below(d.dim, pmid);
    if (less != 0 && less != m) {
      d.split = 1;
      d.half = m / 2;
    }
  }
  return d;
}

__global__ void __launch_bounds__(kThreads) k_seg_decide(Segs g, const uint32_t* S_dev, uint32_t S_bound,
                                                         const uint32_t* __restrict__ lists, uint32_t n,
                                                         const float* __restrict__ cen) {
  uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= S_bound) return;
  if (k >= *S_dev) {  // past this level's segments: no split (the scan runs over S_bound flags)
    g.split[k] = 0;
    return;
  }
  const uint32_t s = g.start[k], e = g.end[k], m = e - s;
  float lo[3], hi[3], cf[3] = {0.f, 0.f, 0.f}, cl[3] = {0.f, 0.f, 0.f};
  for (int a = 0; a < 3; ++a) {
    lo[a] = ordered_to_float(g.box[6 * (size_t)k + a]);
    hi[a] = ordered_to_float(g.box[6 * (size_t)k + 3 + a]);
    if (m > 1) {
      cf[a] = __ldg(cen + 3 * (size_t)lists[(size_t)a * n + s] + a);
      cl[a] = __ldg(cen + 3 * (size_t)lists[(size_t)a * n + e - 1] + a);
    }
  }
  const SplitDecision d = decide_split(lo, hi, cf, cl, m, [&](uint32_t dim, float pmid) {
    const uint32_t* L = lists + (size_t)dim * n;
    uint32_t a = s, b = e;  // first position whose centroid is >= pmid
    while (a < b) {
      uint32_t q = (a + b) >> 1;
      if (__ldg(cen + 3 * (size_t)L[q] + dim) < pmid) a = q + 1;
      else b = q;
    }
    return a - s;
  });
  g.split[k] = d.split;
  g.mid[k] = d.split ? s + d.half : s;
  g.dim[k] = d.dim;
}

// ctl[2 * level] = segments of the level, ctl[2 * level + 1] = the level's
// first node index; thread 0 also writes the next level's pair.
__global__ void __launch_bounds__(kThreads) k_seg_link(Segs g, uint32_t* ctl, int level, const uint32_t* splits,
                                                       Segs next, float4* __restrict__ nodes,
                                                       float* __restrict__ root) {
  uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t S = ctl[2 * level], node_base = ctl[2 * level + 1];
  if (k == 0) {
    ctl[2 * level + 2] = 2 * *splits;
    ctl[2 * level + 3] = node_base + *splits;
  }
  if (k >= S) return;
  const uint32_t s = g.start[k], e = g.end[k];
  float lo[3], hi[3];
  for (int a = 0; a < 3; ++a) {
    lo[a] = ordered_to_float(g.box[6 * (size_t)k + a]);
    hi[a] = ordered_to_float(g.box[6 * (size_t)k + 3 + a]);
  }
  const bool split = g.split[k] != 0;
  const uint32_t node = node_base + g.rank[k];
  const uint32_t pw = g.parent[k];
  if (pw == kRoot) {
    for (int a = 0; a < 3; ++a) { root[a] = lo[a]; root[3 + a] = hi[a]; }
  } else {
    const uint32_t pn = pw >> 1, side = pw & 1u;
    nodes[4 * (size_t)pn + side] = make_float4(lo[0], hi[0], lo[1], hi[1]);
    reinterpret_cast<float2*>(nodes + 4 * (size_t)pn + 2)[side] = make_float2(lo[2], hi[2]);
    int* link = reinterpret_cast<int*>(nodes + 4 * (size_t)pn + 3);
    link[side] = split ? (int)node : ~(int)s;
    link[2 + side] = split ? 0 : (int)(e - s);
  }
  if (split) {
    const uint32_t r = 2 * g.rank[k], mid = g.mid[k];
    next.start[r] = s;      next.end[r] = mid;     next.parent[r] = node << 1;
    next.start[r + 1] = mid; next.end[r + 1] = e;  next.parent[r + 1] = (node << 1) | 1u;
  }
}

// Left/right side of every primitive in a splitting segment.
__global__ void __launch_bounds__(kThreads) k_mark(Segs g, const int32_t* __restrict__ seg_id,
                                                   const uint32_t* __restrict__ lists, uint32_t n,
                                                   uint8_t* __restrict__ left) {
  uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  int32_t k = seg_id[p];
  if (k < 0 || !g.split[k]) return;
  const uint32_t d = g.dim[k];
  left[lists[(size_t)d * n + p]] = p < g.mid[k] ? 1 : 0;
}

// Scan input: 1 for a left-side element of a splitting segment, per list.
__global__ void __launch_bounds__(kThreads) k_left_flags(Segs g, const int32_t* __restrict__ seg_id,
                                                         const uint32_t* __restrict__ lists, uint32_t n,
                                                         const uint8_t* __restrict__ left,
                                                         uint32_t* __restrict__ flags) {
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 3ull * n) return;
  const uint32_t p = (uint32_t)(i % n);
  int32_t k = seg_id[p];
  flags[i] = (k >= 0 && g.split[k]) ? left[lists[i]] : 0u;
}

// Stable partition of the three lists inside every splitting segment.
__global__ void __launch_bounds__(kThreads) k_partition(Segs g, const int32_t* __restrict__ seg_id,
                                                        const uint32_t* __restrict__ in, uint32_t n,
                                                        const uint8_t* __restrict__ left,
                                                        const uint32_t* __restrict__ scan,
                                                        uint32_t* __restrict__ out) {
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 3ull * n) return;
  const uint64_t a0 = (i / n) * n;
  const uint32_t p = (uint32_t)(i - a0);
  const uint32_t v = in[i];
  int32_t k = seg_id[p];
  if (k < 0 || !g.split[k]) {
    out[i] = v;
    return;
  }
  const uint32_t s = g.start[k], mid = g.mid[k];
  const uint32_t lb = scan[i] - scan[a0 + s];
  const uint32_t np = left[v] ? s + lb : mid + ((p - s) - lb);
  if (np < g.end[k]) out[a0 + np] = v;  // always true while the three lists hold the same sets
}

// ---------------------------------------------------------------- small subtrees
// Segments of at most kFinishSpan primitives finish inside one block each:
// the block loads the segment's three sorted lists (as local indices), boxes
// and centroids into shared memory and runs the same levels there (one warp
// per segment: box, decide_split, then a stable ballot partition of the three
// lists).  Internal nodes are numbered breadth-first over the whole tree, so
// the block runs twice: the first pass counts each subtree's internal nodes
// per relative level (counts[d * S_bound + b]); an exclusive scan of that
// level-major table gives every subtree's first index at every level; the
// second pass writes the nodes with those indices and the final slot order.
constexpr uint32_t kFinishSpan = 512;
constexpr int kFinishThreads = 256;
constexpr int kFinishDepth = 13;  // levels of a subtree of kFinishSpan leaves (median halving), with margin

struct FinishShared {
  uint32_t id[kFinishSpan];                     // global primitive id by local index
  float box[kFinishSpan][6];                    // primitive boxes (lo xyz, hi xyz) by local index
  float cen[kFinishSpan][3];                    // centroids by local index
  uint16_t list[2][3][kFinishSpan];             // the three sorted lists, local indices, double buffered
  uint8_t left[kFinishSpan];                    // side of a primitive in its splitting segment
  uint16_t seg_start[2][kFinishSpan], seg_end[2][kFinishSpan];
  uint32_t seg_parent[2][kFinishSpan];          // global node << 1 | side, kRoot for the root
  uint32_t rank[kFinishSpan];                   // split flags, then their exclusive prefix
  uint16_t half[kFinishSpan];                   // left size of a splitting segment, 0 otherwise
  uint8_t dim[kFinishSpan];
  uint32_t warp_sum[kFinishThreads / 32];
  uint32_t nsplit;
};

// Exclusive prefix of rank[0 .. n) in place (n <= kFinishSpan), total in
// sh.nsplit; the whole block calls it.
__device__ __forceinline__ void finish_scan(FinishShared& sh, uint32_t n) {
  constexpr int kPer = kFinishSpan / kFinishThreads;
  const uint32_t t = threadIdx.x, lane = t & 31u, warp = t >> 5;
  uint32_t v[kPer], sum = 0;
  for (int k = 0; k < kPer; ++k) {
    const uint32_t i = t * kPer + k;
    v[k] = i < n ? sh.rank[i] : 0u;
    sum += v[k];
  }
  uint32_t x = sum;
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= (uint32_t)o) x += y;
  }
  if (lane == 31) sh.warp_sum[warp] = x;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = lane < kFinishThreads / 32 ? sh.warp_sum[lane] : 0u;
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= (uint32_t)o) w += y;
    }
    if (lane < kFinishThreads / 32) sh.warp_sum[lane] = w;
    if (lane == kFinishThreads / 32 - 1) sh.nsplit = w;
  }
  __syncthreads();
  uint32_t run = (warp ? sh.warp_sum[warp - 1] : 0u) + x - sum;
  for (int k = 0; k < kPer; ++k) {
    const uint32_t i = t * kPer + k;
    if (i < n) sh.rank[i] = run;
    run += v[k];
  }
  __syncthreads();
}

// Box of segment [st, en) of the current lists, over a group of W lanes
// (W = 32: a warp, every lane gets the box; W = 1: one thread).
template <int W>
__device__ __forceinline__ void finish_box(const FinishShared& sh, int cb, uint32_t st, uint32_t en, uint32_t lane,
                                           float* lo, float* hi) {
  for (int a = 0; a < 3; ++a) { lo[a] = INFINITY; hi[a] = -INFINITY; }
  for (uint32_t i = st + lane; i < en; i += W) {
    const float* b = sh.box[sh.list[cb][0][i]];
    for (int a = 0; a < 3; ++a) { lo[a] = fminf(lo[a], b[a]); hi[a] = fmaxf(hi[a], b[3 + a]); }
  }
  if (W == 32)
    for (int o = 16; o > 0; o >>= 1)
      for (int a = 0; a < 3; ++a) {
        lo[a] = fminf(lo[a], __shfl_xor_sync(0xffffffffu, lo[a], o));
        hi[a] = fmaxf(hi[a], __shfl_xor_sync(0xffffffffu, hi[a], o));
      }
}

// Split decision of every segment of the level (group g of ng takes
// segments g, g + ng, ...): half, dim, and the split flag in rank.
template <int W>
__device__ __forceinline__ void finish_decide(FinishShared& sh, int cb, int sb, uint32_t nseg, uint32_t g, uint32_t lane,
                                              uint32_t ng) {
  for (uint32_t j = g; j < nseg; j += ng) {
    const uint32_t st = sh.seg_start[sb][j], en = sh.seg_end[sb][j];
    float lo[3], hi[3];
    finish_box<W>(sh, cb, st, en, lane, lo, hi);
    if (lane == 0) {
      float cf[3], cl[3];
      for (int a = 0; a < 3; ++a) {
        cf[a] = sh.cen[sh.list[cb][a][st]][a];
        cl[a] = sh.cen[sh.list[cb][a][en - 1]][a];
      }
      const SplitDecision dd = decide_split(lo, hi, cf, cl, en - st, [&](uint32_t dim, float pmid) {
        uint32_t x = st, y = en;  // first position whose centroid is >= pmid
        while (x < y) {
          const uint32_t q = (x + y) >> 1;
          if (sh.cen[sh.list[cb][dim][q]][dim] < pmid) x = q + 1;
          else y = q;
        }
        return x - st;
      });
      sh.half[j] = (uint16_t)(dd.split ? dd.half : 0u);
      sh.dim[j] = (uint8_t)dd.dim;
      sh.rank[j] = dd.split;
    }
  }
}

// Write every segment into its parent (WRITE), emit the next level's
// segments and the left flags of the splitting ones.
template <int W, bool WRITE>
__device__ __forceinline__ void finish_emit(FinishShared& sh, int cb, int sb, uint32_t nseg, uint32_t g, uint32_t lane,
                                            uint32_t ng, uint32_t s, uint32_t level_base, uint32_t node_cap,
                                            float4* __restrict__ nodes, float* __restrict__ root, uint32_t* err) {
  for (uint32_t j = g; j < nseg; j += ng) {
    const uint32_t st = sh.seg_start[sb][j], en = sh.seg_end[sb][j], hf = sh.half[j];
    const uint32_t node = level_base + sh.rank[j];
    if (WRITE) {
      float lo[3], hi[3];
      finish_box<W>(sh, cb, st, en, lane, lo, hi);
      if (lane == 0) {
        const uint32_t pw = sh.seg_parent[sb][j];
        if (pw == kRoot) {
          for (int a = 0; a < 3; ++a) { root[a] = lo[a]; root[3 + a] = hi[a]; }
        } else if ((pw >> 1) >= node_cap || (hf && node >= node_cap)) {
          atomicOr(err, kErrCorrupt);  // indices come from the scan of the first pass's counts
        } else {
          const uint32_t pn = pw >> 1, side = pw & 1u;
          nodes[4 * (size_t)pn + side] = make_float4(lo[0], hi[0], lo[1], hi[1]);
          reinterpret_cast<float2*>(nodes + 4 * (size_t)pn + 2)[side] = make_float2(lo[2], hi[2]);
          int* link = reinterpret_cast<int*>(nodes + 4 * (size_t)pn + 3);
          link[side] = hf ? (int)node : ~(int)(s + st);
          link[2 + side] = hf ? 0 : (int)(en - st);
        }
      }
    }
    if (hf) {
      if (lane == 0) {
        const uint32_t r = 2 * sh.rank[j];
        sh.seg_start[sb ^ 1][r] = (uint16_t)st;
        sh.seg_end[sb ^ 1][r] = (uint16_t)(st + hf);
        sh.seg_parent[sb ^ 1][r] = node << 1;
        sh.seg_start[sb ^ 1][r + 1] = (uint16_t)(st + hf);
        sh.seg_end[sb ^ 1][r + 1] = (uint16_t)en;
        sh.seg_parent[sb ^ 1][r + 1] = (node << 1) | 1u;
      }
      const uint32_t dm = sh.dim[j];
      for (uint32_t i = st + lane; i < en; i += W) sh.left[sh.list[cb][dm][i]] = (i - st) < hf ? 1 : 0;
    }
  }
}

// Stable partition of the three lists inside every splitting segment (the
// others are copied) into the other buffer.
template <int W>
__device__ __forceinline__ void finish_partition(FinishShared& sh, int cb, int sb, uint32_t nseg, uint32_t g,
                                                 uint32_t lane, uint32_t ng) {
  for (uint32_t j = g; j < nseg; j += ng) {
    const uint32_t st = sh.seg_start[sb][j], en = sh.seg_end[sb][j], hf = sh.half[j];
    for (int a = 0; a < 3; ++a) {
      const uint16_t* in = sh.list[cb][a];
      uint16_t* out = sh.list[cb ^ 1][a];
      if (W == 1) {
        uint32_t nl = 0, nr = 0;
        for (uint32_t i = st; i < en; ++i) {
          const uint16_t x = in[i];
          if (hf == 0 || sh.left[x]) out[st + nl++] = x;
          else out[st + hf + nr++] = x;
        }
        continue;
      }
      uint32_t nl = 0, nr = 0;
      for (uint32_t c = st; c < en; c += 32) {
        const uint32_t i = c + lane;
        const bool live = i < en;
        const uint16_t x = live ? in[i] : (uint16_t)0;
        const bool goes_left = live && (hf == 0 || sh.left[x]);
        const bool goes_right = live && hf != 0 && !sh.left[x];
        const uint32_t ml = __ballot_sync(0xffffffffu, goes_left), mr = __ballot_sync(0xffffffffu, goes_right);
        const uint32_t below = (1u << lane) - 1u;
        if (goes_left) out[st + nl + __popc(ml & below)] = x;
        if (goes_right) out[st + hf + nr + __popc(mr & below)] = x;
        nl += __popc(ml);
        nr += __popc(mr);
      }
    }
  }
}

template <bool WRITE>
__global__ void __launch_bounds__(kFinishThreads) k_finish(Segs g, const uint32_t* S_dev, uint32_t S_bound,
                                                          uint32_t* lists0, const uint32_t* __restrict__ lists1,
                                                          const uint32_t* __restrict__ lists2,
                                                          const float* __restrict__ aabb, const float* __restrict__ cen,
                                                          uint32_t* loc, uint32_t* counts,
                                                          const uint32_t* __restrict__ offs, const uint32_t* base_dev,
                                                          uint32_t node_cap, float4* __restrict__ nodes,
                                                          float* __restrict__ root, uint32_t* err) {
  extern __shared__ __align__(16) unsigned char finish_smem[];
  FinishShared& sh = *reinterpret_cast<FinishShared*>(finish_smem);
  const uint32_t b = blockIdx.x, t = threadIdx.x, lane = t & 31u, warp = t >> 5;
  constexpr uint32_t kWarps = kFinishThreads / 32;
  if (b >= *S_dev) {
    if (!WRITE)
      for (int d = (int)t; d < kFinishDepth; d += kFinishThreads) counts[(size_t)d * S_bound + b] = 0u;
    return;
  }
  const uint32_t s = g.start[b], e = g.end[b], cnt = e - s;
  if (cnt > kFinishSpan) {  // the level loop stops only when every segment fits
    if (t == 0) atomicOr(err, kErrCorrupt);
    return;
  }
  const uint32_t node_base = WRITE ? *base_dev : 0u;
  for (uint32_t i = t; i < cnt; i += kFinishThreads) {
    const uint32_t gid = lists0[s + i];
    sh.id[i] = gid;
    loc[gid] = i;
    for (int a = 0; a < 6; ++a) sh.box[i][a] = __ldg(aabb + 6 * (size_t)gid + a);
    for (int a = 0; a < 3; ++a) sh.cen[i][a] = __ldg(cen + 3 * (size_t)gid + a);
    sh.list[0][0][i] = (uint16_t)i;
  }
  if (t == 0) {
    sh.seg_start[0][0] = 0;
    sh.seg_end[0][0] = (uint16_t)cnt;
    sh.seg_parent[0][0] = g.parent[b];
  }
  __syncthreads();  // loc of this block's ids is visible to the block
  for (uint32_t i = t; i < cnt; i += kFinishThreads) {
    sh.list[0][1][i] = (uint16_t)loc[__ldg(lists1 + s + i)];
    sh.list[0][2][i] = (uint16_t)loc[__ldg(lists2 + s + i)];
  }
  __syncthreads();
  int cb = 0, sb = 0;
  uint32_t nseg = 1;
  for (int d = 0; nseg > 0; ++d) {
    if (d >= kFinishDepth) {
      if (t == 0) atomicOr(err, kErrCorrupt);
      return;
    }
    // Groups of W lanes per segment: a warp while segments are large, one
    // thread once the largest (at most ceil(cnt / 2^d) under median halving)
    // has 64 primitives or fewer.
    const bool small = ((cnt + (1u << d) - 1) >> d) <= 64u;
    if (small) finish_decide<1>(sh, cb, sb, nseg, t, 0u, kFinishThreads);
    else finish_decide<32>(sh, cb, sb, nseg, warp, lane, kWarps);
    __syncthreads();
    finish_scan(sh, nseg);
    const uint32_t nsplit = sh.nsplit;
    if (!WRITE && t == 0) counts[(size_t)d * S_bound + b] = nsplit;
    const uint32_t level_base = WRITE ? node_base + offs[(size_t)d * S_bound + b] : 0u;
    if (small) finish_emit<1, WRITE>(sh, cb, sb, nseg, t, 0u, kFinishThreads, s, level_base, node_cap, nodes, root, err);
    else finish_emit<32, WRITE>(sh, cb, sb, nseg, warp, lane, kWarps, s, level_base, node_cap, nodes, root, err);
    __syncthreads();
    if (small) finish_partition<1>(sh, cb, sb, nseg, t, 0u, kFinishThreads);
    else finish_partition<32>(sh, cb, sb, nseg, warp, lane, kWarps);
    __syncthreads();
    cb ^= 1;
    sb ^= 1;
    nseg = 2 * nsplit;
  }
  if (WRITE)
    for (uint32_t i = t; i < cnt; i += kFinishThreads) lists0[s + i] = sh.id[sh.list[cb][0][i]];
}

#define MB_TRY(call, what)                                           \
  do {                                                               \
    cudaError_t e_ = (call);                                         \
    if (e_ != cudaSuccess) return BuildResult::cuda_error(e_, what); \
  } while (0)

// S: an upper bound of the level's segments (the kernels read the count);
// max_size: an upper bound of their sizes.
template <int G>
void seg_bounds(const uint32_t* list0, const float* aabb, const Segs& g, const uint32_t* S_dev, uint32_t S,
                uint32_t max_size, cudaStream_t st) {
  const uint32_t per_slice = G * 8;
  const uint32_t slices = (max_size + per_slice - 1) / per_slice;
  if (slices > 1) {
    count_launch();
    k_box_init<<<(6 * S + kThreads - 1) / kThreads, kThreads, 0, st>>>(g.box, S);
  }
  const uint64_t groups = (uint64_t)S * slices;
  const uint64_t blocks = (groups * G + kThreads - 1) / kThreads;
  count_launch();
  k_seg_bounds<G><<<(unsigned)blocks, kThreads, 0, st>>>(list0, aabb, g.start, g.end, S_dev, slices, g.box);
}

void seg_bounds_dispatch(const uint32_t* list0, const float* aabb, const Segs& g, const uint32_t* S_dev, uint32_t S,
                         uint32_t max_size, cudaStream_t st) {
  if (max_size <= 8) seg_bounds<1>(list0, aabb, g, S_dev, S, max_size, st);
  else if (max_size <= 32) seg_bounds<4>(list0, aabb, g, S_dev, S, max_size, st);
  else if (max_size <= 256) seg_bounds<32>(list0, aabb, g, S_dev, S, max_size, st);
  else seg_bounds<256>(list0, aabb, g, S_dev, S, max_size, st);
}

Segs segs_at(uint32_t* base, uint32_t cap) {
  Segs g;
  g.start = base;
  g.end = base + cap;
  g.parent = base + 2 * (size_t)cap;
  g.split = base + 3 * (size_t)cap;
  g.mid = base + 4 * (size_t)cap;
  g.dim = base + 5 * (size_t)cap;
  g.rank = base + 6 * (size_t)cap;
  g.box = reinterpret_cast<int32_t*>(base + 7 * (size_t)cap);  // 6 words per segment
  return g;
}

inline unsigned grid(uint64_t n) { return (unsigned)((n + kThreads - 1) / kThreads); }

}  // namespace

BuildResult build_median_bvh(const SceneView& s, AccelBuffers& a, BuildScratch& sc, uint32_t* err,
                             cudaStream_t st) {
  const uint32_t n = s.n;
  const size_t payload = s.kind == kTriangles ? 48 : 16;
  MB_TRY(a.nodes.ensure((size_t)(n > 1 ? n - 1 : 1) * 64), "BVH nodes");
  MB_TRY(a.prims.ensure((size_t)n * payload), "BVH payload");
  MB_TRY(a.order.ensure((size_t)n * 4), "BVH order");
  MB_TRY(a.root.ensure(32), "BVH root");
  // working memory
  const uint32_t cap = n + 1;  // segments per level
  MB_TRY(sc.m0.ensure((size_t)n * 9 * 4), "BVH scratch");              // aabb (6) + centroid (3)
  MB_TRY(sc.m1.ensure((size_t)n * 6 * 4), "BVH scratch");              // lists, double buffered
  MB_TRY(sc.m2.ensure((size_t)n * 3 * 4), "BVH scratch");              // sort keys / scan input
  MB_TRY(sc.m3.ensure(((size_t)n * 3 + scan_tmp_words(3ull * n) + 8) * 4), "BVH scratch");  // scan
  MB_TRY(sc.m4.ensure((size_t)n * 5), "BVH scratch");                  // seg id (4 B) + left flag (1 B)
  MB_TRY(sc.m5.ensure((size_t)cap * 13 * 4), "BVH scratch");           // segments, this level
  MB_TRY(sc.m6.ensure((size_t)cap * 13 * 4), "BVH scratch");           // segments, next level
  float* aabb = sc.m0.as<float>();
  float* cen = aabb + 6 * (size_t)n;
  uint32_t* lists = sc.m1.as<uint32_t>();
  uint32_t* lists_alt = lists + 3 * (size_t)n;
  uint32_t* keys = sc.m2.as<uint32_t>();
  uint32_t* scan = sc.m3.as<uint32_t>();
  uint32_t* scan_tmp = scan + 3 * (size_t)n;
  uint32_t* total = scan_tmp + scan_tmp_words(3ull * n) + 4;
  int32_t* seg_id = sc.m4.as<int32_t>();
  uint8_t* left = reinterpret_cast<uint8_t*>(seg_id + n);
  Segs cur = segs_at(sc.m5.as<uint32_t>(), cap), nxt = segs_at(sc.m6.as<uint32_t>(), cap);

  count_launch();
  k_prim_info<<<grid(n), kThreads, 0, st>>>(s.kind, s.verts, s.idx, s.sph, n, aabb, cen, keys, lists);
  MB_TRY(cudaGetLastError(), "BVH prim info");
  for (int ax = 0; ax < 3; ++ax) {
    BuildResult r = sort_pairs(keys + (size_t)ax * n, lists + (size_t)ax * n, n, 4, true, sc, err, st);
    if (!r.ok()) return r;
  }
  // Level 0: one segment, the root.  The host runs a fixed number of levels
  // (median splits halve the largest segment, so after ceil(log2 n) + 1
  // levels none can split) with upper bounds for the segment counts and
  // sizes; the counts themselves and each level's first node index stay on
  // the device (ctl), so the levels run without a host round trip.
  MB_TRY(sc.m7.ensure(2 * 72 * 4), "BVH scratch");
  uint32_t* ctl = sc.m7.as<uint32_t>();
  const uint32_t h_root[3] = {0u, n, kRoot}, h_ctl[2] = {1u, 0u};
  MB_TRY(cudaMemcpyAsync(cur.start, &h_root[0], 4, cudaMemcpyHostToDevice, st), "BVH init");
  MB_TRY(cudaMemcpyAsync(cur.end, &h_root[1], 4, cudaMemcpyHostToDevice, st), "BVH init");
  MB_TRY(cudaMemcpyAsync(cur.parent, &h_root[2], 4, cudaMemcpyHostToDevice, st), "BVH init");
  MB_TRY(cudaMemcpyAsync(ctl, h_ctl, 8, cudaMemcpyHostToDevice, st), "BVH init");
  uint32_t S = 1, max_size = n;  // upper bounds of this level's segments and their sizes
  int level = 0;
  for (;; ++level) {
    if (level > 64) return BuildResult::error(RQ_ERROR_INVALID_ARGUMENT, "median BVH deeper than 64 levels");
    if (max_size <= kFinishSpan) break;  // every segment finishes inside one block
    const uint32_t* S_dev = ctl + 2 * level;
    count_launch(1);
    k_seg_id<<<grid(n), kThreads, 0, st>>>(cur.start, cur.end, S_dev, n, seg_id);
    seg_bounds_dispatch(lists, aabb, cur, S_dev, S, max_size, st);
    count_launch(1);
    k_seg_decide<<<grid(S), kThreads, 0, st>>>(cur, S_dev, S, lists, n, cen);
    launch_scan_excl(cur.split, cur.rank, S, scan_tmp, total, st);
    count_launch(1);
    k_seg_link<<<grid(S), kThreads, 0, st>>>(cur, ctl, level, total, nxt, a.nodes.as<float4>(), a.root.as<float>());
    MB_TRY(cudaGetLastError(), "BVH level");
    count_launch(3);
    k_mark<<<grid(n), kThreads, 0, st>>>(cur, seg_id, lists, n, left);
    k_left_flags<<<grid(3ull * n), kThreads, 0, st>>>(cur, seg_id, lists, n, left, keys);
    launch_scan_excl(keys, scan, 3ull * n, scan_tmp, nullptr, st);
    k_partition<<<grid(3ull * n), kThreads, 0, st>>>(cur, seg_id, lists, n, left, scan, lists_alt);
    MB_TRY(cudaGetLastError(), "BVH partition");
    uint32_t* t = lists; lists = lists_alt; lists_alt = t;
    S = (uint32_t)std::min<uint64_t>(2ull * S, n);
    max_size = (max_size + 1) / 2;
    Segs tg = cur; cur = nxt; nxt = tg;
  }
  // The remaining segments (level `level`, at most S, each of at most
  // kFinishSpan primitives): count, scan, write.
  {
    int dev = 0;
    MB_TRY(cudaGetDevice(&dev), "BVH finish");
    static std::atomic<uint64_t> attr_set{0};  // devices whose k_finish allows its shared memory
    const uint64_t bit = 1ull << (dev & 63);
    if (!(attr_set.load() & bit)) {
      MB_TRY(cudaFuncSetAttribute(k_finish<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)sizeof(FinishShared)), "BVH finish");
      MB_TRY(cudaFuncSetAttribute(k_finish<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)sizeof(FinishShared)), "BVH finish");
      attr_set.fetch_or(bit);
    }
    const uint64_t cells = (uint64_t)kFinishDepth * S;
    MB_TRY(sc.keys.ensure((2 * cells + scan_tmp_words(cells) + 8) * 4), "BVH scratch");
    uint32_t* counts = sc.keys.as<uint32_t>();
    uint32_t* offs = counts + cells;
    uint32_t* ftmp = offs + cells;
    uint32_t* ftotal = ftmp + scan_tmp_words(cells) + 4;
    const uint32_t* S_dev = ctl + 2 * level;
    const uint32_t* base_dev = ctl + 2 * level + 1;
    MB_TRY(cudaMemsetAsync(counts, 0, cells * 4, st), "BVH finish");
    count_launch(1);
    k_finish<false><<<S, kFinishThreads, sizeof(FinishShared), st>>>(
        cur, S_dev, S, lists, lists + n, lists + 2 * (size_t)n, aabb, cen, reinterpret_cast<uint32_t*>(seg_id),
        counts, nullptr, nullptr, n > 1 ? n - 1 : 1, a.nodes.as<float4>(), a.root.as<float>(), err);
    launch_scan_excl(counts, offs, cells, ftmp, ftotal, st);
    count_launch(1);
    k_finish<true><<<S, kFinishThreads, sizeof(FinishShared), st>>>(
        cur, S_dev, S, lists, lists + n, lists + 2 * (size_t)n, aabb, cen, reinterpret_cast<uint32_t*>(seg_id),
        counts, offs, base_dev, n > 1 ? n - 1 : 1, a.nodes.as<float4>(), a.root.as<float>(), err);
    MB_TRY(cudaGetLastError(), "BVH finish");
    MB_TRY(cudaMemcpyAsync(ctl + 2 * 71, ftotal, 4, cudaMemcpyDeviceToDevice, st), "BVH nodes");
  }
  uint32_t h_nodes[2] = {0u, 0u};
  MB_TRY(cudaMemcpyAsync(&h_nodes[0], ctl + 2 * level + 1, 4, cudaMemcpyDeviceToHost, st), "BVH nodes");
  MB_TRY(cudaMemcpyAsync(&h_nodes[1], ctl + 2 * 71, 4, cudaMemcpyDeviceToHost, st), "BVH nodes");
  MB_TRY(cudaStreamSynchronize(st), "BVH nodes");
  const uint32_t node_base = h_nodes[0] + h_nodes[1];
  // slot order = the x-sorted list; gather the payload in that order
  MB_TRY(cudaMemcpyAsync(a.order.p, lists, (size_t)n * 4, cudaMemcpyDeviceToDevice, st), "BVH order");
  launch_prims_gather(s.kind, s.verts, s.idx, s.sph, a.order.as<uint32_t>(), n, a.prims.as<float4>(), st);
  MB_TRY(cudaGetLastError(), "BVH payload");
  a.n_nodes = node_base;
  a.n_slots = n;
  a.max_depth = 0;
  return {};
}

}  // namespace rq
