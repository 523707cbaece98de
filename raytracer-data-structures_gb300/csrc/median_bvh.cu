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
#include <algorithm>
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

// The split decision of one segment (constructBVHNew's rules).
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
  uint32_t split = 0, mid = s, dim = 0;
  if (m > 1) {
    float lo[3], hi[3];
    for (int a = 0; a < 3; ++a) {
      lo[a] = ordered_to_float(g.box[6 * (size_t)k + a]);
      hi[a] = ordered_to_float(g.box[6 * (size_t)k + 3 + a]);
      // centroid bounds seeded with the node bounds (:275-277); the extremes of
      // the centroids along axis a are the ends of that axis' sorted list
      float cmin = __ldg(cen + 3 * (size_t)lists[(size_t)a * n + s] + a);
      float cmax = __ldg(cen + 3 * (size_t)lists[(size_t)a * n + e - 1] + a);
      lo[a] = cmin < lo[a] ? cmin : lo[a];
      hi[a] = cmax > hi[a] ? cmax : hi[a];
    }
    float ax = __fsub_rn(hi[0], lo[0]), ay = __fsub_rn(hi[1], lo[1]), az = __fsub_rn(hi[2], lo[2]);
    dim = (ax > ay && ax > az) ? 0u : (ay > az ? 1u : 2u);
    if (hi[dim] != lo[dim]) {
      float pmid = __fdiv_rn(__fadd_rn(lo[dim], hi[dim]), 2.0f);
      const uint32_t* L = lists + (size_t)dim * n;
      uint32_t a = s, b = e;  // first position whose centroid is >= pmid
      while (a < b) {
        uint32_t q = (a + b) >> 1;
        if (__ldg(cen + 3 * (size_t)L[q] + dim) < pmid) a = q + 1;
        else b = q;
      }
      const uint32_t less = a - s;
      if (less != 0 && less != m) {
        split = 1;
        mid = s + m / 2;
      }
    }
  }
  g.split[k] = split;
  g.mid[k] = mid;
  g.dim[k] = dim;
}

// Write each segment into its parent (box, link, count) and emit the next
// level's segments.
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
    if (max_size <= 1) {  // no segment of this level can split: it was the last
      ++level;
      break;
    }
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
  uint32_t node_base = 0;
  MB_TRY(cudaMemcpyAsync(&node_base, ctl + 2 * level + 1, 4, cudaMemcpyDeviceToHost, st), "BVH nodes");
  MB_TRY(cudaStreamSynchronize(st), "BVH nodes");
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
