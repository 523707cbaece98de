// SAH KD tree on the GPU: constructKDTreeNew / buildTree (accelerators.h:815-988)
// built breadth first, then laid out depth first exactly as the reference lays
// it out (below child = node + 1, above child = next free node after the below
// subtree, accelerators.h:940-947), plus its traversal (kdtreeIntersect,
// accelerators.h:997-1086).
//
// Parameters are the reference's effective ones: maxPrims = 5, isectCost = 80,
// traversalCost = 1, emptyBonus = 0 (the global `char emptyBonus = 0.5f`
// truncates, accelerators.h:767-770); maxDepth = round(8 + 1.3 log2 N).
//
// Edges are sorted once: at the root, one list per axis, ordered by (t,
// start before end, primitive id), the order of buildTree's edge sort
// (:872-879) with ties in id order.  A node's edges are a contiguous segment
// of each list, and a stable partition hands every child its segments still
// sorted.  Per level, for every node still splitting:
//  * the SAH cost of every edge on every axis, with the reference's float
//    operations (no fused multiply-add); nBelow is carried with each edge;
//  * per node and axis, a 64-bit atomicMin of (cost, edge offset) takes the
//    first cheapest edge (buildTree's strict <); the axis is the first from
//    the longest on with a candidate edge, as the retries (:915-919) choose;
//  * the leaf rules (maxPrims, depth, 4x old cost under 16 primitives, three
//    bad refines, :843, :920-925) decide; primitives whose start edge precedes
//    the split go below, those whose end edge follows it go above (:928-934).
// Leaves list their primitives by id (the reference's order inside a leaf
// comes from an unstable sort).
#include <algorithm>
#include <vector>

#include "rq_build.hpp"
#include "rq_device.cuh"

namespace rq {
namespace {

constexpr int kThreads = 256;
constexpr int kMaxPrims = 5;
constexpr float kIsect = 80.f, kTrav = 1.f, kEmptyBonus = 0.f;
constexpr unsigned long long kNone = ~0ull;

inline unsigned grid(uint64_t n) { return n ? (unsigned)((n + kThreads - 1) / kThreads) : 1u; }

__device__ __forceinline__ uint32_t float_key(float f) {
  uint32_t b = __float_as_uint(__fadd_rn(f, 0.0f));
  return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float key_float(uint32_t k) {
  return __uint_as_float((k & 0x80000000u) ? (k & 0x7FFFFFFFu) : ~k);
}

// Level-local node state.
struct LevelNodes {
  float* box;         // 6 per node
  int32_t* depth;
  int32_t* bad;       // badRefines
  uint32_t* rs;       // first ref
  uint32_t* rc;       // ref count
  int32_t* axis0;     // longest axis of the node box
  unsigned long long* best;  // 3 per node, one per axis: (cost key << 32) | edge offset in the node
  int32_t* state;     // 0 undecided, 1 leaf, 2 interior
  int32_t* best_axis;
  uint32_t* best_off;
  float* tsplit;
  uint32_t* split_key;  // the split edge: ordered t key and (ref << 1 | end)
  uint32_t* split_v;
  float4* sa;           // node box extents d[0..2] and 1 / surface area, for the cost
  uint4* plan;          // interior nodes: (sA[rs], sB[rs], sB[rs + rc], first child) for the partition
};

// Edge lists: one per axis, each holding 2 edges per ref of the level (the
// node's refs' edges at [2 rs, 2 rs + 2 rc)), sorted inside every node by
// (t, start before end, ref), the order buildTree's edge sort gives
// (:872-879) with ties in primitive-id order.  Structure of arrays:
// t[a] (ordered float keys), v[a] (ref << 1 | end), n[a] (node) and s[a]
// (the number of start edges before the edge in its node: the nBelow of the
// cost, carried through the partitions).  A child's lists come
// from its parent's by a stable partition, so the edges are sorted once, at
// the root.
struct EdgeLists {
  uint32_t* base;
  size_t cap;  // edges per list
  __host__ __device__ uint32_t* t(int a) const { return base + (size_t)a * cap; }
  __host__ __device__ uint32_t* v(int a) const { return base + (size_t)(3 + a) * cap; }
  __host__ __device__ uint32_t* n(int a) const { return base + (size_t)(6 + a) * cap; }  // the edge's node
  __host__ __device__ uint32_t* s(int a) const { return base + (size_t)(9 + a) * cap; }  // start edges before it in its node
};
constexpr int kEdgeWords = 12;  // t, v, node and start-rank arrays of the three lists

// Pre-leaf test and first axis (:843, :860); also clears the level's ref
// side flags (R + 1 each).
__global__ void k_node_init(LevelNodes L, uint32_t M, uint32_t* __restrict__ below, uint32_t* __restrict__ above,
                            uint32_t R) {
  uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k <= R) {
    below[k] = 0u;
    above[k] = 0u;
  }
  if (k >= M) return;
  const float* b = L.box + 6 * (size_t)k;
  for (int a = 0; a < 3; ++a) L.best[3 * (size_t)k + a] = kNone;
  L.best_axis[k] = -1;
  if ((int)L.rc[k] <= kMaxPrims || L.depth[k] == 0) {
    L.state[k] = 1;
    return;
  }
  float ax = __fsub_rn(b[3], b[0]), ay = __fsub_rn(b[4], b[1]), az = __fsub_rn(b[5], b[2]);
  L.state[k] = 0;
  L.axis0[k] = (ax > ay && ax > az) ? 0 : (ay > az ? 1 : 2);
  // totalSA and its inverse as buildTree computes them (:855-857)
  const float totalSA = __fmul_rn(2.f, __fadd_rn(__fadd_rn(__fmul_rn(ax, ay), __fmul_rn(ax, az)), __fmul_rn(ay, az)));
  L.sa[k] = make_float4(ax, ay, az, __fdiv_rn(1.f, totalSA));
}

// Root edge lists before the sort: starts of refs 0..n-1, then their ends,
// so a stable sort by t alone orders equal t start-first and by ref.
__global__ void k_root_edges(const float* __restrict__ aabb, uint32_t n, int a, uint32_t* __restrict__ t,
                             uint32_t* __restrict__ v) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const float* q = aabb + 6 * (size_t)p;
  t[p] = float_key(__ldg(q + a));
  v[p] = p << 1;
  t[n + p] = float_key(__ldg(q + 3 + a));
  v[n + p] = (p << 1) | 1u;
}

__global__ void k_start_flags(const uint32_t* __restrict__ v, uint32_t E, uint32_t* __restrict__ f) {
  const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e < E) f[e] = (v[e] & 1u) ? 0u : 1u;
}

constexpr int kEdgeItems = 8;
constexpr uint32_t kEdgeRun = 32 * kEdgeItems;               // edges per warp: lane l takes 32 j + l in round j
constexpr uint32_t kEdgeTile = kEdgeRun * (kThreads / 32);  // edges per block of the partition passes

// SAH cost of splitting at every edge of every undecided node, on all three
// axes at once (buildTree :883-912, same float operations).  buildTree tries
// the longest axis and moves to the next only when it has no candidate edge
// (:915-919); every axis's minimum is kept and k_decide takes the first axis
// in that order that has a candidate, which is the same choice.
//
// One warp per run of 256 consecutive edges of one list, lane l taking edge
// 32 j + l in round j.  The lanes that share a node are consecutive, so each
// round takes every node's minimum by a segmented shuffle reduction; the
// run that reaches lane 31 is carried into the next round, and only runs
// that end issue an atomicMin (near the root a level has a few nodes of
// millions of edges, and one atomic per edge on one address serialises in
// L2).
__device__ __forceinline__ void flush_best(LevelNodes L, uint32_t k, int a, unsigned long long ck) {
  if (ck != kNone) atomicMin(L.best + 3 * (size_t)k + a, ck);
}

__global__ void __launch_bounds__(kThreads) k_cost(EdgeLists el, uint32_t E2, uint32_t runs_per_list, uint32_t M,
                                                   LevelNodes L, uint32_t* err) {
  const uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (gw >= 3 * runs_per_list) return;  // whole warps
  const int lane = threadIdx.x & 31;
  const int a = (int)(gw / runs_per_list);
  const uint32_t run0 = (gw - (uint32_t)a * runs_per_list) * kEdgeRun;
  const uint32_t* __restrict__ tl = el.t(a);
  const uint32_t* __restrict__ vl = el.v(a);
  const uint32_t* __restrict__ nl = el.n(a);
  const uint32_t* __restrict__ sl = el.s(a);
  uint32_t carry_k = 0xFFFFFFFFu;  // the open run from the previous round (warp-uniform)
  unsigned long long carry = kNone;
#pragma unroll 2
  for (int j = 0; j < kEdgeItems; ++j) {
    const uint32_t e = run0 + 32 * j + lane;
    const bool in = e < E2;
    uint32_t k = in ? __ldg(nl + e) : 0xFFFFFFFFu;
    if (in && k >= M) { atomicOr(err, kErrCorrupt); k = 0xFFFFFFFFu; }
    unsigned long long ck = kNone;
    if (k != 0xFFFFFFFFu && L.state[k] == 0) {
      const float t = key_float(__ldg(tl + e));
      const float* b = L.box + 6 * (size_t)k;
      const float lo = b[a], hi = b[3 + a];
      if (t > lo && t < hi) {
        const uint32_t rs = L.rs[k], n = L.rc[k];
        const uint32_t nBelow = __ldg(sl + e);
        const uint32_t off = e - 2 * rs;
        const uint32_t nEndIncl = off - nBelow + (__ldg(vl + e) & 1u);
        const uint32_t nAbove = n - nEndIncl;
        const float4 q = L.sa[k];
        const float invTotalSA = q.w;
        const float d0 = a == 0 ? q.y : a == 1 ? q.z : q.x;  // the other two axes, (a + 1) % 3 and (a + 2) % 3
        const float d1 = a == 0 ? q.z : a == 1 ? q.x : q.y;
        float dd = __fmul_rn(d0, d1), ds = __fadd_rn(d0, d1);
        float belowSA = __fmul_rn(2.f, __fadd_rn(dd, __fmul_rn(__fsub_rn(t, lo), ds)));
        float aboveSA = __fmul_rn(2.f, __fadd_rn(dd, __fmul_rn(__fsub_rn(hi, t), ds)));
        float pB = __fmul_rn(belowSA, invTotalSA), pA = __fmul_rn(aboveSA, invTotalSA);
        float eb = (nAbove == 0 || nBelow == 0) ? kEmptyBonus : 0.f;
        float cost = __fadd_rn(kTrav, __fmul_rn(__fmul_rn(kIsect, __fsub_rn(1.f, eb)),
                                                __fadd_rn(__fmul_rn(pB, (float)nBelow),
                                                          __fmul_rn(pA, (float)nAbove))));
        ck = ((unsigned long long)float_key(cost) << 32) | (unsigned long long)off;
      }
    }
    // Minimum over the lane's run of equal nodes from this lane on.
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned long long x = __shfl_down_sync(0xffffffffu, ck, o);
      const uint32_t kk = __shfl_down_sync(0xffffffffu, k, o);
      if (lane + o < 32 && kk == k && x < ck) ck = x;
    }
    const uint32_t kprev = __shfl_up_sync(0xffffffffu, k, 1);
    const bool head = lane == 0 || kprev != k;
    const uint32_t heads = __ballot_sync(0xffffffffu, head);
    const int last = 31 - __clz(heads);  // head of the run that reaches lane 31
    // the carried run continues into lane 0's run or ends here
    const uint32_t k0 = __shfl_sync(0xffffffffu, k, 0);
    if (lane == 0) {
      if (carry_k == k0) { if (carry < ck) ck = carry; }
      else if (carry_k != 0xFFFFFFFFu) flush_best(L, carry_k, a, carry);
    }
    if (head && lane != last && k != 0xFFFFFFFFu) flush_best(L, k, a, ck);
    carry_k = __shfl_sync(0xffffffffu, k, last);
    carry = __shfl_sync(0xffffffffu, ck, last);
  }
  if (lane == 0 && carry_k != 0xFFFFFFFFu) flush_best(L, carry_k, a, carry);
}

// Split decision (:915-925): the first axis from the longest on with a
// candidate edge; none -> leaf.
__device__ void decide_node(EdgeLists el, LevelNodes L, uint32_t k, uint32_t E2, uint32_t* err);

// Decides every undecided node, then writes each node's interior flag and
// leaf ref count (M + 1 entries, the last 0) for the level's scans.
__global__ void k_decide(EdgeLists el, LevelNodes L, uint32_t M, uint32_t E2, uint32_t* __restrict__ iflag,
                         uint32_t* __restrict__ lcnt, uint32_t* err) {
  uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k > M) return;
  if (k == M) {
    iflag[k] = 0u;
    lcnt[k] = 0u;
    return;
  }
  if (L.state[k] == 0) decide_node(el, L, k, E2, err);
  const int st = L.state[k];
  iflag[k] = st == 2 ? 1u : 0u;
  lcnt[k] = st == 1 ? L.rc[k] : 0u;
}

__device__ void decide_node(EdgeLists el, LevelNodes L, uint32_t k, uint32_t E2, uint32_t* err) {
  for (int q = 0; q < 3; ++q) {
    const int a = (L.axis0[k] + q) % 3;
    const unsigned long long b = L.best[3 * (size_t)k + a];
    if (b == kNone) continue;
    const float bestCost = key_float((uint32_t)(b >> 32));
    const float oldCost = __fmul_rn(kIsect, (float)L.rc[k]);
    const int bad = L.bad[k] + (bestCost > oldCost ? 1 : 0);
    L.bad[k] = bad;
    const bool leaf = (bestCost > __fmul_rn(4.f, oldCost) && L.rc[k] < 16) || bad == 3;
    L.state[k] = leaf ? 1 : 2;
    L.best_axis[k] = a;
    const uint32_t off = (uint32_t)(b & 0xFFFFFFFFull), e = 2 * L.rs[k] + off;
    L.best_off[k] = off;
    if (e >= E2) { atomicOr(err, kErrCorrupt); L.state[k] = 1; return; }
    const uint32_t key = el.t(a)[e];
    L.split_key[k] = key;
    L.split_v[k] = el.v(a)[e];
    L.tsplit[k] = key_float(key);
    return;
  }
  L.state[k] = 1;  // no split found on any axis
}

// Below/above sides (:928-934): a ref whose start edge precedes the split
// edge in the chosen axis's sorted order goes below, one whose end edge
// follows it goes above.  The order is (t key, start before end, ref), so
// the comparison needs only the ref's box and the split edge, not the list.
__global__ void k_classify(const uint32_t* __restrict__ ref_prim, const uint32_t* __restrict__ ref_node,
                           uint32_t R, uint32_t M, const float* __restrict__ aabb, LevelNodes L,
                           uint32_t* __restrict__ below, uint32_t* __restrict__ above, uint32_t* err) {
  const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= R) return;
  const uint32_t k = __ldg(ref_node + r);
  if (k >= M) { atomicOr(err, kErrCorrupt); return; }
  if (L.state[k] != 2) return;
  const int a = L.best_axis[k];
  const uint32_t sk = L.split_key[k], sv = L.split_v[k], sr = sv >> 1;
  const float* q = aabb + 6 * (size_t)__ldg(ref_prim + r);
  const uint32_t lo = float_key(__ldg(q + a)), hi = float_key(__ldg(q + 3 + a));
  below[r] = (lo < sk || (lo == sk && ((sv & 1u) || r < sr))) ? 1u : 0u;   // (lo, start, r) < split
  above[r] = (hi > sk || (hi == sk && (!(sv & 1u) || r > sr))) ? 1u : 0u;  // (hi, end, r) > split
}

// Children's edge lists: a stable partition of every interior node's edges,
// on each axis, into its below child (refs with below[r]) and above child
// (refs with above[r]); straddling refs go to both.  With sB / sA the
// exclusive scans of below / above over the level's refs, and BS, BE, AS, AE
// the list-wide counts of below-start, below-end, above-start and above-end
// edges before e:
//   below child: position BS + BE + 2 sA[rs], ref sA[rs] + sB[r],
//                start rank BS - sB[rs]
//   above child: position AS + AE + 2 sB[re], ref sB[re] + sA[r],
//                start rank AS - sA[rs]
// (re = rs + rc; children are laid out node by node, below before above,
// and leaf refs count in neither scan), matching k_emit_refs's numbering of
// the refs.  Per node the bases come from plan[k] = (sA[rs], sB[rs], sB[re],
// first child), written by k_spawn.
//
// Three passes, none waiting on another block: k_part_count counts each
// tile's (BS, BE) and (AS, AE), packed 31 bits apiece in two 64-bit words
// (lists hold fewer than 2^31 edges, so the fields never carry), and keeps
// the side flags as one ballot word per 32 edges; k_part_scan turns the tile
// counts of each list into exclusive prefixes; k_partition adds the warp
// offsets inside the tile and scatters.
__global__ void __launch_bounds__(kThreads) k_part_count(EdgeLists el, uint32_t E2, uint32_t tiles_per_list,
                                                         uint32_t R, uint32_t M, const uint32_t* __restrict__ below,
                                                         const uint32_t* __restrict__ above,
                                                         uint32_t* __restrict__ sideB, uint32_t* __restrict__ sideA,
                                                         unsigned long long* __restrict__ tile_cnt, uint32_t* err) {
  __shared__ unsigned long long wsum[2][kThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t tile = blockIdx.x, a = tile / tiles_per_list;
  const uint32_t run0 = (tile - a * tiles_per_list) * kEdgeTile + (uint32_t)warp * kEdgeRun;
  const size_t words = (size_t)(E2 + 31) / 32;  // ballot words per list
  unsigned long long t0 = 0, t1 = 0;
#pragma unroll
  for (int j = 0; j < kEdgeItems; ++j) {
    const uint32_t e = run0 + 32 * j + lane;
    const bool in = e < E2;
    const uint32_t v = in ? __ldg(el.v(a) + e) : 0u;
    bool b = false, ab = false;
    if (in) {
      const uint32_t r = v >> 1, k = __ldg(el.n(a) + e);
      if (r < R && k < M) {
        b = __ldg(below + r) != 0u;
        ab = __ldg(above + r) != 0u;
      } else {
        atomicOr(err, kErrCorrupt);
      }
    }
    const uint32_t kb = __ballot_sync(0xffffffffu, b), ka = __ballot_sync(0xffffffffu, ab);
    const uint32_t em = __ballot_sync(0xffffffffu, (v & 1u) != 0u);
    const uint32_t w = (run0 >> 5) + (uint32_t)j;
    if (lane == 0 && w < words) {
      sideB[(size_t)a * words + w] = kb;
      sideA[(size_t)a * words + w] = ka;
    }
    t0 += ((unsigned long long)__popc(kb & em) << 31) | (unsigned long long)__popc(kb & ~em);
    t1 += ((unsigned long long)__popc(ka & em) << 31) | (unsigned long long)__popc(ka & ~em);
  }
  if (lane == 0) {
    wsum[0][warp] = t0;
    wsum[1][warp] = t1;
  }
  __syncthreads();
  if (threadIdx.x < 2) {
    unsigned long long x = 0;
    for (int w = 0; w < kThreads / 32; ++w) x += wsum[threadIdx.x][w];
    tile_cnt[2 * (size_t)tile + threadIdx.x] = x;
  }
}

// Exclusive prefix of the tile counts of list blockIdx.x, both words, in
// place (one block per list; each thread sums a contiguous chunk).
__global__ void __launch_bounds__(1024) k_part_scan(unsigned long long* tile_cnt, uint32_t tiles_per_list) {
  __shared__ unsigned long long part[2][1024];
  const uint32_t t = threadIdx.x, per = (tiles_per_list + 1023) / 1024;
  unsigned long long* c = tile_cnt + 2 * (size_t)blockIdx.x * tiles_per_list;
  const uint32_t lo = t * per, hi = min(lo + per, tiles_per_list);
  unsigned long long s0 = 0, s1 = 0;
  for (uint32_t i = lo; i < hi; ++i) {
    s0 += c[2 * (size_t)i];
    s1 += c[2 * (size_t)i + 1];
  }
  part[0][t] = s0;
  part[1][t] = s1;
  __syncthreads();
  for (uint32_t o = 1; o < 1024; o <<= 1) {  // inclusive Hillis-Steele scan of the chunk sums
    const unsigned long long x0 = t >= o ? part[0][t - o] : 0ull, x1 = t >= o ? part[1][t - o] : 0ull;
    __syncthreads();
    part[0][t] += x0;
    part[1][t] += x1;
    __syncthreads();
  }
  unsigned long long r0 = part[0][t] - s0, r1 = part[1][t] - s1;
  for (uint32_t i = lo; i < hi; ++i) {
    const unsigned long long v0 = c[2 * (size_t)i], v1 = c[2 * (size_t)i + 1];
    c[2 * (size_t)i] = r0;
    c[2 * (size_t)i + 1] = r1;
    r0 += v0;
    r1 += v1;
  }
}

__global__ void __launch_bounds__(kThreads) k_partition(EdgeLists el, uint32_t E2, uint32_t tiles_per_list,
                                                        LevelNodes L, const uint32_t* __restrict__ sideB,
                                                        const uint32_t* __restrict__ sideA,
                                                        const unsigned long long* __restrict__ tile_pre,
                                                        const uint32_t* __restrict__ sB,
                                                        const uint32_t* __restrict__ sA, EdgeLists out,
                                                        uint32_t E2next, uint32_t* err) {
  __shared__ unsigned long long wpre[2][kThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t tile = blockIdx.x, a = tile / tiles_per_list;
  const uint32_t run0 = (tile - a * tiles_per_list) * kEdgeTile + (uint32_t)warp * kEdgeRun;
  const size_t words = (size_t)(E2 + 31) / 32;
  // Side-flag words and end-edge ballots of round j (read twice: for the
  // warp totals, then for the scatter; the second read hits the cache).
  auto round_flags = [&](int j, uint32_t& kb, uint32_t& ka, uint32_t& em, uint32_t& v) {
    const uint32_t e = run0 + 32 * j + lane;
    const uint32_t w = (run0 >> 5) + (uint32_t)j;
    const bool wv = w < words;
    kb = wv ? __ldg(sideB + (size_t)a * words + w) : 0u;
    ka = wv ? __ldg(sideA + (size_t)a * words + w) : 0u;
    v = e < E2 ? __ldg(el.v(a) + e) : 0u;
    em = __ballot_sync(0xffffffffu, (v & 1u) != 0u);
  };
  unsigned long long t0 = 0, t1 = 0;
#pragma unroll
  for (int j = 0; j < kEdgeItems; ++j) {
    uint32_t kb, ka, em, v;
    round_flags(j, kb, ka, em, v);
    t0 += ((unsigned long long)__popc(kb & em) << 31) | (unsigned long long)__popc(kb & ~em);
    t1 += ((unsigned long long)__popc(ka & em) << 31) | (unsigned long long)__popc(ka & ~em);
  }
  if (lane == 0) {
    wpre[0][warp] = t0;
    wpre[1][warp] = t1;
  }
  __syncthreads();
  unsigned long long p0 = __ldg(tile_pre + 2 * (size_t)tile), p1 = __ldg(tile_pre + 2 * (size_t)tile + 1);
  for (int w = 0; w < warp; ++w) {
    p0 += wpre[0][w];
    p1 += wpre[1][w];
  }
  uint32_t cbs = (uint32_t)(p0 & 0x7FFFFFFFull), cbe = (uint32_t)(p0 >> 31);
  uint32_t cas = (uint32_t)(p1 & 0x7FFFFFFFull), cae = (uint32_t)(p1 >> 31);
  const uint32_t lt = (1u << lane) - 1u, me = 1u << lane;
#pragma unroll 2
  for (int j = 0; j < kEdgeItems; ++j) {
    uint32_t kb, ka, em, v;
    round_flags(j, kb, ka, em, v);
    const uint32_t bs = kb & ~em, be = kb & em, as = ka & ~em, ae = ka & em;
    const bool b = (kb & me) != 0u, ab = (ka & me) != 0u;
    if (b || ab) {
      const uint32_t e = run0 + 32 * j + lane;
      const uint32_t tk = __ldg(el.t(a) + e), k = __ldg(el.n(a) + e);
      const uint32_t r = v >> 1, end = v & 1u;
      const uint4 pl = L.plan[k];  // (sA[rs], sB[rs], sB[re], first child)
      if (b) {
        const uint32_t nbs = cbs + __popc(bs & lt), nbe = cbe + __popc(be & lt);
        const uint32_t pos = nbs + nbe + 2 * pl.x;
        if (pos >= E2next) { atomicOr(err, kErrCorrupt); }
        else {
          out.t(a)[pos] = tk;
          out.v(a)[pos] = ((pl.x + __ldg(sB + r)) << 1) | end;
          out.n(a)[pos] = pl.w;
          out.s(a)[pos] = nbs - pl.y;
        }
      }
      if (ab) {
        const uint32_t nas = cas + __popc(as & lt), nae = cae + __popc(ae & lt);
        const uint32_t pos = nas + nae + 2 * pl.z;
        if (pos >= E2next) { atomicOr(err, kErrCorrupt); }
        else {
          out.t(a)[pos] = tk;
          out.v(a)[pos] = ((pl.z + __ldg(sA + r)) << 1) | end;
          out.n(a)[pos] = pl.w + 1;
          out.s(a)[pos] = nas - pl.x;
        }
      }
    }
    cbs += __popc(bs);
    cbe += __popc(be);
    cas += __popc(as);
    cae += __popc(ae);
  }
}


// Global node table (breadth-first ids).
struct Table {
  int32_t* leaf;        // 1 leaf, 0 interior
  int32_t* axis;
  float* split;
  uint32_t* child0;
  uint32_t* child1;
  uint32_t* count;      // leaf primitive count
  uint32_t* pool_off;   // leaf primitives in the pool
};

// Interior nodes spawn their two children; every node fills its table entry.
__global__ void k_spawn(LevelNodes L, uint32_t M, const uint32_t* __restrict__ irank, const uint32_t* __restrict__ sB,
                        const uint32_t* __restrict__ sA, const uint32_t* __restrict__ lrank_cnt, uint32_t pool_base,
                        uint32_t level_base, uint32_t next_base, Table T, LevelNodes N,
                        uint32_t* __restrict__ child_cnt, uint32_t M2, uint32_t* err) {
  uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k == 0) child_cnt[M2] = 0u;  // the scan's last entry
  if (k >= M) return;
  const uint32_t g = level_base + k;
  const uint32_t rs = L.rs[k], rc = L.rc[k];
  if (L.state[k] != 2) {
    T.leaf[g] = 1;
    T.count[g] = rc;
    T.pool_off[g] = pool_base + lrank_cnt[k];
    return;
  }
  const uint32_t c = 2 * irank[k];
  if (c + 1 >= M2 + 1 || L.best_axis[k] < 0) { atomicOr(err, kErrCorrupt); return; }
  const int axis = L.best_axis[k];
  const float ts = L.tsplit[k];
  T.leaf[g] = 0;
  T.axis[g] = axis;
  T.split[g] = ts;
  T.child0[g] = next_base + c;
  T.child1[g] = next_base + c + 1;
  const float* b = L.box + 6 * (size_t)k;
  for (int side = 0; side < 2; ++side) {
    float* nb = N.box + 6 * (size_t)(c + side);
    for (int q = 0; q < 6; ++q) nb[q] = b[q];
    if (side == 0) nb[3 + axis] = ts;  // bounds0.max[axis] = tSplit
    else nb[axis] = ts;                // bounds1.min[axis] = tSplit
    N.depth[c + side] = L.depth[k] - 1;
    N.bad[c + side] = L.bad[k];
  }
  child_cnt[c] = sB[rs + rc] - sB[rs];
  child_cnt[c + 1] = sA[rs + rc] - sA[rs];
  L.plan[k] = make_uint4(sA[rs], sB[rs], sB[rs + rc], c);
}

__global__ void k_set_ref_starts(LevelNodes N, uint32_t M2, const uint32_t* __restrict__ child_cnt,
                                 const uint32_t* __restrict__ child_off) {
  uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= M2) return;
  N.rs[c] = child_off[c];
  N.rc[c] = child_cnt[c];
}

// Stable filter of every interior node's refs into its children; leaf refs to the pool.
__global__ void k_emit_refs(const uint32_t* __restrict__ ref_prim, const uint32_t* __restrict__ ref_node, uint32_t R,
                            LevelNodes L, const uint32_t* __restrict__ irank, const uint32_t* __restrict__ below,
                            const uint32_t* __restrict__ above, const uint32_t* __restrict__ sB,
                            const uint32_t* __restrict__ sA, LevelNodes N, uint32_t* __restrict__ out_prim,
                            uint32_t* __restrict__ out_node, const uint32_t* __restrict__ lrank_cnt,
                            uint32_t pool_base, uint32_t* __restrict__ pool, uint32_t R2, uint32_t pool_cap,
                            uint32_t* err) {
  uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= R) return;
  const uint32_t k = ref_node[r];
  const uint32_t p = ref_prim[r];
  const uint32_t rs = L.rs[k];
  if (L.state[k] != 2) {
    const uint32_t q = pool_base + lrank_cnt[k] + (r - rs);
    if (q >= pool_cap) { atomicOr(err, kErrCorrupt); return; }
    pool[q] = p;
    return;
  }
  const uint32_t c = 2 * irank[k];
  if (below[r]) {
    const uint32_t o = N.rs[c] + (sB[r] - sB[rs]);
    if (o >= R2) { atomicOr(err, kErrCorrupt); return; }
    out_prim[o] = p;
    out_node[o] = c;
  }
  if (above[r]) {
    const uint32_t o = N.rs[c + 1] + (sA[r] - sA[rs]);
    if (o >= R2) { atomicOr(err, kErrCorrupt); return; }
    out_prim[o] = p;
    out_node[o] = c + 1;
  }
}

// Depth-first layout: subtree sizes bottom-up, positions top-down.
__global__ void k_sizes(Table T, uint32_t lo, uint32_t hi, uint32_t* __restrict__ size, uint32_t total,
                        uint32_t* err) {
  uint32_t g = lo + blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= hi) return;
  if (!T.leaf[g] && (T.child0[g] >= total || T.child1[g] >= total)) { atomicOr(err, kErrCorrupt); size[g] = 1; return; }
  size[g] = T.leaf[g] ? 1u : 1u + size[T.child0[g]] + size[T.child1[g]];
}

__global__ void k_positions(Table T, uint32_t lo, uint32_t hi, const uint32_t* __restrict__ size,
                            uint32_t* __restrict__ pos, uint32_t total) {
  uint32_t g = lo + blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= hi || T.leaf[g]) return;
  if (T.child0[g] >= total || T.child1[g] >= total) return;
  const uint32_t p = pos[g];
  pos[T.child0[g]] = p + 1;
  pos[T.child1[g]] = p + 1 + size[T.child0[g]];
}

__global__ void k_leaf_counts(Table T, uint32_t total, const uint32_t* __restrict__ pos, uint32_t* __restrict__ cnt) {
  uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g > total) return;
  if (g == total) { cnt[total] = 0; return; }
  if (pos[g] >= total) return;
  cnt[pos[g]] = (T.leaf[g] && T.count[g] >= 2) ? T.count[g] : 0u;
}

// Final KdAccelNode words (accelerators.h:718-761) and leaf primitive indices.
__global__ void k_write_nodes(Table T, uint32_t total, const uint32_t* __restrict__ pos,
                              const uint32_t* __restrict__ off, const uint32_t* __restrict__ pool,
                              int4* __restrict__ nodes, int32_t* __restrict__ prim_idx, uint32_t n_idx,
                              uint32_t pool_cap, uint32_t* err) {
  uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= total) return;
  const uint32_t p = pos[g];
  if (p >= total) { atomicOr(err, kErrCorrupt); return; }
  if (T.leaf[g] && (T.pool_off[g] + T.count[g] > pool_cap ||
                    (T.count[g] >= 2 && off[p] + T.count[g] > n_idx))) {
    atomicOr(err, kErrCorrupt);
    return;
  }
  if (!T.leaf[g] && T.child1[g] >= total) { atomicOr(err, kErrCorrupt); return; }
  if (T.leaf[g]) {
    const uint32_t np = T.count[g];
    int w0 = 0;
    if (np == 1) w0 = (int)pool[T.pool_off[g]];
    else if (np >= 2) {
      w0 = (int)off[p];
      for (uint32_t i = 0; i < np; ++i) prim_idx[off[p] + i] = (int)pool[T.pool_off[g] + i];
    }
    nodes[p] = make_int4(w0, 3 | (int)(np << 2), (int)np, 0);
  } else {
    nodes[p] = make_int4(__float_as_int(T.split[g]), T.axis[g] | (int)(pos[T.child1[g]] << 2), 0, 0);
  }
}

// ------------------------------------------------------------- traversal

struct Todo {
  int node;
  float tMin, tMax;
};

// The walk of ray r; returns whether an any-hit query found a hit (closest-hit
// queries store their hit).
template <int KIND, bool ANY, bool REF>
__device__ __forceinline__ bool kd_walk_ray(const KdView& kd, uint32_t n_nodes, const float4* __restrict__ rays,
                                            uint32_t r, float4* __restrict__ hits, uint32_t* err) {
  bool occluded = false;
  {
    float4 ra = __ldg(rays + 2 * (size_t)r), rb = __ldg(rays + 2 * (size_t)r + 1);
    F3 o = {ra.x, ra.y, ra.z}, d = {rb.x, rb.y, rb.z};
    const float rtmin = ra.w, rtmax = rb.w;
    float best = rtmax, bu = 0.f, bv = 0.f;
    uint32_t bprim = kMiss;
    F3 inv = {__frcp_rn(d.x), __frcp_rn(d.y), __frcp_rn(d.z)};
    const float* R = kd.root;
    float tMin, tMax;
    bool in;
    if (REF) {
      in = box_ref(o, d, R[0], R[3], R[1], R[4], R[2], R[5], tMin, tMax);
    } else {
      float tn;
      const SlabRay sr = slab_ray(o, d);
      if (zero_dir(sr)) {  // the exact box test (rq_device.cuh)
        in = slab_box<true>(sr, o, R[0], R[3], R[1], R[4], R[2], R[5], rtmin, best, tn);
        tMax = __fmaf_rn(slab_exit<true>(sr, o, R[0], R[3], R[1], R[4], R[2], R[5], best), kWidenExact, sr.eps);
      } else {
        in = slab_box<false>(sr, o, R[0], R[3], R[1], R[4], R[2], R[5], rtmin, best, tn);
        tMax = __fmaf_rn(slab_exit<false>(sr, o, R[0], R[3], R[1], R[4], R[2], R[5], best), kWiden, sr.eps);
      }
      tMin = tn;
    }
    if (in) {
      Todo todo[kStackSize];
      int tp = 0, node = 0;
      const float oo[3] = {o.x, o.y, o.z}, dv[3] = {d.x, d.y, d.z}, iv[3] = {inv.x, inv.y, inv.z};
      uint32_t steps = 0;
      // While-while: descend interior nodes to a leaf, then test the leaf, so
      // the lanes of a warp test their leaves together (one loop over node
      // kinds left lanes of both kinds waiting on each other at every step).
      // The per-ray order of visits is unchanged.
      const uint32_t limit = 2u * n_nodes + 8u;
      bool bad = false;
      for (;;) {
        if (++steps > limit) { atomicOr(err, kErrCorrupt); break; }
        if (!REF && best < tMin) break;
        int4 w = __ldg(kd.nodes + node);
        while ((w.y & 3) != 3) {
          const int axis = w.y & 3;
          const float split = __int_as_float(w.x);
          const float tPlane = __fmul_rn(__fsub_rn(split, oo[axis]), iv[axis]);
          const bool belowFirst = (oo[axis] < split) || (oo[axis] == split && dv[axis] <= 0.f);
          const int above = w.y >> 2;
          const int first = belowFirst ? node + 1 : above, second = belowFirst ? above : node + 1;
          if (tPlane > tMax || tPlane <= 0.f) {
            node = first;
          } else if (tPlane < tMin) {
            node = second;
          } else {
            if (tp >= kStackSize) { atomicOr(err, kErrStackOverflow); bad = true; break; }
            todo[tp++] = {second, tPlane, tMax};
            node = first;
            tMax = tPlane;
          }
          if (++steps > limit) { atomicOr(err, kErrCorrupt); bad = true; break; }
          w = __ldg(kd.nodes + node);
        }
        if (bad) break;
        const int np = w.z;
        bool done = false;
        for (int i = 0; i < np; ++i) {
          const uint32_t id = (uint32_t)(np == 1 ? w.x : __ldg(kd.prim_idx + w.x + i));
          if (KIND == kTriangles) {
            const float4* q = kd.prims + 3 * (size_t)id;
            float t, u, v;
            if (tri_mt(__ldg(q), __ldg(q + 1), __ldg(q + 2), o, d, rtmin, ANY ? rtmax : best, t, u, v)) {
              if (ANY) { done = true; break; }
              best = t; bprim = id; bu = u; bv = v;
            }
          } else {
            const float4 s = __ldg(kd.prims + id);
            if (ANY || REF) {
              float t0, t1, t;
              if (REF ? sphere_ref(s, o, d, t0, t1) : sphere_closest(s, o, d, rtmin, rtmax, false, t)) {
                if (ANY) { done = true; break; }
              }
            }
            if (!ANY) {
              float t;
              if (sphere_closest(s, o, d, rtmin, best, REF, t)) { best = t; bprim = id; bu = bv = 0.f; }
            }
          }
        }
        if (done) { occluded = true; break; }
        if (tp > 0) {
          --tp;
          node = todo[tp].node;
          tMin = todo[tp].tMin;
          tMax = todo[tp].tMax;
        } else {
          break;
        }
      }
    }
    if (!ANY) hits[r] = make_float4(best, __uint_as_float(bprim), bu, bv);
  }
  return occluded;
}

template <int KIND, bool ANY, bool REF>
__global__ void __launch_bounds__(128) k_trace_kd(KdView kd, uint32_t n_nodes, const float4* __restrict__ rays,
                                                  uint32_t n, float4* __restrict__ hits,
                                                  uint32_t* __restrict__ occ, uint32_t* err) {
  const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  const bool occluded = r < n && kd_walk_ray<KIND, ANY, REF>(kd, n_nodes, rays, r, hits, err);
  if (ANY) {
    uint32_t bits = __ballot_sync(0xffffffffu, occluded);
    uint32_t w0 = blockIdx.x * blockDim.x + (threadIdx.x & ~31u);
    if ((threadIdx.x & 31) == 0 && w0 < n) occ[w0 >> 5] = bits;
  }
}

// The same walk as persistent warps: a grid the GPU holds at once, each warp
// taking the next 32 rays from a counter (work, zeroed) until none are left.
template <int KIND, bool ANY, bool REF>
__global__ void __launch_bounds__(128) k_trace_kd_warps(KdView kd, uint32_t n_nodes, const float4* __restrict__ rays,
                                                        uint32_t n, float4* __restrict__ hits,
                                                        uint32_t* __restrict__ occ, uint32_t* err, uint32_t* work) {
  const uint32_t lane = threadIdx.x & 31;
  for (;;) {
    uint32_t base = 0;
    if (lane == 0) base = atomicAdd(work, 32u);
    base = __shfl_sync(0xffffffffu, base, 0);
    if (base >= n) break;
    const uint32_t r = base + lane;
    const bool occluded = r < n && kd_walk_ray<KIND, ANY, REF>(kd, n_nodes, rays, r, hits, err);
    if (ANY) {
      const uint32_t bits = __ballot_sync(0xffffffffu, occluded);
      if (lane == 0) occ[base >> 5] = bits;
    }
  }
}

template <typename K>
uint32_t kd_resident_blocks(K k) {
  int per_sm = 0, dev = 0, sms = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, 128, 0) != cudaSuccess || per_sm < 1) per_sm = 1;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      sms < 1)
    sms = 1;
  return (uint32_t)(per_sm * sms);
}

template <int KIND, bool ANY>
void dispatch_kd(int traversal, const KdView& v, uint32_t n_nodes, const float4* rays, uint32_t n, float4* hits,
                 uint32_t* occ, uint32_t* err, uint32_t* work, cudaStream_t s) {
  const unsigned g = (n + 127) / 128;
  if (work) {
    cudaMemsetAsync(work, 0, 4, s);
    const auto k = traversal == RQ_TRAVERSAL_REFERENCE ? k_trace_kd_warps<KIND, ANY, true> : k_trace_kd_warps<KIND, ANY, false>;
    k<<<std::min(g, kd_resident_blocks(k)), 128, 0, s>>>(v, n_nodes, rays, n, hits, occ, err, work);
  } else if (traversal == RQ_TRAVERSAL_REFERENCE) {
    k_trace_kd<KIND, ANY, true><<<g, 128, 0, s>>>(v, n_nodes, rays, n, hits, occ, err);
  } else {
    k_trace_kd<KIND, ANY, false><<<g, 128, 0, s>>>(v, n_nodes, rays, n, hits, occ, err);
  }
}

__global__ void k_box_union(const float* __restrict__ aabb, uint32_t n, int32_t* lohi) {
  float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x)
    for (int a = 0; a < 3; ++a) {
      lo[a] = fminf(lo[a], aabb[6 * (size_t)p + a]);
      hi[a] = fmaxf(hi[a], aabb[6 * (size_t)p + 3 + a]);
    }
  for (int a = 0; a < 3; ++a)
    for (int o = 16; o > 0; o >>= 1) {
      lo[a] = fminf(lo[a], __shfl_xor_sync(0xffffffffu, lo[a], o));
      hi[a] = fmaxf(hi[a], __shfl_xor_sync(0xffffffffu, hi[a], o));
    }
  if ((threadIdx.x & 31) == 0)
    for (int a = 0; a < 3; ++a) {
      atomicMin(lohi + a, float_to_ordered(lo[a]));
      atomicMax(lohi + 3 + a, float_to_ordered(hi[a]));
    }
}

__global__ void k_iota(uint32_t* v, uint32_t n) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) v[i] = i;
}

__global__ void k_root_box(const int32_t* lohi, float* box, float* root) {
  int q = threadIdx.x;
  if (q < 6) {
    float v = ordered_to_float(lohi[q]);
    box[q] = v;
    root[q] = v;
  }
}

// Grow a buffer keeping its first `used` bytes.
cudaError_t grow_keep(DevBuf& b, size_t bytes, size_t used, cudaStream_t st) {
  if (bytes <= b.cap && b.p) return cudaSuccess;
  void* p = nullptr;
  size_t want = bytes + bytes / 2 + 256;
  cudaError_t e = cudaMalloc(&p, want);
  if (e != cudaSuccess) return e;
  if (used && b.p) {
    e = cudaMemcpyAsync(p, b.p, used, cudaMemcpyDeviceToDevice, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
      cudaFree(p);
      return e;
    }
  }
  if (b.p) cudaFree(b.p);
  b.p = p;
  b.cap = want;
  return cudaSuccess;
}

// Grow a scratch buffer that queued kernels may still read: wait for them
// first (the level loop does not otherwise wait at the end of a level).
cudaError_t ensure_after(DevBuf& b, size_t bytes, cudaStream_t st) {
  if (bytes <= b.cap && b.p) return cudaSuccess;
  const cudaError_t e = cudaStreamSynchronize(st);
  return e != cudaSuccess ? e : b.ensure(bytes);
}

#define KD_TRY(call, what)                                           \
  do {                                                               \
    cudaError_t e_ = (call);                                         \
    if (e_ != cudaSuccess) return BuildResult::cuda_error(e_, what); \
  } while (0)

// Level node arrays carved from one buffer.
LevelNodes carve(char* base, uint32_t cap) {
  LevelNodes L;
  size_t o = 0;
  auto take = [&](size_t bytes) { char* p = base + o; o += (bytes + 255) & ~size_t(255); return p; };
  L.box = (float*)take((size_t)cap * 24);
  L.depth = (int32_t*)take((size_t)cap * 4);
  L.bad = (int32_t*)take((size_t)cap * 4);
  L.rs = (uint32_t*)take((size_t)cap * 4);
  L.rc = (uint32_t*)take((size_t)cap * 4);
  L.axis0 = (int32_t*)take((size_t)cap * 4);
  L.best = (unsigned long long*)take((size_t)cap * 24);
  L.state = (int32_t*)take((size_t)cap * 4);
  L.best_axis = (int32_t*)take((size_t)cap * 4);
  L.best_off = (uint32_t*)take((size_t)cap * 4);
  L.tsplit = (float*)take((size_t)cap * 4);
  L.split_key = (uint32_t*)take((size_t)cap * 4);
  L.split_v = (uint32_t*)take((size_t)cap * 4);
  L.sa = (float4*)take((size_t)cap * 16);
  L.plan = (uint4*)take((size_t)cap * 16);
  return L;
}
size_t level_bytes(uint32_t cap) { return (size_t)cap * 124 + 16 * 256; }

Table table_at(char* base, uint32_t cap) {
  Table T;
  size_t o = 0;
  auto take = [&](size_t bytes) { char* p = base + o; o += (bytes + 255) & ~size_t(255); return p; };
  T.leaf = (int32_t*)take((size_t)cap * 4);
  T.axis = (int32_t*)take((size_t)cap * 4);
  T.split = (float*)take((size_t)cap * 4);
  T.child0 = (uint32_t*)take((size_t)cap * 4);
  T.child1 = (uint32_t*)take((size_t)cap * 4);
  T.count = (uint32_t*)take((size_t)cap * 4);
  T.pool_off = (uint32_t*)take((size_t)cap * 4);
  return T;
}
size_t table_bytes(uint32_t cap) { return (size_t)cap * 28 + 8 * 256; }

int bitlen(uint32_t v) {
  int b = 0;
  while (v) { ++b; v >>= 1; }
  return b;
}

}  // namespace

void launch_trace_kd(int kind, int traversal, bool any, const KdView& v, const float4* rays, uint32_t n,
                     float4* hits, uint32_t* occ, uint32_t* err, cudaStream_t s, uint32_t* work) {
  if (n == 0) return;
  count_launch();
  const uint32_t nn = v.n_nodes;
  if (kind == kTriangles) {
    if (any) dispatch_kd<kTriangles, true>(traversal, v, nn, rays, n, hits, occ, err, work, s);
    else dispatch_kd<kTriangles, false>(traversal, v, nn, rays, n, hits, occ, err, work, s);
  } else {
    if (any) dispatch_kd<kSpheres, true>(traversal, v, nn, rays, n, hits, occ, err, work, s);
    else dispatch_kd<kSpheres, false>(traversal, v, nn, rays, n, hits, occ, err, work, s);
  }
}

BuildResult build_kd_tree(const SceneView& s, int max_depth_cfg, AccelBuffers& a, BuildScratch& sc, uint32_t* err,
                          cudaStream_t st) {
  const uint32_t n = s.n;
  int l2 = 0;
  for (uint32_t v = n; v > 1; v >>= 1) ++l2;
  // maxDepth = round(8 + 1.3 * Log2Int(N)) (accelerators.h:957-958)
  const int depth0 = max_depth_cfg > 0 ? max_depth_cfg : (int)std::round(8 + 1.3f * l2);
  const size_t payload = s.kind == kTriangles ? 48 : 16;
  KD_TRY(a.prims.ensure((size_t)n * payload), "KD payload");
  KD_TRY(a.root.ensure(32), "KD root");
  // primitive boxes (and payload by id)
  KD_TRY(sc.m0.ensure((size_t)n * 24), "KD scratch");
  float* aabb = sc.m0.as<float>();
  launch_prims_by_id(s.kind, s.verts, s.idx, s.sph, n, a.prims.as<float4>(), aabb, st);
  KD_TRY(cudaGetLastError(), "KD prims");
  // root bounds: union of every primitive box
  KD_TRY(sc.lohi.ensure(64), "KD scratch");
  int32_t* lohi = sc.lohi.as<int32_t>();
  launch_init_bounds(lohi, st);
  count_launch();
  k_box_union<<<std::min<uint32_t>(grid(n), 1024u), kThreads, 0, st>>>(aabb, n, lohi);

  // refs of the current level, double buffered: prim, node
  uint32_t R = n, M = 1;
  if (2ull * n >= (1ull << 31)) return BuildResult::error(RQ_ERROR_INVALID_ARGUMENT, "KD tree over 2^30 primitives");
  KD_TRY(sc.m1.ensure((size_t)n * 8 * 2), "KD scratch");
  uint32_t* ref_prim = sc.m1.as<uint32_t>();
  uint32_t* ref_node = ref_prim + (size_t)n;
  count_launch();
  k_iota<<<grid(n), kThreads, 0, st>>>(ref_prim, n);
  KD_TRY(cudaMemsetAsync(ref_node, 0, (size_t)n * 4, st), "KD init");
  // root edge lists, one per axis, each sorted once by t (stable: equal t
  // start-first, then by primitive id)
  const uint32_t E0 = 2 * n;
  KD_TRY(sc.keys.ensure((size_t)E0 * kEdgeWords * 4 + 64), "KD edges");
  KD_TRY(sc.vals.ensure((size_t)E0 * 2 * 4 + 64), "KD edges");
  EdgeLists el{sc.keys.as<uint32_t>(), (size_t)E0};
  {
    const size_t zwords = 1024 + 16 + sort_status_words(E0, 4);
    KD_TRY(sc.m4.ensure(zwords * 4 + 64), "KD sort");
    uint32_t* zero = sc.m4.as<uint32_t>();
    SortScratch ss{sc.vals.as<uint32_t>(), sc.vals.as<uint32_t>() + E0, zero, zero + 1024 + 16, zero + 1024};
    for (int ax = 0; ax < 3; ++ax) {
      count_launch();
      k_root_edges<<<grid(n), kThreads, 0, st>>>(aabb, n, ax, el.t(ax), el.v(ax));
      KD_TRY(cudaMemsetAsync(zero, 0, zwords * 4, st), "KD sort");
      launch_histogram(el.t(ax), E0, 4, zero, st);
      launch_onesweep(el.t(ax), el.v(ax), E0, 4, ss, err, st);
    }
    for (int ax = 0; ax < 3; ++ax) {
      KD_TRY(cudaMemsetAsync(el.n(ax), 0, (size_t)E0 * 4, st), "KD root edges");
      count_launch();
      k_start_flags<<<grid(E0), kThreads, 0, st>>>(el.v(ax), E0, el.s(ax));
      launch_scan_excl(el.s(ax), el.s(ax), E0, sc.vals.as<uint32_t>(), nullptr, st);  // in place
    }
    KD_TRY(cudaGetLastError(), "KD root edges");
  }
  // level 0 node
  KD_TRY(sc.m3.ensure(level_bytes(1)), "KD scratch");
  LevelNodes L = carve(sc.m3.as<char>(), 1);
  {
    const int32_t h_depth = depth0, h_bad = 0;
    const uint32_t h_rs = 0, h_rc = n;
    KD_TRY(cudaMemcpyAsync(L.depth, &h_depth, 4, cudaMemcpyHostToDevice, st), "KD init");
    KD_TRY(cudaMemcpyAsync(L.bad, &h_bad, 4, cudaMemcpyHostToDevice, st), "KD init");
    KD_TRY(cudaMemcpyAsync(L.rs, &h_rs, 4, cudaMemcpyHostToDevice, st), "KD init");
    KD_TRY(cudaMemcpyAsync(L.rc, &h_rc, 4, cudaMemcpyHostToDevice, st), "KD init");
    count_launch();
    k_root_box<<<1, 32, 0, st>>>(lohi, L.box, a.root.as<float>());
  }
  DevBuf& tabbuf = sc.m5;
  DevBuf& poolbuf = sc.m6;
  uint32_t table_cap = 0, total = 0, pool_used = 0;
  std::vector<uint32_t> level_lo;
  for (int level = 0; M > 0; ++level) {
    if (level > 200) return BuildResult::error(RQ_ERROR_INVALID_ARGUMENT, "KD tree deeper than 200 levels");
    level_lo.push_back(total);
    // table capacity
    if (total + M > table_cap) {
      uint32_t ncap = (total + M) * 2 + 1024;
      DevBuf nb;
      KD_TRY(nb.ensure(table_bytes(ncap)), "KD table");
      if (table_cap) {
        Table Told = table_at(tabbuf.as<char>(), table_cap), Tnew = table_at(nb.as<char>(), ncap);
        const size_t bytes = (size_t)total * 4;
        KD_TRY(cudaMemcpyAsync(Tnew.leaf, Told.leaf, bytes, cudaMemcpyDeviceToDevice, st), "KD table");
        KD_TRY(cudaMemcpyAsync(Tnew.axis, Told.axis, bytes, cudaMemcpyDeviceToDevice, st), "KD table");
        KD_TRY(cudaMemcpyAsync(Tnew.split, Told.split, bytes, cudaMemcpyDeviceToDevice, st), "KD table");
        KD_TRY(cudaMemcpyAsync(Tnew.child0, Told.child0, bytes, cudaMemcpyDeviceToDevice, st), "KD table");
        KD_TRY(cudaMemcpyAsync(Tnew.child1, Told.child1, bytes, cudaMemcpyDeviceToDevice, st), "KD table");
        KD_TRY(cudaMemcpyAsync(Tnew.count, Told.count, bytes, cudaMemcpyDeviceToDevice, st), "KD table");
        KD_TRY(cudaMemcpyAsync(Tnew.pool_off, Told.pool_off, bytes, cudaMemcpyDeviceToDevice, st), "KD table");
        KD_TRY(cudaStreamSynchronize(st), "KD table");
      }
      tabbuf.release();
      tabbuf = nb;
      nb.p = nullptr;
      nb.cap = 0;
      table_cap = ncap;
    }
    Table T = table_at(tabbuf.as<char>(), table_cap);
    // per-ref scratch: below / above flags and their scans (R + 1 each)
    KD_TRY(ensure_after(sc.m2, ((size_t)R + 1) * 4 * 4 + scan_tmp_words((uint64_t)R + 1) * 8 + 64, st), "KD scratch");
    uint32_t* below = sc.m2.as<uint32_t>();
    uint32_t* above = below + (R + 1);
    uint32_t* sB = above + (R + 1);
    uint32_t* sA = sB + (R + 1);
    uint32_t* tmp = sA + (R + 1);
    // partition scratch: tile counts and the side flags as ballot words
    const uint32_t E2 = 2 * R;
    const uint32_t runs = (E2 + kEdgeRun - 1) / kEdgeRun, tiles = (E2 + kEdgeTile - 1) / kEdgeTile;
    const size_t words = ((size_t)E2 + 31) / 32;
    KD_TRY(ensure_after(sc.m4, (size_t)tiles * 3 * 16 + words * 3 * 8 + 64, st), "KD edges");
    unsigned long long* tile_cnt = sc.m4.as<unsigned long long>();
    uint32_t* sideB = reinterpret_cast<uint32_t*>(tile_cnt + (size_t)tiles * 3 * 2);
    uint32_t* sideA = sideB + words * 3;
    // interior ranks, leaf pool offsets, children's ref counts
    KD_TRY(ensure_after(sc.m7, ((size_t)M + 1) * 4 * 4 + scan_tmp_words((uint64_t)M + 1) * 8 + 64, st), "KD scratch");
    uint32_t* iflag = sc.m7.as<uint32_t>();
    uint32_t* irank = iflag + (M + 1);
    uint32_t* lcnt = irank + (M + 1);
    uint32_t* lofs = lcnt + (M + 1);
    uint32_t* mtmp = lofs + (M + 1);
    uint32_t* mtot = mtmp + 2 * scan_tmp_words((uint64_t)M + 1) + 4;  // 4 totals
    count_launch();
    k_node_init<<<grid(std::max<uint64_t>(M, (uint64_t)R + 1)), kThreads, 0, st>>>(L, M, below, above, R);
    if (E2) {
      count_launch();
      k_cost<<<grid(3ull * runs * 32), kThreads, 0, st>>>(el, E2, runs, M, L, err);
    }
    count_launch(2);
    k_decide<<<grid((uint64_t)M + 1), kThreads, 0, st>>>(el, L, M, E2, iflag, lcnt, err);
    k_classify<<<grid(R), kThreads, 0, st>>>(ref_prim, ref_node, R, M, aabb, L, below, above, err);
    KD_TRY(cudaGetLastError(), "KD split");
    launch_scan2_excl(iflag, irank, lcnt, lofs, (uint64_t)M + 1, mtmp, mtot, mtot + 1, st);
    launch_scan2_excl(below, sB, above, sA, (uint64_t)R + 1, tmp, mtot + 2, mtot + 3, st);
    uint32_t h_tot[4] = {0, 0, 0, 0};
    KD_TRY(cudaMemcpyAsync(h_tot, mtot, 16, cudaMemcpyDeviceToHost, st), "KD level");
    KD_TRY(cudaStreamSynchronize(st), "KD level");
    const uint32_t interiors = h_tot[0], leaf_refs = h_tot[1];
    const uint64_t R2l = (uint64_t)h_tot[2] + h_tot[3];
    if (2 * R2l >= (1ull << 31)) return BuildResult::error(RQ_ERROR_INVALID_ARGUMENT, "KD tree over 2^30 references");
    const uint32_t R2 = (uint32_t)R2l;
    // next level nodes and child ref counts
    const uint32_t M2 = 2 * interiors;
    DevBuf& nextbuf = (level & 1) ? sc.m3 : sc.keys_alt;  // alternate level buffers
    KD_TRY(ensure_after(nextbuf, level_bytes(M2 ? M2 : 1) + ((size_t)M2 + 1) * 8 + scan_tmp_words((uint64_t)M2 + 1) * 4 + 64, st),
           "KD scratch");
    LevelNodes N = carve(nextbuf.as<char>(), M2 ? M2 : 1);
    uint32_t* ccnt = reinterpret_cast<uint32_t*>(nextbuf.as<char>() + level_bytes(M2 ? M2 : 1));
    uint32_t* coff = ccnt + (M2 + 1);
    uint32_t* ctmp = coff + (M2 + 1);
    // leaf pool growth
    KD_TRY(grow_keep(poolbuf, ((size_t)pool_used + leaf_refs + 1) * 4, (size_t)pool_used * 4, st), "KD pool");
    // lofs holds offsets relative to this level; shift by pool_used in the kernels
    count_launch();
    k_spawn<<<grid(M), kThreads, 0, st>>>(L, M, irank, sB, sA, lofs, pool_used, total, total + M, T, N, ccnt, M2,
                                          err);
    KD_TRY(cudaGetLastError(), "KD spawn");
    if (M2) {
      launch_scan_excl(ccnt, coff, (uint64_t)M2 + 1, ctmp, nullptr, st);
      count_launch();
      k_set_ref_starts<<<grid(M2), kThreads, 0, st>>>(N, M2, ccnt, coff);
    }
    // refs of the next level (separate buffer), leaf refs to the pool
    KD_TRY(ensure_after(sc.kd_refs, ((size_t)R2 + 1) * 8, st), "KD refs");
    uint32_t* out_prim = sc.kd_refs.as<uint32_t>();
    uint32_t* out_node = out_prim + (R2 + 1);
    count_launch();
    k_emit_refs<<<grid(R), kThreads, 0, st>>>(ref_prim, ref_node, R, L, irank, below, above, sB, sA, N, out_prim,
                                              out_node, lofs, pool_used, poolbuf.as<uint32_t>(), R2,
                                              (uint32_t)(poolbuf.cap / 4), err);
    KD_TRY(cudaGetLastError(), "KD emit");
    // the children's edge lists
    KD_TRY(ensure_after(sc.vals, (size_t)R2 * 2 * kEdgeWords * 4 + 64, st), "KD edges");
    EdgeLists eln{sc.vals.as<uint32_t>(), (size_t)R2 * 2};
    if (E2 && R2) {
      count_launch(3);
      k_part_count<<<3 * tiles, kThreads, 0, st>>>(el, E2, tiles, R, M, below, above, sideB, sideA, tile_cnt, err);
      k_part_scan<<<3, 1024, 0, st>>>(tile_cnt, tiles);
      k_partition<<<3 * tiles, kThreads, 0, st>>>(el, E2, tiles, L, sideB, sideA, tile_cnt, sB, sA, eln, 2 * R2, err);
      KD_TRY(cudaGetLastError(), "KD partition");
    }
    pool_used += leaf_refs;
    total += M;
    std::swap(sc.m1, sc.kd_refs);  // the children's refs become the current refs
    std::swap(sc.keys, sc.vals);   // and their edge lists
    el = EdgeLists{sc.keys.as<uint32_t>(), (size_t)R2 * 2};
    ref_prim = sc.m1.as<uint32_t>();
    ref_node = ref_prim + (R2 + 1);
    R = R2;
    M = M2;
    L = N;
  }
  // depth-first layout
  level_lo.push_back(total);
  Table T = table_at(tabbuf.as<char>(), table_cap);
  // size, pos, cnt, off: four arrays of total + 2 words
  KD_TRY(ensure_after(sc.m7, ((size_t)total + 2) * 16 + scan_tmp_words((uint64_t)total + 2) * 4 + 64, st), "KD layout");
  uint32_t* size = sc.m7.as<uint32_t>();
  uint32_t* pos = size + (total + 1);
  uint32_t* cnt = pos + (total + 1);
  uint32_t* off = cnt + (total + 1);
  uint32_t* ltmp = off + (total + 2);
  uint32_t* ltot = ltmp + scan_tmp_words((uint64_t)total + 2) + 4;
  for (int lv = (int)level_lo.size() - 2; lv >= 0; --lv) {
    count_launch();
    k_sizes<<<grid(level_lo[lv + 1] - level_lo[lv]), kThreads, 0, st>>>(T, level_lo[lv], level_lo[lv + 1], size,
                                                                         total, err);
  }
  KD_TRY(cudaMemsetAsync(pos, 0, 4, st), "KD layout");
  for (size_t lv = 0; lv + 1 < level_lo.size(); ++lv) {
    count_launch();
    k_positions<<<grid(level_lo[lv + 1] - level_lo[lv]), kThreads, 0, st>>>(T, level_lo[lv], level_lo[lv + 1], size,
                                                                             pos, total);
  }
  count_launch();
  k_leaf_counts<<<grid((uint64_t)total + 1), kThreads, 0, st>>>(T, total, pos, cnt);
  launch_scan_excl(cnt, off, (uint64_t)total + 1, ltmp, ltot, st);
  uint32_t n_idx = 0;
  KD_TRY(cudaMemcpyAsync(&n_idx, ltot, 4, cudaMemcpyDeviceToHost, st), "KD layout");
  KD_TRY(cudaStreamSynchronize(st), "KD layout");
  KD_TRY(a.kd_nodes.ensure((size_t)total * 16), "KD nodes");
  KD_TRY(a.kd_idx.ensure((size_t)(n_idx ? n_idx : 1) * 4), "KD indices");
  count_launch();
  k_write_nodes<<<grid(total), kThreads, 0, st>>>(T, total, pos, off, poolbuf.as<uint32_t>(), a.kd_nodes.as<int4>(),
                                                  a.kd_idx.as<int32_t>(), n_idx, (uint32_t)(poolbuf.cap / 4), err);
  KD_TRY(cudaGetLastError(), "KD write");
  a.n_nodes = total;
  a.n_slots = n_idx;
  a.max_depth = (uint32_t)depth0;
  return {};
}

}  // namespace rq
