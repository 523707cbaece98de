// Treelet restructuring of an LBVH (Karras and Aila 2013, "Fast parallel
// construction of high-quality bounding volume hierarchies"): one bottom-up
// pass over the refitted Karras tree.  At every internal node x the treelet
// grown from x -- its two children, then repeatedly the internal treelet leaf
// of largest surface area replaced by its two children, up to four treelet
// leaves -- is rebuilt with the topology of least SAH cost found by dynamic
// programming over the subsets of its leaves, reusing the treelet's internal
// nodes (x keeps its index, so its parent is untouched).  Every topology of a
// treelet holds the same treelet leaves, whose subtrees' costs are therefore a
// constant: the cost minimised is the sum of the half surface areas of the
// treelet's internal nodes, from the boxes alone.  A node is restructured only
// after every node below it is, and its result depends on its subtree alone,
// so any bottom-up order gives the same tree: the kernels run the nodes of
// each height (longest path to a leaf, on the Karras tree) together, lowest
// height first -- two nodes of equal height are never one below the other, and
// a restructure moves nodes only within its own subtree.
//
// No counterpart in the reference (its "LBVH", accelerators.h:568-665, is a
// median split); the walk's hits do not depend on the tree, only the number of
// nodes a ray visits does.
//
// Two kernels, over the refit decomposition k_karras wrote (node heights
// from the refit): one block per treelet of at most kTreeletSpan leaves,
// several in flight per SM, then one block over the top nodes, skipped when
// the top nodes exceed kRefitTopCap (their Karras topology is kept).  Node data
// stay in global memory (L2): one restructure is a chain of dependent steps,
// and the treelets in flight hide each other's latency.
#include <type_traits>

#include "lbvh_device.cuh"

namespace rq {
namespace {

// A treelet's threads and treelets in flight per SM (119 registers a thread):
// on the 998,000-triangle terrain 0.163 ms per pass, against 0.188 with 3 x
// 128, 0.165 with 5 x 128, 0.207 with 8 x 64 and 0.188 with 2 x 256.
constexpr int kOptThreads = 128;
constexpr int kOptBlocksPerSM = 4;
constexpr int kOptLeaves = 4;     // treelet leaves
constexpr int kOptTopThreads = 256;  // the top nodes: few, one block

struct TBox {
  float lo[3], hi[3];
};

__device__ __forceinline__ void grow(TBox& a, const TBox& b) {
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    a.lo[k] = fminf(a.lo[k], b.lo[k]);
    a.hi[k] = fmaxf(a.hi[k], b.hi[k]);
  }
}

// Half the surface area (the SAH's weights up to a common factor).
__device__ __forceinline__ float half_area(const TBox& b) {
  const float dx = b.hi[0] - b.lo[0], dy = b.hi[1] - b.lo[1], dz = b.hi[2] - b.lo[2];
  return dx * dy + dy * dz + dz * dx;
}

// Compile-time loops (every array index below is a constant, so the dynamic
// program's tables live in registers).
template <int I, int E, int STEP, class F>
__device__ __forceinline__ void unroll(F&& f) {
  if constexpr (STEP > 0 ? I < E : I > E) {
    f(std::integral_constant<int, I>{});
    unroll<I + STEP, E, STEP>(f);
  }
}
constexpr int low_index(int s) { return (s & 1) ? 0 : 1 + low_index(s >> 1); }
constexpr bool single(int s) { return (s & (s - 1)) == 0; }

// Node access for the restructuring: child links and child boxes, in global
// memory (L2; written by this block's threads or by earlier kernels).
struct GlobalNodes {
  float4* nodes;
  __device__ int2 get_link(int id) const {
    const int4 l = __ldcg(reinterpret_cast<const int4*>(nodes) + 4 * (size_t)id + 3);
    return make_int2(l.x, l.y);
  }
  __device__ void get_box(int id, int side, TBox& b) const {
    const float4 xy = __ldcg(nodes + 4 * (size_t)id + side);
    const float2 z = __ldcg(reinterpret_cast<const float2*>(nodes + 4 * (size_t)id + 2) + side);
    b.lo[0] = xy.x; b.hi[0] = xy.y; b.lo[1] = xy.z; b.hi[1] = xy.w; b.lo[2] = z.x; b.hi[2] = z.y;
  }
  __device__ void set(int id, int l, const TBox& bl, int r, const TBox& br) const {
    float4* q = nodes + 4 * (size_t)id;
    q[0] = make_float4(bl.lo[0], bl.hi[0], bl.lo[1], bl.hi[1]);
    q[1] = make_float4(br.lo[0], br.hi[0], br.lo[1], br.hi[1]);
    q[2] = make_float4(bl.lo[2], bl.hi[2], br.lo[2], br.hi[2]);
    reinterpret_cast<int4*>(q)[3] = make_int4(l, r, l < 0 ? 1 : 0, r < 0 ? 1 : 0);
  }
};

// Rebuild the treelet of N leaves (codes, boxes) under the internal nodes
// pool[0..N-2] (pool[0] = the treelet root) with the topology of least sum of
// internal half areas.  The dynamic program visits the subsets S of two or
// more leaves in increasing order and, for each, the parts P of S that hold
// S's lowest leaf in decreasing order, keeping the first least
// best[P] + best[S ^ P] (a single leaf costs 0).  The chosen subsets get the
// pool's nodes in decreasing subset order (the whole set first, so the root
// keeps its index).
template <int N, class Acc>
__device__ __forceinline__ void rebuild(const Acc& A, const int (&code)[kOptLeaves], const TBox (&box)[kOptLeaves],
                                        const int (&pool)[kOptLeaves - 1]) {
  constexpr int F = (1 << N) - 1;
  float best[F + 1];
  int split[F + 1];
  unroll<0, N, 1>([&](auto kc) { constexpr int k = decltype(kc)::value; best[1 << k] = 0.f; });
  unroll<3, F + 1, 1>([&](auto sc) {
    constexpr int S = decltype(sc)::value;
    if constexpr (!single(S)) {
      float acc = __int_as_float(0x7F800000);
      int accp = 0;
      unroll<S - 1, 0, -1>([&](auto pc) {
        constexpr int P = decltype(pc)::value;
        if constexpr ((P & S) == P && (P & (S & -S))) {
          const float c = best[P] + best[S ^ P];
          if (c < acc) { acc = c; accp = P; }
        }
      });
      TBox u = box[low_index(S)];
      unroll<0, N, 1>([&](auto bc) {
        constexpr int b = decltype(bc)::value;
        if constexpr ((S >> b) & 1) grow(u, box[b]);
      });
      best[S] = half_area(u) + acc;
      split[S] = accp;
    }
  });
  uint32_t used = 1u << F;
  unroll<F, 2, -1>([&](auto sc) {
    constexpr int S = decltype(sc)::value;
    if constexpr (!single(S))
      if ((used >> S) & 1u) used |= (1u << split[S]) | (1u << (S ^ split[S]));
  });
  int id_of[F + 1];
  int rank = 0;
  unroll<F, 2, -1>([&](auto sc) {
    constexpr int S = decltype(sc)::value;
    if constexpr (!single(S)) {
      if ((used >> S) & 1u) {
        int id = pool[0];
        unroll<1, N - 1, 1>([&](auto ic) { constexpr int i = decltype(ic)::value; if (rank == i) id = pool[i]; });
        id_of[S] = id;
        ++rank;
      }
    }
  });
  unroll<F, 2, -1>([&](auto sc) {
    constexpr int S = decltype(sc)::value;
    if constexpr (!single(S)) {
      if ((used >> S) & 1u) {
        const int P = split[S], Q = S ^ P;
        int cl = 0, cr = 0;
        TBox bl = box[0], br = box[0];
        bool fl = false, fr = false;
        unroll<0, N, 1>([&](auto bc) {
          constexpr int b = decltype(bc)::value;
          if (P == (1 << b)) cl = code[b];
          if (Q == (1 << b)) cr = code[b];
          if ((P >> b) & 1) { if (fl) grow(bl, box[b]); else bl = box[b]; fl = true; }
          if ((Q >> b) & 1) { if (fr) grow(br, box[b]); else br = box[b]; fr = true; }
        });
        unroll<3, F, 1>([&](auto rc) {
          constexpr int R = decltype(rc)::value;
          if constexpr (!single(R)) {
            if (P == R) cl = id_of[R];
            if (Q == R) cr = id_of[R];
          }
        });
        A.set(id_of[S], cl, bl, cr, br);
      }
    }
  });
}

// Restructure the treelet rooted at internal node x (every node below it done).
template <class Acc>
__device__ __forceinline__ void restructure(const Acc& A, int x) {
  int code[kOptLeaves];
  TBox box[kOptLeaves];
  int pool[kOptLeaves - 1];
  const int2 l = A.get_link(x);
  code[0] = l.x;
  code[1] = l.y;
  A.get_box(x, 0, box[0]);
  A.get_box(x, 1, box[1]);
  pool[0] = x;
  int n = 2;
#pragma unroll
  for (int step = 0; step < kOptLeaves - 2; ++step) {
    // the internal treelet leaf of largest area (first of equals)
    int pick = -1;
    float pa = -1.f;
#pragma unroll
    for (int k = 0; k < kOptLeaves; ++k) {
      if (k < n && code[k] >= 0) {
        const float a = half_area(box[k]);
        if (a > pa) { pa = a; pick = k; }
      }
    }
    if (pick < 0) break;
    int c = 0;
#pragma unroll
    for (int k = 0; k < kOptLeaves; ++k)
      if (k == pick) c = code[k];
    pool[step + 1] = c;
    const int2 cl = A.get_link(c);
    TBox b0, b1;
    A.get_box(c, 0, b0);
    A.get_box(c, 1, b1);
#pragma unroll
    for (int k = 0; k < kOptLeaves; ++k) {
      if (k == pick) { code[k] = cl.x; box[k] = b0; }
      if (k == n) { code[k] = cl.y; box[k] = b1; }
    }
    ++n;
  }
  if (n == 4) rebuild<4>(A, code, box, pool);
  else if (n == 3) rebuild<3>(A, code, box, pool);
}

constexpr uint32_t kMaxHeight = 128;  // Karras trees are at most 64 deep

struct OptShared {
  uint32_t height[kTreeletSpan];   // the treelet's internal nodes (0: not one of them)
  uint16_t order[kTreeletSpan];    // nodes of height 2 and more, by height
  uint32_t level[kMaxHeight + 1];  // starts of each height's nodes in order[]
  uint32_t next;
};

// The nodes of heights 2 .. top_h (slots [0, cnt) with height[w]) listed by
// height into order[] (level[h] .. level[h + 1]); the counts are summed per
// warp (one shared atomic per height and warp).
__device__ __forceinline__ void list_by_height(uint32_t cnt, uint32_t top_h, const uint32_t* height, uint32_t* level,
                                               uint16_t* order) {
  const uint32_t lane = threadIdx.x & 31u;
  for (uint32_t h = threadIdx.x; h <= top_h + 1; h += blockDim.x) level[h] = 0u;
  __syncthreads();
  for (uint32_t w0 = 0; w0 < cnt; w0 += blockDim.x) {
    const uint32_t w = w0 + threadIdx.x;
    const bool v = w < cnt && height[w] >= 2u && height[w] <= top_h;
    const uint32_t h = v ? height[w] : ~0u;
    const uint32_t peers = __match_any_sync(0xffffffffu, h);
    if (v && lane == (uint32_t)(__ffs(peers) - 1)) atomicAdd(&level[h], (uint32_t)__popc(peers));
  }
  __syncthreads();
  if (threadIdx.x == 0) {  // counts -> starts; level[h] then serves as the cursor
    uint32_t run = 0;
    for (uint32_t h = 0; h <= top_h; ++h) {
      const uint32_t c = level[h];
      level[h] = run;
      run += c;
    }
    level[top_h + 1] = run;
  }
  __syncthreads();
  for (uint32_t w0 = 0; w0 < cnt; w0 += blockDim.x) {
    const uint32_t w = w0 + threadIdx.x;
    const bool v = w < cnt && height[w] >= 2u && height[w] <= top_h;
    const uint32_t h = v ? height[w] : ~0u;
    const uint32_t peers = __match_any_sync(0xffffffffu, h);
    const uint32_t leader = (uint32_t)(__ffs(peers) - 1);
    uint32_t base = 0;
    if (v && lane == leader) base = atomicAdd(&level[h], (uint32_t)__popc(peers));
    base = __shfl_sync(0xffffffffu, base, (int)leader);
    if (v) order[base + __popc(peers & ((1u << lane) - 1u))] = (uint16_t)w;
  }
  __syncthreads();
  if (threadIdx.x == 0) {  // cursors (starts + counts) -> starts
    for (uint32_t h = top_h + 1; h > 0; --h) level[h] = level[h - 1];
    level[0] = 0u;
  }
  __syncthreads();
}

// Persistent blocks over the refit treelets (queue counter count[3]), several
// per SM so that their level-by-level latencies overlap: a treelet's internal
// nodes listed by height (heights from the refit), then restructured one
// height at a time, node data in global memory.  A treelet covering leaves
// [lo, lo + cnt) is a subtree of the Karras tree whose root is lo (a right
// child) or lo + cnt - 1 (a left child); its internal nodes are the other
// cnt - 1 indices of that range (the index at the far end from the root
// belongs to another subtree).
__global__ void __launch_bounds__(kOptThreads, kOptBlocksPerSM) k_treelet_opt(float4* nodes,
                                                                              const uint8_t* __restrict__ heights,
                                                                              const uint32_t* __restrict__ treelets,
                                                                              uint32_t* count, uint32_t n,
                                                                              uint32_t* err) {
  __shared__ OptShared sh;
  const uint32_t ntl = __ldcg(count + 1);
  const uint2* tl = reinterpret_cast<const uint2*>(treelets);
  for (;;) {
    if (threadIdx.x == 0) sh.next = atomicAdd(count + 3, 1u);
    __syncthreads();
    const uint32_t t = sh.next;
    if (t >= ntl) break;  // uniform per block
    const uint2 rec = __ldcg(tl + t);
    const uint32_t lo = rec.x, cnt = rec.y & ~kTreeletRight;
    if (cnt == 0 || cnt > kTreeletSpan || lo + cnt > n) {  // uniform per block
      if (threadIdx.x == 0) atomicOr(err, kErrCorrupt);
      __syncthreads();
      continue;
    }
    if (cnt < 3) {  // no treelet of three leaves
      __syncthreads();
      continue;
    }
    const bool right = rec.y & kTreeletRight;
    const uint32_t root_w = right ? 0u : cnt - 1, other_w = right ? cnt - 1 : 0u;
    for (uint32_t w = threadIdx.x; w < cnt; w += blockDim.x)
      sh.height[w] = w == other_w ? 0u : __ldg(heights + lo + w);
    __syncthreads();
    const uint32_t top_h = sh.height[root_w];
    if (top_h >= kMaxHeight) {  // uniform per block
      if (threadIdx.x == 0) atomicOr(err, kErrCorrupt);
      __syncthreads();
      continue;
    }
    list_by_height(cnt, top_h, sh.height, sh.level, sh.order);
    const GlobalNodes A{nodes};
    for (uint32_t h = 2; h <= top_h; ++h) {  // height 1: both children are leaves
      for (uint32_t i = sh.level[h] + threadIdx.x; i < sh.level[h + 1]; i += blockDim.x)
        restructure(A, (int)(lo + sh.order[i]));
      __syncthreads();
    }
  }
}

struct TopOptShared {
  uint32_t node[kRefitTopCap];
  uint32_t up[kRefitTopCap];       // parent slot << 1 | side; ~0u for the root
  uint32_t arrived[kRefitTopCap];  // children finished
  uint32_t height[kRefitTopCap];   // longest path to a node below the top nodes
  uint8_t start[kRefitTopCap];     // both children below the top nodes
  uint16_t order[kRefitTopCap];
  uint32_t level[kMaxHeight + 1];
  uint32_t max_height;
};

// The top nodes, one block: heights over the top nodes (a node whose children
// are both below the top nodes has height 1; the root's is the largest), then
// one height at a time, node data in global memory (the treelets below are
// done).
__global__ void __launch_bounds__(kOptTopThreads) k_treelet_opt_top(float4* nodes, const uint32_t* __restrict__ parent,
                                                                  const uint32_t* __restrict__ mark,
                                                                  const uint32_t* __restrict__ top,
                                                                  const uint32_t* __restrict__ top_count,
                                                                  uint32_t* err) {
  __shared__ TopOptShared sh;
  const uint32_t cnt = __ldg(top_count);
  if (cnt == 0 || cnt > kRefitTopCap) return;
  if (threadIdx.x == 0) sh.max_height = 0u;
  for (uint32_t k = threadIdx.x; k < cnt; k += blockDim.x) {
    const uint32_t i = __ldg(top + k);
    sh.node[k] = i;
    const int4 l = __ldcg(reinterpret_cast<const int4*>(nodes) + 4 * (size_t)i + 3);
    uint32_t ready = 0;
    const int32_t ch[2] = {l.x, l.y};
    for (int side = 0; side < 2; ++side)
      if (!(ch[side] >= 0 && (__ldg(mark + ch[side]) & kTopMark))) ++ready;
    sh.arrived[k] = ready;
    sh.start[k] = ready == 2;
    sh.height[k] = 0u;
    uint32_t up = ~0u;
    if (i != 0) {
      const uint32_t pw = __ldg(parent + i);
      const uint32_t pm = __ldg(mark + (pw >> 1));
      if (!(pm & kTopMark) || (pm & kSlotMask) >= cnt) {
        atomicOr(err, kErrCorrupt);
        sh.start[k] = 0;
      } else {
        up = ((pm & kSlotMask) << 1) | (pw & 1u);
      }
    }
    sh.up[k] = up;
  }
  __syncthreads();
  // Each top child adds its height + 1 to its parent before it counts its
  // arrival; the second arrival finds the parent's height final.
  for (uint32_t k = threadIdx.x; k < cnt; k += blockDim.x) {
    if (!sh.start[k]) continue;
    uint32_t cur = k, h = 1;
    atomicMax(&sh.height[cur], h);
    for (uint32_t step = 0; step <= cnt; ++step) {
      const uint32_t up = sh.up[cur];
      if (up == ~0u) {
        sh.max_height = h;
        break;
      }
      const uint32_t ps = up >> 1;
      atomicMax(&sh.height[ps], h + 1);
      __threadfence_block();
      if (atomicAdd(&sh.arrived[ps], 1u) != 1u) break;
      __threadfence_block();
      h = sh.height[ps];
      cur = ps;
    }
  }
  __syncthreads();
  const uint32_t top_h = sh.max_height;
  if (top_h + 1 >= kMaxHeight) {
    if (threadIdx.x == 0) atomicOr(err, kErrCorrupt);
    return;
  }
  // Height 1 here (both children below the top nodes) has treelets too: list
  // heights from 1 by counting each top node's height one up.
  for (uint32_t k = threadIdx.x; k < cnt; k += blockDim.x) sh.height[k] += 1u;
  __syncthreads();
  list_by_height(cnt, top_h + 1, sh.height, sh.level, sh.order);
  const GlobalNodes A{nodes};
  for (uint32_t h = 2; h <= top_h + 1; ++h) {
    for (uint32_t i = sh.level[h] + threadIdx.x; i < sh.level[h + 1]; i += blockDim.x)
      restructure(A, (int)sh.node[sh.order[i]]);
    __syncthreads();
  }
}

}  // namespace

cudaError_t launch_treelet_opt(uint32_t n, float4* nodes, const uint32_t* parent, const RefitTop& t,
                               const uint8_t* heights, uint32_t* err, cudaStream_t s) {
  if (n < 3) return cudaSuccess;
  count_launch();
  k_treelet_opt<<<kOptBlocksPerSM * device_sm_count(), kOptThreads, 0, s>>>(nodes, heights, t.treelets, t.count, n,
                                                                             err);
  count_launch();
  k_treelet_opt_top<<<1, kOptTopThreads, 0, s>>>(nodes, parent, t.mark, t.top, t.count, err);
  return cudaGetLastError();
}

}  // namespace rq
