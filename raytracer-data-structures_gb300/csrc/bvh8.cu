// Collapse of a binary BVH (LBVH or median BVH) into a compressed 8-wide BVH
// (after Ylitie, Karras and Laine 2017, "Efficient incoherent ray traversal
// on GPUs through compressed wide BVHs": quantised child boxes, children
// placed by direction so a ray's octant gives the visiting order).
//
// Every binary node at a depth divisible by 3 becomes one 8-wide node whose
// children are its descendants three levels down (a binary leaf met on the
// way stays a single child).  Nodes are numbered by an exclusive scan over
// those flags in binary-index order, so the root is node 0 and the layout does
// not depend on thread timing.
//
// 8-wide node, 128 bytes = 8 x 16 B:
//   w0     pm.x, pm.y, pm.z (float), then E.x | E.y << 8 | E.z << 16 | valid << 24
//   w1     qlo.x[8] (one byte per slot, slots 0-3 in the first word), qhi.x[8]
//   w2, w3 the same for y and z
//   w4-w7  (link, count) per slot: count 0 -> 8-wide node `link`; count > 0 ->
//          leaf of binary slots [link, link + count); unused slots are not in `valid`
// A child's plane on axis a with quantised value q decodes as
//   plane(q) = fma(S_a, F(q), pm_a),  S_a = 2^(E_a - 127),  F(q) = 1 + q * 2^-15
// (F(q) is the float whose bits are 0x3F800000 | q << 8, one byte permute on
// the device), so plane(q) ~ lo_a + q * S_a * 2^-15.  The builder evaluates
// exactly these operations and moves every q outward until the decoded box
// contains the child's box: the walk's box test on a decoded box is then at
// least as permissive as on the exact box, so it reaches every primitive the
// binary walk reaches and the closest-hit rule returns the same hits.
// Slots: bit a of the slot says the child lies on the + side of axis a from
// the node's centre (greedy assignment by the largest score); a ray whose
// direction has sign bits `oct` (bit a set when d_a < 0) meets the children
// roughly in the order slot = k ^ oct, k = 0..7.
//
// Pipeline (build stream, no host synchronisation):
//   k_parents (bvh4.cu)  parent of every binary node
//   k_depth3             depth mod 3 by walking parent links to the root
//   scan                 8-wide index of every flagged node, total -> root word 6
//   k_fill8              one thread per flagged node writes its 128-byte node
// The reference's trees are binary only; this is the engine's node-width
// option for FAST traversal.
#include "rq_build.hpp"
#include "rq_device.cuh"

namespace rq {

void launch_parents(const float4* nodes, uint32_t n, uint32_t* parent, uint32_t* err, cudaStream_t st);

namespace {

constexpr int kThreads = 256;

// flag[i] = 1 when binary node i sits at a depth divisible by 3.
__global__ void __launch_bounds__(kThreads) k_depth3(const uint32_t* __restrict__ parent, uint32_t n,
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
  flag[i] = (d % 3u) ? 0u : 1u;
}

struct Kid {
  float lo[3], hi[3];
  int32_t link, count;  // count 0: binary internal node `link`; else leaf slots [link, link + count)
};

__device__ __forceinline__ Kid side_of(const float4* nd, int side) {
  const float4 a = __ldg(nd), b = __ldg(nd + 1), z = __ldg(nd + 2);
  const int4 l = __ldg(reinterpret_cast<const int4*>(nd + 3));
  Kid k;
  if (side == 0) {
    k.lo[0] = a.x; k.hi[0] = a.y; k.lo[1] = a.z; k.hi[1] = a.w; k.lo[2] = z.x; k.hi[2] = z.y;
    k.link = l.x; k.count = l.z;
  } else {
    k.lo[0] = b.x; k.hi[0] = b.y; k.lo[1] = b.z; k.hi[1] = b.w; k.lo[2] = z.z; k.hi[2] = z.w;
    k.link = l.y; k.count = l.w;
  }
  if (k.link < 0) k.link = ~k.link;  // leaf: first slot
  else k.count = 0;
  return k;
}

__device__ __forceinline__ float qdecode(float S, uint32_t q, float pm) {
  return __fmaf_rn(S, __uint_as_float(0x3F800000u | (q << 8)), pm);
}

__global__ void __launch_bounds__(kThreads) k_fill8(const float4* __restrict__ nodes, uint32_t n,
                                                    const uint32_t* __restrict__ flag,
                                                    const uint32_t* __restrict__ idx8, uint32_t cap,
                                                    float4* __restrict__ out, uint32_t* err) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || !__ldg(flag + i)) return;
  const uint32_t o = __ldg(idx8 + i);
  if (o >= cap) {
    atomicOr(err, kErrCorrupt);
    return;
  }
  // Descendants three levels down (binary leaves met earlier stay children).
  Kid kid[8];
  int nk = 0;
  bool bad = false;
  for (int s1 = 0; s1 < 2; ++s1) {
    const Kid c1 = side_of(nodes + 4 * (size_t)i, s1);
    if (c1.count) { kid[nk++] = c1; continue; }
    if ((uint32_t)c1.link >= n) { bad = true; break; }
    for (int s2 = 0; s2 < 2; ++s2) {
      const Kid c2 = side_of(nodes + 4 * (size_t)c1.link, s2);
      if (c2.count) { kid[nk++] = c2; continue; }
      if ((uint32_t)c2.link >= n) { bad = true; break; }
      for (int s3 = 0; s3 < 2; ++s3) {
        Kid c3 = side_of(nodes + 4 * (size_t)c2.link, s3);
        if (!c3.count) {
          if ((uint32_t)c3.link >= n) { bad = true; break; }
          c3.link = (int32_t)__ldg(idx8 + c3.link);
        }
        kid[nk++] = c3;
      }
      if (bad) break;
    }
    if (bad) break;
  }
  if (bad) {
    atomicOr(err, kErrCorrupt);
    return;
  }
  float lo[3], hi[3];
  for (int a = 0; a < 3; ++a) {
    lo[a] = kid[0].lo[a];
    hi[a] = kid[0].hi[a];
    for (int k = 1; k < nk; ++k) {
      lo[a] = fminf(lo[a], kid[k].lo[a]);
      hi[a] = fmaxf(hi[a], kid[k].hi[a]);
    }
  }
  // Direction slots: greedy, the largest score first, ties to the lowest (kid, slot).
  int slot_of[8];
  uint32_t used = 0, placed = 0;
  for (int round = 0; round < nk; ++round) {
    float best = -__int_as_float(0x7F800000);
    int bk = -1, bs = -1;
    for (int k = 0; k < nk; ++k) {
      if (placed >> k & 1u) continue;
      float d[3];
      for (int a = 0; a < 3; ++a)
        d[a] = __fsub_rn(__fadd_rn(kid[k].lo[a], kid[k].hi[a]), __fadd_rn(lo[a], hi[a]));
      for (int s = 0; s < 8; ++s) {
        if (used >> s & 1u) continue;
        const float sc = __fadd_rn(__fadd_rn((s & 1) ? d[0] : -d[0], (s & 2) ? d[1] : -d[1]), (s & 4) ? d[2] : -d[2]);
        if (bk < 0 || sc > best) { best = sc; bk = k; bs = s; }
      }
    }
    slot_of[bk] = bs;
    used |= 1u << bs;
    placed |= 1u << bk;
  }
  // Per axis: the scale S = 2^(e + 15) with 255 steps of 2^e spanning the box,
  // pm with plane(0) <= lo; then every child's bytes, moved outward until the
  // decoded planes contain the child's.
  float S[3], pm[3];
  uint32_t E[3];
  uint32_t qlo[3][2] = {}, qhi[3][2] = {};
  for (int a = 0; a < 3; ++a) {
    const float ext = __fsub_ru(hi[a], lo[a]);
    int e = -141;  // the smallest step whose S is a normal float
    if (ext > 0.f) {
      int ex;
      frexpf(__fdiv_ru(ext, 255.f), &ex);
      e = max(ex, -141);
    }
    for (;;) {
      if (e > 112) {  // S would overflow: a box beyond 2^120 across
        atomicOr(err, kErrCorrupt);
        return;
      }
      S[a] = ldexpf(1.f, e + 15);
      pm[a] = __fsub_rn(lo[a], S[a]);
      for (int t = 0; t < 64 && qdecode(S[a], 0, pm[a]) > lo[a]; ++t)
        pm[a] = nextafterf(pm[a], -__int_as_float(0x7F800000));
      if (qdecode(S[a], 0, pm[a]) <= lo[a] && qdecode(S[a], 255, pm[a]) >= hi[a]) break;
      ++e;
    }
    E[a] = (uint32_t)(e + 15 + 127);
    const float inv_step = ldexpf(1.f, -e);
    for (int k = 0; k < nk; ++k) {
      float fl = floorf(__fmul_rd(__fsub_rd(kid[k].lo[a], lo[a]), inv_step));
      float fh = ceilf(__fmul_ru(__fsub_ru(kid[k].hi[a], lo[a]), inv_step));
      uint32_t ql = (uint32_t)fminf(fmaxf(fl, 0.f), 255.f), qh = (uint32_t)fminf(fmaxf(fh, 0.f), 255.f);
      while (ql > 0 && qdecode(S[a], ql, pm[a]) > kid[k].lo[a]) --ql;
      while (qh < 255 && qdecode(S[a], qh, pm[a]) < kid[k].hi[a]) ++qh;
      const int s = slot_of[k];
      qlo[a][s >> 2] |= ql << (8 * (s & 3));
      qhi[a][s >> 2] |= qh << (8 * (s & 3));
    }
  }
  int2 lc[8];
  for (int s = 0; s < 8; ++s) lc[s] = make_int2(0, -1);
  for (int k = 0; k < nk; ++k) lc[slot_of[k]] = make_int2(kid[k].link, kid[k].count);
  float4* w = out + 8 * (size_t)o;
  w[0] = make_float4(pm[0], pm[1], pm[2], __uint_as_float(E[0] | E[1] << 8 | E[2] << 16 | used << 24));
  for (int a = 0; a < 3; ++a)
    reinterpret_cast<uint4*>(w)[1 + a] = make_uint4(qlo[a][0], qlo[a][1], qhi[a][0], qhi[a][1]);
  int4* c = reinterpret_cast<int4*>(w + 4);
  for (int s = 0; s < 4; ++s) c[s] = make_int4(lc[2 * s].x, lc[2 * s].y, lc[2 * s + 1].x, lc[2 * s + 1].y);
}

#define RQ_B8(call, what)                                            \
  do {                                                               \
    cudaError_t e_ = (call);                                         \
    if (e_ != cudaSuccess) return BuildResult::cuda_error(e_, what); \
  } while (0)

}  // namespace

// Upper bound of the 8-wide node count.  With F flagged internal nodes
// (depth 0 mod 3) and U1, U2 internal nodes at depths 1 and 2 mod 3: every
// flagged node but the root has a parent in U2, each with at most two
// children, so F <= 1 + 2 U2; likewise U2 <= 2 U1, hence U1 >= U2 / 2 and
// U2 <= 2 (n - F) / 3, which gives F <= (4 n + 3) / 7.
uint32_t bvh8_node_cap(uint32_t n_internal) { return (uint32_t)((4ull * n_internal + 3) / 7) + 2; }

BuildResult collapse_bvh8(AccelBuffers& a, BuildScratch& sc, uint32_t* err, cudaStream_t st) {
  const uint32_t n = a.n_nodes;
  a.node_width = 8;
  if (n == 0) {
    RQ_B8(cudaMemsetAsync(a.root.as<uint32_t>() + 6, 0, 4, st), "memset");
    return {};
  }
  const uint32_t cap = bvh8_node_cap(n);
  RQ_B8(a.nodes4.ensure((size_t)cap * 128), "8-wide nodes");
  RQ_B8(sc.m0.ensure((size_t)n * 4), "collapse scratch");
  RQ_B8(sc.m1.ensure((size_t)n * 4), "collapse scratch");
  RQ_B8(sc.m2.ensure((size_t)n * 4), "collapse scratch");
  RQ_B8(sc.m3.ensure(scan_tmp_words(n) * 4), "collapse scratch");
  uint32_t* parent = sc.m0.as<uint32_t>();
  uint32_t* flag = sc.m1.as<uint32_t>();
  uint32_t* idx8 = sc.m2.as<uint32_t>();
  RQ_B8(cudaMemsetAsync(parent, 0xFF, (size_t)n * 4, st), "memset");
  const uint32_t g = (n + kThreads - 1) / kThreads;
  launch_parents(a.nodes.as<const float4>(), n, parent, err, st);
  count_launch(2);
  k_depth3<<<g, kThreads, 0, st>>>(parent, n, flag, err);
  launch_scan_excl(flag, idx8, n, sc.m3.as<uint32_t>(), a.root.as<uint32_t>() + 6, st);
  k_fill8<<<g, kThreads, 0, st>>>(a.nodes.as<const float4>(), n, flag, idx8, cap, a.nodes4.as<float4>(), err);
  RQ_B8(cudaGetLastError(), "collapse launch");
  a.n4_cap = cap;
  return {};
}

}  // namespace rq
