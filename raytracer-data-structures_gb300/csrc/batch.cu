// Batched LBVH build: every scene of a batch in one pass of kernels (scene
// boxes, Morton codes, one segmented radix sort, Karras topology, refit)
// instead of one pipeline per scene.  Each scene's arrays come out exactly
// as a single build would write them (same device helpers, same stable
// order), laid out back to back in one allocation:
//   prims, order, codes at slot offset P_s (P = prefix sum of primitive counts)
//   internal nodes at I_s = P_s - s, parent links at 2 P_s - s
//   root box (8 floats) at 8 s
// The reference has no batched build; this is the engine's many-scene path
// (one launch per stage for all scenes).
//
// The sort key of primitive i of scene s is (s << 30) | morton(i): a 64-bit
// onesweep over ceil((30 + bits(s)) / 8) digits orders the batch by scene,
// then by code, stably by primitive index, which within a scene is the
// single build's order.
#include <algorithm>

#include "lbvh_device.cuh"
#include "rq_build.hpp"

namespace rq {
namespace {

constexpr int kThreads = 256;
constexpr uint32_t kCodeMask = (1u << 30) - 1u;

__global__ void k_batch_init_bounds(int32_t* lohi, uint32_t n_scenes) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 6 * n_scenes) return;
  lohi[i] = (i % 6) < 3 ? ordered_pos_inf() : ordered_neg_inf();
}

// Box of each scene's points (triangle vertices, or sphere centres).  Each
// warp takes kBoundsGroups groups of 32 consecutive points and folds a
// running box for the current scene, flushing it (one warp reduction, six
// atomics) only when the scene changes and at the end; a group that
// straddles two scenes uses per-lane atomics.  (One flush per 32 points put
// about two million atomics on the 6 x n_scenes words.)
constexpr int kBoundsGroups = 16;

__global__ void __launch_bounds__(kThreads) k_batch_point_bounds(const BatchDesc* __restrict__ desc, int kind,
                                                                 const uint32_t* __restrict__ voff, uint32_t n_scenes,
                                                                 int32_t* lohi) {
  const uint32_t total = __ldg(voff + n_scenes);
  const uint32_t lane = threadIdx.x & 31u;
  const uint64_t base = (uint64_t)((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * (32u * kBoundsGroups);
  float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  uint32_t cur = ~0u;  // scene of the running box (warp-uniform)
  auto flush = [&]() {
    for (int k = 0; k < 3; ++k)
      for (int o = 16; o > 0; o >>= 1) {
        lo[k] = fminf(lo[k], __shfl_xor_sync(0xffffffffu, lo[k], o));
        hi[k] = fmaxf(hi[k], __shfl_xor_sync(0xffffffffu, hi[k], o));
      }
    if (lane == 0 && lo[0] <= hi[0])
      for (int k = 0; k < 3; ++k) {
        atomicMin(&lohi[6 * cur + k], float_to_ordered(lo[k]));
        atomicMax(&lohi[6 * cur + 3 + k], float_to_ordered(hi[k]));
      }
    for (int k = 0; k < 3; ++k) { lo[k] = INFINITY; hi[k] = -INFINITY; }
  };
  for (int g = 0; g < kBoundsGroups; ++g) {
    const uint64_t first = base + (uint64_t)g * 32u;
    if (first >= total) break;  // warp-uniform
    const uint32_t v = (uint32_t)first + lane;
    const bool active = (uint64_t)v < total;
    // scene of the group's first point; the group is in one scene when its
    // last active point lies before that scene's end
    uint32_t s0 = 0, end0 = 0;
    if (lane == 0) {
      s0 = segment_of(voff, n_scenes, (uint32_t)first);
      end0 = __ldg(voff + s0 + 1);
    }
    s0 = __shfl_sync(0xffffffffu, s0, 0);
    end0 = __shfl_sync(0xffffffffu, end0, 0);
    const uint64_t last = first + 31u < (uint64_t)total ? first + 31u : (uint64_t)total - 1u;
    const bool uniform = last < (uint64_t)end0;
    const uint32_t s = uniform ? s0 : (active ? segment_of(voff, n_scenes, v) : 0u);
    float p[3] = {0.f, 0.f, 0.f};
    if (active) {
      const uint32_t local = v - __ldg(voff + s);
      if (kind == kTriangles) {
        const float* q = desc[s].verts + 3 * (size_t)local;
        p[0] = __ldg(q); p[1] = __ldg(q + 1); p[2] = __ldg(q + 2);
      } else {
        const float4 c = __ldg(desc[s].sph + local);
        p[0] = c.x; p[1] = c.y; p[2] = c.z;
      }
    }
    if (uniform) {
      if (s0 != cur) {
        if (cur != ~0u) flush();
        cur = s0;
      }
      if (active)
        for (int k = 0; k < 3; ++k) { lo[k] = fminf(lo[k], p[k]); hi[k] = fmaxf(hi[k], p[k]); }
    } else if (active) {
      for (int k = 0; k < 3; ++k) {
        atomicMin(&lohi[6 * s + k], float_to_ordered(p[k]));
        atomicMax(&lohi[6 * s + 3 + k], float_to_ordered(p[k]));
      }
    }
  }
  if (cur != ~0u) flush();
}

__global__ void __launch_bounds__(kThreads) k_batch_morton(const BatchDesc* __restrict__ desc, int kind, int mode,
                                                           const uint32_t* __restrict__ poff, uint32_t n_scenes,
                                                           const int32_t* __restrict__ lohi,
                                                           uint64_t* __restrict__ keys, uint32_t* __restrict__ vals) {
  const uint32_t total = __ldg(poff + n_scenes);
  const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= total) return;
  const uint32_t s = segment_of(poff, n_scenes, g);
  const uint32_t i = g - __ldg(poff + s);
  uint32_t code;
  if (kind == kTriangles) {
    float lo[3], ext[3];
    bounds_from(lohi + 6 * s, lo, ext);
    if (mode == RQ_MORTON_SCENE_CUBE) cube_extent(ext);
    code = code_scene(tri_centroid(desc[s].verts, desc[s].idx, i), lo, ext);
  } else {
    const float4 c = __ldg(desc[s].sph + i);
    if (mode == RQ_MORTON_REFERENCE) {
      // (center + 30) / 1000, accelerators.h:577
      code = morton3d(__fdiv_rn(__fadd_rn(c.x, 30.f), 1000.f), __fdiv_rn(__fadd_rn(c.y, 30.f), 1000.f),
                      __fdiv_rn(__fadd_rn(c.z, 30.f), 1000.f));
    } else {
      float lo[3], ext[3];
      bounds_from(lohi + 6 * s, lo, ext);
      if (mode == RQ_MORTON_SCENE_CUBE) cube_extent(ext);
      code = code_scene({c.x, c.y, c.z}, lo, ext);
    }
  }
  keys[g] = ((uint64_t)s << 30) | code;
  vals[g] = g;
}

// Sorted (key, global index) -> per-scene codes and local order.
__global__ void __launch_bounds__(kThreads) k_batch_split(const uint64_t* __restrict__ keys,
                                                          const uint32_t* __restrict__ vals,
                                                          const uint32_t* __restrict__ poff, uint32_t n_scenes,
                                                          uint32_t* __restrict__ codes, uint32_t* __restrict__ order,
                                                          uint32_t* err) {
  const uint32_t total = __ldg(poff + n_scenes);
  const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= total) return;
  const uint64_t k = keys[g];
  const uint32_t s = segment_of(poff, n_scenes, g);
  const uint32_t v = vals[g], p0 = __ldg(poff + s);
  // the sort keeps scenes contiguous: the source primitive is in the same scene
  if ((uint32_t)(k >> 30) != s || v < p0 || v >= __ldg(poff + s + 1)) {
    atomicOr(err, kErrCorrupt);
    return;
  }
  codes[g] = (uint32_t)k & kCodeMask;
  order[g] = v - p0;
}

__global__ void __launch_bounds__(kThreads) k_batch_karras(const uint32_t* __restrict__ codes,
                                                           const uint32_t* __restrict__ poff,
                                                           const uint32_t* __restrict__ ioff, uint32_t n_scenes,
                                                           float4* __restrict__ nodes, uint32_t* __restrict__ parent) {
  const uint32_t total = __ldg(ioff + n_scenes);
  const uint32_t gi = blockIdx.x * blockDim.x + threadIdx.x;
  const bool active = gi < total;  // every lane stays for the warp searches
  uint32_t s = 0, p0 = 0, i0 = 0, ki = 0;
  int N = 2, i = 0, dprev = -1, dnext = -1;
  if (active) {
    s = segment_of(ioff, n_scenes, gi);
    p0 = __ldg(poff + s);
    i0 = __ldg(ioff + s);
    N = (int)(__ldg(poff + s + 1) - p0);
    i = (int)(gi - i0);
    ki = __ldg(codes + p0 + i);
    dnext = delta32(codes + p0, N, i, i + 1, ki);
    dprev = delta32(codes + p0, N, i, i - 1, ki);
  }
  const int4 ch = karras_node_warp(codes + p0, N, i, ki, dprev, dnext, active);
  if (!active) return;
  float4* nd = nodes + 4 * (size_t)i0;
  uint32_t* par = parent + (2 * (size_t)p0 - s);
  reinterpret_cast<int4*>(nd)[4 * (size_t)i + 3] = make_int4(ch.x, ch.y, ch.x < 0 ? 1 : 0, ch.y < 0 ? 1 : 0);
  par[ch.x >= 0 ? ch.x : (N - 1 + ~ch.x)] = ((uint32_t)i << 1) | 0u;
  par[ch.y >= 0 ? ch.y : (N - 1 + ~ch.y)] = ((uint32_t)i << 1) | 1u;
}

__global__ void __launch_bounds__(kThreads) k_batch_refit(const BatchDesc* __restrict__ desc, int kind,
                                                          const uint32_t* __restrict__ poff,
                                                          const uint32_t* __restrict__ ioff, uint32_t n_scenes,
                                                          const uint32_t* __restrict__ order, float4* nodes,
                                                          const uint32_t* __restrict__ parent, uint32_t* flags,
                                                          float4* __restrict__ prims, float* __restrict__ roots,
                                                          uint32_t* err) {
  const uint32_t total = __ldg(poff + n_scenes);
  const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= total) return;
  const uint32_t s = segment_of(poff, n_scenes, g);
  const uint32_t p0 = __ldg(poff + s), i0 = __ldg(ioff + s);
  const uint32_t n = __ldg(poff + s + 1) - p0, j = g - p0;
  const size_t payload = kind == kTriangles ? 3 : 1;
  Box6 b = emit_prim(kind, desc[s].verts, desc[s].idx, desc[s].sph, __ldg(order + g), prims + payload * p0, j);
  refit_climb(n, j, b, nodes + 4 * (size_t)i0, parent + (2 * (size_t)p0 - s), flags + i0, roots + 8 * (size_t)s, err);
}

#define RQ_BB(call, what)                                            \
  do {                                                               \
    cudaError_t e_ = (call);                                         \
    if (e_ != cudaSuccess) return BuildResult::cuda_error(e_, what); \
  } while (0)

inline unsigned grid(uint64_t n) { return (unsigned)((n + kThreads - 1) / kThreads); }

}  // namespace

int batch_sort_passes(uint32_t n_scenes) {
  int sbits = 0;
  while (n_scenes > 1 && (1u << sbits) < n_scenes) ++sbits;
  return (30 + sbits + 7) / 8;
}

cudaError_t BatchStore::allocate() {
  const uint32_t n = n_scenes, total = poff.back();
  const size_t payload = kind == kTriangles ? 48 : 16;
  const int passes = batch_sort_passes(n);
  cudaError_t e;
  if ((e = desc.ensure(sizeof(BatchDesc) * n)) != cudaSuccess) return e;
  if ((e = offs.ensure(4 * (3 * (size_t)n + 3))) != cudaSuccess) return e;
  if ((e = lohi.ensure(24 * (size_t)n)) != cudaSuccess) return e;
  if ((e = nodes.ensure(64 * std::max<size_t>(1, (size_t)total - n))) != cudaSuccess) return e;
  if ((e = prims.ensure(payload * total)) != cudaSuccess) return e;
  if ((e = order.ensure(4 * (size_t)total)) != cudaSuccess) return e;
  if ((e = codes.ensure(4 * (size_t)total)) != cudaSuccess) return e;
  if ((e = roots.ensure(32 * (size_t)n)) != cudaSuccess) return e;
  if ((e = parent.ensure(4 * (2 * (size_t)total))) != cudaSuccess) return e;
  if ((e = keys.ensure(8 * (size_t)total)) != cudaSuccess) return e;
  if ((e = keys_alt.ensure(8 * (size_t)total)) != cudaSuccess) return e;
  if ((e = vals.ensure(4 * (size_t)total)) != cudaSuccess) return e;
  if ((e = vals_alt.ensure(4 * (size_t)total)) != cudaSuccess) return e;
  zero_words = 2048 + 16 + sort_status_words64(total, passes) + (size_t)total;
  if ((e = zero.ensure(4 * zero_words)) != cudaSuccess) return e;
  return cudaSuccess;
}

cudaError_t BatchStore::upload_tables(cudaStream_t st) {
  // offs = [P (n + 1)] [V (n + 1)] [I (n + 1)]
  std::vector<uint32_t> t;
  t.insert(t.end(), poff.begin(), poff.end());
  t.insert(t.end(), voff.begin(), voff.end());
  for (uint32_t s = 0; s <= n_scenes; ++s) t.push_back(poff[s] - s);
  cudaError_t e = cudaMemcpyAsync(offs.p, t.data(), t.size() * 4, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(desc.p, host_desc.data(), sizeof(BatchDesc) * n_scenes, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);  // the host tables may change after this call
  return e;
}

BuildResult build_batch(BatchStore& b, int morton_mode, uint32_t* err, cudaStream_t st) {
  const uint32_t n = b.n_scenes, total = b.poff.back(), vtotal = b.voff.back();
  const int passes = batch_sort_passes(n);
  const uint32_t* P = b.offs.as<const uint32_t>();
  const uint32_t* V = P + (n + 1);
  const uint32_t* I = V + (n + 1);
  const BatchDesc* desc = b.desc.as<const BatchDesc>();
  uint32_t* z = b.zero.as<uint32_t>();
  RQ_BB(cudaMemsetAsync(z, 0, 4 * b.zero_words, st), "memset");
  uint32_t* flags = z + 2048 + 16 + sort_status_words64(total, passes);
  int32_t* lohi = b.lohi.as<int32_t>();
  count_launch(2);
  k_batch_init_bounds<<<grid(6 * (uint64_t)n), kThreads, 0, st>>>(lohi, n);
  const uint64_t bound_warps = (vtotal + 32u * kBoundsGroups - 1) / (32u * kBoundsGroups);
  k_batch_point_bounds<<<grid(bound_warps * 32), kThreads, 0, st>>>(desc, b.kind, V, n, lohi);
  count_launch();
  k_batch_morton<<<grid(total), kThreads, 0, st>>>(desc, b.kind, morton_mode, P, n, lohi, b.keys.as<uint64_t>(),
                                                   b.vals.as<uint32_t>());
  launch_histogram64(b.keys.as<uint64_t>(), total, passes, z, st);
  launch_onesweep64(b.keys.as<uint64_t>(), b.vals.as<uint32_t>(), total, passes, b.keys_alt.as<uint64_t>(),
                    b.vals_alt.as<uint32_t>(), z, z + 2048 + 16, z + 2048, err, st);
  count_launch(3);
  k_batch_split<<<grid(total), kThreads, 0, st>>>(b.keys.as<const uint64_t>(), b.vals.as<const uint32_t>(), P, n,
                                                  b.codes.as<uint32_t>(), b.order.as<uint32_t>(), err);
  if (total > n)
    k_batch_karras<<<grid(total - n), kThreads, 0, st>>>(b.codes.as<const uint32_t>(), P, I, n, b.nodes.as<float4>(),
                                                          b.parent.as<uint32_t>());
  k_batch_refit<<<grid(total), kThreads, 0, st>>>(desc, b.kind, P, I, n, b.order.as<const uint32_t>(),
                                                  b.nodes.as<float4>(), b.parent.as<const uint32_t>(), flags,
                                                  b.prims.as<float4>(), b.roots.as<float>(), err);
  RQ_BB(cudaGetLastError(), "batched build launch");
  return {};
}

void BatchStore::view(uint32_t s, AccelBuffers& a) const {
  const size_t payload = kind == kTriangles ? 48 : 16;
  const uint32_t p0 = poff[s], n = poff[s + 1] - p0, i0 = p0 - s;
  auto slice = [](DevBuf& d, const DevBuf& base, size_t off, size_t bytes) {
    d.p = static_cast<char*>(base.p) + off;
    d.cap = bytes;
    d.owned = false;
  };
  slice(a.nodes, nodes, 64 * (size_t)i0, 64 * (size_t)std::max<uint32_t>(n - 1, 1));
  slice(a.prims, prims, payload * p0, payload * n);
  slice(a.order, order, 4 * (size_t)p0, 4 * (size_t)n);
  slice(a.codes, codes, 4 * (size_t)p0, 4 * (size_t)n);
  slice(a.root, roots, 32 * (size_t)s, 32);
  a.n_nodes = n > 1 ? n - 1 : 0;
  a.n_slots = n;
  a.max_depth = 0;
  a.node_width = 2;
  a.unit_leaves = true;
}

}  // namespace rq
