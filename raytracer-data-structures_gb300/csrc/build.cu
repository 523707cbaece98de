// Build orchestration: the dataStructure switch of main() (main.cpp:791-843)
// over the engine's kernels, the LBVH pipeline, query dispatch and
// device-side input validation.
#include <atomic>

#include "rq_build.hpp"
#include "rq_device.cuh"

namespace rq {

static std::atomic<uint64_t> g_launches{0};
void count_launch(uint64_t k) { g_launches.fetch_add(k, std::memory_order_relaxed); }
uint64_t launch_total() { return g_launches.load(std::memory_order_relaxed); }

namespace {

constexpr int kSortPasses = 4;  // 30-bit Morton codes, 8-bit digits

#define RQ_B(call, what)                                           \
  do {                                                             \
    cudaError_t e_ = (call);                                       \
    if (e_ != cudaSuccess) return BuildResult::cuda_error(e_, what); \
  } while (0)

__global__ void k_validate(const float* __restrict__ verts, uint32_t nv, const uint32_t* __restrict__ idx,
                           uint32_t nt, const float4* __restrict__ sph, uint32_t n, uint32_t* err) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  bool bad = false;
  if (i < nv * 3ull) bad |= !isfinite(verts[i]);
  if (i < nt * 3ull) bad |= idx[i] >= nv;
  if (i < n) {
    float4 s = sph[i];
    bad |= !(isfinite(s.x) && isfinite(s.y) && isfinite(s.z) && isfinite(s.w) && s.w >= 0.f);
  }
  if (bad) atomicOr(err, kErrBadInput);
}

}  // namespace

void launch_validate(const float* verts, uint32_t nv, const uint32_t* idx, uint32_t nt,
                     const float4* sph, uint32_t n, uint32_t* err, cudaStream_t st) {
  uint64_t m = (uint64_t)nv * 3;
  if ((uint64_t)nt * 3 > m) m = (uint64_t)nt * 3;
  if (n > m) m = n;
  if (m == 0) return;
  count_launch();
  k_validate<<<(unsigned)((m + 255) / 256), 256, 0, st>>>(verts, nv, idx, nt, sph, n, err);
}

// Zero region layout: [hist 1024][counters 16][status words][refit flags]
// [hist 1024][counters 16][look-back status][refit flags n - 1][top count 4]
static size_t zero_words(uint32_t n, int passes) {
  return 1024 + 16 + sort_status_words(n, passes) + (n > 1 ? n - 1 : 0) + 4;
}

BuildResult sort_pairs(uint32_t* keys, uint32_t* vals, uint32_t n, int passes, bool compute_hist,
                       BuildScratch& sc, uint32_t* err, cudaStream_t st) {
  if (n <= 1) return {};
  RQ_B(sc.keys_alt.ensure((size_t)n * 4), "sort scratch");
  RQ_B(sc.vals_alt.ensure((size_t)n * 4), "sort scratch");
  if (compute_hist) {
    RQ_B(sc.zero.ensure(zero_words(n, passes) * 4), "sort scratch");
    RQ_B(cudaMemsetAsync(sc.zero.p, 0, (1024 + 16 + sort_status_words(n, passes)) * 4, st), "memset");
    launch_histogram(keys, n, passes, sc.zero.as<uint32_t>(), st);
  }
  uint32_t* z = sc.zero.as<uint32_t>();
  SortScratch s{sc.keys_alt.as<uint32_t>(), sc.vals_alt.as<uint32_t>(), z, z + 1040, z + 1024, sc.stall};
  launch_onesweep(keys, vals, n, passes, s, err, st);
  RQ_B(cudaGetLastError(), "radix sort launch");
  return {};
}

// sort_pairs for a permutation whose digit histogram is already in sc.zero
// (zeroed with its look-back words before the histogram was counted): the
// sorted values stay in whichever buffer the last pass wrote (no copy back);
// *perm names it.
BuildResult sort_perm(uint32_t* keys, uint32_t* vals, uint32_t n, int passes, BuildScratch& sc, uint32_t* err,
                      cudaStream_t st, const uint32_t** perm) {
  *perm = vals;
  if (n <= 1) return {};
  RQ_B(sc.keys_alt.ensure((size_t)n * 4), "sort scratch");
  RQ_B(sc.vals_alt.ensure((size_t)n * 4), "sort scratch");
  uint32_t* z = sc.zero.as<uint32_t>();
  SortScratch s{sc.keys_alt.as<uint32_t>(), sc.vals_alt.as<uint32_t>(), z, z + 1040, z + 1024};
  *perm = launch_onesweep_vals(keys, vals, n, passes, s, err, st);
  RQ_B(cudaGetLastError(), "radix sort launch");
  return {};
}

BuildResult morton_codes(const SceneView& s, int mode, uint32_t* codes, uint32_t* vals,
                         uint32_t* hist, BuildScratch& sc, cudaStream_t st) {
  RQ_B(sc.lohi.ensure(64), "scratch");
  int32_t* lohi = sc.lohi.as<int32_t>();
  if (s.kind == kTriangles) {
    launch_init_bounds(lohi, st);
    launch_point_bounds(s.verts, s.nv, 3, lohi, st);
    if (!s.verts4 || !s.idx4) return BuildResult::error(RQ_ERROR_INVALID_ARGUMENT, "triangle scene without packed copies");
    launch_morton_tris(s.verts4, s.idx4, s.n, mode, lohi, codes, vals, hist, st);
  } else {
    if (mode != RQ_MORTON_REFERENCE) {
      launch_init_bounds(lohi, st);
      launch_point_bounds(reinterpret_cast<const float*>(s.sph), s.n, 4, lohi, st);
    }
    launch_morton_spheres(s.sph, s.n, mode, lohi, codes, vals, hist, st);
  }
  RQ_B(cudaGetLastError(), "morton launch");
  return {};
}

static BuildResult build_lbvh(const SceneView& s, const rq_settings_t& cfg, AccelBuffers& a,
                              BuildScratch& sc, uint32_t* err, cudaStream_t st) {
  const uint32_t n = s.n;
  const size_t payload = s.kind == kTriangles ? 48 : 16;
  RQ_B(a.nodes.ensure((size_t)(n > 1 ? n - 1 : 1) * 64), "LBVH nodes");
  RQ_B(a.prims.ensure((size_t)n * payload), "LBVH payload");
  RQ_B(a.order.ensure((size_t)n * 4), "LBVH order");
  RQ_B(a.codes.ensure((size_t)n * 4), "LBVH codes");
  RQ_B(a.root.ensure(32), "LBVH root");
  RQ_B(sc.keys_alt.ensure((size_t)n * 4), "sort scratch");
  RQ_B(sc.vals_alt.ensure((size_t)n * 4), "sort scratch");
  RQ_B(sc.zero.ensure(zero_words(n, kSortPasses) * 4), "build scratch");
  RQ_B(sc.parent.ensure((size_t)(2 * (uint64_t)n) * 4), "parent links");
  RQ_B(sc.mark.ensure(refit_mark_words(n) * 4), "refit marks");
  uint32_t* z = sc.zero.as<uint32_t>();
  RQ_B(cudaMemsetAsync(z, 0, zero_words(n, kSortPasses) * 4, st), "memset");
  uint32_t* codes = a.codes.as<uint32_t>();
  uint32_t* order = a.order.as<uint32_t>();
  BuildResult r = morton_codes(s, cfg.morton, codes, order, z, sc, st);
  if (!r.ok()) return r;
  r = sort_pairs(codes, order, n, kSortPasses, false, sc, err, st);
  if (!r.ok()) return r;
  uint32_t* flags = z + 1040 + sort_status_words(n, kSortPasses);
  uint32_t* mk = sc.mark.as<uint32_t>();
  const RefitTop top{mk, mk + n, mk + refit_treelet_offset(n), flags + (n > 1 ? n - 1 : 0)};
  launch_karras(codes, n, a.nodes.as<float4>(), sc.parent.as<uint32_t>(), top, st);
  const bool treelets = cfg.lbvh_quality == RQ_LBVH_TREELETS && n > 2;
  if (treelets) RQ_B(sc.heights.ensure(n), "treelet scratch");
  RQ_B(launch_refit(s.kind, s.verts4, s.idx4, s.sph, order, n, a.nodes.as<float4>(), sc.parent.as<uint32_t>(),
                    top, flags, a.prims.as<float4>(), a.root.as<float>(), err, st,
                    treelets ? sc.heights.as<uint8_t>() : nullptr),
       "LBVH refit launch");
  if (treelets)
    RQ_B(launch_treelet_opt(n, a.nodes.as<float4>(), sc.parent.as<uint32_t>(), top, sc.heights.as<uint8_t>(), err, st),
         "LBVH treelet launch");
  RQ_B(cudaGetLastError(), "LBVH launch");
  a.n_nodes = n > 1 ? n - 1 : 0;
  a.n_slots = n;
  a.max_depth = 0;
  a.unit_leaves = true;  // Karras leaves are single primitives
  return {};
}

static BuildResult build_none(const SceneView& s, AccelBuffers& a, cudaStream_t st) {
  const size_t payload = s.kind == kTriangles ? 48 : 16;
  RQ_B(a.prims.ensure((size_t)s.n * payload), "payload");
  launch_prims_by_id(s.kind, s.verts, s.idx, s.sph, s.n, a.prims.as<float4>(), nullptr, st);
  RQ_B(cudaGetLastError(), "payload launch");
  a.n_nodes = 0;
  a.n_slots = 0;
  return {};
}

BuildResult build_accel(int type, const SceneView& s, const rq_settings_t& cfg, AccelBuffers& a,
                        BuildScratch& sc, uint32_t* err, cudaStream_t st) {
  if (s.n == 0) return BuildResult::error(RQ_ERROR_EMPTY_SCENE, "empty scene");
  a.node_width = 2;
  a.unit_leaves = false;
  if (cfg.lbvh_quality != RQ_LBVH_KARRAS && cfg.lbvh_quality != RQ_LBVH_TREELETS)
    return BuildResult::error(RQ_ERROR_INVALID_ARGUMENT, "lbvh_quality must be RQ_LBVH_KARRAS or RQ_LBVH_TREELETS");
  if (type == RQ_LBVH || type == RQ_BVH) {
    if (cfg.node_width != RQ_NODE_WIDTH_2 && cfg.node_width != 2 && cfg.node_width != RQ_NODE_WIDTH_4 &&
        cfg.node_width != RQ_NODE_WIDTH_8)
      return BuildResult::error(RQ_ERROR_INVALID_ARGUMENT, "node_width must be 2, 4 or 8");
    BuildResult r = type == RQ_LBVH ? build_lbvh(s, cfg, a, sc, err, st) : build_median_bvh(s, a, sc, err, st);
    if (r.ok() && cfg.node_width == RQ_NODE_WIDTH_4) r = collapse_bvh4(a, sc, err, st);
    if (r.ok() && cfg.node_width == RQ_NODE_WIDTH_8) r = collapse_bvh8(a, sc, err, st);
    return r;
  }
  switch (type) {
    case RQ_KDTREE: return build_kd_tree(s, cfg.kd_max_depth, a, sc, err, st);
    case RQ_NONE: return build_none(s, a, st);
    default: return BuildResult::error(RQ_ERROR_UNSUPPORTED, "unsupported dataStructure");
  }
}

static Bvh4View bvh4_view(const AccelBuffers& a) {
  return {a.nodes4.as<const float4>(), a.prims.as<const float4>(), a.order.as<const uint32_t>(),
          a.root.as<const float>(), a.n_nodes, a.n_slots};
}

static Bvh8View bvh8_view(const AccelBuffers& a) {
  return {a.nodes4.as<const float4>(), a.prims.as<const float4>(), a.order.as<const uint32_t>(),
          a.root.as<const float>(), a.n_nodes, a.n_slots};
}

void launch_query(int type, const SceneView& s, const AccelBuffers& a, int traversal, bool any,
                  const QueryTarget& q, uint32_t* err, cudaStream_t st) {
  if (type == RQ_NONE) {
    launch_trace_brute(s.kind, traversal, any, a.prims.as<const float4>(), s.n, q.rays, q.n, q.hits,
                       q.occ, st);
  } else if (type == RQ_KDTREE) {
    KdView v{a.kd_nodes.as<const int4>(), a.kd_idx.as<const int32_t>(), a.prims.as<const float4>(),
             a.root.as<const float>(), a.n_nodes};
    launch_trace_kd(s.kind, traversal, any, v, q.rays, q.n, q.hits, q.occ, err, st, q.work);
  } else if (a.node_width == 4 && traversal == RQ_TRAVERSAL_FAST) {
    launch_trace_bvh4(s.kind, any, bvh4_view(a), q.rays, q.n, q.hits, q.occ, err, st);
  } else if (a.node_width == 8 && traversal == RQ_TRAVERSAL_FAST) {
    launch_trace_bvh8(s.kind, any, bvh8_view(a), q.rays, q.n, q.hits, q.occ, err, st);
  } else {
    Bvh2View v{a.nodes.as<const float4>(), a.prims.as<const float4>(), a.order.as<const uint32_t>(),
               a.root.as<const float>(), a.n_nodes, a.n_slots, a.unit_leaves ? 1u : 0u};
    launch_trace_bvh2(s.kind, traversal, any, v, q.rays, q.n, q.hits, q.occ, err, st, nullptr, q.small_stack,
                      q.exact);
  }
}

BuildResult launch_query_sorted(int type, const SceneView& s, const AccelBuffers& a, const rq_settings_t& cfg,
                                bool any, const QueryTarget& q, BuildScratch& sc, uint32_t* err, cudaStream_t st) {
  const bool bvh2 = type == RQ_LBVH || type == RQ_BVH;
  const bool fast = bvh2 && cfg.traversal == RQ_TRAVERSAL_FAST;
  const bool sorted = fast && cfg.ray_sort != RQ_RAY_SORT_NONE && q.n >= kRaySortMin;
  const bool wide = a.node_width == 4 || a.node_width == 8;
  const bool refill = fast && cfg.scheduling == RQ_SCHEDULING_LANE_REFILL && !wide;
  const bool spec = fast && cfg.scheduling == RQ_SCHEDULING_SPECULATIVE && !wide;
  const bool packet = fast && cfg.scheduling == RQ_SCHEDULING_WARP_PACKET && !wide;
  const bool top = fast && cfg.scheduling == RQ_SCHEDULING_SHARED_TOP && !wide && !q.small_stack;
  QueryTarget qx = q;
  if (type == RQ_KDTREE) {
    RQ_B(sc.work.ensure(256), "traversal work counter");
    qx.work = sc.work.as<uint32_t>();
  }
  if (bvh2 && cfg.traversal == RQ_TRAVERSAL_FAST && a.node_width == 2 && !q.small_stack) {
    RQ_B(sc.exact.ensure(((size_t)q.n + 2) * 4), "exact-ray list");  // count, work counter, rays
    qx.exact = sc.exact.as<uint32_t>();
  }
  if (!sorted && !refill && !spec && !packet && !top) {
    launch_query(type, s, a, cfg.traversal, any, qx, err, st);
    RQ_B(cudaGetLastError(), "trace launch");
    return {};
  }
  const uint32_t* perm = nullptr;
  if (sorted) {
    // Coherence order: sort (octant | origin Morton, index) pairs, then trace
    // through the permutation; results keep the caller's order.
    RQ_B(sc.vals.ensure((size_t)q.n * 4), "ray sort scratch");
    uint32_t* p = sc.vals.as<uint32_t>();
    if (cfg.ray_sort == RQ_RAY_SORT_OCTANT || cfg.ray_sort == RQ_RAY_SORT_OCTANT_MORTON3) {
      // keys of 3 or 6 bits: a stable counting sort, same order
      RQ_B(sc.keys.ensure(ray_order_small_bytes(q.n, cfg.ray_sort)), "ray sort scratch");
      launch_ray_order_small(q.rays, q.n, a.root.as<const float>(), cfg.ray_sort, sc.keys.p, p, st);
      RQ_B(cudaGetLastError(), "ray order launch");
      perm = p;
    } else {
      RQ_B(sc.keys.ensure((size_t)q.n * 4), "ray sort scratch");
      uint32_t* keys = sc.keys.as<uint32_t>();
      const int passes = cfg.ray_sort == RQ_RAY_SORT_OCTANT_MORTON12 ? 2 : 4;
      RQ_B(sc.zero.ensure(zero_words(q.n, passes) * 4), "sort scratch");
      RQ_B(cudaMemsetAsync(sc.zero.p, 0, (1024 + 16 + sort_status_words(q.n, passes)) * 4, st), "memset");
      launch_ray_keys(q.rays, q.n, a.root.as<const float>(), cfg.ray_sort, keys, p, st, sc.zero.as<uint32_t>(), passes);
      BuildResult r = sort_perm(keys, p, q.n, passes, sc, err, st, &perm);
      if (!r.ok()) return r;
    }
  }
  Bvh2View v{a.nodes.as<const float4>(), a.prims.as<const float4>(), a.order.as<const uint32_t>(),
             a.root.as<const float>(), a.n_nodes, a.n_slots, a.unit_leaves ? 1u : 0u};
  if (top) {
    RQ_B(sc.top.ensure(64 * 64), "top-level copy");
    launch_trace_bvh2_top(s.kind, any, v, sc.top.as<float4>(), q.rays, q.n, q.hits, q.occ, err, perm, st);
    RQ_B(cudaGetLastError(), "trace launch");
    return {};
  }
  if (packet) {
    launch_trace_bvh2_packet(s.kind, any, v, q.rays, q.n, q.hits, q.occ, err, perm, st);
    RQ_B(cudaGetLastError(), "trace launch");
    return {};
  }
  if (spec) {
    launch_trace_bvh2_spec(s.kind, any, v, q.rays, q.n, q.hits, q.occ, err, perm, st);
    RQ_B(cudaGetLastError(), "trace launch");
    return {};
  }
  if (refill) {
    RQ_B(sc.work.ensure(256), "traversal work counter");
    RQ_B(launch_trace_bvh2_refill(s.kind, any, v, q.rays, q.n, q.hits, q.occ, err, perm, sc.work.as<uint32_t>(), st),
         "trace launch");
    return {};
  }
  if (a.node_width == 4) launch_trace_bvh4(s.kind, any, bvh4_view(a), q.rays, q.n, q.hits, q.occ, err, st, perm);
  else if (a.node_width == 8) launch_trace_bvh8(s.kind, any, bvh8_view(a), q.rays, q.n, q.hits, q.occ, err, st, perm);
  else launch_trace_bvh2(s.kind, cfg.traversal, any, v, q.rays, q.n, q.hits, q.occ, err, st, perm, q.small_stack,
                         qx.exact);
  RQ_B(cudaGetLastError(), "trace launch");
  return {};
}

BuildResult trace_counted(int type, const SceneView& s, const AccelBuffers& a, bool any, const QueryTarget& q,
                          unsigned long long* counters, uint32_t* err, cudaStream_t st) {
  if (type != RQ_LBVH && type != RQ_BVH)
    return BuildResult::error(RQ_ERROR_UNSUPPORTED, "traversal counters exist for BVH2 structures");
  if (a.node_width == 4) {
    launch_trace_bvh4(s.kind, any, bvh4_view(a), q.rays, q.n, q.hits, q.occ, err, st, nullptr, counters);
    RQ_B(cudaGetLastError(), "counted trace launch");
    return {};
  }
  if (a.node_width == 8) {
    launch_trace_bvh8(s.kind, any, bvh8_view(a), q.rays, q.n, q.hits, q.occ, err, st, nullptr, counters);
    RQ_B(cudaGetLastError(), "counted trace launch");
    return {};
  }
  Bvh2View v{a.nodes.as<const float4>(), a.prims.as<const float4>(), a.order.as<const uint32_t>(),
             a.root.as<const float>(), a.n_nodes, a.n_slots};
  launch_trace_bvh2_counted(s.kind, any, v, q.rays, q.n, q.hits, q.occ, err, counters, st);
  RQ_B(cudaGetLastError(), "counted trace launch");
  return {};
}

}  // namespace rq
