// rq_render: the render step for any scene (triangles or spheres) around the
// ray queries, as a wavefront of kernels on the context's stream:
//
//   k_view_rays      pinhole camera rays, spp jittered samples per pixel
//   per depth d = 0..bounces:
//     closest-hit query            (the structure's own traversal)
//     k_shade_hits     Lambert + ambient at the hit, one shadow ray towards the
//                      point light, the mirror ray of the next depth
//     any-hit query on the shadow rays
//     k_shadow_accum   adds the light term of unoccluded samples
//   k_pixels         average of the samples, clamp to [0, 1], x255, truncate
//
// On BVH structures with FAST traversal the shading kernel also compacts the
// samples that emitted a shadow or a mirror ray into index lists (warp
// ballots, one atomic per warp), and later queries run over those lists only.
//
// It generalises castRay's DIFFUSE_AND_GLOSSY shading (main.cpp:390-497) to
// triangle meshes: the reference's own path is rq_render_reference
// (sphere scenes, its camera and light, its pixels); this one drives the
// triangle workloads (one point light, Lambert with a real shadow ray where
// the reference's trace_more is a stub, optional mirror bounces) with every
// operation in IEEE single precision in a fixed order (no fused
// multiply-adds), so the CPU oracle reproduces each pixel.
//
// Per sample: radiance = sum over depths k of w_k * f_k * albedo *
// (ambient + visible_k * max(0, N.L)) + w_miss * background, where w_0 = 1,
// w_{k+1} = w_k * mirror, f_k = (1 - mirror) below the last depth and 1 at
// it.  Normals face the incoming ray; shadow and mirror rays start at
// P + bias * N.
#include "view_device.cuh"

namespace rq {
namespace {

constexpr int kThreads = 128;

__global__ void __launch_bounds__(kThreads) k_view_rays(ViewDev v, uint64_t nray, float4* __restrict__ rays,
                                                        float4* __restrict__ cw) {
  uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nray) return;
  V3 o, d;
  view_ray(v, r, o, d);
  store_ray(rays, r, o, 0.f, d, __int_as_float(0x7F800000));
  cw[r] = make_float4(0.f, 0.f, 0.f, 1.f);
}

// counters[0] += shadow rays emitted, counters[1] += mirror rays emitted.
template <int KIND>
__global__ void __launch_bounds__(kThreads) k_shade_hits(ViewDev v, SceneView sc, uint64_t nray, bool last,
                                                         float4* __restrict__ rays, const float4* __restrict__ hits,
                                                         float4* __restrict__ shadow, float4* __restrict__ cw,
                                                         float4* __restrict__ pend,
                                                         unsigned long long* __restrict__ counters) {
  uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  bool emit_shadow = false, emit_mirror = false;
  if (r < nray) shade_sample<KIND>(v, sc, r, last, rays, hits, shadow, cw, pend, emit_shadow, emit_mirror);
  const uint32_t bs = __ballot_sync(0xffffffffu, emit_shadow), bm = __ballot_sync(0xffffffffu, emit_mirror);
  if ((threadIdx.x & 31) == 0 && (bs | bm)) {
    if (bs) atomicAdd(counters, (unsigned long long)__popc(bs));
    if (bm) atomicAdd(counters + 1, (unsigned long long)__popc(bm));
  }
}

__global__ void __launch_bounds__(kThreads) k_shadow_accum(uint64_t nray, const uint32_t* __restrict__ bits,
                                                           const float4* __restrict__ pend, float4* __restrict__ cw) {
  uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r < nray) shadow_accum(r, bits, pend, cw);
}

__global__ void __launch_bounds__(kThreads) k_pixels(uint64_t npix, uint32_t spp, const float4* __restrict__ cw,
                                                     uint8_t* __restrict__ pixels, float* __restrict__ rgb) {
  uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p < npix) resolve_pixel(p, spp, cw, pixels, rgb);
}

// Warp-aggregated append of r to list when `take` (one atomic per warp).
__device__ __forceinline__ void warp_append(bool take, uint32_t r, uint32_t* __restrict__ list,
                                            uint32_t* __restrict__ count) {
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t bits = __ballot_sync(0xffffffffu, take);
  if (!bits) return;
  const uint32_t leader = __ffs(bits) - 1;
  uint32_t base = 0;
  if (lane == leader) base = atomicAdd(count, (uint32_t)__popc(bits));
  base = __shfl_sync(0xffffffffu, base, leader);
  if (take) list[base + __popc(bits & ((1u << lane) - 1u))] = r;
}

// Shading over a list of live samples (all samples when list is null) that
// also compacts the samples that emitted a shadow ray and a mirror ray into
// s_list / m_list (counts[0], counts[1]).
template <int KIND>
__global__ void __launch_bounds__(kThreads) k_shade_list(ViewDev v, SceneView sc, const uint32_t* __restrict__ list,
                                                         uint32_t n, bool last, float4* __restrict__ rays,
                                                         const float4* __restrict__ hits, float4* __restrict__ shadow,
                                                         float4* __restrict__ cw, float4* __restrict__ pend,
                                                         uint32_t* __restrict__ s_list, uint32_t* __restrict__ m_list,
                                                         uint32_t* __restrict__ counts,
                                                         unsigned long long* __restrict__ counters) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  bool es = false, em = false;
  uint32_t r = 0;
  if (i < n) {
    r = list ? __ldg(list + i) : i;
    shade_sample<KIND, true>(v, sc, r, last, rays, hits, shadow, cw, pend, es, em);
  }
  warp_append(es, r, s_list, counts);
  warp_append(em, r, m_list, counts + 1);
  const uint32_t bs = __ballot_sync(0xffffffffu, es), bm = __ballot_sync(0xffffffffu, em);
  if ((threadIdx.x & 31) == 0 && (bs | bm)) {
    if (bs) atomicAdd(counters, (unsigned long long)__popc(bs));
    if (bm) atomicAdd(counters + 1, (unsigned long long)__popc(bm));
  }
}

__global__ void __launch_bounds__(kThreads) k_accum_list(const uint32_t* __restrict__ list, uint32_t n,
                                                         const uint32_t* __restrict__ bits,
                                                         const float4* __restrict__ pend, float4* __restrict__ cw) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) shadow_accum(__ldg(list + i), bits, pend, cw);
}

}  // namespace

cudaError_t render_view(int type, const SceneView& s, const AccelBuffers& a, const rq_settings_t& cfg,
                        const rq_view_t& view, float tan_half, RenderScratch& rs, BuildScratch& sc,
                        uint8_t* pixels, float* rgb, unsigned long long* counters, uint32_t* err,
                        cudaStream_t st, rq_status_t* status) {
  *status = RQ_SUCCESS;
  const ViewDev v = make_view_dev(view, cfg.width, cfg.height, cfg.aa_samples, cfg.backgroundColor, cfg.bias, tan_half);
  const uint64_t npix = (uint64_t)v.ww * v.wh;
  const uint64_t nray = npix * v.spp;
  cudaError_t e;
  if ((e = rs.rays.ensure(nray * 32)) != cudaSuccess) return e;
  if ((e = rs.shadow.ensure(nray * 32)) != cudaSuccess) return e;
  if ((e = rs.hits.ensure(nray * 16)) != cudaSuccess) return e;
  if ((e = rs.cw.ensure(nray * 16)) != cudaSuccess) return e;
  if ((e = rs.pend.ensure(nray * 16)) != cudaSuccess) return e;
  if ((e = rs.bits.ensure(((nray + 31) / 32) * 4)) != cudaSuccess) return e;
  float4* rays = rs.rays.as<float4>();
  float4* shadow = rs.shadow.as<float4>();
  float4* hits = rs.hits.as<float4>();
  float4* cw = rs.cw.as<float4>();
  float4* pend = rs.pend.as<float4>();
  uint32_t* bits = rs.bits.as<uint32_t>();
  const unsigned gr = (unsigned)((nray + kThreads - 1) / kThreads);
  count_launch();
  k_view_rays<<<gr, kThreads, 0, st>>>(v, nray, rays, cw);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  const bool compact = (type == RQ_LBVH || type == RQ_BVH) && cfg.traversal == RQ_TRAVERSAL_FAST;
  if (compact) {
    // Live-ray compaction: after the camera hits, shadow and mirror queries
    // run over the samples that emitted those rays (lists built by warp
    // ballots in the shading kernel), not over every sample slot.
    if ((e = rs.list_a.ensure(nray * 4)) != cudaSuccess) return e;
    if ((e = rs.list_b.ensure(nray * 4)) != cudaSuccess) return e;
    if ((e = rs.list_s.ensure(nray * 4)) != cudaSuccess) return e;
    if ((e = rs.list_n.ensure(64)) != cudaSuccess) return e;
    if ((e = sc.exact.ensure((nray + 2) * 4)) != cudaSuccess) return e;  // count, work counter, rays
    uint32_t* exact = sc.exact.as<uint32_t>();
    uint32_t* live = nullptr;  // null: every sample (depth 0)
    uint32_t* next = rs.list_a.as<uint32_t>();
    uint32_t* spare = rs.list_b.as<uint32_t>();
    uint32_t* slist = rs.list_s.as<uint32_t>();
    uint32_t* counts = rs.list_n.as<uint32_t>();
    uint32_t n_live = (uint32_t)nray;
    const Bvh2View bv{a.nodes.as<const float4>(), a.prims.as<const float4>(), a.order.as<const uint32_t>(),
                      a.root.as<const float>(), a.n_nodes, a.n_slots, a.unit_leaves ? 1u : 0u};
    const Bvh4View b4{a.nodes4.as<const float4>(), a.prims.as<const float4>(), a.order.as<const uint32_t>(),
                      a.root.as<const float>(), a.n_nodes, a.n_slots};
    const Bvh8View b8{a.nodes4.as<const float4>(), a.prims.as<const float4>(), a.order.as<const uint32_t>(),
                      a.root.as<const float>(), a.n_nodes, a.n_slots};
    for (uint32_t depth = 0; depth <= v.bounces && n_live > 0; ++depth) {
      const bool last = depth == v.bounces;
      if (depth == 0) {
        QueryTarget q;
        q.rays = rays;
        q.n = (uint32_t)nray;
        q.hits = hits;
        BuildResult br = launch_query_sorted(type, s, a, cfg, false, q, sc, err, st);
        if (!br.ok()) {
          *status = br.status;
          return br.cuda;
        }
      } else if (a.node_width == 4) {
        launch_trace_bvh4(s.kind, false, b4, rays, n_live, hits, nullptr, err, st, live);
      } else if (a.node_width == 8) {
        launch_trace_bvh8(s.kind, false, b8, rays, n_live, hits, nullptr, err, st, live);
      } else {
        launch_trace_bvh2(s.kind, RQ_TRAVERSAL_FAST, false, bv, rays, n_live, hits, nullptr, err, st, live, false,
                          exact);
      }
      if ((e = cudaMemsetAsync(counts, 0, 8, st)) != cudaSuccess) return e;
      count_launch();
      const unsigned gl = (n_live + kThreads - 1) / kThreads;
      if (s.kind == kTriangles)
        k_shade_list<kTriangles><<<gl, kThreads, 0, st>>>(v, s, live, n_live, last, rays, hits, shadow, cw, pend,
                                                           slist, next, counts, counters);
      else
        k_shade_list<kSpheres><<<gl, kThreads, 0, st>>>(v, s, live, n_live, last, rays, hits, shadow, cw, pend,
                                                         slist, next, counts, counters);
      if ((e = cudaGetLastError()) != cudaSuccess) return e;
      uint32_t host_counts[2] = {0, 0};
      if ((e = cudaMemcpyAsync(host_counts, counts, 8, cudaMemcpyDeviceToHost, st)) != cudaSuccess) return e;
      if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
      const uint32_t n_shadow = host_counts[0];
      if (n_shadow > 0) {
        // occlusion bits are indexed by sample: clear them all, trace the list
        if ((e = cudaMemsetAsync(bits, 0, ((nray + 31) / 32) * 4, st)) != cudaSuccess) return e;
        if (a.node_width == 4)
          launch_trace_bvh4(s.kind, true, b4, shadow, n_shadow, nullptr, bits, err, st, slist);
        else if (a.node_width == 8)
          launch_trace_bvh8(s.kind, true, b8, shadow, n_shadow, nullptr, bits, err, st, slist);
        else
          launch_trace_bvh2(s.kind, RQ_TRAVERSAL_FAST, true, bv, shadow, n_shadow, nullptr, bits, err, st, slist,
                            false, exact);
        count_launch();
        k_accum_list<<<(n_shadow + kThreads - 1) / kThreads, kThreads, 0, st>>>(slist, n_shadow, bits, pend, cw);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
      }
      n_live = host_counts[1];
      uint32_t* t = next;
      next = live ? live : spare;
      if (!live) spare = nullptr;
      live = t;
    }
  } else {
    for (uint32_t depth = 0; depth <= v.bounces; ++depth) {
      const bool last = depth == v.bounces;
      QueryTarget q;
      q.rays = rays;
      q.n = (uint32_t)nray;
      q.hits = hits;
      BuildResult br = launch_query_sorted(type, s, a, cfg, false, q, sc, err, st);
      if (!br.ok()) {
        *status = br.status;
        return br.cuda;
      }
      count_launch();
      if (s.kind == kTriangles)
        k_shade_hits<kTriangles><<<gr, kThreads, 0, st>>>(v, s, nray, last, rays, hits, shadow, cw, pend, counters);
      else
        k_shade_hits<kSpheres><<<gr, kThreads, 0, st>>>(v, s, nray, last, rays, hits, shadow, cw, pend, counters);
      if ((e = cudaGetLastError()) != cudaSuccess) return e;
      QueryTarget qs;
      qs.rays = shadow;
      qs.n = (uint32_t)nray;
      qs.occ = bits;
      br = launch_query_sorted(type, s, a, cfg, true, qs, sc, err, st);
      if (!br.ok()) {
        *status = br.status;
        return br.cuda;
      }
      count_launch();
      k_shadow_accum<<<gr, kThreads, 0, st>>>(nray, bits, pend, cw);
      if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
  }
  count_launch();
  k_pixels<<<(unsigned)((npix + kThreads - 1) / kThreads), kThreads, 0, st>>>(npix, v.spp, cw, pixels, rgb);
  return cudaGetLastError();
}

}  // namespace rq
