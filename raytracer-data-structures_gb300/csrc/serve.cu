// Serving loop (rq_server_*): render requests against a library of meshes,
// served by one worker thread that owns its own context.
//
//  * Admission: a request must name a registered mesh and fit the ray limit
//    of one batch; its mesh must fit the HBM budget.  Others complete at once
//    with an error status.
//  * Residency: meshes live on the host; a request's mesh is uploaded and its
//    LBVH built when needed.  Resident scenes + structures stay within the
//    HBM budget by evicting the least recently used meshes that the batch
//    being formed does not need.
//  * Continuous batching: each step takes the waiting requests in arrival
//    order up to the batch limits and renders all of them as one wavefront:
//    camera rays of every request, one persistent many-structure closest-hit
//    query, shading, one many-structure shadow query, the light terms and
//    every request's pixels, then one download.  batching = 0 serves one
//    request per step (the one-request-per-launch comparison).
//  * Latency: from rq_server_submit to the moment the request's pixels are
//    in host memory; the worker keeps every completed request's latency for
//    the percentile statistics.
//
// A request renders exactly what rq_render renders for the same view with
// bounces = 0 (the same per-sample device code), whether it is served alone
// or among others.  The reference has no serving path; this is the engine's.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <unordered_map>

#include "rq_handles.hpp"
#include "view_device.cuh"

namespace rq {
namespace {

constexpr int kThreads = 128;

struct ServeReq {  // device table entry: one request of a batch
  ViewDev v;
  SceneView sc;
};

__global__ void __launch_bounds__(kThreads) k_serve_rays(const ServeReq* __restrict__ reqs,
                                                         const uint32_t* __restrict__ roff, uint32_t n_req,
                                                         uint32_t nray, float4* __restrict__ rays,
                                                         float4* __restrict__ cw) {
  const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nray) return;
  const uint32_t q = segment_of(roff, n_req, r);
  V3 o, d;
  view_ray(reqs[q].v, r - __ldg(roff + q), o, d);
  store_ray(rays, r, o, 0.f, d, __int_as_float(0x7F800000));
  cw[r] = make_float4(0.f, 0.f, 0.f, 1.f);
}

__global__ void __launch_bounds__(kThreads) k_serve_shade(const ServeReq* __restrict__ reqs,
                                                          const uint32_t* __restrict__ roff, uint32_t n_req,
                                                          uint32_t nray, float4* __restrict__ rays,
                                                          const float4* __restrict__ hits, float4* __restrict__ shadow,
                                                          float4* __restrict__ cw, float4* __restrict__ pend,
                                                          unsigned long long* __restrict__ counters) {
  const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  bool es = false, em = false;
  if (r < nray) {
    const uint32_t q = segment_of(roff, n_req, r);
    shade_sample<kTriangles>(reqs[q].v, reqs[q].sc, r, true, rays, hits, shadow, cw, pend, es, em);
  }
  const uint32_t bs = __ballot_sync(0xffffffffu, es);
  if ((threadIdx.x & 31) == 0 && bs) atomicAdd(counters, (unsigned long long)__popc(bs));
}

__global__ void __launch_bounds__(kThreads) k_serve_accum(uint32_t nray, const uint32_t* __restrict__ bits,
                                                          const float4* __restrict__ pend, float4* __restrict__ cw) {
  const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r < nray) shadow_accum(r, bits, pend, cw);
}

__global__ void __launch_bounds__(kThreads) k_serve_pixels(const ServeReq* __restrict__ reqs,
                                                           const uint32_t* __restrict__ roff,
                                                           const uint32_t* __restrict__ poff, uint32_t n_req,
                                                           uint32_t npix, const float4* __restrict__ cw,
                                                           uint8_t* __restrict__ pixels) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= npix) return;
  const uint32_t q = segment_of(poff, n_req, p);
  const uint32_t p0 = __ldg(poff + q);
  resolve_pixel(p - p0, reqs[q].v.spp, cw + __ldg(roff + q), pixels + 3 * (size_t)p0, nullptr);
}

using Clock = std::chrono::steady_clock;

struct Mesh {
  std::vector<float> verts;
  std::vector<uint32_t> idx;
  rq_scene_t scene = nullptr;
  rq_accel_t accel = nullptr;
  uint64_t bytes = 0;     // device bytes while resident
  uint64_t last_use = 0;  // batch counter of the last use
};

struct Pending {
  uint64_t ticket = 0;
  rq_request_t req{};
  Clock::time_point t_submit;
  bool done = false;
  rq_status_t status = RQ_SUCCESS;
  std::vector<uint8_t> pixels;
};

}  // namespace
}  // namespace rq

using namespace rq;

struct rq_server {
  rq_server_config_t cfg{};
  rq_ctx_t ctx = nullptr;
  std::mutex m;
  std::condition_variable cv_work, cv_done;
  std::deque<Pending*> queue;
  std::unordered_map<uint64_t, std::unique_ptr<Pending>> reqs;
  std::unordered_map<uint32_t, std::unique_ptr<Mesh>> meshes;
  uint64_t next_ticket = 1;
  bool stop = false;
  std::thread worker;
  // worker-only state
  uint64_t batch_no = 0;
  uint64_t resident = 0;
  DevBuf rays, shadow, hits, cw, pend, bits, pix, table, counters;
  uint8_t* host_pix = nullptr;  // pinned download buffer
  size_t host_pix_cap = 0;
  // statistics (under m)
  rq_server_stats_t st{};
  std::vector<double> lat_ms;
  std::string worker_error;

  void run();
  void serve(std::vector<Pending*>& batch);
  rq_status_t make_resident(Mesh& mesh, const std::vector<Mesh*>& keep);
  void finish(std::vector<Pending*>& batch, const std::vector<rq_status_t>& status);
};

namespace {

uint64_t mesh_device_bytes(const Mesh& m) {
  const uint64_t nt = m.idx.size() / 3, nv = m.verts.size() / 3;
  // scene (vertices + indices) + LBVH (nodes, payload, order, codes, root)
  return nv * 12 + nt * 12 + (nt > 1 ? nt - 1 : 1) * 64 + nt * 48 + nt * 8 + 256;
}

}  // namespace

rq_status_t rq_server::make_resident(Mesh& mesh, const std::vector<Mesh*>& keep) {
  if (mesh.accel) return RQ_SUCCESS;
  const uint64_t need = mesh_device_bytes(mesh);
  if (need > cfg.hbm_budget) return RQ_ERROR_OUT_OF_MEMORY;
  // least recently used first, never a mesh the current batch needs
  while (resident + need > cfg.hbm_budget) {
    Mesh* lru = nullptr;
    {
      std::lock_guard<std::mutex> g(m);
      for (auto& kv : meshes) {
        Mesh* c = kv.second.get();
        if (!c->accel || std::find(keep.begin(), keep.end(), c) != keep.end()) continue;
        if (!lru || c->last_use < lru->last_use) lru = c;
      }
    }
    if (!lru) return RQ_ERROR_OUT_OF_MEMORY;
    rq_accel_destroy(lru->accel);
    rq_scene_destroy(lru->scene);
    lru->accel = nullptr;
    lru->scene = nullptr;
    resident -= lru->bytes;
    lru->bytes = 0;
    std::lock_guard<std::mutex> g(m);
    ++st.evictions;
  }
  rq_status_t s = rq_scene_create_triangles(ctx, mesh.verts.data(), (uint32_t)(mesh.verts.size() / 3),
                                            mesh.idx.data(), (uint32_t)(mesh.idx.size() / 3), 0, &mesh.scene);
  if (s != RQ_SUCCESS) return s;
  s = rq_build(ctx, mesh.scene, RQ_LBVH, &mesh.accel);
  if (s != RQ_SUCCESS) {
    rq_scene_destroy(mesh.scene);
    mesh.scene = nullptr;
    return s;
  }
  mesh.bytes = need;
  resident += need;
  std::lock_guard<std::mutex> g(m);
  ++st.builds;
  return RQ_SUCCESS;
}

void rq_server::finish(std::vector<Pending*>& batch, const std::vector<rq_status_t>& status) {
  const Clock::time_point now = Clock::now();
  {
    std::lock_guard<std::mutex> g(m);
    for (size_t k = 0; k < batch.size(); ++k) {
      Pending* p = batch[k];
      p->status = status[k];
      p->done = true;
      if (status[k] == RQ_SUCCESS) {
        ++st.completed;
        lat_ms.push_back(std::chrono::duration<double, std::milli>(now - p->t_submit).count());
      } else {
        ++st.rejected;
      }
    }
  }
  cv_done.notify_all();
}

void rq_server::serve(std::vector<Pending*>& batch) {
  const size_t n = batch.size();
  std::vector<rq_status_t> status(n, RQ_SUCCESS);
  std::vector<Mesh*> mesh(n, nullptr);
  ++batch_no;
  {
    std::lock_guard<std::mutex> g(m);
    for (size_t k = 0; k < n; ++k) {
      auto it = meshes.find(batch[k]->req.mesh_id);
      if (it == meshes.end()) status[k] = RQ_ERROR_INVALID_ARGUMENT;
      else mesh[k] = it->second.get();
    }
  }
  for (size_t k = 0; k < n; ++k) {
    if (status[k] != RQ_SUCCESS) continue;
    status[k] = make_resident(*mesh[k], mesh);
    if (status[k] == RQ_SUCCESS) mesh[k]->last_use = batch_no;
  }
  // Tables of the requests that go ahead.
  std::vector<ServeReq> sreq;
  std::vector<Bvh2View> views;
  std::vector<uint32_t> roff(1, 0), poff(1, 0);
  std::vector<size_t> which;
  for (size_t k = 0; k < n; ++k) {
    if (status[k] != RQ_SUCCESS) continue;
    const rq_request_t& r = batch[k]->req;
    const float tan_half = (float)std::tan((double)r.view.fov_deg * 3.141592653589793 / 360.0);
    rq_view_t view = r.view;
    view.bounces = 0;
    view.window[0] = view.window[1] = view.window[2] = view.window[3] = 0;
    ServeReq q;
    q.v = make_view_dev(view, r.width, r.height, r.spp, r.background, ctx->settings.bias, tan_half);
    rq_scene_t sc = mesh[k]->scene;
    q.sc.kind = kTriangles;
    q.sc.n = sc->n;
    q.sc.nv = sc->nv;
    q.sc.verts = sc->verts.as<const float>();
    q.sc.idx = sc->idx.as<const uint32_t>();
    q.sc.sph = nullptr;
    q.sc.verts4 = sc->verts4.as<const float4>();
    q.sc.idx4 = sc->idx4.as<const uint4>();
    sreq.push_back(q);
    const AccelBuffers& b = mesh[k]->accel->buf;
    views.push_back({b.nodes.as<const float4>(), b.prims.as<const float4>(), b.order.as<const uint32_t>(),
                     b.root.as<const float>(), b.n_nodes, b.n_slots});
    roff.push_back(roff.back() + r.width * r.height * r.spp);
    poff.push_back(poff.back() + r.width * r.height);
    which.push_back(k);
  }
  const uint32_t nq = (uint32_t)which.size();
  const uint32_t nray = roff.back(), npix = poff.back();
  cudaStream_t s = ctx->stream;
  cudaError_t e = cudaSuccess;
  if (nq > 0) {
    // device table: [ServeReq n][Bvh2View n][roff n+1][poff n+1][work]
    const size_t a0 = 0, a1 = (sizeof(ServeReq) * nq + 15) & ~size_t(15);
    const size_t a2 = a1 + ((sizeof(Bvh2View) * nq + 15) & ~size_t(15));
    const size_t a3 = a2 + ((4 * ((size_t)nq + 1) + 15) & ~size_t(15));
    const size_t a4 = a3 + ((4 * ((size_t)nq + 1) + 15) & ~size_t(15));
    std::vector<char> host(a4 + 16, 0);
    std::memcpy(host.data() + a0, sreq.data(), sizeof(ServeReq) * nq);
    std::memcpy(host.data() + a1, views.data(), sizeof(Bvh2View) * nq);
    std::memcpy(host.data() + a2, roff.data(), 4 * ((size_t)nq + 1));
    std::memcpy(host.data() + a3, poff.data(), 4 * ((size_t)nq + 1));
    if (e == cudaSuccess) e = table.ensure(host.size());
    if (e == cudaSuccess) e = rays.ensure((size_t)nray * 32);
    if (e == cudaSuccess) e = shadow.ensure((size_t)nray * 32);
    if (e == cudaSuccess) e = hits.ensure((size_t)nray * 16);
    if (e == cudaSuccess) e = cw.ensure((size_t)nray * 16);
    if (e == cudaSuccess) e = pend.ensure((size_t)nray * 16);
    if (e == cudaSuccess) e = bits.ensure((((size_t)nray + 31) / 32) * 4);
    if (e == cudaSuccess) e = pix.ensure((size_t)npix * 3);
    if (e == cudaSuccess) e = counters.ensure(16);
    if (e == cudaSuccess) e = cudaMemcpyAsync(table.p, host.data(), host.size(), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(counters.p, 0, 16, s);
    char* tb = table.as<char>();
    const ServeReq* d_req = reinterpret_cast<const ServeReq*>(tb + a0);
    const uint32_t* d_roff = reinterpret_cast<const uint32_t*>(tb + a2);
    const uint32_t* d_poff = reinterpret_cast<const uint32_t*>(tb + a3);
    const unsigned gr = (nray + kThreads - 1) / kThreads;
    if (e == cudaSuccess) {
      count_launch();
      k_serve_rays<<<gr, kThreads, 0, s>>>(d_req, d_roff, nq, nray, rays.as<float4>(), cw.as<float4>());
      e = cudaGetLastError();
    }
    BatchedTrace t;
    t.kind = kTriangles;
    t.width = 2;
    t.views = reinterpret_cast<const Bvh2View*>(tb + a1);
    t.roff = d_roff;
    t.n_views = nq;
    t.n = nray;
    t.work = reinterpret_cast<uint32_t*>(tb + a4);
    t.err = ctx->d_err;
    if (e == cudaSuccess) {
      t.any = false;
      t.rays = rays.as<const float4>();
      t.hits = hits.as<float4>();
      e = launch_trace_batched(t, 128, 1, s);
    }
    if (e == cudaSuccess) {
      count_launch();
      k_serve_shade<<<gr, kThreads, 0, s>>>(d_req, d_roff, nq, nray, rays.as<float4>(), hits.as<const float4>(),
                                            shadow.as<float4>(), cw.as<float4>(), pend.as<float4>(),
                                            counters.as<unsigned long long>());
      e = cudaGetLastError();
    }
    if (e == cudaSuccess) {
      t.any = true;
      t.rays = shadow.as<const float4>();
      t.hits = nullptr;
      t.occ = bits.as<uint32_t>();
      e = launch_trace_batched(t, 128, 1, s);
    }
    if (e == cudaSuccess) {
      count_launch(2);
      k_serve_accum<<<gr, kThreads, 0, s>>>(nray, bits.as<const uint32_t>(), pend.as<const float4>(), cw.as<float4>());
      k_serve_pixels<<<(npix + kThreads - 1) / kThreads, kThreads, 0, s>>>(d_req, d_roff, d_poff, nq, npix,
                                                                            cw.as<const float4>(), pix.as<uint8_t>());
      e = cudaGetLastError();
    }
    uint64_t shadow_rays = 0;
    if (e == cudaSuccess && host_pix_cap < (size_t)npix * 3) {
      if (host_pix) cudaFreeHost(host_pix);
      host_pix = nullptr;
      host_pix_cap = 0;
      e = cudaMallocHost(&host_pix, (size_t)npix * 3);
      if (e == cudaSuccess) host_pix_cap = (size_t)npix * 3;
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(host_pix, pix.p, (size_t)npix * 3, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&shadow_rays, counters.p, 8, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    uint32_t derr = 0;
    if (e == cudaSuccess) e = cudaMemcpy(&derr, ctx->d_err, 4, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && derr) e = cudaMemset(ctx->d_err, 0, 4);
    if (e != cudaSuccess || derr) {
      std::lock_guard<std::mutex> g(m);
      worker_error = e != cudaSuccess ? cudaGetErrorString(e) : "device error flag set during a batch";
      cudaGetLastError();
    }
    for (uint32_t j = 0; j < nq; ++j) {
      const size_t k = which[j];
      if (e != cudaSuccess || derr) {
        status[k] = e != cudaSuccess ? RQ_ERROR_CUDA : RQ_ERROR_INVALID_ARGUMENT;
        continue;
      }
      if (batch[k]->req.keep_pixels)
        batch[k]->pixels.assign(host_pix + 3 * (size_t)poff[j], host_pix + 3 * (size_t)poff[j + 1]);
    }
    std::lock_guard<std::mutex> g(m);
    ++st.batches;
    st.camera_rays += nray;
    st.shadow_rays += shadow_rays;
    st.resident_bytes = resident;
  }
  finish(batch, status);
}

void rq_server::run() {
  if (cudaSetDevice(cfg.device) != cudaSuccess) return;
  for (;;) {
    std::vector<Pending*> batch;
    {
      std::unique_lock<std::mutex> lk(m);
      cv_work.wait(lk, [&] { return stop || !queue.empty(); });
      if (stop) return;
      // continuous batching: everything waiting, in arrival order, up to the limits
      uint64_t rays_in = 0;
      while (!queue.empty()) {
        Pending* p = queue.front();
        const uint64_t r = (uint64_t)p->req.width * p->req.height * p->req.spp;
        if (!batch.empty() && (!cfg.batching || batch.size() >= cfg.max_batch_requests ||
                               rays_in + r > cfg.max_batch_rays))
          break;
        batch.push_back(p);
        rays_in += r;
        queue.pop_front();
      }
    }
    const Clock::time_point t0 = Clock::now();
    serve(batch);
    const double dt = std::chrono::duration<double>(Clock::now() - t0).count();
    std::lock_guard<std::mutex> g(m);
    st.busy_s += dt;
  }
}

extern "C" {

rq_status_t rq_server_create(const rq_server_config_t* cfg, rq_server_t* out) {
  if (!out) return RQ_ERROR_INVALID_ARGUMENT;
  *out = nullptr;
  std::unique_ptr<rq_server> s(new (std::nothrow) rq_server());
  if (!s) return RQ_ERROR_OUT_OF_MEMORY;
  if (cfg) s->cfg = *cfg;
  else s->cfg.batching = 1;
  if (s->cfg.hbm_budget == 0) s->cfg.hbm_budget = 80ull << 30;
  if (s->cfg.max_batch_rays == 0) s->cfg.max_batch_rays = 1u << 25;
  if (s->cfg.max_batch_requests == 0) s->cfg.max_batch_requests = 256;
  if (s->cfg.max_batch_rays >= (1u << 31)) return RQ_ERROR_INVALID_ARGUMENT;
  // the server's own context: cube Morton normalisation (tighter LBVHs on
  // flat scenes; results do not depend on the tree)
  rq_settings_t settings;
  rq_settings_default(&settings);
  settings.morton = RQ_MORTON_SCENE_CUBE;
  rq_status_t st = rq_create(&settings, s->cfg.device, &s->ctx);
  if (st != RQ_SUCCESS) return st;
  rq_server* raw = s.get();
  s->worker = std::thread([raw] { raw->run(); });
  *out = s.release();
  return RQ_SUCCESS;
}

rq_status_t rq_server_add_mesh(rq_server_t s, uint32_t mesh_id, const float* verts, uint32_t nv,
                               const uint32_t* idx, uint32_t nt) {
  if (!s || !verts || !idx || nv == 0) return RQ_ERROR_INVALID_ARGUMENT;
  if (nt == 0) return RQ_ERROR_EMPTY_SCENE;
  if (nt >= (1u << 30)) return RQ_ERROR_INVALID_ARGUMENT;
  for (size_t i = 0; i < (size_t)nt * 3; ++i)
    if (idx[i] >= nv) return RQ_ERROR_INVALID_ARGUMENT;
  for (size_t i = 0; i < (size_t)nv * 3; ++i)
    if (!std::isfinite(verts[i])) return RQ_ERROR_INVALID_ARGUMENT;
  auto mesh = std::make_unique<Mesh>();
  mesh->verts.assign(verts, verts + (size_t)nv * 3);
  mesh->idx.assign(idx, idx + (size_t)nt * 3);
  std::lock_guard<std::mutex> g(s->m);
  if (s->meshes.count(mesh_id)) return RQ_ERROR_INVALID_ARGUMENT;
  s->meshes.emplace(mesh_id, std::move(mesh));
  return RQ_SUCCESS;
}

rq_status_t rq_server_submit(rq_server_t s, const rq_request_t* req, uint64_t* ticket) {
  if (!s || !req || !ticket) return RQ_ERROR_INVALID_ARGUMENT;
  const uint64_t r = (uint64_t)req->width * req->height * req->spp;
  if (req->width == 0 || req->height == 0 || req->spp == 0 || r > s->cfg.max_batch_rays ||
      !(req->view.fov_deg > 0.f && req->view.fov_deg < 180.f))
    return RQ_ERROR_INVALID_ARGUMENT;
  auto p = std::make_unique<Pending>();
  p->req = *req;
  p->t_submit = Clock::now();
  {
    std::lock_guard<std::mutex> g(s->m);
    p->ticket = s->next_ticket++;
    *ticket = p->ticket;
    s->queue.push_back(p.get());
    s->reqs.emplace(p->ticket, std::move(p));
    ++s->st.submitted;
  }
  s->cv_work.notify_one();
  return RQ_SUCCESS;
}

rq_status_t rq_server_wait(rq_server_t s, uint64_t ticket, uint8_t* pixels, double timeout_s) {
  if (!s) return RQ_ERROR_INVALID_ARGUMENT;
  std::unique_lock<std::mutex> lk(s->m);
  auto it = s->reqs.find(ticket);
  if (it == s->reqs.end()) return RQ_ERROR_INVALID_ARGUMENT;
  Pending* p = it->second.get();
  const auto pred = [&] { return p->done; };
  if (timeout_s >= 0) {
    if (!s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), pred)) return RQ_ERROR_TIMEOUT;
  } else {
    s->cv_done.wait(lk, pred);
  }
  const rq_status_t st = p->status;
  if (st == RQ_SUCCESS && pixels && !p->pixels.empty()) std::memcpy(pixels, p->pixels.data(), p->pixels.size());
  s->reqs.erase(it);
  return st;
}

rq_status_t rq_server_drain(rq_server_t s, double timeout_s) {
  if (!s) return RQ_ERROR_INVALID_ARGUMENT;
  std::unique_lock<std::mutex> lk(s->m);
  const auto pred = [&] { return s->st.completed + s->st.rejected == s->st.submitted; };
  if (timeout_s >= 0) {
    if (!s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), pred)) return RQ_ERROR_TIMEOUT;
  } else {
    s->cv_done.wait(lk, pred);
  }
  return RQ_SUCCESS;
}

rq_status_t rq_server_get_stats(rq_server_t s, rq_server_stats_t* out) {
  if (!s || !out) return RQ_ERROR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> g(s->m);
  *out = s->st;
  uint64_t resident_meshes = 0;
  for (auto& kv : s->meshes) resident_meshes += kv.second->accel ? 1 : 0;
  out->resident_meshes = resident_meshes;
  std::vector<double> l = s->lat_ms;
  if (!l.empty()) {
    std::sort(l.begin(), l.end());
    auto pct = [&](double q) {
      size_t i = (size_t)std::ceil(q * (double)l.size()) - 1;
      return l[std::min(i, l.size() - 1)];
    };
    double sum = 0;
    for (double x : l) sum += x;
    out->latency_ms_p50 = pct(0.50);
    out->latency_ms_p99 = pct(0.99);
    out->latency_ms_mean = sum / (double)l.size();
    out->latency_ms_max = l.back();
  }
  return RQ_SUCCESS;
}

rq_status_t rq_server_reset_stats(rq_server_t s) {
  if (!s) return RQ_ERROR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> g(s->m);
  const uint64_t outstanding = s->st.submitted - s->st.completed - s->st.rejected;
  const uint64_t resident = s->st.resident_bytes;
  s->st = rq_server_stats_t{};
  s->st.submitted = outstanding;
  s->st.resident_bytes = resident;
  s->lat_ms.clear();
  return RQ_SUCCESS;
}

const char* rq_server_last_error(rq_server_t s) {
  if (!s) return "";
  std::lock_guard<std::mutex> g(s->m);
  return s->worker_error.c_str();
}

rq_status_t rq_server_destroy(rq_server_t s) {
  if (!s) return RQ_ERROR_INVALID_ARGUMENT;
  {
    std::lock_guard<std::mutex> g(s->m);
    s->stop = true;
  }
  s->cv_work.notify_all();
  if (s->worker.joinable()) s->worker.join();
  cudaSetDevice(s->cfg.device);
  for (auto& kv : s->meshes) {
    if (kv.second->accel) rq_accel_destroy(kv.second->accel);
    if (kv.second->scene) rq_scene_destroy(kv.second->scene);
  }
  s->rays.release(); s->shadow.release(); s->hits.release(); s->cw.release(); s->pend.release();
  s->bits.release(); s->pix.release(); s->table.release(); s->counters.release();
  if (s->host_pix) cudaFreeHost(s->host_pix);
  rq_destroy(s->ctx);
  delete s;
  return RQ_SUCCESS;
}

}  // extern "C"
