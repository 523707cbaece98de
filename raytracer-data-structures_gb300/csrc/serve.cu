// Serving loop (rq_server_*): render requests against a library of meshes,
// served by one worker thread that owns its own contexts.
//
//  * Admission: a request must name a registered mesh and fit the ray limit
//    of one batch; its mesh must fit the HBM budget.  Others complete at once
//    with an error status.
//  * Residency: meshes live on the host; a request's mesh is uploaded and its
//    LBVH built when needed, through a second context on its own stream, so
//    uploads and builds run on the GPU beside the rendering already in
//    flight.  Resident scenes + structures and the wavefront buffers stay
//    within the HBM budget: the least recently used meshes that neither the
//    batch being formed nor a batch in flight needs are evicted.
//  * Continuous batching (batching = 1): two wavefront slots, each with its
//    own stream and buffers.  A step takes rows of the waiting requests, in
//    arrival order, up to a bounded number of camera rays (step_rays); a
//    larger request is split by rows (a window of its image: the same
//    samples as the whole image's) and finished in later steps, so no
//    request holds the GPU for long.  While one slot's step runs, the rows
//    waiting are formed into the next step on the other slot, which starts
//    on the GPU beside it.  A step renders all its rows as one wavefront:
//    camera rays, one persistent many-structure closest-hit query, shading,
//    one many-structure shadow query, the light terms and the pixels, then
//    one download; a host callback on the slot's stream tells the worker
//    when it has landed, and a request completes with its last rows.
//    batching = 0 serves one whole request per step on one slot, each step
//    waited for before the next (the one-request-per-launch comparison).
//  * Latency: from rq_server_submit to the moment the request's pixels are
//    in host memory; the worker keeps every completed request's latency for
//    the percentile statistics.  Busy time is the time at least one step is
//    in flight.
//
// A request renders exactly what rq_render renders for the same view with
// bounces = 0 (the same per-sample device code), whether it is served alone
// or among others.  The reference has no serving path; this is the engine's.
#include <algorithm>
#include <atomic>
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

// Wavefront bytes per camera sample: camera/mirror ray 32, shadow ray 32,
// hit 16, colour + weight 16, pending light term 16, occlusion bit.
constexpr uint64_t kSampleBytes = 112;

struct Mesh {
  std::vector<float> verts;
  std::vector<uint32_t> idx;
  rq_scene_t scene = nullptr;
  rq_accel_t accel = nullptr;
  uint64_t bytes = 0;     // device bytes while resident (scene copies + structure)
  uint64_t last_use = 0;  // batch counter of the last use
  int in_flight = 0;      // steps in flight that read it (never evicted then)
};

struct Pending {
  uint64_t ticket = 0;
  rq_request_t req{};
  Clock::time_point t_submit;
  bool done = false;
  rq_status_t status = RQ_SUCCESS;
  std::vector<uint8_t> pixels;
  uint32_t next_row = 0;     // rows handed to steps (worker)
  uint32_t rows_landed = 0;  // rows whose step has landed or failed (worker)
  int in_flight = 0;         // steps in flight with rows of this request (worker)
};

// A step's share of one request: image rows [y0, y0 + rows).
struct Item {
  Pending* p = nullptr;
  uint32_t y0 = 0, rows = 0;
};

// One wavefront slot: a stream, its buffers and the step in flight on it.
struct Slot {
  cudaStream_t stream = nullptr;
  DevBuf rays, shadow, hits, cw, pend, bits, pix, table, counters, err;
  uint8_t* host = nullptr;  // pinned: pixels, then 16 bytes of shadow count and error word
  size_t host_cap = 0;
  bool busy = false;
  uint64_t seq = 0;
  std::atomic<bool> landed{false};
  std::vector<Item> items;
  std::vector<rq_status_t> status;  // per item
  std::vector<Mesh*> mesh;          // per item
  std::vector<uint32_t> poff;
  std::vector<size_t> which;        // items that went ahead
  uint32_t npix = 0;
  uint64_t nray = 0;
  uint64_t device_bytes() const {
    return rays.cap + shadow.cap + hits.cap + cw.cap + pend.cap + bits.cap + pix.cap + table.cap + counters.cap +
           err.cap;
  }
  void release() {
    rays.release(); shadow.release(); hits.release(); cw.release(); pend.release(); bits.release();
    pix.release(); table.release(); counters.release(); err.release();
    if (host) cudaFreeHost(host);
    host = nullptr;
    host_cap = 0;
    if (stream) cudaStreamDestroy(stream);
    stream = nullptr;
  }
};

uint64_t mesh_estimate_bytes(const Mesh& m) {
  const uint64_t nt = m.idx.size() / 3, nv = m.verts.size() / 3;
  // scene (vertices, indices and their 16-byte copies) + LBVH (nodes, payload,
  // order, codes, root)
  return nv * (12 + 16) + nt * (12 + 16) + (nt > 1 ? nt - 1 : 1) * 64 + nt * (48 + 4 + 4) + 512;
}

uint64_t scratch_bytes(const BuildScratch& sc) {
  return sc.keys_alt.cap + sc.vals_alt.cap + sc.zero.cap + sc.parent.cap + sc.mark.cap + sc.lohi.cap +
         sc.keys.cap + sc.vals.cap + sc.m0.cap + sc.m1.cap + sc.m2.cap + sc.m3.cap + sc.m4.cap + sc.m5.cap +
         sc.m6.cap + sc.m7.cap + sc.kd_refs.cap + sc.work.cap;
}

}  // namespace
}  // namespace rq

using namespace rq;

struct rq_server {
  rq_server_config_t cfg{};
  rq_ctx_t ctx = nullptr;        // rendering (slot streams)
  rq_ctx_t build_ctx = nullptr;  // uploads and LBVH builds, on its own stream
  std::mutex m;
  std::condition_variable cv_work, cv_done;
  std::deque<Pending*> queue;
  std::unordered_map<uint64_t, std::unique_ptr<Pending>> reqs;
  std::unordered_map<uint32_t, std::unique_ptr<Mesh>> meshes;
  uint64_t next_ticket = 1;
  bool stop = false;
  std::thread worker;
  // worker-only state
  Slot slots[2];
  int n_slots = 1;
  uint64_t batch_no = 0, launch_no = 0;
  uint64_t resident = 0;
  Clock::time_point busy_since;
  // statistics (under m)
  rq_server_stats_t st{};
  std::vector<double> lat_ms;
  std::string worker_error;

  void run();
  Slot* free_slot();
  Slot* oldest_busy();
  bool launch(Slot& sl, std::vector<Item>& items);
  void retire(Slot& sl);
  uint64_t engine_bytes() const;
  rq_status_t make_resident(Mesh& mesh, const std::vector<Mesh*>& keep, uint64_t wavefront);
  bool evict_one(const std::vector<Mesh*>& keep);
  void land(const Item& it, rq_status_t status, const uint8_t* pixels);
};

namespace {

void CUDART_CB on_landed(void* arg) {
  // Runs on a CUDA callback thread: no CUDA calls here, only the flag.
  auto* pr = static_cast<std::pair<rq_server*, Slot*>*>(arg);
  {
    std::lock_guard<std::mutex> g(pr->first->m);
    pr->second->landed.store(true);
  }
  pr->first->cv_work.notify_one();
  delete pr;
}

}  // namespace

// Device memory the server holds besides resident meshes: the slots'
// wavefront buffers and the two contexts' build and render scratch.
uint64_t rq_server::engine_bytes() const {
  uint64_t b = 0;
  for (int k = 0; k < n_slots; ++k) b += slots[k].device_bytes();
  b += scratch_bytes(ctx->scratch) + scratch_bytes(build_ctx->scratch);
  b += build_ctx->stage_in.cap + build_ctx->stage_out.cap + build_ctx->stage_aux.cap;
  return b;
}

bool rq_server::evict_one(const std::vector<Mesh*>& keep) {
  Mesh* lru = nullptr;
  {
    std::lock_guard<std::mutex> g(m);
    for (auto& kv : meshes) {
      Mesh* c = kv.second.get();
      if (!c->accel || c->in_flight > 0 || std::find(keep.begin(), keep.end(), c) != keep.end()) continue;
      if (!lru || c->last_use < lru->last_use) lru = c;
    }
  }
  if (!lru) return false;
  rq_accel_destroy(lru->accel);
  rq_scene_destroy(lru->scene);
  lru->accel = nullptr;
  lru->scene = nullptr;
  resident -= lru->bytes;
  lru->bytes = 0;
  std::lock_guard<std::mutex> g(m);
  ++st.evictions;
  return true;
}

// Upload + build `mesh` if needed, evicting least recently used meshes (not in
// `keep`, not in flight) until resident meshes, the engine's buffers and
// `wavefront` more bytes fit the budget.
rq_status_t rq_server::make_resident(Mesh& mesh, const std::vector<Mesh*>& keep, uint64_t wavefront) {
  if (mesh.accel) return RQ_SUCCESS;
  const uint64_t need = mesh_estimate_bytes(mesh);
  while (resident + engine_bytes() + wavefront + need > cfg.hbm_budget)
    if (!evict_one(keep)) return RQ_ERROR_OUT_OF_MEMORY;
  rq_status_t s = rq_scene_create_triangles(build_ctx, mesh.verts.data(), (uint32_t)(mesh.verts.size() / 3),
                                            mesh.idx.data(), (uint32_t)(mesh.idx.size() / 3), 0, &mesh.scene);
  if (s != RQ_SUCCESS) return s;
  s = rq_build(build_ctx, mesh.scene, RQ_LBVH, &mesh.accel);  // returns once the build has finished
  if (s != RQ_SUCCESS) {
    rq_scene_destroy(mesh.scene);
    mesh.scene = nullptr;
    return s;
  }
  const rq_scene_t sc = mesh.scene;
  mesh.bytes = sc->verts.cap + sc->idx.cap + sc->verts4.cap + sc->idx4.cap + mesh.accel->buf.device_bytes();
  resident += mesh.bytes;
  std::lock_guard<std::mutex> g(m);
  ++st.builds;
  return RQ_SUCCESS;
}

// Rows of a request have landed (or failed): copy its pixels in; the
// request completes with its last rows.
void rq_server::land(const Item& it, rq_status_t status, const uint8_t* pixels) {
  Pending* p = it.p;
  const rq_request_t& r = p->req;
  if (status != RQ_SUCCESS && p->status == RQ_SUCCESS) p->status = status;
  if (status == RQ_SUCCESS && r.keep_pixels && pixels) {
    if (p->pixels.empty()) p->pixels.resize((size_t)r.width * r.height * 3);
    std::memcpy(p->pixels.data() + (size_t)it.y0 * r.width * 3, pixels, (size_t)it.rows * r.width * 3);
  }
  p->rows_landed += it.rows;
  if (p->rows_landed < r.height) return;
  const Clock::time_point now = Clock::now();
  {
    std::lock_guard<std::mutex> g(m);
    p->done = true;
    if (p->status == RQ_SUCCESS) {
      ++st.completed;
      lat_ms.push_back(std::chrono::duration<double, std::milli>(now - p->t_submit).count());
    } else {
      p->pixels.clear();
      ++st.rejected;
    }
  }
  cv_done.notify_all();
}

Slot* rq_server::free_slot() {
  for (int k = 0; k < n_slots; ++k)
    if (!slots[k].busy) return &slots[k];
  return nullptr;
}

Slot* rq_server::oldest_busy() {
  Slot* o = nullptr;
  for (int k = 0; k < n_slots; ++k)
    if (slots[k].busy && (!o || slots[k].seq < o->seq)) o = &slots[k];
  return o;
}

// Resolve meshes, make them resident, build the step's tables and enqueue the
// whole wavefront on the slot's stream.  Returns true when a step went in
// flight; items that cannot go ahead land at once with their error.
bool rq_server::launch(Slot& sl, std::vector<Item>& items) {
  const size_t n = items.size();
  sl.items = items;
  sl.status.assign(n, RQ_SUCCESS);
  sl.mesh.assign(n, nullptr);
  ++batch_no;
  {
    std::lock_guard<std::mutex> g(m);
    for (size_t k = 0; k < n; ++k) {
      auto it = meshes.find(items[k].p->req.mesh_id);
      if (it == meshes.end()) sl.status[k] = RQ_ERROR_INVALID_ARGUMENT;
      else sl.mesh[k] = it->second.get();
    }
  }
  // Wavefront growth this step would add to the slot's buffers.
  uint64_t rays_all = 0, pix_all = 0;
  for (size_t k = 0; k < n; ++k) {
    const rq_request_t& r = items[k].p->req;
    rays_all += (uint64_t)r.width * items[k].rows * r.spp;
    pix_all += (uint64_t)r.width * items[k].rows;
  }
  const uint64_t want = rays_all * kSampleBytes + pix_all * 3 + 4096;
  const uint64_t have = sl.device_bytes();
  const uint64_t grow = want > have ? want - have : 0;
  for (size_t k = 0; k < n; ++k) {
    if (sl.status[k] != RQ_SUCCESS) continue;
    sl.status[k] = make_resident(*sl.mesh[k], sl.mesh, grow);
    if (sl.status[k] == RQ_SUCCESS) sl.mesh[k]->last_use = batch_no;
  }
  while (resident + engine_bytes() + grow > cfg.hbm_budget && evict_one(sl.mesh)) {
  }
  // Tables of the items that go ahead: each renders its rows as a window of
  // the request's full image.
  std::vector<ServeReq> sreq;
  std::vector<Bvh2View> views;
  std::vector<uint32_t> roff(1, 0);
  sl.poff.assign(1, 0);
  sl.which.clear();
  for (size_t k = 0; k < n; ++k) {
    if (sl.status[k] != RQ_SUCCESS) continue;
    const rq_request_t& r = items[k].p->req;
    const float tan_half = (float)std::tan((double)r.view.fov_deg * 3.141592653589793 / 360.0);
    rq_view_t view = r.view;
    view.bounces = 0;
    view.window[0] = 0;
    view.window[1] = items[k].y0;
    view.window[2] = r.width;
    view.window[3] = items[k].rows;
    ServeReq q;
    q.v = make_view_dev(view, r.width, r.height, r.spp, r.background, ctx->settings.bias, tan_half);
    rq_scene_t sc = sl.mesh[k]->scene;
    q.sc.kind = kTriangles;
    q.sc.n = sc->n;
    q.sc.nv = sc->nv;
    q.sc.verts = sc->verts.as<const float>();
    q.sc.idx = sc->idx.as<const uint32_t>();
    q.sc.sph = nullptr;
    q.sc.verts4 = sc->verts4.as<const float4>();
    q.sc.idx4 = sc->idx4.as<const uint4>();
    sreq.push_back(q);
    const AccelBuffers& b = sl.mesh[k]->accel->buf;
    views.push_back({b.nodes.as<const float4>(), b.prims.as<const float4>(), b.order.as<const uint32_t>(),
                     b.root.as<const float>(), b.n_nodes, b.n_slots});
    roff.push_back(roff.back() + r.width * items[k].rows * r.spp);
    sl.poff.push_back(sl.poff.back() + r.width * items[k].rows);
    sl.which.push_back(k);
  }
  const uint32_t nq = (uint32_t)sl.which.size();
  if (nq == 0) {
    for (size_t k = 0; k < n; ++k) land(items[k], sl.status[k], nullptr);
    return false;
  }
  const uint32_t nray = roff.back(), npix = sl.poff.back();
  cudaStream_t s = sl.stream;
  cudaError_t e = cudaSuccess;
  // device table: [ServeReq n][Bvh2View n][roff n+1][poff n+1][work]
  const size_t a0 = 0, a1 = (sizeof(ServeReq) * nq + 15) & ~size_t(15);
  const size_t a2 = a1 + ((sizeof(Bvh2View) * nq + 15) & ~size_t(15));
  const size_t a3 = a2 + ((4 * ((size_t)nq + 1) + 15) & ~size_t(15));
  const size_t a4 = a3 + ((4 * ((size_t)nq + 1) + 15) & ~size_t(15));
  const size_t host_need = (((size_t)npix * 3 + 15) & ~size_t(15)) + 16 + a4 + 16;
  if (sl.host_cap < host_need) {
    if (sl.host) cudaFreeHost(sl.host);
    sl.host = nullptr;
    sl.host_cap = 0;
    e = cudaMallocHost(&sl.host, host_need);
    if (e == cudaSuccess) sl.host_cap = host_need;
  }
  const size_t pix_bytes = ((size_t)npix * 3 + 15) & ~size_t(15);
  char* host_tab = reinterpret_cast<char*>(sl.host) + pix_bytes + 16;
  if (e == cudaSuccess) {
    std::memset(host_tab, 0, a4 + 16);
    std::memcpy(host_tab + a0, sreq.data(), sizeof(ServeReq) * nq);
    std::memcpy(host_tab + a1, views.data(), sizeof(Bvh2View) * nq);
    std::memcpy(host_tab + a2, roff.data(), 4 * ((size_t)nq + 1));
    std::memcpy(host_tab + a3, sl.poff.data(), 4 * ((size_t)nq + 1));
  }
  if (e == cudaSuccess) e = sl.table.ensure(a4 + 16);
  if (e == cudaSuccess) e = sl.rays.ensure((size_t)nray * 32);
  if (e == cudaSuccess) e = sl.shadow.ensure((size_t)nray * 32);
  if (e == cudaSuccess) e = sl.hits.ensure((size_t)nray * 16);
  if (e == cudaSuccess) e = sl.cw.ensure((size_t)nray * 16);
  if (e == cudaSuccess) e = sl.pend.ensure((size_t)nray * 16);
  if (e == cudaSuccess) e = sl.bits.ensure((((size_t)nray + 31) / 32) * 4);
  if (e == cudaSuccess) e = sl.pix.ensure((size_t)npix * 3);
  if (e == cudaSuccess) e = sl.counters.ensure(16);
  if (e == cudaSuccess) e = sl.err.ensure(16);
  if (e == cudaSuccess) e = cudaMemcpyAsync(sl.table.p, host_tab, a4 + 16, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(sl.counters.p, 0, 16, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(sl.err.p, 0, 16, s);
  char* tb = sl.table.as<char>();
  const ServeReq* d_req = reinterpret_cast<const ServeReq*>(tb + a0);
  const uint32_t* d_roff = reinterpret_cast<const uint32_t*>(tb + a2);
  const uint32_t* d_poff = reinterpret_cast<const uint32_t*>(tb + a3);
  const unsigned gr = (nray + kThreads - 1) / kThreads;
  if (e == cudaSuccess) {
    count_launch();
    k_serve_rays<<<gr, kThreads, 0, s>>>(d_req, d_roff, nq, nray, sl.rays.as<float4>(), sl.cw.as<float4>());
    e = cudaGetLastError();
  }
  BatchedTrace t;
  t.kind = kTriangles;
  t.width = 2;
  t.unit = true;  // the server builds LBVHs: single-primitive leaves
  t.views = reinterpret_cast<const Bvh2View*>(tb + a1);
  t.roff = d_roff;
  t.n_views = nq;
  t.n = nray;
  t.work = reinterpret_cast<uint32_t*>(tb + a4);
  t.err = sl.err.as<uint32_t>();
  if (e == cudaSuccess) {
    t.any = false;
    t.rays = sl.rays.as<const float4>();
    t.hits = sl.hits.as<float4>();
    e = launch_trace_batched(t, 128, 1, s);
  }
  if (e == cudaSuccess) {
    count_launch();
    k_serve_shade<<<gr, kThreads, 0, s>>>(d_req, d_roff, nq, nray, sl.rays.as<float4>(), sl.hits.as<const float4>(),
                                          sl.shadow.as<float4>(), sl.cw.as<float4>(), sl.pend.as<float4>(),
                                          sl.counters.as<unsigned long long>());
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) {
    t.any = true;
    t.rays = sl.shadow.as<const float4>();
    t.hits = nullptr;
    t.occ = sl.bits.as<uint32_t>();
    e = launch_trace_batched(t, 128, 1, s);
  }
  if (e == cudaSuccess) {
    count_launch(2);
    k_serve_accum<<<gr, kThreads, 0, s>>>(nray, sl.bits.as<const uint32_t>(), sl.pend.as<const float4>(),
                                          sl.cw.as<float4>());
    k_serve_pixels<<<(npix + kThreads - 1) / kThreads, kThreads, 0, s>>>(d_req, d_roff, d_poff, nq, npix,
                                                                          sl.cw.as<const float4>(), sl.pix.as<uint8_t>());
    e = cudaGetLastError();
  }
  uint8_t* tail = sl.host + pix_bytes;  // shadow-ray count (8 bytes) and error word (4 bytes)
  if (e == cudaSuccess) e = cudaMemcpyAsync(sl.host, sl.pix.p, (size_t)npix * 3, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(tail, sl.counters.p, 8, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(tail + 8, sl.err.p, 4, cudaMemcpyDeviceToHost, s);
  sl.landed.store(false);
  if (e == cudaSuccess) e = cudaLaunchHostFunc(s, on_landed, new std::pair<rq_server*, Slot*>(this, &sl));
  if (e != cudaSuccess) {
    cudaStreamSynchronize(s);
    {
      std::lock_guard<std::mutex> g(m);
      worker_error = cudaGetErrorString(e);
    }
    cudaGetLastError();
    for (size_t j = 0; j < sl.which.size(); ++j) sl.status[sl.which[j]] = RQ_ERROR_CUDA;
    for (size_t k = 0; k < n; ++k) land(items[k], sl.status[k], nullptr);
    return false;
  }
  for (size_t j = 0; j < sl.which.size(); ++j) {
    ++sl.mesh[sl.which[j]]->in_flight;
    ++sl.items[sl.which[j]].p->in_flight;
  }
  for (size_t k = 0; k < n; ++k)  // items that could not go ahead land now
    if (sl.status[k] != RQ_SUCCESS) land(items[k], sl.status[k], nullptr);
  sl.npix = npix;
  sl.nray = nray;
  sl.busy = true;
  sl.seq = ++launch_no;
  return true;
}

// A landed step: hand out pixels and statuses, release its meshes.
void rq_server::retire(Slot& sl) {
  const size_t pix_bytes = ((size_t)sl.npix * 3 + 15) & ~size_t(15);
  uint64_t shadow_rays = 0;
  uint32_t derr = 0;
  std::memcpy(&shadow_rays, sl.host + pix_bytes, 8);
  std::memcpy(&derr, sl.host + pix_bytes + 8, 4);
  if (derr) {
    std::lock_guard<std::mutex> g(m);
    worker_error = "device error flag set during a batch";
  }
  sl.busy = false;
  {
    std::lock_guard<std::mutex> g(m);
    ++st.batches;
    st.camera_rays += sl.nray;
    st.shadow_rays += shadow_rays;
    st.resident_bytes = resident;
  }
  for (size_t j = 0; j < sl.which.size(); ++j) {
    const size_t k = sl.which[j];
    --sl.mesh[k]->in_flight;
    --sl.items[k].p->in_flight;
    const rq_status_t stt =
        derr ? ((derr & kErrStackOverflow) ? RQ_ERROR_STACK_OVERFLOW : RQ_ERROR_INVALID_ARGUMENT) : RQ_SUCCESS;
    land(sl.items[k], stt, sl.host + 3 * (size_t)sl.poff[j]);
  }
}

void rq_server::run() {
  if (cudaSetDevice(cfg.device) != cudaSuccess) return;
  for (;;) {
    // Retire every step that has landed, oldest first.
    for (;;) {
      Slot* o = oldest_busy();
      if (!o || !o->landed.load()) break;
      retire(*o);
      if (!oldest_busy()) {
        std::lock_guard<std::mutex> g(m);
        st.busy_s += std::chrono::duration<double>(Clock::now() - busy_since).count();
      }
    }
    std::vector<Item> items;
    Slot* sl = free_slot();
    {
      std::unique_lock<std::mutex> lk(m);
      if (stop && !oldest_busy()) return;
      if (sl && !queue.empty() && !stop) {
        if (!cfg.batching) {  // one whole request per step
          Pending* p = queue.front();
          queue.pop_front();
          items.push_back({p, 0, p->req.height});
          p->next_row = p->req.height;
        } else {
          // Rows of the waiting requests, in arrival order, up to the step's
          // ray budget.  While others wait, one request takes at most half
          // of a step and is finished in later steps, so requests that
          // arrive behind a large one start at the next step; steps stay
          // few requests wide (their meshes stay in L2) and large (a step's
          // fixed cost is small beside it).
          // A request with rows in flight waits for them (the other slot
          // stays free for requests that arrive meanwhile); the two slots'
          // wavefronts use at most half of the HBM budget.
          std::vector<Pending*> cand;
          for (Pending* p : queue) {
            if (p->in_flight) continue;
            cand.push_back(p);
            if (cand.size() >= cfg.max_batch_requests) break;
          }
          const uint64_t budget =
              std::max<uint64_t>(1, std::min<uint64_t>(cfg.step_rays, cfg.hbm_budget / (4 * kSampleBytes)));
          const uint64_t cap = cand.size() > 1 ? std::max<uint64_t>(1, budget / 2) : budget;
          std::vector<uint32_t> take(cand.size(), 0);
          uint64_t used = 0;
          for (size_t k = 0; k < cand.size() && used < budget; ++k) {
            const Pending* p = cand[k];
            const uint64_t row_rays = (uint64_t)p->req.width * p->req.spp;
            const uint64_t rows_left = p->req.height - p->next_row;
            uint64_t t = std::min(budget - used, cap) / row_rays;
            if (t == 0 && used == 0) t = 1;  // a row wider than the budget still goes, alone
            t = std::min<uint64_t>(t, rows_left);
            take[k] = (uint32_t)t;
            used += t * row_rays;
          }
          for (size_t k = 0; k < cand.size(); ++k) {
            if (!take[k]) continue;
            items.push_back({cand[k], cand[k]->next_row, take[k]});
            cand[k]->next_row += take[k];
          }
          for (auto it = queue.begin(); it != queue.end();) {  // fully handed out: leave the queue
            if ((*it)->next_row == (*it)->req.height) it = queue.erase(it);
            else ++it;
          }
        }
      }
      if (items.empty()) {
        // wait for an arrival (when a slot is free) or for a step to land
        // (slot states change only on this thread; `landed` is set under m)
        cv_work.wait(lk, [&] {
          Slot* o = oldest_busy();
          if (o && o->landed.load()) return true;
          if (stop) return o == nullptr;
          if (free_slot() == nullptr) return false;
          for (const Pending* p : queue)
            if (!p->in_flight) return true;
          return false;
        });
        continue;
      }
    }
    const bool was_idle = oldest_busy() == nullptr;
    const Clock::time_point t0 = Clock::now();
    if (launch(*sl, items) && was_idle) busy_since = t0;
    if (!cfg.batching) {  // the plain path: each step waited for before the next
      cudaStreamSynchronize(sl->stream);
    }
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
  if (s->cfg.step_rays == 0) s->cfg.step_rays = 1u << 24;
  if (s->cfg.max_batch_rays >= (1u << 31)) return RQ_ERROR_INVALID_ARGUMENT;
  // the server's own context: cube Morton normalisation (tighter LBVHs on
  // flat scenes; results do not depend on the tree)
  rq_settings_t settings;
  rq_settings_default(&settings);
  settings.morton = RQ_MORTON_SCENE_CUBE;
  rq_status_t st = rq_create(&settings, s->cfg.device, &s->ctx);
  if (st != RQ_SUCCESS) return st;
  st = rq_create(&settings, s->cfg.device, &s->build_ctx);
  if (st != RQ_SUCCESS) {
    rq_destroy(s->ctx);
    return st;
  }
  s->n_slots = s->cfg.batching ? 2 : 1;
  for (int k = 0; k < s->n_slots; ++k) {
    if (cudaStreamCreateWithFlags(&s->slots[k].stream, cudaStreamNonBlocking) != cudaSuccess) {
      cudaGetLastError();
      for (int j = 0; j < k; ++j) s->slots[j].release();
      rq_destroy(s->build_ctx);
      rq_destroy(s->ctx);
      return RQ_ERROR_CUDA;
    }
  }
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
  for (int k = 0; k < s->n_slots; ++k) {
    if (s->slots[k].stream) cudaStreamSynchronize(s->slots[k].stream);
    s->slots[k].release();
  }
  rq_destroy(s->build_ctx);
  rq_destroy(s->ctx);
  delete s;
  return RQ_SUCCESS;
}

}  // extern "C"
