// The C ABI (include/rq.h): contexts, scenes, the dataStructure build switch
// and the ray queries, over the kernels of the other translation units.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <new>
#include <random>
#include <string>
#include <vector>

#include "rq_device.cuh"
#include "rq_handles.hpp"

namespace {

rq_status_t fail(rq_ctx_t ctx, rq_status_t st, const std::string& msg) {
  if (ctx) ctx->last_error = msg;
  return st;
}

rq_status_t cuda_fail(rq_ctx_t ctx, cudaError_t e, const char* what) {
  std::string m = std::string(what) + ": " + cudaGetErrorString(e);
  cudaGetLastError();  // clear a sticky launch error where possible
  return fail(ctx, e == cudaErrorMemoryAllocation ? RQ_ERROR_OUT_OF_MEMORY : RQ_ERROR_CUDA, m);
}

#define RQ_TRY_CUDA(ctx, call)                                   \
  do {                                                           \
    cudaError_t e_ = (call);                                     \
    if (e_ != cudaSuccess) return cuda_fail((ctx), e_, #call);   \
  } while (0)

#define RQ_TRY(call)                  \
  do {                                \
    rq_status_t s_ = (call);          \
    if (s_ != RQ_SUCCESS) return s_;  \
  } while (0)

rq_status_t bind(rq_ctx_t ctx) {
  if (!ctx) return RQ_ERROR_INVALID_ARGUMENT;
  RQ_TRY_CUDA(ctx, cudaSetDevice(ctx->device));
  return RQ_SUCCESS;
}

// Read and clear the device error word; map it to a status.
rq_status_t collect_device_errors(rq_ctx_t ctx) {
  uint32_t e = 0;
  RQ_TRY_CUDA(ctx, cudaMemcpyAsync(&e, ctx->d_err, 4, cudaMemcpyDeviceToHost, ctx->stream));
  RQ_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (e) {
    RQ_TRY_CUDA(ctx, cudaMemsetAsync(ctx->d_err, 0, 4, ctx->stream));
    if (e & kErrStackOverflow)
      return fail(ctx, RQ_ERROR_STACK_OVERFLOW, "traversal stack overflow (tree deeper than 64)");
    if (e & kErrTimeout) return fail(ctx, RQ_ERROR_TIMEOUT, "a bounded device-side wait gave up");
    if (e & kErrBadInput) return fail(ctx, RQ_ERROR_INVALID_ARGUMENT, "invalid scene data (NaN/Inf or index out of range)");
    if (e & kErrCorrupt) return fail(ctx, RQ_ERROR_INVALID_ARGUMENT, "malformed acceleration structure (walk bound exceeded)");
  }
  return RQ_SUCCESS;
}

rq_status_t check_launch(rq_ctx_t ctx, const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(ctx, e, what);
  return RQ_SUCCESS;
}

// Copy a caller buffer to the device (or pass a device pointer through).
template <typename T>
rq_status_t to_device(rq_ctx_t ctx, DevBuf& stage, const T* src, size_t bytes, uint32_t flags,
                      const T** out) {
  if (flags & RQ_DEVICE_POINTERS) {
    *out = src;
    return RQ_SUCCESS;
  }
  RQ_TRY_CUDA(ctx, stage.ensure(bytes));
  RQ_TRY_CUDA(ctx, cudaMemcpyAsync(stage.p, src, bytes, cudaMemcpyHostToDevice, ctx->stream));
  *out = stage.as<const T>();
  return RQ_SUCCESS;
}

bool finite3(const float* p, size_t n) {
  for (size_t i = 0; i < n; ++i)
    if (!std::isfinite(p[i])) return false;
  return true;
}

}  // namespace

extern "C" {

void rq_settings_default(rq_settings_t* s) {
  if (!s) return;
  std::memset(s, 0, sizeof(*s));
  s->width = 640;
  s->height = 480;
  s->fov = 90;
  s->backgroundColor[0] = s->backgroundColor[1] = s->backgroundColor[2] = 1.f;
  s->bias = 0.0001f;
  s->aa_samples = 1;
  s->dataStructure = RQ_BVH;
  s->sceneModel = RQ_BUNNY;
  s->traversal = RQ_TRAVERSAL_FAST;
  s->morton = RQ_MORTON_SCENE_BOUNDS;
  s->kd_max_depth = -1;
}

const char* rq_status_string(rq_status_t st) {
  switch (st) {
    case RQ_SUCCESS: return "success";
    case RQ_ERROR_INVALID_ARGUMENT: return "invalid argument";
    case RQ_ERROR_UNSUPPORTED: return "unsupported";
    case RQ_ERROR_OUT_OF_MEMORY: return "out of device memory";
    case RQ_ERROR_CUDA: return "CUDA error";
    case RQ_ERROR_STACK_OVERFLOW: return "traversal stack overflow";
    case RQ_ERROR_TIMEOUT: return "device wait timed out";
    case RQ_ERROR_EMPTY_SCENE: return "empty scene";
    case RQ_ERROR_NO_DEVICE: return "no CUDA device";
  }
  return "unknown status";
}

rq_status_t rq_create(const rq_settings_t* settings, int device, rq_ctx_t* out) {
  if (!out) return RQ_ERROR_INVALID_ARGUMENT;
  *out = nullptr;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
    cudaGetLastError();
    return RQ_ERROR_NO_DEVICE;
  }
  if (device < 0 || device >= count) return RQ_ERROR_INVALID_ARGUMENT;
  rq_context* ctx = new (std::nothrow) rq_context();
  if (!ctx) return RQ_ERROR_OUT_OF_MEMORY;
  ctx->device = device;
  if (settings) ctx->settings = *settings;
  else rq_settings_default(&ctx->settings);
  cudaError_t e = cudaSetDevice(device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking);
  // d_err[0]: the device error word; d_err[1]: a word that nothing writes
  // (the sort test hook of rq_set_debug waits on it).
  if (e == cudaSuccess) e = cudaMalloc(&ctx->d_err, 8);
  if (e == cudaSuccess) e = cudaMemset(ctx->d_err, 0, 8);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, device);
  if (e != cudaSuccess) {
    rq_status_t st = e == cudaErrorMemoryAllocation ? RQ_ERROR_OUT_OF_MEMORY : RQ_ERROR_CUDA;
    if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
    if (ctx->d_err) cudaFree(ctx->d_err);
    delete ctx;
    cudaGetLastError();
    return st;
  }
  ctx->stream = ctx->own_stream;
  *out = ctx;
  return RQ_SUCCESS;
}

rq_status_t rq_destroy(rq_ctx_t ctx) {
  if (!ctx) return RQ_ERROR_INVALID_ARGUMENT;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  ctx->stage_in.release();
  ctx->stage_out.release();
  ctx->stage_aux.release();
  ctx->ref_jitter.release();
  ctx->scratch.release();
  ctx->render.release();
  ctx->pipe.release();
  ctx->batch_table.release();
  if (ctx->d_err) cudaFree(ctx->d_err);
  if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
  delete ctx;
  return RQ_SUCCESS;
}

rq_status_t rq_get_settings(rq_ctx_t ctx, rq_settings_t* out) {
  if (!ctx || !out) return RQ_ERROR_INVALID_ARGUMENT;
  *out = ctx->settings;
  return RQ_SUCCESS;
}

rq_status_t rq_set_settings(rq_ctx_t ctx, const rq_settings_t* s) {
  if (!ctx || !s) return RQ_ERROR_INVALID_ARGUMENT;
  if (s->traversal != RQ_TRAVERSAL_FAST && s->traversal != RQ_TRAVERSAL_REFERENCE)
    return fail(ctx, RQ_ERROR_INVALID_ARGUMENT, "settings.traversal must be FAST or REFERENCE");
  if (s->morton != RQ_MORTON_SCENE_BOUNDS && s->morton != RQ_MORTON_REFERENCE && s->morton != RQ_MORTON_SCENE_CUBE)
    return fail(ctx, RQ_ERROR_INVALID_ARGUMENT, "settings.morton must be SCENE_BOUNDS, REFERENCE or SCENE_CUBE");
  if (s->node_width != RQ_NODE_WIDTH_2 && s->node_width != 2 && s->node_width != RQ_NODE_WIDTH_4 &&
      s->node_width != RQ_NODE_WIDTH_8)
    return fail(ctx, RQ_ERROR_INVALID_ARGUMENT, "settings.node_width must be 2, 4 or 8");
  if (s->ray_sort < RQ_RAY_SORT_NONE || s->ray_sort > RQ_RAY_SORT_OCTANT_MORTON3)
    return fail(ctx, RQ_ERROR_INVALID_ARGUMENT, "settings.ray_sort out of range");
  if (s->scheduling < RQ_SCHEDULING_THREAD_PER_RAY || s->scheduling > RQ_SCHEDULING_SHARED_TOP)
    return fail(ctx, RQ_ERROR_INVALID_ARGUMENT, "settings.scheduling out of range (rq_scheduling_t)");
  ctx->settings = *s;
  return RQ_SUCCESS;
}

rq_status_t rq_set_stream(rq_ctx_t ctx, void* stream) {
  if (!ctx) return RQ_ERROR_INVALID_ARGUMENT;
  ctx->stream = static_cast<cudaStream_t>(stream);
  return RQ_SUCCESS;
}

rq_status_t rq_synchronize(rq_ctx_t ctx) {
  RQ_TRY(bind(ctx));
  return collect_device_errors(ctx);
}

const char* rq_last_error(rq_ctx_t ctx) { return ctx ? ctx->last_error.c_str() : "null context"; }

// ------------------------------------------------------------------ scenes

rq_status_t rq_scene_create_triangles(rq_ctx_t ctx, const float* verts, uint32_t nv,
                                      const uint32_t* idx, uint32_t nt, uint32_t flags,
                                      rq_scene_t* out) {
  if (!out) return RQ_ERROR_INVALID_ARGUMENT;
  *out = nullptr;
  RQ_TRY(bind(ctx));
  if (nt == 0) return fail(ctx, RQ_ERROR_EMPTY_SCENE, "scene has no triangles");
  if (!verts || !idx || nv == 0) return fail(ctx, RQ_ERROR_INVALID_ARGUMENT, "null vertex or index buffer");
  if (nt >= (1u << 30)) return fail(ctx, RQ_ERROR_INVALID_ARGUMENT, "2^30 or more triangles");
  rq_scene* s = new (std::nothrow) rq_scene();
  if (!s) return RQ_ERROR_OUT_OF_MEMORY;
  s->ctx = ctx;
  s->kind = kTriangles;
  s->n = nt;
  s->nv = nv;
  cudaMemcpyKind k = (flags & RQ_DEVICE_POINTERS) ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  cudaError_t e = s->verts.ensure((size_t)nv * 12);
  if (e == cudaSuccess) e = s->idx.ensure((size_t)nt * 12);
  if (e == cudaSuccess) e = cudaMemcpyAsync(s->verts.p, verts, (size_t)nv * 12, k, ctx->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(s->idx.p, idx, (size_t)nt * 12, k, ctx->stream);
  if (e == cudaSuccess) e = s->verts4.ensure((size_t)nv * 16);
  if (e == cudaSuccess) e = s->idx4.ensure((size_t)nt * 16);
  if (e == cudaSuccess) {  // finite vertices, indices < nv: checked on the device
    launch_validate(s->verts.as<float>(), nv, s->idx.as<uint32_t>(), nt, nullptr, 0, ctx->d_err, ctx->stream);
    launch_pack_tris(s->verts.as<float>(), nv, s->idx.as<uint32_t>(), nt, s->verts4.as<float4>(),
                     s->idx4.as<uint4>(), ctx->stream);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  auto drop = [&]() {
    s->verts.release();
    s->idx.release();
    s->verts4.release();
    s->idx4.release();
    delete s;
  };
  if (e != cudaSuccess) {
    drop();
    return cuda_fail(ctx, e, "scene upload");
  }
  rq_status_t st = collect_device_errors(ctx);
  if (st != RQ_SUCCESS) {
    drop();
    return st;
  }
  *out = s;
  return RQ_SUCCESS;
}

rq_status_t rq_scene_create_spheres(rq_ctx_t ctx, const float* sph, uint32_t n, uint32_t flags,
                                    rq_scene_t* out) {
  if (!out) return RQ_ERROR_INVALID_ARGUMENT;
  *out = nullptr;
  RQ_TRY(bind(ctx));
  if (n == 0) return fail(ctx, RQ_ERROR_EMPTY_SCENE, "scene has no spheres");
  if (!sph) return fail(ctx, RQ_ERROR_INVALID_ARGUMENT, "null sphere buffer");
  if (n >= (1u << 30)) return fail(ctx, RQ_ERROR_INVALID_ARGUMENT, "2^30 or more spheres");
  rq_scene* s = new (std::nothrow) rq_scene();
  if (!s) return RQ_ERROR_OUT_OF_MEMORY;
  s->ctx = ctx;
  s->kind = kSpheres;
  s->n = n;
  cudaMemcpyKind k = (flags & RQ_DEVICE_POINTERS) ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  cudaError_t e = s->sph.ensure((size_t)n * 16);
  if (e == cudaSuccess) e = cudaMemcpyAsync(s->sph.p, sph, (size_t)n * 16, k, ctx->stream);
  if (e == cudaSuccess) {  // finite, radius >= 0: checked on the device
    launch_validate(nullptr, 0, nullptr, 0, s->sph.as<float4>(), n, ctx->d_err, ctx->stream);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) {
    s->sph.release();
    delete s;
    return cuda_fail(ctx, e, "scene upload");
  }
  rq_status_t st = collect_device_errors(ctx);
  if (st != RQ_SUCCESS) {
    s->sph.release();
    delete s;
    return st;
  }
  *out = s;
  return RQ_SUCCESS;
}

rq_status_t rq_scene_update(rq_ctx_t ctx, rq_scene_t s, const float* data, const uint32_t* idx,
                            uint32_t flags) {
  if (!s || !data) return fail(ctx, RQ_ERROR_INVALID_ARGUMENT, "null scene or data");
  RQ_TRY(bind(ctx));
  const bool dev = flags & RQ_DEVICE_POINTERS;
  const bool tri = s->kind == kTriangles;
  const size_t bytes = tri ? (size_t)s->nv * 12 : (size_t)s->n * 16;
  const size_t idx_bytes = (idx && tri) ? (size_t)s->n * 12 : 0;
  void* dst = tri ? s->verts.p : s->sph.p;
  if (dev) {
    RQ_TRY_CUDA(ctx, cudaMemcpyAsync(dst, data, bytes, cudaMemcpyDeviceToDevice, ctx->stream));
    if (idx_bytes) RQ_TRY_CUDA(ctx, cudaMemcpyAsync(s->idx.p, idx, idx_bytes, cudaMemcpyDeviceToDevice, ctx->stream));
    launch_validate(tri ? s->verts.as<float>() : nullptr, tri ? s->nv : 0, idx_bytes ? s->idx.as<uint32_t>() : nullptr,
                    idx_bytes ? s->n : 0, tri ? nullptr : s->sph.as<float4>(), tri ? 0 : s->n, ctx->d_err, ctx->stream);
    if (tri)
      launch_pack_tris(s->verts.as<float>(), s->nv, s->idx.as<uint32_t>(), s->n, s->verts4.as<float4>(),
                       idx_bytes ? s->idx4.as<uint4>() : nullptr, ctx->stream);
    RQ_TRY(check_launch(ctx, "validate launch"));
    return RQ_SUCCESS;  // device-side validation result arrives with rq_synchronize
  }
  // Host data: upload to a staging buffer, validate there on the device, and
  // only then replace the scene's geometry, so a rejected update leaves the
  // scene as it was.
  const size_t off = (bytes + 255) & ~size_t(255);
  RQ_TRY_CUDA(ctx, ctx->stage_aux.ensure(off + idx_bytes));
  char* st = ctx->stage_aux.as<char>();
  RQ_TRY_CUDA(ctx, cudaMemcpyAsync(st, data, bytes, cudaMemcpyHostToDevice, ctx->stream));
  if (idx_bytes) RQ_TRY_CUDA(ctx, cudaMemcpyAsync(st + off, idx, idx_bytes, cudaMemcpyHostToDevice, ctx->stream));
  launch_validate(tri ? reinterpret_cast<const float*>(st) : nullptr, tri ? s->nv : 0,
                  idx_bytes ? reinterpret_cast<const uint32_t*>(st + off) : nullptr, idx_bytes ? s->n : 0,
                  tri ? nullptr : reinterpret_cast<const float4*>(st), tri ? 0 : s->n, ctx->d_err, ctx->stream);
  RQ_TRY(check_launch(ctx, "validate launch"));
  RQ_TRY(collect_device_errors(ctx));
  RQ_TRY_CUDA(ctx, cudaMemcpyAsync(dst, st, bytes, cudaMemcpyDeviceToDevice, ctx->stream));
  if (idx_bytes) RQ_TRY_CUDA(ctx, cudaMemcpyAsync(s->idx.p, st + off, idx_bytes, cudaMemcpyDeviceToDevice, ctx->stream));
  if (tri) {
    launch_pack_tris(s->verts.as<float>(), s->nv, s->idx.as<uint32_t>(), s->n, s->verts4.as<float4>(),
                     idx_bytes ? s->idx4.as<uint4>() : nullptr, ctx->stream);
    RQ_TRY(check_launch(ctx, "pack launch"));
  }
  return RQ_SUCCESS;
}

rq_status_t rq_scene_destroy(rq_scene_t s) {
  if (!s) return RQ_ERROR_INVALID_ARGUMENT;
  cudaSetDevice(s->ctx->device);
  cudaStreamSynchronize(s->ctx->stream);
  s->verts.release();
  s->idx.release();
  s->sph.release();
  s->verts4.release();
  s->idx4.release();
  delete s;
  return RQ_SUCCESS;
}

// ------------------------------------------------------------------ builds

static SceneView scene_view(rq_scene_t s) {
  SceneView v;
  v.kind = s->kind;
  v.n = s->n;
  v.nv = s->nv;
  v.verts = s->verts.as<const float>();
  v.idx = s->idx.as<const uint32_t>();
  v.sph = s->sph.as<const float4>();
  v.verts4 = s->verts4.as<const float4>();
  v.idx4 = s->idx4.as<const uint4>();
  return v;
}

static rq_status_t do_build(rq_ctx_t ctx, rq_accel_t a) {
  SceneView sv = scene_view(a->scene);
  BuildResult r = build_accel(a->type, sv, ctx->settings, a->buf, ctx->scratch, ctx->d_err, ctx->stream);
  if (r.cuda != cudaSuccess) return cuda_fail(ctx, r.cuda, r.what ? r.what : "build");
  if (r.status != RQ_SUCCESS) return fail(ctx, r.status, r.what ? r.what : "build failed");
  return RQ_SUCCESS;
}

rq_status_t rq_build(rq_ctx_t ctx, rq_scene_t scene, int32_t acc_type, rq_accel_t* out) {
  if (!out) return RQ_ERROR_INVALID_ARGUMENT;
  *out = nullptr;
  RQ_TRY(bind(ctx));
  if (!scene) return fail(ctx, RQ_ERROR_INVALID_ARGUMENT, "null scene");
  if (acc_type == RQ_UNIFORM_GRID)
    return fail(ctx, RQ_ERROR_UNSUPPORTED, "UNIFORM_GRID is declared by the reference but never implemented");
  if (acc_type != RQ_BVH && acc_type != RQ_KDTREE && acc_type != RQ_LBVH && acc_type != RQ_NONE)
    return fail(ctx, RQ_ERROR_INVALID_ARGUMENT, "unknown dataStructure");
  rq_accel* a = new (std::nothrow) rq_accel();
  if (!a) return RQ_ERROR_OUT_OF_MEMORY;
  a->ctx = ctx;
  a->scene = scene;
  a->type = acc_type;
  rq_status_t st = do_build(ctx, a);
  if (st == RQ_SUCCESS) st = collect_device_errors(ctx);
  if (st != RQ_SUCCESS) {
    a->buf.release();
    delete a;
    return st;
  }
  *out = a;
  return RQ_SUCCESS;
}

rq_status_t rq_accel_rebuild(rq_ctx_t ctx, rq_accel_t a) {
  if (!a) return fail(ctx, RQ_ERROR_INVALID_ARGUMENT, "null accel");
  RQ_TRY(bind(ctx));
  if (a->imported) return fail(ctx, RQ_ERROR_UNSUPPORTED, "an imported structure has no builder to rerun");
  return do_build(ctx, a);
}

rq_status_t rq_accel_import_bvh2(rq_ctx_t ctx, rq_scene_t scene, const float* nodes, uint32_t n_nodes,
                                 const uint32_t* order, uint32_t n_slots, const float* root_bounds,
                                 rq_accel_t* out) {
  if (!out) return RQ_ERROR_INVALID_ARGUMENT;
  *out = nullptr;
  RQ_TRY(bind(ctx));
  if (!scene || !order || !root_bounds || (n_nodes && !nodes))
    return fail(ctx, RQ_ERROR_INVALID_ARGUMENT, "null scene, nodes, order or root bounds");
  if (n_slots == 0 || n_slots > (1u << 30)) return fail(ctx, RQ_ERROR_INVALID_ARGUMENT, "n_slots must be 1..2^30");
  if (n_nodes >= n_slots + (1u << 30)) return fail(ctx, RQ_ERROR_INVALID_ARGUMENT, "too many nodes");
  if (!finite3(root_bounds, 6)) return fail(ctx, RQ_ERROR_INVALID_ARGUMENT, "root bounds not finite");
  for (uint32_t k = 0; k < n_slots; ++k)
    if (order[k] >= scene->n) return fail(ctx, RQ_ERROR_INVALID_ARGUMENT, "order entry is not a primitive id");
  // Every link must stay inside the arrays, so a walk never reads outside
  // them; what is left unchecked (cycles, boxes that do not bound their
  // primitives) is caught or tolerated by the walks' own bounds.  A tree whose
  // leaves all hold one primitive (an exported LBVH, for one) is walked with
  // 4-byte stack entries, as the engine's own LBVH.
  bool unit = n_nodes > 0;
  for (uint32_t i = 0; i < n_nodes; ++i) {
    const float* nd = nodes + 16 * (size_t)i;
    if (!finite3(nd, 12)) return fail(ctx, RQ_ERROR_INVALID_ARGUMENT, "node box not finite");
    int32_t l[4];
    std::memcpy(l, nd + 12, 16);
    for (int c = 0; c < 2; ++c) {
      const int32_t link = l[c], count = l[2 + c];
      if (link >= 0 ? (uint32_t)link >= n_nodes
                    : (count < 1 || (uint64_t)(uint32_t)(~link) + (uint64_t)count > n_slots))
        return fail(ctx, RQ_ERROR_INVALID_ARGUMENT, "node link outside the node or slot arrays");
      if (link < 0 && count != 1) unit = false;
    }
  }
  rq_accel* a = new (std::nothrow) rq_accel();
  if (!a) return RQ_ERROR_OUT_OF_MEMORY;
  a->ctx = ctx;
  a->scene = scene;
  a->type = RQ_BVH;
  a->imported = true;
  AccelBuffers& b = a->buf;
  cudaError_t e = b.nodes.ensure((size_t)n_nodes * 64);
  if (e == cudaSuccess) e = b.order.ensure((size_t)n_slots * 4);
  if (e == cudaSuccess) e = b.root.ensure(32);
  if (e == cudaSuccess) e = b.prims.ensure((size_t)n_slots * (scene->kind == kTriangles ? 48 : 16));
  if (e == cudaSuccess && n_nodes)
    e = cudaMemcpyAsync(b.nodes.p, nodes, (size_t)n_nodes * 64, cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(b.order.p, order, (size_t)n_slots * 4, cudaMemcpyHostToDevice, ctx->stream);
  float root8[8] = {root_bounds[0], root_bounds[1], root_bounds[2], root_bounds[3], root_bounds[4], root_bounds[5], 0.f, 0.f};
  if (e == cudaSuccess) e = cudaMemcpyAsync(b.root.p, root8, 32, cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess) {
    const SceneView sv = scene_view(scene);
    launch_prims_gather(sv.kind, sv.verts, sv.idx, sv.sph, b.order.as<const uint32_t>(), n_slots,
                        b.prims.as<float4>(), ctx->stream);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);  // root8 lives on this stack frame
  if (e != cudaSuccess) {
    b.release();
    delete a;
    return cuda_fail(ctx, e, "import");
  }
  b.n_nodes = n_nodes;
  b.n_slots = n_slots;
  b.node_width = 2;
  b.unit_leaves = unit;
  *out = a;
  return RQ_SUCCESS;
}

rq_status_t rq_set_debug(rq_ctx_t ctx, const rq_debug_t* debug) {
  if (!ctx) return RQ_ERROR_INVALID_ARGUMENT;
  if (debug) ctx->debug = *debug;
  else ctx->debug = rq_debug_t{};
  return RQ_SUCCESS;
}

rq_status_t rq_accel_destroy(rq_accel_t a) {
  if (!a) return RQ_ERROR_INVALID_ARGUMENT;
  cudaSetDevice(a->ctx->device);
  cudaStreamSynchronize(a->ctx->stream);
  a->buf.release();
  a->batch.reset();  // the batch's arrays go with its last structure
  delete a;
  return RQ_SUCCESS;
}

rq_status_t rq_build_batched(rq_ctx_t ctx, const rq_scene_t* scenes, uint32_t n, int32_t acc_type, rq_accel_t* out) {
  if (!out || !scenes || n == 0) return fail(ctx, RQ_ERROR_INVALID_ARGUMENT, "null or empty scene list");
  RQ_TRY(bind(ctx));
  for (uint32_t k = 0; k < n; ++k) out[k] = nullptr;
  for (uint32_t k = 0; k < n; ++k)
    if (!scenes[k]) return fail(ctx, RQ_ERROR_INVALID_ARGUMENT, "null scene in the list");
  auto undo = [&](uint32_t upto) {
    for (uint32_t k = 0; k < upto; ++k)
      if (out[k]) rq_accel_destroy(out[k]);
    for (uint32_t k = 0; k < n; ++k) out[k] = nullptr;
  };
  if (acc_type != RQ_LBVH) {  // the other builders run scene by scene
    for (uint32_t k = 0; k < n; ++k) {
      rq_status_t st = rq_build(ctx, scenes[k], acc_type, &out[k]);
      if (st != RQ_SUCCESS) {
        std::string msg = ctx->last_error;
        undo(k);
        return fail(ctx, st, msg);
      }
    }
    return RQ_SUCCESS;
  }
  auto store = std::make_shared<BatchStore>();
  store->kind = scenes[0]->kind;
  store->n_scenes = n;
  store->poff.assign(1, 0);
  store->voff.assign(1, 0);
  for (uint32_t k = 0; k < n; ++k) {
    rq_scene_t sc = scenes[k];
    if (sc->kind != store->kind) return fail(ctx, RQ_ERROR_INVALID_ARGUMENT, "a batch mixes triangles and spheres");
    const uint64_t p = (uint64_t)store->poff.back() + sc->n;
    const uint64_t v = (uint64_t)store->voff.back() + (sc->kind == kTriangles ? sc->nv : sc->n);
    if (p >= (1ull << 30) || v >= (1ull << 31))
      return fail(ctx, RQ_ERROR_INVALID_ARGUMENT, "batch of 2^30 or more primitives");
    store->poff.push_back((uint32_t)p);
    store->voff.push_back((uint32_t)v);
    store->host_desc.push_back({sc->verts.as<const float>(), sc->idx.as<const uint32_t>(), sc->sph.as<const float4>()});
  }
  RQ_TRY_CUDA(ctx, store->allocate());
  RQ_TRY_CUDA(ctx, store->upload_tables(ctx->stream));
  BuildResult br = build_batch(*store, ctx->settings.morton, ctx->d_err, ctx->stream);
  if (br.cuda != cudaSuccess) return cuda_fail(ctx, br.cuda, br.what);
  if (br.status != RQ_SUCCESS) return fail(ctx, br.status, br.what);
  for (uint32_t k = 0; k < n; ++k) {
    rq_accel* a = new (std::nothrow) rq_accel();
    if (!a) {
      undo(k);
      return fail(ctx, RQ_ERROR_OUT_OF_MEMORY, "accel handle");
    }
    a->ctx = ctx;
    a->scene = scenes[k];
    a->type = RQ_LBVH;
    store->view(k, a->buf);
    a->batch = store;
    a->batch_index = k;
    out[k] = a;
    if (ctx->settings.node_width == RQ_NODE_WIDTH_4 || ctx->settings.node_width == RQ_NODE_WIDTH_8) {
      BuildResult r = ctx->settings.node_width == RQ_NODE_WIDTH_4
                          ? collapse_bvh4(a->buf, ctx->scratch, ctx->d_err, ctx->stream)
                          : collapse_bvh8(a->buf, ctx->scratch, ctx->d_err, ctx->stream);
      if (!r.ok()) {
        undo(k + 1);
        return r.cuda != cudaSuccess ? cuda_fail(ctx, r.cuda, r.what) : fail(ctx, r.status, r.what);
      }
    }
  }
  rq_status_t st = collect_device_errors(ctx);
  if (st != RQ_SUCCESS) undo(n);
  return st;
}

rq_status_t rq_accel_rebuild_batched(rq_ctx_t ctx, const rq_accel_t* accels, uint32_t n) {
  if (!accels || n == 0 || !accels[0]) return fail(ctx, RQ_ERROR_INVALID_ARGUMENT, "null or empty structure list");
  RQ_TRY(bind(ctx));
  std::shared_ptr<BatchStore> store = accels[0]->batch;
  if (!store) {  // not one batch: rebuild one by one
    for (uint32_t k = 0; k < n; ++k) RQ_TRY(rq_accel_rebuild(ctx, accels[k]));
    return RQ_SUCCESS;
  }
  if (n != store->n_scenes) return fail(ctx, RQ_ERROR_INVALID_ARGUMENT, "not the whole batch");
  for (uint32_t k = 0; k < n; ++k)
    if (!accels[k] || accels[k]->batch != store || accels[k]->batch_index != k)
      return fail(ctx, RQ_ERROR_INVALID_ARGUMENT, "structures not in the order rq_build_batched returned them");
  BuildResult br = build_batch(*store, ctx->settings.morton, ctx->d_err, ctx->stream);
  if (br.cuda != cudaSuccess) return cuda_fail(ctx, br.cuda, br.what);
  if (br.status != RQ_SUCCESS) return fail(ctx, br.status, br.what);
  for (uint32_t k = 0; k < n; ++k) {
    AccelBuffers& b = accels[k]->buf;
    b.node_width = 2;
    if (ctx->settings.node_width == RQ_NODE_WIDTH_4 || ctx->settings.node_width == RQ_NODE_WIDTH_8) {
      BuildResult r = ctx->settings.node_width == RQ_NODE_WIDTH_4 ? collapse_bvh4(b, ctx->scratch, ctx->d_err, ctx->stream)
                                                                  : collapse_bvh8(b, ctx->scratch, ctx->d_err, ctx->stream);
      if (!r.ok()) return r.cuda != cudaSuccess ? cuda_fail(ctx, r.cuda, r.what) : fail(ctx, r.status, r.what);
    }
  }
  return RQ_SUCCESS;
}

rq_status_t rq_accel_get_info(rq_accel_t a, rq_accel_info_t* info) {
  if (!a || !info) return RQ_ERROR_INVALID_ARGUMENT;
  rq_ctx_t ctx = a->ctx;
  RQ_TRY(bind(ctx));
  std::memset(info, 0, sizeof(*info));
  info->type = a->type;
  info->prim_kind = a->scene->kind;
  info->n_prims = a->scene->n;
  info->n_nodes = a->buf.n_nodes;
  info->n_slots = a->buf.n_slots;
  info->max_depth = a->buf.max_depth;
  info->device_bytes = a->buf.device_bytes();
  const bool bvh2 = a->type == RQ_BVH || a->type == RQ_LBVH;
  info->node_width = bvh2 ? a->buf.node_width : 0;
  if (a->buf.root.p) {
    float words[8];
    RQ_TRY_CUDA(ctx, cudaMemcpyAsync(words, a->buf.root.p, 32, cudaMemcpyDeviceToHost, ctx->stream));
    RQ_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    std::memcpy(info->root_bounds, words, 24);
    if (bvh2 && (a->buf.node_width == 4 || a->buf.node_width == 8)) std::memcpy(&info->n_wide_nodes, words + 6, 4);
  }
  return RQ_SUCCESS;
}

rq_status_t rq_accel_export_bvh2(rq_ctx_t ctx, rq_accel_t a, float* nodes, uint32_t* order,
                                 uint32_t* sorted_codes) {
  if (!a) return fail(ctx, RQ_ERROR_INVALID_ARGUMENT, "null accel");
  RQ_TRY(bind(ctx));
  if (a->type != RQ_BVH && a->type != RQ_LBVH)
    return fail(ctx, RQ_ERROR_INVALID_ARGUMENT, "not a BVH2 structure");
  if (nodes && a->buf.n_nodes)
    RQ_TRY_CUDA(ctx, cudaMemcpyAsync(nodes, a->buf.nodes.p, (size_t)a->buf.n_nodes * 64, cudaMemcpyDeviceToHost, ctx->stream));
  if (order)
    RQ_TRY_CUDA(ctx, cudaMemcpyAsync(order, a->buf.order.p, (size_t)a->buf.n_slots * 4, cudaMemcpyDeviceToHost, ctx->stream));
  if (sorted_codes && a->type == RQ_LBVH)
    RQ_TRY_CUDA(ctx, cudaMemcpyAsync(sorted_codes, a->buf.codes.p, (size_t)a->scene->n * 4, cudaMemcpyDeviceToHost, ctx->stream));
  RQ_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return RQ_SUCCESS;
}

rq_status_t rq_accel_export_bvh4(rq_ctx_t ctx, rq_accel_t a, float* nodes, uint32_t* n_nodes) {
  if (!a || !n_nodes) return fail(ctx, RQ_ERROR_INVALID_ARGUMENT, "null accel or count");
  RQ_TRY(bind(ctx));
  if ((a->type != RQ_BVH && a->type != RQ_LBVH) || (a->buf.node_width != 4 && a->buf.node_width != 8))
    return fail(ctx, RQ_ERROR_INVALID_ARGUMENT, "not built with node_width 4 or 8");
  uint32_t n4 = 0;
  RQ_TRY_CUDA(ctx, cudaMemcpyAsync(&n4, a->buf.root.as<uint32_t>() + 6, 4, cudaMemcpyDeviceToHost, ctx->stream));
  RQ_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (n4 > a->buf.n4_cap) return fail(ctx, RQ_ERROR_INVALID_ARGUMENT, "malformed wide node count");
  *n_nodes = n4;
  if (nodes && n4) {
    RQ_TRY_CUDA(ctx, cudaMemcpyAsync(nodes, a->buf.nodes4.p, (size_t)n4 * 128, cudaMemcpyDeviceToHost, ctx->stream));
    RQ_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  }
  return RQ_SUCCESS;
}

rq_status_t rq_accel_export_kd(rq_ctx_t ctx, rq_accel_t a, int32_t* nodes, int32_t* prim_idx) {
  if (!a) return fail(ctx, RQ_ERROR_INVALID_ARGUMENT, "null accel");
  RQ_TRY(bind(ctx));
  if (a->type != RQ_KDTREE) return fail(ctx, RQ_ERROR_INVALID_ARGUMENT, "not a KD tree");
  if (nodes && a->buf.n_nodes) {
    std::vector<int4> tmp(a->buf.n_nodes);
    RQ_TRY_CUDA(ctx, cudaMemcpyAsync(tmp.data(), a->buf.kd_nodes.p, tmp.size() * 16, cudaMemcpyDeviceToHost, ctx->stream));
    RQ_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    for (size_t i = 0; i < tmp.size(); ++i) {
      nodes[3 * i] = tmp[i].x;
      nodes[3 * i + 1] = tmp[i].y;
      nodes[3 * i + 2] = tmp[i].z;
    }
  }
  if (prim_idx && a->buf.n_slots)
    RQ_TRY_CUDA(ctx, cudaMemcpyAsync(prim_idx, a->buf.kd_idx.p, (size_t)a->buf.n_slots * 4, cudaMemcpyDeviceToHost, ctx->stream));
  RQ_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return RQ_SUCCESS;
}

// ----------------------------------------------------------------- queries

// Streamed query over host buffers: per chunk, upload on pipe.up, trace on
// the context's stream, download on pipe.down, with kPipeSlots device slots
// in rotation (a slot is re-filled only after its previous download).
static rq_status_t trace_streamed_enqueue(rq_ctx_t ctx, rq_accel_t a, const rq_ray_t* rays, uint32_t n,
                                          void* out, bool any, const rq_settings_t& cfg, bool join_downloads = true) {
  HostPipe& p = ctx->pipe;
  RQ_TRY_CUDA(ctx, p.init());
  const size_t out_chunk = any ? kPipeChunk / 8 : (size_t)kPipeChunk * 16;
  for (int k = 0; k < kPipeSlots; ++k) {
    RQ_TRY_CUDA(ctx, p.rays[k].ensure((size_t)kPipeChunk * 32));
    RQ_TRY_CUDA(ctx, p.out[k].ensure(out_chunk));
  }
  // Traversals start after everything already queued on the context's
  // stream (a rebuild, say); uploads start at once, overlapping that work,
  // after only the previous call's use of each slot (events never recorded
  // are complete).
  RQ_TRY_CUDA(ctx, cudaEventRecord(p.start, ctx->stream));
  RQ_TRY_CUDA(ctx, cudaStreamWaitEvent(p.down, p.start, 0));
  RQ_TRY_CUDA(ctx, cudaStreamWaitEvent(p.lane2, p.start, 0));
  for (int k = 0; k < kPipeSlots; ++k) RQ_TRY_CUDA(ctx, cudaStreamWaitEvent(p.up, p.downloaded[k], 0));
  const SceneView sv = scene_view(a->scene);
  // Chunk plan: a quarter and a half chunk first (a short first upload), full
  // chunks, then halving chunks at the end (a short last traversal and
  // download).  Every chunk but the last is a multiple of 32 rays, so
  // occlusion words never straddle chunks.
  std::vector<uint32_t> plan;
  for (uint64_t left = n; left > 0;) {
    uint64_t size = plan.empty() ? kPipeChunk / 4 : plan.size() == 1 ? kPipeChunk / 2 : kPipeChunk;
    if (left <= 2ull * kPipeChunk) {
      uint64_t half = (left / 2) & ~uint64_t(31);
      size = std::min<uint64_t>(size, std::max<uint64_t>(kPipeChunk / 4, half));
    }
    size = std::min<uint64_t>(size, left);
    plan.push_back((uint32_t)size);
    left -= size;
  }
  uint64_t first = 0;
  for (uint32_t c = 0; c < (uint32_t)plan.size(); first += plan[c], ++c) {
    const int sl = (int)(c % kPipeSlots);
    const uint32_t m = plan[c];
    if (c >= (uint32_t)kPipeSlots) RQ_TRY_CUDA(ctx, cudaStreamWaitEvent(p.up, p.downloaded[sl], 0));
    RQ_TRY_CUDA(ctx, cudaMemcpyAsync(p.rays[sl].p, rays + first, (size_t)m * 32, cudaMemcpyHostToDevice, p.up));
    RQ_TRY_CUDA(ctx, cudaEventRecord(p.uploaded[sl], p.up));
    cudaStream_t lane = (c & 1) ? p.lane2 : ctx->stream;
    BuildScratch& lane_scratch = (c & 1) ? p.scratch2 : ctx->scratch;
    RQ_TRY_CUDA(ctx, cudaStreamWaitEvent(lane, p.uploaded[sl], 0));
    QueryTarget q;
    q.rays = p.rays[sl].as<const float4>();
    q.n = m;
    q.hits = any ? nullptr : p.out[sl].as<float4>();
    q.occ = any ? p.out[sl].as<uint32_t>() : nullptr;
    BuildResult br = launch_query_sorted(a->type, sv, a->buf, cfg, any, q, lane_scratch, ctx->d_err, lane);
    if (br.cuda != cudaSuccess) return cuda_fail(ctx, br.cuda, br.what);
    if (br.status != RQ_SUCCESS) return fail(ctx, br.status, br.what);
    RQ_TRY_CUDA(ctx, cudaEventRecord(p.traced[sl], lane));
    RQ_TRY_CUDA(ctx, cudaStreamWaitEvent(p.down, p.traced[sl], 0));
    if (any) {
      // chunks are multiples of 32 rays, so bit words never straddle chunks
      RQ_TRY_CUDA(ctx, cudaMemcpyAsync(static_cast<uint32_t*>(out) + first / 32, p.out[sl].p,
                                       (size_t)((m + 31) / 32) * 4, cudaMemcpyDeviceToHost, p.down));
    } else {
      RQ_TRY_CUDA(ctx, cudaMemcpyAsync(static_cast<rq_hit_t*>(out) + first, p.out[sl].p, (size_t)m * 16,
                                       cudaMemcpyDeviceToHost, p.down));
    }
    RQ_TRY_CUDA(ctx, cudaEventRecord(p.downloaded[sl], p.down));
  }
  if (join_downloads) {
    // the context's stream is ordered after the last download
    RQ_TRY_CUDA(ctx, cudaEventRecord(p.start, p.down));
    RQ_TRY_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, p.start, 0));
  } else {
    // only after the other lane's traversals (later work reuses the lanes)
    RQ_TRY_CUDA(ctx, cudaEventRecord(p.start, p.lane2));
    RQ_TRY_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, p.start, 0));
  }
  return RQ_SUCCESS;
}

static rq_status_t trace_streamed(rq_ctx_t ctx, rq_accel_t a, const rq_ray_t* rays, uint32_t n, void* out,
                                  bool any) {
  rq_status_t st = trace_streamed_enqueue(ctx, a, rays, n, out, any, ctx->settings);
  if (st != RQ_SUCCESS) {
    // nothing may still read or write the caller's buffers after an error
    if (ctx->pipe.up) cudaStreamSynchronize(ctx->pipe.up);
    if (ctx->pipe.lane2) cudaStreamSynchronize(ctx->pipe.lane2);
    if (ctx->pipe.down) cudaStreamSynchronize(ctx->pipe.down);
    cudaStreamSynchronize(ctx->stream);
    return st;
  }
  return collect_device_errors(ctx);
}

static rq_status_t trace(rq_ctx_t ctx, rq_accel_t a, const rq_ray_t* rays, uint32_t n, void* out,
                         uint32_t flags, bool any) {
  RQ_TRY(bind(ctx));
  if (!a) return fail(ctx, RQ_ERROR_INVALID_ARGUMENT, "null accel");
  if (n == 0) return RQ_SUCCESS;
  if (!rays || !out) return fail(ctx, RQ_ERROR_INVALID_ARGUMENT, "null ray or result buffer");
  const bool dev = flags & RQ_DEVICE_POINTERS;
  if (!dev && n >= 2 * kPipeChunk) return trace_streamed(ctx, a, rays, n, out, any);
  const float4* d_rays = nullptr;
  RQ_TRY(to_device(ctx, ctx->stage_in, reinterpret_cast<const float4*>(rays), (size_t)n * 32, flags, &d_rays));
  const size_t out_bytes = any ? (size_t)((n + 31) / 32) * 4 : (size_t)n * 16;
  void* d_out = out;
  if (!dev) {
    RQ_TRY_CUDA(ctx, ctx->stage_out.ensure(out_bytes));
    d_out = ctx->stage_out.p;
  }
  QueryTarget q;
  q.rays = d_rays;
  q.n = n;
  q.hits = any ? nullptr : static_cast<float4*>(d_out);
  q.occ = any ? static_cast<uint32_t*>(d_out) : nullptr;
  q.small_stack = ctx->debug.small_stack != 0;
  BuildResult br = launch_query_sorted(a->type, scene_view(a->scene), a->buf, ctx->settings, any, q, ctx->scratch,
                                       ctx->d_err, ctx->stream);
  if (br.cuda != cudaSuccess) return cuda_fail(ctx, br.cuda, br.what);
  if (br.status != RQ_SUCCESS) return fail(ctx, br.status, br.what);
  if (!dev) {
    RQ_TRY_CUDA(ctx, cudaMemcpyAsync(out, d_out, out_bytes, cudaMemcpyDeviceToHost, ctx->stream));
    return collect_device_errors(ctx);
  }
  return RQ_SUCCESS;
}

rq_status_t rq_trace_closest(rq_ctx_t ctx, rq_accel_t a, const rq_ray_t* rays, uint32_t n,
                             rq_hit_t* hits, uint32_t flags) {
  return trace(ctx, a, rays, n, hits, flags, false);
}

rq_status_t rq_trace_any(rq_ctx_t ctx, rq_accel_t a, const rq_ray_t* rays, uint32_t n,
                         uint32_t* occluded_bits, uint32_t flags) {
  return trace(ctx, a, rays, n, occluded_bits, flags, true);
}

rq_status_t rq_trace_candidates(rq_ctx_t ctx, rq_accel_t a, const rq_ray_t* rays, uint32_t n, uint32_t* counts,
                                uint32_t* ids, uint64_t ids_cap, uint64_t* total, uint32_t flags) {
  RQ_TRY(bind(ctx));
  if (!a || !counts || !total) return fail(ctx, RQ_ERROR_INVALID_ARGUMENT, "null accel, counts or total");
  if (a->type != RQ_BVH && a->type != RQ_LBVH)
    return fail(ctx, RQ_ERROR_UNSUPPORTED, "candidate lists exist for BVH structures (RQ_BVH, RQ_LBVH)");
  *total = 0;
  if (n == 0) return RQ_SUCCESS;
  if (!rays) return fail(ctx, RQ_ERROR_INVALID_ARGUMENT, "null rays");
  const bool dev = flags & RQ_DEVICE_POINTERS;
  const float4* d_rays = nullptr;
  RQ_TRY(to_device(ctx, ctx->stage_in, reinterpret_cast<const float4*>(rays), (size_t)n * 32, flags, &d_rays));
  BuildScratch& sc = ctx->scratch;
  uint32_t* d_counts = counts;
  if (!dev) {
    RQ_TRY_CUDA(ctx, sc.m4.ensure((size_t)n * 4));
    d_counts = sc.m4.as<uint32_t>();
  }
  RQ_TRY_CUDA(ctx, sc.m5.ensure((size_t)n * 4));
  RQ_TRY_CUDA(ctx, sc.m6.ensure(scan_tmp_words(n) * 4 + 16));
  const AccelBuffers& b = a->buf;
  const Bvh2View v{b.nodes.as<const float4>(), b.prims.as<const float4>(), b.order.as<const uint32_t>(),
                   b.root.as<const float>(), b.n_nodes, b.n_slots};
  // m6 words: [0] 32-bit scan total, [2..3] 64-bit count total, [4..] scan temporaries
  uint32_t* d_total = sc.m6.as<uint32_t>();
  unsigned long long* d_total64 = reinterpret_cast<unsigned long long*>(d_total + 2);
  RQ_TRY_CUDA(ctx, cudaMemsetAsync(d_total64, 0, 8, ctx->stream));
  launch_candidates(v, d_rays, n, d_counts, nullptr, nullptr, d_total64, ctx->d_err, ctx->stream);
  RQ_TRY(check_launch(ctx, "candidate count launch"));
  uint32_t* offs = sc.m5.as<uint32_t>();
  launch_scan_excl(d_counts, offs, n, d_total + 4, d_total, ctx->stream);
  unsigned long long t = 0;
  RQ_TRY_CUDA(ctx, cudaMemcpyAsync(&t, d_total64, 8, cudaMemcpyDeviceToHost, ctx->stream));
  if (!dev) RQ_TRY_CUDA(ctx, cudaMemcpyAsync(counts, d_counts, (size_t)n * 4, cudaMemcpyDeviceToHost, ctx->stream));
  RQ_TRY(collect_device_errors(ctx));
  *total = t;
  if (!ids) return RQ_SUCCESS;
  if (t > 0xFFFFFFFFull)
    return fail(ctx, RQ_ERROR_INVALID_ARGUMENT, "more than 2^32-1 candidates in one call: split the rays");
  if (ids_cap < t) return fail(ctx, RQ_ERROR_INVALID_ARGUMENT, "ids buffer smaller than the total count");
  uint32_t* d_ids = ids;
  if (!dev) {
    RQ_TRY_CUDA(ctx, ctx->stage_out.ensure((size_t)t * 4 + 4));
    d_ids = ctx->stage_out.as<uint32_t>();
  }
  launch_candidates(v, d_rays, n, d_counts, offs, d_ids, nullptr, ctx->d_err, ctx->stream);
  RQ_TRY(check_launch(ctx, "candidate fill launch"));
  if (!dev && t) RQ_TRY_CUDA(ctx, cudaMemcpyAsync(ids, d_ids, (size_t)t * 4, cudaMemcpyDeviceToHost, ctx->stream));
  return collect_device_errors(ctx);
}

// Several host-buffer queries in one call: the first streams chunk by chunk,
// the others upload whole (on the upload stream, behind the first's chunks)
// while earlier queries trace, trace as full batches on the context's stream
// and download while later ones trace.
static rq_status_t trace_queries_enqueue(rq_ctx_t ctx, rq_accel_t a, const rq_query_t* qs, uint32_t nq) {
  HostPipe& p = ctx->pipe;
  RQ_TRY_CUDA(ctx, p.init());
  const SceneView sv = scene_view(a->scene);
  auto cfg_of = [&](const rq_query_t& q) {
    rq_settings_t c = ctx->settings;
    if (q.ray_sort >= 0) c.ray_sort = q.ray_sort;
    if (q.scheduling >= 0) c.scheduling = q.scheduling;
    return c;
  };
  // The first query streams in chunks unless it has a ray order: an order
  // pays off over the whole batch (sorted chunks of 2M rays trace about as
  // slowly as unsorted ones), so such a query uploads whole like the others.
  uint32_t first = 0;
  if (qs[0].n >= 2 * kPipeChunk && cfg_of(qs[0]).ray_sort == RQ_RAY_SORT_NONE) {
    RQ_TRY(trace_streamed_enqueue(ctx, a, qs[0].rays, qs[0].n, qs[0].out, qs[0].any != 0, cfg_of(qs[0]), false));
    first = 1;
  } else {
    RQ_TRY_CUDA(ctx, cudaEventRecord(p.start, ctx->stream));
    RQ_TRY_CUDA(ctx, cudaStreamWaitEvent(p.down, p.start, 0));
  }
  if (p.q_rays.size() < nq) {
    p.q_rays.resize(nq);
    p.q_out.resize(nq);
  }
  while (p.q_events.size() < 2 * (size_t)nq) {
    cudaEvent_t e;
    RQ_TRY_CUDA(ctx, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    p.q_events.push_back(e);
  }
  for (uint32_t k = first; k < nq; ++k) {
    const rq_query_t& q = qs[k];
    if (q.n == 0) continue;
    const size_t out_bytes = q.any ? (size_t)((q.n + 31) / 32) * 4 : (size_t)q.n * 16;
    RQ_TRY_CUDA(ctx, p.q_rays[k].ensure((size_t)q.n * 32));
    RQ_TRY_CUDA(ctx, p.q_out[k].ensure(out_bytes));
  }
  for (uint32_t k = first; k < nq; ++k) {
    const rq_query_t& q = qs[k];
    if (q.n == 0) continue;
    cudaEvent_t up = p.q_events[2 * k], done = p.q_events[2 * k + 1];
    // the upload overwrites this query's buffer once the previous call's
    // traversal of it is done (uploads overlap work queued before the call)
    RQ_TRY_CUDA(ctx, cudaStreamWaitEvent(p.up, done, 0));
    RQ_TRY_CUDA(ctx, cudaMemcpyAsync(p.q_rays[k].p, q.rays, (size_t)q.n * 32, cudaMemcpyHostToDevice, p.up));
    RQ_TRY_CUDA(ctx, cudaEventRecord(up, p.up));
    RQ_TRY_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, up, 0));
    QueryTarget t;
    t.rays = p.q_rays[k].as<const float4>();
    t.n = q.n;
    t.hits = q.any ? nullptr : p.q_out[k].as<float4>();
    t.occ = q.any ? p.q_out[k].as<uint32_t>() : nullptr;
    BuildResult br = launch_query_sorted(a->type, sv, a->buf, cfg_of(q), q.any != 0, t, ctx->scratch, ctx->d_err,
                                         ctx->stream);
    if (br.cuda != cudaSuccess) return cuda_fail(ctx, br.cuda, br.what);
    if (br.status != RQ_SUCCESS) return fail(ctx, br.status, br.what);
    RQ_TRY_CUDA(ctx, cudaEventRecord(done, ctx->stream));
    RQ_TRY_CUDA(ctx, cudaStreamWaitEvent(p.down, done, 0));
    const size_t out_bytes = q.any ? (size_t)((q.n + 31) / 32) * 4 : (size_t)q.n * 16;
    RQ_TRY_CUDA(ctx, cudaMemcpyAsync(q.out, p.q_out[k].p, out_bytes, cudaMemcpyDeviceToHost, p.down));
  }
  RQ_TRY_CUDA(ctx, cudaEventRecord(p.start, p.down));
  RQ_TRY_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, p.start, 0));
  return RQ_SUCCESS;
}

rq_status_t rq_trace_queries(rq_ctx_t ctx, rq_accel_t a, const rq_query_t* queries, uint32_t n_queries) {
  RQ_TRY(bind(ctx));
  if (!a || (n_queries && !queries)) return fail(ctx, RQ_ERROR_INVALID_ARGUMENT, "null accel or query list");
  if (n_queries == 0) return RQ_SUCCESS;
  for (uint32_t k = 0; k < n_queries; ++k) {
    const rq_query_t& q = queries[k];
    if (q.n && (!q.rays || !q.out)) return fail(ctx, RQ_ERROR_INVALID_ARGUMENT, "null ray or result buffer");
    if (q.ray_sort > RQ_RAY_SORT_OCTANT_MORTON3 || q.scheduling > RQ_SCHEDULING_SHARED_TOP)
      return fail(ctx, RQ_ERROR_INVALID_ARGUMENT, "query ray_sort or scheduling out of range");
  }
  rq_status_t st = trace_queries_enqueue(ctx, a, queries, n_queries);
  if (st != RQ_SUCCESS) {
    if (ctx->pipe.up) cudaStreamSynchronize(ctx->pipe.up);
    if (ctx->pipe.lane2) cudaStreamSynchronize(ctx->pipe.lane2);
    if (ctx->pipe.down) cudaStreamSynchronize(ctx->pipe.down);
    cudaStreamSynchronize(ctx->stream);
    return st;
  }
  return collect_device_errors(ctx);
}

// Device tables of a many-structure query: one Bvh2View per structure (the
// 4-wide nodes when they were built with node width 4), the ray offsets and
// the work counter, in `table`; fills t except rays / outputs.
static rq_status_t batch_tables(rq_ctx_t ctx, const rq_accel_t* accels, uint32_t n, const uint32_t* ray_offsets,
                                bool any, DevBuf& table, BatchedTrace& t) {
  if (!accels || n == 0 || !ray_offsets) return fail(ctx, RQ_ERROR_INVALID_ARGUMENT, "null or empty structure list");
  if (ray_offsets[0] != 0) return fail(ctx, RQ_ERROR_INVALID_ARGUMENT, "ray_offsets[0] must be 0");
  std::vector<Bvh2View> views(n);
  for (uint32_t k = 0; k < n; ++k) {
    rq_accel_t a = accels[k];
    if (!a || a->ctx != ctx) return fail(ctx, RQ_ERROR_INVALID_ARGUMENT, "null structure or another context's");
    if (a->type != RQ_BVH && a->type != RQ_LBVH)
      return fail(ctx, RQ_ERROR_UNSUPPORTED, "many-structure queries walk BVH structures (RQ_BVH, RQ_LBVH)");
    if (a->scene->kind != accels[0]->scene->kind || a->buf.node_width != accels[0]->buf.node_width)
      return fail(ctx, RQ_ERROR_INVALID_ARGUMENT, "structures mix primitive kinds or node widths");
    if (ray_offsets[k + 1] < ray_offsets[k]) return fail(ctx, RQ_ERROR_INVALID_ARGUMENT, "ray_offsets decrease");
    const AccelBuffers& b = a->buf;
    views[k] = {b.node_width != 2 ? b.nodes4.as<const float4>() : b.nodes.as<const float4>(), b.prims.as<const float4>(),
                b.order.as<const uint32_t>(), b.root.as<const float>(), b.n_nodes, b.n_slots};
  }
  if (ray_offsets[n] >= (1u << 31)) return fail(ctx, RQ_ERROR_INVALID_ARGUMENT, "2^31 or more rays");
  const size_t vbytes = ((sizeof(Bvh2View) * n + 15) & ~size_t(15));
  const size_t obytes = ((4 * ((size_t)n + 1) + 15) & ~size_t(15));
  RQ_TRY_CUDA(ctx, table.ensure(vbytes + obytes + 16));
  char* base = table.as<char>();
  RQ_TRY_CUDA(ctx, cudaMemcpyAsync(base, views.data(), sizeof(Bvh2View) * n, cudaMemcpyHostToDevice, ctx->stream));
  RQ_TRY_CUDA(ctx, cudaMemcpyAsync(base + vbytes, ray_offsets, 4 * ((size_t)n + 1), cudaMemcpyHostToDevice, ctx->stream));
  RQ_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream));  // the host tables may change after the call
  t = BatchedTrace();
  t.kind = accels[0]->scene->kind;
  t.any = any;
  t.width = (int)accels[0]->buf.node_width;
  t.unit = true;
  for (uint32_t k = 0; k < n; ++k) t.unit = t.unit && accels[k]->buf.unit_leaves;
  t.views = reinterpret_cast<const Bvh2View*>(base);
  t.roff = reinterpret_cast<const uint32_t*>(base + vbytes);
  t.n_views = n;
  t.n = ray_offsets[n];
  t.work = reinterpret_cast<uint32_t*>(base + vbytes + obytes);
  t.err = ctx->d_err;
  return RQ_SUCCESS;
}

// The per-scene ray order of a many-structure query: keys, a stable sort,
// and t.perm pointing at the permutation.
static BuildResult enqueue_batch_order(BatchedTrace& t, DevBuf& keys, DevBuf& vals, BuildScratch& sc, uint32_t* err,
                                       cudaStream_t st) {
  const int bits = batch_key_bits(t.n_views);
  if (bits > 32) return BuildResult::error(RQ_ERROR_UNSUPPORTED, "ray order: more than 2^17 structures");
  cudaError_t e = keys.ensure((size_t)t.n * 4);
  if (e == cudaSuccess) e = vals.ensure((size_t)t.n * 4);
  if (e != cudaSuccess) return BuildResult::cuda_error(e, "ray order buffers");
  launch_batch_ray_keys(t, keys.as<uint32_t>(), vals.as<uint32_t>(), st);
  BuildResult r = sort_pairs(keys.as<uint32_t>(), vals.as<uint32_t>(), t.n, (bits + 7) / 8, true, sc, err, st);
  t.perm = vals.as<const uint32_t>();
  return r;
}

rq_status_t rq_trace_batched(rq_ctx_t ctx, const rq_accel_t* accels, uint32_t n_accels, const rq_ray_t* rays,
                             const uint32_t* ray_offsets, int32_t any, void* out, uint32_t flags) {
  RQ_TRY(bind(ctx));
  BatchedTrace t;
  RQ_TRY(batch_tables(ctx, accels, n_accels, ray_offsets, any != 0, ctx->batch_table, t));
  if (t.n == 0) return RQ_SUCCESS;
  if (!rays || !out) return fail(ctx, RQ_ERROR_INVALID_ARGUMENT, "null ray or result buffer");
  const bool dev = flags & RQ_DEVICE_POINTERS;
  const float4* d_rays = nullptr;
  RQ_TRY(to_device(ctx, ctx->stage_in, reinterpret_cast<const float4*>(rays), (size_t)t.n * 32, flags, &d_rays));
  const size_t out_bytes = any ? (size_t)((t.n + 31) / 32) * 4 : (size_t)t.n * 16;
  void* d_out = out;
  if (!dev) {
    RQ_TRY_CUDA(ctx, ctx->stage_out.ensure(out_bytes));
    d_out = ctx->stage_out.p;
  }
  t.rays = d_rays;
  t.hits = any ? nullptr : static_cast<float4*>(d_out);
  t.occ = any ? static_cast<uint32_t*>(d_out) : nullptr;
  if (ctx->settings.ray_sort != RQ_RAY_SORT_NONE && batch_key_bits(t.n_views) <= 32) {
    BuildResult br = enqueue_batch_order(t, ctx->scratch.keys, ctx->scratch.vals, ctx->scratch, ctx->d_err, ctx->stream);
    if (br.cuda != cudaSuccess) return cuda_fail(ctx, br.cuda, br.what);
    if (br.status != RQ_SUCCESS) return fail(ctx, br.status, br.what);
  }
  RQ_TRY_CUDA(ctx, launch_trace_batched(t, 128, 1, ctx->stream));
  if (dev) return RQ_SUCCESS;
  RQ_TRY_CUDA(ctx, cudaMemcpyAsync(out, d_out, out_bytes, cudaMemcpyDeviceToHost, ctx->stream));
  return collect_device_errors(ctx);
}

// Read and clear the device error word without mapping it to a status.
static cudaError_t take_device_errors(rq_ctx_t ctx, uint32_t* e) {
  *e = 0;
  cudaError_t c = cudaMemcpyAsync(e, ctx->d_err, 4, cudaMemcpyDeviceToHost, ctx->stream);
  if (c == cudaSuccess) c = cudaStreamSynchronize(ctx->stream);
  if (c == cudaSuccess && *e) c = cudaMemsetAsync(ctx->d_err, 0, 4, ctx->stream);
  return c;
}

rq_status_t rq_plan_create(rq_ctx_t ctx, const rq_accel_t* accels, uint32_t n_accels, int32_t rebuild,
                           const rq_ray_t* rays, const uint32_t* ray_offsets, int32_t any, void* out,
                           rq_plan_t* out_plan) {
  if (!out_plan) return fail(ctx, RQ_ERROR_INVALID_ARGUMENT, "null plan");
  *out_plan = nullptr;
  RQ_TRY(bind(ctx));
  std::unique_ptr<rq_plan> p(new (std::nothrow) rq_plan());
  if (!p) return RQ_ERROR_OUT_OF_MEMORY;
  p->ctx = ctx;
  RQ_TRY(batch_tables(ctx, accels, n_accels, ray_offsets, any != 0, p->table, p->trace));
  if (p->trace.n > 0 && (!rays || !out)) return fail(ctx, RQ_ERROR_INVALID_ARGUMENT, "null ray or result buffer");
  p->trace.rays = reinterpret_cast<const float4*>(rays);
  p->trace.hits = any ? nullptr : static_cast<float4*>(out);
  p->trace.occ = any ? static_cast<uint32_t*>(out) : nullptr;
  p->accels.assign(accels, accels + n_accels);
  if (rebuild) {
    p->store = accels[0]->batch;
    if (!p->store || p->store->n_scenes != n_accels)
      return fail(ctx, RQ_ERROR_INVALID_ARGUMENT, "a rebuilding plan needs the whole batch of one rq_build_batched call");
    // one rebuild outside the capture sizes every scratch array it touches
    RQ_TRY(rq_accel_rebuild_batched(ctx, accels, n_accels));
    RQ_TRY(collect_device_errors(ctx));
  }
  // The per-scene ray order, once outside the capture (sizes its buffers
  // and sort scratch), when the keys fit 32 bits.
  const bool can_order = p->trace.n > 0 && batch_key_bits(p->trace.n_views) <= 32;
  if (can_order) {
    BatchedTrace t = p->trace;
    BuildResult br = enqueue_batch_order(t, p->order_keys, p->order_vals, p->order_scratch, ctx->d_err, ctx->stream);
    if (br.cuda != cudaSuccess) return cuda_fail(ctx, br.cuda, br.what);
    if (br.status != RQ_SUCCESS) return fail(ctx, br.status, br.what);
    RQ_TRY(collect_device_errors(ctx));
  }
  // Autotuning: time every launch shape on these rays, without and with the
  // ray order (whose time includes its keys and sort); a shape whose stack
  // overflows on these trees is dropped.  A rebuilding plan owns its batch
  // and also tries every node width (binary, collapsed 4-wide, compressed
  // 8-wide): the structures keep the width the plan picks.
  const int shapes[4][2] = {{128, 0}, {128, 1}, {256, 0}, {256, 1}};
  const uint32_t width0 = accels[0]->buf.node_width;
  std::vector<uint32_t> widths;
  if (rebuild) widths = {2, 4, 8};
  else widths = {width0};
  auto set_width = [&](uint32_t w) -> rq_status_t {
    for (uint32_t k = 0; k < n_accels; ++k) {
      AccelBuffers& b = accels[k]->buf;
      if (b.node_width == w) continue;
      b.node_width = 2;
      BuildResult r;
      if (w == 4) r = collapse_bvh4(b, ctx->scratch, ctx->d_err, ctx->stream);
      else if (w == 8) r = collapse_bvh8(b, ctx->scratch, ctx->d_err, ctx->stream);
      if (!r.ok()) return r.cuda != cudaSuccess ? cuda_fail(ctx, r.cuda, r.what) : fail(ctx, r.status, r.what);
    }
    RQ_TRY(collect_device_errors(ctx));
    BatchedTrace keep = p->trace;
    RQ_TRY(batch_tables(ctx, accels, n_accels, ray_offsets, any != 0, p->table, p->trace));
    p->trace.rays = keep.rays;
    p->trace.hits = keep.hits;
    p->trace.occ = keep.occ;
    return RQ_SUCCESS;
  };
  float best = -1.f;
  uint32_t best_width = width0;
  auto wi = [](uint32_t w) { return w == 4 ? 1 : w == 8 ? 2 : 0; };
  float tab[3][2][4];
  for (auto& a : tab)
    for (auto& b : a)
      for (float& x : b) x = -1.f;
  if (p->trace.n > 0) {
    cudaEvent_t e0, e1;
    RQ_TRY_CUDA(ctx, cudaEventCreate(&e0));
    RQ_TRY_CUDA(ctx, cudaEventCreate(&e1));
    for (uint32_t w : widths) {
      if (widths.size() > 1) {
        rq_status_t sw = set_width(w);
        if (sw != RQ_SUCCESS) {
          cudaEventDestroy(e0);
          cudaEventDestroy(e1);
          return sw;
        }
      }
      float best_w = -1.f;
      for (int v = 0; v < (can_order ? 2 : 1); ++v) {
        for (int k = 0; k < 4; ++k) {
          float ms = 1e30f;
          cudaError_t ce = cudaSuccess;
          for (int rep = 0; rep < 3 && ce == cudaSuccess; ++rep) {
            BatchedTrace t = p->trace;
            ce = cudaEventRecord(e0, ctx->stream);
            if (ce == cudaSuccess && v == 1) {
              BuildResult br = enqueue_batch_order(t, p->order_keys, p->order_vals, p->order_scratch, ctx->d_err,
                                                   ctx->stream);
              if (!br.ok()) ce = br.cuda != cudaSuccess ? br.cuda : cudaErrorInvalidValue;
            }
            if (ce == cudaSuccess) ce = launch_trace_batched(t, shapes[k][0], shapes[k][1], ctx->stream);
            if (ce == cudaSuccess) ce = cudaEventRecord(e1, ctx->stream);
            if (ce == cudaSuccess) ce = cudaEventSynchronize(e1);
            float tm = 0.f;
            if (ce == cudaSuccess) ce = cudaEventElapsedTime(&tm, e0, e1);
            if (ce == cudaSuccess && rep > 0) ms = std::min(ms, tm);
          }
          uint32_t derr = 0;
          if (ce == cudaSuccess) ce = take_device_errors(ctx, &derr);
          if (ce != cudaSuccess) {
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            return cuda_fail(ctx, ce, "plan autotuning");
          }
          if (derr & ~kErrStackOverflow) {
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            return fail(ctx, RQ_ERROR_INVALID_ARGUMENT, "malformed structure or input seen while autotuning");
          }
          if (derr & kErrStackOverflow) continue;
          tab[wi(w)][v][k] = ms;
          if (best_w < 0.f || ms < best_w) best_w = ms;
          if (best < 0.f || ms < best) {
            best = ms;
            best_width = w;
            p->block = shapes[k][0];
            p->deep = shapes[k][1];
            p->ordered = v == 1;
          }
        }
      }
      p->width_ms[wi(w)] = best_w;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (best < 0.f) return fail(ctx, RQ_ERROR_STACK_OVERFLOW, "every launch shape overflowed its traversal stack");
    if (widths.size() > 1) RQ_TRY(set_width(best_width));
    for (int k = 0; k < 4; ++k) {
      p->shape_ms[k] = tab[wi(best_width)][0][k];
      p->ordered_ms[k] = tab[wi(best_width)][1][k];
    }
  }
  p->node_width = best_width;
  // Capture [rebuild] + query into one graph on a private stream.
  cudaStream_t cap = nullptr;
  RQ_TRY_CUDA(ctx, cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
  const uint64_t k0 = launch_total();
  cudaError_t ce = cudaStreamBeginCapture(cap, cudaStreamCaptureModeRelaxed);
  BuildResult br;
  if (ce == cudaSuccess && p->store) {
    br = build_batch(*p->store, ctx->settings.morton, ctx->d_err, cap);
    for (uint32_t k = 0; br.ok() && k < n_accels; ++k)
      if (accels[k]->buf.node_width == 4) br = collapse_bvh4(accels[k]->buf, ctx->scratch, ctx->d_err, cap);
      else if (accels[k]->buf.node_width == 8) br = collapse_bvh8(accels[k]->buf, ctx->scratch, ctx->d_err, cap);
  }
  BatchedTrace qt = p->trace;
  if (ce == cudaSuccess && br.ok() && p->ordered)
    br = enqueue_batch_order(qt, p->order_keys, p->order_vals, p->order_scratch, ctx->d_err, cap);
  if (ce == cudaSuccess && br.ok()) ce = launch_trace_batched(qt, p->block, p->deep, cap);
  cudaError_t end = cudaStreamEndCapture(cap, &p->graph);
  p->kernels = launch_total() - k0;
  cudaStreamDestroy(cap);
  if (ce == cudaSuccess && !br.ok()) ce = br.cuda != cudaSuccess ? br.cuda : cudaErrorInvalidValue;
  if (ce == cudaSuccess) ce = end;
  if (ce == cudaSuccess) ce = cudaGraphInstantiate(&p->exec, p->graph, 0);
  if (ce != cudaSuccess) {
    if (p->graph) cudaGraphDestroy(p->graph);
    cudaGetLastError();
    return cuda_fail(ctx, ce, "plan capture");
  }
  *out_plan = p.release();
  return RQ_SUCCESS;
}

rq_status_t rq_plan_launch(rq_plan_t p) {
  if (!p) return RQ_ERROR_INVALID_ARGUMENT;
  rq_ctx_t ctx = p->ctx;
  RQ_TRY(bind(ctx));
  RQ_TRY_CUDA(ctx, cudaGraphLaunch(p->exec, ctx->stream));
  count_launch(p->kernels);
  return RQ_SUCCESS;
}

rq_status_t rq_plan_get_info(rq_plan_t p, rq_plan_info_t* info) {
  if (!p || !info) return RQ_ERROR_INVALID_ARGUMENT;
  std::memset(info, 0, sizeof(*info));
  info->block_threads = (uint32_t)p->block;
  info->stack_entries = (uint32_t)batched_stack_entries(p->trace.width, p->deep);
  info->graph_kernels = (uint32_t)p->kernels;
  info->n_rays = p->trace.n;
  info->rebuilds = p->store ? 1 : 0;
  for (int k = 0; k < 4; ++k) info->shape_ms[k] = p->shape_ms[k];
  info->ray_order = p->ordered ? 1u : 0u;
  for (int k = 0; k < 4; ++k) info->ordered_ms[k] = p->ordered_ms[k];
  info->node_width = p->node_width;
  for (int k = 0; k < 3; ++k) info->width_ms[k] = p->width_ms[k];
  return RQ_SUCCESS;
}

rq_status_t rq_plan_destroy(rq_plan_t p) {
  if (!p) return RQ_ERROR_INVALID_ARGUMENT;
  cudaSetDevice(p->ctx->device);
  cudaStreamSynchronize(p->ctx->stream);
  if (p->exec) cudaGraphExecDestroy(p->exec);
  if (p->graph) cudaGraphDestroy(p->graph);
  p->table.release();
  p->order_keys.release();
  p->order_vals.release();
  p->order_scratch.release();
  delete p;
  return RQ_SUCCESS;
}

rq_status_t rq_trace_counters(rq_ctx_t ctx, rq_accel_t a, const rq_ray_t* rays, uint32_t n, int32_t any,
                              void* out, uint64_t* counters, uint32_t flags) {
  RQ_TRY(bind(ctx));
  if (!a || !counters) return fail(ctx, RQ_ERROR_INVALID_ARGUMENT, "null accel or counters");
  counters[0] = counters[1] = 0;
  if (n == 0) return RQ_SUCCESS;
  if (!rays || !out) return fail(ctx, RQ_ERROR_INVALID_ARGUMENT, "null ray or result buffer");
  const bool dev = flags & RQ_DEVICE_POINTERS;
  const float4* d_rays = nullptr;
  RQ_TRY(to_device(ctx, ctx->stage_in, reinterpret_cast<const float4*>(rays), (size_t)n * 32, flags, &d_rays));
  const size_t out_bytes = any ? (size_t)((n + 31) / 32) * 4 : (size_t)n * 16;
  void* d_out = out;
  if (!dev) {
    RQ_TRY_CUDA(ctx, ctx->stage_out.ensure(out_bytes));
    d_out = ctx->stage_out.p;
  }
  RQ_TRY_CUDA(ctx, ctx->stage_aux.ensure(64));
  unsigned long long* d_cnt = ctx->stage_aux.as<unsigned long long>();
  RQ_TRY_CUDA(ctx, cudaMemsetAsync(d_cnt, 0, 16, ctx->stream));
  QueryTarget q;
  q.rays = d_rays;
  q.n = n;
  q.hits = any ? nullptr : static_cast<float4*>(d_out);
  q.occ = any ? static_cast<uint32_t*>(d_out) : nullptr;
  BuildResult r = trace_counted(a->type, scene_view(a->scene), a->buf, any != 0, q, d_cnt, ctx->d_err, ctx->stream);
  if (r.cuda != cudaSuccess) return cuda_fail(ctx, r.cuda, r.what);
  if (r.status != RQ_SUCCESS) return fail(ctx, r.status, r.what);
  RQ_TRY_CUDA(ctx, cudaMemcpyAsync(counters, d_cnt, 16, cudaMemcpyDeviceToHost, ctx->stream));
  if (!dev) RQ_TRY_CUDA(ctx, cudaMemcpyAsync(out, d_out, out_bytes, cudaMemcpyDeviceToHost, ctx->stream));
  return collect_device_errors(ctx);
}

uint64_t rq_kernel_launch_count(void) { return launch_total(); }

// -------------------------------------------------------- component kernels

rq_status_t rq_morton_codes(rq_ctx_t ctx, rq_scene_t s, uint32_t* codes, uint32_t flags) {
  RQ_TRY(bind(ctx));
  if (!s || !codes) return fail(ctx, RQ_ERROR_INVALID_ARGUMENT, "null scene or output");
  uint32_t* d_codes = codes;
  if (!(flags & RQ_DEVICE_POINTERS)) {
    RQ_TRY_CUDA(ctx, ctx->stage_out.ensure((size_t)s->n * 4));
    d_codes = ctx->stage_out.as<uint32_t>();
  }
  RQ_TRY_CUDA(ctx, ctx->stage_aux.ensure((size_t)s->n * 4 + 64));
  uint32_t* d_vals = ctx->stage_aux.as<uint32_t>();
  BuildResult r = morton_codes(scene_view(s), ctx->settings.morton, d_codes, d_vals, nullptr, ctx->scratch, ctx->stream);
  if (r.cuda != cudaSuccess) return cuda_fail(ctx, r.cuda, r.what);
  RQ_TRY(check_launch(ctx, "morton launch"));
  if (!(flags & RQ_DEVICE_POINTERS)) {
    RQ_TRY_CUDA(ctx, cudaMemcpyAsync(codes, d_codes, (size_t)s->n * 4, cudaMemcpyDeviceToHost, ctx->stream));
    RQ_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  }
  return RQ_SUCCESS;
}

rq_status_t rq_sort_pairs(rq_ctx_t ctx, uint32_t* keys, uint32_t* values, uint32_t n,
                          uint32_t key_bits, uint32_t flags) {
  RQ_TRY(bind(ctx));
  if (n == 0) return RQ_SUCCESS;
  if (!keys || !values) return fail(ctx, RQ_ERROR_INVALID_ARGUMENT, "null keys or values");
  if (key_bits == 0 || key_bits > 32) return fail(ctx, RQ_ERROR_INVALID_ARGUMENT, "key_bits must be 1..32");
  if (n > (1u << 30) - 1) return fail(ctx, RQ_ERROR_INVALID_ARGUMENT, "more than 2^30-1 pairs");
  const bool dev = flags & RQ_DEVICE_POINTERS;
  uint32_t* dk = keys;
  uint32_t* dv = values;
  if (!dev) {
    RQ_TRY_CUDA(ctx, ctx->stage_in.ensure((size_t)n * 4));
    RQ_TRY_CUDA(ctx, ctx->stage_out.ensure((size_t)n * 4));
    dk = ctx->stage_in.as<uint32_t>();
    dv = ctx->stage_out.as<uint32_t>();
    RQ_TRY_CUDA(ctx, cudaMemcpyAsync(dk, keys, (size_t)n * 4, cudaMemcpyHostToDevice, ctx->stream));
    RQ_TRY_CUDA(ctx, cudaMemcpyAsync(dv, values, (size_t)n * 4, cudaMemcpyHostToDevice, ctx->stream));
  }
  ctx->scratch.stall = ctx->debug.sort_stall ? ctx->d_err + 1 : nullptr;
  BuildResult r = sort_pairs(dk, dv, n, (int)((key_bits + 7) / 8), true, ctx->scratch, ctx->d_err, ctx->stream);
  ctx->scratch.stall = nullptr;
  if (r.cuda != cudaSuccess) return cuda_fail(ctx, r.cuda, r.what);
  RQ_TRY(check_launch(ctx, "sort launch"));
  if (!dev) {
    RQ_TRY_CUDA(ctx, cudaMemcpyAsync(keys, dk, (size_t)n * 4, cudaMemcpyDeviceToHost, ctx->stream));
    RQ_TRY_CUDA(ctx, cudaMemcpyAsync(values, dv, (size_t)n * 4, cudaMemcpyDeviceToHost, ctx->stream));
    return collect_device_errors(ctx);
  }
  return RQ_SUCCESS;
}

rq_status_t rq_render_reference(rq_ctx_t ctx, rq_accel_t a, const rq_settings_t* settings,
                                const double* jitter, const float* surface_rgb, uint8_t* pixels,
                                float* rgb_sum) {
  RQ_TRY(bind(ctx));
  if (!a || !pixels || !surface_rgb) return fail(ctx, RQ_ERROR_INVALID_ARGUMENT, "null accel, colours or pixels");
  if (a->scene->kind != kSpheres) return fail(ctx, RQ_ERROR_UNSUPPORTED, "the reference render shades spheres");
  rq_settings_t s = settings ? *settings : ctx->settings;
  if (s.width == 0 || s.height == 0 || s.aa_samples == 0) return fail(ctx, RQ_ERROR_INVALID_ARGUMENT, "empty image");
  const uint64_t npix = (uint64_t)s.width * s.height;
  const uint64_t nray = npix * s.aa_samples;
  if (nray > (1ull << 31)) return fail(ctx, RQ_ERROR_INVALID_ARGUMENT, "image too large");
  // Jitter: the caller's, or the reference's default-seeded mt19937 draws
  // (random_double, main.cpp:503-508) in render()'s call order.  The
  // default sequence depends only on the sample count: drawn once on the
  // host and kept on the device for later calls.
  bool jitter_on_device = false;
  if (!jitter) {
    if (ctx->ref_jitter_n != nray || !ctx->ref_jitter.p) {
      std::vector<double> own(2 * nray);
      std::mt19937 gen;
      std::uniform_real_distribution<double> dist(0.0, 1.0);
      for (auto& v : own) v = dist(gen);
      ctx->ref_jitter_n = 0;
      RQ_TRY_CUDA(ctx, ctx->ref_jitter.ensure(own.size() * 8));
      RQ_TRY_CUDA(ctx, cudaMemcpy(ctx->ref_jitter.p, own.data(), own.size() * 8, cudaMemcpyHostToDevice));
      ctx->ref_jitter_n = nray;
    }
    jitter = ctx->ref_jitter.as<const double>();
    jitter_on_device = true;
  }
  // render() camera constants (main.cpp:544-546), computed on the host with
  // the same double-precision tan the reference calls.
  float fov = 30, aspect = s.width / float(s.height);
  float angle = (float)std::tan(3.141592653589793 * 0.5 * fov / 180.);
  cudaError_t e = render_reference(a->type, scene_view(a->scene), a->buf, s, angle, aspect, jitter,
                                   jitter_on_device, surface_rgb, ctx->stage_in, ctx->stage_out, ctx->stage_aux,
                                   pixels, rgb_sum, ctx->d_err, ctx->stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "render");
  return collect_device_errors(ctx);
}

rq_status_t rq_render(rq_ctx_t ctx, rq_accel_t a, const rq_view_t* view, uint8_t* pixels, float* rgb,
                      uint64_t* ray_counts, uint32_t flags) {
  RQ_TRY(bind(ctx));
  if (!a || !view || !pixels) return fail(ctx, RQ_ERROR_INVALID_ARGUMENT, "null accel, view or pixels");
  const rq_settings_t& s = ctx->settings;
  const bool dev = (flags & RQ_DEVICE_POINTERS) != 0;
  if (dev && ray_counts) return fail(ctx, RQ_ERROR_INVALID_ARGUMENT, "ray_counts needs a synchronous call");
  if (s.width == 0 || s.height == 0 || s.aa_samples == 0) return fail(ctx, RQ_ERROR_INVALID_ARGUMENT, "empty image");
  const bool whole = view->window[2] == 0 || view->window[3] == 0;
  const uint64_t ww = whole ? s.width : view->window[2], wh = whole ? s.height : view->window[3];
  if (!whole && ((uint64_t)view->window[0] + ww > s.width || (uint64_t)view->window[1] + wh > s.height))
    return fail(ctx, RQ_ERROR_INVALID_ARGUMENT, "window outside the image");
  const uint64_t npix = ww * wh, nray = npix * s.aa_samples;
  if (nray >= (1ull << 31)) return fail(ctx, RQ_ERROR_INVALID_ARGUMENT, "image too large (2^31 samples)");
  const float geo[] = {view->eye[0], view->eye[1], view->eye[2], view->target[0], view->target[1],
                       view->target[2], view->up[0], view->up[1], view->up[2], view->light[0],
                       view->light[1], view->light[2], view->albedo[0], view->albedo[1], view->albedo[2],
                       view->ambient, view->mirror, view->fov_deg};
  if (!finite3(geo, sizeof(geo) / sizeof(geo[0])) || !(view->fov_deg > 0.f && view->fov_deg < 180.f) ||
      !(view->mirror >= 0.f && view->mirror <= 1.f))
    return fail(ctx, RQ_ERROR_INVALID_ARGUMENT, "view: non-finite values, fov outside (0, 180) or mirror outside [0, 1]");
  // tan of half the field of view, in double on the host, then rounded once
  const float tan_half = (float)std::tan((double)view->fov_deg * 3.141592653589793 / 360.0);
  RenderScratch& rs = ctx->render;
  uint8_t* d_pix = pixels;
  float* d_rgb = rgb;
  if (!dev) {
    const size_t pix_bytes = (npix * 3 + 255) & ~size_t(255);
    RQ_TRY_CUDA(ctx, rs.out.ensure(pix_bytes + (rgb ? npix * 12 : 0)));
    d_pix = rs.out.as<uint8_t>();
    d_rgb = rgb ? reinterpret_cast<float*>(rs.out.as<char>() + pix_bytes) : nullptr;
  }
  RQ_TRY_CUDA(ctx, rs.counters.ensure(16));
  RQ_TRY_CUDA(ctx, cudaMemsetAsync(rs.counters.p, 0, 16, ctx->stream));
  rq_status_t est = RQ_SUCCESS;
  cudaError_t e = render_view(a->type, scene_view(a->scene), a->buf, s, *view, tan_half, rs, ctx->scratch, d_pix,
                              d_rgb, rs.counters.as<unsigned long long>(), ctx->d_err, ctx->stream, &est);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "render");
  if (est != RQ_SUCCESS) return fail(ctx, est, "render query");
  if (dev) return RQ_SUCCESS;
  RQ_TRY_CUDA(ctx, cudaMemcpyAsync(pixels, d_pix, npix * 3, cudaMemcpyDeviceToHost, ctx->stream));
  if (rgb) RQ_TRY_CUDA(ctx, cudaMemcpyAsync(rgb, d_rgb, npix * 12, cudaMemcpyDeviceToHost, ctx->stream));
  uint64_t cnt[2] = {0, 0};
  if (ray_counts) RQ_TRY_CUDA(ctx, cudaMemcpyAsync(cnt, rs.counters.p, 16, cudaMemcpyDeviceToHost, ctx->stream));
  RQ_TRY(collect_device_errors(ctx));
  if (ray_counts) {
    ray_counts[0] = nray;
    ray_counts[1] = cnt[0];
    ray_counts[2] = cnt[1];
  }
  return RQ_SUCCESS;
}

}  // extern "C"
