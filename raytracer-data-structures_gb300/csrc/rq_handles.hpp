// Definitions of the C ABI's opaque handles (contexts, scenes, structures,
// plans), shared by the translation units that implement the ABI.
#pragma once
#include <cuda_runtime.h>

#include <memory>
#include <string>
#include <vector>

#include "rq_build.hpp"
#include "rq_internal.hpp"

using namespace rq;

// Host-buffer queries of at least 2 chunks are streamed: chunk k+1 uploads
// (one copy stream) and chunk k-1 downloads (another) while chunk k is traced.
// Chunks alternate between two compute lanes (the context's stream and one
// more, each with its own sort scratch) so that the slow tail of one chunk's
// traversal overlaps the start of the next.
constexpr uint32_t kPipeChunk = 1u << 21;  // rays per chunk: 64 MB up, 32 MB (or 256 KB of bits) down
constexpr int kPipeSlots = 3;
struct HostPipe {
  cudaStream_t up = nullptr, down = nullptr, lane2 = nullptr;
  BuildScratch scratch2;
  cudaEvent_t start = nullptr, uploaded[kPipeSlots] = {}, traced[kPipeSlots] = {}, downloaded[kPipeSlots] = {};
  DevBuf rays[kPipeSlots], out[kPipeSlots];
  std::vector<DevBuf> q_rays, q_out;   // whole-query buffers of rq_trace_queries
  std::vector<cudaEvent_t> q_events;   // uploaded / traced per query
  bool ready = false;
  cudaError_t init() {
    if (ready) return cudaSuccess;
    cudaError_t e = cudaStreamCreateWithFlags(&up, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&down, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&lane2, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&start, cudaEventDisableTiming);
    for (int k = 0; k < kPipeSlots && e == cudaSuccess; ++k) {
      e = cudaEventCreateWithFlags(&uploaded[k], cudaEventDisableTiming);
      if (e == cudaSuccess) e = cudaEventCreateWithFlags(&traced[k], cudaEventDisableTiming);
      if (e == cudaSuccess) e = cudaEventCreateWithFlags(&downloaded[k], cudaEventDisableTiming);
    }
    ready = e == cudaSuccess;
    return e;
  }
  void release() {
    for (int k = 0; k < kPipeSlots; ++k) {
      rays[k].release();
      out[k].release();
      if (uploaded[k]) cudaEventDestroy(uploaded[k]);
      if (traced[k]) cudaEventDestroy(traced[k]);
      if (downloaded[k]) cudaEventDestroy(downloaded[k]);
      uploaded[k] = traced[k] = downloaded[k] = nullptr;
    }
    if (start) cudaEventDestroy(start);
    if (up) cudaStreamDestroy(up);
    if (down) cudaStreamDestroy(down);
    if (lane2) cudaStreamDestroy(lane2);
    scratch2.release();
    for (auto& b : q_rays) b.release();
    for (auto& b : q_out) b.release();
    for (cudaEvent_t e : q_events) cudaEventDestroy(e);
    q_rays.clear();
    q_out.clear();
    q_events.clear();
    start = nullptr;
    up = down = lane2 = nullptr;
    ready = false;
  }
};

struct rq_context {
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaStream_t own_stream = nullptr;
  rq_settings_t settings{};
  std::string last_error;
  uint32_t* d_err = nullptr;
  int sm_count = 0;
  DevBuf stage_in, stage_out, stage_aux;
  BuildScratch scratch;
  RenderScratch render;
  HostPipe pipe;
  DevBuf batch_table;  // views + ray offsets + work counter of rq_trace_batched
  DevBuf ref_jitter;   // the reference render's default-seeded jitter, generated once per sample count
  uint64_t ref_jitter_n = 0;
  rq_debug_t debug{};  // test hooks (rq_set_debug); all off by default
};

struct rq_plan {
  rq_ctx_t ctx = nullptr;
  std::vector<rq_accel_t> accels;
  std::shared_ptr<BatchStore> store;  // set when the plan rebuilds a batch
  BatchedTrace trace;
  DevBuf table;
  int block = 128, deep = 1;
  bool ordered = false;                   // the query runs through a per-scene ray order
  float shape_ms[4] = {-1.f, -1.f, -1.f, -1.f};
  float ordered_ms[4] = {-1.f, -1.f, -1.f, -1.f};
  uint32_t node_width = 2;                // the structures' node width the plan runs with
  float width_ms[3] = {-1.f, -1.f, -1.f}; // best query time per node width 2 / 4 / 8 (< 0: not tried)
  DevBuf order_keys, order_vals;          // ray order keys and the permutation
  BuildScratch order_scratch;             // its sort's scratch (sized before the capture)
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  uint64_t kernels = 0;
};

struct rq_scene {
  rq_ctx_t ctx = nullptr;
  int kind = kTriangles;
  uint32_t n = 0;   // primitives
  uint32_t nv = 0;  // vertices (triangles)
  DevBuf verts, idx, sph;
  DevBuf verts4, idx4;  // 16-byte copies of verts and idx for the LBVH build's gathers
};

struct rq_accel {
  rq_ctx_t ctx = nullptr;
  rq_scene_t scene = nullptr;
  int type = RQ_NONE;
  AccelBuffers buf;
  std::shared_ptr<BatchStore> batch;  // set when buf borrows a batched build's arrays
  uint32_t batch_index = 0;
  bool imported = false;  // made by rq_accel_import_bvh2: nothing to rebuild from
};

