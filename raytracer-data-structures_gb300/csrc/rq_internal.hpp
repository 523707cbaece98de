// Host-side internals shared by the engine's translation units: handle
// structures, device buffers and the kernel launchers each .cu file exports.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "rq.h"

namespace rq {

// Grow-only device allocation.  A borrowed buffer (owned = false) is a slice
// of memory owned elsewhere: it never grows and is never freed here.
struct DevBuf {
  void* p = nullptr;
  size_t cap = 0;
  bool owned = true;
  cudaError_t ensure(size_t bytes) {
    if (bytes <= cap && p) return cudaSuccess;
    if (!owned) return cudaErrorInvalidValue;
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
    size_t want = bytes < 256 ? 256 : bytes;
    cudaError_t e = cudaMalloc(&p, want);
    if (e == cudaSuccess) cap = want;
    return e;
  }
  void release() {
    if (p && owned) cudaFree(p);
    p = nullptr;
    cap = 0;
    owned = true;
  }
  template <typename T>
  T* as() const {
    return static_cast<T*>(p);
  }
};

enum PrimKind { kTriangles = 0, kSpheres = 1 };

// Process-wide count of kernel launches made by the engine (rq_kernel_launch_count).
void count_launch(uint64_t k = 1);

// ----------------------------------------------------------- radix sort
struct SortScratch {
  uint32_t* keys_alt;
  uint32_t* vals_alt;
  uint32_t* hist;      // 4 * 256 digit counts
  uint32_t* status;    // passes * tiles * 256 look-back words
  uint32_t* counters;  // one tile counter per pass
  // Test hook: non-null makes tile 1 of the first pass wait (bounded) on this
  // device word, which nothing sets, so the sort reports a timeout.
  const uint32_t* stall = nullptr;
};
uint32_t sort_tiles(uint32_t n);
size_t sort_status_words(uint32_t n, int passes);
// hist must hold the digit histogram of `keys` for every pass (as produced by
// launch_histogram or the fused Morton kernels).  status/counters must be
// zero.  Result lands in keys/vals.
void launch_histogram(const uint32_t* keys, uint32_t n, int passes, uint32_t* hist, cudaStream_t s);
void launch_onesweep(uint32_t* keys, uint32_t* vals, uint32_t n, int passes, const SortScratch& sc,
                     uint32_t* err, cudaStream_t s);
// As launch_onesweep, without copying the result back after an odd number of
// passes: returns the buffer (vals or sc.vals_alt) that holds the sorted values.
uint32_t* launch_onesweep_vals(uint32_t* keys, uint32_t* vals, uint32_t n, int passes, const SortScratch& sc,
                               uint32_t* err, cudaStream_t s);

// 64-bit keys, 32-bit values (tiles of 2,560 keys).  hist: 256 words per pass
// (up to 8 passes); status: sort_status_words64 words; counters: one per pass.
size_t sort_status_words64(uint32_t n, int passes);
void launch_histogram64(const uint64_t* keys, uint32_t n, int passes, uint32_t* hist, cudaStream_t s);
void launch_onesweep64(uint64_t* keys, uint32_t* vals, uint32_t n, int passes, uint64_t* keys_alt,
                       uint32_t* vals_alt, const uint32_t* hist, uint32_t* status, uint32_t* counters,
                       uint32_t* err, cudaStream_t s);

// --------------------------------------------------------- Morton codes
void launch_init_bounds(int32_t* lohi, cudaStream_t s);
void launch_point_bounds(const float* pts, uint32_t n, uint32_t stride, int32_t* lohi,
                         cudaStream_t s);
// mode: rq_morton_t (SCENE_BOUNDS and SCENE_CUBE use lohi).  hist may be
// null; otherwise the 4-pass digit histogram is accumulated into it.
// SM count of the current device (cached per device); 1 if it cannot be read.
int device_sm_count();
// 16-byte copies of a triangle scene (vertices as float4, triangles as uint4,
// w = 0) for the gathers of the LBVH build; idx4 may be null (vertices only).
void launch_pack_tris(const float* verts, uint32_t nv, const uint32_t* idx, uint32_t nt, float4* verts4,
                      uint4* idx4, cudaStream_t s);
void launch_morton_tris(const float4* verts, const uint4* idx, uint32_t nt, int mode, const int32_t* lohi,
                        uint32_t* keys, uint32_t* vals, uint32_t* hist, cudaStream_t s);
void launch_morton_spheres(const float4* sph, uint32_t n, int mode, const int32_t* lohi,
                           uint32_t* keys, uint32_t* vals, uint32_t* hist, cudaStream_t s);

// ---------------------------------------------------------------- LBVH
// Refit decomposition written by launch_karras: mark[n - 1] (per internal
// node), top[2048] (top node list), treelets[2n] (uint2 records) and two
// counters (top nodes, treelets) zeroed before launch_karras.
constexpr uint32_t kRefitTopCapHost = 2048;  // top list capacity (kRefitTopCap on the device)
struct RefitTop {
  uint32_t* mark;
  uint32_t* top;
  uint32_t* treelets;
  uint32_t* count;  // [0] top nodes, [1] treelets
};
inline size_t refit_treelet_offset(uint32_t n) { return ((size_t)n + kRefitTopCapHost + 1) & ~(size_t)1; }  // 8-byte aligned
inline size_t refit_mark_words(uint32_t n) { return refit_treelet_offset(n) + 2 * (size_t)n; }
void launch_karras(const uint32_t* sorted_codes, uint32_t n, float4* nodes, uint32_t* parent,
                   const RefitTop& top, cudaStream_t s);
// Gathers each slot's primitive into the slot-ordered payload and computes
// every node box: treelets in shared memory, one block each, then the top
// nodes in one block (or by device-scope climbing when they exceed its
// capacity); root_out gets 6 floats.  heights (optional, n - 1 bytes): the
// height of every internal node below the top nodes.
cudaError_t launch_refit(int kind, const float4* verts, const uint4* idx, const float4* sph,
                         const uint32_t* order, uint32_t n, float4* nodes, const uint32_t* parent,
                         const RefitTop& top, uint32_t* flags, float4* prims, float* root_out, uint32_t* err,
                         cudaStream_t s, uint8_t* heights = nullptr);
// One bottom-up pass of four-leaf treelet restructuring over a refitted LBVH
// of n one-primitive leaves (the refit decomposition of launch_karras; its
// treelet queue word top.count[3] must be zero; heights from launch_refit).
cudaError_t launch_treelet_opt(uint32_t n, float4* nodes, const uint32_t* parent, const RefitTop& top,
                               const uint8_t* heights, uint32_t* err, cudaStream_t s);
// Payload in primitive-id order (KD and brute force) plus per-primitive boxes.
void launch_prims_by_id(int kind, const float* verts, const uint32_t* idx, const float4* sph,
                        uint32_t n, float4* prims, float* aabb6, cudaStream_t s);

// Payload gathered in slot order (order[slot] = primitive id).
void launch_prims_gather(int kind, const float* verts, const uint32_t* idx, const float4* sph,
                         const uint32_t* order, uint32_t n, float4* prims, cudaStream_t s);

// ----------------------------------------------------------------- scan
// Exclusive prefix sum of n 32-bit values; tmp holds scan_tmp_words(n) words;
// total (may be null) receives the sum.
size_t scan_tmp_words(uint64_t n);
void launch_scan_excl(const uint32_t* in, uint32_t* out, uint64_t n, uint32_t* tmp, uint32_t* total,
                      cudaStream_t s);
// Two arrays of the same length in one set of launches; tmp holds
// 2 * scan_tmp_words(n) words; either total may be null.
void launch_scan2_excl(const uint32_t* in0, uint32_t* out0, const uint32_t* in1, uint32_t* out1, uint64_t n,
                       uint32_t* tmp, uint32_t* total0, uint32_t* total1, cudaStream_t s);

// ------------------------------------------------------------ traversal
struct Bvh2View {
  const float4* nodes;
  const float4* prims;    // slot order: 3 float4 per triangle, 1 per sphere
  const uint32_t* order;  // slot -> primitive id
  const float* root;      // 6 floats
  uint32_t n_internal;
  uint32_t n_slots;
  uint32_t unit_leaves = 0;  // 1: every leaf holds one primitive (LBVH): 4-byte stack entries
};
// perm (optional): trace ray perm[i] in thread i (results stay in caller order).
// small_stack (a test hook): the FAST walk's stack holds kDebugStack entries,
// so moderately deep trees overflow it.
constexpr int kDebugStack = 8;
// exact (optional): n + 2 words of scratch; FAST queries then run as
// persistent warps (word 1 their work counter) and walk the rays that need
// the exact box test in a second, small launch, keeping the main kernel to
// the fused walk.
void launch_trace_bvh2(int kind, int traversal, bool any, const Bvh2View& v, const float4* rays,
                       uint32_t n, float4* hits, uint32_t* occ, uint32_t* err, cudaStream_t s,
                       const uint32_t* perm = nullptr, bool small_stack = false, uint32_t* exact = nullptr);
// boxIntersect's candidate lists: ids == null counts per ray into counts;
// otherwise writes each ray's ids at offs[r] (and checks the counts).
// Count pass (ids null): counts[r] and *total (64-bit sum, zeroed by the
// caller).  Fill pass: ids at offs[r], at most counts[r] per ray.
void launch_candidates(const Bvh2View& v, const float4* rays, uint32_t n, uint32_t* counts, const uint32_t* offs,
                       uint32_t* ids, unsigned long long* total, uint32_t* err, cudaStream_t s);
// FAST traversal by persistent warps that refill finished lanes (one work
// word, zeroed by the launcher); same results as launch_trace_bvh2.
cudaError_t launch_trace_bvh2_refill(int kind, bool any, const Bvh2View& v, const float4* rays, uint32_t n,
                                     float4* hits, uint32_t* occ, uint32_t* err, const uint32_t* perm,
                                     uint32_t* work, cudaStream_t s);
// FAST traversal with speculative leaf postponement (while-while); same results.
// Warp-packet FAST traversal (RQ_SCHEDULING_WARP_PACKET): one stack per warp.
void launch_trace_bvh2_packet(int kind, bool any, const Bvh2View& v, const float4* rays, uint32_t n, float4* hits,
                              uint32_t* occ, uint32_t* err, const uint32_t* perm, cudaStream_t s);
// FAST traversal with the top levels of the tree staged in shared memory per
// block (RQ_SCHEDULING_SHARED_TOP); top: 4 KB of scratch for their copy.
void launch_trace_bvh2_top(int kind, bool any, const Bvh2View& v, float4* top, const float4* rays, uint32_t n,
                           float4* hits, uint32_t* occ, uint32_t* err, const uint32_t* perm, cudaStream_t s);
void launch_trace_bvh2_spec(int kind, bool any, const Bvh2View& v, const float4* rays, uint32_t n, float4* hits,
                            uint32_t* occ, uint32_t* err, const uint32_t* perm, cudaStream_t s);
// Coherence sort keys (mode: rq_ray_sort_t other than NONE, 30 bits); vals = identity.
// With hist (zeroed, 256 words per pass) it also counts the sort's `passes`
// digits, as launch_histogram would.
// Ray orders of at most 6 key bits (RQ_RAY_SORT_OCTANT, RQ_RAY_SORT_OCTANT_MORTON3)
// as a stable counting sort: perm gets the order the stable radix sort of the
// same keys gives; scratch: ray_order_small_bytes(n, mode) bytes.
size_t ray_order_small_bytes(uint32_t n, int mode);
void launch_ray_order_small(const float4* rays, uint32_t n, const float* root, int mode, void* scratch,
                            uint32_t* perm, cudaStream_t s);
void launch_ray_keys(const float4* rays, uint32_t n, const float* root, int mode, uint32_t* keys, uint32_t* vals,
                     cudaStream_t s, uint32_t* hist = nullptr, int passes = 0);
// FAST traversal that also sums internal-node visits and primitive tests
// into counters[0..1] (the inputs of the traversal byte model).
void launch_trace_bvh2_counted(int kind, bool any, const Bvh2View& v, const float4* rays, uint32_t n,
                               float4* hits, uint32_t* occ, uint32_t* err, unsigned long long* counters,
                               cudaStream_t s);
void launch_trace_brute(int kind, int traversal, bool any, const float4* prims, uint32_t n_prims,
                        const float4* rays, uint32_t n, float4* hits, uint32_t* occ,
                        cudaStream_t s);

// Collapsed 4-wide BVH over the same slot-ordered payload.
struct Bvh4View {
  const float4* nodes;    // 8 float4 per node
  const float4* prims;
  const uint32_t* order;
  const float* root;
  uint32_t n_binary;      // binary internal nodes (0: the root is one leaf)
  uint32_t n_slots;
};
void launch_trace_bvh4(int kind, bool any, const Bvh4View& v, const float4* rays, uint32_t n, float4* hits,
                       uint32_t* occ, uint32_t* err, cudaStream_t s, const uint32_t* perm = nullptr,
                       unsigned long long* counters = nullptr);

// Compressed 8-wide BVH over the same slot-ordered payload (layout in bvh8.cu).
struct Bvh8View {
  const float4* nodes;    // 8 float4 per node
  const float4* prims;
  const uint32_t* order;
  const float* root;
  uint32_t n_binary;      // binary internal nodes (0: the root is one leaf)
  uint32_t n_slots;
};
void launch_trace_bvh8(int kind, bool any, const Bvh8View& v, const float4* rays, uint32_t n, float4* hits,
                       uint32_t* occ, uint32_t* err, cudaStream_t s, const uint32_t* perm = nullptr,
                       unsigned long long* counters = nullptr);

// Rays of many BVH structures in one persistent launch (trace_batched.cu).
// views: device array of n_views structures (nodes = 4-wide nodes when
// width == 4); roff: device array of n_views + 1 ray offsets; work: one
// device word (zeroed by the launcher).
struct BatchedTrace {
  int kind = kTriangles;
  bool any = false;
  int width = 2;
  const Bvh2View* views = nullptr;
  const uint32_t* roff = nullptr;
  uint32_t n_views = 0;
  const float4* rays = nullptr;
  uint32_t n = 0;
  float4* hits = nullptr;
  uint32_t* occ = nullptr;
  uint32_t* work = nullptr;
  uint32_t* err = nullptr;
  const uint32_t* perm = nullptr;  // optional ray order: work index -> ray index
  bool unit = false;               // every structure's leaves hold one primitive (LBVH)
};
// block: 128 or 256 threads; deep: the deeper of the two stack sizes.
cudaError_t launch_trace_batched(const BatchedTrace& t, int block, int deep, cudaStream_t s);
int batched_stack_entries(int width, int deep);
// Per-scene ray order: keys (scene << 15 | octant | 12-bit origin cell) and
// vals = ray index for every ray; batch_key_bits = bits the keys use (more
// than 32 when there are over 2^17 structures: no ray order then).
int batch_key_bits(uint32_t n_views);
void launch_batch_ray_keys(const BatchedTrace& t, uint32_t* keys, uint32_t* vals, cudaStream_t s);

struct KdView {
  const int4* nodes;      // {word0, word1, word2, 0}
  const int32_t* prim_idx;
  const float4* prims;    // primitive-id order
  const float* root;      // 6 floats
  uint32_t n_nodes;
};
// work (optional): one word of scratch; the walk then runs as persistent warps.
void launch_trace_kd(int kind, int traversal, bool any, const KdView& v, const float4* rays,
                     uint32_t n, float4* hits, uint32_t* occ, uint32_t* err, cudaStream_t s, uint32_t* work = nullptr);

// --------------------------------------------------------- median BVH
struct MedianScratch;
// --------------------------------------------------------------- render
void launch_camera_rays_ref(uint32_t width, uint32_t height, uint32_t aa, float angle,
                            float aspect, const double* jitter, float4* rays, cudaStream_t s);
void launch_shade_ref(const float4* sph, const float* surface_rgb, const float4* rays,
                      const float4* hits, const uint32_t* kd_bits, uint32_t n, uint32_t aa,
                      float* rgb_sum, uint8_t* pixels, uint32_t npix, cudaStream_t s);

}  // namespace rq
