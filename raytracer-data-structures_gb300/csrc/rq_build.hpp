// Build orchestration shared by the C ABI: device buffers of a structure,
// reusable build scratch, and the per-type build / query entry points.
#pragma once
#include <vector>

#include "rq_internal.hpp"

namespace rq {

struct SceneView {
  int kind = kTriangles;
  uint32_t n = 0;   // primitives
  uint32_t nv = 0;  // vertices
  const float* verts = nullptr;
  const uint32_t* idx = nullptr;
  const float4* sph = nullptr;
  const float4* verts4 = nullptr;  // 16-byte copies of verts and idx (triangle scenes)
  const uint4* idx4 = nullptr;
};

// Device memory held by one acceleration structure.
struct AccelBuffers {
  DevBuf nodes;        // BVH2 nodes, 64 B each
  DevBuf prims;        // BVH2: payload in slot order; KD / NONE: payload in id order
  DevBuf order;        // BVH2: slot -> primitive id
  DevBuf codes;        // LBVH: sorted Morton codes
  DevBuf root;         // 8 floats: root box (min xyz, max xyz)
  DevBuf kd_nodes;     // KD: int4 per node
  DevBuf kd_idx;       // KD: primitive indices
  DevBuf nodes4;       // wide nodes, 128 B each: collapsed 4-wide (node_width 4) or compressed 8-wide (8)
  uint32_t n_nodes = 0;
  uint32_t n_slots = 0;
  uint32_t max_depth = 0;
  uint32_t node_width = 2;  // BVH2 structures: 2, or 4 / 8 when nodes4 holds a wide copy
  uint32_t n4_cap = 0;      // bound of the 4-wide node count (exact count: root word 6)
  bool unit_leaves = false; // every BVH2 leaf holds one primitive (LBVH builds)
  void release() {
    nodes.release(); prims.release(); order.release(); codes.release(); root.release();
    kd_nodes.release(); kd_idx.release(); nodes4.release();
    n_nodes = n_slots = max_depth = n4_cap = 0;
    node_width = 2;
    unit_leaves = false;
  }
  size_t device_bytes() const {
    return nodes.cap + prims.cap + order.cap + codes.cap + root.cap + kd_nodes.cap + kd_idx.cap + nodes4.cap;
  }
};

// Scratch reused across builds of one context (grow-only).
struct BuildScratch {
  DevBuf keys_alt, vals_alt;  // radix sort ping-pong
  DevBuf zero;                // [hist 1024][counters 16][look-back status][refit flags]: zeroed per build
  DevBuf parent;              // Karras parent links
  DevBuf mark;                // refit top nodes: per-node marks, then the top list
  DevBuf lohi;                // ordered-int scene box
  DevBuf keys, vals;          // generic sort input
  DevBuf m0, m1, m2, m3, m4, m5, m6, m7;  // median / KD working arrays
  DevBuf kd_refs;             // KD: next level's primitive references
  DevBuf work;                // work counter of lane-refill traversal
  DevBuf top;                 // top-level node copy of RQ_SCHEDULING_SHARED_TOP queries
  DevBuf exact;               // rays that need the exact box test, set aside by FAST queries
  DevBuf heights;             // LBVH treelet restructuring: internal node heights (bytes)
  const uint32_t* stall = nullptr;  // sort test hook (SortScratch::stall); null in normal use
  void release() {
    work.release();
    top.release();
    exact.release();
    heights.release();
    keys_alt.release(); vals_alt.release(); zero.release(); parent.release(); mark.release(); lohi.release();
    keys.release(); vals.release();
    m0.release(); m1.release(); m2.release(); m3.release(); m4.release(); m5.release(); m6.release(); m7.release();
    kd_refs.release();
  }
};

struct BuildResult {
  rq_status_t status = RQ_SUCCESS;
  cudaError_t cuda = cudaSuccess;
  const char* what = nullptr;
  static BuildResult cuda_error(cudaError_t e, const char* w) {
    BuildResult r;
    r.cuda = e;
    r.what = w;
    return r;
  }
  static BuildResult error(rq_status_t s, const char* w) {
    BuildResult r;
    r.status = s;
    r.what = w;
    return r;
  }
  bool ok() const { return status == RQ_SUCCESS && cuda == cudaSuccess; }
};

BuildResult build_accel(int type, const SceneView& s, const rq_settings_t& settings, AccelBuffers& a,
                        BuildScratch& sc, uint32_t* err, cudaStream_t st);
// Morton codes in primitive order (vals = identity); hist optional.
BuildResult morton_codes(const SceneView& s, int mode, uint32_t* codes, uint32_t* vals,
                         uint32_t* hist, BuildScratch& sc, cudaStream_t st);
// In-place stable sort; compute_hist = false when sc.zero's histogram was
// already filled (fused Morton kernel) and zeroed state is in place.
BuildResult sort_pairs(uint32_t* keys, uint32_t* vals, uint32_t n, int passes, bool compute_hist,
                       BuildScratch& sc, uint32_t* err, cudaStream_t st);

// Builders living in their own translation units.
BuildResult build_median_bvh(const SceneView& s, AccelBuffers& a, BuildScratch& sc, uint32_t* err,
                             cudaStream_t st);
BuildResult build_kd_tree(const SceneView& s, int max_depth, AccelBuffers& a, BuildScratch& sc,
                          uint32_t* err, cudaStream_t st);
// Collapsed 4-wide copy of the binary nodes in a.nodes (a.nodes4; node count
// into the root buffer's word 6).
uint32_t bvh4_node_cap(uint32_t n_internal);
BuildResult collapse_bvh4(AccelBuffers& a, BuildScratch& sc, uint32_t* err, cudaStream_t st);
// Compressed 8-wide copy of the binary nodes (in a.nodes4, 128 B per node;
// node count in root word 6; bvh8.cu).
uint32_t bvh8_node_cap(uint32_t n_internal);
BuildResult collapse_bvh8(AccelBuffers& a, BuildScratch& sc, uint32_t* err, cudaStream_t st);

// ---------------------------------------------------------- batched build
struct BatchDesc {  // device copy per scene: its geometry
  const float* verts;
  const uint32_t* idx;
  const float4* sph;
};
// All arrays of a batch of LBVH structures, back to back (see batch.cu).
struct BatchStore {
  int kind = kTriangles;
  uint32_t n_scenes = 0;
  std::vector<uint32_t> poff, voff;  // n + 1 prefix sums of primitives / points
  std::vector<BatchDesc> host_desc;
  DevBuf desc, offs, lohi, nodes, prims, order, codes, roots, parent, keys, keys_alt, vals, vals_alt, zero;
  size_t zero_words = 0;
  cudaError_t allocate();
  cudaError_t upload_tables(cudaStream_t st);
  // Borrowed views of scene s's arrays (what a single build would own).
  void view(uint32_t s, AccelBuffers& a) const;
  ~BatchStore() { release(); }
  void release() {
    desc.release(); offs.release(); lohi.release(); nodes.release(); prims.release(); order.release();
    codes.release(); roots.release(); parent.release(); keys.release(); keys_alt.release(); vals.release();
    vals_alt.release(); zero.release();
  }
};
int batch_sort_passes(uint32_t n_scenes);
// One pass of batched kernels over every scene (no allocation, no host sync).
BuildResult build_batch(BatchStore& b, int morton_mode, uint32_t* err, cudaStream_t st);

struct QueryTarget {
  const float4* rays = nullptr;
  uint32_t n = 0;
  float4* hits = nullptr;
  uint32_t* occ = nullptr;
  bool small_stack = false;  // test hook: FAST BVH2 walk with a traversal stack of kDebugStack entries
  uint32_t* exact = nullptr;  // n + 2 words: exact-ray count, work counter, rays set aside (launch_trace_bvh2)
  uint32_t* work = nullptr;   // one word: the work counter of the persistent-warp KD walk (launch_trace_kd)
};
// Batches of at least this many rays are reordered when settings.ray_sort asks.
constexpr uint32_t kRaySortMin = 65536;
struct QueryTarget;
BuildResult launch_query_sorted(int type, const SceneView& s, const AccelBuffers& a, const rq_settings_t& cfg,
                                bool any, const QueryTarget& q, BuildScratch& sc, uint32_t* err, cudaStream_t st);
void launch_query(int type, const SceneView& s, const AccelBuffers& a, int traversal, bool any,
                  const QueryTarget& q, uint32_t* err, cudaStream_t st);

uint64_t launch_total();
BuildResult trace_counted(int type, const SceneView& s, const AccelBuffers& a, bool any, const QueryTarget& q,
                          unsigned long long* counters, uint32_t* err, cudaStream_t st);

void launch_validate(const float* verts, uint32_t nv, const uint32_t* idx, uint32_t nt,
                     const float4* sph, uint32_t n, uint32_t* err, cudaStream_t st);

// Working arrays of rq_render (grow-only, per context).
struct RenderScratch {
  DevBuf rays, shadow, hits, cw, pend, bits, out, counters;
  DevBuf list_a, list_b, list_s, list_n;  // live-sample lists of the compacting render
  void release() {
    rays.release(); shadow.release(); hits.release(); cw.release(); pend.release(); bits.release();
    out.release(); counters.release();
    list_a.release(); list_b.release(); list_s.release(); list_n.release();
  }
};
// Wavefront render of `view` into device buffers pixels (3 B per pixel) and
// rgb (3 floats per pixel, may be null); counters (2 x u64, device) gain the
// shadow and mirror rays emitted.  *status reports engine errors.
cudaError_t render_view(int type, const SceneView& s, const AccelBuffers& a, const rq_settings_t& cfg,
                        const rq_view_t& view, float tan_half, RenderScratch& rs, BuildScratch& sc,
                        uint8_t* pixels, float* rgb, unsigned long long* counters, uint32_t* err,
                        cudaStream_t st, rq_status_t* status);
cudaError_t render_reference(int type, const SceneView& s, const AccelBuffers& a,
                             const rq_settings_t& settings, float angle, float aspect,
                             const double* jitter, bool jitter_on_device, const float* surface_rgb_host,
                             DevBuf& stage_a, DevBuf& stage_b, DevBuf& stage_c,
                             uint8_t* pixels_host, float* rgb_sum_host, uint32_t* err,
                             cudaStream_t st);

}  // namespace rq
