// Persistent, work-stealing traversal of many structures in one launch.
//
// Rays of all structures lie back to back; ray_off (n_views + 1 entries)
// gives each structure's range.  The grid is sized to what the SMs hold at
// once; each warp takes blocks of 256 consecutive rays from a global counter
// until none are left, so long and short structures, coherent and incoherent
// rays share the GPU without a tail per structure.  Each ray finds its
// structure by binary search over ray_off and walks it with the same FAST
// walk as a one-structure query (identical results).
//
// Launch shapes (block size, traversal stack depth) are template choices that
// rq_plan_create times on the caller's rays; a stack too shallow for a tree
// reports RQ_ERROR_STACK_OVERFLOW and the tuner drops that shape.
#include "trace_device.cuh"

namespace rq {
namespace {

constexpr uint32_t kGrab = 256;  // rays a warp takes per counter access (8 passes of 32)

// UNIT: every structure of the launch has single-primitive leaves (batched
// LBVH builds): 4-byte stack entries.
template <int KIND, bool ANY, int W, int STACK, int BLOCK, bool UNIT = false>
__global__ void __launch_bounds__(BLOCK) k_trace_batched(const Bvh2View* __restrict__ views,
                                                         const uint32_t* __restrict__ roff, uint32_t n_views,
                                                         const float4* __restrict__ rays, uint32_t n,
                                                         float4* __restrict__ hits, uint32_t* __restrict__ occ,
                                                         uint32_t* __restrict__ work, uint32_t* err,
                                                         const uint32_t* __restrict__ perm) {
  const uint32_t lane = threadIdx.x & 31;
  for (;;) {
    uint32_t base = 0;
    if (lane == 0) base = atomicAdd(work, kGrab);
    base = __shfl_sync(0xffffffffu, base, 0);
    if (base >= n) return;  // the whole warp leaves together
#pragma unroll 1
    for (uint32_t sub = 0; sub < kGrab; sub += 32) {
      const uint32_t w = base + sub + lane;  // work index; the ray itself through perm
      const uint32_t r = (perm && w < n) ? __ldg(perm + w) : w;
      bool occluded = false;
      if (w < n) {
        const Bvh2View v = views[segment_of(roff, n_views, r)];
        const Ray ray = load_ray(rays, r);
        Closest c = {ray.tmax, kMiss, 0.f, 0.f};
        uint32_t visits = 0, tests = 0;
        if (W == 4) {
          const Bvh4View v4{v.nodes, v.prims, v.order, v.root, v.n_internal, v.n_slots};
          occluded = walk_bvh4<KIND, ANY, false, STACK>(v4, ray, c, visits, tests, err);
        } else if (W == 8) {
          const Bvh8View v8{v.nodes, v.prims, v.order, v.root, v.n_internal, v.n_slots};
          occluded = walk_bvh8<KIND, ANY, false, STACK>(v8, ray, c, visits, tests, err);
        } else {
          occluded = walk_bvh2<KIND, ANY, false, STACK, UNIT>(v, ray, c, visits, tests, err);
        }
        if (!ANY) store_hit(hits, r, c);
      }
      if (ANY) {
        if (perm) {  // bits of scattered rays: set one by one in the zeroed words
          if (occluded) atomicOr(occ + (r >> 5), 1u << (r & 31));
        } else {
          const uint32_t bits = __ballot_sync(0xffffffffu, occluded);
          if (lane == 0 && base + sub < n) occ[(base + sub) >> 5] = bits;
        }
      }
    }
  }
}

template <int KIND, bool ANY, int W, int STACK, int BLOCK>
cudaError_t launch_shape(const BatchedTrace& t, cudaStream_t s) {
  auto k = (W == 2 && t.unit) ? k_trace_batched<KIND, ANY, W, STACK, BLOCK, true>
                              : k_trace_batched<KIND, ANY, W, STACK, BLOCK, false>;
  int per_sm = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, BLOCK, 0);
  if (e != cudaSuccess) return e;
  int sms = 0;
  int dev = 0;
  if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
  if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
  const uint64_t want_warps = ((uint64_t)t.n + kGrab - 1) / kGrab;
  uint64_t blocks = (uint64_t)(per_sm > 0 ? per_sm : 1) * sms;
  const uint64_t enough = (want_warps * 32 + BLOCK - 1) / BLOCK;  // no more warps than work blocks
  if (blocks > enough) blocks = enough;
  if (blocks < 1) blocks = 1;
  if ((e = cudaMemsetAsync(t.work, 0, 4, s)) != cudaSuccess) return e;
  if (ANY && t.perm && (e = cudaMemsetAsync(t.occ, 0, (size_t)((t.n + 31) / 32) * 4, s)) != cudaSuccess) return e;
  count_launch();
  k<<<(unsigned)blocks, BLOCK, 0, s>>>(t.views, t.roff, t.n_views, t.rays, t.n, t.hits, t.occ, t.work, t.err,
                                       t.perm);
  return cudaGetLastError();
}

// Per-scene ray order keys: (scene << 15) | octant of the direction (3
// bits) | 12-bit Morton code of the origin, quantised to 16 cells per axis in
// the scene's root box.  Sorted stably, rays stay grouped by scene and, within
// a scene, by direction octant and origin cell (the original order within a
// cell).
__device__ __forceinline__ uint32_t spread4(uint32_t v) {  // 4 bits -> every third bit
  v &= 15u;
  return (v & 1u) | ((v & 2u) << 2) | ((v & 4u) << 4) | ((v & 8u) << 6);
}

__global__ void __launch_bounds__(256) k_batch_ray_keys(const Bvh2View* __restrict__ views,
                                                        const uint32_t* __restrict__ roff, uint32_t n_views,
                                                        const float4* __restrict__ rays, uint32_t n,
                                                        uint32_t* __restrict__ keys, uint32_t* __restrict__ vals) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t sc = segment_of(roff, n_views, i);
  const float* root = views[sc].root;
  const float4 a = __ldg(rays + 2 * (size_t)i), b = __ldg(rays + 2 * (size_t)i + 1);
  const float o[3] = {a.x, a.y, a.z};
  uint32_t q[3];
  for (int k = 0; k < 3; ++k) {
    const float lo = __ldg(root + k), ext = __ldg(root + 3 + k) - lo;
    float u = ext > 0.f ? (o[k] - lo) / ext : 0.f;
    u = fminf(fmaxf(u * 16.f, 0.f), 15.f);
    q[k] = (uint32_t)u;
  }
  const uint32_t oct = (b.x < 0.f ? 4u : 0u) | (b.y < 0.f ? 2u : 0u) | (b.z < 0.f ? 1u : 0u);
  const uint32_t morton = (spread4(q[0]) << 2) | (spread4(q[1]) << 1) | spread4(q[2]);
  keys[i] = (sc << 15) | (oct << 12) | morton;
  vals[i] = i;
}

template <int KIND, bool ANY, int W>
cudaError_t dispatch_shape(const BatchedTrace& t, int block, int deep, cudaStream_t s) {
  constexpr int kShallow = W == 4 ? 48 : W == 8 ? 16 : 32, kDeep = W == 4 ? 96 : W == 8 ? 32 : 64;
  if (block == 256) {
    return deep ? launch_shape<KIND, ANY, W, kDeep, 256>(t, s) : launch_shape<KIND, ANY, W, kShallow, 256>(t, s);
  }
  return deep ? launch_shape<KIND, ANY, W, kDeep, 128>(t, s) : launch_shape<KIND, ANY, W, kShallow, 128>(t, s);
}

template <int KIND, bool ANY>
cudaError_t dispatch_width(const BatchedTrace& t, int block, int deep, cudaStream_t s) {
  if (t.width == 8) return dispatch_shape<KIND, ANY, 8>(t, block, deep, s);
  return t.width == 4 ? dispatch_shape<KIND, ANY, 4>(t, block, deep, s) : dispatch_shape<KIND, ANY, 2>(t, block, deep, s);
}

}  // namespace

int batched_stack_entries(int width, int deep) {
  return width == 4 ? (deep ? 96 : 48) : width == 8 ? (deep ? 32 : 16) : (deep ? 64 : 32);
}

int batch_key_bits(uint32_t n_views) {
  int b = 0;
  while (b < 32 && ((uint64_t)1 << b) < n_views) ++b;
  return 15 + b;
}

void launch_batch_ray_keys(const BatchedTrace& t, uint32_t* keys, uint32_t* vals, cudaStream_t s) {
  if (t.n == 0) return;
  count_launch();
  k_batch_ray_keys<<<(t.n + 255) / 256, 256, 0, s>>>(t.views, t.roff, t.n_views, t.rays, t.n, keys, vals);
}

cudaError_t launch_trace_batched(const BatchedTrace& t, int block, int deep, cudaStream_t s) {
  if (t.n == 0) return cudaSuccess;
  if (block != 128 && block != 256) return cudaErrorInvalidValue;
  if (t.kind == kTriangles)
    return t.any ? dispatch_width<kTriangles, true>(t, block, deep, s) : dispatch_width<kTriangles, false>(t, block, deep, s);
  return t.any ? dispatch_width<kSpheres, true>(t, block, deep, s) : dispatch_width<kSpheres, false>(t, block, deep, s);
}

}  // namespace rq
