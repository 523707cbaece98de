// Morton codes over primitive centroids (accelerators.h:374-394, 575-580),
// fused with the radix sort's digit histogram so the codes are read once.
#include <atomic>

#include "lbvh_device.cuh"

namespace rq {
namespace {

constexpr int kThreads = 256;

__global__ void k_init_bounds(int32_t* lohi) {
  int t = threadIdx.x;
  if (t < 3) lohi[t] = ordered_pos_inf();
  else if (t < 6) lohi[t] = ordered_neg_inf();
}

// Box of n points with `stride` floats between consecutive points.
__global__ void __launch_bounds__(kThreads) k_point_bounds(const float* __restrict__ pts, uint32_t n,
                                                           uint32_t stride, int32_t* lohi) {
  float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float* p = pts + (size_t)i * stride;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      float v = __ldg(p + k);
      lo[k] = fminf(lo[k], v);
      hi[k] = fmaxf(hi[k], v);
    }
  }
#pragma unroll
  for (int k = 0; k < 3; ++k)
    for (int o = 16; o > 0; o >>= 1) {
      lo[k] = fminf(lo[k], __shfl_xor_sync(0xffffffffu, lo[k], o));
      hi[k] = fmaxf(hi[k], __shfl_xor_sync(0xffffffffu, hi[k], o));
    }
  __shared__ float s[kThreads / 32][6];
  int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0)
    for (int k = 0; k < 3; ++k) { s[w][k] = lo[k]; s[w][3 + k] = hi[k]; }
  __syncthreads();
  if (threadIdx.x < 6) {
    int k = threadIdx.x;
    float v = s[0][k];
    for (int q = 1; q < kThreads / 32; ++q) v = k < 3 ? fminf(v, s[q][k]) : fmaxf(v, s[q][k]);
    if (k < 3) atomicMin(&lohi[k], float_to_ordered(v));
    else atomicMax(&lohi[k], float_to_ordered(v));
  }
}

struct SharedHist {
  uint32_t h[4][256];
};

__device__ __forceinline__ void hist_zero(SharedHist& sh) {
  for (int i = threadIdx.x; i < 1024; i += blockDim.x) (&sh.h[0][0])[i] = 0;
}
// One shared atomic per distinct digit value in the warp (the upper digits
// of spatially sorted codes repeat across most lanes).  Called by whole
// warps: `active` is the lanes holding a code.
__device__ __forceinline__ void hist_add(SharedHist& sh, uint32_t code, bool active) {
  const uint32_t lanes = __ballot_sync(0xffffffffu, active);
  if (!active) return;
  const uint32_t lane = threadIdx.x & 31u;
#pragma unroll
  for (int p = 0; p < 4; ++p) {
    const uint32_t d = (code >> (8 * p)) & 255u;
    const uint32_t same = __match_any_sync(lanes, d);
    if ((same & ((1u << lane) - 1u)) == 0u) atomicAdd(&sh.h[p][d], (uint32_t)__popc(same));
  }
}
__device__ __forceinline__ void hist_flush(SharedHist& sh, uint32_t* hist) {
  for (int i = threadIdx.x; i < 1024; i += blockDim.x) {
    uint32_t v = (&sh.h[0][0])[i];
    if (v) atomicAdd(&hist[i], v);
  }
}

// 16-byte copies of the vertices and triangles (w = 0).
__global__ void __launch_bounds__(kThreads) k_pack_tris(const float* __restrict__ verts, uint32_t nv,
                                                        const uint32_t* __restrict__ idx, uint32_t nt,
                                                        float4* __restrict__ verts4, uint4* __restrict__ idx4) {
  const uint32_t m = nv > nt ? nv : nt;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
    if (i < nv)
      verts4[i] = make_float4(__ldg(verts + 3 * (size_t)i), __ldg(verts + 3 * (size_t)i + 1),
                              __ldg(verts + 3 * (size_t)i + 2), 0.f);
    if (idx4 && i < nt)
      idx4[i] = make_uint4(__ldg(idx + 3 * (size_t)i), __ldg(idx + 3 * (size_t)i + 1), __ldg(idx + 3 * (size_t)i + 2), 0u);
  }
}

// Centroid ((v0 + v1) + v2) / 3 per axis, then scene-box normalisation.
__global__ void __launch_bounds__(kThreads) k_morton_tris(const float4* __restrict__ verts,
                                                          const uint4* __restrict__ idx,
                                                          uint32_t nt, int mode, const int32_t* __restrict__ lohi,
                                                          uint32_t* __restrict__ keys,
                                                          uint32_t* __restrict__ vals,
                                                          uint32_t* __restrict__ hist) {
  __shared__ SharedHist sh;
  __shared__ float s_lo[3], s_ext[3];
  if (hist) hist_zero(sh);
  if (threadIdx.x == 0) {
    bounds_from(lohi, s_lo, s_ext);
    if (mode == RQ_MORTON_SCENE_CUBE) cube_extent(s_ext);
  }
  __syncthreads();
  float lo[3] = {s_lo[0], s_lo[1], s_lo[2]}, ext[3] = {s_ext[0], s_ext[1], s_ext[2]};
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t i0 = blockIdx.x * blockDim.x; i0 < nt; i0 += stride) {  // whole warps run every round
    const uint32_t i = i0 + threadIdx.x;
    const bool live = i < nt;
    uint32_t code = 0;
    if (live) {
      code = code_scene(tri_centroid(verts, idx, i), lo, ext);
      keys[i] = code;
      vals[i] = i;
    }
    if (hist) hist_add(sh, code, live);
  }
  if (hist) {
    __syncthreads();
    hist_flush(sh, hist);
  }
}

__global__ void __launch_bounds__(kThreads) k_morton_spheres(const float4* __restrict__ sph, uint32_t n,
                                                             int mode, const int32_t* __restrict__ lohi,
                                                             uint32_t* __restrict__ keys,
                                                             uint32_t* __restrict__ vals,
                                                             uint32_t* __restrict__ hist) {
  __shared__ SharedHist sh;
  __shared__ float s_lo[3], s_ext[3];
  if (hist) hist_zero(sh);
  if (threadIdx.x == 0 && mode != RQ_MORTON_REFERENCE) {
    bounds_from(lohi, s_lo, s_ext);
    if (mode == RQ_MORTON_SCENE_CUBE) cube_extent(s_ext);
  }
  __syncthreads();
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t i0 = blockIdx.x * blockDim.x; i0 < n; i0 += stride) {  // whole warps run every round
    const uint32_t i = i0 + threadIdx.x;
    const bool live = i < n;
    uint32_t code = 0;
    if (live) {
      float4 s = __ldg(sph + i);
      if (mode == RQ_MORTON_REFERENCE) {
        // (center + 30) / 1000, accelerators.h:577
        code = morton3d(__fdiv_rn(__fadd_rn(s.x, 30.f), 1000.f), __fdiv_rn(__fadd_rn(s.y, 30.f), 1000.f),
                        __fdiv_rn(__fadd_rn(s.z, 30.f), 1000.f));
      } else {
        code = code_scene({s.x, s.y, s.z}, s_lo, s_ext);
      }
      keys[i] = code;
      vals[i] = i;
    }
    if (hist) hist_add(sh, code, live);
  }
  if (hist) {
    __syncthreads();
    hist_flush(sh, hist);
  }
}

int grid_for(uint32_t n) {
  uint32_t g = (n + kThreads - 1) / kThreads;
  return (int)(g < 1 ? 1 : (g > 4096 ? 4096 : g));
}

// Morton kernels: a few blocks per SM, each looping over many primitives, so
// that each block's shared histogram flushes once for thousands of codes
// (one block per 256 codes meant over a million global atomics on 1024 bins).
int grid_for_hist(uint32_t n) {
  const int g = grid_for(n), cap = 4 * device_sm_count();
  return g < cap ? g : cap;
}

}  // namespace

int device_sm_count() {
  static std::atomic<int> cache[64];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 1;
  int v = cache[dev & 63].load();
  if (v == 0) {
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0) v = 1;
    cache[dev & 63].store(v);
  }
  return v;
}

void launch_init_bounds(int32_t* lohi, cudaStream_t s) {
  count_launch();
  k_init_bounds<<<1, 32, 0, s>>>(lohi);
}

void launch_point_bounds(const float* pts, uint32_t n, uint32_t stride, int32_t* lohi,
                         cudaStream_t s) {
  if (n == 0) return;
  count_launch();
  k_point_bounds<<<grid_for(n) > 1024 ? 1024 : grid_for(n), kThreads, 0, s>>>(pts, n, stride, lohi);
}

void launch_pack_tris(const float* verts, uint32_t nv, const uint32_t* idx, uint32_t nt, float4* verts4,
                      uint4* idx4, cudaStream_t s) {
  const uint32_t m = nv > nt ? nv : nt;
  if (m == 0) return;
  count_launch();
  k_pack_tris<<<grid_for(m), kThreads, 0, s>>>(verts, nv, idx, idx4 ? nt : 0, verts4, idx4);
}

void launch_morton_tris(const float4* verts, const uint4* idx, uint32_t nt, int mode, const int32_t* lohi,
                        uint32_t* keys, uint32_t* vals, uint32_t* hist, cudaStream_t s) {
  if (nt == 0) return;
  count_launch();
  k_morton_tris<<<hist ? grid_for_hist(nt) : grid_for(nt), kThreads, 0, s>>>(verts, idx, nt, mode, lohi, keys,
                                                                             vals, hist);
}

void launch_morton_spheres(const float4* sph, uint32_t n, int mode, const int32_t* lohi,
                           uint32_t* keys, uint32_t* vals, uint32_t* hist, cudaStream_t s) {
  if (n == 0) return;
  count_launch();
  k_morton_spheres<<<hist ? grid_for_hist(n) : grid_for(n), kThreads, 0, s>>>(sph, n, mode, lohi, keys, vals, hist);
}

}  // namespace rq
