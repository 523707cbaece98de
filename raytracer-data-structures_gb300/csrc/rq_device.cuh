// Device-side building blocks shared by the engine's kernels.
//
// Arithmetic that decides a hit, a box test, a Morton code or a split is
// written with explicit round-to-nearest intrinsics (__fadd_rn, __fmul_rn,
// ...), never contracted into fused multiply-adds, so that every result is the
// IEEE single-precision value the reference's x86-64 build computes with the
// same operations in the same order.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace rq {

// ---------------------------------------------------------------- constants
constexpr float kEps = 1e-6f;             // Moller-Trumbore parallel reject, main.cpp:59
constexpr float kWiden = 0x1.000006p+0f;  // 1 + 2*gamma(3): far end of a robust slab test
constexpr uint32_t kMiss = 0xFFFFFFFFu;
constexpr int kStackSize = 64;            // traversal stack; Karras trees are at most 64 deep

// Device error word bits (context status).
constexpr uint32_t kErrStackOverflow = 1u << 0;
constexpr uint32_t kErrTimeout = 1u << 1;
constexpr uint32_t kErrBadInput = 1u << 2;
constexpr uint32_t kErrCorrupt = 1u << 3;  // a walk exceeded the steps a valid structure allows

struct F3 {
  float x, y, z;
};

__device__ __forceinline__ F3 sub_rn(F3 a, F3 b) {
  return {__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z)};
}
// geometry.h dotProduct: (x*v.x + y*v.y) + z*v.z
__device__ __forceinline__ float dot_rn(F3 a, F3 b) {
  return __fadd_rn(__fadd_rn(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)), __fmul_rn(a.z, b.z));
}
// geometry.h crossProduct
__device__ __forceinline__ F3 cross_rn(F3 a, F3 b) {
  return {__fsub_rn(__fmul_rn(a.y, b.z), __fmul_rn(a.z, b.y)),
          __fsub_rn(__fmul_rn(a.z, b.x), __fmul_rn(a.x, b.z)),
          __fsub_rn(__fmul_rn(a.x, b.y), __fmul_rn(a.y, b.x))};
}

// ------------------------------------------------------------- primitives

// Moller-Trumbore (main.cpp:138-161), no culling, EPS = 1e-6, hit accepted in
// (tmin, tmax).  p0 = (v0, id bits), p1 = (e1 = v1 - v0, 0), p2 = (e2, 0).
__device__ __forceinline__ bool tri_mt(const float4& p0, const float4& p1, const float4& p2, F3 o,
                                       F3 d, float tmin, float tmax, float& t, float& u,
                                       float& v) {
  F3 v0 = {p0.x, p0.y, p0.z}, e1 = {p1.x, p1.y, p1.z}, e2 = {p2.x, p2.y, p2.z};
  F3 pvec = cross_rn(d, e2);
  float det = dot_rn(e1, pvec);
  if (fabsf(det) < kEps) return false;
  float invDet = __frcp_rn(det);
  F3 tvec = sub_rn(o, v0);
  u = __fmul_rn(dot_rn(tvec, pvec), invDet);
  if (u < 0.f || u > 1.f) return false;
  F3 qvec = cross_rn(tvec, e1);
  v = __fmul_rn(dot_rn(d, qvec), invDet);
  if (v < 0.f || __fadd_rn(u, v) > 1.f) return false;
  t = __fmul_rn(dot_rn(e2, qvec), invDet);
  return t > tmin && t < tmax;
}

// Sphere::raySphereIntersect (accelerators.h:79-92).  s = (centre, radius).
__device__ __forceinline__ bool sphere_ref(const float4& s, F3 o, F3 d, float& t0, float& t1) {
  F3 c = {s.x, s.y, s.z};
  float r2 = __fmul_rn(s.w, s.w);
  F3 l = sub_rn(c, o);
  float tca = dot_rn(l, d);
  if (tca < 0.f) return false;
  float d2 = __fsub_rn(dot_rn(l, l), __fmul_rn(tca, tca));
  if (d2 > r2) return false;
  float thc = __fsqrt_rn(__fsub_rn(r2, d2));
  t0 = __fsub_rn(tca, thc);
  t1 = __fadd_rn(tca, thc);
  return true;
}

// castRay's selection for a sphere (main.cpp:349-351): t0, or t1 when t0 < 0.
// reference = true: accepted when t < best with no lower bound (castRay);
// otherwise the hit must lie in (tmin, best).
__device__ __forceinline__ bool sphere_closest(const float4& s, F3 o, F3 d, float tmin, float best,
                                               bool reference, float& t) {
  float t0, t1;
  if (!sphere_ref(s, o, d, t0, t1)) return false;
  t = t0 < 0.f ? t1 : t0;
  return reference ? (t < best) : (t > tmin && t < best);
}

// ---------------------------------------------------------------- boxes

// Per-ray constants of the engine's slab test: inv = 1/d (correctly rounded),
// noi = -(o * inv), and eps = 2^-21 * max over axes of the finite |o * inv|.
struct SlabRay {
  F3 inv, noi;
  float eps;
};
__device__ __forceinline__ SlabRay slab_ray(F3 o, F3 d) {
  SlabRay s;
  s.inv = {__frcp_rn(d.x), __frcp_rn(d.y), __frcp_rn(d.z)};
  float ox = __fmul_rn(o.x, s.inv.x), oy = __fmul_rn(o.y, s.inv.y), oz = __fmul_rn(o.z, s.inv.z);
  s.noi = {-ox, -oy, -oz};
  float m = 0.f;
  const float ax = fabsf(ox), ay = fabsf(oy), az = fabsf(oz);
  if (ax <= 3.402823466e38f) m = fmaxf(m, ax);
  if (ay <= 3.402823466e38f) m = fmaxf(m, ay);
  if (az <= 3.402823466e38f) m = fmaxf(m, az);
  s.eps = __fmul_rn(m, 0x1p-21f);
  return s;
}

// The fused plane distance fma(b, inv, -o*inv) needs o*inv finite.  A
// direction component that is zero (or so small that 1/d or o/d overflows)
// breaks it: inf - inf, or an infinite near distance, which rejects every
// box.  Such rays take the exact form instead (callers pick the form once per
// ray, so ordinary rays pay nothing): per axis (b - o) * inv, whose sign is
// the sign of b - o, and an axis along which the ray does not move (inv
// infinite) constrains nothing when lo <= o <= hi and rejects the box
// otherwise.
constexpr float kWidenExact = 0x1.00001p+0f;  // 1 + 2^-20: covers the roundings of (b - o) * inv
__device__ __forceinline__ bool zero_dir(const SlabRay& r) {
  return !(fabsf(r.noi.x) <= 3.402823466e38f && fabsf(r.noi.y) <= 3.402823466e38f &&
           fabsf(r.noi.z) <= 3.402823466e38f);
}
__device__ __forceinline__ void slab_axis_exact(float l, float h, float o, float inv, float& near, float& far) {
  const float a = __fsub_rn(l, o), b = __fsub_rn(h, o);
  if (fabsf(inv) > 3.402823466e38f) {  // the ray does not move along this axis
    const bool in = a <= 0.f && b >= 0.f;
    near = __int_as_float(in ? (int)0xFF800000u : 0x7F800000);
    far = __int_as_float(in ? 0x7F800000 : (int)0xFF800000u);
  } else {
    const float t0 = __fmul_rn(a, inv), t1 = __fmul_rn(b, inv);
    near = fminf(t0, t1);
    far = fmaxf(t0, t1);
  }
}

// Engine slab test on one box: plane distances b*inv - o*inv with one fused
// multiply-add each (EXACT: (b - o) * inv), NaN-ignoring min/max, clipped to
// [tmin, tfar].  The far end is widened by kWiden (relative rounding) and eps
// (the absolute error of the fused form, proportional to |o*inv|), so no box
// that the ray truly meets is rejected.
template <bool EXACT>
__device__ __forceinline__ bool slab_box(const SlabRay& r, F3 o, float lx, float hx, float ly, float hy, float lz,
                                         float hz, float tmin, float tfar, float& tnear) {
  float tn, tf;
  if (EXACT) {
    float nx, fx, ny, fy, nz, fz;
    slab_axis_exact(lx, hx, o.x, r.inv.x, nx, fx);
    slab_axis_exact(ly, hy, o.y, r.inv.y, ny, fy);
    slab_axis_exact(lz, hz, o.z, r.inv.z, nz, fz);
    tn = fmaxf(fmaxf(nx, ny), fmaxf(nz, tmin));
    tf = fminf(fminf(fx, fy), fminf(fz, tfar));
    tf = __fmaf_rn(tf, kWidenExact, r.eps);
  } else {
    const float tx0 = __fmaf_rn(lx, r.inv.x, r.noi.x), tx1 = __fmaf_rn(hx, r.inv.x, r.noi.x);
    const float ty0 = __fmaf_rn(ly, r.inv.y, r.noi.y), ty1 = __fmaf_rn(hy, r.inv.y, r.noi.y);
    const float tz0 = __fmaf_rn(lz, r.inv.z, r.noi.z), tz1 = __fmaf_rn(hz, r.inv.z, r.noi.z);
    tn = fmaxf(fmaxf(fminf(tx0, tx1), fminf(ty0, ty1)), fmaxf(fminf(tz0, tz1), tmin));
    tf = fminf(fminf(fmaxf(tx0, tx1), fmaxf(ty0, ty1)), fminf(fmaxf(tz0, tz1), tfar));
    tf = __fmaf_rn(tf, kWiden, r.eps);
  }
  tnear = tn;
  return tn <= tf;
}
// The fused form (rays without a zero direction component).
__device__ __forceinline__ bool slab_fast(const SlabRay& r, float lx, float hx, float ly, float hy, float lz,
                                          float hz, float tmin, float tfar, float& tnear) {
  return slab_box<false>(r, F3{0.f, 0.f, 0.f}, lx, hx, ly, hy, lz, hz, tmin, tfar, tnear);
}
// Either form, chosen per call (kernels whose lanes walk together).
__device__ __forceinline__ bool slab_any(bool exact, const SlabRay& r, F3 o, float lx, float hx, float ly, float hy,
                                         float lz, float hz, float tmin, float tfar, float& tnear) {
  return exact ? slab_box<true>(r, o, lx, hx, ly, hy, lz, hz, tmin, tfar, tnear)
               : slab_box<false>(r, o, lx, hx, ly, hy, lz, hz, tmin, tfar, tnear);
}
// Exit distance of the same box (before widening).
template <bool EXACT>
__device__ __forceinline__ float slab_exit(const SlabRay& r, F3 o, float lx, float hx, float ly, float hy, float lz,
                                           float hz, float tfar) {
  if (EXACT) {
    float nx, fx, ny, fy, nz, fz;
    slab_axis_exact(lx, hx, o.x, r.inv.x, nx, fx);
    slab_axis_exact(ly, hy, o.y, r.inv.y, ny, fy);
    slab_axis_exact(lz, hz, o.z, r.inv.z, nz, fz);
    return fminf(fminf(fx, fy), fminf(fz, tfar));
  }
  const float tx0 = __fmaf_rn(lx, r.inv.x, r.noi.x), tx1 = __fmaf_rn(hx, r.inv.x, r.noi.x);
  const float ty0 = __fmaf_rn(ly, r.inv.y, r.noi.y), ty1 = __fmaf_rn(hy, r.inv.y, r.noi.y);
  const float tz0 = __fmaf_rn(lz, r.inv.z, r.noi.z), tz1 = __fmaf_rn(hz, r.inv.z, r.noi.z);
  return fminf(fminf(fmaxf(tx0, tx1), fmaxf(ty0, ty1)), fminf(fmaxf(tz0, tz1), tfar));
}

// boundingBoxIntersection (accelerators.h:628-666): division per axis, swap,
// no clipping to the ray interval.
__device__ __forceinline__ bool box_ref(F3 o, F3 d, float lx, float hx, float ly, float hy,
                                        float lz, float hz, float& tMin, float& tMax) {
  float tmin = __fdiv_rn(__fsub_rn(lx, o.x), d.x);
  float tmax = __fdiv_rn(__fsub_rn(hx, o.x), d.x);
  if (tmin > tmax) { float s = tmin; tmin = tmax; tmax = s; }
  float tymin = __fdiv_rn(__fsub_rn(ly, o.y), d.y);
  float tymax = __fdiv_rn(__fsub_rn(hy, o.y), d.y);
  if (tymin > tymax) { float s = tymin; tymin = tymax; tymax = s; }
  if ((tmin > tymax) || (tymin > tmax)) return false;
  if (tymin > tmin) tmin = tymin;
  if (tymax < tmax) tmax = tymax;
  float tzmin = __fdiv_rn(__fsub_rn(lz, o.z), d.z);
  float tzmax = __fdiv_rn(__fsub_rn(hz, o.z), d.z);
  if (tzmin > tzmax) { float s = tzmin; tzmin = tzmax; tzmax = s; }
  if ((tmin > tzmax) || (tzmin > tmax)) return false;
  if (tzmin > tmin) tmin = tzmin;
  if (tzmax < tmax) tmax = tzmax;
  tMin = tmin;
  tMax = tmax;
  return true;
}

// --------------------------------------------------- ordered float atomics
// Monotone map float -> int32 so that atomicMin/atomicMax on ints order floats.
__device__ __forceinline__ int32_t float_to_ordered(float f) {
  int32_t i = __float_as_int(f);
  return i >= 0 ? i : (i ^ 0x7FFFFFFF);
}
__device__ __forceinline__ float ordered_to_float(int32_t i) {
  return __int_as_float(i >= 0 ? i : (i ^ 0x7FFFFFFF));
}
__host__ __device__ inline int32_t ordered_pos_inf() { return 0x7F800000; }
__host__ __device__ inline int32_t ordered_neg_inf() { return (int32_t)(0xFF800000u ^ 0x7FFFFFFFu); }

// ----------------------------------------------------------- Morton codes
// expandBits (accelerators.h:374-381)
__device__ __forceinline__ uint32_t expand_bits(uint32_t v) {
  v = (v * 0x00010001u) & 0xFF0000FFu;
  v = (v * 0x00000101u) & 0x0F00F00Fu;
  v = (v * 0x00000011u) & 0xC30C30C3u;
  v = (v * 0x00000005u) & 0x49249249u;
  return v;
}
// morton3D (accelerators.h:385-394): clamp(x*1024, 0, 1023), truncate,
// interleave with x in the most significant bit of each triple.
__device__ __forceinline__ uint32_t morton3d(float x, float y, float z) {
  x = fminf(fmaxf(__fmul_rn(x, 1024.0f), 0.0f), 1023.0f);
  y = fminf(fmaxf(__fmul_rn(y, 1024.0f), 0.0f), 1023.0f);
  z = fminf(fmaxf(__fmul_rn(z, 1024.0f), 0.0f), 1023.0f);
  return expand_bits(__float2uint_rz(x)) * 4u + expand_bits(__float2uint_rz(y)) * 2u +
         expand_bits(__float2uint_rz(z));
}

// Bounded spin: returns false once `limit` polls have passed.
template <typename Pred>
__device__ __forceinline__ bool spin_until(Pred pred, uint32_t limit) {
  for (uint32_t i = 0; i < limit; ++i) {
    if (pred()) return true;
    __nanosleep(i < 64 ? 20 : 200);
  }
  return pred();
}

// Largest k with off[k] <= x (off has n + 1 non-decreasing entries, off[0] = 0 <= x < off[n]).
__device__ __forceinline__ uint32_t segment_of(const uint32_t* __restrict__ off, uint32_t n, uint32_t x) {
  uint32_t lo = 0, hi = n;  // answer in [lo, hi)
  while (hi - lo > 1) {
    uint32_t mid = (lo + hi) >> 1;
    if (__ldg(off + mid) <= x) lo = mid;
    else hi = mid;
  }
  return lo;
}

}  // namespace rq
