// Per-sample device code of the render step, shared by rq_render
// (view_render.cu) and the serving loop (serve.cu) so that a served request
// produces exactly rq_render's pixels for the same view.
#pragma once
#include "rq_build.hpp"
#include "rq_device.cuh"

namespace rq {

struct V3 {
  float x, y, z;
};
__device__ __forceinline__ V3 v3add(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ V3 v3sub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ V3 v3mul(V3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ float v3dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ V3 v3cross(V3 a, V3 b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ V3 v3norm(V3 a) {
  float n2 = v3dot(a, a);
  if (!(n2 > 0.f)) return a;
  float inv = 1.0f / sqrtf(n2);
  return v3mul(a, inv);
}

// splitmix64 finaliser (Steele, Lea, Flood 2014) as a counter-based generator.
__device__ __forceinline__ uint64_t mix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}
// Uniform in [0, 1) with 24 bits: exact in float.
__device__ __forceinline__ float jitter01(uint64_t seed, uint64_t sample, uint32_t dim) {
  uint64_t h = mix64(seed ^ mix64(sample * 2u + dim));
  return (float)(uint32_t)(h >> 40) * 0x1p-24f;
}

struct ViewDev {
  V3 eye, target, up, light, albedo, bg;
  float tan_half, aspect, ambient, mirror, bias;
  uint32_t width, height, spp, x0, y0, ww, wh, bounces;
  uint64_t seed;
};

__device__ __forceinline__ void store_ray(float4* rays, uint64_t r, V3 o, float tmin, V3 d, float tmax) {
  rays[2 * r] = make_float4(o.x, o.y, o.z, tmin);
  rays[2 * r + 1] = make_float4(d.x, d.y, d.z, tmax);
}
// A ray no query can hit: tmin above tmax.
__device__ __forceinline__ void store_dead(float4* rays, uint64_t r) {
  store_ray(rays, r, {0.f, 0.f, 0.f}, 1.f, {0.f, 0.f, 1.f}, 0.f);
}

// Device parameters of `view` rendered at width x height with spp samples
// per pixel (the whole image when the view's window is empty); tan_half is
// tan(fov / 2) computed on the host in double and rounded once.
inline ViewDev make_view_dev(const rq_view_t& view, uint32_t width, uint32_t height, uint32_t spp, const float* bg,
                             float bias, float tan_half) {
  ViewDev v;
  v.eye = {view.eye[0], view.eye[1], view.eye[2]};
  v.target = {view.target[0], view.target[1], view.target[2]};
  v.up = {view.up[0], view.up[1], view.up[2]};
  v.light = {view.light[0], view.light[1], view.light[2]};
  v.albedo = {view.albedo[0], view.albedo[1], view.albedo[2]};
  v.bg = {bg[0], bg[1], bg[2]};
  v.tan_half = tan_half;
  v.aspect = (float)width / (float)height;
  v.ambient = view.ambient;
  v.mirror = view.mirror;
  v.bias = bias;
  v.width = width;
  v.height = height;
  v.spp = spp;
  const bool whole = view.window[2] == 0 || view.window[3] == 0;
  v.x0 = whole ? 0 : view.window[0];
  v.y0 = whole ? 0 : view.window[1];
  v.ww = whole ? width : view.window[2];
  v.wh = whole ? height : view.window[3];
  v.bounces = view.bounces;
  v.seed = view.seed;
  return v;
}

// Camera ray of sample r of the view's window (pixel-major, spp samples per
// pixel).  Samples are numbered over the whole image, so a window renders
// exactly the rays of the full image's pixels.
__device__ __forceinline__ void view_ray(const ViewDev& v, uint64_t r, V3& o, V3& d) {
  const uint64_t wp = r / v.spp;
  const uint32_t s = (uint32_t)(r - wp * v.spp);
  const uint32_t x = v.x0 + (uint32_t)(wp % v.ww), y = v.y0 + (uint32_t)(wp / v.ww);
  const uint64_t sample = ((uint64_t)y * v.width + x) * v.spp + s;
  const float jx = jitter01(v.seed, sample, 0), jy = jitter01(v.seed, sample, 1);
  const V3 fwd = v3norm(v3sub(v.target, v.eye));
  const V3 right = v3norm(v3cross(fwd, v.up));
  const V3 upv = v3cross(right, fwd);
  const float px = (2.0f * ((float(x) + jx) / float(v.width)) - 1.0f) * v.tan_half * v.aspect;
  const float py = (1.0f - 2.0f * ((float(y) + jy) / float(v.height))) * v.tan_half;
  o = v.eye;
  d = v3norm(v3add(v3add(fwd, v3mul(right, px)), v3mul(upv, py)));
}

template <int KIND>
__device__ __forceinline__ V3 surface_normal(const SceneView& sc, uint32_t prim, V3 p) {
  if (KIND == kTriangles) {
    const uint32_t* t = sc.idx + 3 * (size_t)prim;
    const uint32_t i0 = __ldg(t), i1 = __ldg(t + 1), i2 = __ldg(t + 2);
    const V3 a = {__ldg(sc.verts + 3 * (size_t)i0), __ldg(sc.verts + 3 * (size_t)i0 + 1), __ldg(sc.verts + 3 * (size_t)i0 + 2)};
    const V3 b = {__ldg(sc.verts + 3 * (size_t)i1), __ldg(sc.verts + 3 * (size_t)i1 + 1), __ldg(sc.verts + 3 * (size_t)i1 + 2)};
    const V3 c = {__ldg(sc.verts + 3 * (size_t)i2), __ldg(sc.verts + 3 * (size_t)i2 + 1), __ldg(sc.verts + 3 * (size_t)i2 + 2)};
    return v3norm(v3cross(v3sub(b, a), v3sub(c, a)));
  } else {
    const float4 s = __ldg(sc.sph + prim);
    return v3norm(v3sub(p, {s.x, s.y, s.z}));
  }
}

// One depth of shading for sample r: background on a miss, else Lambert +
// ambient with a shadow ray and (below the last depth) a mirror ray into
// rays[r].  Sets emit_shadow / emit_mirror for the ray counters.  LISTS: the
// caller drives later queries from lists of the emitting samples, so
// samples that emit nothing get no dead-ray markers and no zero light term.
template <int KIND, bool LISTS = false>
__device__ __forceinline__ void shade_sample(const ViewDev& v, const SceneView& sc, uint64_t r, bool last,
                                             float4* __restrict__ rays, const float4* __restrict__ hits,
                                             float4* __restrict__ shadow, float4* __restrict__ cw,
                                             float4* __restrict__ pend, bool& emit_shadow, bool& emit_mirror) {
  emit_shadow = emit_mirror = false;
  const float4 r0 = rays[2 * r], r1 = rays[2 * r + 1];
  if (!LISTS) pend[r] = make_float4(0.f, 0.f, 0.f, 0.f);
  if (!(r0.w <= r1.w)) {  // finished sample
    if (!LISTS) store_dead(shadow, r);
    return;
  }
  const float4 h = __ldg(hits + r);
  float4 c = cw[r];
  const float w = c.w;
  if (__float_as_uint(h.y) == kMiss) {
    c.x = c.x + w * v.bg.x;
    c.y = c.y + w * v.bg.y;
    c.z = c.z + w * v.bg.z;
    cw[r] = make_float4(c.x, c.y, c.z, 0.f);
    if (!LISTS) {
      store_dead(rays, r);
      store_dead(shadow, r);
    }
    return;
  }
  const V3 o = {r0.x, r0.y, r0.z}, d = {r1.x, r1.y, r1.z};
  const V3 p = v3add(o, v3mul(d, h.x));
  V3 n = surface_normal<KIND>(sc, __float_as_uint(h.y), p);
  if (v3dot(n, d) > 0.f) n = {-n.x, -n.y, -n.z};
  const V3 lv = v3sub(v.light, p);
  const float dist = sqrtf(v3dot(lv, lv));
  const V3 ld = v3mul(lv, 1.0f / dist);
  const float ndl = v3dot(n, ld);
  const float f = last ? w : w * (1.0f - v.mirror);
  const V3 fa = v3mul(v.albedo, f);
  c.x = c.x + fa.x * v.ambient;
  c.y = c.y + fa.y * v.ambient;
  c.z = c.z + fa.z * v.ambient;
  const V3 po = v3add(p, v3mul(n, v.bias));
  if (ndl > 0.f && dist > 0.f) {
    pend[r] = make_float4(fa.x * ndl, fa.y * ndl, fa.z * ndl, 0.f);
    store_ray(shadow, r, po, 0.f, ld, dist);
    emit_shadow = true;
  } else if (!LISTS) {
    store_dead(shadow, r);
  }
  const float wn = w * v.mirror;
  if (!last && wn > 0.f) {
    const V3 rd = v3sub(d, v3mul(n, 2.0f * v3dot(d, n)));
    store_ray(rays, r, po, 0.f, rd, __int_as_float(0x7F800000));
    emit_mirror = true;
  } else if (!LISTS) {
    store_dead(rays, r);
  }
  cw[r] = make_float4(c.x, c.y, c.z, emit_mirror ? wn : 0.f);
}

// Sample r's light term when its shadow ray is unoccluded.
__device__ __forceinline__ void shadow_accum(uint64_t r, const uint32_t* __restrict__ bits,
                                             const float4* __restrict__ pend, float4* __restrict__ cw) {
  const float4 p = __ldg(pend + r);
  if (p.x == 0.f && p.y == 0.f && p.z == 0.f) return;
  if ((__ldg(bits + (r >> 5)) >> (r & 31)) & 1u) return;
  float4 c = cw[r];
  c.x = c.x + p.x;
  c.y = c.y + p.y;
  c.z = c.z + p.z;
  cw[r] = c;
}

// Pixel p: mean of its spp samples, clamp to [0, 1], x255, truncate.
__device__ __forceinline__ void resolve_pixel(uint64_t p, uint32_t spp, const float4* __restrict__ cw,
                                              uint8_t* __restrict__ pixels, float* __restrict__ rgb) {
  float s[3] = {0.f, 0.f, 0.f};
  for (uint32_t k = 0; k < spp; ++k) {
    float4 c = __ldg(cw + p * spp + k);
    s[0] = s[0] + c.x;
    s[1] = s[1] + c.y;
    s[2] = s[2] + c.z;
  }
  const float fs = (float)spp;
  for (int q = 0; q < 3; ++q) {
    float m = s[q] / fs;
    if (rgb) rgb[3 * p + q] = m;
    m = m < 1.f ? (m > 0.f ? m : 0.f) : 1.f;
    pixels[3 * p + q] = (uint8_t)__float2uint_rz(m * 255.f);
  }
}

}  // namespace rq
