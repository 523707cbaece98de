// CPU oracle for the ray-query hot path — TEST INFRASTRUCTURE ONLY.
// See oracle.h for the scope, the data layouts and who may load this library.
// Compiled with -ffp-contract=off: every a*b+c below is two rounded float
// operations, as in the reference's x86-64 build, on every host.
#include "oracle.h"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <numeric>
#include <random>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

struct V3 {
  float x, y, z;
  float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
inline V3 v3(const float* p) { return {p[0], p[1], p[2]}; }
inline V3 sub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
// geometry.h dotProduct: x*v.x + y*v.y + z*v.z, left to right.
inline float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
// geometry.h crossProduct.
inline V3 cross(V3 a, V3 b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
// geometry.h normalize(): the unqualified sqrt there resolves to the double
// overload, so factor = float(1.0 / sqrt(double(n))).
inline V3 normalize_ref(V3 v) {
  float n = v.x * v.x + v.y * v.y + v.z * v.z;
  if (n > 0) {
    float f = (float)(1.0 / std::sqrt((double)n));
    v.x *= f; v.y *= f; v.z *= f;
  }
  return v;
}

struct Box {
  float lo[3], hi[3];
};
// BoxBoundries() default: min = FLT_MAX, max = -FLT_MAX (accelerators.h:108-112).
inline Box empty_box() { return {{FLT_MAX, FLT_MAX, FLT_MAX}, {-FLT_MAX, -FLT_MAX, -FLT_MAX}}; }
inline Box box6(const float* b) { return {{b[0], b[1], b[2]}, {b[3], b[4], b[5]}}; }
// JoinBounds (accelerators.h:201-214), std::min/std::max semantics.
inline Box join(const Box& a, const Box& b) {
  Box r;
  for (int k = 0; k < 3; ++k) {
    r.lo[k] = std::min(a.lo[k], b.lo[k]);
    r.hi[k] = std::max(a.hi[k], b.hi[k]);
  }
  return r;
}
// JoinBoxPopintBounds (accelerators.h:216-229).
inline Box join_pt(const Box& a, const float* p) {
  Box r;
  for (int k = 0; k < 3; ++k) {
    r.lo[k] = std::min(a.lo[k], p[k]);
    r.hi[k] = std::max(a.hi[k], p[k]);
  }
  return r;
}
// GeMaximumAxis (accelerators.h:190-199).
inline int max_axis(const Box& b) {
  float ax = b.hi[0] - b.lo[0], ay = b.hi[1] - b.lo[1], az = b.hi[2] - b.lo[2];
  if (ax > ay && ax > az) return 0;
  if (ay > az) return 1;
  return 2;
}

constexpr float kEps = 1e-6f;                 // main.cpp:59
constexpr float kWiden = 0x1.000006p+0f;      // 1 + 2*gamma(3), robust slab upper bound
constexpr uint32_t kMiss = 0xFFFFFFFFu;

// ---------------------------------------------------------------- primitives

// Sphere test, accelerators.h:79-92.  Inside accelerators.h `using namespace
// std` is in effect, so sqrt(float) is the float overload.
inline bool sphere_ref(const float* s, V3 o, V3 d, float& t0, float& t1) {
  V3 c = v3(s);
  float r2 = s[3] * s[3];
  V3 l = sub(c, o);
  float tca = dot(l, d);
  if (tca < 0) return false;
  float d2 = dot(l, l) - tca * tca;
  if (d2 > r2) return false;
  float thc = std::sqrt(r2 - d2);
  t0 = tca - thc;
  t1 = tca + thc;
  return true;
}

// Moller-Trumbore, main.cpp:138-161 (the MOLLER_TRUMBORE branch, with the
// `v_0` typo read as `v0`), EPS = 1e-6, no culling.  Edges e1 = v1-v0 and
// e2 = v2-v0 are precomputed with the same subtraction.  The reference has
// no t test; the interval (tmin, tmax) is added here (documented deviation).
inline bool tri_mt(const float* p, V3 o, V3 d, float tmin, float tmax, float& t, float& u,
                   float& v) {
  V3 v0 = v3(p), e1 = v3(p + 3), e2 = v3(p + 6);
  V3 pvec = cross(d, e2);
  float det = dot(e1, pvec);
  if (std::fabs(det) < kEps) return false;
  float invDet = 1 / det;
  V3 tvec = sub(o, v0);
  u = dot(tvec, pvec) * invDet;
  if (u < 0 || u > 1) return false;
  V3 qvec = cross(tvec, e1);
  v = dot(d, qvec) * invDet;
  if (v < 0 || u + v > 1) return false;
  t = dot(e2, qvec) * invDet;
  return t > tmin && t < tmax;
}

// One primitive against a ray.  mode REFERENCE with spheres follows castRay's
// selection (main.cpp:346-356): t = t0 unless t0 < 0, accepted when t < best,
// no lower bound.  Otherwise the hit must lie in (tmin, best).
inline bool test_prim(int kind, int mode, const float* prims, uint32_t id, V3 o, V3 d,
                      float tmin, float best, float& t, float& u, float& v) {
  if (kind == ORC_TRIANGLES) return tri_mt(prims + 9 * (size_t)id, o, d, tmin, best, t, u, v);
  float t0 = INFINITY, t1 = INFINITY;
  if (!sphere_ref(prims + 4 * (size_t)id, o, d, t0, t1)) return false;
  if (t0 < 0) t0 = t1;
  t = t0;
  u = v = 0.f;
  if (mode == ORC_MODE_REFERENCE) return t < best;
  return t > tmin && t < best;
}

// FAST closest-hit acceptance: a smaller t, or the same t with a smaller
// primitive id, so that the chosen hit does not depend on the order in which
// a walk meets the primitives (tree shape, node width, scheduling).  Hits
// stay inside (tmin, tmax).
inline bool closest_fast(int kind, const float* prims, uint32_t id, V3 o, V3 d, float tmin, const orc_hit_t& h,
                         float& t, float& u, float& v) {
  const float bound = h.prim == kMiss ? h.t : std::nextafter(h.t, INFINITY);
  if (!test_prim(kind, ORC_MODE_FAST, prims, id, o, d, tmin, bound, t, u, v)) return false;
  return t < h.t || id < h.prim;
}

// Any-hit acceptance.  REFERENCE spheres: kdtreeIntersect returns on any
// successful sphere test (accelerators.h:1020,1030).
inline bool test_prim_any(int kind, int mode, const float* prims, uint32_t id, V3 o, V3 d,
                          float tmin, float tmax) {
  float t, u, v;
  if (kind == ORC_SPHERES && mode == ORC_MODE_REFERENCE) {
    float t0, t1;
    return sphere_ref(prims + 4 * (size_t)id, o, d, t0, t1);
  }
  return test_prim(kind, ORC_MODE_FAST, prims, id, o, d, tmin, tmax, t, u, v);
}

// ---------------------------------------------------------------- box tests

// Reference slab test, accelerators.h:628-666: per-axis division, swap,
// no clipping to the ray's interval.
inline bool box_ref(V3 o, V3 d, const float* lo, const float* hi, float& tMin, float& tMax) {
  float tmin = (lo[0] - o.x) / d.x;
  float tmax = (hi[0] - o.x) / d.x;
  if (tmin > tmax) std::swap(tmin, tmax);
  float tymin = (lo[1] - o.y) / d.y;
  float tymax = (hi[1] - o.y) / d.y;
  if (tymin > tymax) std::swap(tymin, tymax);
  if ((tmin > tymax) || (tymin > tmax)) return false;
  if (tymin > tmin) tmin = tymin;
  if (tymax < tmax) tmax = tymax;
  float tzmin = (lo[2] - o.z) / d.z;
  float tzmax = (hi[2] - o.z) / d.z;
  if (tzmin > tzmax) std::swap(tzmin, tzmax);
  if ((tmin > tzmax) || (tzmin > tmax)) return false;
  if (tzmin > tmin) tmin = tzmin;
  if (tzmax < tmax) tmax = tzmax;
  tMin = tmin;
  tMax = tmax;
  return true;
}

// Engine slab test.  Per ray: inv = 1/d, noi = -(o * inv) and eps = 2^-21 *
// the largest finite |o * inv|.  Per box: plane distances fmaf(b, inv, noi)
// (one correctly rounded fused multiply-add, as the engine's kernels do),
// NaN-ignoring fminf/fmaxf, interval clipped to [tmin, tfar], far end widened
// by the relative 1 + 2*gamma(3) (Ize 2013) and the absolute eps, so that no
// box the ray truly meets is rejected because of rounding.
// The fused form needs o * inv finite on every axis.  Rays where it is not (a
// direction component zero, or so small that 1/d or o/d overflows) use the
// exact form: per axis (b - o) * inv, and an axis along which the ray does not
// move (inv infinite) constrains nothing when lo <= o <= hi and rejects the
// box otherwise; far end widened by 1 + 2^-20.  The engine's kernels perform
// exactly these operations in this order.
constexpr float kWidenExact = 0x1.00001p+0f;
struct SlabRay {
  V3 inv, noi;
  float eps;
  V3 o;
  bool exact;
};
inline SlabRay slab_ray(V3 o, V3 d) {
  SlabRay s;
  s.inv = {1.0f / d.x, 1.0f / d.y, 1.0f / d.z};
  float ox = o.x * s.inv.x, oy = o.y * s.inv.y, oz = o.z * s.inv.z;
  s.noi = {-ox, -oy, -oz};
  float m = 0.f;
  if (std::fabs(ox) <= FLT_MAX) m = fmaxf(m, std::fabs(ox));
  if (std::fabs(oy) <= FLT_MAX) m = fmaxf(m, std::fabs(oy));
  if (std::fabs(oz) <= FLT_MAX) m = fmaxf(m, std::fabs(oz));
  s.eps = m * 0x1p-21f;
  s.o = o;
  s.exact = !(std::fabs(s.noi.x) <= FLT_MAX && std::fabs(s.noi.y) <= FLT_MAX && std::fabs(s.noi.z) <= FLT_MAX);
  return s;
}
inline void slab_axis_exact(float l, float h, float o, float inv, float& near_t, float& far_t) {
  const float a = l - o, b = h - o;
  if (std::fabs(inv) > FLT_MAX) {  // the ray does not move along this axis
    const bool in = a <= 0.f && b >= 0.f;
    near_t = in ? -INFINITY : INFINITY;
    far_t = in ? INFINITY : -INFINITY;
  } else {
    const float t0 = a * inv, t1 = b * inv;
    near_t = fminf(t0, t1);
    far_t = fmaxf(t0, t1);
  }
}
// Per-axis entry and exit distances of one box.
inline void slab_axes(const SlabRay& r, float lx, float hx, float ly, float hy, float lz, float hz, float n[3],
                      float f[3]) {
  if (r.exact) {
    slab_axis_exact(lx, hx, r.o.x, r.inv.x, n[0], f[0]);
    slab_axis_exact(ly, hy, r.o.y, r.inv.y, n[1], f[1]);
    slab_axis_exact(lz, hz, r.o.z, r.inv.z, n[2], f[2]);
    return;
  }
  const float tx0 = std::fmaf(lx, r.inv.x, r.noi.x), tx1 = std::fmaf(hx, r.inv.x, r.noi.x);
  const float ty0 = std::fmaf(ly, r.inv.y, r.noi.y), ty1 = std::fmaf(hy, r.inv.y, r.noi.y);
  const float tz0 = std::fmaf(lz, r.inv.z, r.noi.z), tz1 = std::fmaf(hz, r.inv.z, r.noi.z);
  n[0] = fminf(tx0, tx1); f[0] = fmaxf(tx0, tx1);
  n[1] = fminf(ty0, ty1); f[1] = fmaxf(ty0, ty1);
  n[2] = fminf(tz0, tz1); f[2] = fmaxf(tz0, tz1);
}
inline float slab_exit(const SlabRay& r, float lx, float hx, float ly, float hy, float lz, float hz,
                       float tfar_in) {
  float n[3], f[3];
  slab_axes(r, lx, hx, ly, hy, lz, hz, n, f);
  return fminf(fminf(f[0], f[1]), fminf(f[2], tfar_in));
}
inline float slab_widen(const SlabRay& r) { return r.exact ? kWidenExact : kWiden; }
inline bool box_fast(const SlabRay& r, float lx, float hx, float ly, float hy, float lz, float hz,
                     float tmin, float tfar_in, float& tnear_out) {
  float n[3], f[3];
  slab_axes(r, lx, hx, ly, hy, lz, hz, n, f);
  float tn = fmaxf(fmaxf(n[0], n[1]), fmaxf(n[2], tmin));
  float tf = fminf(fminf(f[0], f[1]), fminf(f[2], tfar_in));
  tf = std::fmaf(tf, slab_widen(r), r.eps);
  tnear_out = tn;
  return tn <= tf;
}

inline int nthreads_or_default(int n) {
#ifdef _OPENMP
  return n > 0 ? n : omp_get_max_threads();
#else
  (void)n;
  return 1;
#endif
}

// ------------------------------------------------------------ BVH2 traversal

struct Entry {
  int32_t node;
  int32_t count;
};

// Closest or any hit through a flattened BVH2 (layout in oracle.h).
//  FAST: near child first (ties -> left), far child pushed, boxes clipped to
//        the current closest hit; the engine's kernels visit in this order.
//  REFERENCE: boxIntersect's pre-order, left subtree before right
//        (accelerators.h:668-690), unclipped division slab test, every
//        candidate tested in visiting order with castRay's strict-< select.
void trace_one_bvh2(int kind, int mode, int query, const float* nodes, uint32_t n_internal,
                    const float* rb, uint32_t n_prims, const uint32_t* order, const float* prims,
                    const orc_ray_t& ray, orc_hit_t& hit, uint8_t& occ, uint64_t& visits,
                    uint64_t& tests) {
  V3 o = v3(ray.org), d = v3(ray.dir);
  float best = ray.tmax;
  hit.t = ray.tmax;
  hit.prim = kMiss;
  hit.u = hit.v = 0.f;
  occ = 0;
  const SlabRay sr = slab_ray(o, d);
  // Root box.
  {
    bool ok;
    if (mode == ORC_MODE_REFERENCE) {
      float a, b;
      ok = box_ref(o, d, rb, rb + 3, a, b);
    } else {
      float tn;
      ok = box_fast(sr, rb[0], rb[3], rb[1], rb[4], rb[2], rb[5], ray.tmin, best, tn);
    }
    if (!ok) return;
  }
  std::vector<Entry> stack;
  stack.reserve(64);
  Entry cur = n_internal == 0 ? Entry{~0, (int32_t)n_prims} : Entry{0, 0};
  for (;;) {
    if (cur.node >= 0) {
      const float* n = nodes + 16 * (size_t)cur.node;
      int32_t ch[4];
      std::memcpy(ch, n + 12, sizeof(ch));
      ++visits;
      bool hl, hr;
      float tl = 0.f, tr = 0.f;
      if (mode == ORC_MODE_REFERENCE) {
        float lo[3] = {n[0], n[2], n[8]}, hi[3] = {n[1], n[3], n[9]};
        float lo2[3] = {n[4], n[6], n[10]}, hi2[3] = {n[5], n[7], n[11]};
        float a, b;
        hl = box_ref(o, d, lo, hi, a, b);
        hr = box_ref(o, d, lo2, hi2, a, b);
        if (hr) stack.push_back({ch[1], ch[3]});
        if (hl) { cur = {ch[0], ch[2]}; continue; }
      } else {
        hl = box_fast(sr, n[0], n[1], n[2], n[3], n[8], n[9], ray.tmin, best, tl);
        hr = box_fast(sr, n[4], n[5], n[6], n[7], n[10], n[11], ray.tmin, best, tr);
        if (hl && hr) {
          Entry nearE = {ch[0], ch[2]}, farE = {ch[1], ch[3]};
          if (tr < tl) std::swap(nearE, farE);
          stack.push_back(farE);
          cur = nearE;
          continue;
        }
        if (hl) { cur = {ch[0], ch[2]}; continue; }
        if (hr) { cur = {ch[1], ch[3]}; continue; }
      }
    } else {
      uint32_t first = (uint32_t)(~cur.node);
      for (int32_t k = 0; k < cur.count; ++k) {
        uint32_t id = order[first + (uint32_t)k];
        ++tests;
        if (query == ORC_ANY) {
          if (test_prim_any(kind, mode, prims, id, o, d, ray.tmin, ray.tmax)) {
            occ = 1;
            return;
          }
        } else {
          float t, u, v;
          const bool take = mode == ORC_MODE_FAST ? closest_fast(kind, prims, id, o, d, ray.tmin, hit, t, u, v)
                                                  : test_prim(kind, mode, prims, id, o, d, ray.tmin, best, t, u, v);
          if (take) {
            best = t;
            hit.t = t;
            hit.prim = id;
            hit.u = u;
            hit.v = v;
          }
        }
      }
    }
    if (stack.empty()) break;
    cur = stack.back();
    stack.pop_back();
  }
}

// -------------------------------------------------------------- KD traversal

struct KdView {
  const int32_t* w;
  bool leaf(int i) const { return (w[3 * i + 1] & 3) == 3; }
  int axis(int i) const { return w[3 * i + 1] & 3; }
  float split(int i) const { float f; std::memcpy(&f, &w[3 * i], 4); return f; }
  int above(int i) const { return w[3 * i + 1] >> 2; }
  int one(int i) const { return w[3 * i]; }
  int ntest(int i) const { return w[3 * i + 2]; }
};

struct KdTodo {
  int node;
  float tMin, tMax;
};

// REFERENCE: kdtreeIntersect (accelerators.h:997-1086), any hit, spheres,
// todo stack of 64.  FAST: the same front-to-back walk (PBRT's, which the
// reference follows) with a robust root clip, hits limited to (tmin, best)
// and PBRT's early exit once the closest hit lies before the next node.
void trace_one_kd(int kind, int mode, int query, const KdView& kd, const int32_t* prim_idx,
                  const float* rb, const float* prims, const orc_ray_t& ray, orc_hit_t& hit,
                  uint8_t& occ, uint64_t& visits, uint64_t& tests) {
  V3 o = v3(ray.org), d = v3(ray.dir);
  hit.t = ray.tmax;
  hit.prim = kMiss;
  hit.u = hit.v = 0.f;
  occ = 0;
  float best = ray.tmax;
  float tMin, tMax;
  V3 inv = {1 / d.x, 1 / d.y, 1 / d.z};
  if (mode == ORC_MODE_REFERENCE) {
    if (!box_ref(o, d, rb, rb + 3, tMin, tMax)) return;
  } else {
    float tn;
    const SlabRay sr = slab_ray(o, d);
    if (!box_fast(sr, rb[0], rb[3], rb[1], rb[4], rb[2], rb[5], ray.tmin, best, tn)) return;
    // exit distance of the root box, clipped and widened the same way
    tMin = tn;
    tMax = std::fmaf(slab_exit(sr, rb[0], rb[3], rb[1], rb[4], rb[2], rb[5], best), slab_widen(sr), sr.eps);
  }
  KdTodo todo[64];
  int todoPos = 0;
  int node = 0;
  for (;;) {
    if (mode != ORC_MODE_REFERENCE && best < tMin) break;
    if (!kd.leaf(node)) {
      ++visits;
      int axis = kd.axis(node);
      float split = kd.split(node);
      float tPlane = (split - o[axis]) * inv[axis];
      bool belowFirst = (o[axis] < split) || (o[axis] == split && d[axis] <= 0);
      int first = belowFirst ? node + 1 : kd.above(node);
      int second = belowFirst ? kd.above(node) : node + 1;
      if (tPlane > tMax || tPlane <= 0) {
        node = first;
      } else if (tPlane < tMin) {
        node = second;
      } else {
        if (todoPos >= 64) return;  // cannot happen below depth 64
        todo[todoPos++] = {second, tPlane, tMax};
        node = first;
        tMax = tPlane;
      }
      continue;
    }
    int np = kd.ntest(node);
    for (int i = 0; i < np; ++i) {
      uint32_t id = (uint32_t)(np == 1 ? kd.one(node) : prim_idx[kd.one(node) + i]);
      ++tests;
      if (query == ORC_ANY || mode == ORC_MODE_REFERENCE) {
        if (test_prim_any(kind, mode, prims, id, o, d, ray.tmin, ray.tmax)) {
          occ = 1;
          if (query == ORC_ANY) return;
        }
      }
      if (query == ORC_CLOSEST) {
        float t, u, v;
        if (test_prim(kind, mode == ORC_MODE_REFERENCE ? ORC_MODE_REFERENCE : ORC_MODE_FAST, prims,
                      id, o, d, ray.tmin, best, t, u, v)) {
          best = t;
          hit.t = t;
          hit.prim = id;
          hit.u = u;
          hit.v = v;
        }
      }
    }
    if (todoPos > 0) {
      --todoPos;
      node = todo[todoPos].node;
      tMin = todo[todoPos].tMin;
      tMax = todo[todoPos].tMax;
    } else {
      break;
    }
  }
}

// ------------------------------------------------------------------ KD build

// PBRT SAH KD build as the reference runs it (accelerators.h:815-948) with
// its effective parameters: maxPrims = 5, isectCost = 80, traversalCost = 1
// and emptyBonus = 0 (the global `char emptyBonus = 0.5f` truncates,
// accelerators.h:767-770).  Edges are ordered by (t, start-before-end,
// primitive id); the reference orders by (t, type) with an unstable sort, which
// yields the same split choices and the same primitive sets per node (the
// order inside a leaf can differ).
struct KdBuilder {
  const float* aabb;
  int maxPrims = 5;
  float isectCost = 80.f, traversalCost = 1.f, emptyBonus = 0.f;
  std::vector<int32_t> nodes;  // 3 words per node
  std::vector<int32_t> prim_idx;

  struct Edge {
    float t;
    int prim;
    int type;  // 0 = start, 1 = end
  };

  void make_leaf(int nodeNum, const std::vector<int>& prims) {
    int np = (int)prims.size();
    int32_t* w = &nodes[3 * (size_t)nodeNum];
    w[1] = 3 | (np << 2);
    w[2] = np;
    if (np == 0) {
      w[0] = 0;
    } else if (np == 1) {
      w[0] = prims[0];
    } else {
      // Leaf lists in primitive-id order: the reference's order inside a
      // leaf comes from an unstable edge sort, so only the set is its own.
      w[0] = (int32_t)prim_idx.size();
      std::vector<int> sorted(prims);
      std::sort(sorted.begin(), sorted.end());
      prim_idx.insert(prim_idx.end(), sorted.begin(), sorted.end());
    }
  }

  void build(int nodeNum, const Box& nb, const std::vector<int>& prims, int depth, int badRefines) {
    nodes.resize(nodes.size() + 3, 0);
    int np = (int)prims.size();
    if (np <= maxPrims || depth == 0) {
      make_leaf(nodeNum, prims);
      return;
    }
    int bestAxis = -1, bestOffset = -1;
    float bestCost = INFINITY;
    float oldCost = isectCost * float(np);
    float dx = nb.hi[0] - nb.lo[0], dy = nb.hi[1] - nb.lo[1], dz = nb.hi[2] - nb.lo[2];
    float totalSA = 2 * (dx * dy + dx * dz + dy * dz);
    float invTotalSA = 1 / totalSA;
    float dd[3] = {dx, dy, dz};
    int axis = max_axis(nb);
    std::vector<Edge> edges(2 * (size_t)np);
    std::vector<Edge> bestEdges;
    for (int retries = 0;; ++retries) {
      for (int i = 0; i < np; ++i) {
        const float* b = aabb + 6 * (size_t)prims[i];
        edges[2 * i] = {b[axis], prims[i], 0};
        edges[2 * i + 1] = {b[3 + axis], prims[i], 1};
      }
      std::sort(edges.begin(), edges.end(), [](const Edge& a, const Edge& b) {
        if (a.t != b.t) return a.t < b.t;
        if (a.type != b.type) return a.type < b.type;
        return a.prim < b.prim;
      });
      int nBelow = 0, nAbove = np;
      for (int i = 0; i < 2 * np; ++i) {
        if (edges[i].type == 1) --nAbove;
        float edgeT = edges[i].t;
        if (edgeT > nb.lo[axis] && edgeT < nb.hi[axis]) {
          int o0 = (axis + 1) % 3, o1 = (axis + 2) % 3;
          float belowSA = 2 * (dd[o0] * dd[o1] + (edgeT - nb.lo[axis]) * (dd[o0] + dd[o1]));
          float aboveSA = 2 * (dd[o0] * dd[o1] + (nb.hi[axis] - edgeT) * (dd[o0] + dd[o1]));
          float pBelow = belowSA * invTotalSA;
          float pAbove = aboveSA * invTotalSA;
          float eb = (nAbove == 0 || nBelow == 0) ? emptyBonus : 0;
          float cost = traversalCost + isectCost * (1 - eb) * (pBelow * nBelow + pAbove * nAbove);
          if (cost < bestCost) {
            bestCost = cost;
            bestAxis = axis;
            bestOffset = i;
          }
        }
        if (edges[i].type == 0) ++nBelow;
      }
      if (bestAxis != -1 || retries >= 2) break;
      axis = (axis + 1) % 3;
    }
    if (bestCost > oldCost) ++badRefines;
    if ((bestCost > 4 * oldCost && np < 16) || bestAxis == -1 || badRefines == 3) {
      make_leaf(nodeNum, prims);
      return;
    }
    // edges[] still holds bestAxis: the loop stops at the first axis that found a split.
    std::vector<int> prims0, prims1;
    for (int i = 0; i < bestOffset; ++i)
      if (edges[i].type == 0) prims0.push_back(edges[i].prim);
    for (int i = bestOffset + 1; i < 2 * np; ++i)
      if (edges[i].type == 1) prims1.push_back(edges[i].prim);
    float tSplit = edges[bestOffset].t;
    Box b0 = nb, b1 = nb;
    b0.hi[bestAxis] = tSplit;
    b1.lo[bestAxis] = tSplit;
    edges.clear();
    edges.shrink_to_fit();
    build(nodeNum + 1, b0, prims0, depth - 1, badRefines);
    int aboveChild = (int)(nodes.size() / 3);
    std::memcpy(&nodes[3 * (size_t)nodeNum], &tSplit, 4);
    nodes[3 * (size_t)nodeNum + 1] = bestAxis | (aboveChild << 2);
    nodes[3 * (size_t)nodeNum + 2] = 0;
    build(aboveChild, b1, prims1, depth - 1, badRefines);
  }
};

// ------------------------------------------------------------ median BVH

struct TmpNode {
  Box b;
  int left = -1, right = -1;
  std::vector<uint32_t> prims;  // leaves only
  bool leaf = false;
};

// constructBVHNew (accelerators.h:246-337).
//
// ENGINE rule (compat == 0): the left child takes the floor(n/2) primitives
// smallest by (centroid[dim], id).  std::nth_element in the reference picks
// the same set whenever no two primitives tie at the median.  Degenerate
// nodes (all centroids on one side of the midpoint, or a zero-extent split
// axis) become one leaf holding the whole range, each leaf ordered by
// (centroid.x, id).  The reference there keeps one primitive, lists the wrong
// objects, or recurses without end (documented deviation).
//
// COMPAT rule (compat == 1): replays the reference's own sequence of
// std::partition and std::nth_element calls on the primitive array (same
// comparators, same initial order), so ties at the median resolve exactly as
// the reference's libstdc++ resolves them, and reproduces its degenerate
// leaves: one primitive (ids[start]) when nothing lies below the midpoint
// (:321-327), the first `n` entries of the whole array when the split axis has
// zero extent (:286-293).  All centroids at or above the midpoint makes the
// reference recurse forever (:329 with midSplitIndex == endIndex); COMPAT
// reports that as an error.
struct MedianBuilder {
  const float* aabb;
  const float* cen;
  int compat = 0;
  bool endless = false;
  std::vector<TmpNode> tmp;
  std::vector<uint32_t> ids;

  int make_leaf(const Box& b, std::vector<uint32_t> prims, bool sort_x) {
    TmpNode t;
    t.b = b;
    t.leaf = true;
    t.prims = std::move(prims);
    if (sort_x)
      std::sort(t.prims.begin(), t.prims.end(), [&](uint32_t a, uint32_t c) {
        float ka = cen[3 * (size_t)a], kc = cen[3 * (size_t)c];
        if (ka != kc) return ka < kc;
        return a < c;
      });
    tmp.push_back(std::move(t));
    return (int)tmp.size() - 1;
  }
  std::vector<uint32_t> range(uint32_t s, uint32_t e) {
    return std::vector<uint32_t>(ids.begin() + s, ids.begin() + e);
  }

  int rec(uint32_t s, uint32_t e) {
    uint32_t n = e - s;
    Box bounds = empty_box();
    for (uint32_t k = s; k < e; ++k) bounds = join(bounds, box6(aabb + 6 * (size_t)ids[k]));
    if (n <= 1) return make_leaf(bounds, range(s, s + 1), false);
    Box cb = bounds;
    for (uint32_t k = s; k < e; ++k) cb = join_pt(cb, cen + 3 * (size_t)ids[k]);
    int dim = max_axis(cb);
    if (cb.hi[dim] == cb.lo[dim])
      return compat ? make_leaf(bounds, range(0, n), false) : make_leaf(bounds, range(s, e), true);
    float pmid = (cb.lo[dim] + cb.hi[dim]) / 2;
    uint32_t mid;
    if (compat) {
      auto it = std::partition(ids.begin() + s, ids.begin() + e,
                               [&](uint32_t a) { return cen[3 * (size_t)a + dim] < pmid; });
      mid = (uint32_t)(it - ids.begin());
      if (mid != s && mid != e) {
        mid = (s + e) / 2;
        std::nth_element(ids.begin() + s, ids.begin() + mid, ids.begin() + e,
                         [&](uint32_t a, uint32_t c) {
                           return cen[3 * (size_t)a + dim] < cen[3 * (size_t)c + dim];
                         });
      }
      if (mid == s) return make_leaf(bounds, range(s, s + 1), false);
      if (mid == e) {
        endless = true;
        return make_leaf(bounds, range(s, e), false);
      }
    } else {
      uint32_t less = 0;
      for (uint32_t k = s; k < e; ++k)
        if (cen[3 * (size_t)ids[k] + dim] < pmid) ++less;
      if (less == 0 || less == n) return make_leaf(bounds, range(s, e), true);
      mid = s + n / 2;
      std::nth_element(ids.begin() + s, ids.begin() + mid, ids.begin() + e,
                       [&](uint32_t a, uint32_t c) {
                         float ka = cen[3 * (size_t)a + dim], kc = cen[3 * (size_t)c + dim];
                         if (ka != kc) return ka < kc;
                         return a < c;
                       });
    }
    int me = (int)tmp.size();
    tmp.push_back(TmpNode{});
    tmp[me].b = bounds;
    int l = rec(s, mid);
    int r = rec(mid, e);
    tmp[me].left = l;
    tmp[me].right = r;
    return me;
  }
};

void write_child_box(float* n, int side, const Box& b) {
  // side 0: words 0..3 (x,y) and 8..9 (z); side 1: 4..7 and 10..11
  float* xy = n + 4 * side;
  xy[0] = b.lo[0]; xy[1] = b.hi[0]; xy[2] = b.lo[1]; xy[3] = b.hi[1];
  n[8 + 2 * side] = b.lo[2];
  n[9 + 2 * side] = b.hi[2];
}

void put_i32(float* n, int word, int32_t v) { std::memcpy(n + word, &v, 4); }

}  // namespace

// =================================================================== C API

extern "C" {

// expandBits, accelerators.h:374-381 (Karras' 10-bit dilation).
uint32_t orc_expand_bits(uint32_t v) {
  v = (v * 0x00010001u) & 0xFF0000FFu;
  v = (v * 0x00000101u) & 0x0F00F00Fu;
  v = (v * 0x00000011u) & 0xC30C30C3u;
  v = (v * 0x00000005u) & 0x49249249u;
  return v;
}

// morton3D, accelerators.h:385-394: x takes the most significant bit of
// every triple.
uint32_t orc_morton3d(float x, float y, float z) {
  x = std::min(std::max(x * 1024.0f, 0.0f), 1023.0f);
  y = std::min(std::max(y * 1024.0f, 0.0f), 1023.0f);
  z = std::min(std::max(z * 1024.0f, 0.0f), 1023.0f);
  uint32_t xx = orc_expand_bits((uint32_t)x);
  uint32_t yy = orc_expand_bits((uint32_t)y);
  uint32_t zz = orc_expand_bits((uint32_t)z);
  return xx * 4 + yy * 2 + zz;
}

// Reference centroid normalisation (center + 30) / 1000, accelerators.h:577.
void orc_morton_spheres_ref(const float* sph, uint32_t n, uint32_t* codes) {
  for (uint32_t i = 0; i < n; ++i) {
    const float* c = sph + 4 * (size_t)i;
    codes[i] = orc_morton3d((c[0] + 30) / 1000, (c[1] + 30) / 1000, (c[2] + 30) / 1000);
  }
}

// Scene-box normalisation for meshes: (c - lo) / (hi - lo) per axis, 0 on a
// zero-extent axis.
void orc_morton_centroids(const float* cen, uint32_t n, const float* lo, const float* hi,
                          uint32_t* codes) {
  float ext[3] = {hi[0] - lo[0], hi[1] - lo[1], hi[2] - lo[2]};
  for (uint32_t i = 0; i < n; ++i) {
    float q[3];
    for (int k = 0; k < 3; ++k)
      q[k] = ext[k] > 0 ? (cen[3 * (size_t)i + k] - lo[k]) / ext[k] : 0.0f;
    codes[i] = orc_morton3d(q[0], q[1], q[2]);
  }
}

// The engine's cube normalisation: every axis divided by the largest extent
// E = max(hi - lo) of the scene box.
void orc_morton_centroids_cube(const float* cen, uint32_t n, const float* lo, const float* hi,
                               uint32_t* codes) {
  const float e = fmaxf(fmaxf(hi[0] - lo[0], hi[1] - lo[1]), hi[2] - lo[2]);
  for (uint32_t i = 0; i < n; ++i) {
    float q[3];
    for (int k = 0; k < 3; ++k) q[k] = e > 0 ? (cen[3 * (size_t)i + k] - lo[k]) / e : 0.0f;
    codes[i] = orc_morton3d(q[0], q[1], q[2]);
  }
}

void orc_tri_prims(const float* verts, uint32_t nv, const uint32_t* idx, uint32_t nt,
                   float* prims9, float* aabb6, float* centroid3) {
  (void)nv;
  for (uint32_t i = 0; i < nt; ++i) {
    V3 a = v3(verts + 3 * (size_t)idx[3 * (size_t)i]);
    V3 b = v3(verts + 3 * (size_t)idx[3 * (size_t)i + 1]);
    V3 c = v3(verts + 3 * (size_t)idx[3 * (size_t)i + 2]);
    if (prims9) {
      V3 e1 = sub(b, a), e2 = sub(c, a);
      float* p = prims9 + 9 * (size_t)i;
      p[0] = a.x; p[1] = a.y; p[2] = a.z;
      p[3] = e1.x; p[4] = e1.y; p[5] = e1.z;
      p[6] = e2.x; p[7] = e2.y; p[8] = e2.z;
    }
    if (aabb6) {
      float* q = aabb6 + 6 * (size_t)i;
      q[0] = fminf(fminf(a.x, b.x), c.x); q[1] = fminf(fminf(a.y, b.y), c.y);
      q[2] = fminf(fminf(a.z, b.z), c.z); q[3] = fmaxf(fmaxf(a.x, b.x), c.x);
      q[4] = fmaxf(fmaxf(a.y, b.y), c.y); q[5] = fmaxf(fmaxf(a.z, b.z), c.z);
    }
    if (centroid3) {
      float* q = centroid3 + 3 * (size_t)i;
      q[0] = (a.x + b.x + c.x) / 3.0f;
      q[1] = (a.y + b.y + c.y) / 3.0f;
      q[2] = (a.z + b.z + c.z) / 3.0f;
    }
  }
}

// Sphere bounds as createScene_new builds them: centre -/+ radius
// (main.cpp:686-688).
void orc_sphere_prims(const float* sph, uint32_t n, float* aabb6, float* centroid3) {
  for (uint32_t i = 0; i < n; ++i) {
    const float* s = sph + 4 * (size_t)i;
    if (aabb6) {
      float* q = aabb6 + 6 * (size_t)i;
      q[0] = s[0] - s[3]; q[1] = s[1] - s[3]; q[2] = s[2] - s[3];
      q[3] = s[0] + s[3]; q[4] = s[1] + s[3]; q[5] = s[2] + s[3];
    }
    if (centroid3) {
      float* q = centroid3 + 3 * (size_t)i;
      q[0] = s[0]; q[1] = s[1]; q[2] = s[2];
    }
  }
}

void orc_bounds3(const float* pts, uint32_t n, uint32_t stride, float* lo, float* hi) {
  for (int k = 0; k < 3; ++k) { lo[k] = FLT_MAX; hi[k] = -FLT_MAX; }
  for (uint32_t i = 0; i < n; ++i)
    for (int k = 0; k < 3; ++k) {
      float v = pts[(size_t)stride * i + k];
      lo[k] = fminf(lo[k], v);
      hi[k] = fmaxf(hi[k], v);
    }
}

// Stable sort of (code, index) pairs: the order radixSort
// (accelerators.h:348-369) would produce if it sorted its argument in place.
void orc_sort_pairs(const uint32_t* keys, uint32_t n, uint32_t* out_keys, uint32_t* out_vals) {
  std::vector<uint32_t> idx(n);
  std::iota(idx.begin(), idx.end(), 0u);
  std::stable_sort(idx.begin(), idx.end(), [&](uint32_t a, uint32_t b) { return keys[a] < keys[b]; });
  for (uint32_t i = 0; i < n; ++i) {
    out_vals[i] = idx[i];
    out_keys[i] = keys[idx[i]];
  }
}

// Karras 2012, "Maximizing Parallelism in the Construction of BVHs, Octrees,
// and k-d Trees", Fig. 4: the construction the reference cites
// (accelerators.h:371,568) in place of its findSplit (accelerators.h:397-449).
// delta(i,j) = clz(k_i ^ k_j), or 32 + clz(i ^ j) for equal codes, -1 out of
// range.  Children: >= 0 internal, ~j for leaf j.  parent: internal nodes at
// [0, n-1), leaves at [n-1, 2n-1); the root's parent is -1.
void orc_karras(const uint32_t* k, uint32_t n, int32_t* left, int32_t* right, int32_t* parent) {
  const int64_t N = n;
  auto delta = [&](int64_t i, int64_t j) -> int {
    if (j < 0 || j >= N) return -1;
    uint32_t a = k[i], b = k[j];
    if (a != b) return __builtin_clz(a ^ b);
    return 32 + __builtin_clz((uint32_t)i ^ (uint32_t)j);
  };
  if (parent)
    for (int64_t i = 0; i < 2 * N - 1; ++i) parent[i] = -1;
  for (int64_t i = 0; i + 1 < N; ++i) {
    int d = (delta(i, i + 1) - delta(i, i - 1)) > 0 ? 1 : -1;
    int dmin = delta(i, i - d);
    int64_t lmax = 2;
    while (delta(i, i + lmax * d) > dmin) lmax *= 2;
    int64_t l = 0;
    for (int64_t t = lmax / 2; t >= 1; t /= 2)
      if (delta(i, i + (l + t) * d) > dmin) l += t;
    int64_t j = i + l * d;
    int dnode = delta(i, j);
    int64_t s = 0, t = l;
    do {
      t = (t + 1) >> 1;
      if (delta(i, i + (s + t) * d) > dnode) s += t;
    } while (t > 1);
    int64_t gamma = i + s * d + std::min(d, 0);
    int64_t lo = std::min(i, j), hi = std::max(i, j);
    int32_t lc = (lo == gamma) ? ~(int32_t)gamma : (int32_t)gamma;
    int32_t rc = (hi == gamma + 1) ? ~(int32_t)(gamma + 1) : (int32_t)(gamma + 1);
    left[i] = lc;
    right[i] = rc;
    if (parent) {
      parent[lc >= 0 ? lc : (N - 1 + ~lc)] = (int32_t)i;
      parent[rc >= 0 ? rc : (N - 1 + ~rc)] = (int32_t)i;
    }
  }
}

// Bottom-up refit: every internal box is the union of its two children
// (the construction the reference cites at accelerators.h:568; absent there).
void orc_refit(uint32_t n, const int32_t* left, const int32_t* right, const float* slot_aabb6,
               float* nodes16, float* root_bounds6) {
  if (n <= 1) {
    if (n == 1) std::memcpy(root_bounds6, slot_aabb6, 6 * sizeof(float));
    return;
  }
  std::vector<Box> nb(n - 1);
  std::vector<uint8_t> done(n - 1, 0);
  auto child_box = [&](int32_t c) { return c < 0 ? box6(slot_aabb6 + 6 * (size_t)(~c)) : nb[c]; };
  // iterative post-order from the root (node 0)
  std::vector<int32_t> st;
  st.push_back(0);
  while (!st.empty()) {
    int32_t v = st.back();
    bool ready = true;
    for (int32_t c : {left[v], right[v]})
      if (c >= 0 && !done[c]) { st.push_back(c); ready = false; }
    if (!ready) continue;
    st.pop_back();
    Box a = child_box(left[v]), b = child_box(right[v]);
    Box u;
    for (int q = 0; q < 3; ++q) { u.lo[q] = fminf(a.lo[q], b.lo[q]); u.hi[q] = fmaxf(a.hi[q], b.hi[q]); }
    nb[v] = u;
    done[v] = 1;
    float* nd = nodes16 + 16 * (size_t)v;
    write_child_box(nd, 0, a);
    write_child_box(nd, 1, b);
    put_i32(nd, 12, left[v]);
    put_i32(nd, 13, right[v]);
    put_i32(nd, 14, left[v] < 0 ? 1 : 0);
    put_i32(nd, 15, right[v] < 0 ? 1 : 0);
  }
  for (int q = 0; q < 3; ++q) { root_bounds6[q] = nb[0].lo[q]; root_bounds6[3 + q] = nb[0].hi[q]; }
}

int orc_build_lbvh(const uint32_t* codes, const float* aabb6, uint32_t n, float* nodes16,
                   uint32_t* order, uint32_t* sorted_codes, float* root_bounds6) {
  if (n == 0) return -1;
  std::vector<uint32_t> sk(n);
  orc_sort_pairs(codes, n, sk.data(), order);
  if (sorted_codes) std::memcpy(sorted_codes, sk.data(), n * sizeof(uint32_t));
  std::vector<float> slot(6 * (size_t)n);
  for (uint32_t s = 0; s < n; ++s) std::memcpy(&slot[6 * (size_t)s], aabb6 + 6 * (size_t)order[s], 24);
  if (n == 1) {
    std::memcpy(root_bounds6, slot.data(), 24);
    return 0;
  }
  std::vector<int32_t> l(n - 1), r(n - 1);
  orc_karras(sk.data(), n, l.data(), r.data(), nullptr);
  orc_refit(n, l.data(), r.data(), slot.data(), nodes16, root_bounds6);
  return 0;
}

namespace treelet {
constexpr int kTreeletLeaves = 4;  // the engine's kOptLeaves
struct TB { float lo[3], hi[3]; };
static void grow(TB& a, const TB& b) {
  for (int k = 0; k < 3; ++k) { a.lo[k] = std::fmin(a.lo[k], b.lo[k]); a.hi[k] = std::fmax(a.hi[k], b.hi[k]); }
}
static float half_area(const TB& b) {
  const float dx = b.hi[0] - b.lo[0], dy = b.hi[1] - b.lo[1], dz = b.hi[2] - b.lo[2];
  return dx * dy + dy * dz + dz * dx;
}
struct Tree {
  float* nd;
  int32_t link(int id, int side) const { int32_t v; std::memcpy(&v, nd + 16 * (size_t)id + 12 + side, 4); return v; }
  TB box(int id, int side) const {
    const float* q = nd + 16 * (size_t)id;
    TB b;
    b.lo[0] = q[4 * side + 0]; b.hi[0] = q[4 * side + 1]; b.lo[1] = q[4 * side + 2]; b.hi[1] = q[4 * side + 3];
    b.lo[2] = q[8 + 2 * side]; b.hi[2] = q[9 + 2 * side];
    return b;
  }
  void set(int id, int32_t l, const TB& bl, int32_t r, const TB& br) {
    float* q = nd + 16 * (size_t)id;
    q[0] = bl.lo[0]; q[1] = bl.hi[0]; q[2] = bl.lo[1]; q[3] = bl.hi[1];
    q[4] = br.lo[0]; q[5] = br.hi[0]; q[6] = br.lo[1]; q[7] = br.hi[1];
    q[8] = bl.lo[2]; q[9] = bl.hi[2]; q[10] = br.lo[2]; q[11] = br.hi[2];
    const int32_t w[4] = {l, r, l < 0 ? 1 : 0, r < 0 ? 1 : 0};
    std::memcpy(q + 12, w, 16);
  }
};
static int low_index(int s) { int k = 0; while (!((s >> k) & 1)) ++k; return k; }
// Least sum of internal half areas over the topologies of the N treelet
// leaves (a leaf costs 0): subsets S in increasing order, parts P of S holding
// S's lowest leaf in decreasing order, first least best[P] + best[S ^ P]; the
// chosen subsets take the pool's nodes in decreasing subset order.
static void rebuild(Tree& t, int N, const int32_t* code, const TB* box, const int* pool) {
  const int F = (1 << N) - 1;
  float best[32];
  int split[32];
  for (int k = 0; k < N; ++k) best[1 << k] = 0.f;
  for (int S = 1; S <= F; ++S) {
    if ((S & (S - 1)) == 0) continue;
    const int low = S & -S;
    float acc = INFINITY;
    int accp = 0;
    for (int P = (S - 1) & S; P > 0; P = (P - 1) & S) {
      if (!(P & low)) continue;
      const float c = best[P] + best[S ^ P];
      if (c < acc) { acc = c; accp = P; }
    }
    TB u = box[low_index(S)];
    for (int b = 0; b < N; ++b)
      if ((S >> b) & 1) grow(u, box[b]);
    best[S] = half_area(u) + acc;
    split[S] = accp;
  }
  uint32_t used = 1u << F;
  for (int S = F; S >= 3; --S)
    if ((S & (S - 1)) && ((used >> S) & 1u)) used |= (1u << split[S]) | (1u << (S ^ split[S]));
  int id_of[32];
  int next = 0;
  for (int S = F; S >= 3; --S)
    if ((S & (S - 1)) && ((used >> S) & 1u)) id_of[S] = pool[next++];
  for (int S = F; S >= 3; --S) {
    if (!(S & (S - 1)) || !((used >> S) & 1u)) continue;
    const int P = split[S], Q = S ^ P;
    int32_t cl = 0, cr = 0;
    TB bl = box[0], br = box[0];
    bool fl = false, fr = false;
    for (int b = 0; b < N; ++b) {
      if (P == (1 << b)) cl = code[b];
      if (Q == (1 << b)) cr = code[b];
      if ((P >> b) & 1) { if (fl) grow(bl, box[b]); else bl = box[b]; fl = true; }
      if ((Q >> b) & 1) { if (fr) grow(br, box[b]); else br = box[b]; fr = true; }
    }
    if (P & (P - 1)) cl = id_of[P];
    if (Q & (Q - 1)) cr = id_of[Q];
    t.set(id_of[S], cl, bl, cr, br);
  }
}
static void restructure(Tree& t, int x) {
  int32_t code[kTreeletLeaves];
  TB box[kTreeletLeaves];
  int pool[kTreeletLeaves - 1];
  code[0] = t.link(x, 0); code[1] = t.link(x, 1);
  box[0] = t.box(x, 0); box[1] = t.box(x, 1);
  pool[0] = x;
  int n = 2;
  for (int step = 0; step < kTreeletLeaves - 2; ++step) {
    int pick = -1;
    float pa = -1.f;
    for (int k = 0; k < n; ++k)
      if (code[k] >= 0) {
        const float a = half_area(box[k]);
        if (a > pa) { pa = a; pick = k; }
      }
    if (pick < 0) break;
    const int c = code[pick];
    pool[step + 1] = c;
    const int32_t l = t.link(c, 0), r = t.link(c, 1);
    const TB b0 = t.box(c, 0), b1 = t.box(c, 1);
    code[pick] = l; box[pick] = b0;
    code[n] = r; box[n] = b1;
    ++n;
  }
  if (n >= 3) rebuild(t, n, code, box, pool);
}
}  // namespace treelet

void orc_treelet_opt(float* nodes16, uint32_t n_internal) {
  if (n_internal < 2) return;
  treelet::Tree t{nodes16};
  // leaf counts (post-order) and the top-node rule
  std::vector<uint32_t> leaves(n_internal, 0), order;
  order.reserve(n_internal);
  std::vector<std::pair<int, int>> st{{0, 0}};
  while (!st.empty()) {  // iterative post-order: (node, children pushed)
    auto [v, done] = st.back();
    st.pop_back();
    if (done) { order.push_back(v); continue; }
    st.push_back({v, 1});
    for (int side = 1; side >= 0; --side) {
      const int32_t c = t.link(v, side);
      if (c >= 0) st.push_back({c, 0});
    }
  }
  uint32_t n_top = 0;
  for (int v : order) {
    uint32_t s = 0;
    for (int side = 0; side < 2; ++side) { const int32_t c = t.link(v, side); s += c < 0 ? 1u : leaves[c]; }
    leaves[v] = s;
    if (s > 2048) ++n_top;
  }
  const bool skip_top = n_top > 2048;
  std::vector<uint8_t> top(n_internal, 0);
  for (int v : order) top[v] = leaves[v] > 2048;
  for (int v : order) {
    if (skip_top && top[v]) continue;
    treelet::restructure(t, v);
  }
}

// Flattened median BVH: internal nodes numbered breadth-first (left before
// right), leaf slots assigned left to right, each leaf's primitives ordered by
// (centroid.x, id).
int orc_build_median(const float* aabb6, const float* centroid3, uint32_t n, int compat,
                     float* nodes16, uint32_t* order, uint32_t cap_order, uint32_t* n_slots,
                     uint32_t* n_internal, float* root_bounds6) {
  if (n == 0) return -1;
  MedianBuilder mb{aabb6, centroid3, compat, false, {}, {}};
  mb.ids.resize(n);
  std::iota(mb.ids.begin(), mb.ids.end(), 0u);
  mb.tmp.reserve(2 * (size_t)n);
  int root = mb.rec(0, n);
  const auto& T = mb.tmp;
  for (int q = 0; q < 3; ++q) { root_bounds6[q] = T[root].b.lo[q]; root_bounds6[3 + q] = T[root].b.hi[q]; }
  // leaf slots, left to right
  std::vector<int64_t> slot_of(T.size(), -1);
  {
    uint32_t next = 0;
    std::vector<int> st{root};
    while (!st.empty()) {
      int v = st.back();
      st.pop_back();
      if (T[v].leaf) {
        slot_of[v] = next;
        for (uint32_t p : T[v].prims) {
          if (next < cap_order) order[next] = p;
          ++next;
        }
      } else {
        st.push_back(T[v].right);
        st.push_back(T[v].left);
      }
    }
    *n_slots = next;
    if (next > cap_order) return 1;
  }
  if (mb.endless) return 2;
  if (T[root].leaf) {
    *n_internal = 0;
    return 0;
  }
  // breadth-first numbering of internal nodes
  std::vector<int> bfs{root};
  std::vector<int64_t> num(T.size(), -1);
  num[root] = 0;
  for (size_t h = 0; h < bfs.size(); ++h) {
    int v = bfs[h];
    for (int c : {T[v].left, T[v].right})
      if (!T[c].leaf) {
        num[c] = (int64_t)bfs.size();
        bfs.push_back(c);
      }
  }
  for (size_t h = 0; h < bfs.size(); ++h) {
    int v = bfs[h];
    float* nd = nodes16 + 16 * h;
    int side = 0;
    for (int c : {T[v].left, T[v].right}) {
      write_child_box(nd, side, T[c].b);
      if (T[c].leaf) {
        put_i32(nd, 12 + side, ~(int32_t)slot_of[c]);
        put_i32(nd, 14 + side, (int32_t)T[c].prims.size());
      } else {
        put_i32(nd, 12 + side, (int32_t)num[c]);
        put_i32(nd, 14 + side, 0);
      }
      ++side;
    }
  }
  *n_internal = (uint32_t)bfs.size();
  return 0;
}

// maxDepth = round(8 + 1.3 * Log2Int(N)) (accelerators.h:957-958).
int orc_kd_max_depth(uint32_t n) {
  int l = 0;
  while (n > 1) { n >>= 1; ++l; }
  return (int)std::round(8 + 1.3f * l);
}

int orc_build_kd(const float* aabb6, uint32_t n, int32_t max_depth, int32_t* nodes3,
                 uint32_t cap_nodes, uint32_t* n_nodes, int32_t* prim_idx, uint32_t cap_idx,
                 uint32_t* n_idx, float* root_bounds6) {
  if (n == 0) return -1;
  KdBuilder kb;
  kb.aabb = aabb6;
  // Root bounds: JoinBounds over every primitive box (accelerators.h:965-969).
  Box rb = empty_box();
  for (uint32_t i = 0; i < n; ++i) rb = join(rb, box6(aabb6 + 6 * (size_t)i));
  std::vector<int> prims(n);
  std::iota(prims.begin(), prims.end(), 0);
  int depth = max_depth > 0 ? max_depth : orc_kd_max_depth(n);
  kb.build(0, rb, prims, depth, 0);
  uint32_t nn = (uint32_t)(kb.nodes.size() / 3);
  *n_nodes = nn;
  *n_idx = (uint32_t)kb.prim_idx.size();
  for (int q = 0; q < 3; ++q) { root_bounds6[q] = rb.lo[q]; root_bounds6[3 + q] = rb.hi[q]; }
  if (nn > cap_nodes || kb.prim_idx.size() > cap_idx) return 1;
  std::memcpy(nodes3, kb.nodes.data(), kb.nodes.size() * sizeof(int32_t));
  if (!kb.prim_idx.empty()) std::memcpy(prim_idx, kb.prim_idx.data(), kb.prim_idx.size() * 4);
  return 0;
}

// boxIntersect (accelerators.h:668-690): every primitive id of every leaf
// that the reference's pre-order walk with the division slab test reaches.
uint64_t orc_candidates_bvh2(const float* nodes, uint32_t n_internal, const float* rb, uint32_t n_prims,
                             const uint32_t* order, const orc_ray_t* rays, uint32_t nrays, uint32_t* counts,
                             uint32_t* ids, uint64_t cap) {
  uint64_t total = 0;
  for (uint32_t r = 0; r < nrays; ++r) {
    const V3 o = v3(rays[r].org), d = v3(rays[r].dir);
    uint32_t c = 0;
    float a, b;
    if (box_ref(o, d, rb, rb + 3, a, b)) {
      std::vector<Entry> stack;
      Entry cur = n_internal == 0 ? Entry{~0, (int32_t)n_prims} : Entry{0, 0};
      for (;;) {
        if (cur.node >= 0) {
          const float* n = nodes + 16 * (size_t)cur.node;
          int32_t ch[4];
          std::memcpy(ch, n + 12, sizeof(ch));
          float lo[3] = {n[0], n[2], n[8]}, hi[3] = {n[1], n[3], n[9]};
          float lo2[3] = {n[4], n[6], n[10]}, hi2[3] = {n[5], n[7], n[11]};
          const bool hl = box_ref(o, d, lo, hi, a, b);
          const bool hr = box_ref(o, d, lo2, hi2, a, b);
          if (hr) stack.push_back({ch[1], ch[3]});
          if (hl) { cur = {ch[0], ch[2]}; continue; }
        } else {
          for (int32_t k = 0; k < cur.count; ++k) {
            if (ids && total + c < cap) ids[total + c] = order[(uint32_t)(~cur.node) + (uint32_t)k];
            ++c;
          }
        }
        if (stack.empty()) break;
        cur = stack.back();
        stack.pop_back();
      }
    }
    counts[r] = c;
    total += c;
  }
  return total;
}

int orc_trace_bvh2(int kind, int mode, int query, const float* nodes16, uint32_t n_internal,
                   const float* root_bounds6, uint32_t n_prims, const uint32_t* order,
                   const float* prims, const orc_ray_t* rays, uint32_t nrays, orc_hit_t* hits,
                   uint8_t* occluded, uint64_t* counters, int nthreads) {
  uint64_t visits = 0, tests = 0;
  int nt = nthreads_or_default(nthreads);
#pragma omp parallel for num_threads(nt) schedule(dynamic, 256) reduction(+ : visits, tests)
  for (int64_t r = 0; r < (int64_t)nrays; ++r) {
    orc_hit_t h;
    uint8_t occ;
    uint64_t v = 0, t = 0;
    trace_one_bvh2(kind, mode, query, nodes16, n_internal, root_bounds6, n_prims, order, prims,
                   rays[r], h, occ, v, t);
    if (hits) hits[r] = h;
    if (occluded) occluded[r] = occ;
    visits += v;
    tests += t;
  }
  if (counters) { counters[0] += visits; counters[1] += tests; }
  return 0;
}

// Order-preserving unsigned image of a non-NaN float.
static inline uint32_t float_order_key(float f) {
  uint32_t u;
  std::memcpy(&u, &f, 4);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

uint32_t orc_collapse_bvh4(const float* nodes16, uint32_t n_internal, float* nodes32) {
  if (n_internal == 0) return 0;
  auto link = [&](uint32_t b, int side) {
    int32_t v;
    std::memcpy(&v, nodes16 + 16 * (size_t)b + 12 + side, 4);
    return v;
  };
  auto cnt = [&](uint32_t b, int side) {
    int32_t v;
    std::memcpy(&v, nodes16 + 16 * (size_t)b + 14 + side, 4);
    return v;
  };
  // depth by breadth-first walk from the root
  std::vector<int32_t> depth(n_internal, -1);
  std::vector<uint32_t> q{0};
  depth[0] = 0;
  for (size_t h = 0; h < q.size(); ++h)
    for (int side = 0; side < 2; ++side) {
      int32_t c = link(q[h], side);
      if (c >= 0) {
        depth[c] = depth[q[h]] + 1;
        q.push_back((uint32_t)c);
      }
    }
  std::vector<uint32_t> idx4(n_internal, 0);
  uint32_t n4 = 0;
  for (uint32_t b = 0; b < n_internal; ++b)
    if (depth[b] % 2 == 0) idx4[b] = n4++;
  // child box of binary node b, side s: {lo.x, hi.x, lo.y, hi.y, lo.z, hi.z}
  auto box = [&](uint32_t b, int s, float* o) {
    const float* n = nodes16 + 16 * (size_t)b;
    o[0] = n[4 * s + 0]; o[1] = n[4 * s + 1]; o[2] = n[4 * s + 2]; o[3] = n[4 * s + 3];
    o[4] = n[8 + 2 * s]; o[5] = n[9 + 2 * s];
  };
  for (uint32_t b = 0; b < n_internal; ++b) {
    if (depth[b] % 2) continue;
    float* w = nodes32 + 32 * (size_t)idx4[b];
    for (int k = 0; k < 4; ++k) {
      w[k] = INFINITY; w[4 + k] = -INFINITY; w[8 + k] = INFINITY; w[12 + k] = -INFINITY;
      w[16 + k] = INFINITY; w[20 + k] = -INFINITY;
      int32_t z = 0, none = -1;
      std::memcpy(w + 24 + k, &z, 4);
      std::memcpy(w + 28 + k, &none, 4);
    }
    int slot = 0;
    auto put = [&](const float* bx, int32_t l, int32_t c) {
      w[slot] = bx[0]; w[4 + slot] = bx[1]; w[8 + slot] = bx[2]; w[12 + slot] = bx[3];
      w[16 + slot] = bx[4]; w[20 + slot] = bx[5];
      std::memcpy(w + 24 + slot, &l, 4);
      std::memcpy(w + 28 + slot, &c, 4);
      ++slot;
    };
    for (int s = 0; s < 2; ++s) {
      int32_t c = link(b, s);
      float bx[6];
      if (c < 0) {
        box(b, s, bx);
        put(bx, c, cnt(b, s));
      } else {
        for (int s2 = 0; s2 < 2; ++s2) {
          int32_t g = link((uint32_t)c, s2);
          box((uint32_t)c, s2, bx);
          if (g < 0) put(bx, g, cnt((uint32_t)c, s2));
          else put(bx, (int32_t)idx4[g], 0);
        }
      }
    }
  }
  return n4;
}

int orc_trace_bvh4(int kind, int query, const float* nodes32, uint32_t n4, const float* rb,
                   uint32_t n_prims, const uint32_t* order, const float* prims, const orc_ray_t* rays,
                   uint32_t nrays, orc_hit_t* hits, uint8_t* occluded, uint64_t* counters, int nthreads) {
  uint64_t visits = 0, tests = 0;
  int nt = nthreads_or_default(nthreads);
#pragma omp parallel for num_threads(nt) schedule(dynamic, 256) reduction(+ : visits, tests)
  for (int64_t r = 0; r < (int64_t)nrays; ++r) {
    const orc_ray_t& ray = rays[r];
    V3 o = v3(ray.org), d = v3(ray.dir);
    orc_hit_t h{ray.tmax, kMiss, 0.f, 0.f};
    uint8_t occ = 0;
    float best = ray.tmax;
    const SlabRay sr = slab_ray(o, d);
    float tn;
    if (box_fast(sr, rb[0], rb[3], rb[1], rb[4], rb[2], rb[5], ray.tmin, best, tn)) {
      std::vector<Entry> stack;
      stack.reserve(96);
      Entry cur = n4 == 0 ? Entry{~0, (int32_t)n_prims} : Entry{0, 0};
      for (;;) {
        if (cur.node >= 0) {
          const float* w = nodes32 + 32 * (size_t)cur.node;
          ++visits;
          const float tfar = query == ORC_ANY ? ray.tmax : best;
          // Hit children ordered by key = (order-preserving bits of the entry
          // distance, low two bits replaced by the slot): nearest first,
          // distances within four ulps in slot order.
          uint32_t key[4];
          int m = 0;
          for (int k = 0; k < 4; ++k) {
            float tk;
            int32_t ck;
            std::memcpy(&ck, w + 28 + k, 4);
            // an unused slot (count -1) is never entered: a slab test alone
            // cannot reject an inverted box for every ray direction
            if (ck >= 0 &&
                box_fast(sr, w[k], w[4 + k], w[8 + k], w[12 + k], w[16 + k], w[20 + k], ray.tmin, tfar, tk))
              key[m++] = (float_order_key(tk) & ~3u) | (uint32_t)k;
          }
          std::sort(key, key + m);
          int slot[4];
          for (int q2 = 0; q2 < m; ++q2) slot[q2] = (int)(key[q2] & 3u);
          if (m > 0) {
            for (int q2 = m - 1; q2 >= 1; --q2) {
              int32_t l, c;
              std::memcpy(&l, w + 24 + slot[q2], 4);
              std::memcpy(&c, w + 28 + slot[q2], 4);
              stack.push_back({l, c});
            }
            int32_t l, c;
            std::memcpy(&l, w + 24 + slot[0], 4);
            std::memcpy(&c, w + 28 + slot[0], 4);
            cur = {l, c};
            continue;
          }
        } else {
          uint32_t first = (uint32_t)(~cur.node);
          bool done = false;
          for (int32_t k = 0; k < cur.count; ++k) {
            uint32_t id = order[first + (uint32_t)k];
            ++tests;
            if (query == ORC_ANY) {
              if (test_prim_any(kind, ORC_MODE_FAST, prims, id, o, d, ray.tmin, ray.tmax)) {
                occ = 1;
                done = true;
                break;
              }
            } else {
              float t, u, v;
              if (closest_fast(kind, prims, id, o, d, ray.tmin, h, t, u, v)) {
                best = t;
                h = {t, id, u, v};
              }
            }
          }
          if (done) break;
        }
        if (stack.empty()) break;
        cur = stack.back();
        stack.pop_back();
      }
    }
    if (hits) hits[r] = h;
    if (occluded) occluded[r] = occ;
  }
  if (counters) { counters[0] += visits; counters[1] += tests; }
  return 0;
}

int orc_trace_kd(int kind, int mode, int query, const int32_t* nodes3, uint32_t n_nodes,
                 const int32_t* prim_idx, const float* root_bounds6, const float* prims,
                 const orc_ray_t* rays, uint32_t nrays, orc_hit_t* hits, uint8_t* occluded,
                 uint64_t* counters, int nthreads) {
  (void)n_nodes;
  KdView kd{nodes3};
  uint64_t visits = 0, tests = 0;
  int nt = nthreads_or_default(nthreads);
#pragma omp parallel for num_threads(nt) schedule(dynamic, 256) reduction(+ : visits, tests)
  for (int64_t r = 0; r < (int64_t)nrays; ++r) {
    orc_hit_t h;
    uint8_t occ;
    uint64_t v = 0, t = 0;
    trace_one_kd(kind, mode, query, kd, prim_idx, root_bounds6, prims, rays[r], h, occ, v, t);
    if (hits) hits[r] = h;
    if (occluded) occluded[r] = occ;
    visits += v;
    tests += t;
  }
  if (counters) { counters[0] += visits; counters[1] += tests; }
  return 0;
}

// NONE: every primitive in id order (main.cpp:373-387).
int orc_trace_brute(int kind, int mode, int query, uint32_t n_prims, const float* prims,
                    const orc_ray_t* rays, uint32_t nrays, orc_hit_t* hits, uint8_t* occluded,
                    int nthreads) {
  int nt = nthreads_or_default(nthreads);
#pragma omp parallel for num_threads(nt) schedule(dynamic, 64)
  for (int64_t r = 0; r < (int64_t)nrays; ++r) {
    const orc_ray_t& ray = rays[r];
    V3 o = v3(ray.org), d = v3(ray.dir);
    orc_hit_t h{ray.tmax, kMiss, 0.f, 0.f};
    uint8_t occ = 0;
    float best = ray.tmax;
    for (uint32_t p = 0; p < n_prims; ++p) {
      if (query == ORC_ANY) {
        if (test_prim_any(kind, mode, prims, p, o, d, ray.tmin, ray.tmax)) { occ = 1; break; }
      } else {
        float t, u, v;
        if (test_prim(kind, mode, prims, p, o, d, ray.tmin, best, t, u, v)) {
          best = t;
          h = {t, p, u, v};
        }
      }
    }
    if (hits) hits[r] = h;
    if (occluded) occluded[r] = occ;
  }
  return 0;
}

// random_double (main.cpp:503-508): a default-seeded std::mt19937 through
// uniform_real_distribution<double>(0, 1), in call order.
void orc_jitter_mt19937(uint64_t count, double* out) {
  std::mt19937 gen;
  std::uniform_real_distribution<double> dist(0.0, 1.0);
  for (uint64_t i = 0; i < count; ++i) out[i] = dist(gen);
}

// Primary rays of render() (main.cpp:544-557): fov hard-coded to 30 degrees,
// mixed double/float arithmetic, jitter pairs (x, y) per sample in y, x,
// sample order.
void orc_camera_rays_ref(uint32_t width, uint32_t height, uint32_t aa, const double* jitter,
                         orc_ray_t* rays) {
  float invWidth = 1 / float(width), invHeight = 1 / float(height);
  float fov = 30, aspectratio = width / float(height);
  float angle = (float)std::tan(3.141592653589793 * 0.5 * fov / 180.);
  size_t k = 0;
  for (uint32_t y = 0; y < height; ++y)
    for (uint32_t x = 0; x < width; ++x)
      for (uint32_t s = 0; s < aa; ++s, ++k) {
        double jx = jitter[2 * k], jy = jitter[2 * k + 1];
        float xx = (float)((2 * ((x + jx) * invWidth) - 1) * angle * aspectratio);
        float yy = (float)((1 - 2 * ((y + jy) * invHeight)) * angle);
        V3 d = normalize_ref({xx, yy, -1});
        rays[k] = {{0.f, 0.f, 0.f}, 0.f, {d.x, d.y, d.z}, INFINITY};
      }
}

// castRay's diffuse branch (main.cpp:390-497) for one point light at
// (0, 3, 30) with emission (1, 1, 1): trace_more is a stub returning false
// (main.cpp:235-245), so no light is ever shadowed.  kd_mode reproduces the
// KDTREE branch (main.cpp:362-372): black on any hit, background otherwise.
void orc_shade_ref(const float* sph, const float* surface_rgb, const orc_ray_t* rays,
                   const orc_hit_t* hits, uint32_t n, int kd_mode, const uint8_t* kd_any,
                   float* rgb) {
  const V3 bg = {0.6f, 0.8f, 1.0f};
  const V3 lc = {0.f, 3.f, 30.f};
  for (uint32_t r = 0; r < n; ++r) {
    V3 col;
    if (kd_mode) {
      col = kd_any[r] ? V3{0.f, 0.f, 0.f} : bg;
    } else if (hits[r].prim == kMiss) {
      col = bg;
    } else {
      const float* s = sph + 4 * (size_t)hits[r].prim;
      V3 o = v3(rays[r].org), d = v3(rays[r].dir);
      float tnear = hits[r].t;
      V3 hp = {o.x + d.x * tnear, o.y + d.y * tnear, o.z + d.z * tnear};
      V3 N = normalize_ref(sub(hp, v3(s)));
      if (dot(d, N) > 0) N = {-N.x, -N.y, -N.z};
      V3 L = normalize_ref(sub(lc, hp));
      float LdotN = std::max(0.f, dot(L, N));
      V3 lightAmt = {0.f + 1.0f * LdotN, 0.f + 1.0f * LdotN, 0.f + 1.0f * LdotN};
      V3 I = {-L.x, -L.y, -L.z};
      float k2 = 2 * dot(I, N);
      V3 R = {I.x - N.x * k2, I.y - N.y * k2, I.z - N.z * k2};
      float sp = powf(std::max(0.f, -dot(R, d)), 25);
      V3 spec = {0.f + 1.0f * sp, 0.f + 1.0f * sp, 0.f + 1.0f * sp};
      const V3 diff = {0.815f, 0.235f, 0.031f};
      V3 dd = {diff.x * 0.8f, diff.y * 0.8f, diff.z * 0.8f};
      V3 c;
      c.x = 0.f + (lightAmt.x * dd.x / 2.0f + spec.x * 0.5f);
      c.y = 0.f + (lightAmt.y * dd.y / 2.0f + spec.y * 0.5f);
      c.z = 0.f + (lightAmt.z * dd.z / 2.0f + spec.z * 0.5f);
      const float* sc = surface_rgb + 3 * (size_t)hits[r].prim;
      col = {c.x + sc[0], c.y + sc[1], c.z + sc[2]};
    }
    rgb[3 * (size_t)r] = col.x;
    rgb[3 * (size_t)r + 1] = col.y;
    rgb[3 * (size_t)r + 2] = col.z;
  }
}

// write_into_file (main.cpp:516-528): min(1, c / aa) * 255, truncated.
// rgb holds the per-pixel sums over samples.
void orc_pixels_ref(const float* rgb, uint32_t npix, uint32_t aa, uint8_t* out) {
  for (size_t i = 0; i < 3 * (size_t)npix; ++i)
    out[i] = (uint8_t)(std::min(float(1), rgb[i] / (float)aa) * 255);
}

}  // extern "C"

// ------------------------------------------------------------------------
// Render of a view: the engine's rq_render restated (camera, Lambert +
// ambient with one shadow ray, mirror bounces, pixel resolve).  It
// generalises castRay's DIFFUSE_AND_GLOSSY shading (main.cpp:390-497) to
// triangle meshes; every operation is one IEEE single-precision rounding in
// the engine's order (this file is compiled without contraction).

namespace {

struct F3v {
  float x, y, z;
};
inline F3v fadd(F3v a, F3v b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline F3v fsub(F3v a, F3v b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline F3v fmulv(F3v a, float s) { return {a.x * s, a.y * s, a.z * s}; }
inline float fdot(F3v a, F3v b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline F3v fcross(F3v a, F3v b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline F3v fnorm(F3v a) {
  float n2 = fdot(a, a);
  if (!(n2 > 0.f)) return a;
  float inv = 1.0f / std::sqrt(n2);
  return fmulv(a, inv);
}
inline F3v f3(const float* p) { return {p[0], p[1], p[2]}; }

// splitmix64 finaliser (Steele, Lea, Flood 2014), counter-based.
inline uint64_t mix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}
inline float jitter01(uint64_t seed, uint64_t sample, uint32_t dim) {
  uint64_t h = mix64(seed ^ mix64(sample * 2u + dim));
  return (float)(uint32_t)(h >> 40) * 0x1p-24f;
}

inline void put_ray(orc_ray_t& r, F3v o, float tmin, F3v d, float tmax) {
  r.org[0] = o.x; r.org[1] = o.y; r.org[2] = o.z; r.tmin = tmin;
  r.dir[0] = d.x; r.dir[1] = d.y; r.dir[2] = d.z; r.tmax = tmax;
}
inline void put_dead(orc_ray_t& r) { put_ray(r, {0.f, 0.f, 0.f}, 1.f, {0.f, 0.f, 1.f}, 0.f); }

}  // namespace

void orc_view_rays(const orc_view_t* v, orc_ray_t* rays, float* cw) {
  const uint64_t nray = (uint64_t)v->ww * v->wh * v->spp;
  const float aspect = (float)v->width / (float)v->height;
  const F3v eye = f3(v->eye);
  const F3v fwd = fnorm(fsub(f3(v->target), eye));
  const F3v right = fnorm(fcross(fwd, f3(v->up)));
  const F3v upv = fcross(right, fwd);
  for (uint64_t r = 0; r < nray; ++r) {
    const uint64_t wp = r / v->spp;
    const uint32_t s = (uint32_t)(r - wp * v->spp);
    const uint32_t x = v->x0 + (uint32_t)(wp % v->ww), y = v->y0 + (uint32_t)(wp / v->ww);
    const uint64_t sample = ((uint64_t)y * v->width + x) * v->spp + s;
    const float jx = jitter01(v->seed, sample, 0), jy = jitter01(v->seed, sample, 1);
    const float px = (2.0f * ((float(x) + jx) / float(v->width)) - 1.0f) * v->tan_half * aspect;
    const float py = (1.0f - 2.0f * ((float(y) + jy) / float(v->height))) * v->tan_half;
    const F3v d = fnorm(fadd(fadd(fwd, fmulv(right, px)), fmulv(upv, py)));
    put_ray(rays[r], eye, 0.f, d, INFINITY);
    cw[4 * r] = cw[4 * r + 1] = cw[4 * r + 2] = 0.f;
    cw[4 * r + 3] = 1.f;
  }
}

void orc_shade_hits(int kind, const float* verts, const uint32_t* idx, const float* sph, const orc_view_t* v,
                    uint64_t nray, int last, orc_ray_t* rays, const orc_hit_t* hits, orc_ray_t* shadow,
                    float* cw, float* pend, uint64_t* counters) {
  const F3v light = f3(v->light), albedo = f3(v->albedo), bg = f3(v->bg);
  uint64_t n_shadow = 0, n_mirror = 0;
  for (uint64_t r = 0; r < nray; ++r) {
    orc_ray_t& ray = rays[r];
    float* c = cw + 4 * r;
    float* pe = pend + 4 * r;
    pe[0] = pe[1] = pe[2] = pe[3] = 0.f;
    if (!(ray.tmin <= ray.tmax)) {
      put_dead(shadow[r]);
      continue;
    }
    const orc_hit_t& h = hits[r];
    const float w = c[3];
    if (h.prim == kMiss) {
      c[0] = c[0] + w * bg.x;
      c[1] = c[1] + w * bg.y;
      c[2] = c[2] + w * bg.z;
      c[3] = 0.f;
      put_dead(ray);
      put_dead(shadow[r]);
      continue;
    }
    const F3v o = f3(ray.org), d = f3(ray.dir);
    const F3v p = fadd(o, fmulv(d, h.t));
    F3v n;
    if (kind == ORC_TRIANGLES) {
      const uint32_t* t = idx + 3 * (size_t)h.prim;
      const F3v a = f3(verts + 3 * (size_t)t[0]), b = f3(verts + 3 * (size_t)t[1]), cc = f3(verts + 3 * (size_t)t[2]);
      n = fnorm(fcross(fsub(b, a), fsub(cc, a)));
    } else {
      n = fnorm(fsub(p, f3(sph + 4 * (size_t)h.prim)));
    }
    if (fdot(n, d) > 0.f) n = {-n.x, -n.y, -n.z};
    const F3v lv = fsub(light, p);
    const float dist = std::sqrt(fdot(lv, lv));
    const F3v ld = fmulv(lv, 1.0f / dist);
    const float ndl = fdot(n, ld);
    const float f = last ? w : w * (1.0f - v->mirror);
    const F3v fa = fmulv(albedo, f);
    c[0] = c[0] + fa.x * v->ambient;
    c[1] = c[1] + fa.y * v->ambient;
    c[2] = c[2] + fa.z * v->ambient;
    const F3v po = fadd(p, fmulv(n, v->bias));
    if (ndl > 0.f && dist > 0.f) {
      pe[0] = fa.x * ndl;
      pe[1] = fa.y * ndl;
      pe[2] = fa.z * ndl;
      put_ray(shadow[r], po, 0.f, ld, dist);
      ++n_shadow;
    } else {
      put_dead(shadow[r]);
    }
    const float wn = w * v->mirror;
    bool mirror = false;
    if (!last && wn > 0.f) {
      const F3v rd = fsub(d, fmulv(n, 2.0f * fdot(d, n)));
      put_ray(ray, po, 0.f, rd, INFINITY);
      mirror = true;
      ++n_mirror;
    } else {
      put_dead(ray);
    }
    c[3] = mirror ? wn : 0.f;
  }
  if (counters) {
    counters[0] += n_shadow;
    counters[1] += n_mirror;
  }
}

void orc_shadow_accum(uint64_t nray, const uint8_t* occluded, const float* pend, float* cw) {
  for (uint64_t r = 0; r < nray; ++r) {
    const float* p = pend + 4 * r;
    if (p[0] == 0.f && p[1] == 0.f && p[2] == 0.f) continue;
    if (occluded[r]) continue;
    cw[4 * r] = cw[4 * r] + p[0];
    cw[4 * r + 1] = cw[4 * r + 1] + p[1];
    cw[4 * r + 2] = cw[4 * r + 2] + p[2];
  }
}

void orc_view_pixels(uint64_t npix, uint32_t spp, const float* cw, uint8_t* pixels, float* rgb) {
  for (uint64_t p = 0; p < npix; ++p) {
    float s[3] = {0.f, 0.f, 0.f};
    for (uint32_t k = 0; k < spp; ++k) {
      const float* c = cw + 4 * (p * spp + k);
      s[0] = s[0] + c[0];
      s[1] = s[1] + c[1];
      s[2] = s[2] + c[2];
    }
    const float fs = (float)spp;
    for (int q = 0; q < 3; ++q) {
      float m = s[q] / fs;
      if (rgb) rgb[3 * p + q] = m;
      m = m < 1.f ? (m > 0.f ? m : 0.f) : 1.f;
      pixels[3 * p + q] = (uint8_t)(m * 255.f);
    }
  }
}
