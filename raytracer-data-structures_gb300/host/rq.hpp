// rq.hpp — C++ host interface over the C ABI (include/rq.h), shaped like the
// reference ray tracer's own interface (project/raytracer/settings.h,
// accelerators.h, main.cpp) so that its call sites map one to one:
//
//   Settings settings;                        settings.h:7-17 (same fields/defaults)
//   AccType  BVH, KDTREE, UNIFORM_GRID, LBVH, NONE      accelerators.h:21
//   build(ctx, scene, settings.dataStructure) the switch in main() (main.cpp:791-843)
//   constructBVHNew / constructLBVHTree / constructKDTreeNew   accelerators.h:246,570,951
//   boxIntersect -> boxIntersect / candidates (candidate ids, accelerators.h:668)
//   boxIntersect + castRay's closest selection -> closestHits  (accelerators.h:668, main.cpp:330-358)
//   kdtreeIntersect -> anyHits                                  (accelerators.h:997)
//   render + write_into_file -> render / write_ppm              (main.cpp:541-566, 516-528)
//
// Header-only; link with librq.so.  Errors throw rq::Error carrying the
// engine's status and message (the reference has no error reporting at all).
#pragma once

#include <cstdint>
#include <cstdio>
#include <fstream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "rq.h"

namespace rq {

enum AccType { BVH = RQ_BVH, KDTREE = RQ_KDTREE, UNIFORM_GRID = RQ_UNIFORM_GRID, LBVH = RQ_LBVH, NONE = RQ_NONE };

struct Settings : rq_settings_t {
  Settings() { rq_settings_default(this); }
};

class Error : public std::runtime_error {
 public:
  Error(rq_status_t s, const std::string& what) : std::runtime_error(what), status(s) {}
  rq_status_t status;
};

inline void check(rq_status_t s, rq_ctx_t ctx) {
  if (s != RQ_SUCCESS)
    throw Error(s, std::string(rq_status_string(s)) + (ctx ? std::string(": ") + rq_last_error(ctx) : ""));
}

class Context {
 public:
  explicit Context(const Settings& s = Settings(), int device = 0) {
    check(rq_create(&s, device, &h_), nullptr);
  }
  ~Context() {
    if (h_) rq_destroy(h_);
  }
  Context(const Context&) = delete;
  Context& operator=(const Context&) = delete;
  rq_ctx_t get() const { return h_; }
  void setSettings(const Settings& s) { check(rq_set_settings(h_, &s), h_); }

 private:
  rq_ctx_t h_ = nullptr;
};

// One sphere per SceneObject (centre, radius), as createScene_new builds them.
struct SphereRecord {
  float center[3];
  float radius;
};

class Scene {
 public:
  static Scene spheres(Context& c, const std::vector<SphereRecord>& s) {
    Scene out(c);
    check(rq_scene_create_spheres(c.get(), &s[0].center[0], (uint32_t)s.size(), 0, &out.h_), c.get());
    out.n_ = (uint32_t)s.size();
    return out;
  }
  static Scene triangles(Context& c, const std::vector<float>& verts, const std::vector<uint32_t>& idx) {
    Scene out(c);
    check(rq_scene_create_triangles(c.get(), verts.data(), (uint32_t)(verts.size() / 3), idx.data(),
                                    (uint32_t)(idx.size() / 3), 0, &out.h_),
          c.get());
    out.n_ = (uint32_t)(idx.size() / 3);
    return out;
  }
  Scene(Scene&& o) noexcept : c_(o.c_), h_(o.h_), n_(o.n_) { o.h_ = nullptr; }
  ~Scene() {
    if (h_) rq_scene_destroy(h_);
  }
  rq_scene_t get() const { return h_; }
  uint32_t size() const { return n_; }

 private:
  explicit Scene(Context& c) : c_(&c) {}
  Context* c_;
  rq_scene_t h_ = nullptr;
  uint32_t n_ = 0;
};

class Accel {
 public:
  Accel(Context& c, const Scene& s, int acc_type) : c_(&c) { check(rq_build(c.get(), s.get(), acc_type, &h_), c.get()); }
  Accel(Accel&& o) noexcept : c_(o.c_), h_(o.h_) { o.h_ = nullptr; }
  ~Accel() {
    if (h_) rq_accel_destroy(h_);
  }
  rq_accel_t get() const { return h_; }
  rq_accel_info_t info() const {
    rq_accel_info_t i;
    check(rq_accel_get_info(h_, &i), c_->get());
    return i;
  }

  // Closest hit of every ray (boxIntersect + castRay's selection, batched).
  std::vector<rq_hit_t> closestHits(const std::vector<rq_ray_t>& rays) const {
    std::vector<rq_hit_t> hits(rays.size());
    if (!rays.empty()) check(rq_trace_closest(c_->get(), h_, rays.data(), (uint32_t)rays.size(), hits.data(), 0), c_->get());
    return hits;
  }
  // Any hit of every ray (kdtreeIntersect / shadow queries, batched).
  std::vector<bool> anyHits(const std::vector<rq_ray_t>& rays) const {
    std::vector<uint32_t> bits((rays.size() + 31) / 32);
    if (!rays.empty()) check(rq_trace_any(c_->get(), h_, rays.data(), (uint32_t)rays.size(), bits.data(), 0), c_->get());
    std::vector<bool> out(rays.size());
    for (size_t r = 0; r < rays.size(); ++r) out[r] = (bits[r >> 5] >> (r & 31)) & 1u;
    return out;
  }
  // boxIntersect (accelerators.h:668-690) for a batch: each ray's candidate
  // primitive ids in the reference's pre-order, concatenated; counts per ray.
  void candidates(const std::vector<rq_ray_t>& rays, std::vector<uint32_t>& counts,
                  std::vector<uint32_t>& ids) const {
    counts.assign(rays.size(), 0);
    ids.clear();
    if (rays.empty()) return;
    uint64_t total = 0;
    check(rq_trace_candidates(c_->get(), h_, rays.data(), (uint32_t)rays.size(), counts.data(), nullptr, 0, &total, 0),
          c_->get());
    ids.resize(total);
    check(rq_trace_candidates(c_->get(), h_, rays.data(), (uint32_t)rays.size(), counts.data(), ids.data(), total,
                              &total, 0),
          c_->get());
  }
  // The reference's signature: append the candidate ids of one ray to boxes
  // (one device round trip per call: batch with candidates() where possible).
  void boxIntersect(const float pos[3], const float dir[3], std::vector<int>& boxes) const {
    std::vector<rq_ray_t> r(1, rq_ray_t{{pos[0], pos[1], pos[2]}, 0.f, {dir[0], dir[1], dir[2]}, __builtin_inff()});
    std::vector<uint32_t> counts, ids;
    candidates(r, counts, ids);
    for (uint32_t id : ids) boxes.push_back((int)id);
  }
  // One ray at a time, the shape of the reference's per-ray calls (each is a
  // device round trip: batch with closestHits/anyHits where possible).
  bool closestHit(const float pos[3], const float dir[3], rq_hit_t& hit) const {
    rq_ray_t r = {{pos[0], pos[1], pos[2]}, 0.f, {dir[0], dir[1], dir[2]}, __builtin_inff()};
    check(rq_trace_closest(c_->get(), h_, &r, 1, &hit, 0), c_->get());
    return hit.prim != RQ_MISS;
  }
  bool kdtreeIntersect(const float pos[3], const float dir[3]) const {
    rq_ray_t r = {{pos[0], pos[1], pos[2]}, 0.f, {dir[0], dir[1], dir[2]}, __builtin_inff()};
    uint32_t bit = 0;
    check(rq_trace_any(c_->get(), h_, &r, 1, &bit, 0), c_->get());
    return bit & 1u;
  }

 private:
  Context* c_;
  rq_accel_t h_ = nullptr;
};

// The builders under the reference's names.
inline Accel constructBVHNew(Context& c, const Scene& s) { return Accel(c, s, BVH); }
inline Accel constructLBVHTree(Context& c, const Scene& s) { return Accel(c, s, LBVH); }
inline Accel constructKDTreeNew(Context& c, const Scene& s) { return Accel(c, s, KDTREE); }
// main()'s switch on settings.dataStructure.
inline Accel build(Context& c, const Scene& s, int dataStructure) { return Accel(c, s, dataStructure); }

// createScene_new's loader (main.cpp:650-718): every `v x y z` line up to the
// first other token becomes a sphere of radius 0.05 at v*100 + (0,-10,-60)
// (+20 per clone), then the ground sphere of radius 100 is appended
// (rq_reference_spheres).
inline std::vector<SphereRecord> loadReferenceScene(const std::string& objPath, int clones = 1) {
  float* p = nullptr;
  uint32_t n = 0;
  rq_status_t st = rq_reference_spheres(objPath.c_str(), clones, &p, &n);
  if (st != RQ_SUCCESS) throw Error(st, "cannot load " + objPath);
  std::vector<SphereRecord> out(n);
  for (uint32_t i = 0; i < n; ++i)
    out[i] = SphereRecord{{p[4 * i], p[4 * i + 1], p[4 * i + 2]}, p[4 * i + 3]};
  rq_free(p);
  return out;
}

// createScene_new's model file for settings.sceneModel under `dir`, the name
// matched without regard to case (rq_model_path).
inline std::string modelPath(const std::string& dir, int sceneModel) {
  char buf[4096];
  rq_status_t st = rq_model_path(dir.c_str(), sceneModel, buf, sizeof(buf));
  if (st != RQ_SUCCESS) throw Error(st, "no model file in " + dir);
  return buf;
}

// A triangle mesh read from / written to a Wavefront OBJ file (v / f records).
struct Mesh {
  std::vector<float> verts;    // nv * 3
  std::vector<uint32_t> idx;   // nt * 3
};
inline Mesh loadObj(const std::string& path) {
  float* v = nullptr;
  uint32_t* f = nullptr;
  uint32_t nv = 0, nt = 0;
  rq_status_t st = rq_obj_load(path.c_str(), &v, &nv, &f, &nt);
  if (st != RQ_SUCCESS) throw Error(st, "cannot load " + path);
  Mesh m;
  m.verts.assign(v, v + (size_t)nv * 3);
  m.idx.assign(f, f + (size_t)nt * 3);
  rq_free(v);
  rq_free(f);
  return m;
}
inline void saveObj(const std::string& path, const Mesh& m) {
  rq_status_t st = rq_obj_save(path.c_str(), m.verts.data(), (uint32_t)(m.verts.size() / 3), m.idx.data(),
                               (uint32_t)(m.idx.size() / 3));
  if (st != RQ_SUCCESS) throw Error(st, "cannot save " + path);
}

// Surface colours of those spheres: (0.8, 0.7, 0) per vertex sphere
// (main.cpp:689), black for the ground (main.cpp:703).
inline std::vector<float> referenceSurfaceColors(size_t n) {
  std::vector<float> c(3 * n);
  for (size_t i = 0; i + 1 < n; ++i) {
    c[3 * i] = 0.8f;
    c[3 * i + 1] = 0.7f;
    c[3 * i + 2] = 0.f;
  }
  return c;
}

// render(): pixels of the P6 image (width*height*3 bytes).
inline std::vector<uint8_t> render(Context& c, const Accel& a, const Settings& s, const std::vector<float>& surface) {
  std::vector<uint8_t> px((size_t)s.width * s.height * 3);
  check(rq_render_reference(c.get(), a.get(), &s, nullptr, surface.data(), px.data(), nullptr), c.get());
  return px;
}

// write_into_file(): P6 header + payload.
inline void write_ppm(const std::string& path, const Settings& s, const std::vector<uint8_t>& px) {
  std::ofstream ofs(path, std::ios::out | std::ios::binary);
  ofs << "P6\n" << s.width << " " << s.height << "\n255\n";
  ofs.write(reinterpret_cast<const char*>(px.data()), (std::streamsize)px.size());
}

}  // namespace rq
