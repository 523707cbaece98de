// ref_dump — golden-vector generator built from the reference ray tracer's own
// sources (project/raytracer/main.cpp + accelerators.h), compiled unchanged
// with main() renamed.  Test infrastructure only: it is built by
// oracle/Makefile into oracle/_ref/ (never committed) in a container that
// holds the reference tree, and its outputs become the committed fixtures
// under tests/golden/ (see tests/golden/make_golden.py).
//
// Every dumped quantity comes from a reference function:
//   morton3D / expandBits              accelerators.h:374-394
//   centroid normalisation (c+30)/1000 accelerators.h:577
//   constructBVHNew                    accelerators.h:246-337
//   constructLBVHTree                  accelerators.h:570-586
//   constructKDTreeNew / buildTree     accelerators.h:815-988
//   boxIntersect                       accelerators.h:668-690
//   kdtreeIntersect                    accelerators.h:997-1086
//   raySphereIntersect                 accelerators.h:79-92
//   closest-hit candidate selection    main.cpp:339-358 (restated below, 10 lines)
//   castRay                            main.cpp:291-500
//   render / write_into_file           main.cpp:516-566
//   createScene_new                    main.cpp:599-721
//   random_double                      main.cpp:503-508
//
// Output: raw little-endian arrays, one file per quantity, plus meta.txt.
#include <cstdint>
#include <memory>
#include <unistd.h>
#define main ref_program_main
#include "main.cpp"
#undef main

#include <cstdio>
#include <string>
#include <vector>

namespace {

std::string g_out;

template <typename T>
void dump(const char* name, const std::vector<T>& v) {
  std::string p = g_out + "/" + name + ".bin";
  FILE* f = std::fopen(p.c_str(), "wb");
  if (!f) { std::perror(p.c_str()); std::exit(2); }
  if (!v.empty()) std::fwrite(v.data(), sizeof(T), v.size(), f);
  std::fclose(f);
}

FILE* g_meta = nullptr;
void meta(const char* key, long long v) { std::fprintf(g_meta, "%s %lld\n", key, v); }

// Scene object exactly as createScene_new builds one (main.cpp:677-692).
SceneObject make_object(int id, Vec3f center, float radius) {
  SceneObject s;
  s.objId = id;
  s.radius = radius;
  s.center = center;
  s.position = s.center;
  s.shininess = 64;
  s.isSphere = true;
  Vec3f minPoint = s.center - s.radius;
  Vec3f maxPoint = s.center + s.radius;
  s.boxBoundries = BoxBoundries(minPoint, maxPoint);
  s.sphere = Sphere(id, s.center, s.radius, Vec3f(0.8, 0.7, 0), 0, 0.0, REFLECTION_AND_REFRACTION);
  return s;
}

// Pre-order walk of the reference's shared_ptr BVH.  Per node: 6 bounds
// floats, then (isleaf, first, count, left, right) into the int stream; leaf
// object ids go to `objs`.
struct TreeDump {
  std::vector<float> bounds;
  std::vector<int32_t> info;
  std::vector<int32_t> objs;
};
int walk(const std::shared_ptr<Node>& n, TreeDump& d) {
  int me = (int)(d.info.size() / 5);
  const BoxBoundries& b = n->boxBoundries;
  float bb[6] = {b.min.x, b.min.y, b.min.z, b.max.x, b.max.y, b.max.z};
  d.bounds.insert(d.bounds.end(), bb, bb + 6);
  d.info.insert(d.info.end(), {0, 0, 0, -1, -1});
  if (n->isleaf) {
    d.info[me * 5 + 0] = 1;
    d.info[me * 5 + 1] = (int)d.objs.size();
    d.info[me * 5 + 2] = (int)n->objs.size();
    for (unsigned o : n->objs) d.objs.push_back((int)o);
  } else {
    int l = walk(n->leftchild, d);
    int r = walk(n->rightchild, d);
    d.info[me * 5 + 3] = l;
    d.info[me * 5 + 4] = r;
  }
  return me;
}

void dump_tree(const char* prefix, const std::shared_ptr<Node>& root) {
  TreeDump d;
  walk(root, d);
  std::string p(prefix);
  dump((p + "_bounds").c_str(), d.bounds);
  dump((p + "_info").c_str(), d.info);
  dump((p + "_objs").c_str(), d.objs);
  meta((p + "_nodes").c_str(), (long long)(d.info.size() / 5));
}

// Closest hit through a reference BVH: candidates from boxIntersect, then
// the selection loop of castRay (main.cpp:339-358).
void bvh_closest(const Vec3f& o, const Vec3f& dir, std::shared_ptr<Node>& root,
                 int32_t& id, float& t) {
  std::vector<int> boxes;
  boxIntersect(o, dir, root, boxes);
  float tnear = INFINITY;
  id = -1;
  for (int box : boxes) {
    float t0 = INFINITY, t1 = INFINITY;
    if (sceneFixed[box].sphere.raySphereIntersect(o, dir, t0, t1)) {
      if (t0 < 0) t0 = t1;
      if (t0 < tnear) { tnear = t0; id = box; }
    }
  }
  t = tnear;
}

// Brute-force closest hit, the NONE branch of castRay (main.cpp:373-387).
void none_closest(const Vec3f& o, const Vec3f& dir, int32_t& id, float& t) {
  float tnear = INFINITY;
  id = -1;
  for (unsigned i = 0; i < sceneFixed.size(); ++i) {
    float t0 = INFINITY, t1 = INFINITY;
    if (sceneFixed[i].sphere.raySphereIntersect(o, dir, t0, t1)) {
      if (t0 < 0) t0 = t1;
      if (t0 < tnear) { tnear = t0; id = (int)i; }
    }
  }
  t = tnear;
}

uint64_t g_lcg = 0;
double lcg01() {  // harness-only input generator (64-bit LCG, top 53 bits)
  g_lcg = g_lcg * 6364136223846793005ULL + 1442695040888963407ULL;
  return (double)(g_lcg >> 11) * (1.0 / 9007199254740992.0);
}

void run_known() {
  // Points on and around the unit cube, including exact cell boundaries.
  std::vector<float> pts;
  std::vector<uint32_t> codes, expand_in, expand_out;
  const float specials[] = {0.f, 1.f, 0.5f, -0.25f, 1.25f, 1.0f / 1024.f, 1023.0f / 1024.f,
                            0.99999994f, 1e-7f, -0.f, 0.0009765625f, 0.3f};
  for (float a : specials)
    for (float b : specials)
      for (float c : specials) pts.insert(pts.end(), {a, b, c});
  g_lcg = 12345;
  for (int i = 0; i < 8192; ++i)
    pts.insert(pts.end(), {(float)(lcg01() * 1.4 - 0.2), (float)(lcg01() * 1.4 - 0.2),
                           (float)(lcg01() * 1.4 - 0.2)});
  for (size_t i = 0; i < pts.size(); i += 3) codes.push_back(morton3D(pts[i], pts[i + 1], pts[i + 2]));
  for (uint32_t v = 0; v < 1024; ++v) { expand_in.push_back(v); expand_out.push_back(expandBits(v)); }
  dump("known_pts", pts);
  dump("known_codes", codes);
  dump("expand_in", expand_in);
  dump("expand_out", expand_out);
  meta("known_n", (long long)codes.size());
}

// Scene-level dumps shared by the bunny and synthetic scenes.  Must be called
// with sceneFixed == scene (castRay and the candidate loop index it).
void dump_scene_structures(std::vector<SceneObject>& scene) {
  const size_t n = scene.size();
  std::vector<float> sph;
  for (auto& s : scene) sph.insert(sph.end(), {s.center.x, s.center.y, s.center.z, s.radius});
  dump("spheres", sph);
  meta("n_spheres", (long long)n);

  // Morton codes with the reference's normalisation (accelerators.h:576-580).
  std::vector<uint32_t> codes(n);
  for (size_t i = 0; i < n; ++i) {
    Vec3f centroid = (scene[i].center + 30) / 1000;
    codes[i] = morton3D(centroid.x, centroid.y, centroid.z);
  }
  dump("morton", codes);
}

std::shared_ptr<Node> g_bvh, g_lbvh;

void build_all(std::vector<SceneObject>& scene, bool do_lbvh) {
  {
    std::vector<SceneObject> work = scene;
    int totalNodes = 0;
    g_bvh = constructBVHNew(work, 0, (int)work.size(), &totalNodes);
    meta("bvh_totalNodes", totalNodes);
    dump_tree("bvh", g_bvh);
  }
  if (do_lbvh) {
    std::vector<SceneObject> work = scene;
    std::vector<std::shared_ptr<Node>> nodes;
    std::shared_ptr<Node> root = std::make_shared<Node>();
    g_lbvh = constructLBVHTree(work, root, nodes);
    dump_tree("lbvh", g_lbvh);
  }
  {
    constructKDTreeNew(scene, 80, 1, 0.5f, 1, -1);
    // KdAccelNode is three 32-bit words: {split|onePrimitive|offset,
    // flags|nPrims|aboveChild, nPrimitivesTest}.  The third word is only
    // initialised for leaves; interior nodes get 0 here.
    std::vector<int32_t> kd(3 * (size_t)nextFreeNode);
    for (int i = 0; i < nextFreeNode; ++i) {
      int32_t w[3];
      std::memcpy(w, &nodes[i], sizeof(w));
      if ((w[1] & 3) != 3) w[2] = 0;
      kd[3 * i + 0] = w[0];
      kd[3 * i + 1] = w[1];
      kd[3 * i + 2] = w[2];
    }
    dump("kd_nodes", kd);
    std::vector<int32_t> pi(kdtreePrimitiveIndices.begin(), kdtreePrimitiveIndices.end());
    dump("kd_prim_indices", pi);
    std::vector<float> kb = {bounds.min.x, bounds.min.y, bounds.min.z,
                             bounds.max.x, bounds.max.y, bounds.max.z};
    dump("kd_root_bounds", kb);
    meta("kd_nodes", nextFreeNode);
    meta("kd_totalKdNodes", totalKdNodes);
    int maxDepth = std::round(8 + 1.3f * Log2Int(int64_t(scene.size())));
    meta("kd_maxDepth", maxDepth);
  }
}

// Per-ray queries through every reference structure.
void trace_all(const std::vector<float>& rays, size_t nrays, bool do_lbvh,
               const std::vector<int32_t>& none_sel, bool colors,
               std::vector<Sphere>& spheres, std::vector<Sphere>& lights,
               std::vector<SceneObject>& scene) {
  std::vector<int32_t> bid(nrays), lid(do_lbvh ? nrays : 0);
  std::vector<float> bt(nrays), lt(do_lbvh ? nrays : 0);
  std::vector<uint8_t> kd(nrays);
  std::vector<float> col;
  Settings settings;
  int start_tests = spheres_intersections_counter;
  for (size_t r = 0; r < nrays; ++r) {
    Vec3f o(rays[6 * r + 0], rays[6 * r + 1], rays[6 * r + 2]);
    Vec3f d(rays[6 * r + 3], rays[6 * r + 4], rays[6 * r + 5]);
    bvh_closest(o, d, g_bvh, bid[r], bt[r]);
  }
  meta("bvh_sphere_tests", spheres_intersections_counter - start_tests);
  if (do_lbvh)
    for (size_t r = 0; r < nrays; ++r) {
      Vec3f o(rays[6 * r + 0], rays[6 * r + 1], rays[6 * r + 2]);
      Vec3f d(rays[6 * r + 3], rays[6 * r + 4], rays[6 * r + 5]);
      bvh_closest(o, d, g_lbvh, lid[r], lt[r]);
    }
  start_tests = spheres_intersections_counter;
  for (size_t r = 0; r < nrays; ++r) {
    Vec3f o(rays[6 * r + 0], rays[6 * r + 1], rays[6 * r + 2]);
    Vec3f d(rays[6 * r + 3], rays[6 * r + 4], rays[6 * r + 5]);
    kd[r] = kdtreeIntersect(o, d) ? 1 : 0;
  }
  meta("kd_sphere_tests", spheres_intersections_counter - start_tests);
  std::vector<int32_t> nid(none_sel.size());
  std::vector<float> nt(none_sel.size());
  for (size_t k = 0; k < none_sel.size(); ++k) {
    size_t r = (size_t)none_sel[k];
    Vec3f o(rays[6 * r + 0], rays[6 * r + 1], rays[6 * r + 2]);
    Vec3f d(rays[6 * r + 3], rays[6 * r + 4], rays[6 * r + 5]);
    none_closest(o, d, nid[k], nt[k]);
  }
  if (colors) {
    settings.dataStructure = BVH;
    col.resize(3 * nrays);
    for (size_t r = 0; r < nrays; ++r) {
      Vec3f o(rays[6 * r + 0], rays[6 * r + 1], rays[6 * r + 2]);
      Vec3f d(rays[6 * r + 3], rays[6 * r + 4], rays[6 * r + 5]);
      Vec3f c = castRay(o, d, spheres, lights, scene, g_bvh, 1, settings);
      col[3 * r + 0] = c.x; col[3 * r + 1] = c.y; col[3 * r + 2] = c.z;
    }
  }
  dump("bvh_hit_id", bid);
  dump("bvh_hit_t", bt);
  if (do_lbvh) { dump("lbvh_hit_id", lid); dump("lbvh_hit_t", lt); }
  dump("kd_any", kd);
  dump("none_sel", none_sel);
  dump("none_hit_id", nid);
  dump("none_hit_t", nt);
  if (colors) dump("bvh_color", col);
}

void scene_lights(std::vector<Sphere>& spheres, std::vector<Sphere>& lights) {
  // Same light and decoy spheres as main() (main.cpp:775-788).
  lights.push_back(Sphere(0, Vec3f(0, 3, 30), 10, Vec3f(1, 1, 1), 0, 0.0, Vec3f(1)));
  spheres.push_back(Sphere(0, Vec3f(-5, 0, -20), 2, Vec3f(0.1, 0.4, 0.6), 1, 0.0));
}

// Bunny scene through createScene_new, camera rays exactly as render()
// generates them (main.cpp:544-557), starting from a fresh mt19937.
void run_bunny(const char* refdir) {
  if (chdir(refdir) != 0) { std::perror(refdir); std::exit(2); }
  Settings settings;
  std::vector<SceneObject> scene = createScene_new(settings);
  dump_scene_structures(scene);
  build_all(scene, true);

  const unsigned W = settings.width, H = settings.height;
  std::vector<float> rays;
  rays.reserve((size_t)W * H * 6);
  std::vector<double> jitter;
  float invWidth = 1 / float(settings.width), invHeight = 1 / float(settings.height);
  float fov = 30, aspectratio = settings.width / float(settings.height);
  float angle = tan(M_PI * 0.5 * fov / 180.);
  for (unsigned y = 0; y < H; ++y)
    for (unsigned x = 0; x < W; ++x)
      for (unsigned sample = 0; sample < settings.aa_samples; ++sample) {
        double jx = random_double();
        float xx = (2 * ((x + jx) * invWidth) - 1) * angle * aspectratio;
        double jy = random_double();
        float yy = (1 - 2 * ((y + jy) * invHeight)) * angle;
        Vec3f raydir(xx, yy, -1);
        raydir.normalize();
        rays.insert(rays.end(), {0.f, 0.f, 0.f, raydir.x, raydir.y, raydir.z});
        jitter.push_back(jx);
        jitter.push_back(jy);
      }
  dump("jitter", jitter);
  dump("rays", rays);
  // NONE on the 64x48 crop centred on the image (3,072 rays).
  std::vector<int32_t> sel;
  for (unsigned y = 216; y < 264; ++y)
    for (unsigned x = 288; x < 352; ++x) sel.push_back((int32_t)(y * W + x));
  std::vector<Sphere> spheres, lights;
  scene_lights(spheres, lights);
  trace_all(rays, (size_t)W * H, true, sel, true, spheres, lights, scene);
}

// Seeded synthetic sphere cloud: n spheres, centres uniform in a box chosen so
// that (c+30)/1000 spans part of [0,1], radii in [rmin, rmax]; rays from
// points around the cloud toward points inside it.
void run_synth(int n, uint64_t seed, int nrays, int lbvh) {
  g_lcg = seed;
  std::vector<SceneObject> scene;
  for (int i = 0; i < n; ++i) {
    Vec3f c((float)(lcg01() * 200.0 - 40.0), (float)(lcg01() * 120.0 - 20.0),
            (float)(lcg01() * 160.0 - 30.0));
    float r = (float)(0.05 + lcg01() * 2.0);
    scene.push_back(make_object(i, c, r));
  }
  sceneFixed = scene;
  dump_scene_structures(scene);
  build_all(scene, lbvh != 0);
  std::vector<float> rays;
  for (int k = 0; k < nrays; ++k) {
    float ox = (float)(lcg01() * 400.0 - 140.0), oy = (float)(lcg01() * 300.0 - 110.0),
          oz = (float)(lcg01() * 360.0 - 130.0);
    float tx = (float)(lcg01() * 200.0 - 40.0), ty = (float)(lcg01() * 120.0 - 20.0),
          tz = (float)(lcg01() * 160.0 - 30.0);
    Vec3f d(tx - ox, ty - oy, tz - oz);
    d.normalize();
    rays.insert(rays.end(), {ox, oy, oz, d.x, d.y, d.z});
  }
  dump("rays", rays);
  std::vector<int32_t> sel;
  for (int k = 0; k < nrays; ++k) sel.push_back(k);
  std::vector<Sphere> spheres, lights;
  scene_lights(spheres, lights);
  trace_all(rays, (size_t)nrays, lbvh != 0, sel, false, spheres, lights, scene);
}

// The reference program's own flow for one dataStructure (main.cpp:751-843):
// load the bunny, build, render into <outdir>/output.ppm.
void run_render(const char* refdir, int acc) {
  if (chdir(refdir) != 0) { std::perror(refdir); std::exit(2); }
  Settings settings;
  settings.dataStructure = (AccType)acc;
  std::vector<SceneObject> scene = createScene_new(settings);
  if (chdir(g_out.c_str()) != 0) { std::perror(g_out.c_str()); std::exit(2); }
  std::vector<Sphere> spheres, lights;
  std::vector<Triangle> triangles;
  lights.push_back(Sphere(0, Vec3f(0, 3, 30), 10, Vec3f(1, 1, 1), 0, 0.0, Vec3f(1)));
  std::shared_ptr<Node> root = std::make_shared<Node>();
  std::vector<std::shared_ptr<Node>> nodes;
  int totalNodes = 0;
  switch (settings.dataStructure) {
    case BVH: root = constructBVHNew(scene, 0, scene.size(), &totalNodes); break;
    case KDTREE: constructKDTreeNew(scene, 80, 1, 0.5f, 1, -1); break;
    case LBVH: root = constructLBVHTree(scene, root, nodes); break;
    default: break;
  }
  render(settings, spheres, lights, triangles, 15, scene, root);
  meta("render_sphere_tests", spheres_intersections_counter);
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 3) {
    std::fprintf(stderr,
                 "usage: ref_dump known <out> | bunny <out> <refdir> | "
                 "synth <out> <n> <seed> <nrays> <lbvh> | render <out> <refdir> <acc>\n");
    return 2;
  }
  std::string mode = argv[1];
  char resolved[4096];
  if (!realpath(argv[2], resolved)) { std::perror(argv[2]); return 2; }
  g_out = resolved;
  g_meta = std::fopen((g_out + "/meta.txt").c_str(), "w");
  if (!g_meta) { std::perror("meta"); return 2; }
  if (mode == "known") run_known();
  else if (mode == "bunny" && argc >= 4) run_bunny(argv[3]);
  else if (mode == "synth" && argc >= 7)
    run_synth(std::atoi(argv[3]), std::strtoull(argv[4], nullptr, 10), std::atoi(argv[5]), std::atoi(argv[6]));
  else if (mode == "render" && argc >= 5) run_render(argv[3], std::atoi(argv[4]));
  else { std::fprintf(stderr, "bad mode\n"); return 2; }
  std::fclose(g_meta);
  return 0;
}
