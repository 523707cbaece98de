// rq_render — the reference program's flow (main.cpp:723-853) on the engine:
// load the scene the way createScene_new does, build the structure chosen by
// settings.dataStructure, render the 640x480 image and write it as P6.
//
//   rq_render [--model file.obj | --spheres file.xyzr | --models DIR --scene-model NAME]
//             [--structure BVH|KDTREE|LBVH|NONE] [--out output.ppm] [--width W]
//             [--height H] [--aa N] [--device D] [--dump-spheres file.xyzr]
//
// Without --model or --spheres the model is settings.sceneModel's file under
// --models (default "models"), as createScene_new picks it, with the name
// matched without regard to case.
// --spheres reads raw little-endian float32 (cx, cy, cz, r) records, the
// sphere list createScene_new produces.
#include <chrono>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include "rq.hpp"

namespace {

std::vector<rq::SphereRecord> read_spheres(const std::string& path) {
  std::ifstream f(path, std::ios::binary);
  if (!f.good()) throw rq::Error(RQ_ERROR_INVALID_ARGUMENT, "cannot open " + path);
  std::vector<rq::SphereRecord> out;
  rq::SphereRecord s;
  while (f.read(reinterpret_cast<char*>(&s), sizeof(s))) out.push_back(s);
  return out;
}

int structure_of(const std::string& name) {
  if (name == "BVH") return rq::BVH;
  if (name == "KDTREE") return rq::KDTREE;
  if (name == "UNIFORM_GRID") return rq::UNIFORM_GRID;
  if (name == "LBVH") return rq::LBVH;
  if (name == "NONE") return rq::NONE;
  throw rq::Error(RQ_ERROR_INVALID_ARGUMENT, "unknown structure " + name);
}

// SceneModel names (settings.h:4).
int scene_model_of(const std::string& name) {
  const char* names[] = {"IGEA", "ARMADILLO", "BUNNY", "BUNNIES", "TEST", "GRASS", "BUDDHA", "CITY"};
  for (int k = 0; k < 8; ++k)
    if (name == names[k]) return k;
  throw rq::Error(RQ_ERROR_INVALID_ARGUMENT, "unknown scene model " + name);
}

double seconds_since(std::chrono::steady_clock::time_point t0) {
  return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

}  // namespace

int main(int argc, char** argv) {
  std::string model, spheres_path, dump, out = "output.ppm", models_dir = "models";
  rq::Settings settings;
  int device = 0;
  for (int i = 1; i < argc; ++i) {
    std::string a = argv[i];
    auto next = [&]() -> std::string {
      if (i + 1 >= argc) throw rq::Error(RQ_ERROR_INVALID_ARGUMENT, "missing value for " + a);
      return argv[++i];
    };
    if (a == "--model") model = next();
    else if (a == "--spheres") spheres_path = next();
    else if (a == "--structure") settings.dataStructure = structure_of(next());
    else if (a == "--out") out = next();
    else if (a == "--width") settings.width = (uint32_t)std::stoul(next());
    else if (a == "--height") settings.height = (uint32_t)std::stoul(next());
    else if (a == "--aa") settings.aa_samples = (uint32_t)std::stoul(next());
    else if (a == "--device") device = std::stoi(next());
    else if (a == "--dump-spheres") dump = next();  // write the loaded sphere list and stop
    else if (a == "--models") models_dir = next();
    else if (a == "--scene-model") settings.sceneModel = scene_model_of(next());
    else {
      std::cerr << "unknown argument " << a << "\n";
      return 2;
    }
  }
  try {
    auto t0 = std::chrono::steady_clock::now();
    if (spheres_path.empty() && model.empty()) model = rq::modelPath(models_dir, settings.sceneModel);
    std::vector<rq::SphereRecord> spheres =
        !spheres_path.empty() ? read_spheres(spheres_path) : rq::loadReferenceScene(model);
    std::cout << "Number of spheres: " << spheres.size() << "\n";
    if (!dump.empty()) {
      std::ofstream f(dump, std::ios::binary);
      f.write(reinterpret_cast<const char*>(spheres.data()), (std::streamsize)(spheres.size() * sizeof(spheres[0])));
      return 0;
    }
    settings.traversal = RQ_TRAVERSAL_REFERENCE;
    rq::Context ctx(settings, device);
    rq::Scene scene = rq::Scene::spheres(ctx, spheres);
    std::cout << "Scene upload: " << seconds_since(t0) << "s\n";
    auto t1 = std::chrono::steady_clock::now();
    rq::Accel accel = rq::build(ctx, scene, settings.dataStructure);
    rq_accel_info_t info = accel.info();
    std::cout << "Build (" << settings.dataStructure << "): " << seconds_since(t1) << "s, nodes " << info.n_nodes
              << "\n";
    auto t2 = std::chrono::steady_clock::now();
    std::vector<uint8_t> px = rq::render(ctx, accel, settings, rq::referenceSurfaceColors(spheres.size()));
    std::cout << "Render: " << seconds_since(t2) << "s\n";
    rq::write_ppm(out, settings, px);
    std::cout << "Wrote " << out << "\n";
  } catch (const rq::Error& e) {
    std::cerr << "error: " << e.what() << "\n";
    return 1;
  }
  return 0;
}
