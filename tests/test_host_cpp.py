"""The C++ host side above the C ABI (raytracer-data-structures_gb300/host):
rq.hpp mirrors the reference's Settings / AccType / builder / query names and
rq_render reproduces the reference program's flow (load, build by
dataStructure, render, write P6)."""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT, golden

PKG = os.path.join(ROOT, "raytracer-data-structures_gb300")
DRIVER = os.path.join(PKG, "rq_render")
REF_BUNNY = os.path.join(os.environ.get("REF_ROOT", "/root/reference"), "project", "raytracer", "models", "bunny.obj")


@pytest.fixture(scope="module")
def driver():
    import rq
    rq.load()  # builds librq.so and the driver when missing
    if not os.path.exists(DRIVER):
        import importlib.util
        spec = importlib.util.spec_from_file_location("rq_build", os.path.join(PKG, "build.py"))
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        mod.build_driver()
    return DRIVER


def test_driver_builds_and_reports_missing_device(driver, tmp_path):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    sph = golden("synth_b")["spheres"]
    p = tmp_path / "s.xyzr"
    sph.astype(np.float32).tofile(p)
    r = subprocess.run([driver, "--spheres", str(p)], capture_output=True, text=True)
    assert r.returncode == 1 and "no CUDA device" in r.stderr


@pytest.mark.skipif(not os.path.exists(REF_BUNNY), reason="needs the reference's bunny.obj")
def test_loader_matches_reference_scene(driver, tmp_path):
    out = tmp_path / "bunny.xyzr"
    subprocess.run([driver, "--model", REF_BUNNY, "--dump-spheres", str(out)], check=True, capture_output=True)
    got = np.fromfile(out, np.float32).reshape(-1, 4)
    assert np.array_equal(got, golden("bunny")["spheres"])  # createScene_new's list, bit for bit


@pytest.mark.gpu
@pytest.mark.parametrize("structure", ["BVH", "LBVH", "KDTREE"])
def test_driver_renders_reference_image(driver, tmp_path, structure):
    b = golden("bunny")
    p = tmp_path / "bunny.xyzr"
    b["spheres"].astype(np.float32).tofile(p)
    out = tmp_path / "out.ppm"
    r = subprocess.run([driver, "--spheres", str(p), "--structure", structure, "--out", str(out)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    data = np.frombuffer(out.read_bytes(), np.uint8)
    assert bytes(data[:15]) == b"P6\n640 480\n255\n"
    if structure == "BVH":  # the shipped golden image is the BVH render
        assert np.array_equal(data[15:], b["golden_ppm"][15:]), int((data[15:] != b["golden_ppm"][15:]).sum())
    else:
        assert data.size == 15 + 640 * 480 * 3


def test_driver_finds_the_model_without_regard_to_case(driver, tmp_path):
    """createScene_new asks for "igea.obj"; the reference ships "Igea.obj"."""
    (tmp_path / "Igea.obj").write_text("v 0.1 0.2 0.3\nv -0.25 0.5 0.125\n")
    out = tmp_path / "igea.xyzr"
    r = subprocess.run([driver, "--models", str(tmp_path), "--scene-model", "IGEA", "--dump-spheres", str(out)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    got = np.fromfile(out, np.float32).reshape(-1, 4)
    assert got.shape == (3, 4) and got[-1, 3] == 100  # two vertex spheres + the ground
    r = subprocess.run([driver, "--models", str(tmp_path), "--scene-model", "ARMADILLO", "--dump-spheres", str(out)],
                       capture_output=True, text=True)
    assert r.returncode == 1 and "no model file" in r.stderr


_SHIM_PROGRAM = r"""
#include <cstdio>
#include <vector>
#include "rq.hpp"
// Reads spheres (x y z r float32) and rays (ox oy oz dx dy dz float32), builds
// with the reference's builder names and writes, per ray, the list
// boxIntersect returns (count, then ids) as int32.
int main(int argc, char** argv) {
  auto slurp = [](const char* p) {
    std::vector<float> v;
    FILE* f = std::fopen(p, "rb");
    float x;
    while (std::fread(&x, 4, 1, f) == 1) v.push_back(x);
    std::fclose(f);
    return v;
  };
  std::vector<float> s = slurp(argv[1]), r = slurp(argv[2]);
  std::vector<rq::SphereRecord> recs(s.size() / 4);
  for (size_t i = 0; i < recs.size(); ++i) recs[i] = {{s[4 * i], s[4 * i + 1], s[4 * i + 2]}, s[4 * i + 3]};
  rq::Context ctx;
  rq::Scene scene = rq::Scene::spheres(ctx, recs);
  rq::Accel acc = argv[4][0] == 'L' ? rq::constructLBVHTree(ctx, scene) : rq::constructBVHNew(ctx, scene);
  FILE* out = std::fopen(argv[3], "wb");
  for (size_t k = 0; k + 6 <= r.size(); k += 6) {
    std::vector<int> boxes;
    acc.boxIntersect(&r[k], &r[k + 3], boxes);
    int n = (int)boxes.size();
    std::fwrite(&n, 4, 1, out);
    if (n) std::fwrite(boxes.data(), 4, boxes.size(), out);
  }
  std::fclose(out);
  return 0;
}
"""


@pytest.mark.gpu
@pytest.mark.parametrize("structure", ["BVH", "LBVH"])
def test_shim_box_intersect_matches_batched_lists(driver, tmp_path, structure):
    """rq::Accel::boxIntersect with the reference's signature (one ray, ids
    appended to a std::vector<int>) returns the batched query's lists."""
    import rq
    src = tmp_path / "shim.cpp"
    src.write_text(_SHIM_PROGRAM)
    exe = tmp_path / "shim"
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"), "-I", os.path.join(PKG, "host"),
                    str(src), "-L", PKG, "-lrq", f"-Wl,-rpath,{PKG}", "-o", str(exe)], check=True)
    b = golden("bunny")
    sph = b["spheres"].astype(np.float32)
    r6 = b["crop_rays"][:200].astype(np.float32)
    sph.tofile(tmp_path / "s.bin")
    r6.tofile(tmp_path / "r.bin")
    res = subprocess.run([str(exe), str(tmp_path / "s.bin"), str(tmp_path / "r.bin"), str(tmp_path / "o.bin"),
                          structure], capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    got = np.fromfile(tmp_path / "o.bin", np.int32)
    with rq.Engine() as e:  # default settings, as rq::Context
        acc = e.build(e.scene_spheres(sph), getattr(rq, structure))
        counts, ids = e.trace_candidates(acc, rq.make_rays(r6[:, :3], r6[:, 3:]))
    want = []
    offs = np.concatenate([[0], np.cumsum(counts.astype(np.int64))])
    for k in range(len(r6)):
        want.append(int(counts[k]))
        want.extend(ids[offs[k]:offs[k + 1]].astype(np.int32).tolist())
    assert np.array_equal(got, np.array(want, np.int32))
    assert counts.sum() > 0
