"""Regenerate the golden fixtures in this directory from the reference itself.

Builds oracle/_ref/ref_dump from the reference's own sources (oracle/Makefile,
target `ref`), runs it on the reference's bunny scene and on seeded synthetic
sphere clouds, and packs what it printed into compressed .npz files.  Needs
the reference tree (REF_ROOT, default /root/reference); the committed .npz
files are what the tests read, so nothing at test time needs the reference.

    python tests/golden/make_golden.py

What each fixture holds (all arrays little-endian):
  known.npz        Morton known answers: points -> morton3D codes, expandBits table
  bunny.npz        the default scene (35,947 vertex spheres + ground sphere) as
                   createScene_new builds it; Morton codes; KD node array and
                   primitive indices; node-set digests of the BVH and "LBVH"
                   trees; the 64x48 centre crop of camera rays with every
                   structure's per-ray result and castRay colour; digests of the
                   full 640x480 per-ray results; the shipped output.ppm bytes
  synth_*.npz      synthetic sphere clouds with their full BVH / LBVH / KD trees
                   and per-ray results for every structure
"""
import hashlib
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
REF_ROOT = os.environ.get("REF_ROOT", "/root/reference")
REF_DIR = os.path.join(REF_ROOT, "project", "raytracer")
DUMP = os.path.join(REPO, "oracle", "_ref", "ref_dump")

sys.path.insert(0, os.path.join(REPO, "tests"))
from golden_util import tree_node_digest  # noqa: E402


def load(d, name, dt, shape=None):
    a = np.fromfile(os.path.join(d, name + ".bin"), dtype=dt)
    return a.reshape(shape) if shape else a


def meta(d):
    out = {}
    with open(os.path.join(d, "meta.txt")) as f:
        for line in f:
            k, v = line.split()
            out[k] = int(v)
    return out


def sha(a):
    return np.frombuffer(hashlib.sha256(np.ascontiguousarray(a).tobytes()).digest(), np.uint8)


def run(*args):
    subprocess.run([DUMP, *args], check=True, stdout=subprocess.DEVNULL)


def tree(d, prefix):
    return (load(d, prefix + "_bounds", np.float32, (-1, 6)),
            load(d, prefix + "_info", np.int32, (-1, 5)),
            load(d, prefix + "_objs", np.int32))


def main():
    subprocess.run(["make", "-C", os.path.join(REPO, "oracle"), "ref", f"REF_DIR={REF_DIR}"],
                   check=True, stdout=subprocess.DEVNULL)
    with tempfile.TemporaryDirectory() as tmp:
        # ---- known answers
        d = os.path.join(tmp, "known"); os.makedirs(d)
        run("known", d)
        np.savez_compressed(os.path.join(HERE, "known.npz"),
                            pts=load(d, "known_pts", np.float32, (-1, 3)),
                            codes=load(d, "known_codes", np.uint32),
                            expand_in=load(d, "expand_in", np.uint32),
                            expand_out=load(d, "expand_out", np.uint32))

        # ---- bunny (the reference's default scene and camera)
        d = os.path.join(tmp, "bunny"); os.makedirs(d)
        run("bunny", d, REF_DIR)
        m = meta(d)
        rays = load(d, "rays", np.float32, (-1, 6))
        sel = load(d, "none_sel", np.int32)
        bb, bi, bo = tree(d, "bvh")
        lb, li, lo = tree(d, "lbvh")
        with open(os.path.join(REF_DIR, "output.ppm"), "rb") as f:
            ppm = np.frombuffer(f.read(), np.uint8)
        np.savez_compressed(
            os.path.join(HERE, "bunny.npz"),
            spheres=load(d, "spheres", np.float32, (-1, 4)),
            morton=load(d, "morton", np.uint32),
            kd_nodes=load(d, "kd_nodes", np.int32, (-1, 3)),
            kd_prim_indices=load(d, "kd_prim_indices", np.int32),
            kd_root_bounds=load(d, "kd_root_bounds", np.float32),
            kd_max_depth=np.int32(m["kd_maxDepth"]),
            bvh_nodes=np.int64(m["bvh_nodes"]),
            bvh_digest=tree_node_digest(bb, bi, bo),
            lbvh_nodes=np.int64(m["lbvh_nodes"]),
            lbvh_digest=tree_node_digest(lb, li, lo),
            crop_index=sel,
            crop_rays=rays[sel],
            crop_jitter=load(d, "jitter", np.float64, (-1, 2))[sel],
            crop_bvh_id=load(d, "bvh_hit_id", np.int32)[sel],
            crop_bvh_t=load(d, "bvh_hit_t", np.float32)[sel],
            crop_lbvh_id=load(d, "lbvh_hit_id", np.int32)[sel],
            crop_lbvh_t=load(d, "lbvh_hit_t", np.float32)[sel],
            crop_kd_any=load(d, "kd_any", np.uint8)[sel],
            crop_none_id=load(d, "none_hit_id", np.int32),
            crop_none_t=load(d, "none_hit_t", np.float32),
            crop_color=load(d, "bvh_color", np.float32, (-1, 3))[sel],
            rays_sha=sha(rays),
            bvh_id_sha=sha(load(d, "bvh_hit_id", np.int32)),
            bvh_t_sha=sha(load(d, "bvh_hit_t", np.float32)),
            lbvh_id_sha=sha(load(d, "lbvh_hit_id", np.int32)),
            kd_any_sha=sha(load(d, "kd_any", np.uint8)),
            color_sha=sha(load(d, "bvh_color", np.float32)),
            bvh_sphere_tests=np.int64(m["bvh_sphere_tests"]),
            kd_sphere_tests=np.int64(m["kd_sphere_tests"]),
            golden_ppm=ppm)

        # ---- synthetic sphere clouds: (n, seed, rays)
        for name, n, seed, nr in (("synth_a", 2000, 7, 4096), ("synth_b", 257, 99, 1024),
                                  ("synth_c", 20000, 2024, 8192)):
            d = os.path.join(tmp, name); os.makedirs(d)
            run("synth", d, str(n), str(seed), str(nr), "1")
            m = meta(d)
            bb, bi, bo = tree(d, "bvh")
            lb, li, lo = tree(d, "lbvh")
            full = name != "synth_c"
            extra = {}
            if full:
                extra = dict(bvh_bounds=bb, bvh_info=bi, bvh_objs=bo,
                             lbvh_bounds=lb, lbvh_info=li, lbvh_objs=lo)
            np.savez_compressed(
                os.path.join(HERE, name + ".npz"),
                spheres=load(d, "spheres", np.float32, (-1, 4)),
                morton=load(d, "morton", np.uint32),
                kd_nodes=load(d, "kd_nodes", np.int32, (-1, 3)),
                kd_prim_indices=load(d, "kd_prim_indices", np.int32),
                kd_root_bounds=load(d, "kd_root_bounds", np.float32),
                kd_max_depth=np.int32(m["kd_maxDepth"]),
                bvh_nodes=np.int64(m["bvh_nodes"]),
                bvh_digest=tree_node_digest(bb, bi, bo),
                lbvh_nodes=np.int64(m["lbvh_nodes"]),
                lbvh_digest=tree_node_digest(lb, li, lo),
                rays=load(d, "rays", np.float32, (-1, 6)),
                bvh_id=load(d, "bvh_hit_id", np.int32),
                bvh_t=load(d, "bvh_hit_t", np.float32),
                lbvh_id=load(d, "lbvh_hit_id", np.int32),
                lbvh_t=load(d, "lbvh_hit_t", np.float32),
                kd_any=load(d, "kd_any", np.uint8),
                none_id=load(d, "none_hit_id", np.int32),
                none_t=load(d, "none_hit_t", np.float32),
                **extra)
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f"{f:16s} {os.path.getsize(os.path.join(HERE, f)):>9d} bytes")


if __name__ == "__main__":
    main()
