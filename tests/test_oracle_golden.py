"""The CPU oracle against vectors produced by the reference's own code
(tests/golden/, generated by tests/golden/make_golden.py from
oracle/ref_dump.cpp, which compiles the reference sources unchanged)."""
import hashlib

import numpy as np
import pytest

from conftest import golden
from golden_util import bvh2_to_preorder, tree_node_digest


def _sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).digest()


def test_morton_known_answers(oracle):
    k = golden("known")
    codes = np.array([oracle.morton3d(*map(float, p)) for p in k["pts"]], np.uint32)
    assert np.array_equal(codes, k["codes"])
    assert all(oracle.expand_bits(int(v)) == int(o) for v, o in zip(k["expand_in"], k["expand_out"]))
    # values quoted from accelerators.h's morton3D
    assert oracle.morton3d(0.5, 0.5, 0.5) == 939524096
    assert oracle.morton3d(0, 0, 0) == 0
    assert oracle.morton3d(1, 1, 1) == 1073741823
    assert oracle.expand_bits(1023) == 0x09249249


@pytest.mark.parametrize("scene", ["bunny", "synth_a", "synth_b", "synth_c"])
def test_morton_reference_normalisation(oracle, scene):
    g = golden(scene)
    assert np.array_equal(oracle.morton_spheres_ref(g["spheres"]), g["morton"])


def test_camera_rays_bit_exact(oracle, bunny):
    jit = oracle.jitter_mt19937(640 * 480 * 2)
    assert np.array_equal(jit.reshape(-1, 2)[bunny["crop_index"]], bunny["crop_jitter"])
    rays = oracle.camera_rays_ref(640, 480, 1, jit)
    r6 = np.concatenate([rays["org"], rays["dir"]], axis=1).astype(np.float32)
    assert _sha(r6) == bytes(bunny["rays_sha"])


@pytest.mark.parametrize("scene", ["bunny", "synth_a", "synth_b", "synth_c"])
def test_median_bvh_compat_matches_reference_node_sets(oracle, scene):
    g = golden(scene)
    aabb, cen = oracle.sphere_prims(g["spheres"])
    m = oracle.build_median(aabb, cen, compat=True)
    b, i, o = bvh2_to_preorder(m.nodes, m.n_internal, m.root_bounds, m.order)
    assert len(i) == int(g["bvh_nodes"])
    assert np.array_equal(tree_node_digest(b, i, o), g["bvh_digest"])
    if "bvh_info" in g.files:  # full trees: same pre-order walk, node by node
        assert np.array_equal(i[:, [0, 2, 3, 4]], g["bvh_info"][:, [0, 2, 3, 4]])
        assert np.array_equal(b, g["bvh_bounds"])


@pytest.mark.parametrize("scene", ["bunny", "synth_a", "synth_b", "synth_c"])
def test_reference_lbvh_is_median_bvh_without_last_primitive(oracle, scene):
    # constructLBVHTree passes size()-1 as the exclusive end (accelerators.h:583)
    # and builds both subtrees with constructBVHNew (:534-552).
    g = golden(scene)
    aabb, cen = oracle.sphere_prims(g["spheres"])
    m = oracle.build_median(aabb[:-1], cen[:-1], compat=True)
    b, i, o = bvh2_to_preorder(m.nodes, m.n_internal, m.root_bounds, m.order)
    assert len(i) == int(g["lbvh_nodes"])
    assert np.array_equal(tree_node_digest(b, i, o), g["lbvh_digest"])


def _leaf_sets(nodes, pidx):
    out = []
    for w0, w1, w2 in nodes:
        if (w1 & 3) == 3:
            np_ = w2
            if np_ == 0:
                out.append(())
            elif np_ == 1:
                out.append((int(w0),))
            else:
                out.append(tuple(sorted(pidx[w0:w0 + np_].tolist())))
    return out


@pytest.mark.parametrize("scene", ["bunny", "synth_a", "synth_b", "synth_c"])
def test_kd_tree_matches_reference(oracle, scene):
    g = golden(scene)
    aabb, _ = oracle.sphere_prims(g["spheres"])
    assert oracle.kd_max_depth(len(aabb)) == int(g["kd_max_depth"])
    kd = oracle.build_kd(aabb)
    # identical node array: split planes, axes, child offsets, leaf sizes and offsets
    assert np.array_equal(kd.nodes, g["kd_nodes"])
    assert np.array_equal(kd.root_bounds, g["kd_root_bounds"])
    # leaf contents equal as sets (the reference's unstable edge sort may order them differently)
    assert _leaf_sets(kd.nodes, kd.prim_idx) == _leaf_sets(g["kd_nodes"], g["kd_prim_indices"])


def test_bunny_per_ray_results_and_golden_image(oracle, bunny):
    sph = bunny["spheres"]
    aabb, cen = oracle.sphere_prims(sph)
    rays = oracle.camera_rays_ref(640, 480, 1, oracle.jitter_mt19937(640 * 480 * 2))
    m = oracle.build_median(aabb, cen, compat=True)
    cnt = np.zeros(2, np.uint64)
    h = oracle.trace_bvh2(oracle.SPHERES, oracle.REFERENCE, oracle.CLOSEST, m, sph, rays, counters=cnt)
    ids = h["prim"].astype(np.int32)
    tt = np.where(h["prim"] == oracle.MISS, np.float32(np.inf), h["t"]).astype(np.float32)
    assert _sha(ids) == bytes(bunny["bvh_id_sha"])
    assert _sha(tt) == bytes(bunny["bvh_t_sha"])
    assert int(cnt[1]) == int(bunny["bvh_sphere_tests"])  # same candidate count as the reference
    sel = bunny["crop_index"]
    assert np.array_equal(ids[sel], bunny["crop_bvh_id"])
    # the reference's LBVH tree
    ml = oracle.build_median(aabb[:-1], cen[:-1], compat=True)
    hl = oracle.trace_bvh2(oracle.SPHERES, oracle.REFERENCE, oracle.CLOSEST, ml, sph, rays)
    assert _sha(hl["prim"].astype(np.int32)) == bytes(bunny["lbvh_id_sha"])
    # KD any-hit
    kd = oracle.build_kd(aabb)
    kcnt = np.zeros(2, np.uint64)
    ka = oracle.trace_kd(oracle.SPHERES, oracle.REFERENCE, oracle.ANY, kd, sph, rays, counters=kcnt)
    assert _sha(ka) == bytes(bunny["kd_any_sha"])
    # Any-hit stops at the first hit, so the test count depends on the order
    # inside a leaf: the oracle lists leaf primitives by id, the reference in
    # the order of its unstable edge sort.
    assert abs(int(kcnt[1]) - int(bunny["kd_sphere_tests"])) <= 1e-2 * int(bunny["kd_sphere_tests"])
    # NONE on the crop
    hn = oracle.trace_brute(oracle.SPHERES, oracle.REFERENCE, oracle.CLOSEST, sph, rays[sel])
    assert np.array_equal(hn["prim"].astype(np.int32), bunny["crop_none_id"])
    assert np.array_equal(np.where(hn["prim"] == oracle.MISS, np.float32(np.inf), hn["t"]), bunny["crop_none_t"])
    # castRay colours and the shipped golden image, byte for byte
    col = oracle.shade_ref(sph, oracle.reference_surface_colors(len(sph)), rays, h)
    assert _sha(col) == bytes(bunny["color_sha"])
    assert np.array_equal(oracle.pixels_ref(col), bunny["golden_ppm"][15:])


@pytest.mark.parametrize("scene", ["synth_a", "synth_b", "synth_c"])
def test_synthetic_per_ray_results(oracle, scene):
    g = golden(scene)
    sph = g["spheres"]
    r6 = g["rays"]
    rays = oracle.make_rays(r6[:, :3], r6[:, 3:])
    aabb, cen = oracle.sphere_prims(sph)
    m = oracle.build_median(aabb, cen, compat=True)
    h = oracle.trace_bvh2(oracle.SPHERES, oracle.REFERENCE, oracle.CLOSEST, m, sph, rays)
    assert np.array_equal(h["prim"].astype(np.int32), g["bvh_id"])
    assert np.array_equal(np.where(h["prim"] == oracle.MISS, np.float32(np.inf), h["t"]), g["bvh_t"])
    ml = oracle.build_median(aabb[:-1], cen[:-1], compat=True)
    hl = oracle.trace_bvh2(oracle.SPHERES, oracle.REFERENCE, oracle.CLOSEST, ml, sph, rays)
    assert np.array_equal(hl["prim"].astype(np.int32), g["lbvh_id"])
    kd = oracle.build_kd(aabb)
    ka = oracle.trace_kd(oracle.SPHERES, oracle.REFERENCE, oracle.ANY, kd, sph, rays)
    assert np.array_equal(ka, g["kd_any"])
    hn = oracle.trace_brute(oracle.SPHERES, oracle.REFERENCE, oracle.CLOSEST, sph, rays)
    assert np.array_equal(hn["prim"].astype(np.int32), g["none_id"])
    assert np.array_equal(np.where(hn["prim"] == oracle.MISS, np.float32(np.inf), hn["t"]), g["none_t"])


def test_candidate_lists_match_reference_counts(oracle, bunny):
    # castRay (main.cpp:330-358) tests every candidate boxIntersect returns,
    # so the reference's sphere-test count over the 640x480 image is the sum
    # of the candidate-list lengths; its closest hits are the first strictly
    # nearer sphere along each list.
    sph = bunny["spheres"]
    aabb, cen = oracle.sphere_prims(sph)
    rays = oracle.camera_rays_ref(640, 480, 1, oracle.jitter_mt19937(640 * 480 * 2))
    m = oracle.build_median(aabb, cen, compat=True)
    counts, ids = oracle.candidates_bvh2(m, rays)
    assert int(counts.sum()) == len(ids) == int(bunny["bvh_sphere_tests"])
    offs = np.concatenate([[0], np.cumsum(counts.astype(np.int64))])
    sel = bunny["crop_index"][::8]
    for r in sel:
        lst = ids[offs[r]:offs[r + 1]]
        h = oracle.trace_brute(oracle.SPHERES, oracle.REFERENCE, oracle.CLOSEST, sph[lst], rays[r:r + 1])
        got = -1 if h["prim"][0] == oracle.MISS else int(lst[h["prim"][0]])
        assert got == int(bunny["crop_bvh_id"][list(bunny["crop_index"]).index(r)])
