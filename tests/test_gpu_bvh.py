"""GPU parity of the median BVH (RQ_BVH, constructBVHNew) and of the render
step (render + castRay shading) through the C ABI.

The GPU builder follows the oracle's engine rule (median ties broken by
primitive id), so its arrays are compared with the oracle's exactly: child
links and counts bit for bit, boxes as floats (==, so -0 equals +0), slot
order element for element.  The render is compared with the reference's own
golden image (the shipped output.ppm): within 1 of 255 per channel."""
import numpy as np
import pytest

import scenes
from conftest import bvh2_from_export, golden, sphere_surface_colors

pytestmark = pytest.mark.gpu


def _compare_median(engine, oracle, rqm, acc, aabb, cen):
    nodes, order, _, root, info = engine.export_bvh2(acc)
    ref = oracle.build_median(aabb, cen)
    assert info.n_nodes == ref.n_internal
    assert np.array_equal(order, ref.order)
    assert np.array_equal(root, ref.root_bounds)
    if ref.n_internal:
        assert np.array_equal(nodes.view(np.int32)[:, 12:], ref.nodes.view(np.int32)[:, 12:])
        assert np.array_equal(nodes[:, :12], ref.nodes[:, :12])
    return nodes, order, root


@pytest.mark.parametrize("level,seed", [(4, 31), (6, 32)])
def test_median_bvh_triangles_matches_oracle(engine, oracle, rqm, level, seed):
    v, f = scenes.displaced_icosphere(level, seed=seed)
    s = engine.scene_triangles(v, f)
    acc = engine.build(s, rqm.BVH)
    prims, aabb, cen = oracle.tri_prims(v, f)
    nodes, order, root = _compare_median(engine, oracle, rqm, acc, aabb, cen)
    lo, hi = oracle.bounds3(v)
    rays = scenes.incoherent_rays(lo, hi, 20_000, seed=seed)
    h = engine.trace_closest(acc, rays)
    hr = oracle.trace_bvh2(oracle.TRIANGLES, oracle.FAST, oracle.CLOSEST, bvh2_from_export(oracle, nodes, order, root),
                           prims, rays)
    assert np.array_equal(h.view(np.uint32), hr.view(np.uint32))


def test_median_bvh_heightfield_matches_oracle(engine, oracle, rqm):
    v, f = scenes.heightfield(401, 200, seed=7)
    s = engine.scene_triangles(v, f)
    acc = engine.build(s, rqm.BVH)
    _, aabb, cen = oracle.tri_prims(v, f)
    _compare_median(engine, oracle, rqm, acc, aabb, cen)


@pytest.mark.parametrize("scene", ["bunny", "synth_a", "synth_c"])
def test_median_bvh_spheres_matches_oracle(engine, oracle, rqm, scene):
    sph = golden(scene)["spheres"]
    s = engine.scene_spheres(sph)
    acc = engine.build(s, rqm.BVH)
    aabb, cen = oracle.sphere_prims(sph)
    _compare_median(engine, oracle, rqm, acc, aabb, cen)


def test_median_bvh_degenerate_inputs(engine, oracle, rqm):
    cases = [np.array([[1, 2, 3, 0.5]], np.float32),                      # one primitive
             np.array([[0, 0, -5, 1]] * 7, np.float32),                    # identical spheres
             np.array([[0, 0, -5, 1], [0, 0, -5, 1], [3, 0, -5, 1]], np.float32)]
    for sph in cases:
        s = engine.scene_spheres(sph)
        acc = engine.build(s, rqm.BVH)
        aabb, cen = oracle.sphere_prims(sph)
        nodes, order, root = _compare_median(engine, oracle, rqm, acc, aabb, cen)
        assert sorted(order.tolist()) == list(range(len(sph)))  # no primitive dropped
        d = np.array([[0, 0, -1], [0.5, 0, -1]], np.float32)
        rays = rqm.make_rays(np.zeros(3), d / np.linalg.norm(d, axis=1, keepdims=True))  # sphere test wants unit dirs
        h = engine.trace_closest(acc, rays)
        hn = oracle.trace_brute(oracle.SPHERES, oracle.FAST, oracle.CLOSEST, sph, rays)
        assert np.array_equal(h["t"], hn["t"])


def test_median_bvh_degenerate_clusters_match_oracle(engine, oracle, rqm):
    """Degenerate nodes (all centroids equal: one leaf for the whole range)
    above and inside the subtrees that finish in one block, and a scene just
    past the in-block span."""
    rng = np.random.default_rng(40)
    same = np.tile(np.array([[1.0, 2.0, 3.0, 0.5]], np.float32), (3000, 1))
    cloud = np.concatenate([rng.random((5000, 3), dtype=np.float32) * 10, np.full((5000, 1), 0.05, np.float32)], 1)
    cloud[1000:1600] = np.array([4.0, 4.0, 4.0, 0.05], np.float32)  # a 600-sphere cluster of one point
    edge = np.concatenate([rng.random((513, 3), dtype=np.float32), np.full((513, 1), 0.01, np.float32)], 1)
    for sph in (same, cloud, edge):
        acc = engine.build(engine.scene_spheres(sph), rqm.BVH)
        aabb, cen = oracle.sphere_prims(sph)
        _compare_median(engine, oracle, rqm, acc, aabb, cen)


def test_render_bvh_reproduces_golden_image(engine, rqm, oracle):
    b = golden("bunny")
    sph = b["spheres"]
    s = engine.scene_spheres(sph)
    acc = engine.build(s, rqm.BVH)
    pixels, rgb = engine.render_reference(acc, rqm.default_settings(), None, sphere_surface_colors(len(sph)))
    gold = b["golden_ppm"][15:]
    # the shipped output.ppm, byte for byte (the parity bar is 1/255 per channel)
    assert np.array_equal(pixels.reshape(-1), gold), int((pixels.reshape(-1) != gold).sum())
    # later calls reuse the context's copy of the default jitter sequence
    again, rgb2 = engine.render_reference(acc, rqm.default_settings(), None, sphere_surface_colors(len(sph)))
    assert np.array_equal(again, pixels) and np.array_equal(rgb2.view(np.uint32), rgb.view(np.uint32))
    # as does a call with the jitter given explicitly
    jit = oracle.jitter_mt19937(640 * 480 * 2)
    given, _ = engine.render_reference(acc, rqm.default_settings(), jit, sphere_surface_colors(len(sph)))
    assert np.array_equal(given, pixels)


@pytest.mark.parametrize("acc_name", ["LBVH", "NONE"])
def test_render_other_structures_match_oracle_shading(engine, rqm, oracle, acc_name):
    b = golden("bunny")
    sph = b["spheres"]
    engine.configure(morton=rqm.MORTON_REFERENCE)
    s = engine.scene_spheres(sph)
    acc = engine.build(s, acc_name)
    pixels, rgb = engine.render_reference(acc, rqm.default_settings(), None, sphere_surface_colors(len(sph)))
    rays = oracle.camera_rays_ref(640, 480, 1, oracle.jitter_mt19937(640 * 480 * 2))
    if acc_name == "NONE":
        # brute force on the 64x48 crop only (the reference's NONE render takes minutes)
        sel = b["crop_index"]
        hr = oracle.trace_brute(oracle.SPHERES, oracle.REFERENCE, oracle.CLOSEST, sph, rays[sel])
        col = oracle.shade_ref(sph, sphere_surface_colors(len(sph)), rays[sel], hr)
        want = oracle.pixels_ref(col).reshape(-1, 3)
        got = pixels.reshape(-1, 3)[sel]
    else:
        nodes, order, codes, root, info = engine.export_bvh2(acc)
        hr = oracle.trace_bvh2(oracle.SPHERES, oracle.REFERENCE, oracle.CLOSEST,
                               bvh2_from_export(oracle, nodes, order, root), sph, rays)
        want = oracle.pixels_ref(oracle.shade_ref(sph, sphere_surface_colors(len(sph)), rays, hr))
        got = pixels
    assert np.array_equal(got, want), int((got != want).sum())
