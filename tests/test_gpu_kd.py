"""GPU parity of the SAH KD tree (RQ_KDTREE, constructKDTreeNew / buildTree)
and its traversal (kdtreeIntersect) through the C ABI.

The node array is compared with the oracle's word for word (split planes as
floats, so -0 equals +0) and with the reference's own array (golden
fixtures); leaf contents as primitive lists.  Traversal results are compared
bit for bit with the oracle walking the same exported tree."""
import numpy as np
import pytest

import scenes
from conftest import golden, sphere_surface_colors

pytestmark = pytest.mark.gpu


def _check_nodes(got_nodes, got_idx, want_nodes, want_idx):
    assert got_nodes.shape == want_nodes.shape
    assert np.array_equal(got_nodes[:, 1:], want_nodes[:, 1:])        # flags / above child / leaf sizes
    interior = (want_nodes[:, 1] & 3) != 3
    assert np.array_equal(got_nodes[~interior, 0], want_nodes[~interior, 0])  # leaf offsets / single prims
    gs = got_nodes[interior, 0].view(np.float32)
    ws = want_nodes[interior, 0].view(np.float32)
    assert np.array_equal(gs, ws)                                        # split planes (== on floats)
    assert np.array_equal(got_idx, want_idx)


@pytest.mark.parametrize("scene", ["bunny", "synth_a", "synth_b", "synth_c"])
def test_kd_spheres_matches_oracle_and_reference(engine, oracle, rqm, scene):
    g = golden(scene)
    sph = g["spheres"]
    s = engine.scene_spheres(sph)
    acc = engine.build(s, rqm.KDTREE)
    nodes, pidx, root, info = engine.export_kd(acc)
    aabb, _ = oracle.sphere_prims(sph)
    ref = oracle.build_kd(aabb)
    _check_nodes(nodes, pidx, ref.nodes, ref.prim_idx)
    assert np.array_equal(root, g["kd_root_bounds"])
    assert info.max_depth == int(g["kd_max_depth"])
    # the reference's own node array: identical except the order inside leaves
    assert np.array_equal(nodes[:, 1:], g["kd_nodes"][:, 1:])


@pytest.mark.parametrize("level,seed", [(4, 41), (5, 42)])
def test_kd_triangles_matches_oracle(engine, oracle, rqm, level, seed):
    v, f = scenes.displaced_icosphere(level, seed=seed)
    s = engine.scene_triangles(v, f)
    acc = engine.build(s, rqm.KDTREE)
    nodes, pidx, root, info = engine.export_kd(acc)
    prims, aabb, _ = oracle.tri_prims(v, f)
    ref = oracle.build_kd(aabb)
    _check_nodes(nodes, pidx, ref.nodes, ref.prim_idx)
    lo, hi = oracle.bounds3(v)
    rays = scenes.incoherent_rays(lo, hi, 20_000, seed=seed)
    kd = oracle.Kd(nodes, pidx, root)
    h = engine.trace_closest(acc, rays)
    hr = oracle.trace_kd(oracle.TRIANGLES, oracle.FAST, oracle.CLOSEST, kd, prims, rays)
    assert np.array_equal(h.view(np.uint32), hr.view(np.uint32))
    occ = oracle.trace_kd(oracle.TRIANGLES, oracle.FAST, oracle.ANY, kd, prims, rays)
    assert np.array_equal(rqm.unpack_bits(engine.trace_any(acc, rays), len(rays)), occ)
    hn = oracle.trace_brute(oracle.TRIANGLES, oracle.FAST, oracle.CLOSEST, prims, rays)
    assert (h["t"] == hn["t"]).mean() > 0.999  # KD split-plane clipping can lose a grazing hit


def test_kd_heightfield_matches_oracle(engine, oracle, rqm):
    v, f = scenes.heightfield(201, 100, seed=8)
    s = engine.scene_triangles(v, f)
    acc = engine.build(s, rqm.KDTREE)
    nodes, pidx, root, info = engine.export_kd(acc)
    _, aabb, _ = oracle.tri_prims(v, f)
    ref = oracle.build_kd(aabb)
    _check_nodes(nodes, pidx, ref.nodes, ref.prim_idx)


def test_kd_any_hit_reference_semantics_bunny(engine, oracle, rqm):
    b = golden("bunny")
    sph = b["spheres"]
    engine.configure(traversal=rqm.TRAVERSAL_REFERENCE)
    s = engine.scene_spheres(sph)
    acc = engine.build(s, rqm.KDTREE)
    rays = oracle.camera_rays_ref(640, 480, 1, oracle.jitter_mt19937(640 * 480 * 2))
    bits = rqm.unpack_bits(engine.trace_any(acc, rays), len(rays))
    import hashlib
    assert hashlib.sha256(bits.tobytes()).digest() == bytes(b["kd_any_sha"])  # the reference's own mask


def test_kd_render_matches_reference_image(engine, oracle, rqm):
    b = golden("bunny")
    sph = b["spheres"]
    s = engine.scene_spheres(sph)
    acc = engine.build(s, rqm.KDTREE)
    pixels, _ = engine.render_reference(acc, rqm.default_settings(dataStructure=rqm.KDTREE), None,
                                        sphere_surface_colors(len(sph)))
    rays = oracle.camera_rays_ref(640, 480, 1, oracle.jitter_mt19937(640 * 480 * 2))
    kd = oracle.build_kd(oracle.sphere_prims(sph)[0])
    occ = oracle.trace_kd(oracle.SPHERES, oracle.REFERENCE, oracle.ANY, kd, sph, rays)
    want = oracle.pixels_ref(oracle.shade_ref(sph, sphere_surface_colors(len(sph)), rays, kd_any=occ))
    assert np.array_equal(pixels, want)


def test_kd_degenerate_inputs(engine, oracle, rqm):
    for sph in (np.array([[1, 2, 3, 0.5]], np.float32), np.array([[0, 0, -5, 1]] * 40, np.float32)):
        s = engine.scene_spheres(sph)
        acc = engine.build(s, rqm.KDTREE)
        nodes, pidx, root, info = engine.export_kd(acc)
        ref = oracle.build_kd(oracle.sphere_prims(sph)[0])
        _check_nodes(nodes, pidx, ref.nodes, ref.prim_idx)


def test_kd_full_size_terrain_matches_oracle(engine, oracle, rqm):
    """The benchmark's 998,000-triangle terrain: about 30 levels, up to 2.4M refs
    a level, so the edge-list partition runs with more than 1024 tiles a list and
    every pass of the level loop at full width.  Rebuilt once more: same tree."""
    v, f = scenes.heightfield(1001, 500, amplitude=0.3, octaves=5, seed=1)
    s = engine.scene_triangles(v, f)
    acc = engine.build(s, rqm.KDTREE)
    nodes, pidx, root, info = engine.export_kd(acc)
    _, aabb, _ = oracle.tri_prims(v, f)
    ref = oracle.build_kd(aabb)
    _check_nodes(nodes, pidx, ref.nodes, ref.prim_idx)
    acc.rebuild()
    nodes2, pidx2, _, _ = engine.export_kd(acc)
    assert np.array_equal(nodes2, nodes) and np.array_equal(pidx2, pidx)
