"""GPU parity of the LBVH treelet restructuring (lbvh_quality RQ_LBVH_TREELETS)
through the C ABI: the exported nodes, bit for bit, equal the oracle's
restatement of the pass applied to the oracle's Karras tree, across the refit
layouts (one treelet, treelets under a top block, more top nodes than the block
holds), and the restructured tree's hits and occlusion bits equal those of the
Karras tree.

No reference implementation (the reference has no treelet pass); parity is
against the restated oracle."""
import numpy as np
import pytest

import scenes
from conftest import bvh2_from_export, golden

pytestmark = pytest.mark.gpu


def _u32(a):
    return np.ascontiguousarray(a).view(np.uint32)


def _check(engine, oracle, rqm, scene, aabb, codes):
    engine.configure(lbvh_quality=rqm.LBVH_TREELETS)
    acc = engine.build(scene, rqm.LBVH)
    nodes, order, sorted_codes, root, info = engine.export_bvh2(acc)
    karras = oracle.build_lbvh(codes, aabb)
    want = oracle.treelet_opt(karras)
    assert np.array_equal(order, karras.order)
    assert np.array_equal(root, karras.root_bounds)
    assert np.array_equal(nodes.view(np.int32), want.nodes.view(np.int32))  # topology + boxes, bitwise
    return acc, karras, want


def _tri(engine, oracle, v, f):
    s = engine.scene_triangles(v, f)
    prims, aabb, cen = oracle.tri_prims(v, f)
    return s, prims, aabb, cen


def test_treelets_icosphere(engine, oracle, rqm):
    v, f = scenes.displaced_icosphere(5, seed=22)
    s, prims, aabb, cen = _tri(engine, oracle, v, f)
    lo, hi = oracle.bounds3(v)
    acc, karras, want = _check(engine, oracle, rqm, s, aabb, oracle.morton_centroids(cen, lo, hi))
    rays = scenes.incoherent_rays(lo, hi, 20_000, seed=23)
    for q in (oracle.CLOSEST, oracle.ANY):
        ref = oracle.trace_bvh2(oracle.TRIANGLES, oracle.FAST, q, karras, prims, rays)
        assert np.array_equal(oracle.trace_bvh2(oracle.TRIANGLES, oracle.FAST, q, want, prims, rays).view(np.uint8),
                              ref.view(np.uint8))
    assert np.array_equal(_u32(engine.trace_closest(acc, rays)),
                          _u32(oracle.trace_bvh2(oracle.TRIANGLES, oracle.FAST, oracle.CLOSEST, karras, prims, rays)))
    assert np.array_equal(rqm.unpack_bits(engine.trace_any(acc, rays), len(rays)),
                          oracle.trace_bvh2(oracle.TRIANGLES, oracle.FAST, oracle.ANY, karras, prims, rays))


def test_treelets_full_size_heightfield(engine, oracle, rqm):
    """The 998,000-triangle terrain with cube Morton codes (about 670
    treelets under a top block of about 670 nodes): the pass cuts the node
    visits of a ray sample, leaves the hits as they are, and a rebuild
    reproduces the tree."""
    v, f = scenes.heightfield(1001, 500, seed=2)
    engine.configure(morton=rqm.MORTON_SCENE_CUBE)
    s, prims, aabb, cen = _tri(engine, oracle, v, f)
    lo, hi = oracle.bounds3(v)
    acc, karras, want = _check(engine, oracle, rqm, s, aabb, oracle.morton_centroids(cen, lo, hi, cube=True))
    first = engine.export_bvh2(acc)[0]
    acc.rebuild()
    assert np.array_equal(engine.export_bvh2(acc)[0].view(np.int32), first.view(np.int32))
    rays = scenes.incoherent_rays(lo, hi, 50_000, seed=24)
    got = engine.trace_closest(acc, rays)
    c0, c1 = np.zeros(2, np.uint64), np.zeros(2, np.uint64)
    ref = oracle.trace_bvh2(oracle.TRIANGLES, oracle.FAST, oracle.CLOSEST, karras, prims, rays, counters=c0)
    oracle.trace_bvh2(oracle.TRIANGLES, oracle.FAST, oracle.CLOSEST, want, prims, rays, counters=c1)
    assert np.array_equal(_u32(got), _u32(ref))
    assert c1[0] < c0[0]  # fewer node visits


@pytest.mark.parametrize("scene", ["bunny", "synth_c"])
def test_treelets_spheres_reference_codes(engine, oracle, rqm, scene):
    g = golden(scene)
    engine.configure(morton=rqm.MORTON_REFERENCE)
    s = engine.scene_spheres(g["spheres"])
    aabb, _ = oracle.sphere_prims(g["spheres"])
    _check(engine, oracle, rqm, s, aabb, g["morton"])


def test_treelets_more_top_nodes_than_the_top_block(engine, oracle, rqm):
    """6M uniform points: about 4,100 nodes of more than 2048 leaves, more
    than the top block holds; those keep their Karras topology."""
    pts = np.random.default_rng(7).random((6_000_000, 3), dtype=np.float32)
    sph = np.concatenate([pts, np.full((len(pts), 1), 1e-4, np.float32)], 1)
    aabb, _ = oracle.sphere_prims(sph)
    _check(engine, oracle, rqm, engine.scene_spheres(sph), aabb, oracle.morton_centroids(pts, pts.min(0), pts.max(0)))


@pytest.mark.parametrize("group,levels", [(32, 30), (64, 20)])
def test_treelets_caterpillar_trees(engine, oracle, rqm, group, levels):
    pts = scenes.chain_clusters(16, group, levels)
    sph = np.concatenate([pts, np.full((len(pts), 1), 1e-3, np.float32)], 1)
    aabb, _ = oracle.sphere_prims(sph)
    lo, hi = oracle.bounds3(pts)
    _check(engine, oracle, rqm, engine.scene_spheres(sph), aabb, oracle.morton_centroids(pts, lo, hi))


@pytest.mark.parametrize("n", [1, 2, 3, 4, 5, 6, 2049, 2050, 5000])
def test_treelets_small_and_boundary_sizes(engine, oracle, rqm, n):
    """Trees of one to six leaves (treelets of three and four leaves at the
    root) and sizes around one refit treelet (2048 leaves)."""
    rng = np.random.default_rng(100 + n)
    pts = rng.random((n, 3), dtype=np.float32)
    sph = np.concatenate([pts, np.full((n, 1), 0.05, np.float32)], 1)
    s = engine.scene_spheres(sph)
    aabb, _ = oracle.sphere_prims(sph)
    lo, hi = oracle.bounds3(pts)
    codes = oracle.morton_centroids(pts, lo, hi)
    if n < 2:
        engine.configure(lbvh_quality=rqm.LBVH_TREELETS)
        acc = engine.build(s, rqm.LBVH)
        assert engine.export_bvh2(acc)[4].n_nodes == 0
        return
    acc, karras, want = _check(engine, oracle, rqm, s, aabb, codes)
    rays = scenes.incoherent_rays(lo - 0.1, hi + 0.1, 4096, seed=n)
    prims = np.ascontiguousarray(sph)
    assert np.array_equal(_u32(engine.trace_closest(acc, rays)),
                          _u32(oracle.trace_bvh2(oracle.SPHERES, oracle.FAST, oracle.CLOSEST, karras, prims, rays)))


def test_treelets_setting_is_validated(engine, rqm):
    v, f = scenes.displaced_icosphere(2, seed=3)
    s = engine.scene_triangles(v, f)
    engine.configure(lbvh_quality=7)
    with pytest.raises(Exception):
        engine.build(s, rqm.LBVH)
    engine.configure(lbvh_quality=rqm.LBVH_KARRAS)
    engine.build(s, rqm.LBVH)
