"""GPU parity of the collapsed 4-wide BVH (settings.node_width = 4): the
engine's collapse equals the oracle's collapse of the engine's own binary
tree bit for bit, and FAST closest / any-hit queries through it equal the
oracle's 4-wide walk bit for bit (hits, occlusion bits, node-visit and
primitive-test counts).  The 4-wide walk visits children in a different order
from the binary walk; FAST closest hit keeps the smallest t and, on exact
ties, the smallest primitive id, so the results equal the binary walk's bit
for bit too."""
import numpy as np
import pytest

import scenes
from conftest import bvh2_from_export, golden

pytestmark = pytest.mark.gpu


def _u32(a):
    return np.ascontiguousarray(a).view(np.uint32)


def _check_collapse(engine, oracle, acc):
    nodes, order, codes, root, info = engine.export_bvh2(acc)
    b = bvh2_from_export(oracle, nodes, order, root, codes)
    want, k = oracle.collapse_bvh4(b)
    got = engine.export_bvh4(acc)
    assert acc.info().node_width == 4
    assert acc.info().n_wide_nodes == k == len(got)
    assert np.array_equal(_u32(got), _u32(want))
    return b, got


def _check_queries(engine, oracle, kind, acc, b, nodes4, prims, rays):
    got_c, cnt_c = engine.trace_counters(acc, rays)
    want_cnt = np.zeros(2, np.uint64)
    want_c = oracle.trace_bvh4(kind, oracle.CLOSEST, nodes4, b, prims, rays, counters=want_cnt)
    assert np.array_equal(_u32(got_c), _u32(want_c))
    assert np.array_equal(cnt_c, want_cnt)
    assert np.array_equal(_u32(engine.trace_closest(acc, rays)), _u32(want_c))
    bits = engine.trace_any(acc, rays)
    want_a = oracle.trace_bvh4(kind, oracle.ANY, nodes4, b, prims, rays)
    got_a = np.unpackbits(bits.view(np.uint8), bitorder="little")[: len(rays)]
    assert np.array_equal(got_a.astype(bool), want_a.astype(bool))
    return want_c


@pytest.mark.parametrize("acc_name", ["LBVH", "BVH"])
def test_bvh4_triangles_match_oracle(engine, oracle, rqm, acc_name):
    v, f = scenes.displaced_icosphere(5, seed=41)
    engine.configure(node_width=rqm.NODE_WIDTH_4)
    s = engine.scene_triangles(v, f)
    acc = engine.build(s, acc_name)
    b, nodes4 = _check_collapse(engine, oracle, acc)
    prims, _, _ = oracle.tri_prims(v, f)
    lo, hi = oracle.bounds3(v)
    rays = scenes.incoherent_rays(lo, hi, 50_000, seed=42)
    h4 = _check_queries(engine, oracle, oracle.TRIANGLES, acc, b, nodes4, prims, rays)
    h2 = oracle.trace_bvh2(oracle.TRIANGLES, oracle.FAST, oracle.CLOSEST, b, prims, rays)
    assert np.array_equal(_u32(h4), _u32(h2))


@pytest.mark.parametrize("acc_name", ["LBVH", "BVH"])
@pytest.mark.parametrize("scene", ["bunny", "synth_c"])
def test_bvh4_spheres_match_oracle(engine, oracle, rqm, acc_name, scene):
    sph = golden(scene)["spheres"]
    engine.configure(node_width=rqm.NODE_WIDTH_4)
    s = engine.scene_spheres(sph)
    acc = engine.build(s, acc_name)
    b, nodes4 = _check_collapse(engine, oracle, acc)
    c = sph[:, :3]
    rays = scenes.incoherent_rays(c.min(0) - 2, c.max(0) + 2, 20_000, seed=43)
    _check_queries(engine, oracle, oracle.SPHERES, acc, b, nodes4, np.ascontiguousarray(sph, np.float32), rays)


def test_bvh4_heightfield_with_ray_sort(engine, oracle, rqm):
    v, f = scenes.heightfield(301, 150, seed=44)
    engine.configure(node_width=rqm.NODE_WIDTH_4)
    s = engine.scene_triangles(v, f)
    acc = engine.build(s, "LBVH")
    b, nodes4 = _check_collapse(engine, oracle, acc)
    prims, _, _ = oracle.tri_prims(v, f)
    primary = scenes.pinhole_rays(320, 180, 2, eye=(0, -0.6, 1.1), target=(0, 0, 0), seed=45)
    h0 = engine.trace_closest(acc, primary)
    sec = scenes.cosine_rays(v, f, primary, h0, seed=46)
    assert len(sec) >= 65536  # above the reordering threshold
    plain_c = _check_queries(engine, oracle, oracle.TRIANGLES, acc, b, nodes4, prims, sec)
    plain_a = engine.trace_any(acc, sec)
    engine.configure(ray_sort=rqm.RAY_SORT_OCTANT_MORTON)
    assert np.array_equal(_u32(engine.trace_closest(acc, sec)), _u32(plain_c))
    assert np.array_equal(engine.trace_any(acc, sec), plain_a)


def test_bvh4_reference_traversal_and_rebuild(engine, oracle, rqm):
    """REFERENCE queries keep the binary nodes; a rebuild re-collapses."""
    v, f = scenes.displaced_icosphere(4, seed=47)
    s = engine.scene_triangles(v, f)
    lo, hi = oracle.bounds3(v)
    rays = scenes.incoherent_rays(lo, hi, 20_000, seed=48)
    engine.configure(traversal=rqm.TRAVERSAL_REFERENCE)
    ref2 = engine.trace_closest(engine.build(s, "LBVH"), rays)
    engine.configure(node_width=rqm.NODE_WIDTH_4)
    acc = engine.build(s, "LBVH")
    assert np.array_equal(_u32(engine.trace_closest(acc, rays)), _u32(ref2))
    engine.configure(traversal=rqm.TRAVERSAL_FAST)
    v2 = (v * np.float32(1.5)).astype(np.float32)
    s.update(v2)
    acc.rebuild()
    b, nodes4 = _check_collapse(engine, oracle, acc)
    prims, _, _ = oracle.tri_prims(v2, f)
    lo2, hi2 = oracle.bounds3(v2)
    _check_queries(engine, oracle, oracle.TRIANGLES, acc, b, nodes4, prims,
                   scenes.incoherent_rays(lo2, hi2, 20_000, seed=49))


def test_bvh4_settings_and_small_scenes(engine, oracle, rqm):
    with pytest.raises(rqm.RqError):
        engine.configure(node_width=3)
    engine.configure(node_width=rqm.NODE_WIDTH_4)
    # KD and NONE ignore the node width
    sph = golden("synth_a")["spheres"]
    s = engine.scene_spheres(sph)
    assert engine.build(s, "KDTREE").info().node_width == 0
    # one and two primitives: no or one internal node
    for n in (1, 2, 3):
        s1 = engine.scene_spheres(sph[:n])
        acc = engine.build(s1, "LBVH")
        b, nodes4 = _check_collapse(engine, oracle, acc)
        c = sph[:n, :3]
        rays = scenes.incoherent_rays(c.min(0) - 2, c.max(0) + 2, 3000, seed=50 + n)
        _check_queries(engine, oracle, oracle.SPHERES, acc, b, nodes4, np.ascontiguousarray(sph[:n], np.float32), rays)
