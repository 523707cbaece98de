"""The engine's device-side guards, made to fire without a GPU fault, and the
context's recovery afterwards.

Each guard bounds something a broken input or a lost GPU block could make
endless or out of range: the radix sort's look-back wait (a bounded spin), the
traversal stack (a depth check before every push) and the walk itself (a step
limit a valid tree never reaches).  The tests trip them with the context's
test hooks (rq_set_debug) and with a cyclic tree brought in through
rq_accel_import_bvh2, check the status the caller sees, then check that the
same context still sorts, builds and traces correctly (against the CPU
oracle).  Nothing here faults, traps or spins without a limit: every wait and
walk involved is bounded in the kernel, and the imported trees pass the
import's range checks, so no walk reads outside its arrays.

The reference itself reports no errors at all (main.cpp:656-660); these are
the engine's own contract.
"""
import numpy as np
import pytest

import scenes

pytestmark = pytest.mark.gpu

TIMEOUT, STACK_OVERFLOW, INVALID_ARGUMENT, UNSUPPORTED = 6, 5, 1, 2


def _status(exc):
    return exc.value.status


def _context_still_traces(engine, oracle, rqm):
    """A fresh LBVH build and closest/any queries on the same context equal the oracle."""
    v, f = scenes.displaced_icosphere(3, seed=17)
    prims, aabb, cen = oracle.tri_prims(v, f)
    lo, hi = oracle.bounds3(v)
    rays = scenes.incoherent_rays(lo, hi, 2048, seed=18)
    s = engine.scene_triangles(v, f)
    acc = engine.build(s, rqm.LBVH)
    ref = oracle.build_lbvh(oracle.morton_centroids(cen, lo, hi), aabb)
    hits = engine.trace_closest(acc, rays)
    want = oracle.trace_bvh2(oracle.TRIANGLES, oracle.FAST, oracle.CLOSEST, ref, prims, rays)
    assert np.array_equal(hits.view(np.uint32), want.view(np.uint32))
    occ = engine.trace_any(acc, rays)
    assert np.array_equal(rqm.unpack_bits(occ, len(rays)),
                          oracle.trace_bvh2(oracle.TRIANGLES, oracle.FAST, oracle.ANY, ref, prims, rays))
    acc.close()
    s.close()


def test_sort_wait_that_never_ends_reports_timeout_and_context_recovers(engine, oracle, rqm):
    n = 100_003  # 27 tiles: tile 1's look-back runs
    rng = np.random.default_rng(5)
    keys = rng.integers(0, 1 << 30, n, dtype=np.uint64).astype(np.uint32)
    vals = np.arange(n, dtype=np.uint32)
    engine.set_debug(sort_stall=1)
    with pytest.raises(rqm.RqError) as e:
        engine.sort_pairs(keys, vals, key_bits=30)
    assert _status(e) == TIMEOUT
    engine.set_debug()
    k, v = engine.sort_pairs(keys, vals, key_bits=30)
    ok, ov = oracle.sort_pairs(keys)
    assert np.array_equal(k, ok) and np.array_equal(v, ov)
    _context_still_traces(engine, oracle, rqm)


def _stacked_quads(n_layers):
    """n_layers unit squares (two triangles each) stacked along z, 0.001 apart:
    a ray down the z axis enters every box of the tree on its way to the first
    leaf, so its walk pushes one far child per level (about log2 of the
    triangle count)."""
    verts, idx = [], []
    for k in range(n_layers):
        z = 0.001 * k
        b = len(verts)
        verts += [(-1, -1, z), (1, -1, z), (1, 1, z), (-1, 1, z)]
        idx += [(b, b + 1, b + 2), (b, b + 2, b + 3)]
    return np.array(verts, np.float32), np.array(idx, np.uint32)


def test_traversal_stack_overflow_is_reported_and_context_recovers(engine, oracle, rqm):
    v, f = _stacked_quads(2048)  # 4,096 triangles: an LBVH about 12 levels deep
    prims, aabb, cen = oracle.tri_prims(v, f)
    s = engine.scene_triangles(v, f)
    acc = engine.build(s, rqm.LBVH)
    org = np.array([[0.01 * i - 0.5, 0.013 * i - 0.4, -1.0] for i in range(64)], np.float32)
    rays = oracle.make_rays(org, np.tile(np.array([[0, 0, 1]], np.float32), (64, 1)))
    engine.set_debug(small_stack=1)  # 8 stack entries
    with pytest.raises(rqm.RqError) as e:
        engine.trace_closest(acc, rays)
    assert _status(e) == STACK_OVERFLOW
    engine.set_debug()
    hits = engine.trace_closest(acc, rays)  # the full 64-entry stack
    nodes, order, codes, root, _ = engine.export_bvh2(acc)
    ref = oracle.Bvh2(nodes, len(nodes), root, order, codes)
    want = oracle.trace_bvh2(oracle.TRIANGLES, oracle.FAST, oracle.CLOSEST, ref, prims, rays)
    assert np.array_equal(hits.view(np.uint32), want.view(np.uint32))
    assert (hits["prim"] < 2).all()  # the z = 0 layer is the closest hit of every ray
    acc.close()
    s.close()
    _context_still_traces(engine, oracle, rqm)


def _node(left_box, right_box, links):
    """One 16-word BVH2 node: boxes as (lo xyz, hi xyz); links (left, right, left count, right count)."""
    (lx0, ly0, lz0, lx1, ly1, lz1), (rx0, ry0, rz0, rx1, ry1, rz1) = left_box, right_box
    f = np.array([lx0, lx1, ly0, ly1, rx0, rx1, ry0, ry1, lz0, lz1, rz0, rz1, 0, 0, 0, 0], np.float32)
    f[12:16] = np.array(links, np.int32).view(np.float32)
    return f


def test_cyclic_imported_tree_trips_the_walk_bound_and_context_recovers(engine, oracle, rqm):
    v = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [5, 5, 5], [6, 5, 5], [5, 6, 5]], np.float32)
    f = np.array([[0, 1, 2], [3, 4, 5]], np.uint32)
    s = engine.scene_triangles(v, f)
    scene_box = (-1, -1, -1, 7, 7, 7)
    far_box = (100, 100, 100, 101, 101, 101)  # no test ray reaches it
    # node 0 -> node 1 -> node 0 -> ...: only the left box of each is entered,
    # so the walk never pushes and only the step limit ends it.
    nodes = np.stack([_node(scene_box, far_box, (1, ~0, 0, 1)),
                      _node(scene_box, far_box, (0, ~1, 0, 1))])
    acc = engine.import_bvh2(s, nodes, np.array([0, 1], np.uint32), np.array(scene_box, np.float32))
    rays = oracle.make_rays(np.array([[0.2, 0.2, -2.0]], np.float32), np.array([[0, 0, 1]], np.float32))
    with pytest.raises(rqm.RqError) as e:
        engine.trace_closest(acc, rays)
    assert _status(e) == INVALID_ARGUMENT
    assert "malformed" in str(e.value)
    with pytest.raises(rqm.RqError) as e:
        acc.rebuild()
    assert _status(e) == UNSUPPORTED
    acc.close()
    # links that leave the arrays are refused at import
    bad = nodes.copy()
    bad[1, 12:13] = np.array([7], np.int32).view(np.float32)  # internal child 7 of 2 nodes
    with pytest.raises(rqm.RqError) as e:
        engine.import_bvh2(s, bad, np.array([0, 1], np.uint32), np.array(scene_box, np.float32))
    assert _status(e) == INVALID_ARGUMENT
    bad = nodes.copy()
    bad[0, 13:14] = np.array([~1], np.int32).view(np.float32)
    bad[0, 15:16] = np.array([2], np.int32).view(np.float32)  # slots 1..2 of 2
    with pytest.raises(rqm.RqError) as e:
        engine.import_bvh2(s, bad, np.array([0, 1], np.uint32), np.array(scene_box, np.float32))
    assert _status(e) == INVALID_ARGUMENT
    s.close()
    _context_still_traces(engine, oracle, rqm)


def test_imported_export_traces_like_the_original(engine, oracle, rqm):
    v, f = scenes.displaced_icosphere(4, seed=29)
    lo, hi = oracle.bounds3(v)
    rays = scenes.incoherent_rays(lo, hi, 8192, seed=30)
    s = engine.scene_triangles(v, f)
    for kind, quality in ((rqm.LBVH, rqm.LBVH_KARRAS), (rqm.LBVH, rqm.LBVH_TREELETS), (rqm.BVH, rqm.LBVH_KARRAS)):
        engine.configure(lbvh_quality=quality)  # one-primitive leaves (LBVH, either tree) or several (BVH)
        acc = engine.build(s, kind)
        nodes, order, _, root, _ = engine.export_bvh2(acc)
        imp = engine.import_bvh2(s, nodes, order, root)
        assert np.array_equal(engine.trace_closest(imp, rays).view(np.uint32),
                              engine.trace_closest(acc, rays).view(np.uint32))
        assert np.array_equal(engine.trace_any(imp, rays), engine.trace_any(acc, rays))
        imp.close()
        acc.close()
    s.close()
