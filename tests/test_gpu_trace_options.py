"""Engine options that change speed, never results: ray reordering for
coherence (settings.ray_sort) must give bit-identical hits and occlusion bits,
in the caller's order, for closest and any-hit queries."""
import numpy as np
import pytest

import scenes

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("acc_name", ["LBVH", "BVH"])
def test_ray_sort_is_result_neutral(engine, oracle, rqm, acc_name):
    v, f = scenes.heightfield(301, 150, seed=12)
    s = engine.scene_triangles(v, f)
    acc = engine.build(s, acc_name)
    primary = scenes.pinhole_rays(320, 180, 2, eye=(0, -0.6, 1.1), target=(0, 0, 0), seed=13)
    h0 = engine.trace_closest(acc, primary)
    sec = scenes.cosine_rays(v, f, primary, h0, seed=14)
    assert len(sec) >= 65536  # above the reordering threshold
    ref_c = engine.trace_closest(acc, sec)
    ref_a = engine.trace_any(acc, sec)
    engine.configure(ray_sort=rqm.RAY_SORT_OCTANT_MORTON)
    got_c = engine.trace_closest(acc, sec)
    got_a = engine.trace_any(acc, sec)
    assert np.array_equal(got_c.view(np.uint32), ref_c.view(np.uint32))
    assert np.array_equal(got_a, ref_a)
    # and against the oracle on the exported tree
    nodes, order, _, root, _ = engine.export_bvh2(acc)
    prims, _, _ = oracle.tri_prims(v, f)
    ref = oracle.Bvh2(nodes, len(nodes), root, order)
    want = oracle.trace_bvh2(oracle.TRIANGLES, oracle.FAST, oracle.CLOSEST, ref, prims, sec)
    assert np.array_equal(got_c.view(np.uint32), want.view(np.uint32))
