"""GPU parity of rq_trace_candidates: boxIntersect's candidate lists
(accelerators.h:668-690) for a batch of rays, compared id for id with the
oracle's walk over the same exported tree, and castRay's selection over those
lists (main.cpp:330-358) compared with the engine's own reference-mode
closest hits."""
import numpy as np
import pytest

import scenes
from conftest import bvh2_from_export, golden

pytestmark = pytest.mark.gpu


def _oracle_lists(engine, oracle, acc, rays):
    nodes, order, _, root, _ = engine.export_bvh2(acc)
    return oracle.candidates_bvh2(bvh2_from_export(oracle, nodes, order, root), rays)


@pytest.mark.parametrize("structure", ["BVH", "LBVH"])
def test_candidates_bunny_match_oracle(engine, oracle, rqm, structure):
    b = golden("bunny")
    sph = b["spheres"]
    engine.configure(morton=rqm.MORTON_REFERENCE)
    acc = engine.build(engine.scene_spheres(sph), getattr(rqm, structure))
    rays = oracle.camera_rays_ref(640, 480, 1, oracle.jitter_mt19937(640 * 480 * 2))
    counts, ids = engine.trace_candidates(acc, rays)
    rc, ri = _oracle_lists(engine, oracle, acc, rays)
    assert np.array_equal(counts, rc)
    assert np.array_equal(ids, ri)
    # castRay over the lists = the engine's reference-mode closest hit
    engine.configure(traversal=1)
    h = engine.trace_closest(acc, rays)
    offs = np.concatenate([[0], np.cumsum(counts.astype(np.int64))])
    for r in b["crop_index"][::16]:
        lst = ids[offs[r]:offs[r + 1]]
        hr = oracle.trace_brute(oracle.SPHERES, oracle.REFERENCE, oracle.CLOSEST, sph[lst], rays[r:r + 1])
        want = rqm.MISS if hr["prim"][0] == oracle.MISS else int(lst[hr["prim"][0]])
        assert int(h["prim"][r]) == want
        if want != rqm.MISS:
            assert h["t"][r] == hr["t"][0]


@pytest.mark.parametrize("structure", ["BVH", "LBVH"])
def test_candidates_triangles_match_oracle(engine, oracle, rqm, structure):
    v, f = scenes.heightfield(201, 100, seed=5)
    acc = engine.build(engine.scene_triangles(v, f), getattr(rqm, structure))
    lo, hi = oracle.bounds3(v)
    rays = scenes.incoherent_rays(lo, hi, 8192, seed=6)
    counts, ids = engine.trace_candidates(acc, rays)
    rc, ri = _oracle_lists(engine, oracle, acc, rays)
    assert np.array_equal(counts, rc)
    assert np.array_equal(ids, ri)
    assert counts.sum() > len(rays)  # the walk reaches leaves
    # every primitive the closest hit names is on its ray's list
    h = engine.trace_closest(acc, rays)
    offs = np.concatenate([[0], np.cumsum(counts.astype(np.int64))])
    for r in np.flatnonzero(h["prim"] != rqm.MISS)[:500]:
        assert h["prim"][r] in ids[offs[r]:offs[r + 1]]


def test_candidates_edges(engine, oracle, rqm):
    import ctypes as C
    sph = golden("synth_a")["spheres"]
    s = engine.scene_spheres(sph)
    acc = engine.build(s, rqm.BVH)
    # no rays
    counts, ids = engine.trace_candidates(acc, np.zeros(0, rqm.RAY_DTYPE))
    assert len(counts) == 0 and len(ids) == 0
    # one primitive: the root is a leaf
    one = engine.build(engine.scene_spheres(sph[:1]), rqm.LBVH)
    d = sph[0, :3] - np.array([0, 0, 10], np.float32)
    rays = rqm.make_rays(np.array([[0, 0, 10]], np.float32), d[None] / np.linalg.norm(d))
    counts, ids = engine.trace_candidates(one, rays)
    assert counts.tolist() == [1] and ids.tolist() == [0]
    # a ray missing the root box: an empty list
    rays = rqm.make_rays(np.array([[0, 0, 1e6]], np.float32), np.array([[0, 0, 1]], np.float32))
    counts, ids = engine.trace_candidates(acc, rays)
    assert counts.tolist() == [0] and len(ids) == 0
    # an ids buffer smaller than the total: an error, counts and total still written
    lo, hi = sph[:, :3].min(0), sph[:, :3].max(0)
    rays = scenes.incoherent_rays(lo, hi, 256, seed=3)
    counts, ids = engine.trace_candidates(acc, rays)
    lib = rqm.load()
    c2 = np.zeros(len(rays), np.uint32)
    small = np.zeros(max(len(ids) - 1, 1), np.uint32)
    total = C.c_uint64(0)
    st = lib.rq_trace_candidates(engine.ctx, acc.handle, rays.ctypes.data, len(rays), c2.ctypes.data,
                                 small.ctypes.data, len(ids) - 1, C.byref(total), 0)
    assert st == 1  # RQ_ERROR_INVALID_ARGUMENT
    assert total.value == len(ids) and np.array_equal(c2, counts)
    # KD trees have no candidate lists
    kd = engine.build(s, rqm.KDTREE)
    with pytest.raises(rqm.RqError):
        engine.trace_candidates(kd, rays)
    # the context stays usable
    c3, i3 = engine.trace_candidates(acc, rays)
    assert np.array_equal(c3, counts) and np.array_equal(i3, ids)
