"""Engine options that change speed, never results: ray reordering for
coherence (settings.ray_sort) must give bit-identical hits and occlusion bits,
in the caller's order, for closest and any-hit queries."""
import os

import numpy as np
import pytest

import scenes

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("acc_name", ["LBVH", "BVH"])
@pytest.mark.parametrize("key", ["OCTANT_MORTON", "ORIGIN_DIRECTION", "DIRECTION_ORIGIN", "OCTANT_MORTON12", "OCTANT",
                                 "OCTANT_MORTON3"])
def test_ray_sort_is_result_neutral(engine, oracle, rqm, acc_name, key):
    v, f = scenes.heightfield(301, 150, seed=12)
    s = engine.scene_triangles(v, f)
    acc = engine.build(s, acc_name)
    primary = scenes.pinhole_rays(320, 180, 2, eye=(0, -0.6, 1.1), target=(0, 0, 0), seed=13)
    h0 = engine.trace_closest(acc, primary)
    sec = scenes.cosine_rays(v, f, primary, h0, seed=14)
    assert len(sec) >= 65536  # above the reordering threshold
    ref_c = engine.trace_closest(acc, sec)
    ref_a = engine.trace_any(acc, sec)
    engine.configure(ray_sort=getattr(rqm, "RAY_SORT_" + key))
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


def test_streamed_host_queries_equal_device_queries(engine, rqm):
    """Host-buffer batches of two or more 2^21-ray chunks are uploaded, traced
    and downloaded chunk by chunk on three streams; results equal the
    device-pointer query, for pageable and pinned host memory."""
    torch = pytest.importorskip("torch")
    v, f = scenes.heightfield(301, 150, seed=15)
    acc = engine.build(engine.scene_triangles(v, f), "LBVH")
    rays = scenes.pinhole_rays(1250, 1000, 4, eye=(0, -0.6, 1.1), target=(0, 0, 0), seed=16)
    n = len(rays)
    assert n > 2 * (1 << 21) and n % (1 << 21) != 0  # three chunks, the last partial
    d_rays = torch.from_numpy(rays.view(np.uint8)).cuda()
    d_hits = torch.empty(n * 16, dtype=torch.uint8, device="cuda")
    d_bits = torch.empty(((n + 31) // 32) * 4, dtype=torch.uint8, device="cuda")
    engine.trace_closest(acc, d_rays, d_hits)
    engine.trace_any(acc, d_rays, d_bits)
    engine.synchronize()
    want_h = d_hits.cpu().numpy().view(np.uint32)
    want_b = d_bits.cpu().numpy().view(np.uint32)
    # pageable
    assert np.array_equal(engine.trace_closest(acc, rays).view(np.uint32).ravel(), want_h)
    assert np.array_equal(engine.trace_any(acc, rays), want_b)
    # pinned
    p_rays = torch.empty(n * 32, dtype=torch.uint8, pin_memory=True)
    p_rays.numpy()[:] = rays.view(np.uint8)
    p_hits = torch.empty(n * 16, dtype=torch.uint8, pin_memory=True)
    hr = p_rays.numpy().view(rqm.RAY_DTYPE)
    hh = p_hits.numpy().view(rqm.HIT_DTYPE)
    engine.configure(ray_sort=rqm.RAY_SORT_OCTANT_MORTON)
    engine.trace_closest(acc, hr, hh)
    assert np.array_equal(hh.view(np.uint32).ravel(), want_h)


@pytest.mark.parametrize("acc_name", ["LBVH", "BVH"])
@pytest.mark.parametrize("ray_sort", [0, 1])
@pytest.mark.parametrize("sched", ["LANE_REFILL", "SPECULATIVE", "WARP_PACKET", "SHARED_TOP"])
def test_scheduling_is_result_neutral(engine, oracle, rqm, acc_name, ray_sort, sched):
    """Persistent warps that refill finished lanes, the speculative
    while-while walk, the warp-packet walk and the walk that stages the top
    tree levels in shared memory (settings.scheduling) give
    bit-identical hits and occlusion bits, with and without ray reordering,
    for camera and secondary rays, triangles and spheres, equal to the
    oracle's plain walk."""
    mode = getattr(rqm, "SCHEDULING_" + sched)
    v, f = scenes.heightfield(301, 150, seed=17)
    s = engine.scene_triangles(v, f)
    acc = engine.build(s, acc_name)
    primary = scenes.pinhole_rays(320, 180, 2, eye=(0, -0.6, 1.1), target=(0, 0, 0), seed=18)
    h0 = engine.trace_closest(acc, primary)
    sec = scenes.cosine_rays(v, f, primary, h0, seed=19)
    ref_c = engine.trace_closest(acc, sec)
    ref_a = engine.trace_any(acc, sec)
    ref_pa = engine.trace_any(acc, primary)
    engine.configure(scheduling=mode, ray_sort=ray_sort)
    assert np.array_equal(engine.trace_closest(acc, primary).view(np.uint32), h0.view(np.uint32))
    assert np.array_equal(engine.trace_any(acc, primary), ref_pa)
    assert np.array_equal(engine.trace_closest(acc, sec).view(np.uint32), ref_c.view(np.uint32))
    assert np.array_equal(engine.trace_any(acc, sec), ref_a)
    for n in (1, 31, 33, 1000):  # partial warps and tiny batches
        assert np.array_equal(engine.trace_closest(acc, sec[:n]).view(np.uint32), ref_c[:n].view(np.uint32))
        want = rqm.unpack_bits(ref_a, len(sec))[:n]
        assert np.array_equal(rqm.unpack_bits(engine.trace_any(acc, sec[:n]), n), want)
    nodes, order, _, root, _ = engine.export_bvh2(acc)
    prims, _, _ = oracle.tri_prims(v, f)
    want = oracle.trace_bvh2(oracle.TRIANGLES, oracle.FAST, oracle.CLOSEST, oracle.Bvh2(nodes, len(nodes), root, order),
                             prims, sec)
    assert np.array_equal(ref_c.view(np.uint32), want.view(np.uint32))
    # spheres
    sph = np.load(os.path.join(os.path.dirname(__file__), "golden", "synth_c.npz"))["spheres"]
    engine.configure(scheduling=rqm.SCHEDULING_THREAD_PER_RAY)
    ss = engine.build(engine.scene_spheres(sph), acc_name)
    c = sph[:, :3]
    rays = scenes.incoherent_rays(c.min(0) - 2, c.max(0) + 2, 70_000, seed=20)
    base_c, base_a = engine.trace_closest(ss, rays), engine.trace_any(ss, rays)
    engine.configure(scheduling=mode)
    assert np.array_equal(engine.trace_closest(ss, rays).view(np.uint32), base_c.view(np.uint32))
    assert np.array_equal(engine.trace_any(ss, rays), base_a)


def test_trace_queries_equal_single_queries(engine, rqm):
    """rq_trace_queries (copies and traversals overlapped across queries, the
    first streamed in chunks) returns exactly the results of one call per
    query, with per-query ray order and scheduling."""
    v, f = scenes.heightfield(301, 150, seed=21)
    acc = engine.build(engine.scene_triangles(v, f), "LBVH")
    primary = scenes.pinhole_rays(1250, 1000, 4, eye=(0, -0.6, 1.1), target=(0, 0, 0), seed=22)  # 5M: streamed
    h0 = engine.trace_closest(acc, primary)
    sec = scenes.cosine_rays(v, f, primary[:700_000], h0[:700_000], seed=23)
    sh = scenes.shadow_rays(v, f, primary[:300_000], h0[:300_000], (1.5, -1.0, 3.0))
    want = [h0, engine.trace_closest(acc, sec), engine.trace_any(acc, sh), engine.trace_closest(acc, primary[:10])]
    got = engine.trace_queries(acc, [(primary, False, None, -1, -1),
                                     (sec, False, None, rqm.RAY_SORT_OCTANT_MORTON12, -1),
                                     (sh, True, None, -1, rqm.SCHEDULING_SPECULATIVE),
                                     (primary[:10], False, None, -1, -1)])
    for g, w in zip(got, want):
        assert np.array_equal(np.ascontiguousarray(g).view(np.uint32), np.ascontiguousarray(w).view(np.uint32))
    # a short first query takes the whole-buffer path too
    got = engine.trace_queries(acc, [(sec, False, None, -1, -1), (sh, True, None, -1, -1)])
    assert np.array_equal(got[0].view(np.uint32), want[1].view(np.uint32))
    assert np.array_equal(got[1], want[2])
    # so does a large first query with a ray order; back-to-back calls reuse the buffers
    for _ in range(2):
        got = engine.trace_queries(acc, [(primary, False, None, rqm.RAY_SORT_OCTANT_MORTON12, -1),
                                         (sec, False, None, -1, -1), (sh, True, None, -1, -1)])
        assert np.array_equal(got[0].view(np.uint32), h0.view(np.uint32))
        assert np.array_equal(got[1].view(np.uint32), want[1].view(np.uint32))
        assert np.array_equal(got[2], want[2])


def test_trace_queries_follow_a_queued_rebuild(engine, rqm):
    """The uploads of rq_trace_queries overlap a rebuild queued just before
    the call; the traversals must still see the rebuilt structure."""
    v, f = scenes.heightfield(301, 150, seed=24)
    s = engine.scene_triangles(v, f)
    acc = engine.build(s, "LBVH")
    primary = scenes.pinhole_rays(1250, 1000, 4, eye=(0, -0.6, 1.1), target=(0, 0, 0), seed=25)
    engine.trace_queries(acc, [(primary, False, None, -1, -1)])  # buffers of the old geometry in flight before
    v2 = v.copy()
    v2[:, 2] += 0.05 * np.sin(7.0 * v[:, 0]).astype(np.float32)
    s.update(v2)
    acc.rebuild()
    got = engine.trace_queries(acc, [(primary, False, None, rqm.RAY_SORT_OCTANT_MORTON12, -1),
                                     (primary[:1_000_000], True, None, -1, -1)])
    ref = engine.build(engine.scene_triangles(v2, f), "LBVH")
    assert np.array_equal(got[0].view(np.uint32), engine.trace_closest(ref, primary).view(np.uint32))
    assert np.array_equal(got[1], engine.trace_any(ref, primary[:1_000_000]))
