"""Many structures at once: the batched LBVH build (rq_build_batched) equals
the single builds bit for bit, scene by scene; the persistent many-structure
query (rq_trace_batched) equals the one-structure queries; a plan replays
[rebuild +] query as one CUDA graph with the same results after the inputs
change; the autotuner's choice is a shape that ran."""
import numpy as np
import pytest

import scenes
from conftest import bvh2_from_export, golden

pytestmark = pytest.mark.gpu


def _meshes(seed=60, count=9):
    rng = np.random.default_rng(seed)
    out = []
    for k in range(count):
        lv = int(rng.integers(1, 5))
        v, f = scenes.displaced_icosphere(lv, seed=seed + k)
        v = (v * np.float32(rng.uniform(0.5, 3.0)) + rng.uniform(-5, 5, 3).astype(np.float32)).astype(np.float32)
        out.append((v, f))
    # degenerate sizes: one and two triangles
    out.append((np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32), np.array([[0, 1, 2]], np.uint32)))
    out.append((np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [1, 1, 1]], np.float32),
                np.array([[0, 1, 2], [1, 3, 2]], np.uint32)))
    return out


def _export(engine, acc):
    nodes, order, codes, root, info = engine.export_bvh2(acc)
    return nodes.view(np.uint32), order, codes, root.view(np.uint32)


def _rays_for(meshes, seed, per=(500, 3000)):
    rng = np.random.default_rng(seed)
    parts, offs = [], [0]
    for k, (v, f) in enumerate(meshes):
        n = int(rng.integers(*per)) if k % 4 != 3 else 0  # some structures get no rays
        if n:
            parts.append(scenes.incoherent_rays(v.min(0), v.max(0), n, seed=seed + k))
        offs.append(offs[-1] + n)
    return np.concatenate(parts), np.array(offs, np.uint32)


def test_batched_build_equals_single_builds(engine, oracle):
    meshes = _meshes()
    sc = [engine.scene_triangles(v, f) for v, f in meshes]
    batch = engine.build_batched(sc, "LBVH")
    for (v, f), s, acc in zip(meshes, sc, batch):
        single = engine.build(s, "LBVH")
        got, want = _export(engine, acc), _export(engine, single)
        for g, w in zip(got, want):
            assert np.array_equal(g, w)
        info = acc.info()
        assert info.n_prims == len(f) and info.n_nodes == max(len(f) - 1, 0)
        prims, aabb, cen = oracle.tri_prims(v, f)
        lo, hi = oracle.bounds3(v)
        ref = oracle.build_lbvh(oracle.morton_centroids(cen, lo, hi), aabb)
        assert np.array_equal(got[1], ref.order)


def test_batched_build_spheres_reference_morton(engine, rqm):
    engine.configure(morton=rqm.MORTON_REFERENCE)
    sph = [golden(n)["spheres"] for n in ("bunny", "synth_a", "synth_c")]
    sph.append(np.array([[1, 2, 3, 0.5]], np.float32))
    sc = [engine.scene_spheres(s) for s in sph]
    batch = engine.build_batched(sc, "LBVH")
    for s, acc in zip(sc, batch):
        single = engine.build(s, "LBVH")
        for g, w in zip(_export(engine, acc), _export(engine, single)):
            assert np.array_equal(g, w)


def test_batched_rebuild_after_updates(engine):
    meshes = _meshes(seed=70, count=5)
    sc = [engine.scene_triangles(v, f) for v, f in meshes]
    batch = engine.build_batched(sc, "LBVH")
    for k, (v, f) in enumerate(meshes):
        if k % 2 == 0:
            sc[k].update((v * np.float32(1.5) + np.float32(k)).astype(np.float32))
    engine.rebuild_batched(batch)
    engine.synchronize()
    for s, acc in zip(sc, batch):
        single = engine.build(s, "LBVH")
        for g, w in zip(_export(engine, acc), _export(engine, single)):
            assert np.array_equal(g, w)
    # rebuilding a single member in place works too
    batch[1].rebuild()
    single = engine.build(sc[1], "LBVH")
    for g, w in zip(_export(engine, batch[1]), _export(engine, single)):
        assert np.array_equal(g, w)


@pytest.mark.parametrize("width", [2, 4])
@pytest.mark.parametrize("ray_order", [0, 1])
def test_batched_query_equals_single_queries(engine, rqm, width, ray_order):
    """Hits and occlusion bits of the many-structure query equal the
    one-structure queries, with and without the per-scene ray order
    (settings.ray_sort)."""
    engine.configure(node_width=rqm.NODE_WIDTH_4 if width == 4 else rqm.NODE_WIDTH_2)
    meshes = _meshes(seed=80)
    sc = [engine.scene_triangles(v, f) for v, f in meshes]
    accs = engine.build_batched(sc, "LBVH")
    accs[2] = engine.build(sc[2], "BVH")  # structures need not come from one batch
    rays, offs = _rays_for(meshes, seed=81)
    engine.configure(ray_sort=ray_order)
    hits = engine.trace_batched(accs, rays, offs)
    bits = engine.trace_batched(accs, rays, offs, any_hit=True)
    engine.configure(ray_sort=rqm.RAY_SORT_NONE)
    occ = rqm.unpack_bits(bits, len(rays))
    for k, acc in enumerate(accs):
        a, b = offs[k], offs[k + 1]
        if a == b:
            continue
        want = engine.trace_closest(acc, rays[a:b])
        assert np.array_equal(hits[a:b].view(np.uint32), want.view(np.uint32))
        assert np.array_equal(occ[a:b], rqm.unpack_bits(engine.trace_any(acc, rays[a:b]), b - a))


def test_plan_replays_rebuild_and_query(engine, rqm):
    torch = pytest.importorskip("torch")
    meshes = _meshes(seed=90)
    sc = [engine.scene_triangles(v, f) for v, f in meshes]
    accs = engine.build_batched(sc, "LBVH")
    rays, offs = _rays_for(meshes, seed=91, per=(2000, 20000))
    n = len(rays)
    d_rays = torch.from_numpy(rays.view(np.uint8)).cuda()
    d_hits = torch.zeros(n * 16, dtype=torch.uint8, device="cuda")
    launches0 = rqm.kernel_launch_count()
    plan = engine.plan(accs, d_rays, offs, d_hits, rebuild=True)
    info = plan.info()
    assert info.block_threads in (128, 256) and info.n_rays == n and info.rebuilds == 1
    assert info.graph_kernels >= 8  # the batched build's stages + the query
    assert max(info.shape_ms) > 0 and max(info.ordered_ms) > 0  # both variants timed
    deep_entries = {2: 64, 4: 96, 8: 32}[info.node_width]  # the tuner also picked the node width
    k = [128, 128, 256, 256].index(info.block_threads) + (1 if info.stack_entries == deep_entries else 0)
    chosen = (info.ordered_ms if info.ray_order else info.shape_ms)[k]
    assert chosen == min(t for t in list(info.shape_ms) + list(info.ordered_ms) if t >= 0)
    assert min(info.width_ms) > 0 and chosen == min(info.width_ms)  # binary, 4-wide and 8-wide all timed
    assert accs[0].info().node_width == info.node_width
    # move every mesh, then one replay rebuilds and traces
    for k2, (v, f) in enumerate(meshes):
        sc[k2].update((v + np.float32(0.25 * k2)).astype(np.float32))
    rays2, _ = _rays_for([(v + np.float32(0.25 * k2), f) for k2, (v, f) in enumerate(meshes)], seed=91,
                         per=(2000, 20000))
    d_rays.copy_(torch.from_numpy(rays2.view(np.uint8)))
    before = rqm.kernel_launch_count()
    plan.launch()
    engine.synchronize()
    assert rqm.kernel_launch_count() - before == info.graph_kernels
    got = d_hits.cpu().numpy().view(rqm.HIT_DTYPE)
    for k2, s in enumerate(sc):
        a, b = offs[k2], offs[k2 + 1]
        if a == b:
            continue
        single = engine.build(s, "LBVH")
        want = engine.trace_closest(single, rays2[a:b])
        assert np.array_equal(got[a:b].view(np.uint32), want.view(np.uint32))
    plan.close()
    assert rqm.kernel_launch_count() > launches0


def test_batch_errors(engine, rqm):
    v, f = scenes.displaced_icosphere(2, seed=3)
    t = engine.scene_triangles(v, f)
    s = engine.scene_spheres(np.array([[0, 0, 0, 1]], np.float32))
    with pytest.raises(rqm.RqError):
        engine.build_batched([t, s], "LBVH")  # mixed kinds
    a = engine.build(t, "LBVH")
    rays = scenes.incoherent_rays(v.min(0), v.max(0), 100, seed=4)
    with pytest.raises(rqm.RqError):
        engine.trace_batched([a], rays, np.array([1, 100], np.uint32))  # offsets must start at 0
    k = engine.build(t, "KDTREE")
    with pytest.raises(rqm.RqError):
        engine.trace_batched([k], rays, np.array([0, 100], np.uint32))  # BVH structures only
    import torch
    d = torch.from_numpy(rays.view(np.uint8)).cuda()
    o = torch.zeros(100 * 16, dtype=torch.uint8, device="cuda")
    with pytest.raises(rqm.RqError):
        engine.plan([a], d, np.array([0, 100], np.uint32), o, rebuild=True)  # not a batch
    # other types build scene by scene
    kd = engine.build_batched([t, t], "KDTREE")
    assert kd[0].info().type == rqm.KDTREE
