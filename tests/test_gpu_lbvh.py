"""GPU parity of the LBVH path (Morton codes, radix sort, Karras topology,
refit) and of BVH2 traversal, through the C ABI, against the CPU oracle on
the same seeded inputs.  Integer results are compared bit for bit; the
traversal performs the oracle's float operations in the oracle's order, so
hit ids, t, u and v are compared bit for bit as well."""
import numpy as np
import pytest

import scenes
from conftest import bvh2_from_export, golden

pytestmark = pytest.mark.gpu


def _tri_scene(level=4, seed=21):
    return scenes.displaced_icosphere(level, seed=seed)


def test_morton_codes_triangles(engine, oracle):
    v, f = _tri_scene()
    s = engine.scene_triangles(v, f)
    codes = engine.morton_codes(s)
    _, _, cen = oracle.tri_prims(v, f)
    lo, hi = oracle.bounds3(v)
    assert np.array_equal(codes, oracle.morton_centroids(cen, lo, hi))


@pytest.mark.parametrize("scene", ["bunny", "synth_a", "synth_c"])
def test_morton_codes_spheres_reference_normalisation(engine, oracle, rqm, scene):
    g = golden(scene)
    engine.configure(morton=rqm.MORTON_REFERENCE)
    s = engine.scene_spheres(g["spheres"])
    assert np.array_equal(engine.morton_codes(s), g["morton"])  # the reference's own codes


def test_morton_codes_spheres_scene_bounds(engine, oracle):
    sph = golden("synth_c")["spheres"]
    s = engine.scene_spheres(sph)
    lo, hi = oracle.bounds3(sph[:, :3])
    assert np.array_equal(engine.morton_codes(s), oracle.morton_centroids(sph[:, :3], lo, hi))


@pytest.mark.parametrize("n", [1, 2, 3, 255, 3840, 3841, 100_003, 1_000_000])
@pytest.mark.parametrize("bits", [30, 32, 24, 7])
def test_sort_pairs_stable(engine, oracle, n, bits):
    rng = np.random.default_rng(n + bits)
    hi = (1 << bits) if n > 1000 else 64  # small cases: heavy duplication
    keys = rng.integers(0, min(hi, 1 << bits), n, dtype=np.uint64).astype(np.uint32)
    vals = np.arange(n, dtype=np.uint32)
    k, v = engine.sort_pairs(keys, vals, key_bits=bits)
    ok, ov = oracle.sort_pairs(keys)
    assert np.array_equal(v, ov)
    assert np.array_equal(k, ok)


def _check_lbvh_against_oracle(engine, oracle, acc, aabb, codes_in):
    nodes, order, codes, root, info = engine.export_bvh2(acc)
    ref = oracle.build_lbvh(codes_in, aabb)
    assert np.array_equal(codes, ref.sorted_codes)
    assert np.array_equal(order, ref.order)
    assert np.array_equal(nodes.view(np.int32), ref.nodes.view(np.int32))  # topology + boxes, bitwise
    assert np.array_equal(root, ref.root_bounds)
    return nodes, order, root


def test_lbvh_triangles_bit_exact(engine, oracle, rqm):
    v, f = _tri_scene(5, seed=22)
    s = engine.scene_triangles(v, f)
    acc = engine.build(s, rqm.LBVH)
    prims, aabb, cen = oracle.tri_prims(v, f)
    lo, hi = oracle.bounds3(v)
    _check_lbvh_against_oracle(engine, oracle, acc, aabb, oracle.morton_centroids(cen, lo, hi))


@pytest.mark.parametrize("scene", ["bunny", "synth_c"])
def test_lbvh_spheres_reference_codes_bit_exact(engine, oracle, rqm, scene):
    g = golden(scene)
    engine.configure(morton=rqm.MORTON_REFERENCE)
    s = engine.scene_spheres(g["spheres"])
    acc = engine.build(s, rqm.LBVH)
    aabb, _ = oracle.sphere_prims(g["spheres"])
    _check_lbvh_against_oracle(engine, oracle, acc, aabb, g["morton"])


def test_lbvh_heightfield_bit_exact(engine, oracle, rqm):
    v, f = scenes.heightfield(201, 100, seed=5)
    s = engine.scene_triangles(v, f)
    acc = engine.build(s, rqm.LBVH)
    prims, aabb, cen = oracle.tri_prims(v, f)
    lo, hi = oracle.bounds3(v)
    _check_lbvh_against_oracle(engine, oracle, acc, aabb, oracle.morton_centroids(cen, lo, hi))


def test_lbvh_full_size_heightfield_bit_exact(engine, oracle, rqm):
    """The 998,000-triangle terrain of the throughput workload with cube
    Morton codes: about 670 treelets and 670 top nodes (the top block); a
    rebuild reproduces the tree."""
    v, f = scenes.heightfield(1001, 500, seed=2)
    engine.configure(morton=rqm.MORTON_SCENE_CUBE)
    s = engine.scene_triangles(v, f)
    acc = engine.build(s, rqm.LBVH)
    _, aabb, cen = oracle.tri_prims(v, f)
    lo, hi = oracle.bounds3(v)
    codes = oracle.morton_centroids(cen, lo, hi, cube=True)
    first = _check_lbvh_against_oracle(engine, oracle, acc, aabb, codes)[0]
    acc.rebuild()
    assert np.array_equal(engine.export_bvh2(acc)[0].view(np.int32), first.view(np.int32))


def test_lbvh_more_top_nodes_than_the_top_block(engine, oracle, rqm):
    """6M uniform points: about 4,100 nodes of more than 2048 leaves, more
    than the top block holds, so the treelet roots climb to the root with
    device-scope arrival counts."""
    pts = np.random.default_rng(7).random((6_000_000, 3), dtype=np.float32)
    sph = np.concatenate([pts, np.full((len(pts), 1), 1e-4, np.float32)], 1)
    acc = engine.build(engine.scene_spheres(sph), rqm.LBVH)
    aabb, _ = oracle.sphere_prims(sph)
    _check_lbvh_against_oracle(engine, oracle, acc, aabb, oracle.morton_centroids(pts, pts.min(0), pts.max(0)))


@pytest.mark.parametrize("group,levels", [(32, 30), (64, 20)])
def test_lbvh_caterpillar_trees_bit_exact(engine, oracle, rqm, group, levels):
    """Caterpillar clusters (each cell's tree peels one group per bit level):
    deep, unbalanced treelets."""
    pts = scenes.chain_clusters(16, group, levels)
    sph = np.concatenate([pts, np.full((len(pts), 1), 1e-3, np.float32)], 1)
    s = engine.scene_spheres(sph)
    acc = engine.build(s, rqm.LBVH)
    aabb, _ = oracle.sphere_prims(sph)
    lo, hi = oracle.bounds3(pts)
    _check_lbvh_against_oracle(engine, oracle, acc, aabb, oracle.morton_centroids(pts, lo, hi))


def test_lbvh_single_and_two_primitives(engine, oracle, rqm):
    for sph in (np.array([[1, 2, 3, 0.5]], np.float32), np.array([[0, 0, -5, 1], [0, 0, -5, 1]], np.float32)):
        s = engine.scene_spheres(sph)
        acc = engine.build(s, rqm.LBVH)
        rays = rqm.make_rays(np.zeros(3), np.array([[0, 0, -1], [0, 1, 0]], np.float32))
        h = engine.trace_closest(acc, rays)
        nodes, order, codes, root, info = engine.export_bvh2(acc)
        ref = bvh2_from_export(oracle, nodes, order, root)
        hr = oracle.trace_bvh2(oracle.SPHERES, oracle.FAST, oracle.CLOSEST, ref, sph, rays)
        assert np.array_equal(h, hr)


def _trace_compare(engine, oracle, acc, kind, prims_by_id, rays, traversal_mode):
    nodes, order, codes, root, info = engine.export_bvh2(acc)
    ref = bvh2_from_export(oracle, nodes, order, root)
    h = engine.trace_closest(acc, rays)
    hr = oracle.trace_bvh2(kind, traversal_mode, oracle.CLOSEST, ref, prims_by_id, rays)
    assert np.array_equal(h.view(np.uint32), hr.view(np.uint32))  # t, prim, u, v bitwise
    bits = engine.trace_any(acc, rays)
    occ = oracle.trace_bvh2(kind, traversal_mode, oracle.ANY, ref, prims_by_id, rays)
    import rq
    assert np.array_equal(rq.unpack_bits(bits, len(rays)), occ)
    return h


def test_trace_triangles_fast_bit_exact(engine, oracle, rqm):
    v, f = _tri_scene(5, seed=23)
    s = engine.scene_triangles(v, f)
    acc = engine.build(s, rqm.LBVH)
    prims, _, _ = oracle.tri_prims(v, f)
    lo, hi = oracle.bounds3(v)
    rays = scenes.incoherent_rays(lo, hi, 50_000, seed=7)
    h = _trace_compare(engine, oracle, acc, oracle.TRIANGLES, prims, rays, oracle.FAST)
    assert (h["prim"] != rqm.MISS).mean() > 0.3
    # the BVH result equals brute force (conservative boxes, same MT arithmetic)
    hn = oracle.trace_brute(oracle.TRIANGLES, oracle.FAST, oracle.CLOSEST, prims, rays[:5000])
    assert np.array_equal(h["t"][:5000], hn["t"])


def test_trace_heightfield_primary_and_secondary(engine, oracle, rqm):
    v, f = scenes.heightfield(301, 150, seed=6)
    s = engine.scene_triangles(v, f)
    acc = engine.build(s, rqm.LBVH)
    prims, _, _ = oracle.tri_prims(v, f)
    rays = scenes.pinhole_rays(160, 90, 2, eye=(0, -2.2, 1.4), target=(0, 0, 0), seed=8)
    h = _trace_compare(engine, oracle, acc, oracle.TRIANGLES, prims, rays, oracle.FAST)
    sec = scenes.cosine_rays(v, f, rays, h, seed=9)
    _trace_compare(engine, oracle, acc, oracle.TRIANGLES, prims, sec, oracle.FAST)
    sh = scenes.shadow_rays(v, f, rays, h, light=(2.0, -1.0, 3.0))
    bits = engine.trace_any(acc, sh)
    nodes, order, codes, root, info = engine.export_bvh2(acc)
    occ = oracle.trace_bvh2(oracle.TRIANGLES, oracle.FAST, oracle.ANY, bvh2_from_export(oracle, nodes, order, root),
                            prims, sh)
    assert np.array_equal(rqm.unpack_bits(bits, len(sh)), occ)


@pytest.mark.parametrize("traversal", [0, 1])
def test_trace_spheres_bunny(engine, oracle, rqm, traversal):
    b = golden("bunny")
    sph = b["spheres"]
    engine.configure(traversal=traversal)
    s = engine.scene_spheres(sph)
    acc = engine.build(s, rqm.LBVH)
    rays = oracle.camera_rays_ref(640, 480, 1, oracle.jitter_mt19937(640 * 480 * 2))
    mode = oracle.REFERENCE if traversal else oracle.FAST
    h = _trace_compare(engine, oracle, acc, oracle.SPHERES, sph, rays, mode)
    if traversal:
        # LBVH + reference semantics against the reference's brute force
        # (NONE) on the 64x48 crop.  Besides ties, the division slab test
        # rejects some grazing boxes the sphere test would accept, so a few
        # rays miss or find a farther sphere -- the reference's own BVH shows
        # the same (118 of 307,200 pixels differ from NONE).
        sel = b["crop_index"]
        ids = h["prim"][sel].astype(np.int32)
        assert (ids == b["crop_none_id"]).mean() > 0.99


@pytest.mark.parametrize("traversal", [0, 1])
def test_none_brute_force(engine, oracle, rqm, traversal):
    b = golden("bunny")
    sph = b["spheres"]
    engine.configure(traversal=traversal)
    s = engine.scene_spheres(sph)
    acc = engine.build(s, rqm.NONE)
    rays = oracle.make_rays(b["crop_rays"][:, :3], b["crop_rays"][:, 3:])
    h = engine.trace_closest(acc, rays)
    mode = oracle.REFERENCE if traversal else oracle.FAST
    hr = oracle.trace_brute(oracle.SPHERES, mode, oracle.CLOSEST, sph, rays)
    assert np.array_equal(h.view(np.uint32), hr.view(np.uint32))
    if traversal:
        assert np.array_equal(h["prim"].astype(np.int32), b["crop_none_id"])
        t = np.where(h["prim"] == rqm.MISS, np.float32(np.inf), h["t"])
        assert np.array_equal(t, b["crop_none_t"])
    v, f = _tri_scene(3, seed=24)
    st = engine.scene_triangles(v, f)
    at = engine.build(st, rqm.NONE)
    prims, _, _ = oracle.tri_prims(v, f)
    lo, hi = oracle.bounds3(v)
    rays = scenes.incoherent_rays(lo, hi, 3072, seed=10)
    h = engine.trace_closest(at, rays)
    hr = oracle.trace_brute(oracle.TRIANGLES, oracle.FAST, oracle.CLOSEST, prims, rays)
    assert np.array_equal(h.view(np.uint32), hr.view(np.uint32))
    occ = oracle.trace_brute(oracle.TRIANGLES, oracle.FAST, oracle.ANY, prims, rays)
    assert np.array_equal(rqm.unpack_bits(engine.trace_any(at, rays), len(rays)), occ)


def test_device_pointer_path_and_rebuild(engine, oracle, rqm):
    import torch
    v, f = _tri_scene(4, seed=25)
    dv = torch.from_numpy(v).cuda()
    df = torch.from_numpy(f.astype(np.int32)).cuda()
    s = engine.scene_triangles(dv, df)
    acc = engine.build(s, rqm.LBVH)
    lo, hi = oracle.bounds3(v)
    rays = scenes.incoherent_rays(lo, hi, 10_000, seed=11)
    dr = torch.from_numpy(rays.view(np.uint8)).cuda()
    dh = torch.zeros(len(rays) * 16, dtype=torch.uint8, device="cuda")
    engine.set_stream(torch.cuda.current_stream().cuda_stream)
    engine.trace_closest(acc, dr, dh)
    engine.synchronize()
    h_dev = dh.cpu().numpy().view(rqm.HIT_DTYPE)
    h_host = engine.trace_closest(acc, rays)
    assert np.array_equal(h_dev.view(np.uint32), h_host.view(np.uint32))
    # move the mesh, rebuild in place, results follow the oracle
    v2 = (v * 0.5 + 0.25).astype(np.float32)
    s.update(v2)
    acc.rebuild()
    prims, aabb, cen = oracle.tri_prims(v2, f)
    lo2, hi2 = oracle.bounds3(v2)
    ref = oracle.build_lbvh(oracle.morton_centroids(cen, lo2, hi2), aabb)
    h2 = engine.trace_closest(acc, rays)
    hr = oracle.trace_bvh2(oracle.TRIANGLES, oracle.FAST, oracle.CLOSEST, ref, prims, rays)
    assert np.array_equal(h2.view(np.uint32), hr.view(np.uint32))


def test_errors_are_reported(engine, rqm):
    with pytest.raises(rqm.RqError) as e:
        engine.scene_spheres(np.zeros((0, 4), np.float32))
    assert e.value.status == 7  # EMPTY_SCENE
    with pytest.raises(rqm.RqError) as e:
        engine.scene_triangles(np.array([[0, 0, np.nan]] * 3, np.float32), np.array([[0, 1, 2]], np.uint32))
    assert e.value.status == 1
    with pytest.raises(rqm.RqError) as e:
        engine.scene_triangles(np.zeros((3, 3), np.float32), np.array([[0, 1, 5]], np.uint32))
    assert e.value.status == 1
    s = engine.scene_spheres(np.array([[0, 0, 0, 1]], np.float32))
    with pytest.raises(rqm.RqError) as e:
        engine.build(s, rqm.UNIFORM_GRID)
    assert e.value.status == 2
    import torch
    bad = torch.tensor([[0, 0, 0, 1], [0, float("nan"), 0, 1]], dtype=torch.float32, device="cuda")
    with pytest.raises(rqm.RqError) as e:
        engine.scene_spheres(bad)
    assert e.value.status == 1
    # the context stays usable afterwards
    acc = engine.build(s, rqm.LBVH)
    h = engine.trace_closest(acc, rqm.make_rays(np.array([0, 0, 5.0]), np.array([[0, 0, -1]], np.float32)))
    assert h["prim"][0] == 0


def test_rejected_host_update_keeps_the_scene(engine, oracle, rqm):
    """Host geometry is validated on the device before it replaces the scene's:
    a rejected update (NaN vertex, index out of range) changes nothing."""
    v, f = scenes.displaced_icosphere(4, seed=23)
    s = engine.scene_triangles(v, f)
    acc = engine.build(s, "LBVH")
    lo, hi = oracle.bounds3(v)
    rays = scenes.incoherent_rays(lo, hi, 5000, seed=24)
    before = engine.trace_closest(acc, rays)
    bad = v.copy()
    bad[7, 1] = np.nan
    with pytest.raises(rqm.RqError) as e:
        s.update(bad)
    assert e.value.status == 1
    bad_idx = f.copy()
    bad_idx[3, 2] = len(v)
    with pytest.raises(rqm.RqError) as e:
        s.update(v * np.float32(2), bad_idx)
    assert e.value.status == 1
    acc.rebuild()
    assert np.array_equal(engine.trace_closest(acc, rays).view(np.uint32), before.view(np.uint32))


def test_cube_morton_normalisation(engine, oracle, rqm):
    """RQ_MORTON_SCENE_CUBE: codes and LBVH equal the oracle's cube
    normalisation bit for bit, batched builds equal single builds, and FAST
    query results equal the per-axis tree's (the closest-hit rule)."""
    v, f = scenes.heightfield(301, 150, seed=31)
    s = engine.scene_triangles(v, f)
    flat = engine.build(s, "LBVH")
    engine.configure(morton=rqm.MORTON_SCENE_CUBE)
    prims, aabb, cen = oracle.tri_prims(v, f)
    lo, hi = oracle.bounds3(v)
    want_codes = oracle.morton_centroids(cen, lo, hi, cube=True)
    assert np.array_equal(engine.morton_codes(s), want_codes)
    assert not np.array_equal(want_codes, oracle.morton_centroids(cen, lo, hi))
    acc = engine.build(s, "LBVH")
    nodes, order, codes, root, _ = engine.export_bvh2(acc)
    ref = oracle.build_lbvh(want_codes, aabb)
    assert np.array_equal(codes, ref.sorted_codes) and np.array_equal(order, ref.order)
    assert np.array_equal(nodes.view(np.uint32), ref.nodes.view(np.uint32))
    rays = scenes.pinhole_rays(200, 120, 2, eye=(0, -0.6, 1.1), target=(0, 0, 0), seed=32)
    hits = engine.trace_closest(acc, rays)
    assert np.array_equal(hits.view(np.uint32), engine.trace_closest(flat, rays).view(np.uint32))
    assert np.array_equal(engine.trace_any(acc, rays), engine.trace_any(flat, rays))
    want = oracle.trace_bvh2(oracle.TRIANGLES, oracle.FAST, oracle.CLOSEST, ref, prims, rays)
    assert np.array_equal(hits.view(np.uint32), want.view(np.uint32))
    # batched, with a sphere batch too
    batch = engine.build_batched([s], "LBVH")
    for g, w in zip(engine.export_bvh2(batch[0])[:3], (nodes, order, codes)):
        assert np.array_equal(np.asarray(g).view(np.uint32), np.asarray(w).view(np.uint32))
    sph = golden("synth_c")["spheres"]
    ss = engine.scene_spheres(sph)
    sa = engine.build(ss, "LBVH")
    slo, shi = oracle.bounds3(sph[:, :3])
    assert np.array_equal(engine.morton_codes(ss), oracle.morton_centroids(sph[:, :3], slo, shi, cube=True))
    sb = engine.build_batched([ss], "LBVH")[0]
    assert np.array_equal(engine.export_bvh2(sb)[0].view(np.uint32), engine.export_bvh2(sa)[0].view(np.uint32))
