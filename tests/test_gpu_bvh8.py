"""GPU parity of the compressed 8-wide BVH (settings.node_width = 8).

The 8-wide copy quantises child boxes to bytes (rounded outward) and visits
children in an order set by each ray's direction signs; FAST closest hit keeps
the smallest t and, on exact ties, the smallest primitive id, so its results
must equal the binary walk's, and the oracle's, bit for bit.  The structure
itself is checked on the host from rq_accel_export_bvh4: every decoded child
box contains every primitive below it and every binary slot sits in exactly
one leaf.

Triangle path: no reference implementation; parity vs the restated oracle."""
import numpy as np
import pytest

import scenes
from conftest import bvh2_from_export, golden

pytestmark = pytest.mark.gpu


def _u32(a):
    return np.ascontiguousarray(a).view(np.uint32)


def _decode(node):
    """(valid mask, lo (8, 3), hi (8, 3), link (8,), count (8,)) of one exported 8-wide node.
    plane = S * (1 + q 2^-15) + pm: exact in double, rounded once to float32 as the device's fma."""
    w = node.view(np.uint32)
    pm = node[:3].astype(np.float64)
    E = np.array([w[3] & 0xFF, (w[3] >> 8) & 0xFF, (w[3] >> 16) & 0xFF], np.int64)
    S = np.ldexp(1.0, E - 127)
    valid = int(w[3] >> 24)
    q = w[4:16].view(np.uint8).reshape(3, 2, 8).astype(np.float64)  # axis, (lo, hi), slot
    F = 1.0 + q * 2.0 ** -15
    planes = (S[:, None, None] * F + pm[:, None, None]).astype(np.float32)
    lo, hi = planes[:, 0, :].T, planes[:, 1, :].T
    lc = w[16:32].view(np.int32).reshape(8, 2)
    return valid, lo, hi, lc[:, 0], lc[:, 1]


def _check_structure(engine, acc, prim_lo, prim_hi):
    nodes, order, _, root, info = engine.export_bvh2(acc)
    wide = engine.export_bvh4(acc)
    assert acc.info().node_width == 8 and len(wide) == acc.info().n_wide_nodes
    n_slots = len(order)
    seen = np.zeros(n_slots, np.int32)

    def subtree(k):  # slots below wide node k
        valid, lo, hi, link, count = _decode(wide[k])
        out = []
        for s in range(8):
            if not (valid >> s) & 1:
                continue
            if count[s] > 0:
                sl = np.arange(link[s], link[s] + count[s])
                seen[sl] += 1
            else:
                assert 0 <= link[s] < len(wide)
                sl = subtree(link[s])
            ids = order[sl]
            assert (lo[s] <= prim_lo[ids].min(0)).all() and (hi[s] >= prim_hi[ids].max(0)).all(), (k, s)
            out.append(sl)
        return np.concatenate(out)

    if len(nodes):
        subtree(0)
        assert (seen == 1).all()
    return nodes, order, root


def _tri_boxes(v, f):
    t = v[f]
    return t.min(1), t.max(1)


@pytest.mark.parametrize("acc_name", ["LBVH", "BVH"])
def test_bvh8_structure_bounds_every_primitive(engine, rqm, acc_name):
    v, f = scenes.displaced_icosphere(4, seed=51)
    engine.configure(node_width=rqm.NODE_WIDTH_8)
    acc = engine.build(engine.scene_triangles(v, f), acc_name)
    _check_structure(engine, acc, *_tri_boxes(v, f))


@pytest.mark.parametrize("acc_name", ["LBVH", "BVH"])
@pytest.mark.parametrize("scene", ["icosphere", "terrain"])
def test_bvh8_triangles_equal_binary_and_oracle(engine, oracle, rqm, acc_name, scene):
    if scene == "icosphere":
        v, f = scenes.displaced_icosphere(5, seed=41)
        lo, hi = oracle.bounds3(v)
        rays = scenes.incoherent_rays(lo, hi, 50_000, seed=42)
    else:
        v, f = scenes.heightfield(201, 100, seed=7)
        cam = scenes.pinhole_rays(320, 180, 2, eye=(0.0, -0.6, 1.1), target=(0.0, 0.0, 0.0), fov_deg=40.0, seed=8)
        rays = np.concatenate([cam, scenes.incoherent_rays(*oracle.bounds3(v), 20_000, seed=9)])
    prims, _, _ = oracle.tri_prims(v, f)
    s = engine.scene_triangles(v, f)
    for morton in (rqm.MORTON_SCENE_BOUNDS, rqm.MORTON_SCENE_CUBE):
        engine.configure(node_width=rqm.NODE_WIDTH_2, morton=morton)
        acc2 = engine.build(s, acc_name)
        engine.configure(node_width=rqm.NODE_WIDTH_8)
        acc8 = engine.build(s, acc_name)
        nodes, order, codes, root, _ = engine.export_bvh2(acc8)
        b = bvh2_from_export(oracle, nodes, order, root, codes)
        want = oracle.trace_bvh2(oracle.TRIANGLES, oracle.FAST, oracle.CLOSEST, b, prims, rays)
        got = engine.trace_closest(acc8, rays)
        assert np.array_equal(_u32(got), _u32(want))
        assert np.array_equal(_u32(got), _u32(engine.trace_closest(acc2, rays)))
        occ = oracle.trace_bvh2(oracle.TRIANGLES, oracle.FAST, oracle.ANY, b, prims, rays)
        assert np.array_equal(rqm.unpack_bits(engine.trace_any(acc8, rays), len(rays)), occ)
        # through a ray order (the permuted launch) and the counting walk
        engine.configure(ray_sort=rqm.RAY_SORT_OCTANT_MORTON)
        assert np.array_equal(_u32(engine.trace_closest(acc8, rays)), _u32(want))
        assert np.array_equal(rqm.unpack_bits(engine.trace_any(acc8, rays), len(rays)), occ)
        engine.configure(ray_sort=rqm.RAY_SORT_NONE)
        got_c, cnt = engine.trace_counters(acc8, rays)
        assert np.array_equal(_u32(got_c), _u32(want)) and cnt[0] > 0


def test_bvh8_spheres_reference_scene(engine, oracle, rqm):
    sph = golden("bunny")["spheres"]
    engine.configure(node_width=rqm.NODE_WIDTH_8)
    s = engine.scene_spheres(sph)
    acc = engine.build(s, rqm.LBVH)
    lo, hi = oracle.bounds3(sph[:, :3])
    rays = scenes.incoherent_rays(lo, hi, 30_000, seed=61)
    nodes, order, codes, root, _ = engine.export_bvh2(acc)
    b = bvh2_from_export(oracle, nodes, order, root, codes)
    want = oracle.trace_bvh2(oracle.SPHERES, oracle.FAST, oracle.CLOSEST, b, sph, rays)
    assert np.array_equal(_u32(engine.trace_closest(acc, rays)), _u32(want))
    r = sph[:, 3:4]
    _check_structure(engine, acc, sph[:, :3] - r, sph[:, :3] + r)


@pytest.mark.parametrize("n_tri", [1, 2, 3, 9])
def test_bvh8_tiny_and_flat_scenes(engine, oracle, rqm, n_tri):
    """A root that is one leaf, nodes with fewer than eight children, and a
    flat mesh (zero extent on z: every quantised z plane decodes to 0)."""
    rng = np.random.default_rng(n_tri)
    v = np.concatenate([rng.random((3 * n_tri, 2), dtype=np.float32), np.zeros((3 * n_tri, 1), np.float32)], 1)
    f = np.arange(3 * n_tri, dtype=np.uint32).reshape(-1, 3)
    engine.configure(node_width=rqm.NODE_WIDTH_8)
    s = engine.scene_triangles(v, f)
    acc = engine.build(s, rqm.LBVH)
    brute = engine.build(s, rqm.NONE)
    org = np.concatenate([rng.random((4000, 2), dtype=np.float32), np.full((4000, 1), 1.0, np.float32)], 1)
    d = np.concatenate([rng.normal(0, 0.05, (4000, 2)).astype(np.float32), -np.ones((4000, 1), np.float32)], 1)
    rays = oracle.make_rays(org, d / np.linalg.norm(d, axis=1, keepdims=True))
    want = engine.trace_closest(brute, rays)
    assert (want["prim"] != rqm.MISS).any()
    assert np.array_equal(_u32(engine.trace_closest(acc, rays)), _u32(want))


def test_bvh8_render_and_batched_equal_binary(engine, rqm):
    v, f = scenes.c1_mesh()
    engine.configure(width=320, height=240, aa_samples=1)
    s = engine.scene_triangles(v, f)
    out = {}
    for w in (rqm.NODE_WIDTH_2, rqm.NODE_WIDTH_8):
        engine.configure(node_width=w)
        acc = engine.build(s, rqm.LBVH)
        out[w] = engine.render(acc, rqm.make_view(**scenes.C1_VIEW))
    two, eight = out[rqm.NODE_WIDTH_2], out[rqm.NODE_WIDTH_8]
    assert np.array_equal(two[0], eight[0])
    assert np.array_equal(two[1].view(np.uint32), eight[1].view(np.uint32))
    # many structures in one persistent launch: equal to one query per scene
    meshes = [scenes.displaced_icosphere(3 + k % 2, seed=70 + k) for k in range(6)]
    sc = [engine.scene_triangles(mv, mf) for mv, mf in meshes]
    rays, offs = [], [0]
    for k, (mv, mf) in enumerate(meshes):
        r = scenes.incoherent_rays(mv.min(0), mv.max(0), 3000 + 500 * k, seed=80 + k)
        rays.append(r)
        offs.append(offs[-1] + len(r))
    rays = np.concatenate(rays)
    engine.configure(node_width=rqm.NODE_WIDTH_8)
    accs = engine.build_batched(sc, rqm.LBVH)
    got = engine.trace_batched(accs, rays, offs)
    for k in range(len(meshes)):
        one = engine.trace_closest(accs[k], rays[offs[k]:offs[k + 1]])
        assert np.array_equal(_u32(got[offs[k]:offs[k + 1]]), _u32(one))
