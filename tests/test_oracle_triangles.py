"""Oracle self-consistency on triangle meshes.  The reference has no working
triangle path (main.cpp:131-215 is never called), so the Moller-Trumbore
closest/any-hit restatement is checked against brute force and against its
own invariants rather than against reference output."""
import numpy as np

import scenes


def _mesh(level=3, seed=11):
    return scenes.displaced_icosphere(level, seed=seed)


def test_lbvh_closest_equals_brute_force(oracle):
    v, f = _mesh()
    prims, aabb, cen = oracle.tri_prims(v, f)
    lo, hi = oracle.bounds3(v)
    codes = oracle.morton_centroids(cen, lo, hi)
    bvh = oracle.build_lbvh(codes, aabb)
    rays = scenes.incoherent_rays(lo, hi, 4000, seed=3)
    hb = oracle.trace_bvh2(oracle.TRIANGLES, oracle.FAST, oracle.CLOSEST, bvh, prims, rays)
    hn = oracle.trace_brute(oracle.TRIANGLES, oracle.FAST, oracle.CLOSEST, prims, rays)
    # FAST closest hit: smallest t, ties to the smallest id, whatever the walk
    assert np.array_equal(hb.view(np.uint32), hn.view(np.uint32))
    ab = oracle.trace_bvh2(oracle.TRIANGLES, oracle.FAST, oracle.ANY, bvh, prims, rays)
    an = oracle.trace_brute(oracle.TRIANGLES, oracle.FAST, oracle.ANY, prims, rays)
    assert np.array_equal(ab, an)


def test_median_and_kd_agree_with_brute_force(oracle):
    v, f = _mesh(3, seed=12)
    prims, aabb, cen = oracle.tri_prims(v, f)
    lo, hi = oracle.bounds3(v)
    rays = scenes.incoherent_rays(lo, hi, 3000, seed=4)
    hn = oracle.trace_brute(oracle.TRIANGLES, oracle.FAST, oracle.CLOSEST, prims, rays)
    m = oracle.build_median(aabb, cen)
    hm = oracle.trace_bvh2(oracle.TRIANGLES, oracle.FAST, oracle.CLOSEST, m, prims, rays)
    assert np.array_equal(hm.view(np.uint32), hn.view(np.uint32))
    kd = oracle.build_kd(aabb)
    hk = oracle.trace_kd(oracle.TRIANGLES, oracle.FAST, oracle.CLOSEST, kd, prims, rays)
    # KD traversal clips at split planes: allow the rare grazing difference
    agree = (hk["t"] == hn["t"]) | ((hk["prim"] == oracle.MISS) & (hn["prim"] == oracle.MISS))
    assert agree.mean() > 0.999


def test_karras_topology_is_a_binary_tree_over_all_leaves(oracle):
    rng = np.random.default_rng(0)
    codes = np.sort(rng.integers(0, 1 << 10, 5000).astype(np.uint32))  # many duplicates
    left, right, parent = oracle.karras(codes)
    n = len(codes)
    seen_leaf = np.zeros(n, int)
    seen_int = np.zeros(n - 1, int)
    for c in np.concatenate([left, right]):
        if c < 0:
            seen_leaf[~c] += 1
        else:
            seen_int[c] += 1
    assert (seen_leaf == 1).all()
    assert seen_int[0] == 0 and (seen_int[1:] == 1).all()
    assert parent[0] == -1


def test_stable_sort_order(oracle):
    rng = np.random.default_rng(1)
    keys = rng.integers(0, 50, 10000).astype(np.uint32)
    k, v = oracle.sort_pairs(keys)
    assert np.array_equal(v, np.argsort(keys, kind="stable"))
    assert np.array_equal(k, keys[v])


def test_lbvh_closest_equals_brute_force_on_terrain(oracle):
    """A flat terrain seen by a camera and by diffuse bounce rays: thin boxes and
    hits just inside a box's entry face, where a box bound that is not the slab
    test's own widened bound drops hits.  The FAST walk must still equal brute
    force bit for bit."""
    v, f = scenes.heightfield(161, 80, amplitude=0.3, octaves=5, seed=5)
    prims, aabb, cen = oracle.tri_prims(v, f)
    lo, hi = oracle.bounds3(v)
    codes = oracle.morton_centroids(cen, lo, hi)
    bvh = oracle.build_lbvh(codes, aabb)
    cam = scenes.pinhole_rays(160, 120, 2, eye=(0.5, -1.2, 1.0), target=(0.5, 0.25, 0.0), seed=6)
    hc = oracle.trace_brute(oracle.TRIANGLES, oracle.FAST, oracle.CLOSEST, prims, cam)
    bounce = scenes.cosine_rays(v, f, cam, hc, seed=7)
    for rays, want in ((cam, hc), (bounce, oracle.trace_brute(oracle.TRIANGLES, oracle.FAST, oracle.CLOSEST,
                                                              prims, bounce))):
        got = oracle.trace_bvh2(oracle.TRIANGLES, oracle.FAST, oracle.CLOSEST, bvh, prims, rays)
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
