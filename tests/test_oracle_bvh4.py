"""Oracle self-consistency of the collapsed 4-wide BVH: the collapse keeps
every leaf exactly once with its binary box, and closest / any-hit queries
through it return what the binary walk and brute force return."""
import numpy as np
import pytest

import scenes


def _mesh(level=3, seed=31):
    return scenes.displaced_icosphere(level, seed=seed)


def _trees(oracle, v, f):
    prims, aabb, cen = oracle.tri_prims(v, f)
    lo, hi = oracle.bounds3(v)
    lbvh = oracle.build_lbvh(oracle.morton_centroids(cen, lo, hi), aabb)
    median = oracle.build_median(aabb, cen)
    return prims, lo, hi, {"LBVH": lbvh, "BVH": median}


def _leaf_boxes_binary(nodes):
    out = {}
    for n in nodes:
        links = n[12:16].view(np.int32)
        for side in range(2):
            if links[side] < 0:
                box = (n[4 * side], n[4 * side + 1], n[4 * side + 2], n[4 * side + 3], n[8 + 2 * side], n[9 + 2 * side])
                out[int(links[side])] = (int(links[2 + side]), box)
    return out


def _leaf_boxes_wide(nodes4):
    out = {}
    for w in nodes4:
        link = w[24:28].view(np.int32)
        cnt = w[28:32].view(np.int32)
        for k in range(4):
            if cnt[k] >= 0 and link[k] < 0:
                assert int(link[k]) not in out
                out[int(link[k])] = (int(cnt[k]), (w[k], w[4 + k], w[8 + k], w[12 + k], w[16 + k], w[20 + k]))
    return out


@pytest.mark.parametrize("tree", ["LBVH", "BVH"])
def test_collapse_keeps_every_leaf(oracle, tree):
    v, f = _mesh()
    _, _, _, trees = _trees(oracle, v, f)
    b = trees[tree]
    n4, k = oracle.collapse_bvh4(b)
    assert 0 < k <= (2 * b.n_internal + 1) // 3 + 1
    wide = _leaf_boxes_wide(n4)
    assert wide == _leaf_boxes_binary(b.nodes)
    # every 4-wide node but the root is referenced once
    links = n4[:, 24:28].view(np.int32)
    cnts = n4[:, 28:32].view(np.int32)
    inner = links[(cnts == 0) & (links >= 0)]
    assert np.array_equal(np.sort(inner), np.arange(1, k))


@pytest.mark.parametrize("tree", ["LBVH", "BVH"])
def test_bvh4_queries_equal_binary_and_brute_force(oracle, tree):
    v, f = _mesh(3, seed=32)
    prims, lo, hi, trees = _trees(oracle, v, f)
    b = trees[tree]
    n4, _ = oracle.collapse_bvh4(b)
    rays = scenes.incoherent_rays(lo, hi, 4000, seed=7)
    h2 = oracle.trace_bvh2(oracle.TRIANGLES, oracle.FAST, oracle.CLOSEST, b, prims, rays)
    h4 = oracle.trace_bvh4(oracle.TRIANGLES, oracle.CLOSEST, n4, b, prims, rays)
    hn = oracle.trace_brute(oracle.TRIANGLES, oracle.FAST, oracle.CLOSEST, prims, rays)
    # smallest t, ties to the smallest id: independent of the walk
    assert np.array_equal(h4.view(np.uint32), h2.view(np.uint32))
    assert np.array_equal(h4.view(np.uint32), hn.view(np.uint32))
    a4 = oracle.trace_bvh4(oracle.TRIANGLES, oracle.ANY, n4, b, prims, rays)
    a2 = oracle.trace_bvh2(oracle.TRIANGLES, oracle.FAST, oracle.ANY, b, prims, rays)
    assert np.array_equal(a4, a2)


def test_bvh4_spheres_and_single_leaf(oracle):
    sph = np.array(scenes_spheres(300), np.float32)
    aabb, cen = oracle.sphere_prims(sph)
    b = oracle.build_median(aabb, cen)
    n4, _ = oracle.collapse_bvh4(b)
    rays = scenes.incoherent_rays(sph[:, :3].min(0) - 1, sph[:, :3].max(0) + 1, 2000, seed=8)
    h4 = oracle.trace_bvh4(oracle.SPHERES, oracle.CLOSEST, n4, b, sph, rays)
    hn = oracle.trace_brute(oracle.SPHERES, oracle.FAST, oracle.CLOSEST, sph, rays)
    assert np.array_equal(h4["t"], hn["t"])
    # one primitive: no internal node, the root is a leaf
    one = sph[:1].copy()
    b1 = oracle.build_median(aabb[:1], cen[:1])
    n41, k1 = oracle.collapse_bvh4(b1)
    assert k1 == 0
    h1 = oracle.trace_bvh4(oracle.SPHERES, oracle.CLOSEST, n41, b1, one, rays)
    assert np.array_equal(h1["t"], oracle.trace_brute(oracle.SPHERES, oracle.FAST, oracle.CLOSEST, one, rays)["t"])


def scenes_spheres(n, seed=9):
    rng = np.random.default_rng(seed)
    c = rng.uniform(-5, 5, (n, 3))
    r = rng.uniform(0.05, 0.4, (n, 1))
    return np.concatenate([c, r], 1)
