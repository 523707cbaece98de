"""Shape of the LBVH test inputs (oracle only).  The GPU refit splits an
LBVH into treelets (maximal subtrees of at most 2048 leaves, one block each)
and top nodes (more than 2048 leaves), which one block finishes when there
are at most 2048 of them; otherwise the treelet roots climb to the root with
device-scope counts.  The 6M-point cloud must exceed that cap and the
benchmark terrain must stay under it, so that the GPU tests cover both."""
import numpy as np

import scenes

SPAN, CAP = 2048, 2048


def leaf_spans(bvh):
    """Leaves under each internal node (pointer jumping to the leftmost and
    rightmost leaf; LBVH leaves hold one slot each)."""
    links = bvh.nodes.view(np.int32)[:, 12:14].astype(np.int64)
    lft, rgt = links[:, 0].copy(), links[:, 1].copy()
    for _ in range(128):
        ml, mr = lft >= 0, rgt >= 0
        if not (ml.any() or mr.any()):
            break
        lft[ml] = links[lft[ml], 0]
        rgt[mr] = links[rgt[mr], 1]
    return (~rgt) - (~lft) + 1


def cloud(n, seed=7):
    pts = np.random.default_rng(seed).random((n, 3), dtype=np.float32)
    return pts


def test_spans_match_a_recursive_count(oracle):
    pts = scenes.chain_clusters(4, 8, 30)
    aabb = np.concatenate([pts - 1e-3, pts + 1e-3], 1).astype(np.float32)
    bvh = oracle.build_lbvh(oracle.morton_centroids(pts, pts.min(0), pts.max(0)), aabb)
    links = bvh.nodes.view(np.int32)[:, 12:16]

    def count(i):
        return sum(count(int(c)) if c >= 0 else int(links[i, 2 + k]) for k, c in enumerate(links[i, :2]))

    s = leaf_spans(bvh)
    assert s[0] == len(pts)
    assert all(s[i] == count(i) for i in range(0, bvh.n_internal, 37))


def test_large_cloud_exceeds_the_top_block(oracle):
    pts = cloud(6_000_000)
    aabb = np.concatenate([pts - 1e-4, pts + 1e-4], 1).astype(np.float32)
    bvh = oracle.build_lbvh(oracle.morton_centroids(pts, pts.min(0), pts.max(0)), aabb)
    assert int((leaf_spans(bvh) > SPAN).sum()) > CAP


def test_terrain_fits_the_top_block(oracle):
    v, f = scenes.heightfield(1001, 500, seed=2)
    _, aabb, cen = oracle.tri_prims(v, f)
    lo, hi = oracle.bounds3(v)
    bvh = oracle.build_lbvh(oracle.morton_centroids(cen, lo, hi, cube=True), aabb)
    top = int((leaf_spans(bvh) > SPAN).sum())
    assert 0 < top <= CAP
