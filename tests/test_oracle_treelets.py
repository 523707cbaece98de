"""The oracle's restatement of the engine's LBVH treelet pass (CPU only): the
restructured tree holds every leaf slot and internal node once, every stored
child box is the union of its subtree's primitive boxes, the sum of internal
half areas does not rise, and closest hits and occlusion equal the Karras
tree's on the same rays.  The GPU pass is compared with this restatement bit
for bit in test_gpu_treelets.py."""
import numpy as np
import pytest

import scenes


def _walk(tree, prim_boxes):
    """(slots seen, internal nodes seen, worst box mismatch, sum of internal half areas)."""
    iw = tree.nodes.view(np.int32)
    nodes = tree.nodes
    seen_slots = np.zeros(len(tree.order), np.int64)
    seen_nodes = np.zeros(tree.n_internal, np.int64)
    area = 0.0

    def box_of(code):
        if code < 0:
            return prim_boxes[tree.order[~code]]
        x = code
        l, r = box_of(iw[x, 12]), box_of(iw[x, 13])
        return np.concatenate([np.minimum(l[:3], r[:3]), np.maximum(l[3:], r[3:])])

    stack = [0]
    bad = 0
    while stack:
        x = stack.pop()
        seen_nodes[x] += 1
        b = nodes[x]
        lb = np.array([b[0], b[2], b[8], b[1], b[3], b[9]], np.float32)
        rb = np.array([b[4], b[6], b[10], b[5], b[7], b[11]], np.float32)
        u = np.concatenate([np.minimum(lb[:3], rb[:3]), np.maximum(lb[3:], rb[3:])])
        d = u[3:] - u[:3]
        area += float(d[0] * d[1] + d[1] * d[2] + d[2] * d[0])
        for side, sb in ((0, lb), (1, rb)):
            c = iw[x, 12 + side]
            if not np.array_equal(box_of(c), sb):
                bad += 1
            if c >= 0:
                stack.append(c)
            else:
                seen_slots[~c] += 1
    return seen_slots, seen_nodes, bad, area


@pytest.mark.parametrize("level,seed", [(2, 3), (3, 4)])
def test_treelet_pass_keeps_the_tree_valid_and_the_hits(oracle, level, seed):
    v, f = scenes.displaced_icosphere(level, seed=seed)
    prims, aabb, cen = oracle.tri_prims(v, f)
    lo, hi = oracle.bounds3(v)
    karras = oracle.build_lbvh(oracle.morton_centroids(cen, lo, hi), aabb)
    tree = oracle.treelet_opt(karras)
    assert not np.array_equal(tree.nodes.view(np.int32), karras.nodes.view(np.int32))
    slots, nodes, bad, area = _walk(tree, aabb)
    assert (slots == 1).all() and (nodes == 1).all() and bad == 0
    assert area <= _walk(karras, aabb)[3]
    rays = scenes.incoherent_rays(lo, hi, 3000, seed=seed + 10)
    for q in (oracle.CLOSEST, oracle.ANY):
        a = oracle.trace_bvh2(oracle.TRIANGLES, oracle.FAST, q, karras, prims, rays)
        b = oracle.trace_bvh2(oracle.TRIANGLES, oracle.FAST, q, tree, prims, rays)
        assert np.array_equal(a.view(np.uint8), b.view(np.uint8))


def test_treelet_pass_small_trees(oracle):
    """One to five leaves: nothing to do below three leaves; three and four
    leaves make one treelet at the root."""
    rng = np.random.default_rng(5)
    for n in range(1, 6):
        pts = rng.random((n, 3), dtype=np.float32)
        sph = np.concatenate([pts, np.full((n, 1), 0.05, np.float32)], 1)
        aabb, _ = oracle.sphere_prims(sph)
        karras = oracle.build_lbvh(oracle.morton_centroids(pts, pts.min(0), pts.max(0)), aabb)
        tree = oracle.treelet_opt(karras)
        if karras.n_internal < 2:
            assert np.array_equal(tree.nodes.view(np.int32), karras.nodes.view(np.int32))
            continue
        slots, nodes, bad, area = _walk(tree, aabb)
        assert (slots == 1).all() and (nodes == 1).all() and bad == 0
