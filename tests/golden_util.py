"""Helpers shared by the fixture generator and the tests: canonical forms of
BVH trees so that the reference's pointer trees and the engine's flattened
BVH2 arrays can be compared node set against node set.

Pre-order form (what oracle/ref_dump.cpp writes for a reference tree):
  bounds[k] = (minx, miny, minz, maxx, maxy, maxz)
  info[k]   = (isleaf, first, count, left, right)   left/right = pre-order ids
  objs[first:first+count] = primitive ids of a leaf
"""
import hashlib

import numpy as np

_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def _splitmix(x):
    x = (x.astype(np.uint64) + np.uint64(0x9E3779B97F4A7C15))
    with np.errstate(over="ignore"):
        x = (x ^ (x >> np.uint64(30))) * _M1
        x = (x ^ (x >> np.uint64(27))) * _M2
    return x ^ (x >> np.uint64(31))


def tree_node_digest(bounds, info, objs):
    """SHA-256 over the sorted multiset of per-node (bounds, |prims|, sum and
    xor of hashed primitive ids).  Independent of node numbering and of the
    order of primitives inside a leaf."""
    bounds = np.asarray(bounds, np.float32).reshape(-1, 6)
    info = np.asarray(info, np.int64).reshape(-1, 5)
    objs = np.asarray(objs, np.int64)
    n = info.shape[0]
    h = _splitmix(objs)
    h2 = _splitmix(objs ^ 0x5DEECE66D)
    cnt = np.zeros(n, np.uint64)
    s = np.zeros(n, np.uint64)
    x = np.zeros(n, np.uint64)
    # pre-order ids: children always follow their parent
    for k in range(n - 1, -1, -1):
        leaf, first, count, l, r = info[k]
        if leaf:
            cnt[k] = count
            with np.errstate(over="ignore"):
                s[k] = np.sum(h[first:first + count], dtype=np.uint64)
            x[k] = np.bitwise_xor.reduce(h2[first:first + count]) if count else 0
        else:
            cnt[k] = cnt[l] + cnt[r]
            with np.errstate(over="ignore"):
                s[k] = s[l] + s[r]
            x[k] = x[l] ^ x[r]
    b = bounds.copy()
    b[b == 0] = 0.0  # -0 -> +0
    rows = np.zeros(n, dtype=[("b", "<u4", 6), ("c", "<u8"), ("s", "<u8"), ("x", "<u8")])
    rows["b"] = b.view(np.uint32)
    rows["c"] = cnt
    rows["s"] = s
    rows["x"] = x
    raw = rows.view(np.uint8).reshape(n, -1)
    order = np.lexsort(raw.T[::-1])
    return np.frombuffer(hashlib.sha256(raw[order].tobytes()).digest(), np.uint8)


def bvh2_to_preorder(nodes16, n_internal, root_bounds, order):
    """Engine/oracle BVH2 arrays -> pre-order form (leaves become nodes)."""
    words = np.asarray(nodes16).reshape(-1, 16)
    f = words.view(np.float32) if words.dtype != np.float32 else words
    iw = f.view(np.int32)
    order = np.asarray(order)
    bounds, info, objs = [], [], []

    def child_box(node, side):
        r = f[node]
        if side == 0:
            return (r[0], r[2], r[8], r[1], r[3], r[9])
        return (r[4], r[6], r[10], r[5], r[7], r[11])

    if n_internal == 0:
        bounds.append(tuple(root_bounds))
        info.append([1, 0, len(order), -1, -1])
        objs.extend(order.tolist())
        return np.array(bounds, np.float32), np.array(info, np.int32), np.array(objs, np.int32)

    # explicit stack of (kind, ref, box, parent_index, side)
    stack = [(0, 0, tuple(root_bounds), -1, -1, 0)]
    while stack:
        is_leaf, ref, box, parent, side, count = stack.pop()
        me = len(info)
        bounds.append(box)
        if parent >= 0:
            info[parent][3 + side] = me
        if is_leaf:
            info.append([1, len(objs), count, -1, -1])
            objs.extend(order[ref:ref + count].tolist())
            continue
        info.append([0, 0, 0, -1, -1])
        kids = []
        for sd in (0, 1):
            c = int(iw[ref, 12 + sd])
            cnt = int(iw[ref, 14 + sd])
            if c < 0:
                kids.append((1, ~c, child_box(ref, sd), me, sd, cnt))
            else:
                kids.append((0, c, child_box(ref, sd), me, sd, 0))
        stack.append(kids[1])
        stack.append(kids[0])
    return np.array(bounds, np.float32), np.array(info, np.int32), np.array(objs, np.int32)
