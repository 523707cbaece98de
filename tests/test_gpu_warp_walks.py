"""The persistent-warp walks (each warp takes 32 rays at a time from a
counter) at ray counts that do not fill a warp, a block or the grid, with and
without a ray order, closest and any hit, for the LBVH, the median BVH and the
KD tree: hits bit for bit and occlusion bits equal to the oracle walking the
engine's exported structure.

Triangle path: no reference implementation; parity is against the restated
oracle."""
import numpy as np
import pytest

import scenes
from conftest import bvh2_from_export

pytestmark = pytest.mark.gpu


def _u32(a):
    return np.ascontiguousarray(a).view(np.uint32)


@pytest.fixture(scope="module")
def mesh():
    return scenes.displaced_icosphere(4, seed=91)


@pytest.mark.parametrize("n_rays", [1, 31, 33, 1000, 70_001])
@pytest.mark.parametrize("acc_name", ["LBVH", "BVH", "KDTREE"])
def test_warp_walks_at_odd_ray_counts(engine, oracle, rqm, mesh, acc_name, n_rays):
    v, f = mesh
    prims, _, _ = oracle.tri_prims(v, f)
    lo, hi = oracle.bounds3(v)
    rays = scenes.incoherent_rays(lo, hi, n_rays, seed=92 + n_rays)
    s = engine.scene_triangles(v, f)
    acc = engine.build(s, getattr(rqm, acc_name))
    if acc_name == "KDTREE":
        nodes, pidx, root, _ = engine.export_kd(acc)
        kd = oracle.Kd(nodes, pidx, root)
        want = oracle.trace_kd(oracle.TRIANGLES, oracle.FAST, oracle.CLOSEST, kd, prims, rays)
        occ = oracle.trace_kd(oracle.TRIANGLES, oracle.FAST, oracle.ANY, kd, prims, rays)
    else:
        nodes, order, codes, root, _ = engine.export_bvh2(acc)
        tree = bvh2_from_export(oracle, nodes, order, root, codes)
        want = oracle.trace_bvh2(oracle.TRIANGLES, oracle.FAST, oracle.CLOSEST, tree, prims, rays)
        occ = oracle.trace_bvh2(oracle.TRIANGLES, oracle.FAST, oracle.ANY, tree, prims, rays)
    # none; octant and octant + 3-bit origin (counting sort); octant + origin Morton (radix sort)
    for sort in (rqm.RAY_SORT_NONE, rqm.RAY_SORT_OCTANT, rqm.RAY_SORT_OCTANT_MORTON3, rqm.RAY_SORT_OCTANT_MORTON):
        engine.configure(ray_sort=sort)  # orders only binary-BVH queries of 65,536 rays or more
        assert np.array_equal(_u32(engine.trace_closest(acc, rays)), _u32(want)), (acc_name, n_rays, sort)
        assert np.array_equal(rqm.unpack_bits(engine.trace_any(acc, rays), n_rays), occ), (acc_name, n_rays, sort)
    engine.configure(ray_sort=rqm.RAY_SORT_NONE)
    acc.close()
    s.close()
