"""Parity at the benchmark's full sizes, against the CPU oracle walking the
engine's own exported structures.

  * The LBVH + incoherent traversal workload (998,000-triangle fBm terrain,
    1920x1080x4 primary rays, cosine secondary and shadow rays from the
    primary hits): every ray is traced on the GPU; a seeded 1% of each class
    is traced again by the oracle, hits compared bit for bit (t, primitive,
    u, v) and occlusion bits exactly; the traversal counters (node visits and
    triangle tests, the inputs of the byte model) are compared on the same
    sample.
  * The large scene (about 10.9M triangles of merged displaced icospheres,
    3840x2160x4, shadow rays, two mirror bounces): the full frame is rendered
    on the GPU and a 64x48 crop is rendered by the oracle, pixels and float
    colours compared exactly.
  * The many-scene workload (256 displaced icospheres and fBm heightfields,
    about 140M rays): one batched build and one persistent many-structure
    query; a seeded 1% of every scene's rays is traced by the oracle on that
    scene's exported structure.

Triangle path: no reference implementation (the reference's triangle code is
never called); parity is against the restated oracle.  The closest-hit rule
(smallest t, ties to the smallest primitive id) makes hits independent of
the walk, so bit equality is the bar.
"""
import os
import sys

import numpy as np
import pytest

import scenes
from conftest import ROOT, bvh2_from_export

pytestmark = pytest.mark.gpu

if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def _sample(n, frac, seed):
    rng = np.random.default_rng(seed)
    return np.sort(rng.choice(n, size=max(1, int(n * frac)), replace=False))


@pytest.mark.parametrize("quality", ["LBVH_KARRAS", "LBVH_TREELETS"])
def test_c2_full_workload_one_percent_sample_matches_oracle(engine, oracle, rqm, quality):
    import bench
    verts, idx, primary = bench.make_inputs()
    assert len(idx) == 998_000 and len(primary) == 1920 * 1080 * 4
    # the benchmark's tuned build (cube Morton codes, treelet restructuring) and the Karras tree
    engine.configure(morton=rqm.MORTON_SCENE_CUBE, lbvh_quality=getattr(rqm, quality))
    s = engine.scene_triangles(verts, idx)
    acc = engine.build(s, rqm.LBVH)
    hits_p = engine.trace_closest(acc, primary)
    secondary = scenes.cosine_rays(verts, idx, primary, hits_p, seed=bench.SEED + 2)
    shadow = scenes.shadow_rays(verts, idx, primary, hits_p, bench.LIGHT)
    engine.configure(ray_sort=rqm.RAY_SORT_OCTANT)  # the benchmark's order for secondary rays
    hits_s = engine.trace_closest(acc, secondary)
    engine.configure(ray_sort=rqm.RAY_SORT_NONE)
    occ = rqm.unpack_bits(engine.trace_any(acc, shadow), len(shadow))
    nodes, order, codes, root, _ = engine.export_bvh2(acc)
    tree = bvh2_from_export(oracle, nodes, order, root, codes)
    prims, _, _ = oracle.tri_prims(verts, idx)
    for name, rays, got, query, seed in (("primary", primary, hits_p, oracle.CLOSEST, 1),
                                         ("secondary", secondary, hits_s, oracle.CLOSEST, 2),
                                         ("shadow", shadow, occ, oracle.ANY, 3)):
        sel = _sample(len(rays), 0.01, seed)
        cnt = np.zeros(2, np.uint64)
        want = oracle.trace_bvh2(oracle.TRIANGLES, oracle.FAST, query, tree, prims, rays[sel], counters=cnt)
        if query == oracle.CLOSEST:
            assert np.array_equal(got[sel].view(np.uint32), want.view(np.uint32)), name
        else:
            assert np.array_equal(got[sel], want), name
        _, gcnt = engine.trace_counters(acc, np.ascontiguousarray(rays[sel]), any_hit=query == oracle.ANY)
        assert np.array_equal(gcnt, cnt), (name, gcnt, cnt)
    assert (hits_p["prim"] != rqm.MISS).mean() > 0.99  # the camera looks into the terrain


def test_c3_full_frame_crop_matches_oracle(engine, oracle, rqm):
    v, f, _ = scenes.merged_icospheres()
    assert len(f) > 9_000_000
    engine.configure(width=3840, height=2160, aa_samples=4)
    s = engine.scene_triangles(v, f)
    acc = engine.build(s, rqm.LBVH)
    pix, rgb, cnt = engine.render(acc, rqm.make_view(**scenes.C3_VIEW))
    assert cnt[0] == 3840 * 2160 * 4 and cnt[2] > 0  # mirror rays were traced
    nodes, order, codes, root, _ = engine.export_bvh2(acc)
    tree = bvh2_from_export(oracle, nodes, order, root, codes)
    prims, _, _ = oracle.tri_prims(v, f)
    st = engine.settings
    # the window with the most geometry (chosen on the GPU image) and a fixed one
    cov = (pix != 255).any(axis=2).astype(np.int64)
    cs = np.pad(cov.cumsum(0).cumsum(1), ((1, 0), (1, 0)))
    dense = cs[48:, 64:] - cs[:-48, 64:] - cs[48:, :-64] + cs[:-48, :-64]
    y_best, x_best = np.unravel_index(int(np.argmax(dense[::8, ::8])), dense[::8, ::8].shape)
    for x0, y0 in ((int(x_best) * 8, int(y_best) * 8), (1200, 700)):
        view = oracle.make_view(3840, 2160, 4, window=(x0, y0, 64, 48), bg=tuple(st.backgroundColor),
                                bias=st.bias, **scenes.C3_VIEW)
        opix, orgb, _ = oracle.render_view(
            oracle.TRIANGLES, view,
            lambda r: oracle.trace_bvh2(oracle.TRIANGLES, oracle.FAST, oracle.CLOSEST, tree, prims, r),
            lambda r: oracle.trace_bvh2(oracle.TRIANGLES, oracle.FAST, oracle.ANY, tree, prims, r),
            verts=v, idx=f)
        crop = pix[y0:y0 + 48, x0:x0 + 64]
        assert np.array_equal(crop, opix)
        assert np.array_equal(rgb[y0:y0 + 48, x0:x0 + 64].view(np.uint32), orgb.view(np.uint32))
    assert dense.max() > 64 * 48 // 4  # the densest window shows geometry


def test_c4_batched_one_percent_sample_matches_oracle(engine, oracle, rqm):
    import torch
    import bench
    dev = torch.device("cuda", 0)
    meshes, ray_n, offs = bench.c4_workload(256)
    sc = [engine.scene_triangles(v, f) for v, f in meshes]
    accs = engine.build_batched(sc, rqm.LBVH)
    d_rays = bench.batch_rays(torch, dev, meshes, ray_n.tolist(), bench.SEED + 41)
    n = int(offs[-1])
    d_hits = torch.empty(n * 16, dtype=torch.uint8, device=dev)
    torch.cuda.synchronize()  # the rays come from torch's stream; the engine traces on its own
    engine.trace_batched(accs, d_rays, offs, out=d_hits)
    engine.synchronize()
    rows = d_rays.view(-1, 32)
    hit_rows = d_hits.view(-1, 16)
    checked = wanted = 0
    for k in range(len(meshes)):
        a, b = int(offs[k]), int(offs[k + 1])
        wanted += max(1, (b - a) // 100)
        sel = torch.from_numpy(_sample(b - a, 0.01, 100 + k) + a).to(dev)
        rays = rows[sel].cpu().numpy().reshape(-1).view(rqm.RAY_DTYPE)
        got = hit_rows[sel].cpu().numpy().reshape(-1).view(rqm.HIT_DTYPE)
        nodes, order, codes, root, _ = engine.export_bvh2(accs[k])
        tree = bvh2_from_export(oracle, nodes, order, root, codes)
        prims, _, _ = oracle.tri_prims(*meshes[k])
        want = oracle.trace_bvh2(oracle.TRIANGLES, oracle.FAST, oracle.CLOSEST, tree, prims, rays)
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), k
        checked += len(rays)
    assert checked == wanted and checked > n // 101  # 1% of every scene's rays
    for a in accs:
        a.close()
