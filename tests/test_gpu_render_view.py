"""GPU parity of rq_render (the render step for triangle and sphere scenes)
against the oracle render on the engine's own exported structure: camera
rays, closest hits, Lambert + ambient with shadow rays, mirror bounces and the
pixel resolve.  The oracle walks the same tree with the same operations, so
pixels are compared exactly (the bar is 1/255 per channel); ray counts too.

Triangle path: no reference implementation (the reference's triangle code is
never called); parity is against the restated oracle."""
import numpy as np
import pytest

import scenes
from conftest import bvh2_from_export, golden

pytestmark = pytest.mark.gpu

ICO_VIEW = scenes.C1_VIEW


def oracle_queries(engine, oracle, acc, kind, prims):
    """Oracle closest / any-hit callables walking the engine's exported structure."""
    if acc.type in (3, 0):  # LBVH, BVH
        nodes, order, codes, root, info = engine.export_bvh2(acc)
        b = bvh2_from_export(oracle, nodes, order, root, codes)
        if info.node_width == 4:
            n4 = engine.export_bvh4(acc)
            return (lambda r: oracle.trace_bvh4(kind, oracle.CLOSEST, n4, b, prims, r),
                    lambda r: oracle.trace_bvh4(kind, oracle.ANY, n4, b, prims, r))
        return (lambda r: oracle.trace_bvh2(kind, oracle.FAST, oracle.CLOSEST, b, prims, r),
                lambda r: oracle.trace_bvh2(kind, oracle.FAST, oracle.ANY, b, prims, r))
    if acc.type == 1:  # KDTREE
        nodes, pidx, root, _ = engine.export_kd(acc)
        kd = oracle.Kd(nodes, pidx, root)
        return (lambda r: oracle.trace_kd(kind, oracle.FAST, oracle.CLOSEST, kd, prims, r),
                lambda r: oracle.trace_kd(kind, oracle.FAST, oracle.ANY, kd, prims, r))
    return (lambda r: oracle.trace_brute(kind, oracle.FAST, oracle.CLOSEST, prims, r),
            lambda r: oracle.trace_brute(kind, oracle.FAST, oracle.ANY, prims, r))


def _oracle_view(oracle, engine, kw, window=(0, 0, 0, 0)):
    s = engine.settings
    return oracle.make_view(s.width, s.height, s.aa_samples, window=window, bg=tuple(s.backgroundColor),
                            bias=s.bias, **kw)


def _check(engine, oracle, rqm, acc, kind, prims, kw, window=(0, 0, 0, 0), **geo):
    pix, rgb, cnt = engine.render(acc, rqm.make_view(window=window, **kw))
    cl, an = oracle_queries(engine, oracle, acc, kind, prims)
    opix, orgb, ocnt = oracle.render_view(kind, _oracle_view(oracle, engine, kw, window), cl, an, **geo)
    assert np.array_equal(cnt, ocnt)
    assert np.abs(pix.astype(int) - opix.astype(int)).max() <= 1  # the 1/255 bar
    assert np.array_equal(pix, opix)
    assert np.array_equal(rgb.view(np.uint32), orgb.view(np.uint32))
    return pix, rgb, cnt


@pytest.mark.parametrize("acc_name", ["LBVH", "BVH", "KDTREE"])
def test_c1_icosphere_render_matches_oracle(engine, oracle, rqm, acc_name):
    """C1: 81,920-triangle displaced icosphere, 640x480, 1 spp, Lambert + 1 shadow ray."""
    v, f = scenes.c1_mesh()
    assert len(f) == 81_920
    engine.configure(width=640, height=480, aa_samples=1)
    s = engine.scene_triangles(v, f)
    acc = engine.build(s, acc_name)
    prims, _, _ = oracle.tri_prims(v, f)
    pix, _, cnt = _check(engine, oracle, rqm, acc, oracle.TRIANGLES, prims, ICO_VIEW, verts=v, idx=f)
    assert cnt[0] == 640 * 480 and cnt[1] > 25_000  # lit samples on the mesh
    bg = (pix == 255).all(axis=2).mean()
    assert 0.8 < bg < 0.95  # a unit-sized mesh 3 units away under a 40 degree field of view


@pytest.mark.parametrize("acc_name", ["LBVH", "BVH", "KDTREE"])
def test_c1_crop_none_vs_structures(engine, oracle, rqm, acc_name):
    """C1's 64x48 crop rendered by brute force (NONE) and by each structure:
    each equals its oracle; BVH structures equal NONE pixel for pixel (the
    same closest-hit rule), the KD walk at most at grazing hits."""
    v, f = scenes.c1_mesh()
    engine.configure(width=640, height=480, aa_samples=1)
    s = engine.scene_triangles(v, f)
    prims, _, _ = oracle.tri_prims(v, f)
    window = (300, 200, 64, 48)
    none = engine.build(s, "NONE")
    pn, rn, _ = _check(engine, oracle, rqm, none, oracle.TRIANGLES, prims, ICO_VIEW, window, verts=v, idx=f)
    acc = engine.build(s, acc_name)
    pa, ra, _ = _check(engine, oracle, rqm, acc, oracle.TRIANGLES, prims, ICO_VIEW, window, verts=v, idx=f)
    full, _, _ = engine.render(acc, rqm.make_view(**ICO_VIEW))
    assert np.array_equal(full[200:248, 300:364], pa)  # the window is a crop of the full render
    if acc_name == "KDTREE":  # the KD walk clips at split planes and keeps its own tie order
        assert (np.abs(pn.astype(int) - pa.astype(int)).max(axis=2) <= 1).mean() > 0.99
    else:  # BVH walks pick the same hit as brute force (smallest t, then smallest id)
        assert np.array_equal(pn, pa)


def test_c3_style_mirror_bounces_and_spp(engine, oracle, rqm):
    """C3's shading on a small merged-icosphere scene: 2 spp, shadow ray and two
    mirror bounces per sample."""
    v, f, _ = scenes.merged_icospheres(count=40, target_tris=150_000, seed=5, levels=(3, 4, 5))
    engine.configure(width=160, height=120, aa_samples=2)
    s = engine.scene_triangles(v, f)
    acc = engine.build(s, "LBVH")
    prims, _, _ = oracle.tri_prims(v, f)
    kw = dict(eye=(0.0, -9.0, 3.0), target=(0, 0, 0), up=(0, 0, 1), fov_deg=50.0, light=(4.0, -6.0, 8.0),
              albedo=(0.7, 0.6, 0.5), ambient=0.05, mirror=0.4, bounces=2, seed=21)
    _, _, cnt = _check(engine, oracle, rqm, acc, oracle.TRIANGLES, prims, kw, verts=v, idx=f)
    assert cnt[2] > 0


def test_render_speed_options_are_neutral(engine, oracle, rqm):
    v, f = scenes.heightfield(201, 100, seed=6)
    engine.configure(width=320, height=240, aa_samples=1)
    s = engine.scene_triangles(v, f)
    kw = dict(eye=(0.0, -0.6, 1.1), target=(0, 0, 0), up=(0, 0, 1), fov_deg=40.0, light=(1.5, -1.0, 3.0),
              albedo=(0.6, 0.7, 0.5), ambient=0.1, mirror=0.2, bounces=1, seed=8)
    base, rgb0, c0 = engine.render(engine.build(s, "LBVH"), rqm.make_view(**kw))
    engine.configure(node_width=rqm.NODE_WIDTH_4, ray_sort=rqm.RAY_SORT_OCTANT_MORTON)
    acc4 = engine.build(s, "LBVH")
    prims, _, _ = oracle.tri_prims(v, f)
    pix, rgb, cnt = _check(engine, oracle, rqm, acc4, oracle.TRIANGLES, prims, kw, verts=v, idx=f)
    assert np.array_equal(pix, base) and np.array_equal(cnt, c0)


def test_sphere_scene_view_render(engine, oracle, rqm):
    sph = golden("synth_c")["spheres"]
    engine.configure(width=96, height=72, aa_samples=3)
    s = engine.scene_spheres(sph)
    c = sph[:, :3].mean(0)
    kw = dict(eye=tuple(float(x) for x in c + np.array([0, -200, 50])), target=tuple(float(x) for x in c),
              up=(0, 0, 1), fov_deg=45.0, light=tuple(float(x) for x in c + np.array([30, -40, 60])),
              albedo=(0.9, 0.5, 0.3), ambient=0.1, mirror=0.25, bounces=1, seed=4)
    for name in ("LBVH", "BVH", "KDTREE", "NONE"):
        acc = engine.build(s, name)
        _check(engine, oracle, rqm, acc, oracle.SPHERES, np.ascontiguousarray(sph, np.float32), kw, sph=sph)


def test_render_device_outputs_and_errors(engine, rqm):
    torch = pytest.importorskip("torch")
    v, f = scenes.c1_mesh()
    engine.configure(width=64, height=48, aa_samples=1)
    acc = engine.build(engine.scene_triangles(v, f), "LBVH")
    host, rgb, _ = engine.render(acc, rqm.make_view(**ICO_VIEW))
    dpix = torch.zeros(64 * 48 * 3, dtype=torch.uint8, device="cuda")
    drgb = torch.zeros(64 * 48 * 3, dtype=torch.float32, device="cuda")
    engine.render(acc, rqm.make_view(**ICO_VIEW), dpix, drgb)
    engine.synchronize()
    assert np.array_equal(dpix.cpu().numpy().reshape(48, 64, 3), host)
    assert np.array_equal(drgb.cpu().numpy().reshape(48, 64, 3), rgb)
    with pytest.raises(rqm.RqError):
        engine.render(acc, rqm.make_view(window=(60, 0, 10, 10), **ICO_VIEW))
    bad = dict(ICO_VIEW, fov_deg=180.0)
    with pytest.raises(rqm.RqError):
        engine.render(acc, rqm.make_view(**bad))
