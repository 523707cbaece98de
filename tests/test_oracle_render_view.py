"""Oracle render of a view (the engine's rq_render restated): analytic
checks on a single sphere, window = crop of the full image, and the shading
terms (ambient only in shadow, background on a miss, mirror weights)."""
import numpy as np

import scenes


def _brute(oracle, kind, prims):
    return (lambda r: oracle.trace_brute(kind, oracle.FAST, oracle.CLOSEST, prims, r),
            lambda r: oracle.trace_brute(kind, oracle.FAST, oracle.ANY, prims, r))


def test_single_sphere_centre_pixel(oracle):
    sph = np.array([[0, 0, 0, 1]], np.float32)
    v = oracle.make_view(33, 33, 1, eye=(0, -5, 0), target=(0, 0, 0), up=(0, 0, 1), fov_deg=30,
                         light=(0, -10, 0), albedo=(0.5, 0.25, 1.0), ambient=0.0, seed=3)
    cl, an = _brute(oracle, oracle.SPHERES, sph)
    pix, rgb, cnt = oracle.render_view(oracle.SPHERES, v, cl, an, sph=sph)
    # the centre sample looks straight at the sphere, lit head-on: colour ~ albedo
    c = rgb[16, 16]
    assert np.allclose(c, [0.5, 0.25, 1.0], atol=2e-3)
    # corners miss: background white
    assert (pix[0, 0] == 255).all()
    assert cnt[0] == 33 * 33 and 0 < cnt[1] < 33 * 33 and cnt[2] == 0


def test_window_is_a_crop_of_the_full_image(oracle):
    v, f = scenes.displaced_icosphere(3, seed=5)
    prims, _, _ = oracle.tri_prims(v, f)
    cl, an = _brute(oracle, oracle.TRIANGLES, prims)
    kw = dict(eye=(0.0, -2.5, 0.8), target=(0, 0, 0), up=(0, 0, 1), fov_deg=40, light=(2, -3, 4),
              albedo=(0.8, 0.7, 0.6), ambient=0.1, mirror=0.3, bounces=1, seed=9)
    full = oracle.render_view(oracle.TRIANGLES, oracle.make_view(48, 36, 2, **kw), cl, an, verts=v, idx=f)
    win = oracle.render_view(oracle.TRIANGLES, oracle.make_view(48, 36, 2, window=(10, 7, 16, 12), **kw), cl, an,
                             verts=v, idx=f)
    assert np.array_equal(win[0], full[0][7:19, 10:26])
    assert np.array_equal(win[1], full[1][7:19, 10:26])


def test_shadowed_point_gets_ambient_only(oracle):
    # a big floor triangle pair and a small occluder between it and the light
    verts = np.array([[-5, -5, 0], [5, -5, 0], [5, 5, 0], [-5, 5, 0],
                      [-0.5, -0.5, 1], [0.5, -0.5, 1], [0.5, 0.5, 1], [-0.5, 0.5, 1]], np.float32)
    idx = np.array([[0, 1, 2], [0, 2, 3], [4, 5, 6], [4, 6, 7]], np.uint32)
    prims, _, _ = oracle.tri_prims(verts, idx)
    cl, an = _brute(oracle, oracle.TRIANGLES, prims)
    view = oracle.make_view(1, 1, 1, eye=(0.0, -3.0, 0.3), target=(0, 0, 0), up=(0, 0, 1), fov_deg=1,
                            light=(0, 0, 5), albedo=(1, 1, 1), ambient=0.25, seed=1)
    pix, rgb, cnt = oracle.render_view(oracle.TRIANGLES, view, cl, an, verts=verts, idx=idx)
    assert np.allclose(rgb[0, 0], 0.25, atol=1e-6)  # occluded: ambient only
    view.light[:] = (0, -3, 5)  # light in front of the occluder: lit
    _, rgb2, _ = oracle.render_view(oracle.TRIANGLES, view, cl, an, verts=verts, idx=idx)
    assert (rgb2[0, 0] > 0.5).all()


def test_mirror_weights_sum_to_one(oracle):
    # a mirror floor under an empty sky: every sample ends on the background
    verts = np.array([[-50, -50, 0], [50, -50, 0], [50, 50, 0], [-50, 50, 0]], np.float32)
    idx = np.array([[0, 1, 2], [0, 2, 3]], np.uint32)
    prims, _, _ = oracle.tri_prims(verts, idx)
    cl, an = _brute(oracle, oracle.TRIANGLES, prims)
    view = oracle.make_view(8, 8, 1, eye=(0, -3, 1), target=(0, 0, 0), up=(0, 0, 1), fov_deg=20,
                            light=(0, 0, 10), albedo=(0, 0, 0), ambient=0.0, mirror=0.75, bounces=2,
                            bg=(1.0, 1.0, 1.0), seed=2)
    _, rgb, cnt = oracle.render_view(oracle.TRIANGLES, view, cl, an, verts=verts, idx=idx)
    # black albedo: only the mirrored sky contributes, with weight 0.75
    assert np.allclose(rgb, 0.75, atol=1e-6)
    assert cnt[2] == 64
