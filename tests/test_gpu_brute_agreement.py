"""The FAST walks against the brute-force query (RQ_NONE, every primitive per
ray) on the GPU, at sizes the CPU oracle cannot brute-force: a terrain seen by
the benchmark's camera and by diffuse bounce rays.  Near-coincident hits in two
sibling boxes, hits on shared edges and hits just inside a box's entry face
are where a culling bound that is not the slab test's own (widened) bound
would drop a closer or tied hit; FAST closest hit must equal brute force bit
for bit whatever the structure."""
import numpy as np
import pytest

import scenes

pytestmark = pytest.mark.gpu

EYE, TARGET = (0.0, -0.6, 1.1), (0.0, 0.0, 0.0)


@pytest.mark.parametrize("acc_name", ["LBVH", "BVH"])
def test_fast_closest_hit_equals_brute_force_on_terrain(engine, rqm, acc_name):
    v, f = scenes.heightfield(401, 200, amplitude=0.3, octaves=5, seed=9)  # 159,600 triangles
    s = engine.scene_triangles(v, f)
    cam = scenes.pinhole_rays(640, 360, 4, eye=EYE, target=TARGET, fov_deg=40.0, seed=10)  # 921,600 rays
    brute = engine.build(s, rqm.NONE)
    want_c = engine.trace_closest(brute, cam)
    bounce = scenes.cosine_rays(v, f, cam, want_c, seed=11)
    want_b = engine.trace_closest(brute, bounce)
    engine.configure(morton=rqm.MORTON_SCENE_CUBE)
    acc = engine.build(engine.scene_triangles(v, f), acc_name)
    for rays, want in ((cam, want_c), (bounce, want_b)):
        got = engine.trace_closest(acc, rays)
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def _grid_aligned_axis_rays(v):
    """Rays straight down (direction (0, 0, -1)) from above every vertex of a
    grid, plus rays along x and y through the grid's rows at vertex height:
    every ray has zero direction components and sits exactly on box planes,
    where the fused plane distance fma(b, inv, -o*inv) breaks down."""
    import oracle_py as O
    down = O.make_rays(np.stack([v[:, 0], v[:, 1], np.full(len(v), 2.0, np.float32)], 1).astype(np.float32),
                       np.tile(np.array([[0, 0, -1]], np.float32), (len(v), 1)))
    row = v[:: 7]
    along_x = O.make_rays(np.stack([np.full(len(row), -3.0, np.float32), row[:, 1], row[:, 2]], 1),
                          np.tile(np.array([[1, 0, 0]], np.float32), (len(row), 1)))
    along_y = O.make_rays(np.stack([row[:, 0], np.full(len(row), 3.0, np.float32), row[:, 2]], 1),
                          np.tile(np.array([[0, -1, 0]], np.float32), (len(row), 1)))
    return np.concatenate([down, along_x, along_y])


@pytest.mark.parametrize("acc_name", ["LBVH", "BVH"])
@pytest.mark.parametrize("width", [2, 4])
def test_axis_aligned_rays_on_box_planes_equal_brute_force(engine, rqm, oracle, acc_name, width):
    v, f = scenes.heightfield(81, 41, amplitude=0.3, octaves=5, seed=13)
    rays = _grid_aligned_axis_rays(v)
    s = engine.scene_triangles(v, f)
    brute = engine.build(s, rqm.NONE)
    want = engine.trace_closest(brute, rays)
    want_any = engine.trace_any(brute, rays)
    assert (want["prim"][:len(v)] != rqm.MISS).all()  # the downward rays all land on the terrain
    engine.configure(node_width=width)
    acc = engine.build(s, acc_name)
    got = engine.trace_closest(acc, rays)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    assert np.array_equal(engine.trace_any(acc, rays), want_any)
    prims, _, _ = oracle.tri_prims(v, f)
    assert np.array_equal(want.view(np.uint32),
                          oracle.trace_brute(oracle.TRIANGLES, oracle.FAST, oracle.CLOSEST, prims, rays).view(np.uint32))
