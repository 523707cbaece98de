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
