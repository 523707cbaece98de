"""CPU-only checks of the boundary: the C-ABI library builds, loads and
exports every function include/rq.h declares; without a GPU it reports
NO_DEVICE instead of crashing.  No compute calls."""
import os
import re

import numpy as np
import pytest

from conftest import ROOT


def _declared():
    with open(os.path.join(ROOT, "include", "rq.h")) as f:
        text = f.read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(rq_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_boundary():
    names = _declared()
    for required in ("rq_create", "rq_destroy", "rq_scene_create_triangles", "rq_scene_create_spheres",
                     "rq_build", "rq_trace_closest", "rq_trace_any", "rq_morton_codes", "rq_sort_pairs",
                     "rq_render_reference", "rq_last_error", "rq_accel_export_bvh2", "rq_accel_export_kd"):
        assert required in names


def test_library_exports_every_declared_symbol():
    import rq
    lib = rq.load()
    missing = [n for n in _declared() if not hasattr(lib, n)]
    assert not missing, missing


def test_settings_defaults_match_reference_settings_h():
    import rq
    s = rq.default_settings()
    # settings.h:9-16
    assert (s.width, s.height, s.fov, s.aa_samples) == (640, 480, 90.0, 1)
    assert tuple(s.backgroundColor) == (1.0, 1.0, 1.0)
    assert abs(s.bias - 1e-4) < 1e-9
    assert s.dataStructure == rq.BVH and s.sceneModel == 2  # BVH, BUNNY
    # AccType order, accelerators.h:21
    assert (rq.BVH, rq.KDTREE, rq.UNIFORM_GRID, rq.LBVH, rq.NONE) == (0, 1, 2, 3, 4)


def test_no_device_is_an_error_not_a_crash():
    import torch
    import rq
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(rq.RqError) as e:
        rq.Engine()
    assert e.value.status == 8  # NO_DEVICE


def test_generators_sizes():
    import scenes
    v, f = scenes.icosphere(6)
    assert (len(v), len(f)) == (40962, 81920)
    v, f = scenes.heightfield(1001, 500)
    assert (len(v), len(f)) == (500500, 998000)
    assert f.max() < len(v)
    v, f = scenes.displaced_icosphere(3, seed=9)
    assert v.min() >= 0 and v.max() <= 1.0 + 1e-6
