import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (os.path.join(ROOT, "tests"), os.path.join(ROOT, "oracle"),
          os.path.join(ROOT, "raytracer-data-structures_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle():
    import oracle_py
    return oracle_py


def golden(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


@pytest.fixture(scope="session")
def bunny():
    return golden("bunny")


@pytest.fixture(scope="session")
def rqm():
    import rq
    return rq


@pytest.fixture()
def engine():
    import rq
    eng = rq.Engine(0)
    yield eng
    eng.close()


def bvh2_from_export(oracle, nodes, order, root, codes=None):
    """Engine-exported BVH2 arrays as an oracle Bvh2."""
    return oracle.Bvh2(np.ascontiguousarray(nodes, np.float32), len(nodes), root, order, codes)


def sphere_surface_colors(n):
    c = np.tile(np.array([0.8, 0.7, 0.0], np.float32), (n, 1))
    c[-1] = 0.0
    return c
