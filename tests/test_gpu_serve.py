"""The serving loop (rq_server_*): a request's pixels are identical whether it
is served alone, among others in a continuous batch, or rendered by
rq_render with the same view; LRU residency under a small HBM budget evicts
and rebuilds without changing any pixel; admission errors are reported per
request; statistics add up."""
import numpy as np
import pytest

import scenes

pytestmark = pytest.mark.gpu


def _library(seed=100, count=5):
    out = {}
    for k in range(count):
        n = 40 + 30 * k
        v, f = scenes.wave_heightfield(n, n + 7, seed=seed + k)
        out[10 + k] = (v, f)
    return out


def _requests(rqm, lib, count, seed):
    rng = np.random.default_rng(seed)
    ids = sorted(lib)
    reqs = []
    for k in range(count):
        mid = ids[int(rng.integers(len(ids)))]
        w, h = [(64, 48), (96, 72), (160, 90), (33, 17)][int(rng.integers(4))]
        spp = int(rng.choice([1, 2, 4]))
        az = rng.uniform(0, 6.28)
        eye = (float(2.2 * np.cos(az)), float(2.2 * np.sin(az)), float(rng.uniform(0.6, 1.5)))
        view = rqm.make_view(eye=eye, target=(0, 0, 0), up=(0, 0, 1), fov_deg=float(rng.uniform(30, 60)),
                             light=(1.0, -2.0, 3.0), albedo=(0.7, 0.65, 0.6), ambient=0.1, seed=int(seed + k))
        reqs.append((mid, view, w, h, spp))
    return reqs


def _render_alone(engine, rqm, lib, accs, req):
    mid, view, w, h, spp = req
    engine.configure(width=w, height=h, aa_samples=spp, backgroundColor=(1.0, 1.0, 1.0))
    pix, _, _ = engine.render(accs[mid], view)
    return pix


def test_served_pixels_equal_alone_and_rq_render(engine, rqm):
    lib = _library()
    reqs = _requests(rqm, lib, 24, seed=7)
    accs = {mid: engine.build(engine.scene_triangles(v, f), "LBVH") for mid, (v, f) in lib.items()}
    want = [_render_alone(engine, rqm, lib, accs, r) for r in reqs]
    # mixed: everything submitted at once, continuous batching
    srv = rqm.Server(batching=True)
    for mid, (v, f) in lib.items():
        srv.add_mesh(mid, v, f)
    tickets = [srv.submit(m, vw, w, h, spp) for m, vw, w, h, spp in reqs]
    got = [srv.wait(t) for t in tickets]
    st = srv.stats()
    srv.close()
    for (status, pix), ref in zip(got, want):
        assert status == 0
        assert np.array_equal(pix, ref)
    assert st.completed == 24 and st.rejected == 0
    assert st.batches < 24  # requests shared batches
    assert st.latency_ms_p50 <= st.latency_ms_p99 <= st.latency_ms_max
    # alone: one request per step
    srv = rqm.Server(batching=False)
    for mid, (v, f) in lib.items():
        srv.add_mesh(mid, v, f)
    for (m, vw, w, h, spp), ref in zip(reqs[:6], want[:6]):
        status, pix = srv.wait(srv.submit(m, vw, w, h, spp))
        assert status == 0 and np.array_equal(pix, ref)
    assert srv.stats().batches == 6
    srv.close()


def test_lru_residency_under_a_small_budget(engine, rqm):
    lib = _library(seed=200, count=4)
    reqs = _requests(rqm, lib, 16, seed=9)
    accs = {mid: engine.build(engine.scene_triangles(v, f), "LBVH") for mid, (v, f) in lib.items()}
    want = [_render_alone(engine, rqm, lib, accs, r) for r in reqs]
    biggest = max(len(f) for _, f in lib.values())
    budget = int(1.2 * biggest * 140)  # the largest mesh fits, the whole library does not
    srv = rqm.Server(batching=False, hbm_budget=budget)
    for mid, (v, f) in lib.items():
        srv.add_mesh(mid, v, f)
    for req, ref in zip(reqs, want):
        status, pix = srv.wait(srv.submit(req[0], req[1], req[2], req[3], req[4]))
        assert status == 0 and np.array_equal(pix, ref)
    st = srv.stats()
    srv.close()
    assert st.evictions > 0 and st.builds > len(lib)
    assert st.resident_bytes <= budget and st.resident_meshes < len(lib)


def test_admission_errors(rqm):
    lib = _library(seed=300, count=2)
    v, f = lib[10]
    srv = rqm.Server(hbm_budget=len(f) * 50, max_batch_rays=100_000)  # too small for any mesh
    srv.add_mesh(10, v, f)
    view = rqm.make_view(eye=(2, 0, 1), target=(0, 0, 0), up=(0, 0, 1))
    status, _ = srv.wait(srv.submit(10, view, 32, 32, 1))
    assert status == 3  # OUT_OF_MEMORY: the mesh cannot fit the budget
    status, _ = srv.wait(srv.submit(99, view, 32, 32, 1))
    assert status == 1  # unknown mesh
    with pytest.raises(rqm.RqError):
        srv.submit(10, view, 1000, 1000, 1)  # over max_batch_rays
    with pytest.raises(rqm.RqError):
        srv.add_mesh(10, v, f)  # id taken
    with pytest.raises(rqm.RqError):
        srv.add_mesh(11, v, np.array([[0, 1, len(v)]], np.uint32))  # index out of range
    st = srv.stats()
    assert st.rejected == 2 and st.completed == 0
    srv.close()
