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
    """Four meshes of about 50k triangles (some 8 MB each on the device with
    their LBVHs) under a 24 MB budget, which also holds the wavefront buffers
    and build scratch: the requests cycle through the library, so meshes are
    evicted and rebuilt, and every image stays the same."""
    lib = {20 + k: scenes.wave_heightfield(160, 160 + k, seed=400 + k) for k in range(4)}
    rng = np.random.default_rng(11)
    reqs = []
    for k in range(16):
        az = rng.uniform(0, 6.28)
        view = rqm.make_view(eye=(float(2.2 * np.cos(az)), float(2.2 * np.sin(az)), 1.0), target=(0, 0, 0),
                             up=(0, 0, 1), fov_deg=45.0, light=(1.0, -2.0, 3.0), albedo=(0.7, 0.65, 0.6),
                             ambient=0.1, seed=int(50 + k))
        reqs.append((20 + k % 4, view, 48, 32, 1))
    accs = {mid: engine.build(engine.scene_triangles(v, f), "LBVH") for mid, (v, f) in lib.items()}
    want = [_render_alone(engine, rqm, lib, accs, r) for r in reqs]
    budget = 24 << 20
    for batching in (False, True):
        srv = rqm.Server(batching=batching, hbm_budget=budget)
        for mid, (v, f) in lib.items():
            srv.add_mesh(mid, v, f)
        for req, ref in zip(reqs, want):
            status, pix = srv.wait(srv.submit(req[0], req[1], req[2], req[3], req[4]))
            assert status == 0 and np.array_equal(pix, ref)
        st = srv.stats()
        srv.close()
        assert st.evictions > 0 and st.builds > len(lib)
        assert st.resident_bytes <= budget and st.resident_meshes < len(lib)


def test_arrivals_are_served_while_a_long_step_runs(engine, rqm):
    """Continuous batching: a small request that arrives while a large one is
    on the GPU goes into the other wavefront slot and lands first; its pixels
    are still exactly rq_render's."""
    import time
    v, f = scenes.heightfield(501, 500, seed=21)  # 499,000 triangles
    small_v, small_f = scenes.wave_heightfield(60, 60, seed=22)
    view = rqm.make_view(eye=(0.0, -2.2, 1.2), target=(0, 0, 0), up=(0, 0, 1), fov_deg=45.0,
                         light=(1.0, -2.0, 3.0), albedo=(0.7, 0.65, 0.6), ambient=0.1, seed=5)
    acc = engine.build(engine.scene_triangles(small_v, small_f), "LBVH")
    engine.configure(width=64, height=48, aa_samples=1, backgroundColor=(1.0, 1.0, 1.0))
    want_small, _, _ = engine.render(acc, view)
    srv = rqm.Server(batching=True)
    srv.add_mesh(1, v, f)
    srv.add_mesh(2, small_v, small_f)
    for mid in (1, 2):  # both resident before timing
        srv.wait(srv.submit(mid, view, 32, 32, 1, keep_pixels=False), want_pixels=False)
    big = srv.submit(1, view, 1920, 1080, 16, keep_pixels=False)  # 33M camera rays
    time.sleep(0.001)
    small = srv.submit(2, view, 64, 48, 1)
    status, pix = srv.wait(small)
    t_small = time.perf_counter()
    assert srv.wait(big, want_pixels=False)[0] == 0
    t_big = time.perf_counter()
    srv.close()
    assert status == 0 and np.array_equal(pix, want_small)
    assert t_big - t_small > 0.001  # the large step was still running when the small one landed


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
