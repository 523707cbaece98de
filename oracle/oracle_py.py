"""ctypes front end of the CPU oracle (liboracle.so) — TEST INFRASTRUCTURE ONLY.

Loaded by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg to
check or time the engine; the engine itself never imports it.  Arrays are
numpy; layouts are described in oracle.h.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")

TRIANGLES, SPHERES = 0, 1
FAST, REFERENCE = 0, 1
CLOSEST, ANY = 0, 1
MISS = 0xFFFFFFFF

RAY_DTYPE = np.dtype([("org", "<f4", 3), ("tmin", "<f4"), ("dir", "<f4", 3), ("tmax", "<f4")])
HIT_DTYPE = np.dtype([("t", "<f4"), ("prim", "<u4"), ("u", "<f4"), ("v", "<f4")])

_lib = None


def build():
    subprocess.run(["make", "-s", "-C", HERE, "oracle"], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        _lib = C.CDLL(LIB_PATH)
        _lib.orc_expand_bits.restype = C.c_uint32
        _lib.orc_morton3d.restype = C.c_uint32
        _lib.orc_morton3d.argtypes = [C.c_float, C.c_float, C.c_float]
        _lib.orc_kd_max_depth.restype = C.c_int
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


def make_rays(org, dirs, tmin=0.0, tmax=np.inf):
    org = np.broadcast_to(np.asarray(org, np.float32), np.asarray(dirs).shape)
    r = np.zeros(len(dirs), RAY_DTYPE)
    r["org"] = org
    r["dir"] = dirs
    r["tmin"] = tmin
    r["tmax"] = tmax
    return r


# ------------------------------------------------------------------ Morton

def expand_bits(v):
    return int(lib().orc_expand_bits(C.c_uint32(v)))


def morton3d(x, y, z):
    return int(lib().orc_morton3d(x, y, z))


def morton_spheres_ref(sph):
    sph = _c(sph, np.float32)
    out = np.zeros(len(sph), np.uint32)
    lib().orc_morton_spheres_ref(_p(sph), C.c_uint32(len(sph)), _p(out))
    return out


def morton_centroids(cen, lo, hi, cube=False):
    """cube=True: the engine's RQ_MORTON_SCENE_CUBE (one scale, the largest extent)."""
    cen = _c(cen, np.float32)
    lo = _c(lo, np.float32)
    hi = _c(hi, np.float32)
    out = np.zeros(len(cen), np.uint32)
    f = lib().orc_morton_centroids_cube if cube else lib().orc_morton_centroids
    f(_p(cen), C.c_uint32(len(cen)), _p(lo), _p(hi), _p(out))
    return out


# --------------------------------------------------------------- primitives

def tri_prims(verts, idx):
    verts = _c(verts, np.float32).reshape(-1, 3)
    idx = _c(idx, np.uint32).reshape(-1, 3)
    nt = len(idx)
    prims = np.zeros((nt, 9), np.float32)
    aabb = np.zeros((nt, 6), np.float32)
    cen = np.zeros((nt, 3), np.float32)
    lib().orc_tri_prims(_p(verts), C.c_uint32(len(verts)), _p(idx), C.c_uint32(nt), _p(prims),
                        _p(aabb), _p(cen))
    return prims, aabb, cen


def sphere_prims(sph):
    sph = _c(sph, np.float32).reshape(-1, 4)
    aabb = np.zeros((len(sph), 6), np.float32)
    cen = np.zeros((len(sph), 3), np.float32)
    lib().orc_sphere_prims(_p(sph), C.c_uint32(len(sph)), _p(aabb), _p(cen))
    return aabb, cen


def bounds3(pts):
    pts = _c(pts, np.float32).reshape(-1, 3)
    lo = np.zeros(3, np.float32)
    hi = np.zeros(3, np.float32)
    lib().orc_bounds3(_p(pts), C.c_uint32(len(pts)), C.c_uint32(3), _p(lo), _p(hi))
    return lo, hi


# ----------------------------------------------------------------- builders

def sort_pairs(keys):
    keys = _c(keys, np.uint32)
    ok = np.zeros_like(keys)
    ov = np.zeros_like(keys)
    lib().orc_sort_pairs(_p(keys), C.c_uint32(len(keys)), _p(ok), _p(ov))
    return ok, ov


def karras(sorted_codes):
    k = _c(sorted_codes, np.uint32)
    n = len(k)
    left = np.zeros(max(n - 1, 0), np.int32)
    right = np.zeros(max(n - 1, 0), np.int32)
    parent = np.zeros(max(2 * n - 1, 0), np.int32)
    lib().orc_karras(_p(k), C.c_uint32(n), _p(left), _p(right), _p(parent))
    return left, right, parent


class Bvh2:
    """Flattened BVH2 (layout in oracle.h)."""

    def __init__(self, nodes, n_internal, root_bounds, order, sorted_codes=None):
        self.nodes = nodes
        self.n_internal = int(n_internal)
        self.root_bounds = root_bounds
        self.order = order
        self.sorted_codes = sorted_codes

    @property
    def iwords(self):
        return self.nodes.view(np.int32)


def build_lbvh(codes, aabb):
    codes = _c(codes, np.uint32)
    aabb = _c(aabb, np.float32).reshape(-1, 6)
    n = len(codes)
    nodes = np.zeros((max(n - 1, 0), 16), np.float32)
    order = np.zeros(n, np.uint32)
    sk = np.zeros(n, np.uint32)
    rb = np.zeros(6, np.float32)
    rc = lib().orc_build_lbvh(_p(codes), _p(aabb), C.c_uint32(n), _p(nodes), _p(order), _p(sk), _p(rb))
    if rc:
        raise ValueError("empty scene")
    return Bvh2(nodes, max(n - 1, 0), rb, order, sk)


def treelet_opt(bvh):
    """The engine's RQ_LBVH_TREELETS pass on a copy of an LBVH (one primitive per leaf)."""
    nodes = np.ascontiguousarray(bvh.nodes, np.float32).copy()
    lib().orc_treelet_opt(_p(nodes), C.c_uint32(bvh.n_internal))
    return Bvh2(nodes, bvh.n_internal, bvh.root_bounds, bvh.order, bvh.sorted_codes)


def build_median(aabb, cen, compat=False):
    """compat=False: the engine's deterministic median rule; True: replay of
    the reference's std::partition / std::nth_element sequence."""
    aabb = _c(aabb, np.float32).reshape(-1, 6)
    cen = _c(cen, np.float32).reshape(-1, 3)
    n = len(aabb)
    cap = 2 * n + 16
    while True:
        nodes = np.zeros((max(n - 1, 1), 16), np.float32)
        order = np.zeros(cap, np.uint32)
        ni, ns = C.c_uint32(0), C.c_uint32(0)
        rb = np.zeros(6, np.float32)
        rc = lib().orc_build_median(_p(aabb), _p(cen), C.c_uint32(n), C.c_int(int(compat)), _p(nodes), _p(order),
                                    C.c_uint32(cap), C.byref(ns), C.byref(ni), _p(rb))
        if rc == 1:
            cap = ns.value
            continue
        if rc == 2:
            raise RecursionError("the reference's constructBVHNew would recurse forever on this input")
        if rc:
            raise ValueError("empty scene")
        return Bvh2(nodes[:ni.value], ni.value, rb, order[:ns.value])


class Kd:
    def __init__(self, nodes, prim_idx, root_bounds):
        self.nodes = nodes
        self.prim_idx = prim_idx
        self.root_bounds = root_bounds


def kd_max_depth(n):
    return int(lib().orc_kd_max_depth(C.c_uint32(n)))


def build_kd(aabb, max_depth=-1):
    aabb = _c(aabb, np.float32).reshape(-1, 6)
    n = len(aabb)
    cap_n, cap_i = 4 * n + 64, 16 * n + 64
    while True:
        nodes = np.zeros((cap_n, 3), np.int32)
        pidx = np.zeros(cap_i, np.int32)
        nn, ni = C.c_uint32(0), C.c_uint32(0)
        rb = np.zeros(6, np.float32)
        rc = lib().orc_build_kd(_p(aabb), C.c_uint32(n), C.c_int32(max_depth), _p(nodes), C.c_uint32(cap_n),
                                C.byref(nn), _p(pidx), C.c_uint32(cap_i), C.byref(ni), _p(rb))
        if rc == 1:
            cap_n, cap_i = max(cap_n, nn.value), max(cap_i, ni.value)
            continue
        if rc:
            raise ValueError("empty scene")
        return Kd(nodes[:nn.value], pidx[:ni.value], rb)


# ------------------------------------------------------------------ queries

def _trace_out(n, query):
    hits = np.zeros(n, HIT_DTYPE) if query == CLOSEST else None
    occ = np.zeros(n, np.uint8) if query == ANY else None
    return hits, occ


def trace_bvh2(kind, mode, query, bvh, prims, rays, nthreads=0, counters=None):
    prims = _c(prims, np.float32)
    rays = np.ascontiguousarray(rays, RAY_DTYPE)
    hits, occ = _trace_out(len(rays), query)
    cnt = np.zeros(2, np.uint64)
    nodes = bvh.nodes if bvh.n_internal else np.zeros((1, 16), np.float32)
    lib().orc_trace_bvh2(C.c_int(kind), C.c_int(mode), C.c_int(query), _p(nodes), C.c_uint32(bvh.n_internal),
                         _p(_c(bvh.root_bounds, np.float32)), C.c_uint32(len(bvh.order)),
                         _p(_c(bvh.order, np.uint32)), _p(prims), _p(rays), C.c_uint32(len(rays)),
                         _p(hits), _p(occ), _p(cnt), C.c_int(nthreads))
    if counters is not None:
        counters += cnt
    return hits if query == CLOSEST else occ


def candidates_bvh2(bvh, rays):
    """boxIntersect's candidate lists: (counts per ray, ids concatenated)."""
    rays = np.ascontiguousarray(rays, RAY_DTYPE)
    counts = np.zeros(len(rays), np.uint32)
    L = lib()
    L.orc_candidates_bvh2.restype = C.c_uint64
    args = [_p(_c(bvh.nodes, np.float32) if bvh.n_internal else np.zeros((1, 16), np.float32)),
            C.c_uint32(bvh.n_internal), _p(_c(bvh.root_bounds, np.float32)), C.c_uint32(len(bvh.order)),
            _p(_c(bvh.order, np.uint32)), _p(rays), C.c_uint32(len(rays)), _p(counts)]
    total = L.orc_candidates_bvh2(*args, None, C.c_uint64(0))
    ids = np.zeros(max(int(total), 1), np.uint32)
    L.orc_candidates_bvh2(*args, _p(ids), C.c_uint64(total))
    return counts, ids[:int(total)]


def collapse_bvh4(bvh):
    """Collapsed 4-wide BVH of a Bvh2: (nodes as (n4, 32) float32, n4)."""
    n = max(bvh.n_internal, 1)
    out = np.zeros((n, 32), np.float32)
    if bvh.n_internal == 0:
        return out[:0], 0
    lib().orc_collapse_bvh4.restype = C.c_uint32
    n4 = lib().orc_collapse_bvh4(_p(_c(bvh.nodes, np.float32)), C.c_uint32(bvh.n_internal), _p(out))
    return out[:n4], int(n4)


def trace_bvh4(kind, query, nodes4, bvh, prims, rays, nthreads=0, counters=None):
    prims = _c(prims, np.float32)
    rays = np.ascontiguousarray(rays, RAY_DTYPE)
    hits, occ = _trace_out(len(rays), query)
    cnt = np.zeros(2, np.uint64)
    nodes = _c(nodes4, np.float32) if len(nodes4) else np.zeros((1, 32), np.float32)
    lib().orc_trace_bvh4(C.c_int(kind), C.c_int(query), _p(nodes), C.c_uint32(len(nodes4)),
                         _p(_c(bvh.root_bounds, np.float32)), C.c_uint32(len(bvh.order)),
                         _p(_c(bvh.order, np.uint32)), _p(prims), _p(rays), C.c_uint32(len(rays)),
                         _p(hits), _p(occ), _p(cnt), C.c_int(nthreads))
    if counters is not None:
        counters += cnt
    return hits if query == CLOSEST else occ


def trace_kd(kind, mode, query, kd, prims, rays, nthreads=0, counters=None):
    prims = _c(prims, np.float32)
    rays = np.ascontiguousarray(rays, RAY_DTYPE)
    hits, occ = _trace_out(len(rays), query)
    cnt = np.zeros(2, np.uint64)
    pidx = kd.prim_idx if len(kd.prim_idx) else np.zeros(1, np.int32)
    lib().orc_trace_kd(C.c_int(kind), C.c_int(mode), C.c_int(query), _p(_c(kd.nodes, np.int32)),
                       C.c_uint32(len(kd.nodes)), _p(_c(pidx, np.int32)), _p(_c(kd.root_bounds, np.float32)),
                       _p(prims), _p(rays), C.c_uint32(len(rays)), _p(hits), _p(occ), _p(cnt),
                       C.c_int(nthreads))
    if counters is not None:
        counters += cnt
    return hits if query == CLOSEST else occ


def trace_brute(kind, mode, query, prims, rays, nthreads=0):
    prims = _c(prims, np.float32)
    rays = np.ascontiguousarray(rays, RAY_DTYPE)
    hits, occ = _trace_out(len(rays), query)
    n = len(prims)
    lib().orc_trace_brute(C.c_int(kind), C.c_int(mode), C.c_int(query), C.c_uint32(n), _p(prims), _p(rays),
                          C.c_uint32(len(rays)), _p(hits), _p(occ), C.c_int(nthreads))
    return hits if query == CLOSEST else occ


# ------------------------------------------------------------------- render

def jitter_mt19937(count):
    out = np.zeros(count, np.float64)
    lib().orc_jitter_mt19937(C.c_uint64(count), _p(out))
    return out


def camera_rays_ref(width, height, aa, jitter):
    jitter = _c(jitter, np.float64)
    rays = np.zeros(width * height * aa, RAY_DTYPE)
    lib().orc_camera_rays_ref(C.c_uint32(width), C.c_uint32(height), C.c_uint32(aa), _p(jitter), _p(rays))
    return rays


def shade_ref(sph, surface_rgb, rays, hits=None, kd_any=None):
    sph = _c(sph, np.float32)
    srgb = _c(surface_rgb, np.float32)
    rays = np.ascontiguousarray(rays, RAY_DTYPE)
    n = len(rays)
    rgb = np.zeros((n, 3), np.float32)
    kd_mode = 1 if kd_any is not None else 0
    hits = np.ascontiguousarray(hits, HIT_DTYPE) if hits is not None else np.zeros(n, HIT_DTYPE)
    kd_any = _c(kd_any, np.uint8) if kd_any is not None else np.zeros(n, np.uint8)
    lib().orc_shade_ref(_p(sph), _p(srgb), _p(rays), _p(hits), C.c_uint32(n), C.c_int(kd_mode), _p(kd_any), _p(rgb))
    return rgb


def pixels_ref(rgb, aa=1):
    rgb = _c(rgb, np.float32)
    out = np.zeros(rgb.size, np.uint8)
    lib().orc_pixels_ref(_p(rgb), C.c_uint32(rgb.size // 3), C.c_uint32(aa), _p(out))
    return out


def reference_surface_colors(n_spheres):
    """Surface colours of createScene_new's spheres: every vertex sphere is
    (0.8, 0.7, 0) (main.cpp:689), the trailing ground sphere is black
    (main.cpp:703)."""
    c = np.tile(np.array([0.8, 0.7, 0.0], np.float32), (n_spheres, 1))
    c[-1] = 0.0
    return c


# ---------------------------------------------------------- render of a view

class View(C.Structure):
    _fields_ = [("eye", C.c_float * 3), ("target", C.c_float * 3), ("up", C.c_float * 3),
                ("light", C.c_float * 3), ("albedo", C.c_float * 3), ("bg", C.c_float * 3),
                ("tan_half", C.c_float), ("ambient", C.c_float), ("mirror", C.c_float), ("bias", C.c_float),
                ("width", C.c_uint32), ("height", C.c_uint32), ("spp", C.c_uint32), ("x0", C.c_uint32),
                ("y0", C.c_uint32), ("ww", C.c_uint32), ("wh", C.c_uint32), ("bounces", C.c_uint32),
                ("seed", C.c_uint64)]


def make_view(width, height, spp, eye, target, up, fov_deg, light, albedo, ambient=0.1, mirror=0.0,
              bounces=0, window=(0, 0, 0, 0), seed=1, bg=(1.0, 1.0, 1.0), bias=1e-4):
    """The engine's view parameters (tan of half the fov in double, rounded once)."""
    v = View()
    v.eye[:], v.target[:], v.up[:] = eye, target, up
    v.light[:], v.albedo[:], v.bg[:] = light, albedo, bg
    v.tan_half = float(np.float32(np.tan(np.float64(np.float32(fov_deg)) * 3.141592653589793 / 360.0)))
    v.ambient, v.mirror, v.bias = ambient, mirror, float(np.float32(bias))
    v.width, v.height, v.spp, v.bounces, v.seed = width, height, spp, bounces, seed
    whole = window[2] == 0 or window[3] == 0
    v.x0, v.y0 = (0, 0) if whole else window[:2]
    v.ww, v.wh = (width, height) if whole else window[2:]
    return v


def render_view(kind, view, closest, anyhit, verts=None, idx=None, sph=None):
    """Oracle render: closest(rays) -> hits and anyhit(rays) -> uint8 mask are
    the oracle traversals of the structure under test.  Returns (pixels
    (h, w, 3) uint8, rgb (h, w, 3) float32, ray counts [camera, shadow, mirror])."""
    L = lib()
    nray = view.ww * view.wh * view.spp
    npix = view.ww * view.wh
    rays = np.zeros(nray, RAY_DTYPE)
    shadow = np.zeros(nray, RAY_DTYPE)
    cw = np.zeros((nray, 4), np.float32)
    pend = np.zeros((nray, 4), np.float32)
    cnt = np.zeros(2, np.uint64)
    L.orc_view_rays(C.byref(view), _p(rays), _p(cw))
    vv = _c(verts, np.float32) if verts is not None else np.zeros(3, np.float32)
    ii = _c(idx, np.uint32) if idx is not None else np.zeros(3, np.uint32)
    ss = _c(sph, np.float32) if sph is not None else np.zeros(4, np.float32)
    for depth in range(view.bounces + 1):
        hits = np.ascontiguousarray(closest(rays), HIT_DTYPE)
        L.orc_shade_hits(C.c_int(kind), _p(vv), _p(ii), _p(ss), C.byref(view), C.c_uint64(nray),
                         C.c_int(int(depth == view.bounces)), _p(rays), _p(hits), _p(shadow), _p(cw), _p(pend),
                         _p(cnt))
        occ = np.ascontiguousarray(anyhit(shadow), np.uint8)
        L.orc_shadow_accum(C.c_uint64(nray), _p(occ), _p(pend), _p(cw))
    pix = np.zeros((npix, 3), np.uint8)
    rgb = np.zeros((npix, 3), np.float32)
    L.orc_view_pixels(C.c_uint64(npix), C.c_uint32(view.spp), _p(cw), _p(pix), _p(rgb))
    return (pix.reshape(view.wh, view.ww, 3), rgb.reshape(view.wh, view.ww, 3),
            np.array([nray, cnt[0], cnt[1]], np.uint64))
