"""Python binding of the engine's C ABI (include/rq.h) over ctypes.

Thin by design: every call goes straight to librq.so.  Arrays are numpy
(host) or anything exposing a CUDA device pointer (`data_ptr()` of a torch
tensor, or an int); device buffers are passed with RQ_DEVICE_POINTERS.
Failures raise RqError carrying the engine's status and message.  There is
no CPU path: without librq.so or a GPU the calls fail.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "librq.so")

BVH, KDTREE, UNIFORM_GRID, LBVH, NONE = 0, 1, 2, 3, 4
ACC_NAMES = {"BVH": BVH, "KDTREE": KDTREE, "UNIFORM_GRID": UNIFORM_GRID, "LBVH": LBVH, "NONE": NONE}
TRAVERSAL_FAST, TRAVERSAL_REFERENCE = 0, 1
RAY_SORT_NONE, RAY_SORT_OCTANT_MORTON, RAY_SORT_ORIGIN_DIRECTION, RAY_SORT_DIRECTION_ORIGIN, RAY_SORT_OCTANT_MORTON12 = \
    0, 1, 2, 3, 4
RAY_SORT_OCTANT, RAY_SORT_OCTANT_MORTON3 = 5, 6
NODE_WIDTH_2, NODE_WIDTH_4, NODE_WIDTH_8 = 0, 4, 8
SCHEDULING_THREAD_PER_RAY, SCHEDULING_LANE_REFILL, SCHEDULING_SPECULATIVE, SCHEDULING_WARP_PACKET = 0, 1, 2, 3
SCHEDULING_SHARED_TOP = 4
MORTON_SCENE_BOUNDS, MORTON_REFERENCE, MORTON_SCENE_CUBE = 0, 1, 2
LBVH_KARRAS, LBVH_TREELETS = 0, 1
# SceneModel (settings.h:4)
IGEA, ARMADILLO, BUNNY_MODEL, BUNNIES, TEST, GRASS, BUDDHA, CITY = range(8)
DEVICE_POINTERS = 0x1
MISS = 0xFFFFFFFF

SUCCESS = 0
STATUS_NAMES = {0: "SUCCESS", 1: "INVALID_ARGUMENT", 2: "UNSUPPORTED", 3: "OUT_OF_MEMORY", 4: "CUDA",
                5: "STACK_OVERFLOW", 6: "TIMEOUT", 7: "EMPTY_SCENE", 8: "NO_DEVICE"}

RAY_DTYPE = np.dtype([("org", "<f4", 3), ("tmin", "<f4"), ("dir", "<f4", 3), ("tmax", "<f4")])
HIT_DTYPE = np.dtype([("t", "<f4"), ("prim", "<u4"), ("u", "<f4"), ("v", "<f4")])


class Settings(C.Structure):
    """rq_settings_t: settings.h's fields in order, then engine fields."""
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("fov", C.c_float),
                ("backgroundColor", C.c_float * 3), ("bias", C.c_float), ("aa_samples", C.c_uint32),
                ("dataStructure", C.c_int32), ("sceneModel", C.c_int32), ("traversal", C.c_int32),
                ("morton", C.c_int32), ("kd_max_depth", C.c_int32), ("ray_sort", C.c_int32),
                ("node_width", C.c_int32), ("scheduling", C.c_int32), ("lbvh_quality", C.c_int32),
                ("reserved", C.c_int32 * 1)]


class AccelInfo(C.Structure):
    _fields_ = [("type", C.c_int32), ("prim_kind", C.c_int32), ("n_prims", C.c_uint32),
                ("n_nodes", C.c_uint32), ("n_slots", C.c_uint32), ("max_depth", C.c_uint32),
                ("root_bounds", C.c_float * 6), ("device_bytes", C.c_uint64),
                ("node_width", C.c_uint32), ("n_wide_nodes", C.c_uint32)]


class View(C.Structure):
    """rq_view_t: a pinhole view with one point light (rq_render)."""
    _fields_ = [("eye", C.c_float * 3), ("target", C.c_float * 3), ("up", C.c_float * 3),
                ("fov_deg", C.c_float), ("light", C.c_float * 3), ("albedo", C.c_float * 3),
                ("ambient", C.c_float), ("mirror", C.c_float), ("bounces", C.c_uint32),
                ("window", C.c_uint32 * 4), ("seed", C.c_uint64)]


def make_view(eye, target, up=(0, 0, 1), fov_deg=40.0, light=(0, 0, 10), albedo=(0.8, 0.8, 0.8),
              ambient=0.1, mirror=0.0, bounces=0, window=(0, 0, 0, 0), seed=1):
    v = View()
    v.eye[:], v.target[:], v.up[:] = eye, target, up
    v.fov_deg, v.light[:], v.albedo[:] = fov_deg, light, albedo
    v.ambient, v.mirror, v.bounces, v.seed = ambient, mirror, bounces, seed
    v.window[:] = window
    return v


class Query(C.Structure):
    _fields_ = [("rays", C.c_void_p), ("n", C.c_uint32), ("any", C.c_int32), ("out", C.c_void_p),
                ("ray_sort", C.c_int32), ("scheduling", C.c_int32)]


class PlanInfo(C.Structure):
    _fields_ = [("block_threads", C.c_uint32), ("stack_entries", C.c_uint32), ("graph_kernels", C.c_uint32),
                ("n_rays", C.c_uint32), ("rebuilds", C.c_uint32), ("shape_ms", C.c_float * 4),
                ("ray_order", C.c_uint32), ("ordered_ms", C.c_float * 4), ("node_width", C.c_uint32),
                ("width_ms", C.c_float * 3)]


class Plan:
    """rq_plan_t: a captured [rebuild +] many-structure query, replayed as one CUDA graph."""

    def __init__(self, engine, handle, keep):
        self.engine, self.handle, self._keep = engine, handle, keep

    def launch(self):
        self.engine._check(load().rq_plan_launch(self.handle))

    def info(self):
        inf = PlanInfo()
        self.engine._check(load().rq_plan_get_info(self.handle, C.byref(inf)))
        return inf

    def close(self):
        if self.handle:
            load().rq_plan_destroy(self.handle)
            self.handle = None


class ServerConfig(C.Structure):
    _fields_ = [("device", C.c_int32), ("batching", C.c_int32), ("hbm_budget", C.c_uint64),
                ("max_batch_rays", C.c_uint32), ("max_batch_requests", C.c_uint32), ("step_rays", C.c_uint32)]


class Request(C.Structure):
    _fields_ = [("mesh_id", C.c_uint32), ("width", C.c_uint32), ("height", C.c_uint32), ("spp", C.c_uint32),
                ("view", View), ("background", C.c_float * 3), ("keep_pixels", C.c_uint32)]


class ServerStats(C.Structure):
    _fields_ = [("submitted", C.c_uint64), ("completed", C.c_uint64), ("rejected", C.c_uint64),
                ("batches", C.c_uint64), ("builds", C.c_uint64), ("evictions", C.c_uint64),
                ("camera_rays", C.c_uint64), ("shadow_rays", C.c_uint64), ("resident_bytes", C.c_uint64),
                ("resident_meshes", C.c_uint64), ("busy_s", C.c_double), ("latency_ms_p50", C.c_double),
                ("latency_ms_p99", C.c_double), ("latency_ms_mean", C.c_double), ("latency_ms_max", C.c_double)]


class Server:
    """rq_server_t: the serving loop (admission, HBM budget with LRU residency,
    continuous batching, latency statistics) on its own worker thread."""

    def __init__(self, device=0, batching=True, hbm_budget=0, max_batch_rays=0, max_batch_requests=0, step_rays=0):
        lib = load()
        cfg = ServerConfig(device, int(batching), hbm_budget, max_batch_rays, max_batch_requests, step_rays)
        self.handle = C.c_void_p()
        self._check(lib.rq_server_create(C.byref(cfg), C.byref(self.handle)))
        self._sizes = {}

    @staticmethod
    def _check(st):
        if st != SUCCESS:
            raise RqError(st, STATUS_NAMES.get(st, str(st)))

    def add_mesh(self, mesh_id, verts, idx):
        verts = np.ascontiguousarray(verts, np.float32)
        idx = np.ascontiguousarray(idx, np.uint32)
        self._check(load().rq_server_add_mesh(self.handle, mesh_id, verts.ctypes.data, verts.size // 3,
                                              idx.ctypes.data, idx.size // 3))

    def submit(self, mesh_id, view, width, height, spp=1, background=(1.0, 1.0, 1.0), keep_pixels=True):
        r = Request()
        r.mesh_id, r.width, r.height, r.spp = mesh_id, width, height, spp
        r.view = view
        r.background[:] = background
        r.keep_pixels = int(keep_pixels)
        t = C.c_uint64()
        self._check(load().rq_server_submit(self.handle, C.byref(r), C.byref(t)))
        self._sizes[t.value] = (height, width)
        return t.value

    def wait(self, ticket, timeout_s=-1.0, want_pixels=True):
        """(status, pixels (h, w, 3) or None)."""
        h, w = self._sizes.pop(ticket, (0, 0))
        pix = np.zeros((h, w, 3), np.uint8) if want_pixels and h else None
        st = load().rq_server_wait(self.handle, C.c_uint64(ticket), pix.ctypes.data if pix is not None else None,
                                   C.c_double(timeout_s))
        return st, pix

    def drain(self, timeout_s=-1.0):
        self._check(load().rq_server_drain(self.handle, C.c_double(timeout_s)))

    def stats(self):
        s = ServerStats()
        self._check(load().rq_server_get_stats(self.handle, C.byref(s)))
        return s

    def reset_stats(self):
        self._check(load().rq_server_reset_stats(self.handle))

    def close(self):
        if self.handle:
            load().rq_server_destroy(self.handle)
            self.handle = None


class RqError(RuntimeError):
    def __init__(self, status, message):
        self.status = status
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")


_lib = None


def load(build_if_missing=True):
    """Load librq.so, compiling it from csrc/ first when it is absent."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        if not build_if_missing:
            raise ImportError(f"{LIB_PATH} is missing: build the engine first")
        import importlib.util
        spec = importlib.util.spec_from_file_location("rq_build", os.path.join(HERE, "build.py"))
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        mod.build()
    lib = C.CDLL(LIB_PATH)
    vp, u32, i32 = C.c_void_p, C.c_uint32, C.c_int32
    sig = {
        "rq_settings_default": (None, [vp]),
        "rq_create": (i32, [vp, C.c_int, vp]),
        "rq_destroy": (i32, [vp]),
        "rq_get_settings": (i32, [vp, vp]),
        "rq_set_settings": (i32, [vp, vp]),
        "rq_set_stream": (i32, [vp, vp]),
        "rq_synchronize": (i32, [vp]),
        "rq_last_error": (C.c_char_p, [vp]),
        "rq_status_string": (C.c_char_p, [i32]),
        "rq_scene_create_triangles": (i32, [vp, vp, u32, vp, u32, u32, vp]),
        "rq_scene_create_spheres": (i32, [vp, vp, u32, u32, vp]),
        "rq_scene_update": (i32, [vp, vp, vp, vp, u32]),
        "rq_scene_destroy": (i32, [vp]),
        "rq_build": (i32, [vp, vp, i32, vp]),
        "rq_accel_rebuild": (i32, [vp, vp]),
        "rq_accel_destroy": (i32, [vp]),
        "rq_accel_get_info": (i32, [vp, vp]),
        "rq_accel_export_bvh2": (i32, [vp, vp, vp, vp, vp]),
        "rq_accel_export_kd": (i32, [vp, vp, vp, vp]),
        "rq_accel_export_bvh4": (i32, [vp, vp, vp, vp]),
        "rq_accel_import_bvh2": (i32, [vp, vp, vp, u32, vp, u32, vp, vp]),
        "rq_set_debug": (i32, [vp, vp]),
        "rq_trace_closest": (i32, [vp, vp, vp, u32, vp, u32]),
        "rq_trace_any": (i32, [vp, vp, vp, u32, vp, u32]),
        "rq_morton_codes": (i32, [vp, vp, vp, u32]),
        "rq_sort_pairs": (i32, [vp, vp, vp, u32, u32, u32]),
        "rq_render_reference": (i32, [vp, vp, vp, vp, vp, vp, vp]),
        "rq_trace_counters": (i32, [vp, vp, vp, u32, i32, vp, vp, u32]),
        "rq_kernel_launch_count": (C.c_uint64, []),
        "rq_sort_pairs_noalloc": (i32, [vp, vp, u32, u32, vp]),
        "rq_render": (i32, [vp, vp, vp, vp, vp, vp, u32]),
        "rq_build_batched": (i32, [vp, vp, u32, i32, vp]),
        "rq_accel_rebuild_batched": (i32, [vp, vp, u32]),
        "rq_trace_batched": (i32, [vp, vp, u32, vp, vp, i32, vp, u32]),
        "rq_trace_queries": (i32, [vp, vp, vp, u32]),
        "rq_trace_candidates": (i32, [vp, vp, vp, u32, vp, vp, C.c_uint64, vp, u32]),
        "rq_plan_create": (i32, [vp, vp, u32, i32, vp, vp, i32, vp, vp]),
        "rq_plan_launch": (i32, [vp]),
        "rq_plan_get_info": (i32, [vp, vp]),
        "rq_plan_destroy": (i32, [vp]),
        "rq_obj_load": (i32, [C.c_char_p, vp, vp, vp, vp]),
        "rq_obj_save": (i32, [C.c_char_p, vp, u32, vp, u32]),
        "rq_free": (None, [vp]),
        "rq_model_path": (i32, [C.c_char_p, i32, vp, u32]),
        "rq_reference_spheres": (i32, [C.c_char_p, i32, vp, vp]),
        "rq_server_create": (i32, [vp, vp]),
        "rq_server_add_mesh": (i32, [vp, u32, vp, u32, vp, u32]),
        "rq_server_submit": (i32, [vp, vp, vp]),
        "rq_server_wait": (i32, [vp, C.c_uint64, vp, C.c_double]),
        "rq_server_drain": (i32, [vp, C.c_double]),
        "rq_server_get_stats": (i32, [vp, vp]),
        "rq_server_reset_stats": (i32, [vp]),
        "rq_server_last_error": (C.c_char_p, [vp]),
        "rq_server_destroy": (i32, [vp]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def _ptr(a):
    """Host numpy array -> (pointer, 0); device buffer -> (pointer, DEVICE_POINTERS)."""
    if a is None:
        return None, 0
    if isinstance(a, np.ndarray):
        return a.ctypes.data, 0
    if hasattr(a, "data_ptr"):
        return a.data_ptr(), DEVICE_POINTERS
    return int(a), DEVICE_POINTERS


def default_settings(**kw):
    s = Settings()
    load().rq_settings_default(C.byref(s))
    for k, v in kw.items():
        setattr(s, k, v)
    return s


class Scene:
    def __init__(self, engine, handle, kind, n):
        self.engine, self.handle, self.kind, self.n = engine, handle, kind, n

    def update(self, data, idx=None):
        p, fl = _ptr(data)
        pi, _ = _ptr(idx)
        self.engine._check(load().rq_scene_update(self.engine.ctx, self.handle, p, pi, fl))

    def close(self):
        if self.handle:
            load().rq_scene_destroy(self.handle)
            self.handle = None


class Accel:
    def __init__(self, engine, handle, scene, acc_type):
        self.engine, self.handle, self.scene, self.type = engine, handle, scene, acc_type

    def info(self):
        inf = AccelInfo()
        self.engine._check(load().rq_accel_get_info(self.handle, C.byref(inf)))
        return inf

    def rebuild(self):
        self.engine._check(load().rq_accel_rebuild(self.engine.ctx, self.handle))

    def close(self):
        if self.handle:
            load().rq_accel_destroy(self.handle)
            self.handle = None


class Engine:
    """One context on one device (rq_create)."""

    def __init__(self, device=0, settings=None):
        lib = load()
        self.ctx = C.c_void_p()
        st = lib.rq_create(C.byref(settings) if settings is not None else None, device, C.byref(self.ctx))
        if st != SUCCESS:
            raise RqError(st, lib.rq_status_string(st).decode())

    # -- plumbing
    def _check(self, st):
        if st != SUCCESS:
            raise RqError(st, (load().rq_last_error(self.ctx) or b"").decode())

    def close(self):
        if self.ctx:
            load().rq_destroy(self.ctx)
            self.ctx = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def settings(self):
        s = Settings()
        self._check(load().rq_get_settings(self.ctx, C.byref(s)))
        return s

    @settings.setter
    def settings(self, s):
        self._check(load().rq_set_settings(self.ctx, C.byref(s)))

    def configure(self, **kw):
        s = self.settings
        for k, v in kw.items():
            setattr(s, k, v)
        self.settings = s

    def set_stream(self, stream_ptr):
        self._check(load().rq_set_stream(self.ctx, stream_ptr))

    def synchronize(self):
        self._check(load().rq_synchronize(self.ctx))

    # -- scenes and builds
    def scene_triangles(self, verts, idx):
        if isinstance(verts, np.ndarray):
            verts = np.ascontiguousarray(verts, np.float32)
            idx = np.ascontiguousarray(idx, np.uint32)
            nv, nt = verts.size // 3, idx.size // 3
        else:
            nv, nt = verts.numel() // 3, idx.numel() // 3
        pv, fl = _ptr(verts)
        pi, _ = _ptr(idx)
        h = C.c_void_p()
        self._check(load().rq_scene_create_triangles(self.ctx, pv, nv, pi, nt, fl, C.byref(h)))
        return Scene(self, h, 0, nt)

    def scene_spheres(self, sph):
        if isinstance(sph, np.ndarray):
            sph = np.ascontiguousarray(sph, np.float32)
            n = sph.size // 4
        else:
            n = sph.numel() // 4
        p, fl = _ptr(sph)
        h = C.c_void_p()
        self._check(load().rq_scene_create_spheres(self.ctx, p, n, fl, C.byref(h)))
        return Scene(self, h, 1, n)

    def build(self, scene, acc_type):
        if isinstance(acc_type, str):
            acc_type = ACC_NAMES[acc_type]
        h = C.c_void_p()
        self._check(load().rq_build(self.ctx, scene.handle, acc_type, C.byref(h)))
        return Accel(self, h, scene, acc_type)

    def build_batched(self, scenes, acc_type):
        """rq_build_batched: one structure per scene (RQ_LBVH: one pass of batched kernels)."""
        if isinstance(acc_type, str):
            acc_type = ACC_NAMES[acc_type]
        n = len(scenes)
        hs = (C.c_void_p * n)(*[sc.handle for sc in scenes])
        out = (C.c_void_p * n)()
        self._check(load().rq_build_batched(self.ctx, hs, n, acc_type, out))
        return [Accel(self, C.c_void_p(out[k]), scenes[k], acc_type) for k in range(n)]

    def rebuild_batched(self, accels):
        hs = (C.c_void_p * len(accels))(*[a.handle.value if isinstance(a.handle, C.c_void_p) else a.handle
                                           for a in accels])
        self._check(load().rq_accel_rebuild_batched(self.ctx, hs, len(accels)))

    @staticmethod
    def _handles(accels):
        return (C.c_void_p * len(accels))(*[a.handle.value if isinstance(a.handle, C.c_void_p) else a.handle
                                            for a in accels])

    def trace_batched(self, accels, rays, ray_offsets, any_hit=False, out=None):
        """rq_trace_batched: rays[ray_offsets[k]:ray_offsets[k+1]] against accels[k]."""
        offs = np.ascontiguousarray(ray_offsets, np.uint32)
        n = int(offs[-1])
        if isinstance(rays, np.ndarray):
            rays = np.ascontiguousarray(rays, RAY_DTYPE)
            if out is None:
                out = np.zeros((n + 31) // 32, np.uint32) if any_hit else np.zeros(n, HIT_DTYPE)
        pr, fl = _ptr(rays)
        po, _ = _ptr(out)
        self._check(load().rq_trace_batched(self.ctx, self._handles(accels), len(accels), pr, offs.ctypes.data,
                                            int(any_hit), po, fl))
        return out

    def plan(self, accels, rays, ray_offsets, out, any_hit=False, rebuild=False):
        """rq_plan_create on device buffers rays / out (torch tensors or pointers)."""
        offs = np.ascontiguousarray(ray_offsets, np.uint32)
        pr, _ = _ptr(rays)
        po, _ = _ptr(out)
        h = C.c_void_p()
        self._check(load().rq_plan_create(self.ctx, self._handles(accels), len(accels), int(rebuild), pr,
                                          offs.ctypes.data, int(any_hit), po, C.byref(h)))
        return Plan(self, h, (accels, rays, out))

    # -- queries
    def trace_closest(self, accel, rays, hits=None):
        if isinstance(rays, np.ndarray):
            rays = np.ascontiguousarray(rays, RAY_DTYPE)
            n = len(rays)
            hits = np.zeros(n, HIT_DTYPE) if hits is None else hits
        else:
            n = rays.numel() * rays.element_size() // 32
        pr, fl = _ptr(rays)
        ph, _ = _ptr(hits)
        self._check(load().rq_trace_closest(self.ctx, accel.handle, pr, n, ph, fl))
        return hits

    def trace_any(self, accel, rays, bits=None):
        if isinstance(rays, np.ndarray):
            rays = np.ascontiguousarray(rays, RAY_DTYPE)
            n = len(rays)
            bits = np.zeros((n + 31) // 32, np.uint32) if bits is None else bits
        else:
            n = rays.numel() * rays.element_size() // 32
        pr, fl = _ptr(rays)
        pb, _ = _ptr(bits)
        self._check(load().rq_trace_any(self.ctx, accel.handle, pr, n, pb, fl))
        return bits

    def trace_candidates(self, accel, rays):
        """rq_trace_candidates (boxIntersect's candidate lists): (counts per ray, ids)."""
        rays = np.ascontiguousarray(rays, RAY_DTYPE)
        n = len(rays)
        counts = np.zeros(n, np.uint32)
        total = C.c_uint64(0)
        self._check(load().rq_trace_candidates(self.ctx, accel.handle, rays.ctypes.data, n, counts.ctypes.data,
                                               None, 0, C.byref(total), 0))
        ids = np.zeros(max(total.value, 1), np.uint32)
        self._check(load().rq_trace_candidates(self.ctx, accel.handle, rays.ctypes.data, n, counts.ctypes.data,
                                               ids.ctypes.data, total.value, C.byref(total), 0))
        return counts, ids[:total.value]

    def trace_queries(self, accel, queries):
        """rq_trace_queries over host arrays: queries = [(rays, any_hit, out or None,
        ray_sort or -1, scheduling or -1), ...]; returns the outputs."""
        qs = (Query * len(queries))()
        outs, keep = [], []
        for k, (rays, any_hit, out, srt, sch) in enumerate(queries):
            rays = np.ascontiguousarray(rays, RAY_DTYPE)
            n = len(rays)
            if out is None:
                out = np.zeros((n + 31) // 32, np.uint32) if any_hit else np.zeros(n, HIT_DTYPE)
            keep.append(rays)
            outs.append(out)
            qs[k] = Query(rays.ctypes.data, n, int(any_hit), out.ctypes.data, srt, sch)
        self._check(load().rq_trace_queries(self.ctx, accel.handle, qs, len(queries)))
        return outs

    def trace_counters(self, accel, rays, any_hit=False):
        """FAST query plus (internal nodes visited, primitives tested) summed over the rays."""
        rays = np.ascontiguousarray(rays, RAY_DTYPE)
        n = len(rays)
        out = np.zeros((n + 31) // 32, np.uint32) if any_hit else np.zeros(n, HIT_DTYPE)
        cnt = np.zeros(2, np.uint64)
        self._check(load().rq_trace_counters(self.ctx, accel.handle, rays.ctypes.data, n, int(any_hit),
                                             out.ctypes.data, cnt.ctypes.data, 0))
        return out, cnt

    # -- component kernels
    def morton_codes(self, scene):
        out = np.zeros(scene.n, np.uint32)
        self._check(load().rq_morton_codes(self.ctx, scene.handle, out.ctypes.data, 0))
        return out

    def sort_pairs(self, keys, vals, key_bits=32):
        if isinstance(keys, np.ndarray):
            keys = np.array(keys, np.uint32, copy=True)
            vals = np.array(vals, np.uint32, copy=True)
            n = len(keys)
        else:
            n = keys.numel()
        pk, fl = _ptr(keys)
        pv, _ = _ptr(vals)
        self._check(load().rq_sort_pairs(self.ctx, pk, pv, n, key_bits, fl))
        return keys, vals

    def export_bvh2(self, accel):
        inf = accel.info()
        nodes = np.zeros((inf.n_nodes, 16), np.float32)
        order = np.zeros(inf.n_slots, np.uint32)
        codes = np.zeros(inf.n_prims, np.uint32) if accel.type == LBVH else None
        self._check(load().rq_accel_export_bvh2(self.ctx, accel.handle, nodes.ctypes.data, order.ctypes.data,
                                                codes.ctypes.data if codes is not None else None))
        return nodes, order, codes, np.array(inf.root_bounds, np.float32), inf

    def import_bvh2(self, scene, nodes, order, root_bounds):
        """rq_accel_import_bvh2: a BVH2 structure from host arrays in export_bvh2's layout."""
        nodes = np.ascontiguousarray(nodes, np.float32).reshape(-1, 16)
        order = np.ascontiguousarray(order, np.uint32)
        root = np.ascontiguousarray(root_bounds, np.float32).reshape(6)
        h = C.c_void_p()
        self._check(load().rq_accel_import_bvh2(self.ctx, scene.handle, nodes.ctypes.data if len(nodes) else None,
                                                len(nodes), order.ctypes.data, len(order), root.ctypes.data,
                                                C.byref(h)))
        return Accel(self, h, scene, BVH)

    def set_debug(self, sort_stall=0, small_stack=0):
        """rq_set_debug: test hooks that make device-side guards fire (all 0: off)."""
        d = (C.c_uint32 * 2)(int(sort_stall), int(small_stack))
        self._check(load().rq_set_debug(self.ctx, C.byref(d)))

    def export_bvh4(self, accel):
        """Collapsed 4-wide nodes, (n, 32) float32 (structures built with node_width 4)."""
        n = C.c_uint32(0)
        self._check(load().rq_accel_export_bvh4(self.ctx, accel.handle, None, C.byref(n)))
        nodes = np.zeros((max(n.value, 1), 32), np.float32)
        self._check(load().rq_accel_export_bvh4(self.ctx, accel.handle, nodes.ctypes.data, C.byref(n)))
        return nodes[:n.value]

    def export_kd(self, accel):
        inf = accel.info()
        nodes = np.zeros((inf.n_nodes, 3), np.int32)
        pidx = np.zeros(max(inf.n_slots, 1), np.int32)
        self._check(load().rq_accel_export_kd(self.ctx, accel.handle, nodes.ctypes.data, pidx.ctypes.data))
        return nodes, pidx[:inf.n_slots], np.array(inf.root_bounds, np.float32), inf

    def render_reference(self, accel, settings=None, jitter=None, surface_rgb=None):
        s = settings if settings is not None else self.settings
        npix = s.width * s.height
        pixels = np.zeros(npix * 3, np.uint8)
        rgb = np.zeros(npix * 3, np.float32)
        jit = np.ascontiguousarray(jitter, np.float64) if jitter is not None else None
        srgb = np.ascontiguousarray(surface_rgb, np.float32)
        self._check(load().rq_render_reference(self.ctx, accel.handle, C.byref(s),
                                               jit.ctypes.data if jit is not None else None,
                                               srgb.ctypes.data, pixels.ctypes.data, rgb.ctypes.data))
        return pixels, rgb.reshape(-1, 3)


    def render(self, accel, view, pixels=None, rgb=None):
        """rq_render.  Host arrays (allocated when None): returns (pixels (h, w, 3) uint8,
        rgb (h, w, 3) float32, ray counts [camera, shadow, mirror]).  Device tensors for
        pixels (and rgb): enqueued without waiting; returns (pixels, rgb, None)."""
        s = self.settings
        whole = view.window[2] == 0 or view.window[3] == 0
        w, h = (s.width, s.height) if whole else (view.window[2], view.window[3])
        if pixels is not None and not isinstance(pixels, np.ndarray):
            pp, fl = _ptr(pixels)
            pr, _ = _ptr(rgb)
            self._check(load().rq_render(self.ctx, accel.handle, C.byref(view), pp, pr, None, fl))
            return pixels, rgb, None
        pixels = np.zeros((h, w, 3), np.uint8)
        rgb = np.zeros((h, w, 3), np.float32)
        cnt = np.zeros(3, np.uint64)
        self._check(load().rq_render(self.ctx, accel.handle, C.byref(view), pixels.ctypes.data, rgb.ctypes.data,
                                     cnt.ctypes.data, 0))
        return pixels, rgb, cnt


SORT_NOALLOC_MAX_PAIRS = 1 << 20


def sort_pairs_noalloc(keys_ptr, vals_ptr, n, key_bits=32, stream_ptr=None):
    """rq_sort_pairs_noalloc on device buffers (pointers as ints); returns the status.
    Allocates nothing: for callers that cannot allocate device memory mid-run."""
    return int(load().rq_sort_pairs_noalloc(keys_ptr, vals_ptr, n, key_bits, stream_ptr))


def _take(ptr, count, dtype, width):
    """Copy a library-allocated array into numpy and release it."""
    try:
        if count == 0:
            return np.zeros((0, width), dtype)
        buf = (C.c_char * (count * width * np.dtype(dtype).itemsize)).from_address(ptr.value)
        return np.frombuffer(bytes(buf), dtype).reshape(count, width).copy()
    finally:
        load().rq_free(ptr)


def obj_load(path):
    """rq_obj_load: (verts (nv, 3) float32, idx (nt, 3) uint32)."""
    pv, pi = C.c_void_p(), C.c_void_p()
    nv, nt = C.c_uint32(), C.c_uint32()
    st = load().rq_obj_load(os.fsencode(path), C.byref(pv), C.byref(nv), C.byref(pi), C.byref(nt))
    if st != SUCCESS:
        raise RqError(st, f"cannot load {path}")
    return _take(pv, nv.value, np.float32, 3), _take(pi, nt.value, np.uint32, 3)


def obj_save(path, verts, idx):
    verts = np.ascontiguousarray(verts, np.float32)
    idx = np.ascontiguousarray(idx, np.uint32)
    st = load().rq_obj_save(os.fsencode(path), verts.ctypes.data, verts.size // 3, idx.ctypes.data, idx.size // 3)
    if st != SUCCESS:
        raise RqError(st, f"cannot save {path}")


def model_path(directory, scene_model):
    """rq_model_path: the model file of a SceneModel value, matched without regard to case."""
    buf = C.create_string_buffer(4096)
    st = load().rq_model_path(os.fsencode(directory), scene_model, buf, len(buf))
    if st != SUCCESS:
        raise RqError(st, f"no model file for {scene_model} in {directory}")
    return buf.value.decode()


def reference_spheres(path, clones=1):
    """rq_reference_spheres: createScene_new's spheres (n, 4) from a model file."""
    ps, n = C.c_void_p(), C.c_uint32()
    st = load().rq_reference_spheres(os.fsencode(path), clones, C.byref(ps), C.byref(n))
    if st != SUCCESS:
        raise RqError(st, f"cannot load {path}")
    return _take(ps, n.value, np.float32, 4)


def kernel_launch_count():
    return int(load().rq_kernel_launch_count())


def make_rays(org, dirs, tmin=0.0, tmax=np.inf):
    dirs = np.asarray(dirs, np.float32)
    r = np.zeros(len(dirs), RAY_DTYPE)
    r["org"] = np.broadcast_to(np.asarray(org, np.float32), dirs.shape)
    r["dir"] = dirs
    r["tmin"] = tmin
    r["tmax"] = tmax
    return r


def unpack_bits(bits, n):
    b = np.asarray(bits, np.uint32)
    return ((b[np.arange(n) >> 5] >> (np.arange(n) & 31).astype(np.uint32)) & 1).astype(np.uint8)
