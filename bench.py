#!/usr/bin/env python3
"""Benchmark of the ray-query hot path on one GB300 (or N replicas).

Workload (one step): rebuild the LBVH of a 998,000-triangle fBm heightfield
(1001 x 500 grid over [-1,1]^2, 5 octaves, amplitude 0.3), then trace
1920 x 1080 x 4 jittered primary rays closest-hit, one cosine-weighted
secondary ray per primary hit closest-hit, and one shadow ray per primary
hit any-hit.  Geometry and rays are seeded synthetic data resident in HBM
when the timed region starts; rays (265 MB per pass) exceed the 129 MB L2
and L2 is additionally flushed (256 MB write) before every timed step.

  value  = rays traced per second over the whole step (build included), Grays/s
  e2e    = the same through the C ABI with pinned host buffers: mesh upload,
           rebuild, and one rq_trace_queries call for the three ray classes
           (ray upload and hit/bit download inside the timed region)
  roofline: the step's dominant kernel against measured HBM bandwidth, with
           algorithmic bytes from the engine's traversal counters
  cpu_baseline: the CPU oracle (the reference's algorithms: median BVH build,
           collect-all division-slab traversal, Moller-Trumbore) on the whole
           job (every ray of the step), all host threads

python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "raytracer-data-structures_gb300"))

METRIC = "closest-hit Grays/s & LBVH build Mtri/s; served p50/p99 latency vs plain"
UNIT = "Grays/s"
WORKLOAD = ("LBVH build + incoherent traversal: 998,000-triangle fBm heightfield (1001x500), "
            "1920x1080x4 jittered primary closest-hit + cosine secondary closest-hit + shadow any-hit")
SEED = 20261203
EYE, TARGET, FOV = (0.0, -0.6, 1.1), (0.0, 0.0, 0.0), 40.0  # the view lies inside the heightfield
LIGHT = (1.5, -1.0, 3.0)
RAY_BYTES, HIT_BYTES, NODE_BYTES, TRI_BYTES = 32, 16, 64, 48


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    return ws, int(os.environ.get("RANK", "0")), int(os.environ.get("LOCAL_RANK", "0"))


def replica_step_ms(mean_ms, ws, device):
    """Step time of an N-replica job: the max over ranks of each rank's mean
    step time (the job ends with its slowest replica).  One process per GPU;
    no collective touches the data path, only this timing reduction."""
    if ws <= 1:
        return float(mean_ms)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(mean_ms)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def weak_value(ws, rays_per_rank, step_ms):
    """Whole-job rays per second (Grays/s) when every rank traces its own full workload."""
    return ws * rays_per_rank / (step_ms * 1e-3) / 1e9


def make_inputs(small=False):
    import scenes
    verts, idx = scenes.heightfield(1001, 500, amplitude=0.3, octaves=5, seed=SEED % 1000)
    w, h = (960, 540) if small else (1920, 1080)  # --small: profiling case, same mesh
    primary = scenes.pinhole_rays(w, h, 4, eye=EYE, target=TARGET, fov_deg=FOV, seed=SEED + 1)
    return verts, idx, primary


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            j = json.load(f)
        return float(j["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profile_value(name, kernel_key, path=os.path.join("profiles", "trace_lbvh_heightfield.md")):
    """A figure `name[kernel_key]: value ...` recorded in a committed ncu summary, or None."""
    p = os.path.join(ROOT, path)
    if not os.path.exists(p):
        return None
    with open(p) as f:
        for line in f:
            if line.startswith(f"{name}[{kernel_key}]:"):
                try:
                    return float(line.split(":", 1)[1].split()[0])
                except ValueError:
                    return None
    return None


def profile_traffic(kernel_key):
    """DRAM bytes per launch (full-size launch) from the committed ncu summary."""
    return profile_value("dram_bytes_per_launch", kernel_key)


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


# ----------------------------------------------------------------- our arm

def run_ours(args):
    import torch
    import rq
    import scenes

    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    # One stream for everything: torch ops, CUDA events and the engine's work.
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)

    verts, idx, primary = make_inputs(args.small)
    n_tri = len(idx)
    eng = rq.Engine(local)
    eng.set_stream(stream.cuda_stream)
    d_verts = torch.from_numpy(verts).to(dev)
    d_idx = torch.from_numpy(idx.view(np.int32)).to(dev)
    scene = eng.scene_triangles(d_verts, d_idx)
    acc = eng.build(scene, rq.LBVH)  # binary tree for the first primary pass

    def dev_rays(r):
        return torch.from_numpy(np.ascontiguousarray(r).view(np.uint8)).to(dev)

    d_prim = dev_rays(primary)
    n_p = len(primary)
    d_hits_p = torch.empty(n_p * HIT_BYTES, dtype=torch.uint8, device=dev)
    eng.trace_closest(acc, d_prim, d_hits_p)
    eng.synchronize()
    hits_p = d_hits_p.cpu().numpy().view(rq.HIT_DTYPE)
    secondary = scenes.cosine_rays(verts, idx, primary, hits_p, seed=SEED + 2)
    shadow = scenes.shadow_rays(verts, idx, primary, hits_p, LIGHT)
    n_s, n_sh = len(secondary), len(shadow)
    d_sec, d_sh = dev_rays(secondary), dev_rays(shadow)
    d_hits_s = torch.empty(n_s * HIT_BYTES, dtype=torch.uint8, device=dev)
    d_bits = torch.empty(((n_sh + 31) // 32) * 4, dtype=torch.uint8, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    total_rays = n_p + n_s + n_sh
    log(f"[bench] tris={n_tri} primary={n_p} secondary={n_s} shadow={n_sh}")

    ev = lambda: torch.cuda.Event(enable_timing=True)  # noqa: E731

    # Autotuning over the engine's speed-only options (results are identical
    # under every choice): BVH node width (binary or collapsed 4-wide, fixed
    # at build time, the collapse counted in the build phase) and ray
    # reordering per ray class.  Each candidate is timed on the real rays.
    def timed(fn, reps=3):
        times = []
        for _ in range(reps):
            a0, a1 = ev(), ev()
            a0.record(stream)
            fn()
            a1.record(stream)
            torch.cuda.synchronize(dev)
            times.append(a0.elapsed_time(a1))
        return min(times)

    def class_call(a, name):
        if name == "primary":
            return lambda: eng.trace_closest(a, d_prim, d_hits_p)
        if name == "secondary":
            return lambda: eng.trace_closest(a, d_sec, d_hits_s)
        return lambda: eng.trace_any(a, d_sh, d_bits)

    # Every (ray order, scheduling) pair per ray class; scheduling variants
    # walk binary nodes only.
    sort_names = {rq.RAY_SORT_NONE: "none", rq.RAY_SORT_OCTANT_MORTON: "octant_morton",
                  rq.RAY_SORT_ORIGIN_DIRECTION: "origin_direction", rq.RAY_SORT_DIRECTION_ORIGIN: "direction_origin",
                  rq.RAY_SORT_OCTANT_MORTON12: "octant_morton12", rq.RAY_SORT_OCTANT: "octant",
                  rq.RAY_SORT_OCTANT_MORTON3: "octant_morton3"}
    sched_names = {rq.SCHEDULING_THREAD_PER_RAY: "thread_per_ray", rq.SCHEDULING_LANE_REFILL: "lane_refill",
                   rq.SCHEDULING_SPECULATIVE: "speculative", rq.SCHEDULING_WARP_PACKET: "warp_packet",
                   rq.SCHEDULING_SHARED_TOP: "shared_top"}
    morton_names = {rq.MORTON_SCENE_BOUNDS: "scene_bounds", rq.MORTON_SCENE_CUBE: "scene_cube"}
    quality_names = {rq.LBVH_KARRAS: "karras", rq.LBVH_TREELETS: "treelets"}
    tuning = {}
    best = None
    candidates = [(w, m, q) for w in (rq.NODE_WIDTH_2, rq.NODE_WIDTH_4, rq.NODE_WIDTH_8) for m in morton_names
                  for q in quality_names]
    if args.no_tune:  # the live tuner's choice on a GB300, for profiling the same kernel mix
        candidates = [(rq.NODE_WIDTH_2, rq.MORTON_SCENE_CUBE, rq.LBVH_TREELETS)]
    for width, morton, quality in candidates:
        if True:
            eng.configure(node_width=width, morton=morton, lbvh_quality=quality, ray_sort=rq.RAY_SORT_NONE,
                          scheduling=rq.SCHEDULING_THREAD_PER_RAY)
            cand = eng.build(scene, rq.LBVH)
            choice, total = {}, timed(cand.rebuild)
            scheds = list(sched_names) if width == rq.NODE_WIDTH_2 else [rq.SCHEDULING_THREAD_PER_RAY]
            for name in ("primary", "secondary", "shadow"):
                opts = {}
                if args.no_tune:
                    fixed = rq.RAY_SORT_OCTANT if name == "secondary" else rq.RAY_SORT_NONE
                    pairs = [(fixed, rq.SCHEDULING_THREAD_PER_RAY)]
                else:
                    pairs = [(srt, sch) for srt in sort_names for sch in scheds]
                for srt, sch in pairs:
                    eng.configure(ray_sort=srt, scheduling=sch)
                    opts[(srt, sch)] = timed(class_call(cand, name))
                choice[name] = min(opts, key=opts.get)
                log(f"[bench] tune width {width} {morton_names[morton]} {quality_names[quality]} {name}: " +
                    ", ".join(f"{sort_names[a]}/{sched_names[b]} {t:.3f}" for (a, b), t in sorted(opts.items(), key=lambda kv: kv[1])))
                total += opts[choice[name]]
            tuning[f"width{max(width, 2)}_{morton_names[morton]}_{quality_names[quality]}"] = {
                "est_step_ms": round(total, 4),
                "choice": {k: [sort_names[v[0]], sched_names[v[1]]] for k, v in choice.items()}}
            if best is None or total < best[0]:
                if best is not None:
                    best[1].close()
                best = (total, cand, (width, morton, quality), choice)
            else:
                cand.close()
    acc.close()
    _, acc, (node_width, morton_mode, lbvh_quality), sort_choice = best
    eng.configure(node_width=node_width, morton=morton_mode, lbvh_quality=lbvh_quality, ray_sort=rq.RAY_SORT_NONE,
                  scheduling=rq.SCHEDULING_THREAD_PER_RAY)
    node_bytes = 128 if node_width in (rq.NODE_WIDTH_4, rq.NODE_WIDTH_8) else NODE_BYTES
    log(f"[bench] tuning: {tuning} -> width {max(node_width, 2)}, morton {morton_names[morton_mode]}, "
        f"lbvh {quality_names[lbvh_quality]}")

    # Traversal work of each query on these exact rays (the byte model's inputs).
    counts = {}
    for name, rays, anyhit in (("primary", primary, False), ("secondary", secondary, False), ("shadow", shadow, True)):
        _, cnt = eng.trace_counters(acc, rays, any_hit=anyhit)
        counts[name] = (int(cnt[0]), int(cnt[1]))

    def trace_class(name, marks=None):
        eng.configure(ray_sort=sort_choice[name][0], scheduling=sort_choice[name][1])
        class_call(acc, name)()

    def step(marks=None):
        if marks: marks[0].record(stream)
        acc.rebuild()
        if marks: marks[1].record(stream)
        trace_class("primary")
        if marks: marks[2].record(stream)
        trace_class("secondary")
        if marks: marks[3].record(stream)
        trace_class("shadow")
        if marks: marks[4].record(stream)

    for _ in range(args.warmup):
        flush.zero_()
        step()
    eng.synchronize()

    launches0 = rq.kernel_launch_count()
    phase = np.zeros((args.steps, 4))
    step_ms = np.zeros(args.steps)
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize(dev)
    with ClockSampler(local) as clk:
        for k in range(args.steps):
            flush.zero_()
            marks = [ev() for _ in range(5)]
            step(marks)
            torch.cuda.synchronize(dev)
            step_ms[k] = marks[0].elapsed_time(marks[4])
            phase[k] = [marks[i].elapsed_time(marks[i + 1]) for i in range(4)]
    eng.synchronize()
    launches = rq.kernel_launch_count() - launches0
    mean_ms = replica_step_ms(float(step_ms.mean()), ws, dev)
    value = weak_value(ws, total_rays, mean_ms)
    ph = phase.mean(0)
    build_ms, prim_ms, sec_ms, sh_ms = ph

    # Roofline of the dominant kernel (largest share of the step).
    kern = {"build": build_ms, "trace_primary": prim_ms, "trace_secondary": sec_ms, "trace_shadow": sh_ms}
    dom = max(kern, key=kern.get)
    peak, peak_kind = measured_peaks()

    def trace_bytes(name, n, closest=True):
        v, t = counts[name]
        return n * RAY_BYTES + (n * HIT_BYTES if closest else ((n + 31) // 32) * 4) + v * node_bytes + t * TRI_BYTES

    build_bytes = build_bytes_per_tri(lbvh_quality == rq.LBVH_TREELETS) * n_tri
    alg = {"build": build_bytes, "trace_primary": trace_bytes("primary", n_p),
           "trace_secondary": trace_bytes("secondary", n_s), "trace_shadow": trace_bytes("shadow", n_sh, False)}
    achieved = alg[dom] / (kern[dom] * 1e-3) / 1e9
    traffic = profile_traffic(dom)
    n_dom = {"trace_primary": n_p, "trace_secondary": n_s, "trace_shadow": n_sh}.get(dom)
    step_work = sum(alg.values())
    roofline = {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 1), "peak": peak,
                "unit": "GB/s", "frac": round(achieved / peak, 4), "peak_source": f"{peak_kind} hbm_gbs",
                "achieved_kind": ("L1/L2-inclusive work bytes: every node visit (node_bytes) and triangle test "
                                  "(48 B) counted as a fetch, plus 32 B ray + hit; most of these fetches hit L1/L2"),
                "traffic": traffic, "algorithmic_bytes": int(alg[dom]),
                # What DRAM itself carries for this kernel (ncu, committed summary) against the
                # live kernel time: the bandwidth actually used.
                "dram_gbs": round(traffic / (kern[dom] * 1e-3) / 1e9, 1) if traffic else None,
                "dram_frac": round(traffic / (kern[dom] * 1e-3) / 1e9 / peak, 4) if traffic else None,
                "issue_active": profile_value("issue_active", dom),
                "lanes_per_inst": profile_value("lanes_per_inst", dom),
                "l2_hit_rate": profile_value("l2_hit_rate", dom),
                "limiter": ("divergence and memory latency (lanes per instruction and long-scoreboard stalls), "
                            "not DRAM bandwidth") if dom != "build" else None,
                "compulsory_frac": round((n_dom * (RAY_BYTES + HIT_BYTES)) / (kern[dom] * 1e-3) / 1e9 / peak, 4)
                if n_dom else None,
                # The whole step's work bytes over the step time: above 1 means the model's
                # fetches are served by the caches, not that DRAM ran above its peak.
                "step_work_frac": round(step_work / (mean_ms * 1e-3) / 1e9 / peak, 4)}

    # The same step through the C ABI with host buffers, right after the
    # device-resident step (before the other legs leave memory and heat behind).
    e2e = None
    if rank == 0 and not args.skip_e2e:
        e2e = run_e2e(eng, scene, acc, verts, idx, primary, secondary, shadow, args, sort_choice)

    # The same rays through the other builders of the dataStructure switch.
    structures = {"LBVH": {"build_ms": round(build_ms, 4), "trace_ms": round(prim_ms + sec_ms + sh_ms, 4),
                           "grays_s": round(total_rays / ((prim_ms + sec_ms + sh_ms) * 1e-3) / 1e9, 4)}}
    if not args.skip_structures:
        for name in ("BVH", "KDTREE"):
            other = eng.build(scene, name)
            bms, tms = [], []
            for k in range(3):
                m = [ev() for _ in range(3)]
                flush.zero_()
                m[0].record(stream)
                other.rebuild()
                m[1].record(stream)
                for cls in ("primary", "secondary", "shadow"):
                    eng.configure(ray_sort=sort_choice[cls][0], scheduling=sort_choice[cls][1])
                    class_call(other, cls)()
                m[2].record(stream)
                torch.cuda.synchronize(dev)
                if k:
                    bms.append(m[0].elapsed_time(m[1]))
                    tms.append(m[1].elapsed_time(m[2]))
            eng.synchronize()
            inf = other.info()
            structures[name] = {"build_ms": round(float(np.mean(bms)), 3), "trace_ms": round(float(np.mean(tms)), 4),
                                "grays_s": round(total_rays / (float(np.mean(tms)) * 1e-3) / 1e9, 4),
                                "nodes": int(inf.n_nodes)}
            other.close()

    render = None
    if not args.skip_render:
        render = run_render_legs(eng, stream, dev, args)
        render["reference_scene"] = run_reference_scene_leg()

    batched = None
    if not args.skip_batch:
        batched = run_batch_leg(eng, stream, dev, args)

    served = None
    if not args.skip_serve and ws == 1:
        served = run_serve_leg(args)

    cpu = None
    if rank == 0 and ws == 1 and not args.skip_cpu:
        cpu = cpu_baseline(verts, idx, primary, secondary, shadow)

    if rank == 0:
        out = {
            "metric": METRIC, "value": round(value, 4), "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(mean_ms, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
            "config": {"workload": WORKLOAD, "dataStructure": "LBVH", "triangles": n_tri, "primary_rays": n_p,
                       "secondary_rays": n_s, "shadow_rays": n_sh, "seed": SEED,
                       "l2": "flushed before every timed step (256 MB write); rays exceed L2",
                       "ray_generation": ("primary rays generated once on the host; secondary (cosine) and shadow "
                                          "rays generated once from the first primary trace's hits; each timed "
                                          "step rebuilds the LBVH and traces all three sets"),
                       "parallelism": f"replicas x{ws}" if ws > 1 else "single GPU",
                       "node_width": max(node_width, 2), "morton": morton_names[morton_mode],
                       "lbvh_quality": quality_names[lbvh_quality],
                       "ray_sort": {k: sort_names[v[0]] for k, v in sort_choice.items()},
                       "scheduling": {k: sched_names[v[1]] for k, v in sort_choice.items()}, "tuning": tuning},
            "lbvh_build_mtri_s": round(n_tri / (build_ms * 1e-3) / 1e6, 2),
            "closest_grays_s": round((n_p + n_s) / ((prim_ms + sec_ms) * 1e-3) / 1e9, 4),
            "any_grays_s": round(n_sh / (sh_ms * 1e-3) / 1e9, 4),
            "phase_ms": {"build": round(build_ms, 4), "trace_primary": round(prim_ms, 4),
                         "trace_secondary": round(sec_ms, 4), "trace_shadow": round(sh_ms, 4)},
            "traversal_work": {k: {"node_bytes": node_bytes, "nodes_per_ray": round(v[0] / max(1, {"primary": n_p, "secondary": n_s, "shadow": n_sh}[k]), 3),
                                   "tris_per_ray": round(v[1] / max(1, {"primary": n_p, "secondary": n_s, "shadow": n_sh}[k]), 3)}
                               for k, v in counts.items()},
            "roofline": roofline,
            "build_roofline": {"achieved": round(build_bytes / (build_ms * 1e-3) / 1e9, 1), "peak": peak,
                               "unit": "GB/s", "bytes_per_tri": build_bytes_per_tri(lbvh_quality == rq.LBVH_TREELETS),
                               "frac": round(build_bytes / (build_ms * 1e-3) / 1e9 / peak, 4)},
            "structures": structures,
            "render": render,
            "batched": batched,
            "served": served,
            "e2e": e2e, "cpu_baseline": cpu, "gpu_launches": int(launches), "clocks": clk.summary(),
        }
        print(json.dumps(out), flush=True)
    eng.close()
    if ws > 1:
        torch.distributed.destroy_process_group()


def run_reference_scene_leg(reps=5):
    """The reference program's own workload: its default bunny scene (35,948
    spheres from createScene_new, taken from the golden fixture) rendered at
    640x480, 1 sample, with render()'s camera and jitter and castRay's shading
    (rq_render_reference), for each builder of the dataStructure switch.  A
    fresh context with the reference's default settings; host output buffers;
    wall time per call, as a caller of the reference's render() sees it."""
    import rq
    sph = np.load(os.path.join(ROOT, "tests", "golden", "bunny.npz"))["spheres"]
    colors = np.tile(np.array([0.8, 0.7, 0.0], np.float32), (len(sph), 1))  # main.cpp:689
    colors[-1] = 0.0  # the ground sphere (main.cpp:703)
    eng = rq.Engine(0)
    s = eng.settings
    out = {"spheres": int(len(sph)), "image": f"{s.width}x{s.height}x{s.aa_samples}",
           "rays": int(s.width * s.height * s.aa_samples)}
    scene = eng.scene_spheres(sph)
    for name in ("BVH", "LBVH", "KDTREE"):
        builds = []
        for _ in range(3):
            eng.synchronize()
            t0 = time.perf_counter()
            acc = eng.build(scene, name)
            eng.synchronize()
            builds.append(time.perf_counter() - t0)
        for _ in range(2):
            eng.render_reference(acc, surface_rgb=colors)
        t0 = time.perf_counter()
        for _ in range(reps):
            eng.render_reference(acc, surface_rgb=colors)
        render_s = (time.perf_counter() - t0) / reps
        out[name] = {"build_ms": round(1e3 * min(builds[1:]), 3), "render_ms": round(1e3 * render_s, 3),
                     "rays_per_s": round(out["rays"] / render_s, 0)}
        acc.close()
    eng.close()
    return out


def run_render_legs(eng, stream, dev, args):
    """The render step (rq_render) on the small plain workload (81,920-triangle
    icosphere, 640x480, 1 spp, Lambert + shadow ray; BVH, KDTREE and LBVH) and
    the large one (~10M-triangle merged icospheres, 3840x2160, 4 spp, shadow ray
    + 2 mirror bounces; LBVH).  Each timed frame = structure rebuild + render
    into device buffers, L2 flushed before it; rays = camera + shadow + mirror
    rays actually traced (the engine's counts)."""
    import torch
    import rq
    import scenes

    ev = lambda: torch.cuda.Event(enable_timing=True)  # noqa: E731
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    saved = eng.settings
    out = {}

    def leg(verts, idx, structures, width, height, spp, view_kw, frames, count_work=False):
        eng.configure(width=width, height=height, aa_samples=spp, ray_sort=rq.RAY_SORT_NONE,
                      scheduling=rq.SCHEDULING_THREAD_PER_RAY)
        dv = torch.from_numpy(verts).to(dev)
        di = torch.from_numpy(idx.view(np.int32)).to(dev)
        scene = eng.scene_triangles(dv, di)
        view = rq.make_view(**view_kw)
        pix = torch.empty(width * height * 3, dtype=torch.uint8, device=dev)
        res = {"triangles": int(len(idx)), "image": f"{width}x{height}x{spp}", "bounces": view_kw["bounces"]}
        cam = scenes.pinhole_rays(width, height, spp, eye=view_kw["eye"], target=view_kw["target"],
                                  up=view_kw["up"], fov_deg=view_kw["fov_deg"], seed=SEED + 7) if count_work else None
        runs = [(name, q) for name in structures
                for q in ((rq.LBVH_KARRAS, rq.LBVH_TREELETS) if name == "LBVH" else (None,))]
        for name, quality in runs:
            if quality is not None:
                eng.configure(lbvh_quality=quality)
            acc = eng.build(scene, name)
            _, _, cnt = eng.render(acc, view)  # synchronous: the ray counts
            rays = int(cnt.sum())
            work = None
            if cam is not None and name != "KDTREE":  # counters exist for BVH structures
                _, wc = eng.trace_counters(acc, cam)
                work = {"rays": "every camera ray of the view (seeded jitter)", "node_bytes": 64,
                        "nodes_per_ray": round(int(wc[0]) / len(cam), 3), "tris_per_ray": round(int(wc[1]) / len(cam), 3)}
            for _ in range(2):
                acc.rebuild()
                eng.render(acc, view, pix)
            times, rtimes = [], []
            for _ in range(frames):
                flush.zero_()
                m = [ev() for _ in range(3)]
                m[0].record(stream)
                acc.rebuild()
                m[1].record(stream)
                eng.render(acc, view, pix)
                m[2].record(stream)
                torch.cuda.synchronize(dev)
                times.append(m[0].elapsed_time(m[2]))
                rtimes.append(m[1].elapsed_time(m[2]))
            eng.synchronize()
            t, tr = float(np.mean(times)), float(np.mean(rtimes))
            entry = {"frame_ms": round(t, 3), "render_ms": round(tr, 3), "build_ms": round(t - tr, 3),
                     "rays": rays, "ray_counts": [int(c) for c in cnt],
                     "grays_s": round(rays / (t * 1e-3) / 1e9, 4)}
            if work:
                entry["traversal_work"] = work
            if quality is not None:  # the LBVH with either build setting: the faster frame is the entry
                qn = "treelets" if quality == rq.LBVH_TREELETS else "karras"
                entry["lbvh_quality"] = qn
                prev = res.get(name)
                if prev is not None:
                    if prev["frame_ms"] <= entry["frame_ms"]:
                        prev["other_lbvh_quality_frame_ms"] = {qn: entry["frame_ms"]}
                        entry = None
                    else:
                        entry["other_lbvh_quality_frame_ms"] = {prev["lbvh_quality"]: prev["frame_ms"]}
            if entry is not None:
                res[name] = entry
            acc.close()
        scene.close()
        return res

    v1, f1 = scenes.c1_mesh()
    out["c1"] = leg(v1, f1, ("BVH", "KDTREE", "LBVH"), 640, 480, 1, scenes.C1_VIEW, 10, count_work=True)
    if not args.small:
        v3, f3, _ = scenes.merged_icospheres()
        out["c3"] = leg(v3, f3, ("LBVH",), 3840, 2160, 4, scenes.C3_VIEW, 3)
    eng.settings = saved
    log(f"[bench] render: {out}")
    return out


def batch_rays(torch, dev, meshes, counts, seed):
    """Rays of each scene, generated on the device from a seeded generator:
    origins uniform on the scene's bounding sphere (radius x 1.05), directions
    towards uniform points inside its box, tmin 0, tmax inf.  Returns a
    (sum counts) x 32-byte uint8 tensor."""
    g = torch.Generator(device=dev)
    g.manual_seed(seed)
    lo = torch.tensor(np.array([v.min(0) for v, _ in meshes]), dtype=torch.float64, device=dev)
    hi = torch.tensor(np.array([v.max(0) for v, _ in meshes]), dtype=torch.float64, device=dev)
    idx = torch.repeat_interleave(torch.arange(len(meshes), device=dev), torch.tensor(counts, device=dev))
    n = int(idx.numel())
    l, h = lo[idx], hi[idx]
    c, R = (l + h) / 2, torch.linalg.norm(h - l, dim=1, keepdim=True) / 2 * 1.05
    sdir = torch.randn(n, 3, generator=g, device=dev, dtype=torch.float64)
    org = c + R * sdir / torch.linalg.norm(sdir, dim=1, keepdim=True)
    tgt = l + torch.rand(n, 3, generator=g, device=dev, dtype=torch.float64) * (h - l)
    d = tgt - org
    d = d / torch.linalg.norm(d, dim=1, keepdim=True)
    out = torch.empty(n, 8, dtype=torch.float32, device=dev)
    out[:, 0:3] = org.float()
    out[:, 3] = 0.0
    out[:, 4:7] = d.float()
    out[:, 7] = float("inf")
    return out.view(torch.uint8).reshape(-1)


def c4_workload(n_sc=256):
    """The many-scene workload: n_sc meshes with triangle counts log-uniform in
    [1k, 500k], each a displaced icosphere or an fBm heightfield chosen by
    seed, and per-scene ray counts log-uniform in [64k, 2M].  Returns
    (meshes [(verts, idx)], ray counts, ray offsets (n_sc + 1, uint32))."""
    import scenes
    mixed = scenes.mixed_meshes(n_sc, 1e3, 5e5, SEED + 40)
    rng = np.random.default_rng(SEED + 41)
    ray_n = np.exp(rng.uniform(np.log(64e3), np.log(2e6), n_sc)).astype(np.int64)
    offs = np.zeros(n_sc + 1, np.uint32)
    offs[1:] = np.cumsum(ray_n)
    return [(v, f) for v, f, _ in mixed], ray_n, offs


def run_batch_leg(eng, stream, dev, args):
    """Many scenes at once: 256 meshes (displaced icospheres or fBm
    heightfields, chosen by seed) with triangle counts log-uniform in [1k,
    500k] and ray counts log-uniform in [64k, 2M] (origins on each scene's
    bounding sphere, directions into its box).  One step =
    rebuild every structure + closest hit for every ray.  'plain' does it one
    scene per launch (rq_accel_rebuild + rq_trace_closest per scene); 'batched'
    replays one plan: the batched LBVH rebuild + one persistent many-structure
    query, captured as a CUDA graph, launch shape autotuned.  Device buffers,
    L2 flushed before every timed step."""
    import torch
    import rq
    import scenes

    ev = lambda: torch.cuda.Event(enable_timing=True)  # noqa: E731
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    n_sc = 32 if args.small else 256
    meshes, ray_n, offs = c4_workload(n_sc)
    n_tri = int(sum(len(f) for _, f in meshes))
    saved = eng.settings
    # the Karras trees the batched rebuild makes, for the one-scene-per-launch path too
    eng.configure(ray_sort=rq.RAY_SORT_NONE, scheduling=rq.SCHEDULING_THREAD_PER_RAY, lbvh_quality=rq.LBVH_KARRAS)
    sc = [eng.scene_triangles(v, f) for v, f in meshes]
    n_rays = int(offs[-1])
    d_rays = batch_rays(torch, dev, meshes, ray_n.tolist(), SEED + 41)
    d_hits = torch.empty(n_rays * HIT_BYTES, dtype=torch.uint8, device=dev)
    log(f"[bench] batch: {n_sc} scenes, {n_tri} tris, {n_rays} rays")

    def timed(fn, reps):
        ts = []
        for _ in range(reps):
            flush.zero_()
            a, b = ev(), ev()
            a.record(stream)
            fn()
            b.record(stream)
            torch.cuda.synchronize(dev)
            ts.append(a.elapsed_time(b))
        return float(np.mean(ts[1:])) if len(ts) > 1 else ts[0]

    # plain: one scene per launch
    singles = [eng.build(s, rq.LBVH) for s in sc]
    views = [(d_rays[int(offs[k]) * 32:int(offs[k + 1]) * 32], d_hits[int(offs[k]) * 16:int(offs[k + 1]) * 16])
             for k in range(n_sc)]

    def plain_step():
        for k in range(n_sc):
            singles[k].rebuild()
            eng.trace_closest(singles[k], views[k][0], views[k][1])

    def plain_build():
        for k in range(n_sc):
            singles[k].rebuild()

    plain_ms = timed(plain_step, 4)
    plain_build_ms = timed(plain_build, 4)
    ref_hits = d_hits.clone()
    for a in singles:
        a.close()

    # batched: one plan = batched rebuild + persistent query, one CUDA graph
    accs = eng.build_batched(sc, rq.LBVH)
    plan = eng.plan(accs, d_rays, offs, d_hits, rebuild=True)
    batched_ms = timed(plan.launch, 6)
    eng.synchronize()
    same = bool(torch.equal(d_hits, ref_hits))
    batched_build_ms = timed(lambda: eng.rebuild_batched(accs), 4)
    # Traversal work (node visits, triangle tests per ray) on a seeded 1% sample
    # of every scene's rays, through the counting walk of the same structures.
    work_rng = np.random.default_rng(SEED + 42)
    ray_rows = d_rays.view(-1, 32)
    visits = tests = sampled = 0
    for k in range(n_sc):
        a, b = int(offs[k]), int(offs[k + 1])
        m = max(1, (b - a) // 100)
        sel = np.sort(work_rng.choice(b - a, size=m, replace=False)) + a
        sample = ray_rows[torch.from_numpy(sel).to(dev)].cpu().numpy().reshape(-1).view(rq.RAY_DTYPE)
        _, cnt = eng.trace_counters(accs[k], sample)
        visits, tests, sampled = visits + int(cnt[0]), tests + int(cnt[1]), sampled + m
    info = plan.info()
    plan.close()
    for a in accs:
        a.close()
    for s in sc:
        s.close()
    eng.settings = saved
    out = {"scenes": n_sc, "triangles": n_tri, "rays": n_rays,
           "plain": {"step_ms": round(plain_ms, 3), "build_ms": round(plain_build_ms, 3),
                     "grays_s": round(n_rays / (plain_ms * 1e-3) / 1e9, 4)},
           "batched": {"step_ms": round(batched_ms, 3), "build_ms": round(batched_build_ms, 3),
                       "grays_s": round(n_rays / (batched_ms * 1e-3) / 1e9, 4),
                       "build_mtri_s": round(n_tri / (batched_build_ms * 1e-3) / 1e6, 1),
                       "graph_kernels": int(info.graph_kernels),
                       "shape": {"block": int(info.block_threads), "stack": int(info.stack_entries),
                                 "ray_order": bool(info.ray_order), "node_width": int(info.node_width),
                                 "width_ms": {"2": round(float(info.width_ms[0]), 3),
                                              "4": round(float(info.width_ms[1]), 3),
                                              "8": round(float(info.width_ms[2]), 3)},
                                 "tuned_ms": [round(float(x), 3) for x in info.shape_ms],
                                 "tuned_ordered_ms": [round(float(x), 3) for x in info.ordered_ms]}},
           "speedup": round(plain_ms / batched_ms, 3), "hits_identical": same,
           "traversal_work": {"sample": f"{sampled} rays (1% of each scene's, seeded)", "node_bytes": 64,
                              "nodes_per_ray": round(visits / sampled, 3), "tris_per_ray": round(tests / sampled, 3)}}
    log(f"[bench] batched: {out}")
    return out


def run_serve_leg(args):
    """The serving loop under load: Poisson arrivals at 400 requests/s (and
    at 1,200/s, more than either path serves) for a few seconds; 32 resident displaced icospheres of 10k-2M triangles (log-uniform)
    plus new meshes (5% of requests name a mesh never seen before: upload +
    LBVH build on demand); resolution uniform over 320x240, 640x480, 1280x720,
    1920x1080, spp over 1, 2, 4, 8, 16; HBM budget 80 GB with LRU eviction.
    The same request stream is served with continuous batching and one
    request per step; latency = submit to pixels in host memory."""
    import rq
    import scenes

    secs = 1.0 if args.small else 4.0
    n_res, n_new_max = 32, 64
    # seeded displaced icospheres, 10k-2M triangles (log-uniform target, nearest subdivision level)
    pool = scenes.mixed_meshes(n_res + n_new_max, 1e4, 2e6, SEED + 200, kinds=("icosphere",))
    lib = {k: pool[k][:2] for k in range(n_res)}
    fresh = {1000 + k: pool[n_res + k][:2] for k in range(n_new_max)}
    res = [(320, 240), (640, 480), (1280, 720), (1920, 1080)]

    def schedule(rate, seed):
        rng = np.random.default_rng(seed)
        arrivals = np.cumsum(rng.exponential(1.0 / rate, int(rate * secs * 1.3) + 16))
        arrivals = arrivals[arrivals < secs]
        sched, new_ids = [], iter(sorted(fresh))
        for k, t in enumerate(arrivals):
            mid = next(new_ids, None) if rng.random() < 0.05 else None
            if mid is None:
                mid = int(rng.integers(n_res))
            w, h = res[int(rng.integers(4))]
            spp = int(rng.choice([1, 2, 4, 8, 16]))
            az = rng.uniform(0, 6.283)
            # an orbit around the mesh's centre (the meshes fill the unit cube)
            view = rq.make_view(eye=(float(0.5 + 2.2 * np.cos(az)), float(0.5 + 2.2 * np.sin(az)),
                                     float(0.5 + rng.uniform(-0.8, 0.8))),
                                target=(0.5, 0.5, 0.5), up=(0.0, 0.0, 1.0), fov_deg=float(rng.uniform(35, 60)),
                                light=(1.5, -2.0, 3.0), albedo=(0.7, 0.65, 0.6), ambient=0.1, seed=int(seed + k))
            sched.append((float(t), mid, view, w, h, spp))
        return sched

    def serve(sched, batching, budget):
        srv = rq.Server(batching=batching, hbm_budget=budget)
        for mid, (v, f) in list(lib.items()) + list(fresh.items()):
            srv.add_mesh(mid, v, f)
        for mid in lib:  # the library starts resident (as far as the budget allows)
            srv.wait(srv.submit(mid, sched[0][2], 32, 32, 1, keep_pixels=False), want_pixels=False)
        srv.reset_stats()
        t0 = time.perf_counter()
        tickets = []
        for t, mid, view, w, h, spp in sched:
            lag = t - (time.perf_counter() - t0)
            if lag > 0:
                time.sleep(lag)
            tickets.append(srv.submit(mid, view, w, h, spp, keep_pixels=False))
        srv.drain()
        wall = time.perf_counter() - t0
        st = srv.stats()
        rays = int(st.camera_rays + st.shadow_rays)
        r = {"completed": int(st.completed), "rejected": int(st.rejected), "steps": int(st.batches),
             "builds": int(st.builds), "evictions": int(st.evictions),
             "p50_ms": round(st.latency_ms_p50, 3), "p99_ms": round(st.latency_ms_p99, 3),
             "mean_ms": round(st.latency_ms_mean, 3), "max_ms": round(st.latency_ms_max, 3),
             "wall_s": round(wall, 3), "busy_s": round(st.busy_s, 3), "rays": rays,
             "grays_s_wall": round(rays / wall / 1e9, 4), "grays_s_busy": round(rays / max(st.busy_s, 1e-9) / 1e9, 4),
             "resident_gb": round(st.resident_bytes / 1e9, 3)}
        for tk in tickets:
            srv.wait(tk, want_pixels=False)
        srv.close()
        return r

    out = {"seconds": secs, "resident_meshes": n_res, "new_meshes": n_new_max,
           "triangles_resident": int(sum(len(f) for _, f in lib.values())),
           "triangles_library": int(sum(len(f) for _, f in list(lib.values()) + list(fresh.values()))),
           "hbm_budget_gb": 80}
    # the configured load, then an overloaded one (arrivals faster than either path serves them)
    for rate in (400.0, 1200.0):
        sched = schedule(rate, SEED + 50 + int(rate))
        leg = {"requests": len(sched), "rate_per_s": rate, "new_mesh_requests": sum(1 for x in sched if x[1] >= 1000)}
        for mode, batching in (("batched", True), ("one_per_step", False)):
            leg[mode] = serve(sched, batching, 80 << 30)
            log(f"[bench] serve {int(rate)}/s {mode}: {leg[mode]}")
        b, o = leg["batched"], leg["one_per_step"]
        leg["busy_rays_ratio"] = round(b["grays_s_busy"] / max(o["grays_s_busy"], 1e-9), 3)
        leg["wall_rays_ratio"] = round(b["grays_s_wall"] / max(o["grays_s_wall"], 1e-9), 3)
        leg["p99_ratio"] = round(o["p99_ms"] / max(b["p99_ms"], 1e-9), 3)
        out[f"load_{int(rate)}"] = leg
    # LRU residency under load: the overloaded schedule with a 4 GB budget
    # (the library needs about 6.5 GB on the device): meshes are evicted and rebuilt
    tight = serve(schedule(1200.0, SEED + 1250), True, 4 << 30)
    tight["hbm_budget_gb"] = 4
    out["tight_budget"] = tight
    log(f"[bench] serve tight budget: {tight}")
    return out


def build_bytes_per_tri(treelets=False):
    """Compulsory bytes per triangle of the LBVH build kernels:
    bounds 6 (12 B per vertex, 0.5 vertex per triangle) + Morton 26 (12 B indices,
    6 B vertices, 8 B code/index write) + 4 sort passes x 16 + Karras 28 (code
    read 4, links 16, parents 8) + refit 150 (order 4, indices 12, vertices 6,
    48 B payload write, 24 B child box write, 48 B sibling reread per internal
    node, 4 B parent link, 4 B flag); with the treelet pass + 140 per internal
    node (64 B node read and write, 4 B cost write, 8 B parent links)."""
    return 6 + 26 + 64 + 28 + 150 + (140 if treelets else 0)


def run_e2e(eng, scene, acc, verts, idx, primary, secondary, shadow, args, sort_choice):
    import torch
    import rq

    def pinned(a):
        a = np.ascontiguousarray(a)
        t = torch.empty(a.nbytes, dtype=torch.uint8, pin_memory=True)
        v = t.numpy().view(a.dtype).reshape(a.shape)
        v[...] = a
        return t, v

    keep = []
    tv, hv = pinned(verts); keep.append(tv)
    ti, hi = pinned(idx); keep.append(ti)
    tp, hp = pinned(primary); keep.append(tp)
    ts, hs = pinned(secondary); keep.append(ts)
    tsh, hsh = pinned(shadow); keep.append(tsh)
    th1, out_p = pinned(np.zeros(len(primary), rq.HIT_DTYPE)); keep.append(th1)
    th2, out_s = pinned(np.zeros(len(secondary), rq.HIT_DTYPE)); keep.append(th2)
    tb, out_b = pinned(np.zeros((len(shadow) + 31) // 32, np.uint32)); keep.append(tb)

    def step():
        # one call for the three queries: copies and traversals overlap across
        # them; the incoherent secondary rays (the longest traversal) first
        scene.update(hv, hi)
        acc.rebuild()
        eng.trace_queries(acc, [(hs, False, out_s, sort_choice["secondary"][0], sort_choice["secondary"][1]),
                                (hp, False, out_p, sort_choice["primary"][0], sort_choice["primary"][1]),
                                (hsh, True, out_b, sort_choice["shadow"][0], sort_choice["shadow"][1])])

    for _ in range(max(1, args.warmup)):
        step()
    eng.synchronize()
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        step()
        times.append(time.perf_counter() - t0)
    eng.synchronize()
    # Each step is timed on the host clock; the value comes from the median
    # step: on a shared host one step in twenty now and then stalls for tens
    # of milliseconds (the other steps unchanged), which a mean would carry
    # into the line.  The mean and the fastest step are reported beside it.
    t = float(np.median(times))
    rays = len(primary) + len(secondary) + len(shadow)
    h2d = hv.nbytes + hi.nbytes + hp.nbytes + hs.nbytes + hsh.nbytes
    d2h = out_p.nbytes + out_s.nbytes + out_b.nbytes
    return {"value": round(rays / t / 1e9, 4), "unit": UNIT, "h2d_bytes_per_step": int(h2d),
            "d2h_bytes_per_step": int(d2h), "ms_per_step": round(t * 1e3, 3),
            "ms_mean": round(float(np.mean(times)) * 1e3, 3), "ms_min": round(float(np.min(times)) * 1e3, 3)}


# -------------------------------------------------------------- CPU baseline

class CpuBaseline:
    """The reference's algorithms on the host cores (the oracle port): median
    BVH build (constructBVHNew's partition + nth_element, one thread as the
    reference runs it), then every ray of the job through the collect-all
    division-slab traversal (boxIntersect) with Moller-Trumbore closest hit
    (primary, secondary) and any hit (shadow), rays in their own order split
    over all host threads in chunks of 256 consecutive rays.  One step = the
    build + all three ray classes: the whole job, nothing extrapolated."""

    def __init__(self, verts, idx, classes):
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle_py as O
        self.O = O
        self.cores = os.cpu_count() or 1
        self.prims, self.aabb, self.cen = O.tri_prims(verts, idx)
        self.n_tri = len(idx)
        self.classes = classes  # name -> (rays, query)
        self.rays = sum(len(r) for r, _ in classes.values())

    def build(self):
        # The reference's partition + nth_element median build; on meshes its
        # degenerate nodes (all centroids at or above the midpoint) would recurse
        # forever, so the oracle's rule (such a node becomes one leaf) is used.
        t0 = time.perf_counter()
        bvh = self.O.build_median(self.aabb, self.cen, compat=False)
        return bvh, time.perf_counter() - t0

    def step(self, threads=None, rows=None):
        """Build + trace; rows (optional): a contiguous slice of each class.
        Returns (total seconds, build seconds, {class: seconds})."""
        O = self.O
        bvh, tb = self.build()
        per = {}
        for k, (rays, q) in self.classes.items():
            r = rays if rows is None else rays[rows(len(rays))]
            t1 = time.perf_counter()
            O.trace_bvh2(O.TRIANGLES, O.REFERENCE, q, bvh, self.prims, r, nthreads=threads or self.cores)
            per[k] = time.perf_counter() - t1
        return tb + sum(per.values()), tb, per

    def record(self, total_s, build_s, per, one_core=True):
        out = {"value": self.rays / total_s / 1e9, "unit": UNIT, "cores": self.cores, "kind": "port",
               "sample": (f"full job: median-BVH build of all {self.n_tri} triangles (1 thread) + all "
                          f"{self.rays} rays (primary/secondary/shadow) through the reference's collect-all "
                          f"traversal on {self.cores} threads, rays in their own order"),
               "build_s": round(build_s, 3), "trace_s": {k: round(v, 3) for k, v in per.items()},
               "step_s": round(total_s, 3), "nproc": self.cores, "cpu_model": cpu_model()}
        if one_core:
            # One thread on a contiguous 1/64 of each class (pixel tiles in order),
            # scaled to the class; the build is the same single-threaded build.
            frac = 64

            def rows(n):
                a = n // 2
                return slice(a, a + max(1, n // frac))
            _, tb, part = self.step(threads=1, rows=rows)
            whole = build_s + sum(part[k] * len(self.classes[k][0]) / max(1, len(self.classes[k][0]) // frac)
                                  for k in part)
            out["one_core"] = {"value": self.rays / whole / 1e9,
                               "sample": f"1 thread, a contiguous 1/{frac} of each ray class from its middle, "
                                         "scaled to the class; build as above"}
        return out


def cpu_model():
    """The host CPU's model name (lscpu, else /proc/cpuinfo, else the machine type)."""
    import platform
    import subprocess
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.strip().startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith("model name"):
                    return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return platform.machine()


def cpu_baseline(verts, idx, primary, secondary, shadow):
    O_any, O_closest = 1, 0
    cb = CpuBaseline(verts, idx, {"primary": (primary, O_closest), "secondary": (secondary, O_closest),
                                  "shadow": (shadow, O_any)})
    return cb.record(*cb.step())


def run_reference(args):
    """The reference's CPU path on the host cores (the oracle port: the
    reference compiled from its sources needs its source tree, which only the
    build container has).  Secondary and shadow rays start at this arm's own
    primary hits (closest hit on its median BVH, equal to the GPU arm's hits:
    the closest hit does not depend on the tree), so the rays are the GPU
    arm's rays.  Every step is the whole job: build + all rays."""
    ws, rank, _ = dist_env()
    if ws > 1 and rank != 0:
        return
    verts, idx, primary = make_inputs()
    import scenes
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle_py as O
    prims, aabb, cen = O.tri_prims(verts, idx)
    bvh = O.build_median(aabb, cen)
    h = O.trace_bvh2(O.TRIANGLES, O.FAST, O.CLOSEST, bvh, prims, primary)
    secondary = scenes.cosine_rays(verts, idx, primary, h, seed=SEED + 2)
    shadow = scenes.shadow_rays(verts, idx, primary, h, LIGHT)
    counts = {"primary": len(primary), "secondary": len(secondary), "shadow": len(shadow)}
    cb = CpuBaseline(verts, idx, {"primary": (primary, O.CLOSEST), "secondary": (secondary, O.CLOSEST),
                                  "shadow": (shadow, O.ANY)})
    times, last = [], None
    for k in range(args.warmup + args.steps):
        last = cb.step()
        if k >= args.warmup:
            times.append(last[0])
    t = float(np.mean(times))
    rec = cb.record(t, last[1], last[2], one_core=False)
    v = rec["value"]
    out = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": ws,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(t * 1e3, 1), "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
           "config": {"workload": WORKLOAD, "dataStructure": "BVH (the reference's median builder)",
                      "triangles": len(idx), "primary_rays": counts["primary"],
                      "secondary_rays": counts["secondary"], "shadow_rays": counts["shadow"], "seed": SEED},
           "cpu_baseline": rec,
           "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def run_case(args):
    """Profiling driver (no bench line): one query class of the benchmark
    workload run warmup + steps times, for ncu captures of a single kernel.
    Cases: primary, secondary, shadow (the LBVH traversal kernels, with
    --ray-sort 0/1), build (the LBVH rebuild), build-bvh / build-kd (the median
    BVH and SAH KD rebuilds of the same mesh), batched (the many-structure
    persistent query on the many-scene workload, 32 scenes with --small),
    build-batched (the batched LBVH rebuild of the same scenes), render-c1
    (rq_render of the small plain workload: camera rays, shading, shadow
    rays, pixels), reference-render (rq_render_reference: the reference's
    sphere render with the REFERENCE walk), brute (RQ_NONE on C1's 64x48
    crop), serve (the serving loop's kernels: a few batched requests).
    --node-width 4/8 walks the wide copies for primary/secondary/shadow."""
    import torch
    import rq
    import scenes

    if args.case in ("render-c1", "reference-render", "brute", "serve"):
        run_case_render(args)
        return

    dev = torch.device("cuda", 0)
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    eng = rq.Engine(0)
    eng.set_stream(stream.cuda_stream)
    eng.configure(morton=rq.MORTON_SCENE_CUBE, lbvh_quality=args.lbvh_quality)  # the tuner's build choice (--no-tune)
    if args.case in ("batched", "build-batched"):
        meshes, ray_n, offs = c4_workload(32 if args.small else 256)
        sc = [eng.scene_triangles(v, f) for v, f in meshes]
        accs = eng.build_batched(sc, rq.LBVH)
        d_rays = batch_rays(torch, dev, meshes, ray_n.tolist(), SEED + 41)
        d_hits = torch.empty(int(offs[-1]) * HIT_BYTES, dtype=torch.uint8, device=dev)
        call = lambda: eng.trace_batched(accs, d_rays, offs, out=d_hits)  # noqa: E731
        if args.case == "build-batched":
            call = lambda: eng.rebuild_batched(accs)  # noqa: E731
    else:
        verts, idx, primary = make_inputs(args.small)
        scene = eng.scene_triangles(verts, idx)
        acc = eng.build(scene, rq.LBVH)
        hits_p = eng.trace_closest(acc, primary)
        if args.node_width != 2 and args.case in ("primary", "secondary", "shadow"):
            eng.configure(node_width=args.node_width)
            acc = eng.build(scene, rq.LBVH)
        if args.structure != "LBVH" and args.case in ("primary", "secondary", "shadow"):
            acc = eng.build(scene, args.structure)  # the same rays through another structure
        rays = {"primary": primary, "build": primary, "build-bvh": primary, "build-kd": primary,
                "secondary": scenes.cosine_rays(verts, idx, primary, hits_p, seed=SEED + 2),
                "shadow": scenes.shadow_rays(verts, idx, primary, hits_p, LIGHT)}[args.case]
        d_rays = torch.from_numpy(np.ascontiguousarray(rays).view(np.uint8)).to(dev)
        d_out = torch.empty(len(rays) * HIT_BYTES, dtype=torch.uint8, device=dev)
        eng.configure(ray_sort=args.ray_sort, scheduling=args.scheduling)
        if args.case == "build":
            call = acc.rebuild
        elif args.case in ("build-bvh", "build-kd"):
            other = eng.build(scene, rq.BVH if args.case == "build-bvh" else rq.KDTREE)
            call = other.rebuild
        elif args.case == "shadow":
            call = lambda: eng.trace_any(acc, d_rays, d_out)  # noqa: E731
        else:
            call = lambda: eng.trace_closest(acc, d_rays, d_out)  # noqa: E731
    for _ in range(args.warmup + args.steps):
        call()
    eng.synchronize()
    log(f"[bench] case {args.case}: {args.warmup + args.steps} launches done")
    eng.close()


def run_case_render(args):
    """The render-step and serving kernels for profiling (see run_case)."""
    import rq
    import scenes

    eng = rq.Engine(0)
    if args.case == "reference-render":
        sph = np.load(os.path.join(ROOT, "tests", "golden", "bunny.npz"))["spheres"]
        colors = np.tile(np.array([0.8, 0.7, 0.0], np.float32), (len(sph), 1))
        colors[-1] = 0.0
        acc = eng.build(eng.scene_spheres(sph), rq.BVH)
        eng.configure(traversal=rq.TRAVERSAL_REFERENCE)
        call = lambda: eng.render_reference(acc, surface_rgb=colors)  # noqa: E731
    elif args.case == "serve":
        srv = rq.Server(batching=True)
        meshes = scenes.mixed_meshes(8, 1e4, 2e5, SEED + 60, kinds=("icosphere",))
        for k, (v, f, _) in enumerate(meshes):
            srv.add_mesh(k, v, f)
        view = rq.make_view(eye=(2.7, 0.5, 0.9), target=(0.5, 0.5, 0.5), up=(0.0, 0.0, 1.0), fov_deg=45.0,
                            light=(1.5, -2.0, 3.0), albedo=(0.7, 0.65, 0.6), ambient=0.1, seed=7)

        def call():
            tickets = [srv.submit(k % 8, view, 640, 480, 2, keep_pixels=False) for k in range(16)]
            for t in tickets:
                srv.wait(t, want_pixels=False)
    else:
        v, f = scenes.c1_mesh()
        s = eng.scene_triangles(v, f)
        eng.configure(width=640, height=480, aa_samples=1)
        if args.case == "brute":
            acc = eng.build(s, rq.NONE)
            view = rq.make_view(window=(288, 216, 64, 48), **scenes.C1_VIEW)
        else:
            acc = eng.build(s, rq.LBVH)
            view = rq.make_view(**scenes.C1_VIEW)
        call = lambda: eng.render(acc, view)  # noqa: E731
    for _ in range(args.warmup + args.steps):
        call()
    eng.synchronize()
    log(f"[bench] case {args.case}: {args.warmup + args.steps} calls done")
    if args.case == "serve":
        srv.close()
    eng.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--skip-e2e", action="store_true")
    ap.add_argument("--small", action="store_true", help="960x540x4 rays (profiling case)")
    ap.add_argument("--skip-structures", action="store_true", help="skip the BVH / KDTREE comparison")
    ap.add_argument("--skip-render", action="store_true", help="skip the render-step legs")
    ap.add_argument("--skip-batch", action="store_true", help="skip the many-scene leg")
    ap.add_argument("--skip-serve", action="store_true", help="skip the serving-loop leg")
    ap.add_argument("--case", choices=["primary", "secondary", "shadow", "build", "build-bvh", "build-kd",
                                       "batched", "build-batched", "render-c1", "reference-render", "brute",
                                       "serve"],
                    help="profiling driver: run one query class, print no bench line")
    ap.add_argument("--structure", choices=["LBVH", "BVH", "KDTREE"], default="LBVH",
                    help="structure traced by --case primary/secondary/shadow")
    ap.add_argument("--ray-sort", type=int, default=0, help="ray reordering for --case")
    ap.add_argument("--node-width", type=int, default=2, choices=[2, 4, 8], help="--case: settings.node_width")
    ap.add_argument("--scheduling", type=int, default=0, help="--case: settings.scheduling (0-3)")
    ap.add_argument("--lbvh-quality", type=int, default=0, choices=[0, 1],
                    help="--case: settings.lbvh_quality (1: treelet restructuring)")
    ap.add_argument("--no-tune", action="store_true",
                    help="skip the autotuner and use its GB300 choice (binary nodes, cube Morton codes, "
                         "treelet restructuring, octant ray order for secondary rays): profiling the measured "
                         "kernel mix")
    args = ap.parse_args()
    if args.case:
        run_case(args)
        return
    if args.warmup < 3:
        log("[bench] warm-up raised to 3 steps")
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
