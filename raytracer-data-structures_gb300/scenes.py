"""Seeded synthetic inputs for the engine's workloads (numpy only).

Meshes
  icosphere(level)                 regular icosahedron subdivided `level` times
  displaced_icosphere(level, ...)  radial displacement by 3-octave value noise,
                                   scaled into the unit cube (plain small scene)
  heightfield(nx, ny, ...)         grid over [-1,1]^2, z = fBm value noise
                                   (LBVH build + incoherent traversal scene)
  merged_icospheres(...)           many displaced icospheres in one mesh (large scene)
Rays (rq_ray_t records, see rq.RAY_DTYPE)
  pinhole_rays(...)                jittered primary rays of a pinhole camera
  cosine_rays(...)                 cosine-weighted hemisphere rays from hit points
  shadow_rays(...)                 rays from hit points toward a point light
  incoherent_rays(...)             origins on a bounding sphere toward points in the box

Value noise: pseudo-random values on the integer lattice, blended with
smoothstep weights; fBm sums octaves with lacunarity 2 and gain 0.5.  Lattice
values come from a 32-bit integer hash of (ix, iy, iz, seed).
"""
import functools

import numpy as np

from rq import RAY_DTYPE, MISS

# ------------------------------------------------------------------- noise

_M = np.uint32(0x27D4EB2D)


def _hash3(ix, iy, iz, seed):
    with np.errstate(over="ignore"):
        h = (ix.astype(np.uint32) * np.uint32(0x8DA6B343)) ^ (iy.astype(np.uint32) * np.uint32(0xD8163841)) \
            ^ (iz.astype(np.uint32) * np.uint32(0xCB1AB31F)) ^ np.uint32(seed * 0x9E3779B1 & 0xFFFFFFFF)
        h = (h ^ (h >> np.uint32(15))) * _M
        h = (h ^ (h >> np.uint32(13))) * np.uint32(0x85EBCA6B)
        h = h ^ (h >> np.uint32(16))
    return h.astype(np.float64) / 4294967295.0 * 2.0 - 1.0  # [-1, 1]


def _smooth(t):
    return t * t * (3.0 - 2.0 * t)


def value_noise3(p, seed):
    """Trilinear smoothstep blend of lattice values; p: (n, 3) float64."""
    f = np.floor(p)
    i = f.astype(np.int64)
    w = _smooth(p - f)
    out = np.zeros(len(p))
    for dx in (0, 1):
        for dy in (0, 1):
            for dz in (0, 1):
                v = _hash3(i[:, 0] + dx, i[:, 1] + dy, i[:, 2] + dz, seed)
                wx = w[:, 0] if dx else 1 - w[:, 0]
                wy = w[:, 1] if dy else 1 - w[:, 1]
                wz = w[:, 2] if dz else 1 - w[:, 2]
                out += v * wx * wy * wz
    return out


def fbm3(p, octaves, seed, base_freq=1.0):
    out = np.zeros(len(p))
    amp, freq, norm = 1.0, base_freq, 0.0
    for o in range(octaves):
        out += amp * value_noise3(p * freq, seed + 101 * o)
        norm += amp
        amp *= 0.5
        freq *= 2.0
    return out / norm


# ------------------------------------------------------------------ meshes

@functools.lru_cache(maxsize=None)
def icosphere(level):
    """Unit icosphere subdivided `level` times: 20 * 4^level triangles.  Cached
    per level; the arrays are read-only (callers derive new arrays from them)."""
    v, f = _icosphere(level)
    v.flags.writeable = False
    f.flags.writeable = False
    return v, f


def _icosphere(level):
    t = (1.0 + 5 ** 0.5) / 2.0
    v = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t], [0, -1, -t],
                  [0, 1, -t], [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], np.float64)
    f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4],
                  [11, 10, 2], [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8],
                  [3, 8, 9], [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], np.int64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    for _ in range(level):
        nv = len(v)
        e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]])
        e.sort(axis=1)
        key = e[:, 0] * nv + e[:, 1]
        uk, inv = np.unique(key, return_inverse=True)
        a, b = uk // nv, uk % nv
        mid = v[a] + v[b]
        mid /= np.linalg.norm(mid, axis=1, keepdims=True)
        m = (nv + inv).reshape(3, -1)
        m01, m12, m20 = m[0], m[1], m[2]
        v = np.concatenate([v, mid])
        f = np.concatenate([np.stack([f[:, 0], m01, m20], 1), np.stack([f[:, 1], m12, m01], 1),
                            np.stack([f[:, 2], m20, m12], 1), np.stack([m01, m12, m20], 1)])
    return v, f


def displaced_icosphere(level=6, amplitude=0.15, octaves=3, seed=1, unit_cube=True):
    v, f = icosphere(level)
    n = fbm3(v * 2.0, octaves, seed)
    v = v * (1.0 + amplitude * n)[:, None]
    if unit_cube:
        lo = v.min(0)
        v = (v - lo) / (v.max(0) - lo).max()
    return v.astype(np.float32), f.astype(np.uint32)


def wave_heightfield(nx, ny, seed=0, size=1.0):
    """A cheap seeded terrain for many-scene batches: an nx x ny vertex grid
    over [-size, size]^2, z = a sum of four products of sines with seeded
    frequencies and phases; 2 (nx - 1)(ny - 1) triangles."""
    rng = np.random.default_rng(seed)
    x = np.linspace(-size, size, nx, dtype=np.float32)
    y = np.linspace(-size, size, ny, dtype=np.float32)
    X, Y = np.meshgrid(x, y, indexing="xy")
    Z = np.zeros_like(X)
    for _ in range(4):
        a, fx, fy, px, py = rng.uniform([0.02, 1, 1, 0, 0], [0.15, 9, 9, 6.3, 6.3])
        Z += np.float32(a) * np.sin(np.float32(fx) * X + np.float32(px)) * np.cos(np.float32(fy) * Y + np.float32(py))
    v = np.stack([X.ravel(), Y.ravel(), Z.ravel()], 1).astype(np.float32)
    i = np.arange(nx * ny, dtype=np.uint32).reshape(ny, nx)
    a, b, c, d = i[:-1, :-1].ravel(), i[:-1, 1:].ravel(), i[1:, :-1].ravel(), i[1:, 1:].ravel()
    f = np.concatenate([np.stack([a, b, d], 1), np.stack([a, d, c], 1)]).astype(np.uint32)
    return v, f


def c1_mesh(seed=1):
    """The small plain workload's mesh: 81,920-triangle displaced icosphere
    (level 6, 3-octave value noise, amplitude 0.15) scaled into the unit cube
    and centred on the origin."""
    v, f = displaced_icosphere(6, seed=seed)
    v = v - (v.min(0) + v.max(0)) / 2
    return v.astype(np.float32), f


# The small plain workload's view: 640x480, 1 spp, pinhole at (0, 0, 3)
# looking at the origin, 40 degree vertical field of view, one point light,
# Lambert shading with one shadow ray, white background.
C1_VIEW = dict(eye=(0.0, 0.0, 3.0), target=(0.0, 0.0, 0.0), up=(0.0, 1.0, 0.0), fov_deg=40.0,
               light=(2.0, 3.0, 4.0), albedo=(0.8, 0.75, 0.7), ambient=0.1, mirror=0.0, bounces=0, seed=11)


# The large workload's view of merged_icospheres() (150 displaced icospheres
# in [-4, 4]^3): 3840x2160, 4 spp, one shadow ray per hit and two mirror
# bounces.
C3_VIEW = dict(eye=(0.0, -12.0, 5.0), target=(0.0, 0.0, 0.0), up=(0.0, 0.0, 1.0), fov_deg=50.0,
               light=(6.0, -8.0, 10.0), albedo=(0.75, 0.7, 0.65), ambient=0.05, mirror=0.5, bounces=2, seed=33)


def heightfield(nx=1001, ny=500, amplitude=0.3, octaves=5, seed=2):
    """(nx-1)*(ny-1)*2 triangles; 1001 x 500 gives 998,000."""
    x = np.linspace(-1.0, 1.0, nx)
    y = np.linspace(-1.0, 1.0, ny)
    X, Y = np.meshgrid(x, y, indexing="xy")
    p = np.stack([X.ravel() * 2.0, Y.ravel() * 2.0, np.zeros(X.size)], 1)
    z = amplitude * fbm3(p, octaves, seed)
    verts = np.stack([X.ravel(), Y.ravel(), z], 1).astype(np.float32)
    i = np.arange(ny - 1)[:, None] * nx + np.arange(nx - 1)[None, :]
    i = i.ravel()
    a, b, c, d = i, i + 1, i + nx, i + nx + 1
    f = np.concatenate([np.stack([a, b, d], 1), np.stack([a, d, c], 1)]).astype(np.uint32)
    return verts, f


def mixed_meshes(n, tri_lo, tri_hi, seed, kinds=("icosphere", "heightfield")):
    """n seeded meshes whose target triangle counts are log-uniform in
    [tri_lo, tri_hi]; each is, by seed, a displaced icosphere (3-octave value
    noise, amplitude 0.15, in the unit cube; the subdivision level nearest the
    target on a log scale, so counts are 20 * 4^level) or an fBm heightfield
    (5 octaves, amplitude 0.3; a square vertex grid of about the target
    count).  Returns [(verts, idx, kind)]; callers record the actual counts."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n):
        t = float(np.exp(rng.uniform(np.log(tri_lo), np.log(tri_hi))))
        kind = kinds[int(rng.integers(len(kinds)))]
        if kind == "icosphere":
            level = int(np.clip(np.round(np.log(t / 20.0) / np.log(4.0)), 2, 8))
            v, f = displaced_icosphere(level, seed=seed + 1000 + k)
        else:
            nx = max(2, int(round(np.sqrt(t / 2.0)))) + 1
            v, f = heightfield(nx, nx, amplitude=0.3, octaves=5, seed=seed + 1000 + k)
        out.append((v, f, kind))
    return out


def chain_clusters(grid=16, group=32, levels=30):
    """Sphere centres (float32, (grid*grid*levels*group, 3)): grid x grid
    cells, each holding `levels` groups of `group` coincident points at
    offsets of 1/2, 1/4, ... of the cell along x, y, z in turn.  Each cell's
    Morton tree is a caterpillar that peels one group per bit level, so the
    LBVH has far more large nodes than a balanced tree of the same size."""
    pts = []
    cell = 1.0 / grid
    for cx in range(grid):
        for cy in range(grid):
            for k in range(levels):
                p = np.array([cx * cell, cy * cell, 0.0])
                p[k % 3] += cell * 2.0 ** -(k // 3 + 1)
                pts.append(np.repeat(p[None], group, 0))
    return np.concatenate(pts).astype(np.float32)


def merged_icospheres(count=150, target_tris=10_000_000, seed=3, levels=(5, 6, 7)):
    """Many displaced icospheres merged into one mesh; subdivision levels are
    drawn by seed so the total lands near target_tris (the count is recorded
    by the caller)."""
    rng = np.random.default_rng(seed)
    per = {lv: 20 * 4 ** lv for lv in levels}
    chosen = []
    remaining = target_tris
    for k in range(count):
        left = count - k
        want = remaining / left
        lv = min(levels, key=lambda L: abs(per[L] - want))
        if rng.random() < 0.3:
            lv = int(rng.choice(levels))
        chosen.append(lv)
        remaining -= per[lv]
    cache = {lv: icosphere(lv) for lv in set(chosen)}
    vs, fs, off = [], [], 0
    for k, lv in enumerate(chosen):
        v, f = cache[lv]
        r = rng.uniform(0.05, 0.3)
        c = rng.uniform(-4.0, 4.0, 3)
        n = fbm3(v * 2.0 + k * 17.0, 3, seed + k)
        vv = v * (1.0 + 0.15 * n)[:, None] * r + c
        vs.append(vv.astype(np.float32))
        fs.append((f + off).astype(np.uint32))
        off += len(v)
    return np.concatenate(vs), np.concatenate(fs), chosen


# -------------------------------------------------------------------- rays

def _rays(org, dirs, tmin=0.0, tmax=np.inf):
    r = np.zeros(len(dirs), RAY_DTYPE)
    r["org"] = org
    r["dir"] = dirs
    r["tmin"] = tmin
    r["tmax"] = tmax
    return r


def pinhole_rays(width, height, spp, eye, target, up=(0, 0, 1), fov_deg=40.0, seed=4):
    """Jittered primary rays, pixel-major then sample order."""
    rng = np.random.default_rng(seed)
    eye = np.asarray(eye, np.float64)
    w = np.asarray(target, np.float64) - eye
    w /= np.linalg.norm(w)
    u = np.cross(w, np.asarray(up, np.float64))
    u /= np.linalg.norm(u)
    v = np.cross(u, w)
    th = np.tan(np.radians(fov_deg) / 2)
    aspect = width / height
    n = width * height * spp
    pix = np.arange(n) // spp
    px = (pix % width).astype(np.float64) + rng.random(n)
    py = (pix // width).astype(np.float64) + rng.random(n)
    sx = (2 * px / width - 1) * th * aspect
    sy = (1 - 2 * py / height) * th
    d = w[None, :] + sx[:, None] * u[None, :] + sy[:, None] * v[None, :]
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return _rays(eye.astype(np.float32), d.astype(np.float32))


def tri_normals(verts, idx, prim):
    a = verts[idx[prim, 0]].astype(np.float64)
    b = verts[idx[prim, 1]].astype(np.float64)
    c = verts[idx[prim, 2]].astype(np.float64)
    n = np.cross(b - a, c - a)
    return n / np.maximum(np.linalg.norm(n, axis=1, keepdims=True), 1e-30)


def hit_points(rays, hits):
    m = hits["prim"] != MISS
    p = rays["org"][m].astype(np.float64) + rays["dir"][m].astype(np.float64) * hits["t"][m, None]
    return m, p


def cosine_rays(verts, idx, rays, hits, seed=5, bias=1e-4):
    """One cosine-weighted hemisphere ray per primary hit, around the
    geometric normal facing the incoming ray."""
    rng = np.random.default_rng(seed)
    m, p = hit_points(rays, hits)
    n = tri_normals(verts, idx, hits["prim"][m].astype(np.int64))
    flip = np.sum(n * rays["dir"][m], axis=1) > 0
    n[flip] *= -1
    k = len(p)
    r1, r2 = rng.random(k), rng.random(k)
    phi = 2 * np.pi * r1
    sr = np.sqrt(r2)
    local = np.stack([np.cos(phi) * sr, np.sin(phi) * sr, np.sqrt(1 - r2)], 1)
    a = np.where(np.abs(n[:, 0:1]) > 0.9, np.array([[0.0, 1.0, 0.0]]), np.array([[1.0, 0.0, 0.0]]))
    t1 = np.cross(n, a)
    t1 /= np.linalg.norm(t1, axis=1, keepdims=True)
    t2 = np.cross(n, t1)
    d = local[:, 0:1] * t1 + local[:, 1:2] * t2 + local[:, 2:3] * n
    return _rays((p + bias * n).astype(np.float32), d.astype(np.float32))


def shadow_rays(verts, idx, rays, hits, light, bias=1e-4):
    m, p = hit_points(rays, hits)
    n = tri_normals(verts, idx, hits["prim"][m].astype(np.int64))
    flip = np.sum(n * rays["dir"][m], axis=1) > 0
    n[flip] *= -1
    o = p + bias * n
    d = np.asarray(light, np.float64)[None, :] - o
    dist = np.linalg.norm(d, axis=1)
    return _rays(o.astype(np.float32), (d / dist[:, None]).astype(np.float32), 0.0, dist.astype(np.float32))


def incoherent_rays(lo, hi, n, seed=6):
    rng = np.random.default_rng(seed)
    lo, hi = np.asarray(lo, np.float64), np.asarray(hi, np.float64)
    c = (lo + hi) / 2
    R = np.linalg.norm(hi - lo) / 2 * 1.05
    s = rng.normal(size=(n, 3))
    s /= np.linalg.norm(s, axis=1, keepdims=True)
    o = c + R * s
    t = lo + rng.random((n, 3)) * (hi - lo)
    d = t - o
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return _rays(o.astype(np.float32), d.astype(np.float32))
