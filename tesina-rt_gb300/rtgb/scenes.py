"""Seeded synthetic scenes for the Whitted-ray-tracer workloads.

The reference's own benchmark scenes are OBJ files that are not part of its
repository; these generators stand in for them with the shapes, sizes and
value distributions of the five workloads:

- ``soup``: random triangle soup (10,000 triangles, centroids U[-1,1]^3,
  vertex offsets N(0, 0.03) per axis, 20% mirrors with reflectance 0.5, the
  rest Lambertian with albedo U[0.2, 0.9]^3, one point light at (0, 4, -2)).
- ``terrain``: an fBm value-noise heightfield (4 octaves, amplitude 1,
  lacunarity 2, gain 0.5) with mirror UV spheres (32 x 16 segments, 960
  triangles each) scattered above it; heights animated per frame by
  0.1 * sin(x + t) with t = 0.1 * frame.

All geometry is float32; the vertex normal of a soup triangle is its face
normal, terrain normals come from central differences of the height field,
sphere normals are radial.
"""
import math

import numpy as np

from . import abi

MAT_MIRROR_SOUP = dict(diffuse=(0.0, 0.0, 0.0), reflectiveness=0.5)


class Scene:
    """Host scene in the C ABI's data model (see rt_scene_desc)."""

    def __init__(self, pos4, nrm4, idx, mats, mat_map, lights):
        self.pos4 = np.ascontiguousarray(pos4, dtype=np.float32)
        self.nrm4 = np.ascontiguousarray(nrm4, dtype=np.float32)
        self.idx = np.ascontiguousarray(idx, dtype=np.uint32).reshape(-1, 3)
        self.mats = np.ascontiguousarray(mats)
        self.mat_map = np.ascontiguousarray(mat_map, dtype=np.uint32)
        self.lights = lights
        assert self.mats.dtype == abi.MATERIAL_DTYPE
        assert self.pos4.shape == self.nrm4.shape and self.pos4.shape[1] == 4
        assert self.mat_map.shape[0] == self.idx.shape[0]

    @property
    def n_tris(self):
        return self.idx.shape[0]

    @property
    def n_verts(self):
        return self.pos4.shape[0]


def _materials(n):
    m = np.zeros(n, dtype=abi.MATERIAL_DTYPE)
    m["texture"] = -1
    return m


def _normalize(v):
    v = v.astype(np.float32)
    n = np.sqrt((v * v).sum(axis=-1, keepdims=True)).astype(np.float32)
    n[n == 0] = 1
    return (v / n).astype(np.float32)


def _f4(v3):
    out = np.zeros((v3.shape[0], 4), dtype=np.float32)
    out[:, :3] = v3
    return out


def soup(n_tris=10000, seed=0, mirror_frac=0.2, offset_sigma=0.03,
         light_pos=(0.0, 4.0, -2.0), ambient=0.1):
    """Random triangle soup (the small plain workload and the batched scenes)."""
    rng = np.random.default_rng(seed)
    c = rng.uniform(-1.0, 1.0, size=(n_tris, 1, 3)).astype(np.float32)
    off = rng.normal(0.0, offset_sigma, size=(n_tris, 3, 3)).astype(np.float32)
    v = (c + off).astype(np.float32)                         # (N, 3 verts, 3)
    fn = _normalize(np.cross(v[:, 1] - v[:, 0], v[:, 2] - v[:, 0]))
    pos = _f4(v.reshape(-1, 3))
    nrm = _f4(np.repeat(fn, 3, axis=0))
    idx = np.arange(3 * n_tris, dtype=np.uint32).reshape(-1, 3)
    mirror = rng.random(n_tris) < mirror_frac
    albedo = rng.uniform(0.2, 0.9, size=(n_tris, 3)).astype(np.float32)
    mats = _materials(n_tris + 1)
    mats["reflectiveness"][0] = MAT_MIRROR_SOUP["reflectiveness"]
    mats["diffuse"][1:, :3] = albedo
    mat_map = np.where(mirror, 0, np.arange(1, n_tris + 1)).astype(np.uint32)
    lights = abi.make_lights((ambient,) * 3, [dict(type=abi.RT_POINT_L, pos=light_pos,
                                                   color=(1.0, 1.0, 1.0))])
    return Scene(pos, nrm, idx, mats, mat_map, lights)


def with_glass(sc, frac=0.3, index=1.333, reflectiveness=0.9, seed=0):
    """A copy of sc in which a fraction of the triangles take a refracting
    material (the reference's scenes use refractive_index 1.333): one extra
    material, diffuse 0.1, reflectiveness splitting the light between the
    reflected and the refracted ray by Schlick's factor."""
    rng = np.random.default_rng(seed)
    mats = np.concatenate([sc.mats, _materials(1)])
    g = mats.shape[0] - 1
    mats["diffuse"][g, :3] = 0.1
    mats["reflectiveness"][g] = reflectiveness
    mats["refractive_index"][g] = index
    mat_map = sc.mat_map.copy()
    mat_map[rng.random(sc.n_tris) < frac] = g
    return Scene(sc.pos4, sc.nrm4, sc.idx, mats, mat_map, sc.lights)


# ---------------------------------------------------------------------------
# value-noise fBm
# ---------------------------------------------------------------------------
def _hash(ix, iz, octave, seed):
    """32-bit integer hash of a lattice point -> float32 in [-1, 1)."""
    h = (ix.astype(np.uint32) * np.uint32(0x8DA6B343)) ^ \
        (iz.astype(np.uint32) * np.uint32(0xD8163841)) ^ \
        np.uint32((octave * 0x2545F491 + seed * 0x9E3779B9) & 0xFFFFFFFF)
    h ^= h >> np.uint32(16)
    h *= np.uint32(0x7FEB352D)
    h ^= h >> np.uint32(15)
    h *= np.uint32(0x846CA68B)
    h ^= h >> np.uint32(16)
    return (h >> np.uint32(8)).astype(np.float32) * np.float32(2.0 / (1 << 24)) - np.float32(1.0)


def _value_noise(x, z, octave, seed):
    fx, fz = np.floor(x), np.floor(z)
    ix, iz = fx.astype(np.int64), fz.astype(np.int64)
    tx, tz = (x - fx).astype(np.float32), (z - fz).astype(np.float32)
    sx = tx * tx * (3 - 2 * tx)
    sz = tz * tz * (3 - 2 * tz)
    a = _hash(ix, iz, octave, seed)
    b = _hash(ix + 1, iz, octave, seed)
    c = _hash(ix, iz + 1, octave, seed)
    d = _hash(ix + 1, iz + 1, octave, seed)
    return (a + (b - a) * sx) * (1 - sz) + (c + (d - c) * sx) * sz


def fbm(x, z, seed=0, octaves=4, amplitude=1.0, lacunarity=2.0, gain=0.5, base_freq=0.5):
    """fBm of value noise; base_freq lattice cells per unit (documented choice)."""
    h = np.zeros(np.broadcast(x, z).shape, dtype=np.float32)
    amp, freq = amplitude, base_freq
    for o in range(octaves):
        h += np.float32(amp) * _value_noise(x * freq, z * freq, o, seed)
        amp *= gain
        freq *= lacunarity
    return h.astype(np.float32)


def _uv_sphere(center, radius, seg=32, rings=16):
    """UV sphere without degenerate pole triangles: seg*(2*(rings-1)) tris."""
    cx, cy, cz = center
    verts = [(0.0, 1.0, 0.0)]
    for r in range(1, rings):
        th = math.pi * r / rings
        for s in range(seg):
            ph = 2 * math.pi * s / seg
            verts.append((math.sin(th) * math.cos(ph), math.cos(th), math.sin(th) * math.sin(ph)))
    verts.append((0.0, -1.0, 0.0))
    unit = np.array(verts, dtype=np.float32)
    tris = []
    for s in range(seg):                                   # top cap
        tris.append((0, 1 + s, 1 + (s + 1) % seg))
    for r in range(rings - 2):                             # bands
        a0, b0 = 1 + r * seg, 1 + (r + 1) * seg
        for s in range(seg):
            s1 = (s + 1) % seg
            tris.append((a0 + s, b0 + s, b0 + s1))
            tris.append((a0 + s, b0 + s1, a0 + s1))
    last = len(verts) - 1                                  # bottom cap
    base = 1 + (rings - 2) * seg
    for s in range(seg):
        tris.append((base + s, last, base + (s + 1) % seg))
    pos = (unit * np.float32(radius) + np.array(center, dtype=np.float32)).astype(np.float32)
    return pos, unit, np.array(tris, dtype=np.uint32)


SPHERE_TEMPLATE = {}


def _sphere_template(seg, rings):
    key = (seg, rings)
    if key not in SPHERE_TEMPLATE:
        _, unit, tris = _uv_sphere((0, 0, 0), 1.0, seg, rings)
        SPHERE_TEMPLATE[key] = (unit, tris)
    return SPHERE_TEMPLATE[key]


class Terrain:
    """fBm heightfield plus mirror spheres; ``frame(f)`` gives animated vertices."""

    def __init__(self, nx=1024, nz=512, extent=(-8.0, 8.0, -4.0, 4.0), n_spheres=200,
                 seed=1, lights=None, ambient=0.1, sphere_seg=(32, 16)):
        self.nx, self.nz = nx, nz
        x0, x1, z0, z1 = extent
        xs = np.linspace(x0, x1, nx + 1, dtype=np.float32)
        zs = np.linspace(z0, z1, nz + 1, dtype=np.float32)
        self.gx, self.gz = np.meshgrid(xs, zs)               # (nz+1, nx+1)
        self.h0 = fbm(self.gx, self.gz, seed=seed)
        self.dx = (x1 - x0) / nx
        self.dz = (z1 - z0) / nz
        # grid triangles, 2 per cell
        j, i = np.meshgrid(np.arange(nz, dtype=np.uint32), np.arange(nx, dtype=np.uint32),
                           indexing="ij")
        v00 = (j * (nx + 1) + i).ravel()
        v10 = v00 + 1
        v01 = v00 + (nx + 1)
        v11 = v01 + 1
        grid_tris = np.empty((2 * nx * nz, 3), dtype=np.uint32)
        grid_tris[0::2] = np.stack([v00, v10, v11], axis=1)
        grid_tris[1::2] = np.stack([v00, v11, v01], axis=1)
        self.n_grid_verts = (nx + 1) * (nz + 1)
        # spheres
        rng = np.random.default_rng(seed + 1000)
        unit, stris = _sphere_template(*sphere_seg)
        radii = rng.uniform(0.1, 0.5, n_spheres).astype(np.float32)
        cx = rng.uniform(x0 + 0.5, x1 - 0.5, n_spheres).astype(np.float32)
        cz = rng.uniform(z0 + 0.5, z1 - 0.5, n_spheres).astype(np.float32)
        lift = rng.uniform(0.2, 1.0, n_spheres).astype(np.float32)
        cy = fbm(cx, cz, seed=seed) + radii + np.float32(0.1) + lift
        centers = np.stack([cx, cy, cz], axis=1).astype(np.float32)
        nv = unit.shape[0]
        sp_pos = (unit[None] * radii[:, None, None] + centers[:, None, :]).reshape(-1, 3)
        sp_nrm = np.broadcast_to(unit[None], (n_spheres, nv, 3)).reshape(-1, 3)
        sp_tris = (stris[None] + (self.n_grid_verts + nv * np.arange(n_spheres,
                                                                    dtype=np.uint32))[:, None, None])
        self.sp_pos = _f4(sp_pos.astype(np.float32))
        self.sp_nrm = _f4(sp_nrm.astype(np.float32))
        self.idx = np.concatenate([grid_tris, sp_tris.reshape(-1, 3)]).astype(np.uint32)
        n_grid_tris = grid_tris.shape[0]
        mats = _materials(2)
        mats["diffuse"][0, :3] = (0.55, 0.5, 0.4)          # terrain, Lambertian
        mats["diffuse"][1, :3] = (0.1, 0.1, 0.1)           # mirror spheres
        mats["reflectiveness"][1] = 0.8
        self.mats = mats
        self.mat_map = np.concatenate([np.zeros(n_grid_tris, np.uint32),
                                       np.ones(self.idx.shape[0] - n_grid_tris, np.uint32)])
        if lights is None:
            lights = [dict(type=abi.RT_POINT_L, pos=(-4.0, 6.0, -3.0), color=(0.7, 0.7, 0.7)),
                      dict(type=abi.RT_POINT_L, pos=(5.0, 5.0, 2.0), color=(0.5, 0.5, 0.6))]
        self.lights = abi.make_lights((ambient,) * 3, lights)

    @property
    def n_tris(self):
        return self.idx.shape[0]

    def heights(self, f):
        t = np.float32(0.1 * f)
        return (self.h0 + np.float32(0.1) * np.sin(self.gx + t)).astype(np.float32)

    def frame_vertices(self, f):
        """(pos4, nrm4) of frame f: terrain heights animated, spheres fixed."""
        h = self.heights(f)
        gxs = np.gradient(h, self.dx, axis=1).astype(np.float32)
        gzs = np.gradient(h, self.dz, axis=0).astype(np.float32)
        n = _normalize(np.stack([-gxs, np.ones_like(h), -gzs], axis=-1).reshape(-1, 3))
        gp = np.stack([self.gx, h, self.gz], axis=-1).reshape(-1, 3)
        pos = np.concatenate([_f4(gp), self.sp_pos])
        nrm = np.concatenate([_f4(n), self.sp_nrm])
        return pos, nrm

    def scene(self, f=0):
        pos, nrm = self.frame_vertices(f)
        return Scene(pos, nrm, self.idx, self.mats, self.mat_map, self.lights)


def camera(pos, target, up=(0.0, 1.0, 0.0), fov_deg=60.0, aspect=1.0, right_handed=False):
    """Camera::set (src/rt/camera.cpp:31-59) in float32: returns abi.Camera."""
    f32 = np.float32
    p = np.array(pos, dtype=f32)
    d = np.array(target, dtype=f32) - p
    d = (d / np.sqrt(f32((d * d).sum()))).astype(f32)
    u = np.array(up, dtype=f32)
    right = np.cross(d, u) if right_handed else np.cross(u, d)
    upv = np.cross(right, d) if right_handed else np.cross(d, right)
    ph = f32(math.tan(math.radians(fov_deg) * 0.5))
    right = (right * (ph * f32(aspect)) / np.sqrt(f32((right * right).sum()))).astype(f32)
    upv = (upv * ph / np.sqrt(f32((upv * upv).sum()))).astype(f32)
    cam = abi.Camera()
    cam.pos[:3] = [float(v) for v in p]
    cam.dir[:3] = [float(v) for v in d]
    cam.right[:3] = [float(v) for v in right]
    cam.up[:3] = [float(v) for v in upv]
    return cam


# ---------------------------------------------------------------------------
# named workloads
# ---------------------------------------------------------------------------
def workload_small(seed=0):
    """Plain method, small: 10k-triangle soup, 512x512, depth 3, 1 point light."""
    sc = soup(10000, seed=seed)
    cam = camera((0.0, 0.0, -4.0), (0.0, 0.0, 0.0), fov_deg=60.0, aspect=1.0)
    return dict(name="soup10k_512x512_d3", scene=sc, camera=cam, width=512, height=512,
                max_bounces=3, depth=30, min_leaf=1)


def workload_mid(seed=1):
    """Plain method, mid scale: 1024x512-cell fBm field + 200 mirror spheres,
    1920x1080, 2 point lights, depth 4, full LBVH rebuild per frame."""
    ter = Terrain(1024, 512, n_spheres=200, seed=seed)
    cam = camera((0.0, 9.0, -2.5), (0.0, 0.0, 2.0), fov_deg=60.0, aspect=1920 / 1080)
    return dict(name="terrain1M_1920x1080_d4", terrain=ter, camera=cam, width=1920,
                height=1080, max_bounces=4, depth=30, min_leaf=1)


def workload_stress(seed=2):
    """Plain method, stress: 4096x2048-cell field + 1000 spheres, 3840x2160,
    3 point lights, depth 6, 8 camera poses on a radius-10 sphere."""
    lights = [dict(type=abi.RT_POINT_L, pos=(-4.0, 6.0, -3.0), color=(0.6, 0.6, 0.6)),
              dict(type=abi.RT_POINT_L, pos=(5.0, 5.0, 2.0), color=(0.4, 0.4, 0.5)),
              dict(type=abi.RT_POINT_L, pos=(0.0, 8.0, 6.0), color=(0.3, 0.3, 0.3))]
    ter = Terrain(4096, 2048, n_spheres=1000, seed=seed, lights=lights)
    rng = np.random.default_rng(seed + 7)
    poses = []
    for _ in range(8):
        v = rng.normal(size=3)
        v[1] = abs(v[1]) + 0.2          # above the field
        v = v / np.linalg.norm(v) * 10.0
        poses.append(camera(tuple(v), (0.0, 0.0, 0.0), fov_deg=60.0, aspect=3840 / 2160))
    return dict(name="terrain17M_3840x2160_d6", terrain=ter, cameras=poses, width=3840,
                height=2160, max_bounces=6, depth=30, min_leaf=1)


def workload_batched(seed=3, count=64):
    """Batched: 64 triangle soups (as the small workload) with triangle counts
    log-uniform in [1k, 500k], resolutions from {256x256, 512x512, 1024x768},
    reflection depth uniform in 1..4."""
    rng = np.random.default_rng(seed)
    items = []
    res = [(256, 256), (512, 512), (1024, 768)]
    for k in range(count):
        n = int(round(math.exp(rng.uniform(math.log(1000), math.log(500000)))))
        w, h = res[int(rng.integers(0, 3))]
        depth = int(rng.integers(1, 5))
        sc = soup(n, seed=seed * 1000 + k)
        cam = camera((0.0, 0.0, -4.0), (0.0, 0.0, 0.0), fov_deg=60.0, aspect=w / h)
        items.append(dict(scene=sc, camera=cam, width=w, height=h, max_bounces=depth))
    return dict(name="soups64_1k-500k_mixed-res", items=items)


def transform(rot_y_deg=0.0, scale=(1.0, 1.0, 1.0), t=(0.0, 0.0, 0.0)):
    """Row-major 4x4 object-to-world matrix (rotation about y, then scale and
    translation) and its inverse, both float32 (inverse taken in float64)."""
    a = math.radians(rot_y_deg)
    r = np.array([[math.cos(a), 0, math.sin(a)], [0, 1, 0], [-math.sin(a), 0, math.cos(a)]])
    m = np.eye(4)
    m[:3, :3] = r @ np.diag(scale)
    m[:3, 3] = t
    return m.astype(np.float32), np.linalg.inv(m).astype(np.float32)


def workload_instances(seed=6):
    """Multi-root (instanced) scene: one mesh per object, as the reference's
    per-object BVHs.  A 256x128-cell fBm tile with 20 mirror spheres (≈86k
    triangles) placed 2x2 as the ground, and a 50k-triangle soup placed 12
    times above it with random turns and scales: 16 roots, 2 meshes.
    1920x1080, depth 4, the tile's two point lights."""
    rng = np.random.default_rng(seed)
    tile = Terrain(256, 128, n_spheres=20, seed=seed)
    blob = soup(50000, seed=seed + 1)
    inst, ms, mis = [], [], []
    for ix in (-1, 1):
        for iz in (-1, 1):
            m, mi = transform(t=(8.0 * ix, 0.0, 4.0 * iz))
            inst.append(0), ms.append(m), mis.append(mi)
    for _ in range(12):
        s = float(rng.uniform(0.4, 1.0))
        m, mi = transform(float(rng.uniform(0, 360)), (s, s, s),
                          (float(rng.uniform(-12, 12)), float(rng.uniform(2.0, 4.0)),
                           float(rng.uniform(-6, 6))))
        inst.append(1), ms.append(m), mis.append(mi)
    cam = camera((0.0, 12.0, -16.0), (0.0, 0.0, 0.0), fov_deg=60.0, aspect=1920 / 1080)
    return dict(name="instances16_tile86k+soup50k_1920x1080_d4",
                meshes=[tile.scene(0), blob], inst=np.array(inst, np.int32),
                tr=np.array(ms), tr_inv=np.array(mis), lights=tile.lights, camera=cam,
                width=1920, height=1080, max_bounces=4)


def _served_scene(kind, n, seed):
    """One scene of the served pool: a soup of n triangles, or an fBm field of
    about n triangles (2 per cell, cells 2:1) over [-2,2]x[-1,1] with 16 mirror
    spheres (16x8 segments)."""
    if kind == "soup":
        return soup(n, seed=seed)
    nz = max(2, int(round(math.sqrt(max(n - 16 * 256, 8) / 4.0))))
    ter = Terrain(2 * nz, nz, extent=(-2.0, 2.0, -1.0, 1.0), n_spheres=16, seed=seed,
                  sphere_seg=(16, 8))
    return ter.scene(0)


def workload_served(seed=5, pool=32, uploads=8, n_min=10_000, n_max=2_000_000):
    """Served: a pool of resident scenes (soups and fBm fields alternating,
    triangle counts log-uniform in [n_min, n_max]) and a set of scenes that
    upload requests bring in.  Scenes are described here and made on demand
    (``make``), so that a caller holds only what it uploads."""
    rng = np.random.default_rng(seed)

    def spec(k, base):
        n = int(round(math.exp(rng.uniform(math.log(n_min), math.log(n_max)))))
        return ("soup" if k % 2 == 0 else "field", n, base + k)

    return dict(name="served%d_soups+fields_%dk-%dM" % (pool, n_min // 1000, n_max // 1_000_000),
                pool=[spec(k, seed * 1000) for k in range(pool)],
                uploads=[spec(k, seed * 1000 + 500) for k in range(uploads)],
                make=lambda s: _served_scene(*s))


def served_requests(count, rate, seed=7, upload_frac=0.05, min_px=128 * 128,
                    max_px=1920 * 1080, depth=(1, 5), radius=(3.0, 6.0)):
    """A Poisson request stream: ``count`` requests at ``rate`` per second
    (rate None: all at time 0).  Renders have a camera on a sphere of radius
    uniform in ``radius`` aimed at the origin, a pixel count log-uniform in
    [min_px, max_px] at a 16:9 or 4:3 or 1:1 aspect, and a reflection depth
    uniform in ``depth``; ``upload_frac`` of the requests upload a scene.  A
    render names its scene by a uniform draw ``u`` in [0,1) over the scenes
    the client can target at that point."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    aspects = (16 / 9, 4 / 3, 1.0)
    for k in range(count):
        if rate:
            t += float(rng.exponential(1.0 / rate))
        if rng.random() < upload_frac:
            out.append(dict(kind="upload", t=t, index=int(rng.integers(0, 1 << 30))))
            continue
        px = math.exp(rng.uniform(math.log(min_px), math.log(max_px)))
        a = aspects[int(rng.integers(0, 3))]
        w = max(16, min(1920, int(round(math.sqrt(px * a)))))
        h = max(16, min(1080, int(round(px / w))))
        v = rng.normal(size=3)
        v = v / np.linalg.norm(v) * rng.uniform(*radius)
        cam = camera(tuple(float(x) for x in v), (0.0, 0.0, 0.0), fov_deg=60.0, aspect=w / h)
        out.append(dict(kind="render", t=t, width=w, height=h,
                        max_bounces=int(rng.integers(depth[0], depth[1] + 1)),
                        camera=cam, u=float(rng.random())))
    return out
