"""Procedural, seeded scenes and rays for the benchmark configurations.

Geometry and rays use only IEEE float arithmetic, sqrt, floor and integer
hashing (no transcendental functions), so the same seed yields bit-identical
inputs on every machine.  The sky envmap calls numpy's sin/cos, whose last
bit may differ between machines; parity tests that use it compare the GPU and
the oracle on the same machine.

* :func:`cornell_box` — 36 triangles: 5 walls, two boxes of 12, a 2-triangle
  area light of radiance (17, 12, 4); albedos 0.73 white, (0.65, 0.05, 0.05)
  red, (0.12, 0.45, 0.15) green.
* :func:`displaced_icosphere` — an icosahedron subdivided ``level`` times
  (level 8: 1,310,720 triangles, 655,362 vertices), each vertex displaced
  radially by 0.1 x 3-octave value noise.
* :func:`closest_hit_rays` — 2048^2 coherent pinhole primary rays plus the same
  number of incoherent rays (origins uniform in the bounding box, directions
  uniform on the sphere).
* :func:`mixed_scene` — the full-render scene: the displaced sphere, a
  2-triangle ground, per-triangle materials drawn from the seed (50 %
  Lambertian, 35 % Ward, 15 % dielectric), a homogeneous-volume box, and a
  1024x512 sky-gradient envmap with a 0.5-degree sun of radiance 1e4.

Triangles are wound so that the reference's geometric normal
``normalize(cross(v2 - v1, v1 - v0))`` (extension_ray_cast_stackless.cl:235)
points to the outside of closed objects and into the Cornell box.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import materials as M

F32 = np.float32


@dataclass
class Mesh:
    points: np.ndarray          # (n, 3) float32
    indices: np.ndarray         # (m, 3) uint32
    materials: list = field(default_factory=list)  # one rgr material record per triangle

    @property
    def ntris(self) -> int:
        return int(self.indices.shape[0])


def _ng(P: np.ndarray, I: np.ndarray) -> np.ndarray:
    v0, v1, v2 = P[I[:, 0]], P[I[:, 1]], P[I[:, 2]]
    return np.cross(v2 - v1, v1 - v0)


def orient(P: np.ndarray, I: np.ndarray, inside_point: np.ndarray, outward: bool) -> np.ndarray:
    """Flip triangles so the reference normal points away from (outward) or
    toward (inward) ``inside_point``."""
    I = I.copy()
    c = P[I].mean(axis=1)
    n = _ng(P, I)
    d = np.einsum("ij,ij->i", n, c - inside_point[None, :])
    flip = (d < 0) if outward else (d > 0)
    I[flip] = I[flip][:, [0, 2, 1]]
    return I


def _quad(a, b, c, d):
    return [a, b, c], [a, c, d]


def _box(lo, hi, rot_y_cos_sin=(1.0, 0.0), center=None):
    lo = np.asarray(lo, dtype=np.float64)
    hi = np.asarray(hi, dtype=np.float64)
    corners = np.array([[x, y, z] for x in (lo[0], hi[0]) for y in (lo[1], hi[1]) for z in (lo[2], hi[2])])
    if center is not None:
        cx, cz = center
        c, s = rot_y_cos_sin
        x = corners[:, 0] - cx
        z = corners[:, 2] - cz
        corners[:, 0] = cx + c * x + s * z
        corners[:, 2] = cz - s * x + c * z
    # corner index = 4*ix + 2*iy + iz
    faces = [(0, 1, 3, 2), (4, 6, 7, 5), (0, 4, 5, 1), (2, 3, 7, 6), (0, 2, 6, 4), (1, 5, 7, 3)]
    tris = []
    for a, b, cc, d in faces:
        t0, t1 = _quad(a, b, cc, d)
        tris += [t0, t1]
    return corners.astype(F32), np.array(tris, dtype=np.uint32)


def cornell_box() -> Mesh:
    white = M.lambertian(r=(0.73, 0.73, 0.73))
    red = M.lambertian(r=(0.65, 0.05, 0.05))
    green = M.lambertian(r=(0.12, 0.45, 0.15))
    light = M.lambertian(le=(17.0, 12.0, 4.0), r=(0.78, 0.78, 0.78))
    P, I, mats = [], [], []
    center = np.array([0.0, 1.0, 0.0], dtype=F32)

    def add(pts, tris, mat, outward, inside):
        base = sum(len(p) for p in P)
        pts = np.asarray(pts, dtype=F32)
        tris = orient(pts, np.asarray(tris, dtype=np.uint32), np.asarray(inside, dtype=F32), outward)
        P.append(pts)
        I.append(tris + base)
        mats.extend([mat] * len(tris))

    q = [[0, 1, 2], [0, 2, 3]]
    # walls (normals toward the box interior)
    add([[-1, 0, -1], [1, 0, -1], [1, 0, 1], [-1, 0, 1]], q, white, False, center)       # floor
    add([[-1, 2, -1], [1, 2, -1], [1, 2, 1], [-1, 2, 1]], q, white, False, center)       # ceiling
    add([[-1, 0, -1], [1, 0, -1], [1, 2, -1], [-1, 2, -1]], q, white, False, center)     # back
    add([[-1, 0, -1], [-1, 2, -1], [-1, 2, 1], [-1, 0, 1]], q, red, False, center)       # left
    add([[1, 0, -1], [1, 2, -1], [1, 2, 1], [1, 0, 1]], q, green, False, center)         # right
    # boxes (normals outward)
    for lo, hi, cs, cen in (
        ([-0.65, 0.0, -0.05], [-0.05, 1.2, 0.55], (0.9563, 0.2924), (-0.35, 0.25)),
        ([0.05, 0.0, -0.45], [0.65, 0.6, 0.15], (0.9563, -0.2924), (0.35, -0.15)),
    ):
        pts, tris = _box(lo, hi, cs, cen)
        add(pts, tris, white, True, pts.mean(axis=0))
    # light, just below the ceiling, facing down
    add([[-0.25, 1.98, -0.25], [0.25, 1.98, -0.25], [0.25, 1.98, 0.25], [-0.25, 1.98, 0.25]], q, light, False,
        [0.0, 0.0, 0.0])
    mesh = Mesh(np.concatenate(P), np.concatenate(I).astype(np.uint32), mats)
    assert mesh.ntris == 36
    return mesh


def cornell_camera(w: int = 256, h: int = 256):
    return dict(eye=(0.0, 1.0, 3.6), target=(0.0, 1.0, 0.0), up=(0.0, 1.0, 0.0), vfov=40.0, w=w, h=h)


# ------------------------------------------------------------------ icosphere
def _icosahedron():
    t = (1.0 + np.sqrt(5.0)) / 2.0
    v = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
                  [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], dtype=np.float64)
    f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4], [11, 10, 2],
                  [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9], [4, 9, 5],
                  [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], dtype=np.int64)
    v /= np.sqrt((v * v).sum(1, keepdims=True))
    return v, f


def icosphere(level: int):
    v, f = _icosahedron()
    for _ in range(level):
        nv = v.shape[0]
        e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]])
        e.sort(axis=1)
        key = e[:, 0] * (nv + 1) + e[:, 1]
        uniq, inv = np.unique(key, return_inverse=True)
        a = uniq // (nv + 1)
        b = uniq % (nv + 1)
        mid = v[a] + v[b]
        mid /= np.sqrt((mid * mid).sum(1, keepdims=True))
        v = np.concatenate([v, mid])
        m = inv.reshape(3, -1).T + nv  # midpoints of (01, 12, 20)
        f = np.concatenate([
            np.stack([f[:, 0], m[:, 0], m[:, 2]], 1),
            np.stack([f[:, 1], m[:, 1], m[:, 0]], 1),
            np.stack([f[:, 2], m[:, 2], m[:, 1]], 1),
            np.stack([m[:, 0], m[:, 1], m[:, 2]], 1),
        ])
    return v, f


def _hash3(ix, iy, iz, seed):
    h = (ix.astype(np.uint64) * np.uint64(0x9E3779B1) ^ iy.astype(np.uint64) * np.uint64(0x85EBCA77)
         ^ iz.astype(np.uint64) * np.uint64(0xC2B2AE3D) ^ np.uint64(seed) * np.uint64(0x27D4EB2F))
    h &= np.uint64(0xFFFFFFFF)
    h ^= h >> np.uint64(15)
    h = (h * np.uint64(0x2C1B3C6D)) & np.uint64(0xFFFFFFFF)
    h ^= h >> np.uint64(12)
    h = (h * np.uint64(0x297A2D39)) & np.uint64(0xFFFFFFFF)
    h ^= h >> np.uint64(15)
    return (h & np.uint64(0xFFFFFF)).astype(np.float64) / float(0xFFFFFF) * 2.0 - 1.0


def value_noise3(p: np.ndarray, seed: int, octaves: int = 3) -> np.ndarray:
    """Sum of ``octaves`` lattice value-noise layers (frequency 2^k * 2,
    amplitude 2^-k), smoothstep-interpolated, normalised to [-1, 1]."""
    total = np.zeros(p.shape[0])
    norm = 0.0
    for o in range(octaves):
        freq = 2.0 * (2 ** o)
        amp = 0.5 ** o
        q = p * freq
        i0 = np.floor(q)
        fr = q - i0
        s = fr * fr * (3.0 - 2.0 * fr)
        i0 = i0.astype(np.int64)
        acc = np.zeros(p.shape[0])
        for dx in (0, 1):
            wx = s[:, 0] if dx else 1.0 - s[:, 0]
            for dy in (0, 1):
                wy = s[:, 1] if dy else 1.0 - s[:, 1]
                for dz in (0, 1):
                    wz = s[:, 2] if dz else 1.0 - s[:, 2]
                    acc += wx * wy * wz * _hash3(i0[:, 0] + dx, i0[:, 1] + dy, i0[:, 2] + dz, seed + 1013 * o)
        total += amp * acc
        norm += amp
    return total / norm


def displaced_icosphere(level: int = 8, seed: int = 7, amplitude: float = 0.1) -> Mesh:
    v, f = icosphere(level)
    n = value_noise3(v, seed)
    P = (v * (1.0 + amplitude * n)[:, None]).astype(F32)
    I = orient(P, f.astype(np.uint32), np.zeros(3, dtype=F32), outward=True)
    return Mesh(P, I, [M.lambertian(r=(0.8, 0.8, 0.8))] * int(I.shape[0]))


# ------------------------------------------------------------------ rays
@dataclass
class Rays:
    o: np.ndarray     # (n, 3) float32
    d: np.ndarray     # (n, 3) float32
    tmax: np.ndarray  # (n,) float32

    def soa(self):
        return [np.ascontiguousarray(self.o[:, k]) for k in range(3)] + \
               [np.ascontiguousarray(self.d[:, k]) for k in range(3)] + [np.ascontiguousarray(self.tmax)]

    def packed8(self) -> np.ndarray:
        r = np.zeros((self.o.shape[0], 8), dtype=F32)
        r[:, 0:3] = self.o
        r[:, 3] = self.tmax
        r[:, 4:7] = self.d
        return r

    def __len__(self):
        return int(self.o.shape[0])

    def subset(self, idx):
        return Rays(self.o[idx], self.d[idx], self.tmax[idx])


FLT_MAX = np.float32(3.4028234663852886e38)


def pinhole_rays(eye, target, up, vfov_deg_tan_half: float, w: int, h: int) -> Rays:
    """Pixel-centre rays of a pinhole camera (image plane at distance 1)."""
    eye = np.asarray(eye, dtype=np.float64)
    fwd = np.asarray(target, dtype=np.float64) - eye
    fwd /= np.sqrt((fwd * fwd).sum())
    right = np.cross(fwd, np.asarray(up, dtype=np.float64))
    right /= np.sqrt((right * right).sum())
    upv = np.cross(right, fwd)
    ph = 2.0 * vfov_deg_tan_half
    pw = ph * w / h
    xs = (np.arange(w) + 0.5) / w - 0.5
    ys = 0.5 - (np.arange(h) + 0.5) / h
    X, Y = np.meshgrid(xs * pw, ys * ph)
    d = fwd[None, :] + X.reshape(-1, 1) * right[None, :] + Y.reshape(-1, 1) * upv[None, :]
    d /= np.sqrt((d * d).sum(1, keepdims=True))
    o = np.broadcast_to(eye.astype(F32), d.shape).copy()
    return Rays(o, d.astype(F32), np.full(d.shape[0], FLT_MAX, dtype=F32))


def random_rays(n: int, lo, hi, seed: int) -> Rays:
    rng = np.random.default_rng(seed)
    lo = np.asarray(lo, dtype=np.float64)
    hi = np.asarray(hi, dtype=np.float64)
    o = lo + (hi - lo) * rng.random((n, 3))
    d = np.empty((n, 3))
    filled = 0
    while filled < n:
        c = rng.random((2 * (n - filled) + 64, 3)) * 2.0 - 1.0
        r2 = (c * c).sum(1)
        c = c[(r2 <= 1.0) & (r2 > 1e-6)]
        take = min(n - filled, c.shape[0])
        d[filled:filled + take] = c[:take] / np.sqrt((c[:take] * c[:take]).sum(1, keepdims=True))
        filled += take
    return Rays(o.astype(F32), d.astype(F32), np.full(n, FLT_MAX, dtype=F32))


# tan(22.5 deg), the half field of view of the closest-hit benchmark camera
TAN_22_5 = 0.41421356237309503


def closest_hit_rays(mesh: Mesh, res: int = 2048, n_random: int | None = None, seed: int = 11):
    """The ray-cast microbenchmark's two ray sets: (coherent, incoherent)."""
    prim = pinhole_rays((0.0, 0.35, 3.0), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0), TAN_22_5, res, res)
    lo = mesh.points.min(0)
    hi = mesh.points.max(0)
    rnd = random_rays(n_random if n_random is not None else res * res, lo, hi, seed)
    return prim, rnd


# ------------------------------------------------------------------ full scene
def sky_envmap(w: int = 1024, h: int = 512, sun_dir=(0.45, 0.62, 0.64), sun_radiance: float = 1.0e4,
               sun_radius_deg: float = 0.25) -> np.ndarray:
    """Sky gradient plus a sun disk.  Texel (x, y) looks along
    (sin t sin p, cos t, sin t cos p) with t = pi (y + 0.5) / h and
    p = 2 pi (1 - (x + 0.5) / w), the reference envmap parameterisation
    (envmap_sampling.cl:36-52)."""
    ys = (np.arange(h) + 0.5) / h
    xs = (np.arange(w) + 0.5) / w
    t = np.pi * ys
    p = 2.0 * np.pi * (1.0 - xs)
    st, ct = np.sin(t)[:, None], np.cos(t)[:, None]
    sp, cp = np.sin(p)[None, :], np.cos(p)[None, :]
    dx, dy, dz = st * sp, ct * np.ones_like(sp), st * cp
    up = np.clip(dy, 0.0, 1.0)
    zen = np.array([0.25, 0.45, 1.0])
    hor = np.array([0.85, 0.9, 1.0])
    ground = np.array([0.12, 0.11, 0.10])
    img = np.where((dy >= 0)[..., None], hor + (zen - hor) * np.sqrt(up)[..., None], ground)
    s = np.asarray(sun_dir, dtype=np.float64)
    s /= np.sqrt((s * s).sum())
    cosang = dx * s[0] + dy * s[1] + dz * s[2]
    disk = cosang >= np.cos(np.radians(sun_radius_deg))
    if not disk.any():
        disk = cosang == cosang.max()
    img[disk] = sun_radiance
    out = np.ones((h, w, 4), dtype=F32)
    out[..., :3] = img
    return out


def mixed_scene(level: int = 8, seed: int = 3, volume: bool = True, env: bool = True):
    """Sphere + ground + optional volume box, per-triangle random materials."""
    sph = displaced_icosphere(level, seed=7)
    rng = np.random.default_rng(seed)
    ground_P = np.array([[-12, -1.2, -12], [12, -1.2, -12], [12, -1.2, 12], [-12, -1.2, 12]], dtype=F32)
    ground_I = orient(ground_P, np.array([[0, 1, 2], [0, 2, 3]], dtype=np.uint32), np.array([0, -5, 0], F32), True)
    P = [sph.points, ground_P]
    I = [sph.indices, ground_I + sph.points.shape[0]]
    ntri = sph.ntris + 2
    mats = M.random_mix(ntri, rng)
    if volume:
        bp, bi = _box([1.0, -1.2, 0.2], [2.2, 0.0, 1.4])
        bi = orient(bp, bi, bp.mean(0), outward=True)
        base = sum(p.shape[0] for p in P)
        P.append(bp)
        I.append(bi + base)
        vol = M.as_array([M.homogeneous_volume(c=0.55, r=(0.5 / 0.55,) * 3)] * bi.shape[0])
        mats = np.concatenate([mats, vol])
    mesh = Mesh(np.concatenate(P).astype(F32), np.concatenate(I).astype(np.uint32), mats)
    envmap = sky_envmap() if env else None
    camera = dict(eye=(0.0, 0.6, 4.6), target=(0.2, -0.25, 0.0), up=(0.0, 1.0, 0.0), vfov=38.0, w=1920, h=1080)
    return mesh, envmap, camera


def sky_room(level: int = 4, seed: int = 3):
    """A closed room lit only through a skylight: Lambertian walls, floor and
    ceiling (normals inward), a 1.2 x 1.2 opening in the ceiling, the
    displaced sphere (radius ~0.55, full-render material mix) and a Ward box
    inside, and the sky envmap (4x brighter) with a high sun whose patch falls
    on the floor.
    Most envmap directions from inside are blocked, so envmap and BSDF
    sampling both waste samples: the case learned guiding is for."""
    rng = np.random.default_rng(seed)
    P, I, mats = [], [], []
    center = np.array([0.0, 1.25, 0.0], dtype=F32)

    def add(pts, tris, m, outward, inside):
        base = sum(len(p) for p in P)
        pts = np.asarray(pts, dtype=F32)
        tris = orient(pts, np.asarray(tris, dtype=np.uint32), np.asarray(inside, dtype=F32), outward)
        P.append(pts)
        I.append(tris + base)
        if isinstance(m, np.ndarray):
            mats.append(m)
        else:
            mats.append(M.as_array([m] * len(tris)))

    q = [[0, 1, 2], [0, 2, 3]]
    wall = M.lambertian(r=(0.7, 0.7, 0.7))
    floor = M.lambertian(r=(0.55, 0.5, 0.45))
    X, Y, Z = 2.0, 2.5, 2.0
    add([[-X, 0, -Z], [X, 0, -Z], [X, 0, Z], [-X, 0, Z]], q, floor, False, center)
    add([[-X, 0, -Z], [X, 0, -Z], [X, Y, -Z], [-X, Y, -Z]], q, wall, False, center)
    add([[-X, 0, Z], [X, 0, Z], [X, Y, Z], [-X, Y, Z]], q, wall, False, center)
    add([[-X, 0, -Z], [-X, Y, -Z], [-X, Y, Z], [-X, 0, Z]], q, M.lambertian(r=(0.7, 0.25, 0.2)), False, center)
    add([[X, 0, -Z], [X, Y, -Z], [X, Y, Z], [X, 0, Z]], q, M.lambertian(r=(0.2, 0.45, 0.7)), False, center)
    # ceiling around the skylight x in [0.3, 1.1], z in [-1.2, -0.4]
    wx0, wx1, wz0, wz1 = 0.1, 1.3, -1.4, -0.2
    for x0, x1, z0, z1 in ((-X, wx0, -Z, Z), (wx1, X, -Z, Z), (wx0, wx1, -Z, wz0), (wx0, wx1, wz1, Z)):
        add([[x0, Y, z0], [x1, Y, z0], [x1, Y, z1], [x0, Y, z1]], q, wall, False, center)
    sph = displaced_icosphere(level, seed=7)
    sp = sph.points * 0.55 + np.array([-0.4, 0.6, -0.2], dtype=F32)
    add(sp, sph.indices, M.random_mix(sph.ntris, rng), True, sp.mean(axis=0))
    bp, bi = _box([0.5, 0.0, 0.3], [1.2, 0.9, 1.0], (0.94, 0.34), (0.85, 0.65))
    add(bp, bi, M.ward(alpha=0.15, reflectance=(0.04,) * 3, edgetint=(0.04,) * 3), True, bp.mean(axis=0))
    mesh = Mesh(np.concatenate(P).astype(F32), np.concatenate(I).astype(np.uint32), np.concatenate(mats))
    envmap = sky_envmap(sun_dir=(0.3, 0.9, 0.3))
    envmap[..., :3] *= 4.0
    camera = dict(eye=(-0.2, 1.4, 1.9), target=(0.0, 0.7, -0.6), up=(0.0, 1.0, 0.0), vfov=62.0, w=640, h=360)
    return mesh, envmap, camera


# ------------------------------------------------------------------ batched requests
_ICO = {}


def _ico(level: int) -> Mesh:
    if level not in _ICO:
        _ICO[level] = displaced_icosphere(level, seed=7)
    return _ICO[level]


def _loguniform(rng, lo: float, hi: float) -> float:
    return float(np.exp(rng.uniform(np.log(lo), np.log(hi))))


def request_scene(target_tris: int, rng, volume: bool) -> tuple:
    """A scene of about `target_tris` triangles: displaced icospheres of the
    levels that sum to the target (each level L has 20 * 4^L triangles),
    scattered above a ground quad, with the full-render material mix and,
    optionally, a homogeneous-volume box.  Returns (mesh, camera dict)."""
    P, I = [], []
    remaining = max(int(target_tris), 1280)
    base = 0
    centres = []
    while remaining >= 1280 or not P:
        level = int(min(8, max(3, np.floor(np.log(max(remaining, 1280) / 20.0) / np.log(4.0)))))
        m = _ico(level)
        r = 0.3 + 0.7 * rng.random()
        c = np.array([rng.uniform(-2.5, 2.5), r - 1.2, rng.uniform(-2.5, 2.5)])
        centres.append(c)
        P.append((m.points * r + c).astype(F32))
        I.append(m.indices + base)
        base += m.points.shape[0]
        remaining -= m.ntris
    gp = np.array([[-8, -1.2, -8], [8, -1.2, -8], [8, -1.2, 8], [-8, -1.2, 8]], dtype=F32)
    P.append(gp)
    I.append(orient(gp, np.array([[0, 1, 2], [0, 2, 3]], np.uint32), np.array([0, -5, 0], F32), True) + base)
    base += 4
    ntri = int(sum(x.shape[0] for x in I))
    mats = M.random_mix(ntri, rng)
    if volume:
        lo = np.array([rng.uniform(-2, 1), -1.2, rng.uniform(-2, 1)])
        bp, bi = _box(lo, lo + np.array([1.0, 1.2, 1.0]))
        bi = orient(bp, bi, bp.mean(0), outward=True)
        P.append(bp)
        I.append(bi + base)
        mats = np.concatenate([mats, M.as_array([M.homogeneous_volume(c=0.55, r=(0.5 / 0.55,) * 3)] * 12)])
    mesh = Mesh(np.concatenate(P).astype(F32), np.concatenate(I).astype(np.uint32), mats)
    look = np.mean(centres, axis=0)
    ang = rng.uniform(0, 2 * np.pi)
    eye = look + np.array([6.0 * np.sin(ang), 2.5, 6.0 * np.cos(ang)])
    cam = dict(eye=tuple(eye), target=tuple(look), up=(0.0, 1.0, 0.0), vfov=45.0)
    return mesh, cam


def batch_requests(n: int = 32, seed: int = 21, max_tris: int = 2_000_000):
    """The batched-requests workload: `n` requests with resolution (square
    side) log-uniform in 64..1024, spp log-uniform in 1..256, triangles
    log-uniform in 1k..max_tris, the full-render material mix and envmap,
    half of them with a volume box.  Returns a list of dicts."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        side = int(round(_loguniform(rng, 64, 1024)))
        spp = int(round(_loguniform(rng, 1, 256)))
        tris = int(round(_loguniform(rng, 1000, max_tris)))
        volume = (i % 2) == 1
        mesh, cam = request_scene(tris, rng, volume)
        cam.update(w=side, h=side)
        out.append(dict(mesh=mesh, camera=cam, spp=spp, max_depth=8, volume=volume))
    return out
