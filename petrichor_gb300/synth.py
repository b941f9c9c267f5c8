"""Seeded synthetic scenes for the path-tracing workloads.

Every draw comes from a SplitMix64 counter stream evaluated with numpy uint64
arithmetic, so the same seed gives the same scene bytes on any host (no
``np.random`` distributions, whose algorithms may change between versions).
Geometry uses float64 math rounded once to float32.

Workloads (sizes as named by the benchmark description):

* ``cornell``      -- 5 wall quads (open front) + 2 rotated boxes = 34 triangles,
  plus a 2-triangle ceiling quad light of radiance 15; Lambert albedo in
  [0.1, 0.8] per channel; 256x256, 40 deg vertical FOV pinhole, 16 spp.
* ``spheres_grids`` -- 64 seeded UV-spheres and displaced grids (1.0M triangles at
  full size); 40% Lambert / 40% GGX / 20% glass (IOR 1.5); lit by a procedural
  equirect sky (gradient x log-normal background + Gaussian sun lobe);
  1920x1080, 64 spp, max 16 bounces, MIS next-event estimation.
* ``terrain_rocks`` -- a displaced terrain grid plus many randomised rock meshes,
  mostly GGX with 10% glass (the memory-bound stress case).
"""
from __future__ import annotations

import dataclasses
import math
from typing import List, Tuple

import numpy as np

from .scene_io import (Camera, Environment, Material, Scene, Settings, MAT_EMISSION,
                       MAT_GLASS, MAT_GLOSSY, MAT_LAMBERT, MAT_MIX, SHADING_FLAT, SHADING_SMOOTH,
                       INTEGRATOR_PT, INTEGRATOR_SIMPLE)

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


class Rng:
    """SplitMix64 counter stream; ``uniform(n)`` returns float64 in [0, 1)."""

    def __init__(self, seed: int):
        self.state = np.uint64(seed & 0xFFFFFFFFFFFFFFFF)

    def u64(self, n: int) -> np.ndarray:
        with np.errstate(over="ignore"):
            k = np.arange(1, n + 1, dtype=np.uint64)
            z = self.state + k * np.uint64(0x9E3779B97F4A7C15)
            self.state = self.state + np.uint64(n) * np.uint64(0x9E3779B97F4A7C15)
            z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
            z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
            z = z ^ (z >> np.uint64(31))
        return z

    def uniform(self, n: int, lo: float = 0.0, hi: float = 1.0) -> np.ndarray:
        u = (self.u64(n) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)
        return lo + (hi - lo) * u

    def normal(self, n: int) -> np.ndarray:
        """Box-Muller from two uniform streams."""
        u1 = self.uniform(n)
        u2 = self.uniform(n)
        return np.sqrt(-2.0 * np.log1p(-u1)) * np.cos(2.0 * math.pi * u2)

    def one(self, lo=0.0, hi=1.0) -> float:
        return float(self.uniform(1, lo, hi)[0])


class _Builder:
    def __init__(self):
        self.pos: List[np.ndarray] = []
        self.nrm: List[np.ndarray] = []
        self.uv: List[np.ndarray] = []
        self.idx: List[np.ndarray] = []
        self.mat: List[np.ndarray] = []
        self.sh: List[np.ndarray] = []
        self.nv = 0
        self.nt = 0

    def add(self, pos, idx, mat, shading, nrm=None, uv=None) -> Tuple[int, int]:
        pos = np.asarray(pos, np.float64)
        n = pos.shape[0]
        if nrm is None:
            nrm = np.tile([0.0, 0.0, 1.0], (n, 1))
        if uv is None:
            uv = np.zeros((n, 3))
        idx = np.asarray(idx, np.int64) + self.nv
        t0 = self.nt
        self.pos.append(pos)
        self.nrm.append(np.asarray(nrm, np.float64))
        self.uv.append(np.asarray(uv, np.float64))
        self.idx.append(idx)
        self.mat.append(np.full(idx.shape[0], mat, np.int32))
        self.sh.append(np.full(idx.shape[0], shading, np.uint8))
        self.nv += n
        self.nt += idx.shape[0]
        return t0, self.nt

    def arrays(self):
        return (np.concatenate(self.pos).astype(np.float32),
                np.concatenate(self.nrm).astype(np.float32),
                np.concatenate(self.uv).astype(np.float32),
                np.concatenate(self.idx).astype(np.int32),
                np.concatenate(self.mat).astype(np.int32),
                np.concatenate(self.sh).astype(np.uint8))


def _quad(p0, p1, p2, p3):
    return np.array([p0, p1, p2, p3], np.float64), np.array([[0, 1, 2], [0, 2, 3]])


def _box(center, size, angle):
    """12-triangle box rotated by ``angle`` about +Z, resting on z = center.z - size.z/2."""
    cx, cy, cz = center
    sx, sy, sz = [s * 0.5 for s in size]
    c, s = math.cos(angle), math.sin(angle)
    corners = []
    for z in (-sz, sz):
        for (x, y) in ((-sx, -sy), (sx, -sy), (sx, sy), (-sx, sy)):
            corners.append((cx + c * x - s * y, cy + s * x + c * y, cz + z))
    P = np.array(corners)
    faces = [(0, 1, 2, 3), (4, 7, 6, 5), (0, 4, 5, 1), (1, 5, 6, 2), (2, 6, 7, 3), (3, 7, 4, 0)]
    idx = []
    for a, b, cc, d in faces:
        idx += [[a, b, cc], [a, cc, d]]
    return P, np.array(idx)


def cornell(seed: int = 1, width: int = 256, height: int = 256, spp: int = 16,
            max_bounces: int = 3, integrator: int = INTEGRATOR_SIMPLE,
            light_radiance: float = 15.0, mixed: bool = False, aperture: float = 0.0,
            tile: int = 16, env_texture: bool = False) -> Scene:
    """Cornell-box-style scene: 34 geometry triangles + 2-triangle ceiling light.

    ``max_bounces=3`` is the bounce count after which the reference's
    SimplePathTracing starts Russian roulette (``SimplePathTracing.cpp:78-91``).
    ``mixed=True`` swaps in every material kind (GGX tall box, glass short box,
    a Lambert/GGX mix on the back wall) for parity coverage; ``aperture`` > 0
    turns on the thin lens focused on the tall box; ``env_texture`` lights the
    open front with a small procedural sky.
    """
    rng = Rng(seed)
    b = _Builder()
    mats: List[Material] = []

    def lambert():
        kd = tuple(float(x) for x in rng.uniform(3, 0.1, 0.8))
        mats.append(Material(MAT_LAMBERT, color=kd))
        return len(mats) - 1

    X, Y, Z = 1.0, 1.0, 2.0
    walls = [
        ((-X, -Y, 0), (X, -Y, 0), (X, Y, 0), (-X, Y, 0)),        # floor
        ((-X, -Y, Z), (-X, Y, Z), (X, Y, Z), (X, -Y, Z)),        # ceiling
        ((-X, Y, 0), (X, Y, 0), (X, Y, Z), (-X, Y, Z)),          # back
        ((-X, -Y, 0), (-X, Y, 0), (-X, Y, Z), (-X, -Y, Z)),      # left
        ((X, -Y, 0), (X, -Y, Z), (X, Y, Z), (X, Y, 0)),          # right
    ]
    for w in walls:
        P, I = _quad(*w)
        b.add(P, I, lambert(), SHADING_FLAT)
    P, I = _box((-0.35, 0.3, 0.6), (0.6, 0.6, 1.2), math.radians(17.0))
    tall = lambert()
    b.add(P, I, tall, SHADING_FLAT)
    P, I = _box((0.35, -0.3, 0.3), (0.6, 0.6, 0.6), math.radians(-17.0))
    short = lambert()
    b.add(P, I, short, SHADING_FLAT)
    assert b.nt == 34
    if mixed:
        mats[tall] = Material(MAT_GLOSSY, color=(2.5 * math.sqrt(0.6),) * 3, roughness=0.3)
        mats[short] = Material(MAT_GLASS, ior=1.5)
        mats.append(Material(MAT_GLOSSY, color=(1.2, 0.9, 0.5), roughness=0.15))
        mats.append(Material(MAT_MIX, mix=0.4, mat0=2, mat1=len(mats) - 1))
        b.mat[2][:] = len(mats) - 1   # back wall -> mix
    mats.append(Material(MAT_EMISSION, color=(light_radiance,) * 3))
    lz = Z - 1e-3
    P, I = _quad((-0.3, -0.3, lz), (-0.3, 0.3, lz), (0.3, 0.3, lz), (0.3, -0.3, lz))
    t0, t1 = b.add(P, I, len(mats) - 1, SHADING_FLAT)
    pos, nrm, uv, idx, tm, sh = b.arrays()
    cam = Camera(pos=(0.0, -4.8, 1.0), view_dir=(0.0, 1.0, 0.0), fov=math.radians(40.0),
                 focus_target=(-0.35, 0.3, 0.6) if aperture > 0 else None, aperture=aperture)
    st = Settings(width=width, height=height, spp=spp, max_bounces=max_bounces,
                  tile_width=tile, tile_height=tile, integrator=integrator)
    env = Environment()
    if env_texture:
        env = Environment(base_color=(1.0, 1.0, 1.0), texture=sky_env(rng, 64, 32))
    return Scene(pos, nrm, uv, idx, tm, sh, np.arange(t0, t1, dtype=np.int32), mats, cam,
                 env, st)


def _uv_sphere(center, radius, nu, nv):
    """UV sphere with pole fans: 2*nu*(nv-1) triangles, smooth normals."""
    th = np.linspace(0.0, math.pi, nv + 1)[1:-1]           # interior rings
    ph = np.linspace(0.0, 2.0 * math.pi, nu, endpoint=False)
    T, Ph = np.meshgrid(th, ph, indexing="ij")
    d = np.stack([np.sin(T) * np.cos(Ph), np.sin(T) * np.sin(Ph), np.cos(T)], -1).reshape(-1, 3)
    d = np.concatenate([[[0, 0, 1.0]], d, [[0, 0, -1.0]]])
    P = np.asarray(center) + radius * d
    # texture coordinates (phi / 2 pi, theta / pi, 0); the poles take u = 0
    uv = np.zeros_like(P)
    uv[1:-1, 0] = (Ph / (2.0 * math.pi)).reshape(-1)
    uv[1:-1, 1] = (T / math.pi).reshape(-1)
    uv[-1, 1] = 1.0
    rings = nv - 1
    idx = []
    ring = lambda r, k: 1 + r * nu + (k % nu)
    k = np.arange(nu)
    idx.append(np.stack([np.zeros(nu, int), ring(0, k), ring(0, k + 1)], -1))
    for r in range(rings - 1):
        a, bb = ring(r, k), ring(r, k + 1)
        c, dd = ring(r + 1, k), ring(r + 1, k + 1)
        idx.append(np.stack([a, c, dd], -1))
        idx.append(np.stack([a, dd, bb], -1))
    south = 1 + rings * nu
    idx.append(np.stack([np.full(nu, south), ring(rings - 1, k + 1), ring(rings - 1, k)], -1))
    return P, np.concatenate(idx), d, uv


def _displaced_grid(rng: Rng, center, size, n, amp, tilt, yaw):
    """n x n quad heightfield (2n^2 triangles) with a few random bumps, tilted and rotated."""
    g = np.linspace(-0.5, 0.5, n + 1)
    X, Y = np.meshgrid(g, g, indexing="ij")
    H = np.zeros_like(X)
    for _ in range(6):
        cx, cy = rng.uniform(2, -0.5, 0.5)
        s = rng.one(0.08, 0.3)
        a = rng.one(-1.0, 1.0)
        H += a * np.exp(-((X - cx) ** 2 + (Y - cy) ** 2) / (2 * s * s))
    H += 0.15 * np.sin(9.0 * X + rng.one(0, 6.28)) * np.cos(7.0 * Y + rng.one(0, 6.28))
    P = np.stack([X * size, Y * size, H * amp], -1).reshape(-1, 3)
    ct, st_ = math.cos(tilt), math.sin(tilt)
    cy_, sy_ = math.cos(yaw), math.sin(yaw)
    Rx = np.array([[1, 0, 0], [0, ct, -st_], [0, st_, ct]])
    Rz = np.array([[cy_, -sy_, 0], [sy_, cy_, 0], [0, 0, 1]])
    R = Rz @ Rx
    P = P @ R.T + np.asarray(center)
    i = np.arange(n)
    I, J = np.meshgrid(i, i, indexing="ij")
    v00 = (I * (n + 1) + J).ravel()
    v10 = v00 + (n + 1)
    idx = np.concatenate([np.stack([v00, v10, v10 + 1], -1), np.stack([v00, v10 + 1, v00 + 1], -1)])
    # vertex normals from the heightfield gradient
    dHx = np.gradient(H * amp, size / n, axis=0)
    dHy = np.gradient(H * amp, size / n, axis=1)
    Nl = np.stack([-dHx, -dHy, np.ones_like(H)], -1).reshape(-1, 3)
    Nl /= np.linalg.norm(Nl, axis=1, keepdims=True)
    return P, idx, Nl @ R.T


def sky_env(rng: Rng, width: int, height: int, sun_elev_deg=35.0, sun_azim_deg=60.0,
            sun_sigma_deg=1.0, sun_peak_over_median=1.0e4, sigma_ln=0.5) -> np.ndarray:
    """Equirect RGB float32 (height, width, 3) in the reference's mapping.

    Texel (i, j) is direction theta = pi*(j+0.5)/H from +Z and
    phi = 2*pi*(1 - (i+0.5)/W) (``Environment.cpp:29-48`` inverted, no rotation).
    """
    v = (np.arange(height) + 0.5) / height
    u = (np.arange(width) + 0.5) / width
    theta = (math.pi * v)[:, None]
    phi = (2.0 * math.pi * (1.0 - u))[None, :]
    dz = np.cos(theta) * np.ones_like(phi)
    horizon = np.clip(dz, 0.0, 1.0)
    sky = np.stack([0.35 + 0.25 * (1 - horizon), 0.55 + 0.2 * (1 - horizon),
                    0.95 + 0.05 * (1 - horizon)], -1)
    ground = np.array([0.25, 0.22, 0.2])
    w_ground = (dz < 0)[..., None]
    base = np.where(w_ground, ground * (0.5 + 0.5 * (1 + dz[..., None])), sky)
    noise = np.exp(sigma_ln * rng.normal(height * width)).reshape(height, width, 1)
    img = base * noise
    med = float(np.median(img.mean(-1)))
    se, sa = math.radians(sun_elev_deg), math.radians(sun_azim_deg)
    sdir = np.array([math.cos(se) * math.cos(sa), math.cos(se) * math.sin(sa), math.sin(se)])
    d = np.stack([np.sin(theta) * np.cos(phi), np.sin(theta) * np.sin(phi), dz], -1)
    cosang = np.clip(d @ sdir, -1.0, 1.0)
    ang = np.arccos(cosang)
    lobe = np.exp(-0.5 * (ang / math.radians(sun_sigma_deg)) ** 2)
    sun_col = np.array([1.0, 0.95, 0.85])
    img = img + (sun_peak_over_median * med) * lobe[..., None] * sun_col
    return img.astype(np.float32)


def _mixed_material(rng: Rng, p_lambert=0.4, p_ggx=0.4,
                    rough_lo=0.05, rough_hi=0.8) -> Material:
    r = rng.one()
    if r < p_lambert:
        return Material(MAT_LAMBERT, color=tuple(float(x) for x in rng.uniform(3, 0.1, 0.8)))
    if r < p_lambert + p_ggx:
        rough = rng.one(rough_lo, rough_hi)
        f0 = rng.one(0.02, 0.95)
        c = 2.5 * math.sqrt(f0)   # GGX::GetF0 = 0.16 * c^2 (GGX.h:126-139)
        return Material(MAT_GLOSSY, color=(c, c, c), roughness=rough)
    return Material(MAT_GLASS, color=(1.0, 1.0, 1.0), ior=1.5)


def spheres_grids(seed: int = 2, tri_budget: int = 1_000_000, n_objects: int = 64,
                  width: int = 1920, height: int = 1080, spp: int = 64, max_bounces: int = 16,
                  env_width: int = 2048, env_height: int = 1024,
                  sun_peak_over_median: float = 1.0e4, env_texture=None) -> Scene:
    """64 seeded UV-spheres and displaced grids totalling ~``tri_budget`` triangles.

    ``sun_peak_over_median`` scales the sun lobe (1e4 in the benchmark workload;
    lower values give low-variance variants for statistical tests)."""
    rng = Rng(seed)
    b = _Builder()
    mats: List[Material] = []
    per_obj = max(8, tri_budget // n_objects)
    side = int(math.ceil(math.sqrt(n_objects)))
    spacing = 2.2
    for o in range(n_objects):
        gx, gy = o % side, o // side
        cx = (gx - (side - 1) / 2) * spacing + rng.one(-0.3, 0.3)
        cy = (gy - (side - 1) / 2) * spacing + rng.one(-0.3, 0.3)
        mats.append(_mixed_material(rng))
        m = len(mats) - 1
        if rng.one() < 0.5:
            # sphere: 2*nu*(nv-1) ~= per_obj with nu = 4*(nv-1)
            nvm1 = max(2, int(round(math.sqrt(per_obj / 8.0))))
            nu = max(3, int(round(per_obj / (2.0 * nvm1))))
            r = rng.one(0.45, 0.95)
            P, I, N, UV = _uv_sphere((cx, cy, r + rng.one(0.0, 0.4)), r, nu, nvm1 + 1)
            b.add(P, I, m, SHADING_SMOOTH, nrm=N, uv=UV)
        else:
            n = max(1, int(round(math.sqrt(per_obj / 2.0))))
            P, I, N = _displaced_grid(rng, (cx, cy, rng.one(0.3, 1.2)), rng.one(1.4, 2.0), n,
                                      rng.one(0.1, 0.35), rng.one(-0.9, 0.9), rng.one(0, 6.28))
            b.add(P, I, m, SHADING_SMOOTH, nrm=N)
    pos, nrm, uv, idx, tm, sh = b.arrays()
    if env_texture is None:
        env_texture = sky_env(rng, env_width, env_height, sun_peak_over_median=sun_peak_over_median)
    env = Environment(base_color=(1.0, 1.0, 1.0), texture=env_texture)
    extent = side * spacing
    cam = Camera(pos=(0.0, -0.95 * extent, 0.5 * extent), view_dir=(0.0, 0.95 * extent, -0.5 * extent + 0.5),
                 fov=math.radians(45.0), focus_target=None, aperture=0.0)
    st = Settings(width=width, height=height, spp=spp, max_bounces=max_bounces,
                  integrator=INTEGRATOR_PT)
    return Scene(pos, nrm, uv, idx, tm, sh, np.zeros(0, np.int32), mats, cam, env, st)


def textured_spheres(seed: int = 4, tri_budget: int = 4000, width: int = 48, height: int = 27,
                     spp: int = 2, max_bounces: int = 6, env_width: int = 64, env_height: int = 32,
                     integrator: int = INTEGRATOR_PT) -> Scene:
    """A small spheres_grids scene whose materials carry texture maps: Lambert albedo
    maps, GGX reflectance, roughness and normal maps (with their strengths), on a few
    procedural RGB textures. Spheres keep their (phi, theta) uvs; grids get planar uvs."""
    sc = spheres_grids(seed=seed, tri_budget=tri_budget, width=width, height=height, spp=spp,
                       max_bounces=max_bounces, env_width=env_width, env_height=env_height,
                       sun_peak_over_median=30.0)
    rng = Rng(seed + 1000)
    textures = []
    for k, (w, h) in enumerate([(32, 32), (48, 24), (16, 40), (24, 24)]):
        y, x = np.mgrid[0:h, 0:w].astype(np.float64)
        f = rng.uniform(3, 1.0, 6.0)
        base = 0.5 + 0.5 * np.sin(f[0] * 2 * math.pi * x / w)[..., None] * \
            np.cos(f[1] * 2 * math.pi * y / h)[..., None] * np.array([1.0, 0.7, 0.4])
        noise = np.array([rng.one() for _ in range(w * h * 3)]).reshape(h, w, 3)
        textures.append(np.clip(0.05 + 0.8 * base + 0.15 * noise, 0.0, 1.0).astype(np.float32))
    mats = []
    for m in sc.materials:
        m = dataclasses.replace(m)
        if m.kind == MAT_LAMBERT and rng.one() < 0.7:
            m.albedo_tex = int(rng.one() * 4) % 4
        elif m.kind == MAT_GLOSSY:
            if rng.one() < 0.5:
                m.f0_tex = int(rng.one() * 4) % 4
            if rng.one() < 0.5:
                m.roughness_tex = int(rng.one() * 4) % 4
                m.roughness_map_strength = rng.one(0.5, 1.5)
            if rng.one() < 0.5:
                m.normal_tex = int(rng.one() * 4) % 4
                m.normal_map_strength = rng.one(0.0, 1.0)
        mats.append(m)
    uv = sc.uvs.copy()
    flat = ~np.any(uv != 0.0, axis=1)
    uv[flat, 0] = 0.37 * sc.positions[flat, 0]
    uv[flat, 1] = 0.29 * sc.positions[flat, 1]
    st = dataclasses.replace(sc.settings, integrator=integrator)
    return sc.copy_with(materials=mats, uvs=uv.astype(np.float32), textures=textures, settings=st)


def terrain_rocks(seed: int = 5, terrain_n: int = 3000, n_rocks: int = 4000, rock_tris: int = 500,
                  width: int = 3840, height: int = 2160, spp: int = 256, max_bounces: int = 12,
                  env_width: int = 8192, env_height: int = 4096) -> Scene:
    """Displaced terrain (2*terrain_n^2 triangles) + ``n_rocks`` distinct randomised rocks.

    The defaults give 18M + 2M = 20M unique triangles.
    """
    rng = Rng(seed)
    b = _Builder()
    mats: List[Material] = []
    mats.append(Material(MAT_GLOSSY, color=(2.5 * math.sqrt(0.04),) * 3, roughness=0.5))
    P, I, N = _displaced_grid(rng, (0.0, 0.0, 0.0), 100.0, terrain_n, 6.0, 0.0, 0.0)
    b.add(P, I, 0, SHADING_SMOOTH, nrm=N)
    nvm1 = max(2, int(round(math.sqrt(rock_tris / 8.0))))
    nu = max(3, int(round(rock_tris / (2.0 * nvm1))))
    for _ in range(n_rocks):
        if rng.one() < 0.1:
            mats.append(Material(MAT_GLASS, ior=1.5))
        else:
            f0 = rng.one(0.02, 0.95)
            mats.append(Material(MAT_GLOSSY, color=(2.5 * math.sqrt(f0),) * 3,
                                 roughness=rng.one(0.1, 0.6)))
        r = rng.one(0.2, 1.5)
        c = (rng.one(-45, 45), rng.one(-45, 45), rng.one(0.0, 6.0))
        P, I, Nd, UV = _uv_sphere(c, r, nu, nvm1 + 1)
        k = rng.uniform(3, 0.6, 1.4)
        bump = 1.0 + 0.15 * np.sin(5.0 * Nd[:, 0] + rng.one(0, 6.28)) * np.cos(4.0 * Nd[:, 1])
        P = np.asarray(c) + (P - np.asarray(c)) * k * bump[:, None]
        b.add(P, I, len(mats) - 1, SHADING_FLAT, uv=UV)
    pos, nrm, uv, idx, tm, sh = b.arrays()
    env = Environment(base_color=(1.0, 1.0, 1.0), texture=sky_env(rng, env_width, env_height))
    cam = Camera(pos=(0.0, -60.0, 25.0), view_dir=(0.0, 60.0, -22.0), fov=math.radians(50.0),
                 aperture=0.0)
    st = Settings(width=width, height=height, spp=spp, max_bounces=max_bounces,
                  integrator=INTEGRATOR_PT)
    return Scene(pos, nrm, uv, idx, tm, sh, np.zeros(0, np.int32), mats, cam, env, st)


def bvh_ties(seed: int = 6, n_lattice: int = 2400, n_zero: int = 500, n_free: int = 300,
             width: int = 32, height: int = 18, spp: int = 1) -> Scene:
    """Triangles whose binned-SAH tree depends on how std::sort orders equal keys and on
    signed zeros: centroids on a coarse lattice (exact, with many equal keys on every
    axis and exact duplicates), a slab in the plane x = 0 whose vertices carry +0.0 or
    -0.0, and a few free triangles; all shuffled together."""
    rng = Rng(seed)
    tris = []
    cell = np.floor(rng.uniform(3 * n_lattice).reshape(n_lattice, 3) * [12, 10, 8])
    lift = np.floor(rng.uniform(n_lattice) * 2) * 3.0
    for (ix, iy, iz), s in zip(cell, lift):
        o = np.array([3 * ix, 3 * iy, 3 * iz])
        tris.append([o, o + [3, 0, 0], o + [0, 3, s]])
    for k in range(n_zero):
        yz = rng.uniform(6).reshape(3, 2) * 30.0
        sign = np.where(rng.uniform(3) < 0.5, -0.0, 0.0)
        tris.append([[sign[j], yz[j, 0], yz[j, 1]] for j in range(3)])
    for k in range(n_free):
        c = rng.uniform(3) * [36, 30, 24]
        tris.append([c + (rng.uniform(3) - 0.5) * 2.0 for _ in range(3)])
    order = np.argsort(rng.uniform(len(tris)), kind="stable")
    P = np.array([tris[i] for i in order], np.float64).reshape(-1, 3)
    I = np.arange(P.shape[0]).reshape(-1, 3)
    b = _Builder()
    b.add(P, I, 0, SHADING_FLAT)
    pos, nrm, uv, idx, tm, sh = b.arrays()
    mats = [Material(MAT_LAMBERT, color=(0.6, 0.6, 0.6))]
    env = Environment(base_color=(1.0, 1.0, 1.0), texture=None)
    cam = Camera(pos=(18.0, -40.0, 30.0), view_dir=(0.0, 40.0, -18.0), fov=math.radians(50.0),
                 focus_target=None, aperture=0.0)
    st = Settings(width=width, height=height, spp=spp, max_bounces=3)
    return Scene(pos, nrm, uv, idx, tm, sh, np.zeros(0, np.int32), mats, cam, env, st)


def batch_instance_params(seed: int = 3, n: int = 64, tri_lo: float = 1e4, tri_hi: float = 2e6,
                          px_lo: float = 256 ** 2, px_hi: float = 1024 ** 2, spps=(4, 16, 64, 256)):
    """(triangle budget, width, height, spp) of each of ``batch_instances``' scenes."""
    rng = Rng(seed)
    out = []
    for _ in range(n):
        tris = int(math.exp(rng.one(math.log(tri_lo), math.log(tri_hi))))
        px = math.exp(rng.one(math.log(px_lo), math.log(px_hi)))
        aspect = rng.one(0.5, 2.0)
        w = max(8, int(round(math.sqrt(px * aspect))))
        h = max(8, int(round(px / w)))
        spp = spps[int(rng.one() * len(spps)) % len(spps)]
        out.append((tris, w, h, spp))
    return out


def batch_instance(k: int, seed: int = 3, env_width: int = 1024, env_height: int = 512,
                   max_bounces: int = 16, **ranges):
    """Scene k of ``batch_instances`` alone."""
    tris, w, h, spp = batch_instance_params(seed, k + 1, **ranges)[k]
    return spheres_grids(seed=1000 + k, tri_budget=tris, width=w, height=h, spp=spp,
                         max_bounces=max_bounces, env_width=env_width, env_height=env_height)


def batch_instances(seed: int = 3, n: int = 64, tri_lo: float = 1e4, tri_hi: float = 2e6,
                    px_lo: float = 256 ** 2, px_hi: float = 1024 ** 2, spps=(4, 16, 64, 256),
                    env_width: int = 1024, env_height: int = 512, max_bounces: int = 16):
    """``n`` independent spheres-and-grids scenes of uneven size: triangle counts and
    pixel counts log-uniform, aspect uniform in [0.5, 2], spp drawn from ``spps``."""
    return [spheres_grids(seed=1000 + k, tri_budget=tris, width=w, height=h, spp=spp,
                          max_bounces=max_bounces, env_width=env_width, env_height=env_height)
            for k, (tris, w, h, spp) in enumerate(batch_instance_params(
                seed, n, tri_lo, tri_hi, px_lo, px_hi, spps))]


def _map_texture(seed: int, size: int) -> np.ndarray:
    """A procedural RGB material map in [0.05, 0.95]: a product of sinusoids times a
    bilinear value-noise field on a 64x64 lattice (seeded), (size, size, 3) float32."""
    rng = Rng(seed)
    f = rng.uniform(4, 2.0, 9.0)
    x = (np.arange(size, dtype=np.float32) + 0.5) / size
    wave = 0.5 + 0.5 * np.sin(np.float32(f[0] * 2 * math.pi) * x)[None, :] * \
        np.cos(np.float32(f[1] * 2 * math.pi) * x)[:, None]
    lat = rng.uniform(65 * 65).astype(np.float32).reshape(65, 65)
    g = x * 64.0
    i0 = np.minimum(g.astype(np.int32), 63)
    w1 = (g - i0).astype(np.float32)
    rows = lat[i0] * (1 - w1)[:, None] + lat[i0 + 1] * w1[:, None]          # (size, 65)
    noise = rows[:, i0] * (1 - w1)[None, :] + rows[:, i0 + 1] * w1[None, :]  # (size, size)
    v = (0.05 + 0.6 * wave + 0.3 * noise).astype(np.float32)
    tint = np.array([1.0, 0.8, 0.6], np.float32)
    return np.clip(v[..., None] * tint, 0.05, 0.95).astype(np.float32)


def serving_scenes(seed: int = 4, n: int = 8, tri_lo: float = 1e5, tri_hi: float = 4e6,
                   env_width: int = 8192, env_height: int = 4096, map_size: int = 4096,
                   maps_per_scene: int = 3):
    """``n`` resident scenes for the serving workload, triangle counts spread
    log-uniformly over [tri_lo, tri_hi] (first and last at the ends). Each scene has
    its own sky (the procedural sky turned about +Z by a per-scene azimuth, so the sun
    stands elsewhere) and ``maps_per_scene`` material maps of ``map_size``^2 texels
    (Lambert albedo maps; GGX reflectance and roughness maps), each its own variant of
    one procedural map (shifted and tinted). At the defaults that is about 12 GB of
    BVH, triangles, skies and maps resident on the device."""
    sky = sky_env(Rng(seed), env_width, env_height)
    base_map = _map_texture(seed + 77, map_size) if maps_per_scene > 0 else None
    out = []
    for k in range(n):
        f = k / max(1, n - 1)
        tris = int(math.exp(math.log(tri_lo) + f * (math.log(tri_hi) - math.log(tri_lo))))
        rng = Rng(3000 + k + seed)
        env_k = np.roll(sky, (k * env_width) // n, axis=1)
        sc = spheres_grids(seed=2000 + k + seed, tri_budget=tris, width=64, height=64, spp=1,
                           env_texture=env_k)
        if maps_per_scene <= 0:
            out.append(sc)
            continue
        textures = []
        for m in range(maps_per_scene):
            sh = (int(rng.one() * map_size), int(rng.one() * map_size))
            tint = rng.uniform(3, 0.6, 1.0).astype(np.float32)
            textures.append(np.roll(base_map, sh, axis=(0, 1)) * tint)
        mats = []
        for mat in sc.materials:
            mat = dataclasses.replace(mat)
            if mat.kind == MAT_LAMBERT:
                mat.albedo_tex = int(rng.one() * maps_per_scene) % maps_per_scene
            elif mat.kind == MAT_GLOSSY:
                if rng.one() < 0.5:
                    mat.f0_tex = int(rng.one() * maps_per_scene) % maps_per_scene
                if rng.one() < 0.5:
                    mat.roughness_tex = int(rng.one() * maps_per_scene) % maps_per_scene
                    mat.roughness_map_strength = rng.one(0.5, 1.2)
            mats.append(mat)
        uv = sc.uvs.copy()
        flat = ~np.any(uv != 0.0, axis=1)  # grids: planar uvs
        uv[flat, 0] = 0.37 * sc.positions[flat, 0]
        uv[flat, 1] = 0.29 * sc.positions[flat, 1]
        out.append(sc.copy_with(materials=mats, uvs=uv.astype(np.float32), textures=textures))
    return out


def request_stream(seed: int, rate: float, count: int, n_scenes: int = 8,
                   px_lo: float = 128 ** 2, px_hi: float = 2048 ** 2, spps=(1, 8, 32, 128),
                   depth_lo: int = 4, depth_hi: int = 16):
    """Poisson arrivals: list of (arrival_s, scene index, width, height, spp, max_bounces)."""
    rng = Rng(seed)
    t = 0.0
    out = []
    for _ in range(count):
        t += -math.log1p(-rng.one()) / rate
        sc = int(rng.one() * n_scenes) % n_scenes
        px = math.exp(rng.one(math.log(px_lo), math.log(px_hi)))
        aspect = rng.one(0.5, 2.0)
        w = max(8, int(round(math.sqrt(px * aspect))))
        h = max(8, int(round(px / w)))
        spp = spps[int(rng.one() * len(spps)) % len(spps)]
        depth = depth_lo + int(rng.one() * (depth_hi - depth_lo + 1))
        out.append((t, sc, w, h, spp, min(depth, depth_hi)))
    return out


def uniform_lambert(scene: Scene, stride: int = 2) -> Scene:
    """The scene with importance sampling switched off (MaterialBase::
    EnableImportanceSampling(false): uniform hemisphere sampling) on every ``stride``-th
    Lambert material, counted in material order."""
    mats, k = [], 0
    for m in scene.materials:
        if m.kind == MAT_LAMBERT:
            if k % stride == 0:
                m = dataclasses.replace(m, importance_sampling=False)
            k += 1
        mats.append(m)
    return dataclasses.replace(scene, materials=mats)
