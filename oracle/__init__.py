"""CPU oracle for the path-tracing hot path (TEST INFRASTRUCTURE ONLY).

``liboracle.so`` (built from ``oracle/port/pt_oracle.cpp``) restates the
reference renderer's arithmetic; this module wraps its C ABI with ctypes.
Only the tests, ``__graft_entry__.smoke()`` and the benchmark's CPU-baseline leg
use it, as the checker. The reference renderer itself, compiled from its own
sources by ``oracle/ref/Makefile`` into ``oracle/_ref/``, pins this restatement
(see ``tests/golden/make_golden.py``).
"""
from __future__ import annotations

import ctypes
import io
import os
import subprocess
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "build", "liboracle.so")
REF_HARNESS = os.path.join(HERE, "_ref", "ref_harness")

_lib = None


def build(force: bool = False) -> str:
    """Compile the oracle restatement (plain g++, no FMA contraction)."""
    src = os.path.join(HERE, "port", "pt_oracle.cpp")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
        os.makedirs(os.path.dirname(LIB_PATH), exist_ok=True)
        subprocess.check_call(["g++", "-std=c++17", "-O3", "-ffp-contract=off", "-fno-fast-math",
                               "-shared", "-fPIC", "-pthread", "-o", LIB_PATH, src])
    return LIB_PATH


def reference_root() -> Optional[str]:
    """Where the reference checkout lives: $PETRICHOR_REF, else a ``reference``
    directory beside this repository; None when neither holds LibPetrichor."""
    env = os.environ.get("PETRICHOR_REF")
    cands = [env] if env else [os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")]
    for c in cands:
        if c and os.path.isdir(os.path.join(c, "LibPetrichor")):
            return c
    return None


def build_reference(ref_root: Optional[str] = None, jobs: int = 8) -> Optional[str]:
    """Compile the reference renderer's own sources + harness into oracle/_ref (if present)."""
    ref_root = ref_root or reference_root()
    if not ref_root or not os.path.isdir(os.path.join(ref_root, "LibPetrichor")):
        return None
    subprocess.check_call(["make", "-s", "-C", os.path.join(HERE, "ref"), f"REF={ref_root}",
                           f"-j{jobs}"])
    return REF_HARNESS


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        vp, i32, f32p, i32p = ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_float), \
            ctypes.POINTER(ctypes.c_int32)
        L.oracle_scene_parse.restype = vp
        L.oracle_scene_parse.argtypes = [ctypes.c_char_p, ctypes.c_size_t]
        L.oracle_scene_free.argtypes = [vp]
        L.oracle_bvh_build.restype = ctypes.c_double
        L.oracle_bvh_build.argtypes = [vp]
        L.oracle_bvh_size.argtypes = [vp, i32p, i32p, i32p]
        L.oracle_bvh_dump.argtypes = [vp, f32p, i32p, i32p]
        L.oracle_render.restype = ctypes.c_double
        L.oracle_render.argtypes = [vp, f32p, i32, i32, i32]
        L.oracle_num_tiles.argtypes = [vp]
        L.oracle_render_decorrelated.restype = ctypes.c_double
        L.oracle_render_decorrelated.argtypes = [vp, f32p, i32, ctypes.c_uint32]
        L.oracle_render_tiles_decorrelated.restype = ctypes.c_double
        L.oracle_render_tiles_decorrelated.argtypes = [vp, f32p, i32, i32p, i32, ctypes.c_uint32]
        L.oracle_render_tiles.restype = ctypes.c_double
        L.oracle_render_tiles.argtypes = [vp, f32p, i32, i32p, i32]
        L.oracle_hits.argtypes = [vp, ctypes.c_uint32, ctypes.c_uint32, f32p, i32p]
        L.oracle_trace.argtypes = [vp, i32, f32p, ctypes.c_float, ctypes.c_float, i32p, f32p]
        L.oracle_env.argtypes = [vp, i32, f32p]
        L.oracle_render_aov.restype = ctypes.c_double
        L.oracle_render_aov.argtypes = [vp, f32p, i32, i32, i32]
        _lib = L
    return _lib


def _fp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def _ip(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))


class OracleScene:
    """A parsed scene inside the oracle library."""

    def __init__(self, scene):
        from petrichor_gb300 import scene_io
        buf = io.BytesIO()
        scene_io.write_scene(buf, scene)
        data = buf.getvalue()
        self.scene = scene
        self._h = lib().oracle_scene_parse(data, len(data))
        if not self._h:
            raise ValueError("oracle could not parse the scene")

    def __del__(self):
        if getattr(self, "_h", None):
            lib().oracle_scene_free(self._h)
            self._h = None

    def build_bvh(self) -> float:
        return lib().oracle_bvh_build(self._h)

    def bvh(self):
        nn, ni, d = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        lib().oracle_bvh_size(self._h, ctypes.byref(nn), ctypes.byref(ni), ctypes.byref(d))
        b = np.zeros((nn.value, 6), np.float32)
        q = np.zeros((nn.value, 5), np.int32)
        ids = np.zeros(ni.value, np.int32)
        lib().oracle_bvh_dump(self._h, _fp(b), _ip(q), _ip(ids))
        return b, q, ids, d.value

    def num_tiles(self) -> int:
        return lib().oracle_num_tiles(self._h)

    def render(self, threads: int = 0, tile_begin: int = 0, tile_end: int = -1):
        s = self.scene.settings
        film = np.zeros((s.height, s.width, 3), np.float32)
        secs = lib().oracle_render(self._h, _fp(film), threads, tile_begin, tile_end)
        return film, secs

    def render_aov(self, aov: int, denoising_spp: int = 1, threads: int = 0):
        """AOV pass of Petrichor::Render: 0 UV, 1 denoising albedo, 2 denoising normal."""
        s = self.scene.settings
        film = np.zeros((s.height, s.width, 3), np.float32)
        lib().oracle_render_aov(self._h, _fp(film), threads, aov, denoising_spp)
        return film

    def render_decorrelated(self, seed: int, threads: int = 0):
        """Same integrator and arithmetic with independent per-tile random streams."""
        s = self.scene.settings
        film = np.zeros((s.height, s.width, 3), np.float32)
        secs = lib().oracle_render_decorrelated(self._h, _fp(film), threads, seed)
        return film, secs

    def render_tiles(self, tiles, threads: int = 0):
        """Render only the listed tile indices; returns (film, seconds, pixels rendered)."""
        s = self.scene.settings
        film = np.zeros((s.height, s.width, 3), np.float32)
        t = np.ascontiguousarray(tiles, np.int32)
        secs = lib().oracle_render_tiles(self._h, _fp(film), threads, _ip(t), t.size)
        nx, ny = s.width // s.tile_width, s.height // s.tile_height
        px = 0
        for k in t:
            i, j = int(k) % (nx + 1), int(k) // (nx + 1)
            w = s.tile_width if i != nx else s.width - nx * s.tile_width
            h = s.tile_height if j != ny else s.height - ny * s.tile_height
            px += w * h
        return film, secs, px

    def render_tiles_decorrelated(self, tiles, seed: int, threads: int = 0):
        """The listed tiles with independent per-tile random streams (seeded as in
        render_decorrelated); returns (film, seconds)."""
        s = self.scene.settings
        film = np.zeros((s.height, s.width, 3), np.float32)
        t = np.ascontiguousarray(tiles, np.int32)
        secs = lib().oracle_render_tiles_decorrelated(self._h, _fp(film), threads, _ip(t), t.size,
                                                      seed)
        return film, secs

    def tile_mask(self, tiles) -> np.ndarray:
        """Boolean (H, W) mask of the pixels of the listed tiles."""
        s = self.scene.settings
        m = np.zeros((s.height, s.width), bool)
        nx = s.width // s.tile_width
        for k in np.asarray(tiles).ravel():
            i, j = int(k) % (nx + 1), int(k) // (nx + 1)
            m[j * s.tile_height:(j + 1) * s.tile_height, i * s.tile_width:(i + 1) * s.tile_width] = True
        return m

    def hits(self, seed_a: int = 7, seed_b: int = 11):
        s = self.scene.settings
        rays = np.zeros((s.height * s.width, 8), np.float32)
        hits = np.zeros((s.height * s.width, 2), np.int32)
        lib().oracle_hits(self._h, seed_a, seed_b, _fp(rays), _ip(hits))
        return rays, hits

    def trace(self, rays: np.ndarray, dist_min: float = 0.0, dist_max: float = 3.4028235e38):
        rays = np.ascontiguousarray(rays[:, :6], np.float32)
        n = rays.shape[0]
        tri = np.zeros(n, np.int32)
        dist = np.zeros(n, np.float32)
        lib().oracle_trace(self._h, n, _fp(rays), dist_min, dist_max, _ip(tri), _fp(dist))
        return tri, dist

    def env_samples(self, n: int = 4096) -> np.ndarray:
        out = np.zeros((n, 8), np.float32)
        lib().oracle_env(self._h, n, _fp(out))
        return out


# ------------------------------------------------------------------ reference harness
def ref_available() -> bool:
    return os.path.exists(REF_HARNESS)


def run_reference(mode: str, scene, workdir: str, *args) -> bytes:
    """Run the compiled reference harness (present only where the reference was built)."""
    from petrichor_gb300 import scene_io
    os.makedirs(workdir, exist_ok=True)
    sp = os.path.join(workdir, f"scene_{os.getpid()}.ptscene")
    op = os.path.join(workdir, f"out_{os.getpid()}_{mode}.bin")
    scene_io.write_scene(sp, scene)
    subprocess.check_call([REF_HARNESS, mode, sp, op] + [str(a) for a in args],
                          stdout=subprocess.DEVNULL)
    with open(op, "rb") as fh:
        data = fh.read()
    os.remove(sp)
    os.remove(op)
    return data
