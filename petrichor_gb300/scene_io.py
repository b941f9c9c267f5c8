"""Scene description shared by the GPU path, the CPU oracle and the reference harness.

A scene is a plain set of numpy arrays plus a few scalars, mirroring what the
reference's C++ scene API receives (``LibPetrichor/Core/Scene.h:60-218``):

* vertices (``Vertex`` = pos, normal, uv; ``Core/Geometry/Vertex.h:20-22``),
* triangles with a shading type and a material index (``Triangle``,
  ``Core/Geometry/Triangle.h``; ``GeometryBase::SetMaterial``),
* a material table (Lambert / GGX / Glass / Emission / Mix,
  ``Core/Material/*.h``),
* the light list (``Scene::AppendLight``, ``Core/Scene.h:77-92``),
* the camera (``Core/Camera.h``), the environment (``Core/Environment.h``) and
  the render settings (``Core/RenderSetting.h``).

On disk the same content is one little-endian binary file (``.ptscene``)
so that the C++ reference harness, the CPU oracle and the C-ABI loader read
identical bytes.
"""
from __future__ import annotations

import dataclasses
import io
import struct
from typing import List, Optional

import numpy as np

MAGIC = b"PTSCENE1"

# Material kinds (values match MaterialTypes order in Core/Material/MaterialBase.h:15-22)
MAT_LAMBERT = 0
MAT_GLASS = 1
MAT_EMISSION = 2
MAT_GLOSSY = 3  # GGX
MAT_MIX = 4

SHADING_FLAT = 0
SHADING_SMOOTH = 1

INTEGRATOR_SIMPLE = 0  # SimplePathTracing (what Petrichor::Render runs)
INTEGRATOR_PT = 1      # PathTracing (MIS next-event estimation)


@dataclasses.dataclass
class Material:
    kind: int
    # Lambert: kd; GGX: reflectance strength ("f0" ctor argument); Glass: color; Emission: color
    color: tuple = (1.0, 1.0, 1.0)
    roughness: float = 1.0   # GGX
    ior: float = 1.333       # Glass (Glass::IOR::Water default)
    mix: float = 0.0         # Mix
    mat0: int = -1           # Mix
    mat1: int = -1           # Mix
    # texture maps (indices into Scene.textures, -1 = none): Lambert albedo
    # (Lambert::SetTexAlbedo); GGX reflectance, roughness and normal maps
    # (GGX::SetF0Texture / SetRoughnessMap / SetNormalMap) with their strengths
    albedo_tex: int = -1
    f0_tex: int = -1
    roughness_tex: int = -1
    normal_tex: int = -1
    roughness_map_strength: float = 1.0
    normal_map_strength: float = 1.0
    # MaterialBase::EnableImportanceSampling (MaterialBase.h:52-62); only Lambert reads it
    # (Lambert.cpp:40-47,66-107: off = uniform hemisphere sampling)
    importance_sampling: bool = True


@dataclasses.dataclass
class Camera:
    pos: tuple = (0.0, 0.0, 0.0)
    view_dir: tuple = (1.0, 0.0, 0.0)
    fov: float = 0.0            # vertical FOV in radians; <= 0 keeps the focal length
    focal_length: float = 55e-3  # used when fov <= 0 (Camera::SetFocalLength)
    focus_target: Optional[tuple] = None  # Camera::FocusTo; None keeps focusDist = 1
    aperture: float = 25e-3      # Camera::SetApeture (reference default 25 mm)


@dataclasses.dataclass
class Settings:
    width: int = 256
    height: int = 256
    spp: int = 16
    max_bounces: int = 16
    tile_width: int = 16
    tile_height: int = 16
    num_threads: int = 0
    integrator: int = INTEGRATOR_SIMPLE


@dataclasses.dataclass
class Environment:
    base_color: tuple = (0.0, 0.0, 0.0)
    z_rotation: float = 0.0
    texture: Optional[np.ndarray] = None   # (H, W, 3) float32, row-major, or None
    use_importance_sampling: bool = True


@dataclasses.dataclass
class Scene:
    positions: np.ndarray       # (V, 3) float32
    normals: np.ndarray         # (V, 3) float32
    uvs: np.ndarray             # (V, 3) float32
    indices: np.ndarray         # (T, 3) int32
    tri_material: np.ndarray    # (T,) int32
    tri_shading: np.ndarray     # (T,) uint8
    lights: np.ndarray          # (L,) int32 triangle indices
    materials: List[Material]
    camera: Camera
    env: Environment
    settings: Settings
    textures: List[np.ndarray] = dataclasses.field(default_factory=list)  # (H, W, 3) float32

    @property
    def num_triangles(self) -> int:
        return int(self.indices.shape[0])

    def copy_with(self, **kw) -> "Scene":
        return dataclasses.replace(self, **kw)


def _f32(a, shape_last=None):
    a = np.ascontiguousarray(np.asarray(a, dtype=np.float32))
    return a


def material_table(mats: List[Material]) -> np.ndarray:
    """Pack materials as a (M, 8) float32 table + (M, 4) int32 table.

    float row: color.rgb, roughness, ior, mix, roughness-map strength, normal-map strength
    int row:   kind, mat0, mat1, texture references (one byte each, texture index + 1,
               0 = none: albedo | f0 << 8 | roughness << 16 | normal << 24)
    """
    f = np.zeros((len(mats), 8), np.float32)
    i = np.zeros((len(mats), 4), np.int32)
    for k, m in enumerate(mats):
        f[k, 0:3] = m.color
        f[k, 3] = m.roughness
        f[k, 4] = m.ior
        f[k, 5] = m.mix
        f[k, 6] = m.roughness_map_strength
        f[k, 7] = m.normal_map_strength
        i[k, 0] = m.kind
        i[k, 1] = m.mat0
        i[k, 2] = m.mat1
        refs = (m.albedo_tex, m.f0_tex, m.roughness_tex, m.normal_tex)
        assert all(-1 <= r < 255 for r in refs)
        i[k, 3] = np.int32(np.uint32(sum((r + 1) << (8 * j) for j, r in enumerate(refs))))
    return f, i


def write_scene(path_or_buf, sc: Scene) -> None:
    out = io.BytesIO()
    w = out.write
    w(MAGIC)
    s = sc.settings
    w(struct.pack("<8i", s.width, s.height, s.spp, s.max_bounces, s.tile_width,
                  s.tile_height, s.num_threads, s.integrator))
    c = sc.camera
    has_focus = 1 if c.focus_target is not None else 0
    ft = c.focus_target if c.focus_target is not None else (0.0, 0.0, 0.0)
    w(struct.pack("<3f3ff f3ffI", *c.pos, *c.view_dir, c.fov, c.focal_length, *ft,
                  c.aperture, has_focus))
    e = sc.env
    tex = e.texture
    ew, eh = (0, 0) if tex is None else (tex.shape[1], tex.shape[0])
    w(struct.pack("<3ffiiI", *e.base_color, e.z_rotation, ew, eh,
                  1 if e.use_importance_sampling else 0))
    if tex is not None:
        w(np.ascontiguousarray(tex, np.float32).tobytes())
    mf, mi = material_table(sc.materials)
    w(struct.pack("<I", len(sc.materials)))
    w(mf.tobytes())
    w(mi.tobytes())
    V = sc.positions.shape[0]
    w(struct.pack("<I", V))
    for a in (sc.positions, sc.normals, sc.uvs):
        a = np.ascontiguousarray(a, np.float32)
        assert a.shape == (V, 3)
        w(a.tobytes())
    T = sc.indices.shape[0]
    w(struct.pack("<I", T))
    w(np.ascontiguousarray(sc.indices, np.int32).tobytes())
    w(np.ascontiguousarray(sc.tri_material, np.int32).tobytes())
    sh = np.ascontiguousarray(sc.tri_shading, np.uint8)
    pad = (-T) % 4
    w(sh.tobytes() + b"\0" * pad)
    L = sc.lights.shape[0]
    w(struct.pack("<I", L))
    w(np.ascontiguousarray(sc.lights, np.int32).tobytes())
    flags = [0 if m.importance_sampling else 1 for m in sc.materials]
    if sc.textures or any(flags):  # optional trailing section: material texture maps
        w(struct.pack("<I", len(sc.textures)))
        for t in sc.textures:
            t = np.ascontiguousarray(t, np.float32)
            w(struct.pack("<ii", t.shape[1], t.shape[0]))
            w(t.tobytes())
    if any(flags):  # optional trailing section: per-material flags (bit 0: importance sampling off)
        w(struct.pack("<I", len(flags)))
        w(np.asarray(flags, np.uint32).tobytes())
    data = out.getvalue()
    if hasattr(path_or_buf, "write"):
        path_or_buf.write(data)
    else:
        with open(path_or_buf, "wb") as fh:
            fh.write(data)


def read_scene(path) -> Scene:
    with open(path, "rb") as fh:
        return read_scene_bytes(fh.read())


def scene_bytes(sc: Scene) -> bytes:
    buf = io.BytesIO()
    write_scene(buf, sc)
    return buf.getvalue()


def read_scene_bytes(data: bytes) -> Scene:
    off = 0

    def take(n):
        nonlocal off
        b = data[off:off + n]
        if len(b) != n:
            raise ValueError("truncated .ptscene")
        off += n
        return b

    if take(8) != MAGIC:
        raise ValueError("not a .ptscene file")
    st = struct.unpack("<8i", take(32))
    settings = Settings(*st)
    cv = struct.unpack("<3f3ff f3ffI", take(4 * 13))
    cam = Camera(pos=tuple(cv[0:3]), view_dir=tuple(cv[3:6]), fov=cv[6], focal_length=cv[7],
                 focus_target=tuple(cv[8:11]) if cv[12] else None, aperture=cv[11])
    ev = struct.unpack("<3ffiiI", take(4 * 7))
    ew, eh = ev[4], ev[5]
    tex = None
    if ew > 0 and eh > 0:
        tex = np.frombuffer(take(ew * eh * 12), np.float32).reshape(eh, ew, 3).copy()
    env = Environment(base_color=tuple(ev[0:3]), z_rotation=ev[3], texture=tex,
                      use_importance_sampling=bool(ev[6]))
    (M,) = struct.unpack("<I", take(4))
    mf = np.frombuffer(take(M * 32), np.float32).reshape(M, 8)
    mi = np.frombuffer(take(M * 16), np.int32).reshape(M, 4)
    def refs(v):
        u = int(np.uint32(v))
        return [((u >> (8 * j)) & 255) - 1 for j in range(4)]
    mats = [Material(kind=int(mi[k, 0]), color=tuple(float(x) for x in mf[k, 0:3]),
                     roughness=float(mf[k, 3]), ior=float(mf[k, 4]), mix=float(mf[k, 5]),
                     mat0=int(mi[k, 1]), mat1=int(mi[k, 2]),
                     albedo_tex=refs(mi[k, 3])[0], f0_tex=refs(mi[k, 3])[1],
                     roughness_tex=refs(mi[k, 3])[2], normal_tex=refs(mi[k, 3])[3],
                     roughness_map_strength=float(mf[k, 6]), normal_map_strength=float(mf[k, 7]))
            for k in range(M)]
    (V,) = struct.unpack("<I", take(4))
    pos = np.frombuffer(take(V * 12), np.float32).reshape(V, 3).copy()
    nrm = np.frombuffer(take(V * 12), np.float32).reshape(V, 3).copy()
    uv = np.frombuffer(take(V * 12), np.float32).reshape(V, 3).copy()
    (T,) = struct.unpack("<I", take(4))
    idx = np.frombuffer(take(T * 12), np.int32).reshape(T, 3).copy()
    tm = np.frombuffer(take(T * 4), np.int32).copy()
    sh = np.frombuffer(take(T + ((-T) % 4)), np.uint8)[:T].copy()
    (L,) = struct.unpack("<I", take(4))
    lights = np.frombuffer(take(L * 4), np.int32).copy()
    textures = []
    if off < len(data):
        (NT,) = struct.unpack("<I", take(4))
        for _ in range(NT):
            tw, th = struct.unpack("<ii", take(8))
            textures.append(np.frombuffer(take(tw * th * 12), np.float32).reshape(th, tw, 3).copy())
    if off < len(data):
        (NM,) = struct.unpack("<I", take(4))
        if NM != M:
            raise ValueError("material flag count does not match the material table")
        fl = np.frombuffer(take(4 * NM), np.uint32)
        mats = [dataclasses.replace(m, importance_sampling=not bool(f & 1)) for m, f in zip(mats, fl)]
    return Scene(pos, nrm, uv, idx, tm, sh, lights, mats, cam, env, settings, textures)
