"""ctypes binding of the C ABI in ``include/petrichor_gb300.h``.

This is the host-side mirror of the reference's render call for Python users:
``Context.upload(scene)`` plays the part of filling a ``Petrichor::Core::Scene``
and ``Context.render(...)`` the part of ``Petrichor::Render(scene)``
(``LibPetrichor/Core/Petrichor.cpp:35-264``), writing a film with the layout of
``Texture2D::GetRawDataPtr`` (row-major RGB float32).

The library is built in-tree (``petrichor_gb300/_lib``); there is no fallback:
if it is missing or no CUDA device is present, the calls raise.
"""
from __future__ import annotations

import ctypes
import os
from typing import Optional

import numpy as np

from . import _build
from .scene_io import Scene, INTEGRATOR_SIMPLE, INTEGRATOR_PT

PT_OK = 0
MODE_REPLAY = 0
MODE_WAVEFRONT = 1
ENV_SAMPLING_REFERENCE, ENV_SAMPLING_ALIAS = 0, 1
AOV_UV, AOV_DENOISING_ALBEDO, AOV_DENOISING_NORMAL = 0, 1, 2

_f3 = ctypes.c_float * 3


class PtMaterial(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("color", _f3), ("roughness", ctypes.c_float),
                ("ior", ctypes.c_float), ("mix", ctypes.c_float), ("mat0", ctypes.c_int32),
                ("mat1", ctypes.c_int32), ("tex_albedo", ctypes.c_int32),
                ("tex_f0", ctypes.c_int32), ("tex_roughness", ctypes.c_int32),
                ("tex_normal", ctypes.c_int32), ("roughness_strength", ctypes.c_float),
                ("normal_strength", ctypes.c_float), ("uniform_sampling", ctypes.c_int32)]


class PtTexture(ctypes.Structure):
    _fields_ = [("width", ctypes.c_int32), ("height", ctypes.c_int32), ("rgb", ctypes.c_void_p)]


class PtSceneDesc(ctypes.Structure):
    _fields_ = [("num_vertices", ctypes.c_uint32), ("positions", ctypes.c_void_p),
                ("normals", ctypes.c_void_p), ("uvs", ctypes.c_void_p),
                ("num_triangles", ctypes.c_uint32), ("indices", ctypes.c_void_p),
                ("tri_material", ctypes.c_void_p), ("tri_shading", ctypes.c_void_p),
                ("num_materials", ctypes.c_uint32), ("materials", ctypes.POINTER(PtMaterial)),
                ("num_lights", ctypes.c_uint32), ("lights", ctypes.c_void_p),
                ("env_base_color", _f3), ("env_z_rotation", ctypes.c_float),
                ("env_width", ctypes.c_int32), ("env_height", ctypes.c_int32),
                ("env_rgb", ctypes.c_void_p), ("num_textures", ctypes.c_uint32),
                ("textures", ctypes.POINTER(PtTexture))]


class PtCamera(ctypes.Structure):
    _fields_ = [("pos", _f3), ("right", _f3), ("up", _f3), ("forward", _f3),
                ("h_perf", ctypes.c_float), ("focus_dist", ctypes.c_float),
                ("aperture", ctypes.c_float), ("reserved", ctypes.c_float)]


class PtSettings(ctypes.Structure):
    _fields_ = [("width", ctypes.c_int32), ("height", ctypes.c_int32), ("spp", ctypes.c_int32),
                ("max_bounces", ctypes.c_int32), ("tile_width", ctypes.c_int32),
                ("tile_height", ctypes.c_int32), ("integrator", ctypes.c_int32),
                ("mode", ctypes.c_int32), ("seed", ctypes.c_uint32),
                ("wave_paths", ctypes.c_int32), ("denoising_spp", ctypes.c_int32),
                ("env_sampling", ctypes.c_int32)]


class PtJob(ctypes.Structure):
    _fields_ = [("scene", ctypes.c_int32), ("camera", PtCamera), ("settings", PtSettings),
                ("film_device", ctypes.c_void_p)]


class PtServeConfig(ctypes.Structure):
    _fields_ = [("wave_paths", ctypes.c_int32), ("max_active", ctypes.c_int32),
                ("state_budget", ctypes.c_uint64)]


class PtRequestStatus(ctypes.Structure):
    _fields_ = [("state", ctypes.c_int32), ("status", ctypes.c_int32), ("submit_s", ctypes.c_double),
                ("admit_s", ctypes.c_double), ("done_s", ctypes.c_double),
                ("samples_done", ctypes.c_uint32), ("samples_total", ctypes.c_uint32)]


REQ_QUEUED, REQ_RUNNING, REQ_DONE, REQ_CANCELLED, REQ_FAILED = range(5)


class PtBvhBuildStats(ctypes.Structure):
    _fields_ = [("device_ms", ctypes.c_double), ("levels", ctypes.c_int32), ("rounds", ctypes.c_int32),
                ("heapsorts", ctypes.c_int32), ("launches", ctypes.c_int32)]


class PtSceneInfo(ctypes.Structure):
    _fields_ = [("num_triangles", ctypes.c_uint32), ("num_nodes", ctypes.c_uint32),
                ("tree_height", ctypes.c_uint32), ("num_lights", ctypes.c_uint32),
                ("device_bytes", ctypes.c_uint64), ("build_seconds", ctypes.c_double),
                ("bvh_builder", ctypes.c_int32), ("reserved", ctypes.c_int32)]


class PtStats(ctypes.Structure):
    _fields_ = [("last_render_ms", ctypes.c_double), ("kernel_launches", ctypes.c_uint64),
                ("device_bytes_in_use", ctypes.c_uint64), ("memory_budget", ctypes.c_uint64),
                ("renders", ctypes.c_uint64), ("last_device_status", ctypes.c_int32),
                ("reserved", ctypes.c_int32)]


class PtProfile(ctypes.Structure):
    _fields_ = [("raygen_ms", ctypes.c_double), ("extend_ms", ctypes.c_double),
                ("shade_ms", ctypes.c_double), ("shadow_ms", ctypes.c_double),
                ("accumulate_ms", ctypes.c_double), ("extend_rays", ctypes.c_uint64),
                ("shadow_rays", ctypes.c_uint64), ("extend_launches", ctypes.c_uint64),
                ("shadow_launches", ctypes.c_uint64), ("ref_node_tests", ctypes.c_uint64),
                ("ref_tri_tests", ctypes.c_uint64), ("ref_rays", ctypes.c_uint64),
                ("raster_ms", ctypes.c_double), ("raster_paths", ctypes.c_uint64)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class PtTuning(ctypes.Structure):
    _fields_ = [("wave_paths", ctypes.c_int32), ("blocks_per_sm", ctypes.c_int32),
                ("band_rows", ctypes.c_int32), ("use_graphs", ctypes.c_int32),
                ("sort_rays", ctypes.c_int32), ("tail_bounce", ctypes.c_int32),
                ("primary_traversal", ctypes.c_int32), ("reserved", ctypes.c_int32),
                ("probe_ms", ctypes.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


# Every symbol declared in include/petrichor_gb300.h (checked by the CPU tests).
EXPORTED = [
    "pt_abi_version", "pt_status_string", "pt_context_create", "pt_context_destroy",
    "pt_last_error", "pt_camera_init", "pt_scene_upload", "pt_scene_release",
    "pt_scene_info_get", "pt_render", "pt_render_device", "pt_trace_closest", "pt_get_stats",
    "pt_get_progress", "pt_bvh_build", "pt_render_profile", "pt_render_replay_noalloc", "pt_batch_render",
    "pt_probe_bandwidth",
    "pt_serve_start", "pt_serve_submit", "pt_serve_poll", "pt_serve_wait", "pt_serve_cancel",
    "pt_serve_release", "pt_serve_stop", "pt_autotune", "pt_set_tuning", "pt_get_tuning",
    "pt_render_aov", "pt_render_aov_device", "pt_bvh_build_device", "pt_set_bvh_builder",
    "pt_denoise", "pt_denoise_device", "pt_serve_set_deadline", "pt_primary_hits",
]

BVH_BUILDER_HOST, BVH_BUILDER_DEVICE = 0, 1

_lib = None


class PtError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{msg} (status {status})")
        self.status = status


def load(build: bool = True):
    """Load (building first if needed) the in-tree CUDA library. PT_GB300_CHECKED=1
    loads the checked build instead (device-side bounds checks; for the tests)."""
    global _lib
    if _lib is not None:
        return _lib
    if os.environ.get("PT_GB300_CHECKED") == "1":
        path = _build.build_checked() if build else os.path.join(_build.CHECK_DIR, "libpetrichor_gb300.so")
    else:
        path = _build.build() if build else _build.LIB
    if not os.path.exists(path):
        raise RuntimeError(f"CUDA library not built: {path}")
    L = ctypes.CDLL(path)
    vp, i32, u32 = ctypes.c_void_p, ctypes.c_int32, ctypes.c_uint32
    L.pt_abi_version.restype = ctypes.c_int
    L.pt_status_string.restype = ctypes.c_char_p
    L.pt_status_string.argtypes = [ctypes.c_int]
    L.pt_context_create.argtypes = [ctypes.c_int, ctypes.c_uint64, ctypes.POINTER(vp)]
    L.pt_context_destroy.argtypes = [vp]
    L.pt_last_error.restype = ctypes.c_char_p
    L.pt_last_error.argtypes = [vp]
    L.pt_camera_init.argtypes = [ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float),
                                 ctypes.c_float, ctypes.c_float, ctypes.POINTER(ctypes.c_float),
                                 ctypes.c_float, ctypes.POINTER(PtCamera)]
    L.pt_scene_upload.argtypes = [vp, ctypes.POINTER(PtSceneDesc), ctypes.POINTER(i32)]
    L.pt_scene_release.argtypes = [vp, i32]
    L.pt_scene_info_get.argtypes = [vp, i32, ctypes.POINTER(PtSceneInfo)]
    L.pt_render.argtypes = [vp, i32, ctypes.POINTER(PtCamera), ctypes.POINTER(PtSettings), vp]
    L.pt_render_device.argtypes = [vp, i32, ctypes.POINTER(PtCamera), ctypes.POINTER(PtSettings),
                                   vp, vp]
    L.pt_trace_closest.argtypes = [vp, i32, i32, vp, ctypes.c_float, ctypes.c_float, vp, vp, vp]
    L.pt_primary_hits.argtypes = [vp, i32, ctypes.POINTER(PtCamera), ctypes.POINTER(PtSettings),
                                  vp, vp, vp, vp]
    L.pt_get_stats.argtypes = [vp, ctypes.POINTER(PtStats)]
    L.pt_batch_render.argtypes = [vp, i32, ctypes.POINTER(PtJob), vp]
    u64 = ctypes.c_uint64
    L.pt_serve_start.argtypes = [vp, ctypes.POINTER(PtServeConfig)]
    L.pt_serve_submit.argtypes = [vp, ctypes.POINTER(PtJob), vp, ctypes.POINTER(u64)]
    L.pt_serve_poll.argtypes = [vp, u64, ctypes.POINTER(PtRequestStatus)]
    L.pt_serve_wait.argtypes = [vp, u64, ctypes.c_double, ctypes.POINTER(PtRequestStatus)]
    L.pt_serve_cancel.argtypes = [vp, u64]
    L.pt_serve_release.argtypes = [vp, u64]
    L.pt_serve_stop.argtypes = [vp]
    L.pt_render_replay_noalloc.argtypes = [vp, i32, ctypes.POINTER(PtCamera),
                                           ctypes.POINTER(PtSettings), vp, vp]
    L.pt_render_profile.argtypes = [vp, i32, ctypes.POINTER(PtCamera), ctypes.POINTER(PtSettings),
                                    vp, i32, ctypes.POINTER(PtProfile)]
    L.pt_get_progress.argtypes = [vp, ctypes.POINTER(u32), ctypes.POINTER(u32)]
    L.pt_probe_bandwidth.argtypes = [vp, ctypes.c_uint64, i32, i32, ctypes.POINTER(ctypes.c_double)]
    L.pt_autotune.argtypes = [vp, i32, ctypes.POINTER(PtCamera), ctypes.POINTER(PtSettings), i32,
                              ctypes.POINTER(PtTuning)]
    L.pt_set_tuning.argtypes = [vp, ctypes.POINTER(PtTuning)]
    L.pt_render_aov.argtypes = [vp, i32, ctypes.POINTER(PtCamera), ctypes.POINTER(PtSettings), i32, vp]
    L.pt_render_aov_device.argtypes = [vp, i32, ctypes.POINTER(PtCamera), ctypes.POINTER(PtSettings),
                                       i32, vp, vp]
    L.pt_get_tuning.argtypes = [vp, ctypes.POINTER(PtTuning)]
    L.pt_bvh_build.argtypes = [vp, u32, vp, u32, i32, ctypes.POINTER(u32), ctypes.POINTER(u32),
                               vp, vp, vp]
    L.pt_bvh_build_device.argtypes = [vp, vp, u32, vp, u32, ctypes.POINTER(u32), ctypes.POINTER(u32),
                                      vp, vp, vp, ctypes.POINTER(PtBvhBuildStats)]
    L.pt_set_bvh_builder.argtypes = [vp, i32]
    L.pt_denoise.argtypes = [vp, i32, i32, vp, vp, vp, i32, vp]
    L.pt_serve_set_deadline.argtypes = [vp, ctypes.c_uint64, ctypes.c_double]
    L.pt_denoise_device.argtypes = [vp, i32, i32, vp, vp, vp, i32, vp, vp]
    _lib = L
    return L


def _fptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def camera_from_scene(scene: Scene) -> PtCamera:
    L = load()
    c = scene.camera
    pos = np.asarray(c.pos, np.float32)
    d = np.asarray(c.view_dir, np.float32)
    ft = None if c.focus_target is None else np.asarray(c.focus_target, np.float32)
    out = PtCamera()
    rc = L.pt_camera_init(_fptr(pos), _fptr(d), c.fov, c.focal_length,
                          _fptr(ft) if ft is not None else None, c.aperture, ctypes.byref(out))
    if rc != PT_OK:
        raise PtError(rc, "pt_camera_init failed")
    return out


def settings_from_scene(scene: Scene, mode: int = MODE_REPLAY, seed: int = 1, **over) -> PtSettings:
    s = scene.settings
    st = PtSettings()
    st.width = over.get("width", s.width)
    st.height = over.get("height", s.height)
    st.spp = over.get("spp", s.spp)
    st.max_bounces = over.get("max_bounces", s.max_bounces)
    st.tile_width = over.get("tile_width", s.tile_width)
    st.tile_height = over.get("tile_height", s.tile_height)
    st.integrator = over.get("integrator", s.integrator)
    st.mode = mode
    st.seed = seed
    st.wave_paths = over.get("wave_paths", 0)
    st.denoising_spp = over.get("denoising_spp", 0)
    st.env_sampling = over.get("env_sampling", ENV_SAMPLING_REFERENCE)
    return st


class Context:
    """One CUDA device context of the path-tracing core."""

    def __init__(self, device: int = 0, memory_budget: int = 0):
        self.L = load()
        h = ctypes.c_void_p()
        rc = self.L.pt_context_create(device, memory_budget, ctypes.byref(h))
        if rc != PT_OK:
            raise PtError(rc, "pt_context_create failed: " +
                          self.L.pt_status_string(rc).decode())
        self.h = h
        self._keep = {}

    def close(self):
        if getattr(self, "h", None):
            self.L.pt_context_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, rc: int, what: str):
        if rc != PT_OK:
            raise PtError(rc, f"{what}: {self.L.pt_last_error(self.h).decode()}")

    def upload(self, scene: Scene) -> int:
        pos = np.ascontiguousarray(scene.positions, np.float32)
        nrm = np.ascontiguousarray(scene.normals, np.float32)
        uvs = np.ascontiguousarray(scene.uvs, np.float32)
        idx = np.ascontiguousarray(scene.indices, np.int32)
        tm = np.ascontiguousarray(scene.tri_material, np.int32)
        sh = np.ascontiguousarray(scene.tri_shading, np.uint8)
        lights = np.ascontiguousarray(scene.lights, np.int32)
        mats = (PtMaterial * max(1, len(scene.materials)))()
        for k, m in enumerate(scene.materials):
            mats[k].kind = m.kind
            mats[k].color = _f3(*m.color)
            mats[k].roughness = m.roughness
            mats[k].ior = m.ior
            mats[k].mix = m.mix
            mats[k].mat0 = m.mat0
            mats[k].mat1 = m.mat1
            # texture references are 1 + index (0: none)
            mats[k].tex_albedo = m.albedo_tex + 1
            mats[k].tex_f0 = m.f0_tex + 1
            mats[k].tex_roughness = m.roughness_tex + 1
            mats[k].tex_normal = m.normal_tex + 1
            mats[k].roughness_strength = m.roughness_map_strength
            mats[k].normal_strength = m.normal_map_strength
            mats[k].uniform_sampling = 0 if m.importance_sampling else 1
        texels = [np.ascontiguousarray(t, np.float32) for t in scene.textures]
        texs = (PtTexture * max(1, len(texels)))()
        for k, t in enumerate(texels):
            texs[k].width, texs[k].height = t.shape[1], t.shape[0]
            texs[k].rgb = t.ctypes.data
        d = PtSceneDesc()
        d.num_textures = len(texels)
        d.textures = texs
        d.num_vertices = pos.shape[0]
        d.positions = pos.ctypes.data
        d.normals = nrm.ctypes.data
        d.uvs = uvs.ctypes.data
        d.num_triangles = idx.shape[0]
        d.indices = idx.ctypes.data
        d.tri_material = tm.ctypes.data
        d.tri_shading = sh.ctypes.data
        d.num_materials = len(scene.materials)
        d.materials = mats
        d.num_lights = lights.shape[0]
        d.lights = lights.ctypes.data if lights.size else None
        e = scene.env
        d.env_base_color = _f3(*e.base_color)
        d.env_z_rotation = e.z_rotation
        env = None
        if e.texture is not None:
            env = np.ascontiguousarray(e.texture, np.float32)
            d.env_width, d.env_height = env.shape[1], env.shape[0]
            d.env_rgb = env.ctypes.data
        sid = ctypes.c_int32()
        self._check(self.L.pt_scene_upload(self.h, ctypes.byref(d), ctypes.byref(sid)),
                    "pt_scene_upload")
        return sid.value

    def release(self, sid: int):
        self._check(self.L.pt_scene_release(self.h, sid), "pt_scene_release")

    def scene_info(self, sid: int) -> PtSceneInfo:
        info = PtSceneInfo()
        self._check(self.L.pt_scene_info_get(self.h, sid, ctypes.byref(info)), "pt_scene_info_get")
        return info

    def render(self, sid: int, camera: PtCamera, settings: PtSettings,
               out: Optional[np.ndarray] = None) -> np.ndarray:
        if out is None:
            out = np.empty((settings.height, settings.width, 3), np.float32)
        assert out.flags.c_contiguous and out.dtype == np.float32
        assert out.size == settings.width * settings.height * 3
        self._check(self.L.pt_render(self.h, sid, ctypes.byref(camera), ctypes.byref(settings),
                                     out.ctypes.data), "pt_render")
        return out

    def render_aov(self, sid: int, camera: PtCamera, settings: PtSettings, aov: int,
                   out: Optional[np.ndarray] = None) -> np.ndarray:
        """AOV pass (AOV_UV, AOV_DENOISING_ALBEDO, AOV_DENOISING_NORMAL) into a host film."""
        if out is None:
            out = np.empty((settings.height, settings.width, 3), np.float32)
        assert out.flags.c_contiguous and out.dtype == np.float32
        assert out.size == settings.width * settings.height * 3
        self._check(self.L.pt_render_aov(self.h, sid, ctypes.byref(camera), ctypes.byref(settings),
                                         aov, out.ctypes.data), "pt_render_aov")
        return out

    def render_aov_device(self, sid: int, camera: PtCamera, settings: PtSettings, aov: int,
                          film_ptr: int, stream_ptr: int = 0):
        self._check(self.L.pt_render_aov_device(self.h, sid, ctypes.byref(camera),
                                                ctypes.byref(settings), aov, film_ptr,
                                                stream_ptr or None), "pt_render_aov_device")

    def render_device(self, sid: int, camera: PtCamera, settings: PtSettings, film_ptr: int,
                      stream_ptr: int = 0):
        self._check(self.L.pt_render_device(self.h, sid, ctypes.byref(camera),
                                            ctypes.byref(settings), film_ptr, stream_ptr or None),
                    "pt_render_device")

    def batch_render(self, jobs, stream_ptr: int = 0):
        """jobs: list of (scene id, PtCamera, PtSettings, device film pointer)."""
        arr = (PtJob * len(jobs))()
        for k, (sid, cam, st, film) in enumerate(jobs):
            arr[k].scene = sid
            arr[k].camera = cam
            arr[k].settings = st
            arr[k].film_device = film
        self._check(self.L.pt_batch_render(self.h, len(jobs), arr, stream_ptr or None),
                    "pt_batch_render")

    # ---- serving loop
    def serve_start(self, wave_paths: int = 0, max_active: int = 0, state_budget: int = 0):
        cfg = PtServeConfig(wave_paths, max_active, state_budget)
        self._check(self.L.pt_serve_start(self.h, ctypes.byref(cfg)), "pt_serve_start")

    def serve_submit(self, sid: int, camera: PtCamera, settings: PtSettings, film_device: int = 0,
                     film_host: Optional[np.ndarray] = None) -> int:
        job = PtJob()
        job.scene = sid
        job.camera = camera
        job.settings = settings
        job.film_device = film_device or None
        rid = ctypes.c_uint64()
        host = film_host.ctypes.data if film_host is not None else None
        self._check(self.L.pt_serve_submit(self.h, ctypes.byref(job), host, ctypes.byref(rid)),
                    "pt_serve_submit")
        return rid.value

    def serve_poll(self, rid: int) -> PtRequestStatus:
        st = PtRequestStatus()
        self._check(self.L.pt_serve_poll(self.h, rid, ctypes.byref(st)), "pt_serve_poll")
        return st

    def serve_wait(self, rid: int, timeout: float = 60.0) -> PtRequestStatus:
        st = PtRequestStatus()
        rc = self.L.pt_serve_wait(self.h, rid, timeout, ctypes.byref(st))
        if rc not in (PT_OK, -4):
            self._check(rc, "pt_serve_wait")
        return st

    def serve_set_deadline(self, rid: int, seconds: float):
        self._check(self.L.pt_serve_set_deadline(self.h, rid, seconds), "pt_serve_set_deadline")

    def serve_cancel(self, rid: int):
        self._check(self.L.pt_serve_cancel(self.h, rid), "pt_serve_cancel")

    def serve_release(self, rid: int):
        self._check(self.L.pt_serve_release(self.h, rid), "pt_serve_release")

    def serve_stop(self):
        self._check(self.L.pt_serve_stop(self.h), "pt_serve_stop")

    def render_profile(self, sid: int, camera: PtCamera, settings: PtSettings, film_ptr: int,
                       count_reference: bool = True) -> PtProfile:
        p = PtProfile()
        self._check(self.L.pt_render_profile(self.h, sid, ctypes.byref(camera), ctypes.byref(settings),
                                             film_ptr, 1 if count_reference else 0, ctypes.byref(p)),
                    "pt_render_profile")
        return p

    def autotune(self, sid: int, camera: PtCamera, settings: PtSettings, probe_spp: int = 0) -> PtTuning:
        t = PtTuning()
        self._check(self.L.pt_autotune(self.h, sid, ctypes.byref(camera), ctypes.byref(settings),
                                       probe_spp, ctypes.byref(t)), "pt_autotune")
        return t

    def denoise(self, color: np.ndarray, albedo: Optional[np.ndarray] = None,
                normal: Optional[np.ndarray] = None, hdr: bool = True) -> np.ndarray:
        """GPU denoiser (pt_denoise) on (H, W, 3) float32 images; albedo/normal optional."""
        c = np.ascontiguousarray(color, np.float32)
        H, W, _ = c.shape
        guides = []
        for g in (albedo, normal):
            if g is None:
                guides.append(None)
                continue
            g = np.ascontiguousarray(g, np.float32)
            assert g.shape == c.shape
            guides.append(g)
        out = np.empty_like(c)
        self._check(self.L.pt_denoise(self.h, W, H, c.ctypes.data,
                                      guides[0].ctypes.data if guides[0] is not None else None,
                                      guides[1].ctypes.data if guides[1] is not None else None,
                                      1 if hdr else 0, out.ctypes.data), "pt_denoise")
        return out

    def denoise_device(self, width: int, height: int, color_ptr: int, albedo_ptr: int, normal_ptr: int,
                       hdr: bool, out_ptr: int, stream_ptr: int = 0):
        self._check(self.L.pt_denoise_device(self.h, width, height, color_ptr, albedo_ptr or None,
                                             normal_ptr or None, 1 if hdr else 0, out_ptr,
                                             stream_ptr or None), "pt_denoise_device")

    def set_bvh_builder(self, builder: int):
        self._check(self.L.pt_set_bvh_builder(self.h, builder), "pt_set_bvh_builder")

    def bvh_build_device(self, positions: np.ndarray, indices: np.ndarray):
        """Device binned-SAH build: (bounds (N,6), ints (N,5), prim_ids (T,), height, stats)."""
        pos = np.ascontiguousarray(positions, np.float32)
        idx = np.ascontiguousarray(indices, np.int32)
        cap = max(1, 2 * idx.shape[0])
        b = np.zeros((cap, 6), np.float32)
        q = np.zeros((cap, 5), np.int32)
        ids = np.zeros(idx.shape[0], np.int32)
        n, h, st = ctypes.c_uint32(), ctypes.c_uint32(), PtBvhBuildStats()
        self._check(self.L.pt_bvh_build_device(self.h, pos.ctypes.data, pos.shape[0], idx.ctypes.data,
                                               idx.shape[0], ctypes.byref(n), ctypes.byref(h),
                                               b.ctypes.data, q.ctypes.data, ids.ctypes.data,
                                               ctypes.byref(st)), "pt_bvh_build_device")
        return b[:n.value], q[:n.value], ids, h.value, st

    def set_tuning(self, wave_paths: int = 0, blocks_per_sm: int = 0, band_rows: int = 0,
                   use_graphs: int = 1, sort_rays: int = 0, tail_bounce: int = 0,
                   primary_traversal: int = 0):
        t = PtTuning(wave_paths, blocks_per_sm, band_rows, use_graphs, sort_rays, tail_bounce,
                     primary_traversal, 0, 0.0)
        self._check(self.L.pt_set_tuning(self.h, ctypes.byref(t)), "pt_set_tuning")

    def get_tuning(self) -> PtTuning:
        t = PtTuning()
        self._check(self.L.pt_get_tuning(self.h, ctypes.byref(t)), "pt_get_tuning")
        return t

    def trace_closest(self, sid: int, n: int, rays_ptr: int, dist_min: float, dist_max: float,
                      tri_ptr: int, dist_ptr: int, stream_ptr: int = 0):
        self._check(self.L.pt_trace_closest(self.h, sid, n, rays_ptr, dist_min, dist_max, tri_ptr,
                                            dist_ptr, stream_ptr or None), "pt_trace_closest")

    def primary_hits(self, sid: int, camera: PtCamera, settings: PtSettings, rays_ptr: int,
                     tri_ptr: int, dist_ptr: int, stream_ptr: int = 0):
        """The render's camera rays and their first closest hits (pt_primary_hits), per
        (pixel row-major, sample), into device buffers."""
        self._check(self.L.pt_primary_hits(self.h, sid, ctypes.byref(camera), ctypes.byref(settings),
                                           rays_ptr, tri_ptr, dist_ptr, stream_ptr or None),
                    "pt_primary_hits")

    def stats(self) -> PtStats:
        s = PtStats()
        self._check(self.L.pt_get_stats(self.h, ctypes.byref(s)), "pt_get_stats")
        return s

    def probe_l2_read_gbs(self, bytes_: int = 0, passes: int = 0, reps: int = 0) -> float:
        """Measured L2 read bandwidth (GB/s) of this context's device (pt_probe_bandwidth)."""
        v = ctypes.c_double()
        self._check(self.L.pt_probe_bandwidth(self.h, bytes_, passes, reps, ctypes.byref(v)),
                    "pt_probe_bandwidth")
        return v.value

    def progress(self):
        d, t = ctypes.c_uint32(), ctypes.c_uint32()
        self._check(self.L.pt_get_progress(self.h, ctypes.byref(d), ctypes.byref(t)), "progress")
        return d.value, t.value


def bvh_build(positions: np.ndarray, indices: np.ndarray, threads: int = 0):
    """Host binned-SAH build: (bounds (N,6), ints (N,5), prim_ids (T,), height)."""
    L = load()
    pos = np.ascontiguousarray(positions, np.float32)
    idx = np.ascontiguousarray(indices, np.int32)
    n, h = ctypes.c_uint32(), ctypes.c_uint32()
    rc = L.pt_bvh_build(pos.ctypes.data, pos.shape[0], idx.ctypes.data, idx.shape[0], threads,
                        ctypes.byref(n), ctypes.byref(h), None, None, None)
    if rc != PT_OK:
        raise PtError(rc, "pt_bvh_build failed")
    b = np.zeros((n.value, 6), np.float32)
    q = np.zeros((n.value, 5), np.int32)
    ids = np.zeros(idx.shape[0], np.int32)
    rc = L.pt_bvh_build(pos.ctypes.data, pos.shape[0], idx.ctypes.data, idx.shape[0], threads,
                        ctypes.byref(n), ctypes.byref(h), b.ctypes.data, q.ctypes.data,
                        ids.ctypes.data)
    if rc != PT_OK:
        raise PtError(rc, "pt_bvh_build failed")
    return b, q, ids, h.value


def render_scene(scene: Scene, mode: int = MODE_REPLAY, seed: int = 1, ctx: Optional[Context] = None,
                 **over) -> np.ndarray:
    """Upload, render and release in one call (the shape of Petrichor::Render)."""
    own = ctx is None
    ctx = ctx or Context()
    try:
        sid = ctx.upload(scene)
        try:
            return ctx.render(sid, camera_from_scene(scene), settings_from_scene(scene, mode, seed, **over))
        finally:
            ctx.release(sid)
    finally:
        if own:
            ctx.close()
