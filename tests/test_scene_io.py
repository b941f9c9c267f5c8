import numpy as np

from conftest import GOLDEN_CASES, golden_scene
from petrichor_gb300 import scene_io, synth


def test_roundtrip_bytes(golden):
    for name in GOLDEN_CASES:
        raw = golden[f"{name}/scene"].tobytes()
        assert scene_io.scene_bytes(scene_io.read_scene_bytes(raw)) == raw


def test_generators_are_deterministic():
    a = scene_io.scene_bytes(synth.spheres_grids(tri_budget=3000, width=8, height=8, spp=1,
                                                 env_width=16, env_height=8))
    b = scene_io.scene_bytes(synth.spheres_grids(tri_budget=3000, width=8, height=8, spp=1,
                                                 env_width=16, env_height=8))
    assert a == b


def test_cornell_counts():
    sc = synth.cornell()
    assert sc.num_triangles == 36 and list(sc.lights) == [34, 35]
    assert sc.materials[sc.tri_material[34]].kind == scene_io.MAT_EMISSION


def test_spheres_grids_full_size_budget():
    sc = synth.spheres_grids(width=8, height=8, spp=1, env_width=16, env_height=8)
    assert 0.98e6 <= sc.num_triangles <= 1.02e6
    kinds = [m.kind for m in sc.materials]
    assert len(kinds) == 64
    assert set(kinds) <= {scene_io.MAT_LAMBERT, scene_io.MAT_GLOSSY, scene_io.MAT_GLASS}


def test_sky_env_sun_peak():
    img = synth.sky_env(synth.Rng(3), 256, 128)
    lum = img.mean(-1)
    assert lum.max() / np.median(lum) > 1e3
