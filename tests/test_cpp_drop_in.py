"""The C++ drop-in API (include/petrichor_gb300/Petrichor.hpp) driven by a client
program that builds scenes with the reference's scene calls (tests/cpp/drop_in_render.cpp).

CPU: the program compiles and links against the library, and reports the missing
device through Petrichor::GetLastStatus. GPU: Petrichor::Render with its defaults
reproduces the reference's own films bit for bit, and in wavefront mode equals the
C-ABI render of the same scene.
"""
import os
import subprocess

import numpy as np
import pytest

from conftest import AOV_CASES, GOLDEN_CASES, golden_scene

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "drop_in_render.cpp")


@pytest.fixture(scope="module")
def client(tmp_path_factory):
    from petrichor_gb300 import _build
    lib = _build.build()
    exe = str(tmp_path_factory.mktemp("cpp") / "drop_in_render")
    libdir = os.path.dirname(lib)
    subprocess.run(["g++", "-std=c++17", "-O2", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                    SRC, "-L", libdir, "-lpetrichor_gb300", f"-Wl,-rpath,{libdir}", "-o", exe],
                   check=True)
    return exe


def _run(exe, golden, name, tmp_path, *extra):
    scene = tmp_path / f"{name}.ptscene"
    scene.write_bytes(golden[f"{name}/scene"].tobytes())
    film = tmp_path / f"{name}.film"
    r = subprocess.run([exe, str(scene), str(film), *extra], capture_output=True, text=True,
                       timeout=300)
    return r, film


def test_client_builds_and_reports_missing_device(client, golden, tmp_path):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a device is present")
    r, film = _run(client, golden, "cornell_simple", tmp_path)
    assert r.returncode == 3, r.stdout + r.stderr
    assert '"status": -10' in r.stdout
    assert not film.exists()


@pytest.mark.gpu
@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_drop_in_render_matches_reference_film(client, golden, tmp_path, name):
    r, film = _run(client, golden, name, tmp_path)
    assert r.returncode == 0, r.stdout + r.stderr
    ref = golden[f"{name}/film"]
    got = np.fromfile(film, np.float32).reshape(ref.shape)
    same = np.mean(got.view(np.uint32) == ref.view(np.uint32))
    print(name, "bit-identical fraction", same)
    assert same == 1.0


@pytest.mark.gpu
@pytest.mark.parametrize("name, mode", [("cornell_mixed_pt", "wavefront"), ("spheres_pt", "wavefront"),
                                        ("spheres_pt", "wavefront-alias")])
def test_drop_in_wavefront_equals_c_abi(client, golden, gpu_ctx, tmp_path, name, mode):
    from petrichor_gb300 import capi
    r, film = _run(client, golden, name, tmp_path, mode)
    assert r.returncode == 0, r.stdout + r.stderr
    sc = golden_scene(golden, name)
    env = capi.ENV_SAMPLING_ALIAS if mode == "wavefront-alias" else capi.ENV_SAMPLING_REFERENCE
    ref = capi.render_scene(sc, mode=capi.MODE_WAVEFRONT, seed=1, ctx=gpu_ctx, env_sampling=env)
    got = np.fromfile(film, np.float32).reshape(ref.shape)
    assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))


@pytest.mark.gpu
@pytest.mark.parametrize("name", AOV_CASES)
def test_drop_in_render_fills_aov_targets(client, golden, tmp_path, name):
    """Rendered + UV + DenoisingAlbedo + DenoisingNormal targets in one Render call."""
    import oracle
    dspp = int(golden[f"{name}/denoising_spp"][0])
    r, film = _run(client, golden, name, tmp_path, "aov", str(dspp))
    assert r.returncode == 0, r.stdout + r.stderr
    ref = golden[f"{name}/aov"]
    got = np.fromfile(film, np.float32).reshape((4,) + ref.shape[1:])
    rendered, _ = oracle.OracleScene(golden_scene(golden, name)).render(threads=4)
    assert np.array_equal(got[0].view(np.uint32), rendered.view(np.uint32))
    for a in range(3):
        assert np.array_equal(got[a + 1].view(np.uint32), ref[a].view(np.uint32)), a
