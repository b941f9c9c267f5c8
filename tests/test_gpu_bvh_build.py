"""Device binned-SAH build (petrichor_gb300/csrc/bvh_gpu.cu, pt_bvh_build_device).

The tree must be the reference's (BinnedSAHBVH::Build), node for node and primitive
for primitive: the same bounds bits (signed zeros included), child indices, ranges and
the primitive order that libstdc++'s std::sort leaves among equal keys. Checked against
the compiled reference's trees (golden fixtures) and against the host builder, which
runs std::sort itself, on scenes full of equal keys, on an adversarial key order that
drives std::sort into its heapsort fallback, and on edge sizes.
"""
import os
import subprocess
import time

import numpy as np
import pytest

from conftest import golden_scene
from petrichor_gb300 import capi, synth

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _same_tree(dev, host):
    b, q, ids, h = dev[:4]
    hb, hq, hids, hh = host[:4]
    assert b.shape == hb.shape
    assert np.array_equal(b.view(np.uint32), hb.view(np.uint32))
    assert np.array_equal(q, hq)
    assert np.array_equal(ids, hids)
    assert h == hh


@pytest.mark.parametrize("name", ["spheres_pt", "bvh_ties"])
def test_device_build_matches_reference_tree(gpu_ctx, golden, name):
    sc = golden_scene(golden, name)
    b, q, ids, h, st = gpu_ctx.bvh_build_device(sc.positions, sc.indices)
    assert np.array_equal(b.view(np.uint32), golden[f"{name}/bvh_bounds"].view(np.uint32))
    assert np.array_equal(q, golden[f"{name}/bvh_ints"])
    assert np.array_equal(ids, golden[f"{name}/bvh_ids"])
    if name == "bvh_ties":  # equal keys on every axis, and bounds at +0 and -0
        zero = b[:, 0] == 0
        assert zero.any() and (np.signbit(b[zero, 0])).any() and (~np.signbit(b[zero, 0])).any()


def _soup(seed, n, dup=0.0, quant=None):
    rng = np.random.default_rng(seed)
    c = rng.uniform(-10, 10, size=(n, 3))
    if quant:  # centroids on a lattice: many equal keys
        c = np.round(c / quant) * quant
    if dup:
        k = int(n * dup)
        c[rng.integers(0, n, k)] = c[rng.integers(0, n, k)]
    off = rng.uniform(-0.3, 0.3, size=(n, 3, 3))
    off -= off.mean(axis=1, keepdims=True)
    P = (c[:, None, :] + off).reshape(-1, 3).astype(np.float32)
    return P, np.arange(3 * n, dtype=np.int32).reshape(n, 3)


def _scenes():
    yield "cornell", synth.cornell(width=16, height=16, spp=1)
    yield "textured", synth.textured_spheres()
    yield "spheres_grids_30k", synth.spheres_grids(tri_budget=30000, width=16, height=16, spp=1,
                                                   env_width=16, env_height=8)
    yield "terrain_rocks_small", synth.terrain_rocks(terrain_n=120, n_rocks=60, rock_tris=100, width=16,
                                                     height=16, spp=1, env_width=16, env_height=8)
    for seed in (7, 8):
        yield f"bvh_ties_{seed}", synth.bvh_ties(seed=seed)


@pytest.mark.parametrize("name", [n for n, _ in _scenes()])
def test_device_build_equals_host_build(gpu_ctx, name):
    sc = dict(_scenes())[name]
    dev = gpu_ctx.bvh_build_device(sc.positions, sc.indices)
    host = capi.bvh_build(sc.positions, sc.indices)
    _same_tree(dev, host)


@pytest.mark.parametrize("kind", ["random", "duplicates", "lattice"])
def test_device_build_on_triangle_soups(gpu_ctx, kind):
    P, I = _soup({"random": 1, "duplicates": 2, "lattice": 3}[kind], 50000,
                 dup=0.3 if kind == "duplicates" else 0.0, quant=0.5 if kind == "lattice" else None)
    _same_tree(gpu_ctx.bvh_build_device(P, I), capi.bvh_build(P, I))


def test_device_build_reproduces_std_sort_heapsort_fallback(gpu_ctx, tmp_path):
    """Centroid keys in McIlroy's adversarial order make std::sort exhaust its depth
    budget at the root; the device build must take the same heapsort path."""
    exe = str(tmp_path / "antiqsort")
    subprocess.run(["g++", "-std=c++17", "-O2", os.path.join(ROOT, "tests", "cpp", "antiqsort.cpp"),
                    "-o", exe], check=True)
    n = 6000
    keys = np.array(subprocess.run([exe, str(n)], capture_output=True, text=True,
                                   check=True).stdout.split(), np.int64)
    # centroid x = 3 key exactly; y and z centroids constant, so x is the widest axis
    x = 3.0 * keys
    P = np.stack([np.stack([x, np.zeros(n), np.zeros(n)], 1),
                  np.stack([x, np.ones(n), np.zeros(n)], 1),
                  np.stack([x, np.zeros(n), np.ones(n)], 1)], 1).reshape(-1, 3).astype(np.float32)
    I = np.arange(3 * n, dtype=np.int32).reshape(n, 3)
    dev = gpu_ctx.bvh_build_device(P, I)
    assert dev[4].heapsorts > 0
    _same_tree(dev, capi.bvh_build(P, I))


@pytest.mark.parametrize("n", [0, 1, 2, 4, 5, 16, 17, 18, 33, 100])
def test_device_build_edge_sizes(gpu_ctx, n):
    P, I = _soup(40 + n, max(n, 1))
    P, I = P[:3 * n], I[:n]
    if n == 0:
        P = np.zeros((0, 3), np.float32)
    _same_tree(gpu_ctx.bvh_build_device(P, I), capi.bvh_build(P, I))


def test_scene_upload_uses_device_builder_and_renders_the_same(gpu_ctx, golden):
    sc = golden_scene(golden, "spheres_pt")
    films = {}
    for builder in (capi.BVH_BUILDER_HOST, capi.BVH_BUILDER_DEVICE):
        gpu_ctx.set_bvh_builder(builder)
        sid = gpu_ctx.upload(sc)
        assert gpu_ctx.scene_info(sid).bvh_builder == builder
        films[builder] = gpu_ctx.render(sid, capi.camera_from_scene(sc),
                                        capi.settings_from_scene(sc, capi.MODE_REPLAY))
        gpu_ctx.release(sid)
    gpu_ctx.set_bvh_builder(capi.BVH_BUILDER_DEVICE)
    assert np.array_equal(films[0].view(np.uint32), films[1].view(np.uint32))
    assert np.array_equal(films[1].view(np.uint32), golden["spheres_pt/film"].view(np.uint32))
    with pytest.raises(capi.PtError):
        gpu_ctx.set_bvh_builder(7)


def test_device_build_full_size_scene(gpu_ctx):
    """The 1.0M-triangle benchmark scene: same tree as the host build, and the time."""
    sc = synth.spheres_grids(width=16, height=16, spp=1, env_width=16, env_height=8)
    t0 = time.perf_counter()
    host = capi.bvh_build(sc.positions, sc.indices)
    t_host = time.perf_counter() - t0
    gpu_ctx.bvh_build_device(sc.positions, sc.indices)  # warm-up (module load, first allocations)
    t0 = time.perf_counter()
    dev = gpu_ctx.bvh_build_device(sc.positions, sc.indices)
    t_dev = time.perf_counter() - t0
    st = dev[4]
    print(f"{sc.indices.shape[0]} triangles: host {t_host * 1e3:.1f} ms, device {t_dev * 1e3:.1f} ms wall "
          f"({st.device_ms:.1f} ms device; {st.levels} levels, {st.rounds} partition rounds, "
          f"{st.launches} launches)")
    _same_tree(dev, host)
