"""The throughput path on the benchmark's own scene, against the reference's estimator.

The scene is the benchmark workload's: 1.0M triangles (64 seeded UV-spheres and
displaced grids; 40% Lambert, 40% GGX, 20% glass), the 2048x1024 procedural sky with a
sun lobe about 1e4 times the median texel, PathTracing (MIS next-event estimation), 16
bounces. Only the resolution is reduced, to 256x144 (the same camera), so that the CPU
oracle finishes in seconds. Two checks, as for the small scenes of
test_gpu_wavefront.py:
* the image mean agrees with the reference estimator (the oracle with the reference's
  random streams) within 0.5%, or within 4.5 standard errors when the sample cannot
  resolve 0.5%; standard errors from replicates;
* equal-spp error against a 65536-spp image is statistically the same as the oracle's
  with independent streams (Mann-Whitney U on 16 replicates each).
"""
import dataclasses

import numpy as np
import pytest

import oracle
from petrichor_gb300 import capi, synth

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

WIDTH, HEIGHT = 256, 144


@pytest.fixture(scope="module")
def bench_scene():
    sc = synth.spheres_grids(width=WIDTH, height=HEIGHT, spp=1)
    assert sc.num_triangles > 990_000 and sc.settings.max_bounces == 16
    assert sc.settings.integrator == 1 and sc.env.texture.shape == (1024, 2048, 3)
    return sc


@pytest.fixture(scope="module")
def resident(gpu_ctx, bench_scene):
    sid = gpu_ctx.upload(bench_scene)
    yield sid
    gpu_ctx.release(sid)


def _with_spp(sc, spp):
    return sc.copy_with(settings=dataclasses.replace(sc.settings, spp=spp))


def _render(ctx, sid, sc, spp, seed):
    return ctx.render(sid, capi.camera_from_scene(sc),
                      capi.settings_from_scene(sc, capi.MODE_WAVEFRONT, seed=seed, spp=spp))


def test_benchmark_scene_image_mean_matches_reference(gpu_ctx, bench_scene, resident):
    sc = bench_scene
    g = np.array([_render(gpu_ctx, resident, sc, 4096, s).mean() for s in range(1, 9)])
    m_g, se_g = g.mean(), g.std(ddof=1) / np.sqrt(len(g))
    m_r = float(oracle.OracleScene(_with_spp(sc, 4096)).render()[0].mean())
    # spread of the reference estimator at 4096 spp, from decorrelated replicates at 1024
    od = oracle.OracleScene(_with_spp(sc, 1024))
    d = np.array([od.render_decorrelated(s)[0].mean() for s in range(1, 5)])
    se_r = d.std(ddof=1) / 2.0
    se = float(np.sqrt(se_g ** 2 + se_r ** 2))
    rel = abs(m_g - m_r) / m_r
    print(f"benchmark scene {WIDTH}x{HEIGHT}: gpu {m_g:.6f}+-{se_g:.6f} reference "
          f"{m_r:.6f}+-{se_r:.6f} rel diff {rel:.4%} (4.5 sigma = {4.5 * se / m_r:.4%})")
    assert rel <= max(0.005, 4.5 * se / m_r)


def test_benchmark_scene_equal_spp_rmse_matches_oracle(gpu_ctx, bench_scene, resident):
    stats = pytest.importorskip("scipy.stats")
    sc = bench_scene
    truth = _render(gpu_ctx, resident, sc, 65536, 1000)
    spp = 64
    mse = lambda a: float(np.mean((a - truth) ** 2))
    e_g = np.array([mse(_render(gpu_ctx, resident, sc, spp, s)) for s in range(1, 17)])
    od = oracle.OracleScene(_with_spp(sc, spp))
    e_d = np.array([mse(od.render_decorrelated(s)[0]) for s in range(1, 17)])
    p = stats.mannwhitneyu(e_g, e_d, alternative="two-sided").pvalue
    ratio = np.median(e_g) / np.median(e_d)
    print(f"benchmark scene: median rmse gpu {np.sqrt(np.median(e_g)):.5f} independent-stream "
          f"oracle {np.sqrt(np.median(e_d)):.5f}; Mann-Whitney p {p:.3g}, median MSE ratio "
          f"{ratio:.3f}")
    assert p >= 1e-3
    assert 0.5 <= ratio <= 2.0
