"""Replay mode on the GPU against the reference's films (bit parity path)."""
import dataclasses
import numpy as np
import pytest

import oracle
from conftest import GOLDEN_CASES, golden_scene
from petrichor_gb300 import capi, synth

pytestmark = pytest.mark.gpu

# Per-pixel tolerance for replay films: FP32 radiance within 1e-4 relative
# (absolute floor 1e-6 for near-black pixels).
RTOL, ATOL = 1e-4, 1e-6


def _render(ctx, sc, mode=capi.MODE_REPLAY, **over):
    sid = ctx.upload(sc)
    try:
        return ctx.render(sid, capi.camera_from_scene(sc), capi.settings_from_scene(sc, mode, **over))
    finally:
        ctx.release(sid)


def _close_fraction(a, b):
    ok = np.all(np.abs(a - b) <= ATOL + RTOL * np.abs(b), axis=-1)
    return ok.mean(), np.all(a.view(np.uint32) == b.view(np.uint32), axis=-1).mean()


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_replay_matches_reference_film(gpu_ctx, golden, name):
    sc = golden_scene(golden, name)
    film = _render(gpu_ctx, sc)
    close, exact = _close_fraction(film, golden[f"{name}/film"])
    print(f"{name}: within 1e-4 {close:.5f}, bit-exact {exact:.5f}")
    assert close >= 0.999
    assert gpu_ctx.stats().last_device_status == 0


def test_replay_cornell_full_size_matches_oracle(gpu_ctx):
    sc = synth.cornell()  # 256x256, 16 spp, SimplePathTracing
    ref, _ = oracle.OracleScene(sc).render()
    film = _render(gpu_ctx, sc)
    close, exact = _close_fraction(film, ref)
    print(f"cornell 256^2: within 1e-4 {close:.5f}, bit-exact {exact:.5f}")
    assert close >= 0.999


def test_replay_ragged_tiles_and_tiny_images(gpu_ctx):
    for (w, h, t) in [(1, 1, 16), (17, 5, 4), (33, 20, 7)]:
        sc = synth.cornell(width=w, height=h, spp=3, tile=t, mixed=True, integrator=1,
                           max_bounces=4, env_texture=True)
        ref, _ = oracle.OracleScene(sc).render()
        film = _render(gpu_ctx, sc)
        close, _ = _close_fraction(film, ref)
        assert close >= 0.99, (w, h, t, close)


@pytest.mark.parametrize("env_shape", [(24, 48), (32, 64), (20, 32), (32, 40)])
def test_replay_env_sampling_any_map_size(gpu_ctx, env_shape):
    """Environment next-event sampling: the closed form used for power-of-two maps and
    the bisections used otherwise both give the reference's samples bit for bit."""
    sc = synth.cornell(width=24, height=16, spp=4, mixed=True, integrator=1, max_bounces=4,
                       env_texture=True)
    rng = np.random.default_rng(env_shape[0] * 100 + env_shape[1])
    tex = rng.lognormal(0.0, 0.7, size=env_shape + (3,)).astype(np.float32)
    sc = sc.copy_with(env=dataclasses.replace(sc.env, texture=tex))
    ref, _ = oracle.OracleScene(sc).render()
    film = _render(gpu_ctx, sc)
    assert np.array_equal(film.view(np.uint32), ref.view(np.uint32)), env_shape


def test_replay_progress_counts_tiles(gpu_ctx, golden):
    sc = golden_scene(golden, "cornell_simple")
    _render(gpu_ctx, sc)
    done, total = gpu_ctx.progress()
    assert total == (64 // 16 + 1) ** 2 and done == total
