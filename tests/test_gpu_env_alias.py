"""Optional alias-table environment sampling (PT_ENV_SAMPLING_ALIAS; the reference's
Math::AliasMethod, Math/AliasMethod.h:26-105, over the environment map's cells).

The reference's own environment tables are never filled (Environment.cpp:56-128 read
unloaded textures), so its next-event estimator samples one meridian and its image is not
the converged one. The alias mode is a different estimator and has no reference film to
match. What is checked instead:
  - it is unbiased: its image mean agrees with SimplePathTracing (BSDF sampling only, no
    environment table involved) on an environment-lit scene of materials that the
    reference samples consistently with their BSDFs;
  - it is the better estimator there: lower per-pixel error at equal samples;
  - the film does not depend on the wave size and is the same through the batch path;
  - a scene without an environment map renders exactly as with the reference tables;
  - misuse is rejected (unknown value, replay mode).
"""
import dataclasses

import numpy as np
import pytest

from petrichor_gb300 import capi, synth
from petrichor_gb300.scene_io import MAT_GLASS, MAT_LAMBERT, Material

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _scene(sun=30.0):
    """Spheres and grids lit by the environment alone (no emitters).

    The reference samples white Lambert (Lambert.cpp:49-98: the throughput is multiplied
    by GetAlbedo, 1 without a texture, while BxDF is kd / pi) and glass consistently with
    their BSDFs; its GGX sampling weight (GGX.cpp:78-138) divides by G1 of the outgoing
    direction. So the other materials are made white Lambert here, where an unbiased
    next-event estimator and BSDF sampling converge to the same image."""
    sc = synth.spheres_grids(tri_budget=20000, width=96, height=54, spp=16, max_bounces=32,
                             env_width=128, env_height=64, sun_peak_over_median=sun)
    mats = [m if m.kind == MAT_GLASS else Material(MAT_LAMBERT, color=(1.0, 1.0, 1.0))
            for m in sc.materials]
    return dataclasses.replace(sc, materials=mats)


def _render(ctx, sid, sc, seed, spp, **kw):
    st = capi.settings_from_scene(sc, capi.MODE_WAVEFRONT, seed=seed, spp=spp, **kw)
    return ctx.render(sid, capi.camera_from_scene(sc), st)


@pytest.fixture(scope="module")
def lit(gpu_ctx):
    sc = _scene()
    sid = gpu_ctx.upload(sc)
    before = gpu_ctx.scene_info(sid).device_bytes
    alias = [_render(gpu_ctx, sid, sc, s, 1024, env_sampling=capi.ENV_SAMPLING_ALIAS) for s in range(1, 7)]
    after = gpu_ctx.scene_info(sid).device_bytes
    simple = [_render(gpu_ctx, sid, sc, s, 1024, integrator=capi.INTEGRATOR_SIMPLE) for s in range(11, 17)]
    ref_pt = _render(gpu_ctx, sid, sc, 21, 1024)
    yield gpu_ctx, sc, sid, alias, simple, ref_pt, before, after
    gpu_ctx.release(sid)


def test_alias_table_is_built_once_per_scene(lit):
    ctx, sc, sid, _, _, _, before, after = lit
    cells = sc.env.texture.shape[0] * sc.env.texture.shape[1]
    assert after - before >= cells * 16
    _render(ctx, sid, sc, 5, 1, env_sampling=capi.ENV_SAMPLING_ALIAS)
    assert ctx.scene_info(sid).device_bytes == after


def test_alias_sampling_is_unbiased_against_bsdf_sampling(lit):
    _, _, _, alias, simple, ref_pt, _, _ = lit
    a = np.array([x.mean(axis=(0, 1)) for x in alias])    # per seed, per channel
    s = np.array([x.mean(axis=(0, 1)) for x in simple])
    ma, ms = a.mean(0), s.mean(0)
    # standard error of the difference from the spread over seeds
    se = np.sqrt(a.var(0, ddof=1) / len(a) + s.var(0, ddof=1) / len(s))
    rel = np.abs(ma - ms) / ms
    print(f"image mean alias-PT {ma}, SimplePathTracing {ms}, reference-table PT "
          f"{ref_pt.mean(axis=(0, 1))}; relative difference {rel}, 4 standard errors {4 * se / ms}")
    assert np.all(np.abs(ma - ms) <= np.maximum(4.0 * se, 0.004 * ms))


@pytest.mark.parametrize("sun, bound", [(30.0, 0.95), (3000.0, 0.2)])
def test_alias_sampling_lowers_error_at_equal_samples(gpu_ctx, sun, bound):
    # a sky (sun lobe 30x the median texel: most light comes from the whole sky, which
    # cosine sampling already follows) and a sun-dominated map (3000x)
    sc = _scene(sun)
    sid = gpu_ctx.upload(sc)
    try:
        truth = _render(gpu_ctx, sid, sc, 41, 4096, env_sampling=capi.ENV_SAMPLING_ALIAS)
        a = _render(gpu_ctx, sid, sc, 31, 16, env_sampling=capi.ENV_SAMPLING_ALIAS)
        s = _render(gpu_ctx, sid, sc, 31, 16, integrator=capi.INTEGRATOR_SIMPLE)
    finally:
        gpu_ctx.release(sid)
    ea, es = float(np.mean((a - truth) ** 2)), float(np.mean((s - truth) ** 2))
    print(f"sun {sun:g}: 16 spp MSE against a 4096 spp image: alias-PT {ea:.4g}, "
          f"SimplePathTracing {es:.4g} (ratio {ea / es:.3f})")
    assert np.isfinite(a).all()
    assert ea < bound * es


def test_alias_film_independent_of_wave_size_and_batch(lit):
    ctx, sc, sid, _, _, _, _, _ = lit
    full = _render(ctx, sid, sc, 7, 8, env_sampling=capi.ENV_SAMPLING_ALIAS)
    small = _render(ctx, sid, sc, 7, 8, env_sampling=capi.ENV_SAMPLING_ALIAS, wave_paths=1 << 14)
    assert np.array_equal(full.view(np.uint32), small.view(np.uint32))
    st = capi.settings_from_scene(sc, capi.MODE_WAVEFRONT, seed=7, spp=8,
                                  env_sampling=capi.ENV_SAMPLING_ALIAS)
    film = torch.zeros(st.height * st.width * 3, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    ctx.batch_render([(sid, capi.camera_from_scene(sc), st, film.data_ptr())])
    torch.cuda.synchronize()
    got = film.cpu().numpy().reshape(st.height, st.width, 3)
    assert np.array_equal(got.view(np.uint32), full.view(np.uint32))


def test_alias_without_environment_map_matches_reference_tables(gpu_ctx):
    sc = synth.cornell(width=48, height=48, spp=4, integrator=1, max_bounces=4)
    sid = gpu_ctx.upload(sc)
    try:
        a = _render(gpu_ctx, sid, sc, 3, 4, env_sampling=capi.ENV_SAMPLING_ALIAS)
        r = _render(gpu_ctx, sid, sc, 3, 4)
        assert np.array_equal(a.view(np.uint32), r.view(np.uint32))
    finally:
        gpu_ctx.release(sid)


def test_alias_sampling_rejects_bad_settings(gpu_ctx):
    sc = synth.cornell(width=16, height=16, spp=1, integrator=1, env_texture=True)
    sid = gpu_ctx.upload(sc)
    try:
        cam = capi.camera_from_scene(sc)
        with pytest.raises(capi.PtError):
            gpu_ctx.render(sid, cam, capi.settings_from_scene(sc, capi.MODE_WAVEFRONT, env_sampling=2))
        with pytest.raises(capi.PtError):
            gpu_ctx.render(sid, cam, capi.settings_from_scene(sc, capi.MODE_REPLAY,
                                                              env_sampling=capi.ENV_SAMPLING_ALIAS))
    finally:
        gpu_ctx.release(sid)


def test_alias_served_request_equals_render(lit):
    _, sc, _, _, _, _, _, _ = lit
    ctx = capi.Context()
    try:
        sid = ctx.upload(sc)
        cam = capi.camera_from_scene(sc)
        st = capi.settings_from_scene(sc, capi.MODE_WAVEFRONT, seed=9, spp=4,
                                      env_sampling=capi.ENV_SAMPLING_ALIAS)
        ref = ctx.render(sid, cam, st)
        # small waves: the request spans several of them
        ctx.serve_start(wave_paths=12000, max_active=4, state_budget=1 << 24)
        try:
            host = np.full((st.height, st.width, 3), np.nan, np.float32)
            rid = ctx.serve_submit(sid, cam, st, film_host=host)
            assert ctx.serve_wait(rid, 60).state == capi.REQ_DONE
            assert np.array_equal(host.view(np.uint32), ref.view(np.uint32))
        finally:
            ctx.serve_stop()
        ctx.release(sid)
    finally:
        ctx.close()


def test_alias_black_map_falls_back_to_area_weights(gpu_ctx):
    # no positive luminance anywhere: the table weighs cells by their area (sin theta)
    sc = _scene()
    sc = dataclasses.replace(sc, env=dataclasses.replace(sc.env, texture=np.zeros_like(sc.env.texture)))
    sid = gpu_ctx.upload(sc)
    try:
        a = _render(gpu_ctx, sid, sc, 3, 2, env_sampling=capi.ENV_SAMPLING_ALIAS)
        r = _render(gpu_ctx, sid, sc, 3, 2)
        assert np.isfinite(a).all()
        assert float(a.max()) == 0.0 and float(r.max()) == 0.0  # a black sky lights nothing
    finally:
        gpu_ctx.release(sid)
