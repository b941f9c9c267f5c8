"""Launch configuration of the wavefront path: captured CUDA graphs, grid sizes,
pixel bands, wave sizes, first-bounce rasterisation and the autotuner.

None of these may change a film: the random stream is keyed by (seed, pixel,
sample), every ray visits its nodes in its own fixed order, each pixel sums its
samples in sample order, and a rasterised first bounce finds the same closest hits as
the traversal (exact ties settled in the reference's order by both).
"""
import numpy as np
import pytest

from petrichor_gb300 import capi, synth

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

CONFIGS = [
    dict(),                                                   # defaults (graphs on)
    dict(use_graphs=0),
    dict(blocks_per_sm=4, band_rows=16, use_graphs=1),
    dict(blocks_per_sm=24, band_rows=4, use_graphs=0),
    dict(blocks_per_sm=12, band_rows=1, use_graphs=1, wave_paths=3000),
    dict(sort_rays=1),
    dict(sort_rays=1, use_graphs=0, wave_paths=3000),
    dict(tail_bounce=1),                                      # one launch from bounce 1 on
    dict(tail_bounce=3, use_graphs=0, wave_paths=3000),
    dict(primary_traversal=1),                                # first bounce traced, not rasterised
    dict(primary_traversal=1, use_graphs=0, wave_paths=3000),
    dict(primary_traversal=2),                                # rasterised at 2+ rays per triangle
    dict(primary_traversal=2, use_graphs=0, wave_paths=3000),
]


def _scenes():
    return {
        "pt": synth.cornell(width=40, height=30, spp=8, mixed=True, integrator=1, max_bounces=6,
                            env_texture=True),
        "simple": synth.cornell(width=33, height=17, spp=5),  # queue-polled bounce blocks
        "tris": synth.spheres_grids(tri_budget=30000, width=64, height=36, spp=4, max_bounces=8,
                                    env_width=128, env_height=64),
        # enough rays per triangle (over 16) for the rasterised first bounce by default; a
        # tilted camera (the camera basis is not unit length)
        "raster": synth.spheres_grids(tri_budget=20000, width=96, height=64, spp=64, max_bounces=6,
                                      env_width=128, env_height=64),
        # a camera inside the box: walls reach behind the camera plane (whole-image rectangles)
        "inside": _inside_box(),
        # two rays per triangle at 1 spp (rasterised with primary_traversal=2): the raster
        # work list fills up, and the triangles that do not fit are visited whole
        "overflow": synth.spheres_grids(tri_budget=60000, width=360, height=340, spp=1,
                                        max_bounces=4, env_width=128, env_height=64),
    }


def _inside_box():
    from petrichor_gb300.scene_io import Camera
    sc = synth.cornell(width=48, height=40, spp=8, mixed=True, integrator=1, max_bounces=5,
                       env_texture=True)
    return sc.copy_with(camera=Camera(pos=(0.05, -0.6, 1.1), view_dir=(0.2, 1.0, -0.1),
                                      fov=1.6, focus_target=None, aperture=0.0))


@pytest.fixture(scope="module")
def tuned_ctx():
    ctx = capi.Context()
    scenes = _scenes()
    jobs = {}
    for name, s in scenes.items():
        jobs[name] = (ctx.upload(s), capi.camera_from_scene(s),
                      capi.settings_from_scene(s, capi.MODE_WAVEFRONT, seed=7))
    yield ctx, jobs
    ctx.close()


def _render(ctx, sid, cam, st):
    film = torch.full((st.width * st.height * 3,), float("nan"), device="cuda")
    ctx.render_device(sid, cam, st, film.data_ptr(), 0)
    torch.cuda.synchronize()
    return film.cpu().numpy()


@pytest.mark.parametrize("name", ["pt", "simple", "tris", "raster", "inside", "overflow"])
def test_films_do_not_depend_on_launch_configuration(tuned_ctx, name):
    ctx, jobs = tuned_ctx
    sid, cam, st = jobs[name]
    ctx.set_tuning()
    ref = _render(ctx, sid, cam, st)
    assert np.isfinite(ref).all()
    for cfg in CONFIGS:
        ctx.set_tuning(**cfg)
        for _ in range(2):  # the second render replays the captured graph
            got = _render(ctx, sid, cam, st)
            assert np.array_equal(got.view(np.uint32), ref.view(np.uint32)), cfg
    ctx.set_tuning()


def test_graph_replay_counts_the_same_kernels(tuned_ctx):
    ctx, jobs = tuned_ctx
    sid, cam, st = jobs["tris"]
    counts = {}
    for graphs in (0, 1):
        ctx.set_tuning(use_graphs=graphs)
        _render(ctx, sid, cam, st)  # capture
        before = ctx.stats().kernel_launches
        _render(ctx, sid, cam, st)
        counts[graphs] = ctx.stats().kernel_launches - before
    ctx.set_tuning()
    assert counts[0] == counts[1] > 0


def test_autotune_picks_a_valid_configuration(tuned_ctx):
    ctx, jobs = tuned_ctx
    sid, cam, st = jobs["tris"]
    ctx.set_tuning()
    ref = _render(ctx, sid, cam, st)
    t = ctx.autotune(sid, cam, st, probe_spp=2)
    assert t.probe_ms > 0
    assert t.blocks_per_sm in (0, 4, 12, 16, 24)
    assert t.band_rows in (0, 4, 8, 16, 32)
    assert t.use_graphs in (0, 1) and t.sort_rays in (0, 1)
    got = ctx.get_tuning()
    assert (got.blocks_per_sm, got.band_rows, got.use_graphs, got.sort_rays) == (
        t.blocks_per_sm, t.band_rows, t.use_graphs, t.sort_rays)
    film = _render(ctx, sid, cam, st)
    assert np.array_equal(film.view(np.uint32), ref.view(np.uint32))
    ctx.set_tuning()


def test_set_tuning_rejects_bad_values(tuned_ctx):
    ctx, _ = tuned_ctx
    for bad in (dict(blocks_per_sm=-1), dict(blocks_per_sm=65), dict(band_rows=-2),
                dict(wave_paths=-5), dict(use_graphs=2), dict(sort_rays=3), dict(tail_bounce=-2),
                dict(tail_bounce=65), dict(primary_traversal=3),
                dict(primary_traversal=-1)):
        with pytest.raises(capi.PtError):
            ctx.set_tuning(**bad)
    ctx.set_tuning()


@pytest.mark.parametrize("name", ["pt", "simple", "tris"])
def test_overlapped_shadow_stage_equals_sequential(tuned_ctx, name):
    """Renders run each bounce's shadow stage beside the next extend on a second stream;
    the profiled render runs every stage in order on one stream. Same film bits."""
    ctx, jobs = tuned_ctx
    sid, cam, st = jobs[name]
    ctx.set_tuning()
    overlapped = _render(ctx, sid, cam, st)
    film = torch.full((st.width * st.height * 3,), float("nan"), device="cuda")
    ctx.render_profile(sid, cam, st, film.data_ptr(), count_reference=False)
    torch.cuda.synchronize()
    sequential = film.cpu().numpy()
    assert np.array_equal(overlapped.view(np.uint32), sequential.view(np.uint32))
