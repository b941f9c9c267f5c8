"""Batched renders and the serving loop (continuous batching) on the GPU.

Every job's film must be bit-identical to its solo pt_render_device film: the
random stream is keyed by (seed, pixel, sample) and each pixel sums its samples
in sample order, whatever else shares the wave.
"""
import time

import numpy as np
import pytest

from petrichor_gb300 import capi, synth

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _scenes():
    return [
        synth.cornell(width=40, height=30, spp=8, mixed=True, integrator=1, max_bounces=6,
                      env_texture=True),
        synth.spheres_grids(tri_budget=30000, width=64, height=36, spp=4, max_bounces=8,
                            env_width=128, env_height=64),
        synth.cornell(width=33, height=17, spp=5),  # SimplePathTracing (polled queue)
        synth.spheres_grids(seed=9, tri_budget=8000, width=20, height=50, spp=16, max_bounces=4,
                            env_width=64, env_height=32),
    ]


def _solo(ctx, sid, cam, st):
    film = torch.empty(st.width * st.height * 3, dtype=torch.float32, device="cuda")
    ctx.render_device(sid, cam, st, film.data_ptr(), 0)
    torch.cuda.synchronize()
    return film.cpu().numpy()


@pytest.fixture(scope="module")
def served():
    ctx = capi.Context()
    scenes = _scenes()
    sids = [ctx.upload(s) for s in scenes]
    jobs = []
    for k, (s, sid) in enumerate(zip(scenes, sids)):
        cam = capi.camera_from_scene(s)
        st = capi.settings_from_scene(s, capi.MODE_WAVEFRONT, seed=100 + k)
        jobs.append((sid, cam, st))
    solo = [_solo(ctx, *j) for j in jobs]
    yield ctx, jobs, solo
    ctx.close()


def test_batch_films_equal_solo_films(served):
    ctx, jobs, solo = served
    films = [torch.full((j[2].width * j[2].height * 3,), float("nan"), device="cuda") for j in jobs]
    ctx.batch_render([(sid, cam, st, f.data_ptr()) for (sid, cam, st), f in zip(jobs, films)])
    torch.cuda.synchronize()
    for f, ref in zip(films, solo):
        got = f.cpu().numpy()
        assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))


def test_batch_of_repeated_jobs(served):
    ctx, jobs, solo = served
    seq = [jobs[1], jobs[0], jobs[1], jobs[3]]
    films = [torch.empty(j[2].width * j[2].height * 3, device="cuda") for j in seq]
    ctx.batch_render([(sid, cam, st, f.data_ptr()) for (sid, cam, st), f in zip(seq, films)])
    torch.cuda.synchronize()
    for f, idx in zip(films, [1, 0, 1, 3]):
        assert np.array_equal(f.cpu().numpy().view(np.uint32), solo[idx].view(np.uint32))


def test_batch_with_tail_kernel_equals_staged_solo_films(served):
    """Late bounces finished in one launch (the tail kernel) inside batched waves, on a
    launch grid other than the default: each film is still its solo, fully staged film.
    The tail kernel and the staged shade kernel run the same shading code, compiled into
    two kernels; their results agree bit for bit because no float operation is left to
    the compiler to fuse."""
    ctx, jobs, solo = served
    for tune in (dict(tail_bounce=2), dict(tail_bounce=3, blocks_per_sm=12, band_rows=4)):
        ctx.set_tuning(**tune)
        films = [torch.empty(j[2].width * j[2].height * 3, device="cuda") for j in jobs]
        ctx.batch_render([(sid, cam, st, f.data_ptr()) for (sid, cam, st), f in zip(jobs, films)])
        torch.cuda.synchronize()
        for f, ref in zip(films, solo):
            assert np.array_equal(f.cpu().numpy().view(np.uint32), ref.view(np.uint32)), tune
    ctx.set_tuning()


def test_batch_first_bounce_traced_or_rasterised_alike(served):
    """In a batched wave the units whose first bounce can be rasterised (pinhole
    PathTracing jobs with enough rays per triangle) are, the others traced; with the
    first bounce traced for every unit, or rasterised wherever the camera allows, the
    films are the same bits."""
    ctx, jobs, solo = served
    seq = [jobs[0], jobs[1], jobs[3], jobs[0]]
    for traced in (1, 2, 0):
        ctx.set_tuning(primary_traversal=traced)
        films = [torch.empty(j[2].width * j[2].height * 3, device="cuda") for j in seq]
        ctx.batch_render([(sid, cam, st, f.data_ptr()) for (sid, cam, st), f in zip(seq, films)])
        torch.cuda.synchronize()
        for f, idx in zip(films, [0, 1, 3, 0]):
            assert np.array_equal(f.cpu().numpy().view(np.uint32), solo[idx].view(np.uint32)), traced
    ctx.set_tuning()


def test_serve_request_same_alone_and_in_mix(served):
    ctx, jobs, solo = served
    # small waves so every request spans several waves and shares them with others
    ctx.serve_start(wave_paths=12000, max_active=8, state_budget=1 << 24)
    try:
        host = [np.full((j[2].height, j[2].width, 3), np.nan, np.float32) for j in jobs]
        rid = ctx.serve_submit(*jobs[0], film_host=host[0])
        st = ctx.serve_wait(rid, 60)
        assert st.state == capi.REQ_DONE and st.samples_done == jobs[0][2].spp
        alone = host[0].copy()
        assert np.array_equal(alone.ravel().view(np.uint32), solo[0].view(np.uint32))
        host = [np.full((j[2].height, j[2].width, 3), np.nan, np.float32) for j in jobs]
        rids = [ctx.serve_submit(*j, film_host=h) for j, h in zip(jobs, host)]
        for r in rids:
            assert ctx.serve_wait(r, 120).state == capi.REQ_DONE
        for h, ref in zip(host, solo):
            assert np.array_equal(h.ravel().view(np.uint32), ref.view(np.uint32))
        # device films work too
        dev = torch.empty(jobs[1][2].width * jobs[1][2].height * 3, device="cuda")
        r = ctx.serve_submit(*jobs[1], film_device=dev.data_ptr())
        assert ctx.serve_wait(r, 60).state == capi.REQ_DONE
        torch.cuda.synchronize()
        assert np.array_equal(dev.cpu().numpy().view(np.uint32), solo[1].view(np.uint32))
    finally:
        ctx.serve_stop()


def test_serve_admits_while_others_run(served):
    ctx, jobs, solo = served
    ctx.serve_start(wave_paths=20000, max_active=4, state_budget=1 << 24)
    try:
        sid, cam, st = jobs[1]
        big = capi.settings_from_scene(_scenes()[1], capi.MODE_WAVEFRONT, seed=5, spp=4096)
        h_big = np.empty((big.height, big.width, 3), np.float32)
        r_big = ctx.serve_submit(sid, cam, big, film_host=h_big)
        time.sleep(0.05)
        small = [np.empty((jobs[0][2].height, jobs[0][2].width, 3), np.float32) for _ in range(3)]
        r_small = [ctx.serve_submit(*jobs[0], film_host=h) for h in small]
        s_small = [ctx.serve_wait(r, 120) for r in r_small]
        s_big = ctx.serve_wait(r_big, 120)
        assert s_big.state == capi.REQ_DONE and all(s.state == capi.REQ_DONE for s in s_small)
        # the small requests were admitted and finished while the large one ran
        assert max(s.done_s for s in s_small) < s_big.done_s
        assert min(s.admit_s for s in s_small) < s_big.done_s
        for h in small:
            assert np.array_equal(h.ravel().view(np.uint32), solo[0].view(np.uint32))
    finally:
        ctx.serve_stop()


def test_serve_cancel_budget_and_busy_scene(served):
    ctx, jobs, _ = served
    ctx.serve_start(wave_paths=4096, max_active=1, state_budget=1 << 20)
    try:
        sid, cam, st = jobs[1]
        long = capi.settings_from_scene(_scenes()[1], capi.MODE_WAVEFRONT, spp=4096)
        h = np.empty((long.height, long.width, 3), np.float32)
        r1 = ctx.serve_submit(sid, cam, long, film_host=h)
        r2 = ctx.serve_submit(sid, cam, long, film_host=h.copy())  # queued behind r1 (1 slot)
        ctx.serve_cancel(r2)
        ctx.serve_cancel(r1)
        assert ctx.serve_wait(r2, 60).state == capi.REQ_CANCELLED
        assert ctx.serve_wait(r1, 60).state == capi.REQ_CANCELLED
        # the scene may be released only when no request uses it
        r3 = ctx.serve_submit(sid, cam, long, film_host=h)
        with pytest.raises(capi.PtError) as e:
            ctx.release(sid)
        assert e.value.status == -8
        ctx.serve_cancel(r3)
        ctx.serve_wait(r3, 60)
        # state larger than the whole budget is refused at submission
        huge = capi.settings_from_scene(_scenes()[1], capi.MODE_WAVEFRONT, width=1024, height=1024)
        with pytest.raises(capi.PtError) as e:
            ctx.serve_submit(sid, cam, huge, film_host=np.empty((1024, 1024, 3), np.float32))
        assert e.value.status == -3
        ctx.serve_release(r1)
        with pytest.raises(capi.PtError):
            ctx.serve_poll(r1)
    finally:
        ctx.serve_stop()


def test_serve_deadline_fails_late_request_and_spares_others(served):
    """A request past its deadline stops taking samples and fails with PT_ERR_TIMEOUT;
    a request rendering beside it is unaffected (film equal to its solo film)."""
    ctx, jobs, solo = served
    ctx.serve_start(wave_paths=1 << 14)
    try:
        sid, cam, _ = jobs[1]
        long = capi.settings_from_scene(_scenes()[1], capi.MODE_WAVEFRONT, spp=1 << 16)
        hl = np.empty((long.height, long.width, 3), np.float32)
        r_late = ctx.serve_submit(sid, cam, long, film_host=hl)
        ctx.serve_set_deadline(r_late, 0.05)
        sid0, cam0, st0 = jobs[0]
        h0 = np.empty((st0.height, st0.width, 3), np.float32)
        r_ok = ctx.serve_submit(sid0, cam0, st0, film_host=h0)
        s_ok = ctx.serve_wait(r_ok, 120)
        s_late = ctx.serve_wait(r_late, 120)
        assert s_ok.state == capi.REQ_DONE and s_ok.status == 0
        assert np.array_equal(h0.reshape(-1).view(np.uint32), solo[0].view(np.uint32))
        assert s_late.state == capi.REQ_FAILED and s_late.status == -4
        assert s_late.samples_done < s_late.samples_total
        assert s_late.done_s - s_late.submit_s < 30.0
        # a finished request takes no deadline; unknown ids are reported
        with pytest.raises(capi.PtError):
            ctx.serve_set_deadline(r_ok, 1.0)
        with pytest.raises(capi.PtError):
            ctx.serve_set_deadline(123456789, 1.0)
    finally:
        ctx.serve_stop()
