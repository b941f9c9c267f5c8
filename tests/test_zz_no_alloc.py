"""The replay render that allocates no device memory (pt_render_replay_noalloc).

It exists for callers that cannot allocate at render time, for instance when
another library owns the device memory or the rendering thread must not take
the driver's allocation lock. The test calls it through the C ABI twice in a row
and compares each film with the allocating replay entry point
(pt_render_device), within the replay tolerance (1e-4 relative per pixel, 1e-6
absolute floor), and checks that each render's device status word reads back as
clean through pt_get_stats. It also checks that the context and the device report no new
allocation across the second call, and that an oversize render is refused.
This file is collected last so a failure here stops a -x run after every other
test has run.
"""
import ctypes

import numpy as np
import pytest

from petrichor_gb300 import capi, synth

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

RTOL, ATOL = 1e-4, 1e-6


def test_noalloc_replay_matches_allocating_replay():
    ctx = capi.Context()
    try:
        sc = synth.cornell(width=48, height=40, spp=4, mixed=True, integrator=1, max_bounces=5,
                           env_texture=True, tile=8)
        sid = ctx.upload(sc)
        cam = capi.camera_from_scene(sc)
        st = capi.settings_from_scene(sc, capi.MODE_REPLAY)
        stream = torch.cuda.Stream()
        n = sc.settings.width * sc.settings.height * 3
        ref = torch.empty(n, dtype=torch.float32, device="cuda")
        ctx.render_device(sid, cam, st, ref.data_ptr(), stream.cuda_stream)
        torch.cuda.synchronize()
        ref = ref.cpu().numpy()
        outs = [torch.full((n,), float("nan"), dtype=torch.float32, device="cuda") for _ in range(2)]
        torch.cuda.synchronize()
        used = ctx.stats().device_bytes_in_use
        free_after = []
        for out in outs:
            rc = ctx.L.pt_render_replay_noalloc(ctx.h, sid, ctypes.byref(cam), ctypes.byref(st),
                                                out.data_ptr(), stream.cuda_stream)
            assert rc == 0, ctx.L.pt_last_error(ctx.h)
            # the render's own status word (stack overflow, bounce cap, bounds bits)
            stats = ctx.stats()
            assert stats.last_device_status == 0
            assert stats.last_render_ms > 0.0
            done, total = ctx.progress()
            assert done == total == (48 // 8 + 1) * (40 // 8 + 1)  # the reference's tile grid
            torch.cuda.synchronize()
            free_after.append(torch.cuda.mem_get_info()[0])
            got = out.cpu().numpy()
            assert np.all(np.isfinite(got))
            assert np.all(np.abs(got - ref) <= ATOL + RTOL * np.abs(ref))
            assert stats.device_bytes_in_use == used
        assert free_after[0] == free_after[1]
        # a render whose stacks exceed the fixed array is refused, not truncated
        big = capi.settings_from_scene(sc, capi.MODE_REPLAY, width=4096, height=4096,
                                       tile_width=1, tile_height=1)
        rc = ctx.L.pt_render_replay_noalloc(ctx.h, sid, ctypes.byref(cam), ctypes.byref(big),
                                            outs[0].data_ptr(), stream.cuda_stream)
        assert rc == -1 and b"scratch" in ctx.L.pt_last_error(ctx.h)
        ctx.release(sid)
    finally:
        ctx.close()
