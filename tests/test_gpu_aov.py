"""AOV passes of Petrichor::Render on the GPU (pt_render_aov): UV coordinates,
denoising albedo and denoising normal, bit for bit against the reference's own
passes (tests/golden: rendered by the compiled reference, Core/AOV/*.cpp)."""
import numpy as np
import pytest

from conftest import AOV_CASES, golden_scene
from petrichor_gb300 import capi

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.mark.parametrize("name", AOV_CASES)
def test_aov_passes_match_reference_bits(golden, gpu_ctx, name):
    sc = golden_scene(golden, name)
    dspp = int(golden[f"{name}/denoising_spp"][0])
    ref = golden[f"{name}/aov"]
    sid = gpu_ctx.upload(sc)
    try:
        cam = capi.camera_from_scene(sc)
        st = capi.settings_from_scene(sc, capi.MODE_REPLAY, denoising_spp=dspp)
        for aov in (capi.AOV_UV, capi.AOV_DENOISING_ALBEDO, capi.AOV_DENOISING_NORMAL):
            got = gpu_ctx.render_aov(sid, cam, st, aov)
            same = float(np.mean(got.view(np.uint32) == ref[aov].view(np.uint32)))
            print(name, aov, "bit-identical fraction", same)
            assert same == 1.0
            dev = torch.full((st.width * st.height * 3,), float("nan"), device="cuda")
            gpu_ctx.render_aov_device(sid, cam, st, aov, dev.data_ptr())
            torch.cuda.synchronize()
            assert np.array_equal(dev.cpu().numpy().view(np.uint32), got.ravel().view(np.uint32))
    finally:
        gpu_ctx.release(sid)


def test_aov_rejects_bad_arguments(golden, gpu_ctx):
    sc = golden_scene(golden, "aov_spheres")
    sid = gpu_ctx.upload(sc)
    try:
        cam = capi.camera_from_scene(sc)
        st = capi.settings_from_scene(sc, capi.MODE_REPLAY, denoising_spp=1)
        for aov in (-1, 3):
            with pytest.raises(capi.PtError):
                gpu_ctx.render_aov(sid, cam, st, aov)
        st.denoising_spp = -2
        with pytest.raises(capi.PtError):
            gpu_ctx.render_aov(sid, cam, st, capi.AOV_DENOISING_ALBEDO)
        st.denoising_spp = 1
        assert np.isfinite(gpu_ctx.render_aov(sid, cam, st, capi.AOV_DENOISING_NORMAL)).all()
    finally:
        gpu_ctx.release(sid)
