"""GPU denoiser (petrichor_gb300/csrc/denoise.cu; pt_denoise; IntelOpenImageDenoiser in the
C++ API).

The reference hands its film to Intel Open Image Denoise, which is not available here,
so there is no reference image to match. What is checked instead: on noisy renders the
filter brings the image closer to a converged render of the same scene (tone-mapped
squared error, what a viewer sees), more so with the albedo and normal AOVs as guides;
constant images pass through; results are deterministic and the same through the host,
device and C++ entry points; bad arguments are rejected.
"""
import os
import subprocess

import numpy as np
import pytest

from petrichor_gb300 import capi, synth

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _tm(a):
    a = np.clip(a, 0.0, None)
    return a / (1.0 + a)


def _tmse(a, truth):
    return float(np.mean((_tm(a) - _tm(truth)) ** 2))


def _case(ctx, sc):
    sid = ctx.upload(sc)
    cam = capi.camera_from_scene(sc)
    noisy = ctx.render(sid, cam, capi.settings_from_scene(sc, capi.MODE_WAVEFRONT, seed=1))
    truth = ctx.render(sid, cam, capi.settings_from_scene(sc, capi.MODE_WAVEFRONT, seed=77, spp=4096))
    st = capi.settings_from_scene(sc, capi.MODE_REPLAY)
    st.denoising_spp = 8
    albedo = ctx.render_aov(sid, cam, st, capi.AOV_DENOISING_ALBEDO)
    normal = ctx.render_aov(sid, cam, st, capi.AOV_DENOISING_NORMAL)
    ctx.release(sid)
    return noisy, truth, albedo, normal


CASES = {
    "cornell": (lambda: synth.cornell(width=128, height=128, spp=8, mixed=True, integrator=1,
                                      max_bounces=6, env_texture=True), 0.4, 0.45),
    "spheres": (lambda: synth.spheres_grids(tri_budget=20000, width=160, height=90, spp=8, max_bounces=8,
                                            env_width=128, env_height=64, sun_peak_over_median=30.0),
                0.8, 0.92),
}


@pytest.fixture(scope="module")
def cases(gpu_ctx):
    return {k: _case(gpu_ctx, f()) for k, (f, _, _) in CASES.items()}


@pytest.mark.parametrize("name", list(CASES))
def test_denoiser_reduces_error_against_converged_render(gpu_ctx, cases, name):
    noisy, truth, albedo, normal = cases[name]
    _, bound_guided, bound_plain = CASES[name]
    e0 = _tmse(noisy, truth)
    guided = gpu_ctx.denoise(noisy, albedo, normal)
    plain = gpu_ctx.denoise(noisy)
    r_guided, r_plain = _tmse(guided, truth) / e0, _tmse(plain, truth) / e0
    print(f"{name}: tone-mapped MSE ratio guided {r_guided:.3f}, colour only {r_plain:.3f}")
    assert np.isfinite(guided).all() and np.isfinite(plain).all()
    assert r_guided <= bound_guided
    assert r_plain <= bound_plain


def test_denoiser_entry_points_agree_and_are_deterministic(gpu_ctx, cases, tmp_path):
    noisy, truth, albedo, normal = cases["cornell"]
    H, W, _ = noisy.shape
    a = gpu_ctx.denoise(noisy, albedo, normal)
    b = gpu_ctx.denoise(noisy, albedo, normal)
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    dev = [torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in (noisy, albedo, normal)]
    out = torch.empty_like(dev[0])
    torch.cuda.synchronize()  # the denoiser runs on the context's own stream
    gpu_ctx.denoise_device(W, H, dev[0].data_ptr(), dev[1].data_ptr(), dev[2].data_ptr(), True,
                           out.data_ptr())
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy().view(np.uint32), a.view(np.uint32))
    # in place
    gpu_ctx.denoise_device(W, H, dev[0].data_ptr(), dev[1].data_ptr(), dev[2].data_ptr(), True,
                           dev[0].data_ptr())
    torch.cuda.synchronize()
    assert np.array_equal(dev[0].cpu().numpy().view(np.uint32), a.view(np.uint32))
    # the C++ class, as an application calls it
    from petrichor_gb300 import _build
    lib = _build.build()
    exe = str(tmp_path / "denoise_client")
    subprocess.run(["g++", "-std=c++17", "-O2", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "denoise_client.cpp"), "-L", os.path.dirname(lib),
                    "-lpetrichor_gb300", f"-Wl,-rpath,{os.path.dirname(lib)}", "-o", exe], check=True)
    np.concatenate([noisy.ravel(), albedo.ravel(), normal.ravel()]).astype(np.float32).tofile(
        tmp_path / "in.bin")
    for mode, ref in (([], a), (["colour-only"], gpu_ctx.denoise(noisy))):
        subprocess.run([exe, str(W), str(H), str(tmp_path / "in.bin"), str(tmp_path / "out.bin"), *mode],
                       check=True, timeout=120)
        got = np.fromfile(tmp_path / "out.bin", np.float32).reshape(H, W, 3)
        assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))


def test_denoiser_keeps_constant_images_and_cleans_non_finite_pixels(gpu_ctx):
    img = np.full((37, 53, 3), 0.37, np.float32)
    img[..., 1] = 1.5
    out = gpu_ctx.denoise(img)
    np.testing.assert_allclose(out, img, rtol=1e-5)
    bad = img.copy()
    bad[5, 7] = np.inf
    bad[9, 11, 2] = np.nan
    out = gpu_ctx.denoise(bad, hdr=False)
    assert np.isfinite(out).all()


def test_denoiser_rejects_bad_arguments(gpu_ctx):
    with pytest.raises(capi.PtError):
        gpu_ctx.denoise_device(0, 4, 1, 0, 0, True, 1)
    with pytest.raises(capi.PtError):
        gpu_ctx.denoise_device(4, 4, 0, 0, 0, True, 1)


def test_denoiser_full_hd_time(gpu_ctx):
    import time
    W, H = 1920, 1080
    rng = np.random.default_rng(3)
    dev = [torch.from_numpy(rng.random((H, W, 3), dtype=np.float32)).cuda() for _ in range(3)]
    out = torch.empty_like(dev[0])
    torch.cuda.synchronize()
    args = (W, H, dev[0].data_ptr(), dev[1].data_ptr(), dev[2].data_ptr(), True, out.data_ptr())
    gpu_ctx.denoise_device(*args)  # runs on the context's stream; synchronize waits for it
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(10):
        gpu_ctx.denoise_device(*args)
    torch.cuda.synchronize()
    ms = (time.perf_counter() - t0) / 10 * 1e3
    print(f"1920x1080 guided denoise: {ms:.2f} ms per image (wall, includes launches)")
    assert ms < 50.0
