"""The checked build (PT_CHECK=1): every node, primitive and queue index is tested on
the device before it is used, and a bad one sets an error bit instead of faulting
(in place of compute-sanitizer, which this pool does not run). The replay, wavefront,
AOV, batch and closest-hit paths run on golden and synthetic scenes under it; every
status word must stay clear and the replay films must still equal the reference's."""
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu
pytest.importorskip("torch")

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SCRIPT = r"""
import sys
import numpy as np
import torch
sys.path.insert(0, ROOT)
sys.path.insert(0, ROOT + "/tests")
from petrichor_gb300 import capi, synth, _build
from conftest import GOLDEN_CASES, golden_scene
L = capi.load()
assert L._name.startswith(_build.CHECK_DIR), L._name
golden = np.load(ROOT + "/tests/golden/golden.npz")
ctx = capi.Context()
def status():
    return ctx.stats().last_device_status
for name in GOLDEN_CASES:
    sc = golden_scene(golden, name)
    film = capi.render_scene(sc, mode=capi.MODE_REPLAY, ctx=ctx)
    assert status() == 0, (name, status())
    assert np.array_equal(film.view(np.uint32), golden[name + "/film"].view(np.uint32)), name
    capi.render_scene(sc, mode=capi.MODE_WAVEFRONT, ctx=ctx)
    assert status() == 0, (name, "wavefront", status())
scenes = [synth.spheres_grids(tri_budget=200000, width=160, height=90, spp=8, env_width=128, env_height=64),
          synth.terrain_rocks(terrain_n=150, n_rocks=80, rock_tris=120, width=96, height=64, spp=4,
                              env_width=64, env_height=32),
          synth.textured_spheres(), synth.bvh_ties()]
jobs = []
for sc in scenes:
    sid = ctx.upload(sc)
    cam = capi.camera_from_scene(sc)
    st = capi.settings_from_scene(sc, capi.MODE_WAVEFRONT, seed=3)
    ctx.render(sid, cam, st)
    assert status() == 0, status()
    for aov in (capi.AOV_UV, capi.AOV_DENOISING_ALBEDO, capi.AOV_DENOISING_NORMAL):
        ctx.render_aov(sid, cam, capi.settings_from_scene(sc, capi.MODE_REPLAY), aov)
    f = torch.empty(st.width * st.height * 3, device="cuda")
    jobs.append((sid, cam, st, f))
ctx.batch_render([(sid, cam, st, f.data_ptr()) for sid, cam, st, f in jobs])
torch.cuda.synchronize()
assert status() == 0, status()
sc = scenes[0]
rays = np.random.default_rng(1).standard_normal((4096, 6)).astype(np.float32)
r = torch.from_numpy(rays).cuda()
tri = torch.empty(4096, dtype=torch.int32, device="cuda")
dist = torch.empty(4096, dtype=torch.float32, device="cuda")
ctx.trace_closest(jobs[0][0], 4096, r.data_ptr(), 0.0, 3.4e38, tri.data_ptr(), dist.data_ptr())
torch.cuda.synchronize()
print("checked build clean")
"""


def test_checked_build_reports_no_bounds_errors():
    env = dict(os.environ, PT_GB300_CHECKED="1")
    r = subprocess.run([sys.executable, "-c", SCRIPT.replace("ROOT", repr(ROOT))], env=env,
                       capture_output=True, text=True, timeout=1500, cwd=ROOT)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-4000:]
    assert "checked build clean" in r.stdout
