"""Wave planning of the batched and served forms, on the host (no device).

A C++ client (tests/cpp/wave_plan.cpp) links the library and runs its wave planner
(PlanWaves) and wave shaping (ShapeOf, with the first-bounce rasterisation choice of
PrepareRasterUnits) on seeded random job lists. The checks are the planner's contract:
- every job's samples are planned exactly once, in increasing sample order across the
  waves (so a job's per-pixel sums, and its film, do not depend on the packing);
- a wave holds at most `cap` paths and `maxUnits` units, and a new wave starts only when
  the next sample block does not fit;
- each wave's path and pixel ranges are consecutive in unit order, after the units whose
  first bounce is rasterised have been moved behind the traced ones;
- a unit is rasterised exactly when its job allows it: a pinhole PathTracing camera near
  the scene (within 2^19 box widenings of the origin), a wave without queue-polled
  SimplePathTracing jobs, and at least 16 of the unit's rays per triangle (2 with
  primary_traversal 2; none with primary_traversal 1); its records follow those of the
  rasterised units before it;
- the wave's bounce count, integrator and sole job follow its units.
"""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "wave_plan.cpp")


@pytest.fixture(scope="module")
def planner(tmp_path_factory):
    from petrichor_gb300 import _build
    lib = _build.build()
    exe = str(tmp_path_factory.mktemp("plan") / "wave_plan")
    libdir = os.path.dirname(lib)
    subprocess.run(["g++", "-std=c++17", "-O2", "-Wall", "-Werror",
                    "-I", os.path.join(ROOT, "petrichor_gb300", "csrc"),
                    "-I", os.path.join(ROOT, "include"),
                    "-I", os.path.join(_build.CUDA_HOME, "include"),
                    SRC, "-L", libdir, "-lpetrichor_gb300", f"-Wl,-rpath,{libdir}", "-o", exe],
                   check=True)
    return exe


def _plan(exe, cap, max_units, primary, jobs):
    lines = [f"{cap} {max_units} {primary} {len(jobs)}"]
    for j in jobs:
        lines.append("{w} {h} {spp} {mb} {integ} {ap} {tris} {camx} {eps}".format(**j))
    r = subprocess.run([exe], input="\n".join(lines) + "\n", capture_output=True, text=True,
                       timeout=60, check=True)
    if r.stdout.strip() == "plan failed":
        return None
    waves = []
    for ln in r.stdout.splitlines():
        f = ln.split()
        if f[0] == "wave":
            keys = ["nPaths", "nPixelUnits", "iters", "integrator", "soleJob", "raster",
                    "rasterFrom", "rasterUnit0", "nUnits"]
            waves.append({**dict(zip(keys, map(int, f[1:]))), "units": []})
        else:
            keys = ["job", "s0", "sw", "pathBase", "pixelBase", "recBase"]
            waves[-1]["units"].append(dict(zip(keys, map(int, f[1:]))))
    return waves


EPS = 2.0 ** -20  # box widening: the camera is near within 2 * 2^18 * EPS = 0.5


def _random_jobs(rng):
    jobs = []
    for _ in range(int(rng.integers(1, 13))):
        jobs.append(dict(w=int(rng.integers(1, 65)), h=int(rng.integers(1, 65)),
                         spp=int(rng.choice([1, 3, 16, 64, 300])),
                         mb=int(rng.integers(0, 17)),
                         integ=int(rng.random() < 0.85),  # 1 PathTracing, 0 SimplePathTracing
                         ap=0.0 if rng.random() < 0.8 else 0.1,
                         tris=int(rng.choice([0, 10, 300, 5000])),
                         camx=float(rng.choice([0.25, -0.5, 0.75])), eps=EPS))
    return jobs


def _eligible(j, unit, primary, wave_polled):
    if primary == 1 or wave_polled:
        return False
    per_tri = 2 if primary == 2 else 16
    near = abs(j["camx"]) <= 2.0 * 2.0 ** 18 * j["eps"]
    return (j["ap"] == 0.0 and j["tris"] > 0 and near and j["integ"] == 1 and
            j["w"] * j["h"] * unit["sw"] >= per_tri * j["tris"])


@pytest.mark.parametrize("seed", range(40))
def test_plans_cover_samples_in_order_and_respect_limits(planner, seed):
    rng = np.random.default_rng(seed)
    jobs = _random_jobs(rng)
    cap = int(rng.choice([500, 4096, 20000, 300000]))
    max_units = int(rng.integers(1, 9))
    primary = int(rng.integers(0, 3))
    waves = _plan(planner, cap, max_units, primary, jobs)
    too_big = any(j["w"] * j["h"] > cap for j in jobs)
    assert (waves is None) == too_big
    if waves is None:
        return
    nxt = [0] * len(jobs)  # next sample of each job, in wave order
    for wi, wv in enumerate(waves):
        units = wv["units"]
        assert wv["nUnits"] == len(units) <= max_units
        assert 0 < wv["nPaths"] <= cap
        # sample blocks: each job's blocks in increasing order, without gaps (within a
        # wave the units may be reordered, but a job has one block per wave at most
        # unless its blocks are consecutive)
        for u in sorted(units, key=lambda u: (u["job"], u["s0"])):
            assert u["s0"] == nxt[u["job"]] and u["sw"] >= 1
            nxt[u["job"]] += u["sw"]
        # consecutive path and pixel ranges in unit order
        paths = pixels = 0
        for u in units:
            P = jobs[u["job"]]["w"] * jobs[u["job"]]["h"]
            assert u["pathBase"] == paths and u["pixelBase"] == pixels
            paths += P * u["sw"]
            pixels += P
        assert paths == wv["nPaths"] and pixels == wv["nPixelUnits"]
        # the wave's bounce count, integrator and sole job
        js = [jobs[u["job"]] for u in units]
        polled = any(j["integ"] == 0 for j in js)
        assert wv["iters"] == (-1 if polled else max(j["mb"] + 1 for j in js))
        integ = {j["integ"] for j in js}
        assert wv["integrator"] == (integ.pop() if len(integ) == 1 else -1)
        ids = {u["job"] for u in units}
        assert wv["soleJob"] == (ids.pop() if len(ids) == 1 else -1)
        # rasterised units: exactly the eligible ones, after the traced ones, in order
        ras = [_eligible(jobs[u["job"]], u, primary, polled) for u in units]
        k0 = wv["rasterUnit0"]
        assert ras == [False] * k0 + [True] * (len(units) - k0)
        if k0 == len(units):
            assert wv["raster"] == 0 and wv["rasterFrom"] == wv["nPaths"]
            assert all(u["recBase"] == -1 for u in units)
        else:
            assert wv["rasterFrom"] == units[k0]["pathBase"]
            rec = 0
            for u in units[k0:]:
                assert u["recBase"] == rec
                rec += jobs[u["job"]]["tris"]
            assert wv["raster"] == rec
            assert all(u["recBase"] == -1 for u in units[:k0])
        # greedy packing: the next wave starts only when its first block (the lowest job
        # of that wave: jobs are planned in order) did not fit
        if wi + 1 < len(waves):
            j0 = min(u["job"] for u in waves[wi + 1]["units"])
            P0 = jobs[j0]["w"] * jobs[j0]["h"]
            assert len(units) == max_units or wv["nPaths"] + P0 > cap
    assert nxt == [j["spp"] for j in jobs]


def test_one_job_larger_than_a_wave_is_refused(planner):
    job = dict(w=64, h=64, spp=4, mb=4, integ=1, ap=0.0, tris=10, camx=0.0, eps=EPS)
    assert _plan(planner, 4095, 8, 0, [job]) is None
    waves = _plan(planner, 4096, 8, 0, [job])
    assert [u["sw"] for wv in waves for u in wv["units"]] == [1, 1, 1, 1]


def test_far_camera_and_thin_lens_are_traced(planner):
    """Rasterisation needs a pinhole camera near the scene: far cameras (beyond 2^19 box
    widenings) and thin lenses keep their first bounce traced."""
    base = dict(w=64, h=64, spp=64, mb=4, integ=1, ap=0.0, tris=100, camx=0.0, eps=EPS)
    near = _plan(planner, 1 << 20, 8, 0, [base])[0]
    assert near["raster"] == 100 and near["rasterUnit0"] == 0
    far = _plan(planner, 1 << 20, 8, 0, [dict(base, camx=0.51)])[0]
    lens = _plan(planner, 1 << 20, 8, 0, [dict(base, ap=0.01)])[0]
    assert far["raster"] == 0 and lens["raster"] == 0
    # 16 rays per triangle by default; 2 with primary_traversal 2
    few = dict(base, spp=1, tris=300)  # 4096 rays, 13.7 per triangle
    assert _plan(planner, 1 << 20, 8, 0, [few])[0]["raster"] == 0
    assert _plan(planner, 1 << 20, 8, 2, [few])[0]["raster"] == 300
    assert _plan(planner, 1 << 20, 8, 1, [base])[0]["raster"] == 0
