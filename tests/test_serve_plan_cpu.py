"""The serving loop's wave plan (PlanServeWave, used by csrc/server.cpp), on the host.

A C++ client (tests/cpp/serve_plan.cpp) links the library and plans waves from request
lists given on stdin, with the server's own rule: least remaining work first, and requests
that have waited `overdue_waves` waves plus `overdue_factor` times their own rendering
time guaranteed `overdue_share` of every wave, oldest first. Timing is simulated, so the
starvation bound that a GPU test could not pin down (it depended on how fast Python
submits) is checked exactly here.
"""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "serve_plan.cpp")

# the server's constants (server.cpp): six waves plus the request's own time, whole waves
SERVER_RULE = dict(overdue_waves=6.0, overdue_factor=1.0, overdue_share=1.0)


@pytest.fixture(scope="module")
def plan(tmp_path_factory):
    from petrichor_gb300 import _build
    lib = _build.build()
    exe = str(tmp_path_factory.mktemp("serve") / "serve_plan")
    libdir = os.path.dirname(lib)
    subprocess.run(["g++", "-std=c++17", "-O2", "-Wall", "-Werror",
                    "-I", os.path.join(ROOT, "petrichor_gb300", "csrc"),
                    "-I", os.path.join(ROOT, "include"),
                    "-I", os.path.join(_build.CUDA_HOME, "include"),
                    SRC, "-L", libdir, "-lpetrichor_gb300", f"-Wl,-rpath,{libdir}", "-o", exe],
                   check=True)

    def run(reqs, cap, now, rate, max_units=8192, overdue_waves=6.0, overdue_factor=1.0,
            overdue_share=1.0):
        """reqs: (pixels, spp, scheduled, submit) tuples; returns [(request, sw), ...]."""
        lines = ["1", f"{cap} {max_units} {now!r} {rate!r} {overdue_waves!r} {overdue_factor!r} "
                      f"{overdue_share!r} {len(reqs)}"]
        lines += [f"{p} {s} {d} {t!r}" for p, s, d, t in reqs]
        r = subprocess.run([exe], input="\n".join(lines) + "\n", capture_output=True, text=True,
                           timeout=60, check=True)
        out = r.stdout.split("\n")
        assert out[0] == "plan 0"
        return [(int(f[1]), int(f[2])) for f in (ln.split() for ln in out[1:] if ln)]
    return run


@pytest.mark.parametrize("seed", range(12))
def test_least_remaining_work_first_when_none_is_overdue(plan, seed):
    rng = np.random.default_rng(seed)
    n = int(rng.integers(1, 40))
    reqs = [(int(rng.integers(1, 5000)), int(rng.integers(1, 64)), 0, 0.0) for _ in range(n)]
    reqs = [(p, s, int(rng.integers(0, s)), t) for p, s, _, t in reqs]  # some samples planned
    cap, max_units = int(rng.choice([4096, 65536, 1 << 20])), int(rng.integers(1, 12))
    picks = plan(reqs, cap, now=0.0, rate=1e9, max_units=max_units)
    remaining = [(s - d) * p for p, s, d, _ in reqs]
    order = sorted(range(n), key=lambda i: (remaining[i], i))  # stable: ties in list order
    # the picks follow that order, each request at most once, each block as large as fits
    seen = [i for i, _ in picks]
    assert len(set(seen)) == len(seen)
    assert seen == [i for i in order if i in set(seen)]
    paths = 0
    picked = dict(picks)
    for i in order:
        p, s, d, _ = reqs[i]
        room = (cap - paths) // p
        if i in picked:
            assert picked[i] == min(s - d, room) and picked[i] >= 1
            paths += p * picked[i]
        else:  # did not fit, or the wave had its blocks
            assert room < 1 or len([j for j in seen if order.index(j) < order.index(i)]) >= max_units
    assert paths <= cap and len(picks) <= max_units


def test_overdue_requests_take_their_share_first(plan):
    """One overdue request (1000 paths left) beside thirty fresh ones of 50 paths each; with
    half of the wave guaranteed to overdue requests, fresh requests fill the first half and
    the overdue one takes the second."""
    cap, rate = 1000, 1e6                    # a wave takes 1 ms
    old = (10, 100, 0, 0.0)                  # own time 1 ms; overdue after 6 + 1 ms
    fresh = [(10, 5, 0, 0.0095)] * 30        # submitted just now
    picks = plan([old] + fresh, cap, now=0.010, rate=rate, overdue_share=0.5)
    assert picks == [(k, 5) for k in range(1, 11)] + [(0, 50)]
    # before it is overdue, it is just the largest request: the fresh ones go first
    picks = plan([old] + fresh, cap, now=0.006, rate=rate, overdue_share=0.5)
    assert picks == [(k, 5) for k in range(1, 21)]
    # with the server's whole-wave share the overdue request takes all it can use
    picks = plan([old] + fresh, cap, now=0.010, rate=rate, **SERVER_RULE)
    assert picks == [(0, 100)]
    # overdue requests go oldest first
    older = (10, 100, 0, -0.001)
    picks = plan([old, older], cap, now=0.010, rate=rate, **SERVER_RULE)
    assert picks == [(1, 100)]


def _simulate(plan, rule, waves=120):
    """One long request (8 waves of work) at t = 0 behind a stream of short requests that
    would fill every wave on their own (one wave of them arrives per wave). Each wave takes
    its paths / rate seconds. Returns (time the long request's last samples were planned or
    None, the longest wait of a short request in waves)."""
    cap, rate = 1 << 16, 1e9
    wave_s = cap / rate
    reqs = [[1 << 12, 128, 0, 0.0]]            # 2^19 paths: 8 waves
    short = (1 << 10, 4)                         # 4096 paths: 16 per wave
    t, done_long, short_wait = 0.0, None, 0.0
    submit_of = {}
    for w in range(waves):
        for _ in range(cap // (short[0] * short[1])):
            submit_of[len(reqs)] = t
            reqs.append([short[0], short[1], 0, t])
        picks = plan([tuple(r) for r in reqs], cap, now=t, rate=rate, **rule)
        paths = 0
        for i, sw in picks:
            reqs[i][2] += sw
            paths += reqs[i][0] * sw
            if i > 0 and reqs[i][2] == reqs[i][1]:
                short_wait = max(short_wait, (t - submit_of[i]) / wave_s)
        if done_long is None and reqs[0][2] == reqs[0][1]:
            done_long = t
        t += max(paths, 1) / rate
    return done_long, short_wait


def test_long_request_is_not_starved_by_a_stream_of_short_ones(plan):
    # least work first alone: the long request never gets a sample while shorts keep coming
    never, _ = _simulate(plan, dict(overdue_waves=1e9, overdue_factor=0.0, overdue_share=1.0))
    assert never is None
    # the server's rule: overdue after 6 waves + its own time (8 waves), then it takes the
    # whole wave until done (8 more waves)
    done, short_wait = _simulate(plan, SERVER_RULE)
    wave_s = (1 << 16) / 1e9
    assert done is not None and done <= (6 + 8 + 8 + 1) * wave_s
    # the short requests waited at most those 8 waves behind it, plus their own wave
    assert short_wait <= 8 + 1
