"""The serving loop's path-rate meter (PathRateMeter, used by csrc/server.cpp), on the host.

The server sizes its overdue rule by the GPU's path rate, measured from wave
retirements. With two wave lanes, two waves run at once and consecutive retirements can
fall a few milliseconds apart; a rate taken from single gaps then overstated the GPU
several times over and made every request look overdue (median latency 590 ms instead
of about 120 ms at 500 requests/s). The meter takes the paths retired over the span of
the last four gaps of a busy period. A C++ client (tests/cpp/path_rate.cpp) feeds it
retirement sequences.
"""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "path_rate.cpp")


@pytest.fixture(scope="module")
def meter(tmp_path_factory):
    from petrichor_gb300 import _build
    lib = _build.build()
    exe = str(tmp_path_factory.mktemp("rate") / "path_rate")
    libdir = os.path.dirname(lib)
    subprocess.run(["g++", "-std=c++17", "-O2", "-Wall", "-Werror",
                    "-I", os.path.join(ROOT, "petrichor_gb300", "csrc"),
                    "-I", os.path.join(ROOT, "include"),
                    "-I", os.path.join(_build.CUDA_HOME, "include"),
                    SRC, "-L", libdir, "-lpetrichor_gb300", f"-Wl,-rpath,{libdir}", "-o", exe],
                   check=True)

    def run(initial, events):
        """events: (now, paths, ok, busy_after); returns the rate after each."""
        text = f"{initial!r}\n" + "".join(f"{t!r} {p} {int(o)} {int(b)}\n" for t, p, o, b in events)
        r = subprocess.run([exe], input=text, capture_output=True, text=True, timeout=60,
                           check=True)
        return [float(x) for x in r.stdout.split()]
    return run


P = 1 << 24  # paths per wave


def _paired(t0, n, short=0.002, long=0.058):
    """Retirements of two lanes: gaps alternate short and long (30 ms per wave on average)."""
    ev, t = [], t0
    for k in range(n):
        t += short if k % 2 else long
        ev.append((t, P, True, True))
    return ev, t


def test_paired_retirements_give_the_mean_rate(meter):
    ev, _ = _paired(0.0, 60)
    rates = meter(1.5e9, ev)
    true = P / 0.030
    assert abs(rates[-1] / true - 1) < 0.03
    # single gaps would have read P / 2 ms, 15 times the true rate, every other wave
    assert max(rates) < 1.6e9 and min(rates[10:]) > 0.5 * true


def test_window_needs_four_gaps_and_enough_paths(meter):
    ev, _ = _paired(0.0, 4)
    assert meter(1.5e9, ev) == [1.5e9] * 4            # three gaps: no estimate yet
    small = [(0.001 * k, 1000, True, True) for k in range(1, 20)]
    assert meter(1.5e9, small) == [1.5e9] * 19         # windows of a few thousand paths


def test_idle_time_between_busy_periods_is_not_counted(meter):
    ev, t = _paired(0.0, 40)
    # the last wave of the period leaves nothing in flight, then the GPU idles for 5 s
    ev.append((t + 0.03, P, True, False))
    ev2, _ = _paired(t + 5.03, 40)
    rates = meter(1.5e9, ev + ev2)
    true = P / 0.030
    # the first retirements after the idle gap start a new window: no dip towards P / 5 s
    assert min(rates[40:]) > 0.8 * true
    assert abs(rates[-1] / true - 1) < 0.03


def test_failed_waves_are_not_counted(meter):
    ev, _ = _paired(0.0, 40)
    bad = [(t, P * 100, False, True) for t, _, _, _ in ev]   # errors carry no rate
    assert meter(1.5e9, bad) == [1.5e9] * 40
