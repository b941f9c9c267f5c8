"""The serving loop's state allocator (ArenaAllocator, used by csrc/server.cpp), on the host.

Admission against the state budget allocates each request's per-pixel sums and film
staging from one device buffer. A C++ client (tests/cpp/arena.cpp) runs seeded random
admit/retire sequences and prints the free list after every step. Checked: allocations
are 256-byte aligned, inside the budget and disjoint; an allocation takes the lowest free
range that fits and fails only when none does; released ranges merge with their free
neighbours (no two free ranges touch), and free plus allocated bytes always make the
budget.
"""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "arena.cpp")


@pytest.fixture(scope="module")
def arena(tmp_path_factory):
    from petrichor_gb300 import _build
    lib = _build.build()
    exe = str(tmp_path_factory.mktemp("arena") / "arena")
    libdir = os.path.dirname(lib)
    subprocess.run(["g++", "-std=c++17", "-O2", "-Wall", "-Werror",
                    "-I", os.path.join(ROOT, "petrichor_gb300", "csrc"),
                    "-I", os.path.join(ROOT, "include"),
                    "-I", os.path.join(_build.CUDA_HOME, "include"),
                    SRC, "-o", exe], check=True)
    return exe


def _round(b):
    return (b + 255) // 256 * 256


@pytest.mark.parametrize("seed", range(10))
def test_random_admit_retire_sequences(arena, seed):
    rng = np.random.default_rng(seed)
    budget = int(rng.choice([1 << 16, 1 << 18, 1 << 20, 1_500_000]))
    cmds, model = [f"reset {budget}"], []
    # the sequence is generated up front; frees pick from what the model expects to be live
    # and are validated against the allocator's replies afterwards
    live_sizes = []
    for _ in range(400):
        if live_sizes and rng.random() < 0.45:
            k = int(rng.integers(len(live_sizes)))
            cmds.append(("free", k))
            live_sizes.pop(k)
        else:
            b = int(rng.choice([1, 255, 256, 257, 4096, 30_000, 250_000]))
            cmds.append(("alloc", b))
            live_sizes.append(b)
    # run step by step, so that frees name the offsets the allocator really returned
    proc = subprocess.Popen([arena], stdin=subprocess.PIPE, stdout=subprocess.PIPE, text=True)

    def step(line):
        proc.stdin.write(line + "\n")
        proc.stdin.flush()
        out = []
        while True:
            ln = proc.stdout.readline().split()
            out.append(ln)
            if ln[0] == "free":
                return out

    def ranges(ln):
        return [tuple(map(int, x.split(":"))) for x in ln[1:]]

    free = ranges(step(cmds[0])[-1])
    assert free == [(0, budget)]
    live = []  # (offset, requested bytes)
    fails = 0
    for c in cmds[1:]:
        if c[0] == "alloc":
            b = _round(c[1])
            fits = [(o, n) for o, n in free if n >= b]
            out = step(f"alloc {c[1]}")
            at = int(out[0][1])
            if at < 0:
                assert not fits
                fails += 1
                live.append(None)
            else:
                assert at == fits[0][0] and at % 256 == 0 and at + b <= budget
                live.append((at, c[1]))
            free = ranges(out[-1])
        else:
            k = c[1]
            item = live.pop(k)
            if item is None:
                continue
            free = ranges(step(f"free {item[0]} {item[1]}")[-1])
        # invariants: disjoint, coalesced, conserved
        used = sorted((o, _round(b)) for o, b in (x for x in live if x))
        spans = sorted(free + used)
        pos = 0
        for o, n in spans:
            assert o == pos and n > 0
            pos += n
        assert pos == budget
        assert all(free[i][0] + free[i][1] < free[i + 1][0] for i in range(len(free) - 1))
    # everything released: one free range again
    for x in live:
        if x:
            free = ranges(step(f"free {x[0]} {x[1]}")[-1])
    assert free == [(0, budget)]
    proc.stdin.close()
    assert proc.wait(timeout=30) == 0
    assert 0 < fails < len(cmds)  # the sequences do exhaust the budget at times


def test_release_merges_both_neighbours(arena):
    script = "\n".join(["reset 4096", "alloc 1000", "alloc 1000", "alloc 1000", "free 0 1000",
                        "free 2048 1000", "free 1024 1000"]) + "\n"
    r = subprocess.run([arena], input=script, capture_output=True, text=True, timeout=30,
                       check=True)
    frees = [ln for ln in r.stdout.splitlines() if ln.startswith("free")]
    assert frees[1:4] == ["free 1024:3072", "free 2048:2048", "free 3072:1024"]
    assert frees[4] == "free 0:1024 3072:1024"
    assert frees[5] == "free 0:1024 2048:2048"
    assert frees[6] == "free 0:4096"
