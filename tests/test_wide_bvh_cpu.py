"""The 4-wide (and 8-wide) BVH of the throughput traversal, checked on the host.

The wide tree is collapsed from the reference's binary tree (CollapseWide,
csrc/bvh_builder.cpp). The traversal tests every slot's box without reading its code
first, so empty slots must carry boxes at +infinity; every triangle must sit in exactly
one leaf whose (widened) box holds its vertices; inner boxes must hold their children's;
leaves of more than 63 triangles become chains of chunks; the collapse of a large tree
runs on several threads and must give the single-threaded array bit for bit. A C++
client (tests/cpp/wide_bvh.cpp) builds the trees of several soups and walks them.
"""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "wide_bvh.cpp")


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    from petrichor_gb300 import _build
    lib = _build.build()
    exe = str(tmp_path_factory.mktemp("wide") / "wide_bvh")
    libdir = os.path.dirname(lib)
    subprocess.run(["g++", "-std=c++17", "-O2", "-Wall", "-Werror",
                    "-I", os.path.join(ROOT, "petrichor_gb300", "csrc"),
                    SRC, "-L", libdir, "-lpetrichor_gb300", f"-Wl,-rpath,{libdir}", "-o", exe],
                   check=True)
    return exe


def _check(exe, tmp_path, pos, idx, width):
    f = tmp_path / "soup.bin"
    with open(f, "wb") as fh:
        np.array([len(pos), len(idx)], np.int32).tofile(fh)
        np.asarray(pos, np.float32).tofile(fh)
        np.asarray(idx, np.int32).tofile(fh)
    r = subprocess.run([exe, str(f), str(width)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.startswith("ok"), r.stdout + r.stderr
    return dict(kv.split("=") for kv in r.stdout.split()[1:])


def _soup(rng, n, scale=10.0):
    c = rng.uniform(-scale, scale, (n, 1, 3))
    pos = (c + rng.normal(0, scale * 0.02, (n, 3, 3))).reshape(-1, 3)
    return pos, np.arange(3 * n).reshape(n, 3)


def _grid(nx, ny, z=lambda x, y: 0.1 * np.sin(x) * np.cos(y)):
    xs, ys = np.meshgrid(np.arange(nx + 1, dtype=np.float64), np.arange(ny + 1, dtype=np.float64))
    pos = np.stack([xs, ys, z(xs, ys)], -1).reshape(-1, 3)
    v = lambda i, j: j * (nx + 1) + i
    idx = []
    for j in range(ny):
        for i in range(nx):
            idx += [[v(i, j), v(i + 1, j), v(i + 1, j + 1)], [v(i, j), v(i + 1, j + 1), v(i, j + 1)]]
    return pos, np.array(idx)


@pytest.mark.parametrize("width", [4, 8])
def test_random_soups(checker, tmp_path, width):
    rng = np.random.default_rng(width)
    for n, scale in [(1, 1.0), (2, 1.0), (5, 3.0), (777, 10.0), (20000, 10.0), (3000, 2.5e4),
                     (150_000, 10.0)]:  # from 65536 triangles the collapse runs on threads
        info = _check(checker, tmp_path, *_soup(rng, n, scale), width)
        assert int(info["leaves"]) >= 1


@pytest.mark.parametrize("width", [4, 8])
def test_height_field_grid(checker, tmp_path, width):
    info = _check(checker, tmp_path, *_grid(200, 180), width)
    assert int(info["maxleaf"]) <= 4           # the binned-SAH leaf rule


def test_many_identical_triangles_on_threads(checker, tmp_path):
    """70,000 copies of one triangle beside a soup: a leaf that no split divides becomes a
    long chain of chunks, collapsed on threads like the rest."""
    rng = np.random.default_rng(11)
    same = np.tile(np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32), (70_000, 1))
    soup, _ = _soup(rng, 5000, 10.0)
    pos = np.concatenate([same, soup + np.array([40.0, 0.0, 0.0])])
    n = len(pos) // 3
    info = _check(checker, tmp_path, pos, np.arange(3 * n).reshape(n, 3), 4)
    assert int(info["maxleaf"]) == 63 and int(info["leaves"]) > 70_000 // 63


def test_identical_triangles_become_a_chain_of_leaf_chunks(checker, tmp_path):
    pos = np.tile(np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32), (300, 1))
    idx = np.arange(900).reshape(300, 3)
    info = _check(checker, tmp_path, pos, idx, 4)
    # one leaf of 300 (no split separates equal centroids): chunks of 63, 63, 63, 63, 48
    assert int(info["leaves"]) == 5 and int(info["maxleaf"]) == 63


def test_widening_follows_the_largest_coordinate(checker, tmp_path):
    rng = np.random.default_rng(3)
    pos, idx = _soup(rng, 500, 1.0)
    pos = pos + np.array([4096.0, 0.0, 0.0])
    info = _check(checker, tmp_path, pos, idx, 4)
    far = float(np.abs(pos).max())
    assert float(info["eps"]) == pytest.approx(np.ldexp(np.float32(far), -18), rel=1e-6)
