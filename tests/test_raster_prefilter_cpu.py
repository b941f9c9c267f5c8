"""The rasterised first bounce's filters never drop a hit (host restatement, float32).

RasterSetupKernel (csrc/raster_primary.cuh) keeps, per triangle, a pixel rectangle and a
cone of directions (three planes through the camera and the triangle's edges, widened by
an angular margin); RasterSegment runs the exact triangle test only for samples inside
both. Here the same float32 operations (no fused multiply-add, as the kernels are built)
are restated with numpy and checked on the benchmark scene's own camera and triangles
(1.0M triangles, 1920x1080) and on a camera inside the Cornell box (walls reaching
behind the camera plane): every (primary ray, triangle) pair that the triangle test
accepts lies in the triangle's rectangle and inside its cone.
"""
import numpy as np
import pytest

from petrichor_gb300 import capi, synth
from petrichor_gb300.scene_io import Camera

f32 = np.float32


def _cross(a, b):
    return np.stack([a[..., 1] * b[..., 2] - a[..., 2] * b[..., 1],
                     a[..., 2] * b[..., 0] - a[..., 0] * b[..., 2],
                     a[..., 0] * b[..., 1] - a[..., 1] * b[..., 0]], -1)


def _dot(a, b):
    return a[..., 0] * b[..., 0] + a[..., 1] * b[..., 1] + a[..., 2] * b[..., 2]


def _rays(cam, W, H, x0, x1, y0, y1, spp, seed):
    """Primary rays of pixels [x0, x1) x [y0, y1): GenerateRay's pinhole form in float32."""
    rng = np.random.default_rng(seed)
    ys, xs = np.mgrid[y0:y1, x0:x1]
    px = np.repeat(xs.ravel(), spp).astype(f32)
    py = np.repeat(ys.ravel(), spp).astype(f32)
    r0 = rng.random(px.size).astype(f32)
    r1 = rng.random(px.size).astype(f32)
    r0[::97] = f32(1.0)  # the sampler can round to 1.0
    pos = np.array(cam.pos[:3], f32)
    right, up, fwd = (np.array(v[:3], f32) for v in (cam.right, cam.up, cam.forward))
    asp = f32(W) / f32(H)
    u = (px + r0) / f32(W) - f32(0.5)
    v = (py + r1) / f32(H) - f32(0.5)
    hp, fd = f32(cam.h_perf), f32(cam.focus_dist)
    s = (pos + right * (u * hp * fd * asp)[:, None] + (-up) * (v * hp * fd)[:, None] + fwd * fd)
    d = s - pos
    d = d / np.sqrt(_dot(d, d))[:, None]
    return pos, d.astype(f32), px.astype(np.int64), py.astype(np.int64)


def _setup(cam, W, H, v0, e1, e2):
    """RasterSetupKernel's cone planes, margins and pixel rectangle, per triangle."""
    pos = np.array(cam.pos[:3], f32)
    right, up, fwd = (np.array(v[:3], f32) for v in (cam.right, cam.up, cam.forward))
    a = [v0 - pos, (v0 + e1) - pos, (v0 + e2) - pos]
    n = [_cross(a[0], e1), _cross(a[1], e2 - e1), _cross(a[2], e2 * f32(-1.0))]
    ce = _cross(e1, e2)
    side = _dot(a[0], ce)
    ok = np.abs(side) > f32(1e-5) * np.sqrt(_dot(a[0], a[0]) * _dot(ce, ce))
    sg = np.where(side > 0, f32(1), f32(-1))
    # the absolute part of the margin: 2^-19 max|edge| (|v0 - camera| + max|edge|)
    emax = np.sqrt(np.maximum(np.maximum(_dot(e1, e1), _dot(e2, e2)), _dot(e2 - e1, e2 - e1)))
    mt = np.ldexp(emax * (np.sqrt(_dot(a[0], a[0])) + emax), -19).astype(f32)
    m = []
    for k in range(3):
        n[k] = np.where(ok[:, None], n[k] * sg[:, None], f32(0))
        m.append(np.where(ok, f32(2e-5) * np.sqrt(_dot(n[k], n[k])) + mt, f32(1)))
    rr, uu = f32(1) / _dot(right, right), f32(1) / _dot(up, up)
    X = np.stack([_dot(av, right) * rr for av in a], 1)
    Y = np.stack([_dot(av, up) * uu for av in a], 1)
    Z = np.stack([_dot(av, fwd) for av in a], 1)
    zc = f32(1e-6) * np.abs(Z).max(1) + f32(1e-30)
    front = (Z > zc[:, None]).all(1)
    anyf = (Z > 0).any(1)
    asp = f32(W) / f32(H)
    with np.errstate(divide="ignore", invalid="ignore"):
        px = np.clip((X / (Z * f32(cam.h_perf) * asp) + f32(0.5)) * f32(W), -1e9, 1e9)
        py = np.clip((-Y / (Z * f32(cam.h_perf)) + f32(0.5)) * f32(H), -1e9, 1e9)
    x0 = np.maximum(0, np.floor(px.min(1) - f32(0.01)).astype(np.int64) - 1)
    x1 = np.minimum(W - 1, np.floor(px.max(1) + f32(0.01)).astype(np.int64))
    y0 = np.maximum(0, np.floor(py.min(1) - f32(0.01)).astype(np.int64) - 1)
    y1 = np.minimum(H - 1, np.floor(py.max(1) + f32(0.01)).astype(np.int64))
    x0 = np.where(front, x0, np.where(anyf, 0, 1))
    x1 = np.where(front, x1, np.where(anyf, W - 1, 0))
    y0 = np.where(front, y0, np.where(anyf, 0, 1))
    y1 = np.where(front, y1, np.where(anyf, H - 1, 0))
    return n, m, (x0, x1, y0, y1)


def _tri_hits(o, d, v0, e1, e2):
    """TriIntersect (Cramer form, correctly rounded 1/det) for every ray x triangle."""
    ce = _cross(e1, e2)[None]
    D = d[:, None, :]
    with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
        inv = f32(1) / _dot(-D, ce)
        vec = (o - v0)[None]
        w1 = _dot(vec, _cross(D, e2[None])) * inv
        w2 = _dot(vec, _cross(e1[None], D)) * inv
        t = _dot(vec, ce) * inv
        return ((w1 >= 0) & (w1 < 1) & (w2 >= 0) & (w2 < 1) & (w1 + w2 < 1) & (t >= 0)
                & np.isfinite(t))


def _check(sc, cam, W, H, window, spp, cand_margin=4.0, seed=0):
    x0, x1, y0, y1 = window
    P = sc.positions.astype(f32)
    I = sc.indices
    v0, v1, v2 = P[I[:, 0]], P[I[:, 1]], P[I[:, 2]]
    e1, e2 = v1 - v0, v2 - v0
    n, m, rect = _setup(cam, W, H, v0, e1, e2)
    # candidates: rectangles near the window (the rectangle itself is under test, so a
    # generous margin)
    near = ((rect[0] <= x1 + cand_margin) & (rect[1] >= x0 - cand_margin) &
            (rect[2] <= y1 + cand_margin) & (rect[3] >= y0 - cand_margin))
    # and triangles whose float64 projection is near (independent of the rectangle)
    cand = np.nonzero(near | _near64(sc, cam, W, H, window, cand_margin))[0]
    o, d, px, py = _rays(cam, W, H, x0, x1, y0, y1, spp, seed)
    hits = 0
    for c in np.array_split(cand, max(1, len(cand) // 512)):
        h = _tri_hits(o, d, v0[c], e1[c], e2[c])
        r_, t_ = np.nonzero(h)
        if r_.size == 0:
            continue
        hits += r_.size
        tri = c[t_]
        dd = d[r_]
        for k in range(3):
            cone = _dot(n[k][tri], dd) + m[k][tri]
            assert np.all(cone >= 0), f"cone plane {k} drops {np.sum(cone < 0)} hits"
        inside = ((px[r_] >= rect[0][tri]) & (px[r_] <= rect[1][tri]) &
                  (py[r_] >= rect[2][tri]) & (py[r_] <= rect[3][tri]))
        assert np.all(inside), f"{np.sum(~inside)} hits outside their rectangle"
    return hits


def _near64(sc, cam, W, H, window, margin):
    x0, x1, y0, y1 = window
    pos = np.array(cam.pos[:3])
    R, U, F = (np.array(v[:3]) for v in (cam.right, cam.up, cam.forward))
    A = sc.positions.astype(np.float64)[sc.indices] - pos
    X = (A @ R) / (R @ R)
    Y = (A @ U) / (U @ U)
    Z = A @ F
    with np.errstate(divide="ignore", invalid="ignore"):
        px = (X / (Z * cam.h_perf * W / H) + 0.5) * W
        py = (-Y / (Z * cam.h_perf) + 0.5) * H
    crossing = (Z <= 0).any(1)
    return crossing | ((px.min(1) <= x1 + margin) & (px.max(1) >= x0 - margin) &
                       (py.min(1) <= y1 + margin) & (py.max(1) >= y0 - margin))


def test_benchmark_scene_filters_keep_every_hit():
    sc = synth.spheres_grids()
    cam = capi.camera_from_scene(sc)
    W, H = sc.settings.width, sc.settings.height
    hits = 0
    for win, seed in (((900, 940, 520, 548), 1), ((300, 330, 800, 824), 2), ((1500, 1530, 200, 220), 3)):
        hits += _check(sc, cam, W, H, win, spp=4, seed=seed)
    assert hits > 3000


def test_sliver_triangles_filters_keep_every_hit():
    """Long thin triangles (edge ratios up to 2000:1), many seen nearly edge-on: relative
    to a short edge, the triangle test's rounding reaches farthest outside such
    triangles; the cone margin's absolute part bounds it whatever the shape."""
    from types import SimpleNamespace
    rng = np.random.default_rng(11)
    n = 4000
    c = rng.uniform(-2.0, 2.0, (n, 3)).astype(f32) * f32([1, 1, 0.5]) + f32([0, 4, 1])
    u = rng.normal(size=(n, 3))
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    w = np.cross(u, rng.normal(size=(n, 3)))
    w /= np.linalg.norm(w, axis=1, keepdims=True)
    length = rng.uniform(0.05, 1.0, n)
    width = length / np.exp(rng.uniform(np.log(5), np.log(2000), n))
    v0 = c
    v1 = (c + u * length[:, None]).astype(f32)
    v2 = (c + u * (0.5 * length)[:, None] + w * width[:, None]).astype(f32)
    pos = np.stack([v0, v1, v2], 1).reshape(-1, 3)
    sc = SimpleNamespace(positions=pos, indices=np.arange(3 * n, dtype=np.int32).reshape(n, 3))
    cam = Camera(pos=(0.0, -3.0, 1.2), view_dir=(0.0, 1.0, -0.05), fov=0.9, focus_target=None,
                 aperture=0.0)
    W, H = 160, 120
    hits = _check(sc, capi.camera_from_scene(SimpleNamespace(camera=cam)), W, H, (0, W, 0, H),
                  spp=4, cand_margin=1e9)
    assert hits > 1000


def test_camera_inside_the_box_filters_keep_every_hit():
    sc = synth.cornell(width=48, height=40, spp=1, mixed=True)
    sc = sc.copy_with(camera=Camera(pos=(0.05, -0.6, 1.1), view_dir=(0.2, 1.0, -0.1), fov=1.6,
                                    focus_target=None, aperture=0.0))
    cam = capi.camera_from_scene(sc)
    hits = _check(sc, cam, 48, 40, (0, 48, 0, 40), spp=8, cand_margin=1e9)
    assert hits > 48 * 40 * 8 * 0.9
