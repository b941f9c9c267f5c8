"""File loaders of the C++ API (petrichor_gb300/csrc/cpp_loaders.cpp): the reference's
JSON scene format (SceneLoaderJson), OBJ assets, Radiance .hdr images and tone-mapped
.png output, driven by tests/cpp/load_scene.cpp.

CPU: what LoadRenderSetting + LoadAssets build (settings, camera in the reference's
call order, environment texels, materials, triangles), and the image writers. GPU: the
loaded scene renders through Petrichor::Render exactly as the oracle renders the same
scene given as arrays.
"""
import math
import os
import struct
import subprocess
import zlib

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "load_scene.cpp")
f32 = np.float32


@pytest.fixture(scope="module")
def exe(tmp_path_factory):
    from petrichor_gb300 import _build
    lib = _build.build()
    out = str(tmp_path_factory.mktemp("cpp") / "load_scene")
    d = os.path.dirname(lib)
    subprocess.run(["g++", "-std=c++17", "-O2", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), SRC,
                    "-L", d, "-lpetrichor_gb300", f"-Wl,-rpath,{d}", "-o", out], check=True)
    return out


def _rgbe_rows(W, H, seed):
    rng = np.random.default_rng(seed)
    px = rng.integers(0, 256, size=(H, W, 4), dtype=np.uint8)
    px[..., 3] = rng.integers(120, 140, size=(H, W))
    px[0, 0] = 0  # a black texel (exponent 0)
    return px


def _write_hdr(path, px, rle):
    H, W, _ = px.shape
    with open(path, "wb") as f:
        f.write(b"#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n\n" + f"-Y {H} +X {W}\n".encode())
        for y in range(H):
            if not rle:
                f.write(px[y].tobytes())
                continue
            f.write(bytes([2, 2, W >> 8, W & 255]))
            for c in range(4):
                row = px[y, :, c]
                x = 0
                while x < W:  # runs of equal bytes, else literal spans
                    run = 1
                    while x + run < W and run < 127 and row[x + run] == row[x]:
                        run += 1
                    if run >= 3:
                        f.write(bytes([128 + run, int(row[x])]))
                        x += run
                        continue
                    n = min(128, W - x)
                    f.write(bytes([n]) + row[x:x + n].tobytes())
                    x += n


def _decode(px):
    m = px[..., :3].astype(np.float64)
    e = px[..., 3:4].astype(np.int64)
    return np.where(e > 0, np.ldexp(m, e - 136), 0.0).astype(np.float32)


OBJ_A = """# quad, textured triangles, negative indices
v 0 0 0
v 1 0 0
v 1 1 0.25
v 0 1 0
v 0.5 0.5 1.5
vt 0 0
vt 1 0
vt 1 1
vt 0.25 0.75
vn 0 0 2
vn 0 1 1
vn 1 0 1
f 1/1/1 2/2/1 3/3/2 4/4/3
f 1/1/1 3/3/2 5/4/3
f -4/-3/-2 -3/-2/-1 -1/-1/-1
"""
OBJ_B = """o positions only
v -1 -1 0
v 2 -1 0
v -1 2 0
v 2 2 -0.5
f 1 2 3
f 2 4 3
"""


def _write_case(d):
    with open(os.path.join(d, "settings.json"), "w") as f:
        f.write('{"outputWidth": 24, "outputHeight": 16, "spp": 2, "denoising_spp": 4, "maxBounces": 3,'
                ' "tileWidth": 8, "tileHeight": 8, "numThreads": 0}')
    with open(os.path.join(d, "a.obj"), "w") as f:
        f.write(OBJ_A)
    with open(os.path.join(d, "b.obj"), "w") as f:
        f.write(OBJ_B)
    px = _rgbe_rows(16, 8, 5)
    _write_hdr(os.path.join(d, "sky.hdr"), px, rle=True)
    with open(os.path.join(d, "scene.json"), "w") as f:
        f.write("""{
 "materials": [
  {"type": "lambert", "name": "white", "base_color": [0.7, 0.6, 0.5]},
  {"type": "glossy", "name": "metal", "color": [0.9, 0.8, 0.4], "roughness": 0.3},
  {"type": "glass", "name": "gl", "color": [1, 1, 1], "ior": 1.45},
  {"type": "emission", "name": "light"},
  {"type": "mix", "name": "mixed", "mat0_name": "white", "mat1_name": "metal", "mix": 0.3}
 ],
 "camera": {"position": [0.5, -3.0, 1.2], "look_at": [0.5, 0.5, 0.3], "focus_pos": [0.5, 0.5, 0.4],
            "f_number": 4.0, "focal_length": 0.035},
 "env": {"base_color": [1.0, 0.9, 0.8], "texture": "sky.hdr"},
 "assets": [{"path": "a.obj", "mat": "mixed"}, {"path": "b.obj"}]
}
""")
    return px


def _parse_dump(path):
    rec = {"texel": [], "material": {}, "tri": [], "mixof": {}}
    h = lambda t: float.fromhex(t)
    for line in open(path):
        t = line.split()
        if t[0] == "settings":
            rec["settings"] = [int(x) for x in t[1:]]
        elif t[0] == "camera":
            v = [h(x) for x in t[1:]]
            rec["camera"] = dict(pos=v[0:3], fwd=v[3:6], right=v[6:9], up=v[9:12], hperf=v[12],
                                 focus=v[13], aperture=v[14])
        elif t[0] == "env":
            rec["env"] = ([h(x) for x in t[1:4]], int(t[4]), int(t[5]))
        elif t[0] == "texel":
            rec["texel"].append([h(x) for x in t[1:]])
        elif t[0] == "material":
            rec["material"][int(t[1])] = (int(t[2]), [h(x) for x in t[3:]])
        elif t[0] == "mixof":
            rec["mixof"][int(t[1])] = (int(t[2]), int(t[3]))
        elif t[0] == "map":
            mat, slot, tw, th = (int(x) for x in t[1:5])
            tex = np.array([h(x) for x in t[6:]], np.float32).reshape(th, tw, 3)
            rec.setdefault("maps", {})[(mat, slot)] = (tex, h(t[5]))
        elif t[0] == "tri":
            v = [h(x) for x in t[3:]]
            rec["tri"].append((int(t[1]), int(t[2]), np.array(v, np.float32).reshape(3, 3, 3)))
    return rec


def test_load_assets_builds_the_reference_scene(exe, tmp_path):
    px = _write_case(str(tmp_path))
    out = tmp_path / "dump.txt"
    r = subprocess.run([exe, "dump", str(tmp_path / "settings.json"), str(tmp_path / "scene.json"), str(out)],
                       capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stderr
    d = _parse_dump(out)
    assert d["settings"] == [24, 16, 2, 4, 3, 8, 8, 0]
    # camera: SetPosition, LookAt, FocusTo, SetFNumber (at the default 55 mm), SetFocalLength
    c = d["camera"]
    pos, look, focus = (np.array(v, f32) for v in ([0.5, -3.0, 1.2], [0.5, 0.5, 0.3], [0.5, 0.5, 0.4]))
    assert np.array_equal(np.array(c["pos"], f32), pos)
    dirv = look - pos
    np.testing.assert_allclose(c["fwd"], dirv / np.linalg.norm(dirv), rtol=0, atol=1e-6)
    assert f32(c["hperf"]) == f32(24e-3) / f32(0.035)
    assert f32(c["focus"]) == f32(math.sqrt(float(np.dot(focus - pos, focus - pos))))
    hperf0 = f32(24e-3) / f32(55e-3)
    assert f32(c["aperture"]) == (f32(24e-3) / hperf0) / f32(4.0)
    # environment: base colour and RGBE texels (run-length encoded file)
    base, w, h = d["env"]
    assert np.array_equal(np.array(base, f32), np.array([1.0, 0.9, 0.8], f32))
    assert (w, h) == (16, 8)
    assert np.array_equal(np.array(d["texel"], f32).reshape(8, 16, 3), _decode(px))
    # triangles: the quad keeps its first three corners; one vertex per face corner
    tris = d["tri"]
    assert len(tris) == 3 + 2
    P = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0.25], [0, 1, 0], [0.5, 0.5, 1.5]], f32)
    T = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0.25, 0.75, 0]], f32)
    N = np.array([[0, 0, 2], [0, 1, 1], [1, 0, 1]], f32)
    N = N / np.linalg.norm(N, axis=1, keepdims=True)
    faces = [[(0, 0, 0), (1, 1, 0), (2, 2, 1)], [(0, 0, 0), (2, 2, 1), (4, 3, 2)],
             [(1, 1, 1), (2, 2, 2), (4, 3, 2)]]
    for (m, smooth, v), face in zip(tris[:3], faces):
        assert smooth == 1
        for k, (pi, ti, ni) in enumerate(face):
            assert np.array_equal(v[k, 0], P[pi])
            assert np.array_equal(v[k, 2], T[ti])
            np.testing.assert_allclose(v[k, 1], N[ni], rtol=0, atol=1e-6)
    mats = d["material"]
    mixed = tris[0][0]
    assert mats[mixed][0] == 4 and np.isclose(mats[mixed][1][0], 0.3)
    m0, m1 = d["mixof"][mixed]
    assert mats[m0] == (0, [np.float32(0.7), np.float32(0.6), np.float32(0.5)])
    assert mats[m1][0] == 3 and np.allclose(mats[m1][1], [0.9, 0.8, 0.4, 0.3])
    for m, smooth, v in tris[3:]:  # positions-only mesh: default material, normal +Z
        assert mats[m] == (0, [1.0, 1.0, 1.0])
        assert np.array_equal(v[:, 1], np.tile(np.array([0, 0, 1], f32), (3, 1)))
        assert np.array_equal(v[:, 2], np.zeros((3, 3), f32))


def _aces(x):
    a, b, c, d, e = f32(2.51), f32(0.03), f32(2.43), f32(0.59), f32(0.14)
    return (x * (a * x + b)) / (x * (c * x + d) + e)


def _tonemap_u8(rgb):
    # dark values go negative before the power curves and become NaN, then 0, as in
    # the reference's float code
    with np.errstate(invalid="ignore"):
        return _tonemap_u8_raw(rgb)


def _tonemap_u8_raw(rgb):
    g = lambda v, p: np.power(v.astype(np.float64), np.float64(f32(p))).astype(f32)
    c = _aces(rgb.astype(f32))
    c = g(c, 1.2)
    x0, x1 = g(f32(0.05), 2.2), g(f32(0.9), 2.2)
    c = (c - x0) / (x1 - x0)
    c[..., 1] = g(c[..., 1], 1.3)
    c[..., 2] = g(c[..., 2], 1.6)
    v = np.power(c.astype(np.float64), 1.1).astype(f32)
    v = np.clip(v, f32(0), f32(1))
    v = np.power(v.astype(np.float64), np.float64(f32(1) / f32(2.2))).astype(f32)
    return ((f32(255) - f32(1e-3)) * v).astype(np.uint8)


def _read_png(path):
    data = open(path, "rb").read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    off, idat, W = 8, b"", None
    while off < len(data):
        n, = struct.unpack(">I", data[off:off + 4])
        typ, body = data[off + 4:off + 8], data[off + 8:off + 8 + n]
        crc, = struct.unpack(">I", data[off + 8 + n:off + 12 + n])
        assert zlib.crc32(typ + body) & 0xffffffff == crc
        if typ == b"IHDR":
            W, H, depth, ctype = struct.unpack(">IIBB", body[:10])
            assert (depth, ctype) == (8, 2)
        elif typ == b"IDAT":
            idat += body
        off += 12 + n
    raw = zlib.decompress(idat)
    rows = np.frombuffer(raw, np.uint8).reshape(H, 1 + W * 3)
    assert (rows[:, 0] == 0).all()
    return rows[:, 1:].reshape(H, W, 3)


def test_texture_save_png_and_hdr(exe, tmp_path):
    px = _rgbe_rows(9, 5, 11)  # width < 8 would force flat scanlines; 9 tests flat rows too
    src = tmp_path / "in.hdr"
    _write_hdr(src, px, rle=False)
    r = subprocess.run([exe, "save", str(src), str(tmp_path / "o.png"), str(tmp_path / "o.hdr")],
                       capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stderr
    img = _read_png(tmp_path / "o.png")
    expect = _tonemap_u8(_decode(px))
    assert img.shape == expect.shape
    assert np.abs(img.astype(int) - expect.astype(int)).max() <= 1
    # .hdr written back: same header form, values within RGBE precision
    data = open(tmp_path / "o.hdr", "rb").read()
    head, body = data.split(b"\n-Y 5 +X 9\n", 1)
    assert head.startswith(b"#?RADIANCE")
    back = _decode(np.frombuffer(body, np.uint8).reshape(5, 9, 4))
    orig = _decode(px)
    np.testing.assert_allclose(back, orig, rtol=1.0 / 128, atol=1e-30)


# ---- PNG reading (Texture2D::Load of a .png): an independent writer covering every
# colour type and bit depth, Adam7 interlacing, the five filters and the three kinds
# of DEFLATE block; the expected texels are stb_image's 3-channel result / 255.

_ADAM7 = [(0, 0, 8, 8), (4, 0, 8, 8), (0, 4, 4, 8), (2, 0, 4, 4), (0, 2, 2, 4), (1, 0, 2, 2), (0, 1, 1, 2)]


def _pack_row(samples, depth):
    """samples: (W*C,) ints -> packed big-endian bytes of one scanline."""
    if depth == 16:
        return samples.astype(">u2").tobytes()
    if depth == 8:
        return samples.astype(np.uint8).tobytes()
    per = 8 // depth
    out = bytearray((len(samples) + per - 1) // per)
    for i, v in enumerate(samples):
        out[i // per] |= int(v) << (8 - depth - (i % per) * depth)
    return bytes(out)


def _filter_row(row, prev, ftype, bpp):
    row = np.frombuffer(row, np.uint8).astype(np.int32)
    prev = np.zeros_like(row) if prev is None else np.frombuffer(prev, np.uint8).astype(np.int32)
    out = np.zeros_like(row)
    for x in range(len(row)):
        a = row[x - bpp] if x >= bpp else 0
        b = prev[x]
        c = prev[x - bpp] if x >= bpp else 0
        if ftype == 0:
            pred = 0
        elif ftype == 1:
            pred = a
        elif ftype == 2:
            pred = b
        elif ftype == 3:
            pred = (a + b) // 2
        else:
            p = a + b - c
            pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
            pred = a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)
        out[x] = (row[x] - pred) & 255
    return bytes([ftype]) + out.astype(np.uint8).tobytes()


def _write_png(path, img, ctype, depth, interlace=False, palette=None, zopts=(9, zlib.Z_DEFAULT_STRATEGY),
               first_filter=0):
    """img: (H, W, C) integer samples (palette: (H, W, 1) indices)."""
    H, W, C = img.shape
    bpp = max(1, C * depth // 8)
    passes = _ADAM7 if interlace else [(0, 0, 1, 1)]
    raw, k = b"", first_filter
    for x0, y0, dx, dy in passes:
        sub = img[y0::dy, x0::dx]
        if sub.size == 0:
            continue
        prev = None
        for y in range(sub.shape[0]):
            row = _pack_row(sub[y].reshape(-1), depth)
            raw += _filter_row(row, prev, k % 5, bpp)
            prev, k = row, k + 1
    level, strategy = zopts
    co = zlib.compressobj(level, zlib.DEFLATED, 15, 9, strategy)
    z = co.compress(raw) + co.flush()

    def chunk(t, b):
        return struct.pack(">I", len(b)) + t + b + struct.pack(">I", zlib.crc32(t + b) & 0xffffffff)
    data = b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", W, H, depth, ctype, 0, 0,
                                                                  1 if interlace else 0))
    if palette is not None:
        data += chunk(b"PLTE", palette.astype(np.uint8).tobytes())
    for i in range(0, len(z), 97):  # several IDAT chunks
        data += chunk(b"IDAT", z[i:i + 97])
    data += chunk(b"IEND", b"")
    open(path, "wb").write(data)


def _expected_rgb8(img, ctype, depth, palette=None):
    if ctype == 3:
        return palette[img[..., 0]].astype(np.uint8)
    v = img.astype(np.int64)
    if depth == 16:
        v = v >> 8
    elif depth < 8:
        v = v * (255 // ((1 << depth) - 1))
    if ctype in (0, 4):
        return np.repeat(v[..., :1], 3, axis=2).astype(np.uint8)
    return v[..., :3].astype(np.uint8)


PNG_FORMATS = [(0, 1), (0, 2), (0, 4), (0, 8), (0, 16), (2, 8), (2, 16), (3, 1), (3, 2), (3, 4),
               (3, 8), (4, 8), (4, 16), (6, 8), (6, 16)]


def _load_tex(exe, path, tmp_path, color):
    out = tmp_path / "tex.bin"
    r = subprocess.run([exe, "tex", str(path), str(out), "color" if color else "noncolor"],
                       capture_output=True, text=True, timeout=60)
    if r.returncode != 0:
        return None
    b = np.fromfile(out, np.uint8)
    W, H = b[:8].view(np.int32)
    return b[8:].view(np.float32).reshape(H, W, 3)


@pytest.mark.parametrize("ctype,depth", PNG_FORMATS)
@pytest.mark.parametrize("interlace", [False, True])
def test_png_texture_decoding(exe, tmp_path, ctype, depth, interlace):
    rng = np.random.default_rng(ctype * 100 + depth + 7 * interlace)
    C = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[ctype]
    H, W = 11, 13  # odd sizes: partial Adam7 passes and partial bytes at low depths
    palette = None
    if ctype == 3:
        n = 1 << depth
        palette = rng.integers(0, 256, size=(n, 3))
        img = rng.integers(0, n, size=(H, W, 1))
    else:
        img = rng.integers(0, 1 << depth, size=(H, W, C))
    for zopts, ff in [((9, zlib.Z_DEFAULT_STRATEGY), 0), ((0, zlib.Z_DEFAULT_STRATEGY), 1),
                      ((6, zlib.Z_FIXED), 2)]:  # dynamic, stored and fixed-code blocks
        path = tmp_path / "t.png"
        _write_png(path, img, ctype, depth, interlace, palette, zopts, ff)
        expect = _expected_rgb8(img, ctype, depth, palette).astype(np.float32) / np.float32(255)
        got = _load_tex(exe, path, tmp_path, color=False)
        assert got is not None
        assert np.array_equal(got, expect), (zopts, ff)
        # colour textures are linearised: powf(v, 2.2f)
        got_c = _load_tex(exe, path, tmp_path, color=True)
        want_c = np.power(expect, np.float32(2.2))
        assert np.abs(got_c.view(np.int32) - want_c.view(np.int32)).max() <= 1


def test_png_rejects_damaged_files(exe, tmp_path):
    rng = np.random.default_rng(3)
    img = rng.integers(0, 256, size=(6, 7, 3))
    path = tmp_path / "ok.png"
    _write_png(path, img, 2, 8)
    data = open(path, "rb").read()
    assert _load_tex(exe, path, tmp_path, False) is not None
    bad = tmp_path / "bad.png"
    for cut in (20, 45, len(data) - 20):  # truncated in the header, data and trailer
        open(bad, "wb").write(data[:cut])
        assert _load_tex(exe, bad, tmp_path, False) is None, cut
    open(bad, "wb").write(b"\x89PNG\r\n\x1a\n" + b"\0" * 40)
    assert _load_tex(exe, bad, tmp_path, False) is None


def _write_textured_case(root):
    """The JSON scene with texture maps: a Lambert colour map and a GGX colour map next
    to the scene file, and a GGX roughness map that the reference reads relative to the
    working directory (root), with the scene file in root/scene."""
    d = os.path.join(root, "scene")
    os.makedirs(d, exist_ok=True)
    px = _write_case(d)
    rng = np.random.default_rng(12)
    albedo = rng.integers(0, 256, size=(8, 8, 3))
    f0 = rng.integers(0, 256, size=(4, 6, 3))
    rough = rng.integers(0, 256, size=(5, 5, 1))
    _write_png(os.path.join(d, "albedo.png"), albedo, 2, 8)
    _write_png(os.path.join(d, "f0.png"), f0, 2, 8, interlace=True)
    _write_png(os.path.join(root, "rough.png"), rough, 0, 8)
    text = open(os.path.join(d, "scene.json")).read()
    text = text.replace('"base_color": [0.7, 0.6, 0.5]}', '"base_color": [0.7, 0.6, 0.5], "color_tex": "albedo.png"}')
    text = text.replace('"roughness": 0.3}', '"roughness": 0.3, "color_tex": "f0.png", "roughness_tex": "rough.png"}')
    open(os.path.join(d, "scene.json"), "w").write(text)
    u8 = lambda a, c: _expected_rgb8(a, c, 8).astype(np.float32) / np.float32(255)
    return px, {"albedo": u8(albedo, 2), "f0": u8(f0, 2), "rough": u8(rough, 0)}


def test_load_assets_attaches_texture_maps(exe, tmp_path):
    _, tex = _write_textured_case(str(tmp_path))
    out = tmp_path / "dump.txt"
    d = str(tmp_path / "scene")
    r = subprocess.run([exe, "dump", os.path.join(d, "settings.json"), os.path.join(d, "scene.json"), str(out)],
                       capture_output=True, text=True, timeout=60, cwd=str(tmp_path))
    assert r.returncode == 0, r.stderr
    rec = _parse_dump(out)
    maps = rec["maps"]
    by_slot = {slot: v for (m, slot), v in maps.items()}
    assert set(by_slot) == {0, 1, 2}
    pw = lambda a: np.power(a, np.float32(2.2))
    close = lambda a, b: np.abs(a.view(np.int32) - b.view(np.int32)).max() <= 1
    assert close(by_slot[0][0], pw(tex["albedo"]))   # Lambert colour map: linearised
    assert close(by_slot[1][0], pw(tex["f0"]))       # GGX colour map: linearised
    assert np.array_equal(by_slot[2][0], tex["rough"])  # roughness map: as stored
    assert by_slot[2][1] == 1.0
    # from another working directory the roughness map is not found (reference quirk)
    r = subprocess.run([exe, "dump", os.path.join(d, "settings.json"), os.path.join(d, "scene.json"), str(out)],
                       capture_output=True, text=True, timeout=60, cwd=d)
    assert r.returncode == 0
    assert {slot for (m, slot) in _parse_dump(out)["maps"]} == {0, 1}


def test_texture_sampling_by_uv(exe, tmp_path):
    """Texture2D::GetPixelByUV (Texture2D.cpp:273-335): wrapped uv, x = u * width with no
    half-texel shift, clamped edges; bilinear weights as the reference forms them."""
    rng = np.random.default_rng(21)
    W, H = 7, 5
    img = rng.random((H, W, 3), dtype=np.float32)
    path = tmp_path / "t.hdr"
    with open(path, "wb") as f:
        f.write(b"PTRAWF32" + struct.pack("<II", W, H) + img.tobytes())
    uvs = [(0.0, 0.0), (0.31, 0.77), (0.999, 0.5), (1.25, -0.4), (-2.6, 3.1), (0.5, 0.9999)]
    out = tmp_path / "s.txt"
    args = [str(x) for uv in uvs for x in uv]
    r = subprocess.run([exe, "sample", str(path), str(out), *args], capture_output=True, text=True,
                       timeout=60)
    assert r.returncode == 0, r.stderr
    got = np.array([[float.fromhex(t) for t in line.split()] for line in open(out)], np.float32)
    f32 = np.float32
    for (u, v), row in zip(uvs, got):
        u, v = f32(u), f32(v)
        u = u - f32(1) * np.floor(u / f32(1))
        v = v - f32(1) * np.floor(v / f32(1))
        x, y = u * f32(W), v * f32(H)
        ix0, ix1, iy0, iy1 = int(x), int(x + f32(1)), int(y), int(y + f32(1))
        wx0, wy0 = x - f32(ix0), y - f32(iy0)
        wx1, wy1 = f32(ix1) - x, f32(iy1) - y
        c = lambda i, j: img[min(max(j, 0), H - 1), min(max(i, 0), W - 1)]
        top = wx1 * c(ix0, iy0) + wx0 * c(ix1, iy0)
        bot = wx1 * c(ix0, iy1) + wx0 * c(ix1, iy1)
        want = wy1 * top + wy0 * bot
        assert np.array_equal(row[:3].view(np.uint32), want.astype(np.float32).view(np.uint32))
        assert np.array_equal(row[3:], img[int(y), int(x)])

@pytest.mark.gpu
@pytest.mark.parametrize("textured", [False, True])
def test_loaded_scene_renders_like_the_oracle(exe, tmp_path, textured):
    """LoadAssets + Petrichor::Render (replay) equals the oracle on the same scene arrays
    (with the texture maps LoadAssets attached, when the scene has them)."""
    import oracle
    from petrichor_gb300 import scene_io
    if textured:
        px, _ = _write_textured_case(str(tmp_path))
        d = str(tmp_path / "scene")
    else:
        px, d = _write_case(str(tmp_path)), str(tmp_path)
    settings, scene = os.path.join(d, "settings.json"), os.path.join(d, "scene.json")
    dump = tmp_path / "dump.txt"
    subprocess.run([exe, "dump", settings, scene, str(dump)], check=True, timeout=60, cwd=str(tmp_path))
    d = _parse_dump(dump)
    r = subprocess.run([exe, "render", settings, scene, str(tmp_path / "film.bin")],
                       capture_output=True, text=True, timeout=300, cwd=str(tmp_path))
    assert r.returncode == 0, r.stderr
    film = np.fromfile(tmp_path / "film.bin", np.float32).reshape(16, 24, 3)
    # the same scene as arrays
    ids = sorted(d["material"])
    textures, refs = [], {}
    for (m, slot), (tex, strength) in sorted(d.get("maps", {}).items()):
        refs[(m, slot)] = len(textures)
        textures.append(tex)
    mats = []
    for k in ids:
        kind, v = d["material"][k]
        if kind == 0:
            mats.append(scene_io.Material(scene_io.MAT_LAMBERT, color=tuple(v[:3]),
                                          albedo_tex=refs.get((k, 0), -1)))
        elif kind == 3:
            mats.append(scene_io.Material(scene_io.MAT_GLOSSY, color=tuple(v[:3]), roughness=v[3],
                                          f0_tex=refs.get((k, 1), -1),
                                          roughness_tex=refs.get((k, 2), -1)))
        else:
            a, b = d["mixof"][k]
            mats.append(scene_io.Material(scene_io.MAT_MIX, mix=v[0], mat0=a, mat1=b))
    assert len(textures) == (3 if textured else 0)
    V = np.concatenate([t[2] for t in d["tri"]])  # (3T, 3 attributes, 3)
    n = len(d["tri"])
    c = d["camera"]
    cam = scene_io.Camera(pos=tuple(c["pos"]), view_dir=tuple(np.array([0.5, 0.5, 0.3], f32) -
                                                                np.array(c["pos"], f32)),
                          fov=0.0, focal_length=0.035, focus_target=(0.5, 0.5, 0.4),
                          aperture=c["aperture"])
    env = scene_io.Environment(base_color=(1.0, 0.9, 0.8), texture=_decode(px))
    st = scene_io.Settings(width=24, height=16, spp=2, max_bounces=3, tile_width=8, tile_height=8,
                           integrator=scene_io.INTEGRATOR_SIMPLE)
    sc = scene_io.Scene(V[:, 0].copy(), V[:, 1].copy(), V[:, 2].copy(),
                        np.arange(3 * n, dtype=np.int32).reshape(n, 3),
                        np.array([t[0] for t in d["tri"]], np.int32), np.ones(n, np.uint8),
                        np.zeros(0, np.int32), mats, cam, env, st, textures)
    ref, _ = oracle.OracleScene(sc).render(threads=2)
    assert np.array_equal(film.view(np.uint32), ref.view(np.uint32))
