"""Scene and image I/O of the headless renderer (include/aurora_gb300_loaders.hpp), on the CPU:
the OBJ / MTL parse and the reference loader's translation (OBJLoader.cpp:155-449: Standard
Surface values from MTL records, unique vertices per shape, flipped V, normalised and generated
normals, one instance per shape with its first face's material), the Radiance HDR reader, the
PNG / PFM writers and the camera fit (Plasma/Camera.cpp:145-178), each against a numpy
restatement."""
import json
import os
import shutil
import struct
import subprocess
import tempfile
import zlib

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def tool():
    from aurora_gb300 import build
    lib = build.build()
    out_dir = os.path.join(ROOT, "aurora_gb300", "_build")
    exe = os.path.join(out_dir, "loader_tool")
    src = os.path.join(ROOT, "tests", "cpp", "loader_tool.cpp")
    hdr = os.path.join(ROOT, "include", "aurora_gb300_loaders.hpp")
    if not os.path.exists(exe) or os.path.getmtime(exe) < max(os.path.getmtime(src), os.path.getmtime(lib),
                                                               os.path.getmtime(hdr)):
        gxx = shutil.which("g++") or "g++"
        subprocess.check_call([gxx, "-std=c++17", "-O2", "-I" + os.path.join(ROOT, "include"), src,
                               "-L" + out_dir, "-lagb_cuda", "-Wl,-rpath," + out_dir, "-o", exe + ".tmp"])
        os.replace(exe + ".tmp", exe)
    return exe


def run(*args):
    return json.loads(subprocess.check_output([tool(), *map(str, args)]).decode())


def srgb_to_linear(c):
    c = np.float32(c)
    return c * (c * (c * np.float32(0.305306011) + np.float32(0.682171111)) + np.float32(0.012522878))


OBJ = """# two shapes
mtllib scene.mtl
v 0 0 0
v 1 0 0
v 1 1 0
v 0 1 0
vt 0 0
vt 1 0
vt 1 0.25
vt 0 1
vn 0 0 2
o quad
usemtl red
f 1/1/1 2/2/1 3/3/1 4/4/1
o tri
usemtl glass
f -4 -3 -1
f 1 3 4
"""

MTL = """newmtl red
Kd 0.8 0.1 0.1
Ks 0.5 0.5 0.5
Pr 0.3
Pm 0.2
Ke 0 0 0
newmtl glass
Kd 1 1 1
Ni 1.33
d 0.25
Tf 0 0 0
Ke 0.5 0.25 0
map_Kd texture.png
"""


def write_scene(tmp):
    path = os.path.join(tmp, "scene.obj")
    open(path, "w").write(OBJ)
    open(os.path.join(tmp, "scene.mtl"), "w").write(MTL)
    return path


def test_obj_translation_follows_reference_loader():
    with tempfile.TemporaryDirectory() as tmp:
        path = write_scene(tmp)
        r = run("obj", path)
    assert r["ok"] and r["triangles"] == 4 and len(r["instances"]) == 2
    red, glass = r["materials"]
    p = red["properties"]
    np.testing.assert_array_equal(np.float32(p["base_color"]), srgb_to_linear([0.8, 0.1, 0.1]))
    np.testing.assert_array_equal(np.float32(p["specular_color"]), srgb_to_linear([0.5] * 3))
    assert p["specular_IOR"] == 1.5 and p["transmission"] == 0.0   # Ni absent (1) -> 1.5; d 1
    assert np.float32(p["specular_roughness"]) == np.float32(0.3)
    assert np.float32(p["metalness"]) == np.float32(0.2)
    assert p["emission"] == 0.0 and p["transmission_color"] == [1.0, 1.0, 1.0]
    g = glass["properties"]
    assert np.float32(g["specular_IOR"]) == np.float32(1.33)
    assert np.float32(g["transmission"]) == np.float32(1.0) - np.float32(0.25)
    assert g["transmission_color"] == [1.0, 1.0, 1.0]                 # black Tf -> white
    assert g["emission"] == 1.0
    np.testing.assert_array_equal(np.float32(g["emission_color"]), srgb_to_linear([0.5, 0.25, 0.0]))
    # map_Kd: an sRGB image path (ImageCache::getImage), the file beside the OBJ file.
    assert g["base_color_image"] == "PlasmaImage/texture.png:linearize:1"
    assert p["base_color_image"] == "" and g["opacity_image"] == "" and g["normal_image"] == ""
    assert r["images"] == [{"path": "PlasmaImage/texture.png:linearize:1",
                            "file": os.path.join(os.path.dirname(path), "texture.png"), "linearize": True}]
    assert red["path"].endswith("-red:OBJFileMaterial-0") and glass["path"].endswith("-glass:OBJFileMaterial-1")

    quad, tri = r["instances"]
    assert quad["material"] == red["path"] and tri["material"] == glass["path"]
    # The quad: fan triangulation, 4 unique vertices, normals normalised, V flipped.
    assert quad["indices"] == [0, 1, 2, 0, 2, 3]
    np.testing.assert_array_equal(np.reshape(quad["positions"], (4, 3)),
                                  [[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0]])
    np.testing.assert_array_equal(np.reshape(quad["normals"], (4, 3)), [[0, 0, 1]] * 4)
    np.testing.assert_array_equal(np.reshape(quad["texcoords"], (4, 2)), [[0, 1], [1, 1], [1, 0.75], [0, 0]])
    # The triangles: relative indices, no normals (generated), no texcoords.
    assert tri["indices"] == [0, 1, 2, 0, 3, 2] and tri["texcoords"] == []
    pos = np.reshape(tri["positions"], (-1, 3)).astype(np.float32)
    np.testing.assert_array_equal(pos, [[0, 0, 0], [1, 0, 0], [0, 1, 0], [1, 1, 0]])
    np.testing.assert_allclose(np.reshape(tri["normals"], (-1, 3)), [[0, 0, 1]] * 4, atol=1e-6)
    np.testing.assert_array_equal(r["bounds"], [[0, 0, 0], [1, 1, 0]])


def angle_weighted_normals(pos, idx):
    """Restates Foundation/Source/Geometry.cpp:29-99 (weights as the reference computes them)."""
    n = np.zeros_like(pos, dtype=np.float64)
    unit = lambda v: v / np.linalg.norm(v)
    for a, b, c in idx.reshape(-1, 3):
        p1, p2, p3 = pos[a], pos[b], pos[c]
        fn = unit(np.cross(p2 - p1, p3 - p1))
        u13, u12, u23 = unit(p3 - p1), unit(p2 - p1), unit(p3 - p2)
        w = [np.arccos(np.dot(u13, u12)), np.arccos(np.dot(u23, u12)), np.arccos(np.dot(u13, u23))]
        for v, wv in zip((a, b, c), w):
            n[v] += fn * abs(wv)
    return n / np.linalg.norm(n, axis=1, keepdims=True)


def test_generated_normals_are_angle_weighted():
    from aurora_gb300 import scenes
    p, _, _, idx = scenes.icosphere(1, radius=1.0, displacement=0.1, seed=2)
    lines = ["v %.9g %.9g %.9g" % tuple(v) for v in p] + \
            ["f %d %d %d" % tuple(t + 1) for t in np.reshape(idx, (-1, 3))]
    with tempfile.TemporaryDirectory() as tmp:
        path = os.path.join(tmp, "ico.obj")
        open(path, "w").write("\n".join(lines) + "\n")
        r = run("obj", path)
    inst = r["instances"][0]
    pos = np.reshape(inst["positions"], (-1, 3)).astype(np.float64)
    got = np.reshape(inst["normals"], (-1, 3))
    want = angle_weighted_normals(pos, np.array(inst["indices"]))
    np.testing.assert_allclose(got, want, atol=2e-6)


def test_obj_parse_errors_and_degenerate_input():
    with tempfile.TemporaryDirectory() as tmp:
        bad = os.path.join(tmp, "bad.obj")
        open(bad, "w").write("v 0 0 0\nv 1 0 0\nf 1 2 9x\n")
        r = run("obj", bad)
        assert not r["ok"] and "bad face index" in r["warnings"]
        empty = os.path.join(tmp, "empty.obj")
        open(empty, "w").write("# nothing\nv 0 0 0\n")
        assert not run("obj", empty)["ok"]                 # no mesh
        assert not run("obj", os.path.join(tmp, "missing.obj"))["ok"]


def rgbe(rgb):
    """Greg Ward's float -> RGBE encoding."""
    m = float(max(rgb))
    if m < 1e-32:
        return [0, 0, 0, 0]
    mant, e = np.frexp(m)
    s = mant * 256.0 / m
    return [int(c * s) for c in rgb] + [e + 128]


def test_hdr_reader_flat_and_run_length():
    rng = np.random.default_rng(1)
    w, h = 40, 3
    img = rng.lognormal(0, 2, (h, w, 3)).astype(np.float32)
    img[1, 5:20] = img[1, 5]                               # a run for the RLE path
    enc = np.array([[rgbe(img[y, x]) for x in range(w)] for y in range(h)], np.uint8)
    want = np.where(enc[..., 3:] > 0, enc[..., :3] * np.ldexp(1.0, enc[..., 3:].astype(int) - 136), 0)
    head = b"#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n\n-Y %d +X %d\n" % (h, w)
    flat = head + enc.tobytes()
    rle = bytearray(head)
    for y in range(h):
        rle += bytes([2, 2, w >> 8, w & 255])
        for c in range(4):
            row, x = enc[y, :, c], 0
            while x < w:
                length = 1
                while x + length < w and length < 127 and row[x + length] == row[x]:
                    length += 1
                if length > 2:
                    rle += bytes([128 + length, row[x]])
                    x += length
                else:
                    n = min(w - x, 128, 2)
                    rle += bytes([n]) + bytes(row[x:x + n])
                    x += n
    with tempfile.TemporaryDirectory() as tmp:
        for name, data in (("flat.hdr", flat), ("rle.hdr", bytes(rle))):
            path = os.path.join(tmp, name)
            open(path, "wb").write(data)
            r = run("hdr", path)
            assert r["ok"] and (r["width"], r["height"]) == (w, h), r["error"]
            np.testing.assert_array_equal(np.reshape(r["rgb"], (h, w, 3)), want.astype(np.float32))
        path = os.path.join(tmp, "bad.hdr")
        open(path, "wb").write(b"P6\n")
        assert not run("hdr", path)["ok"]


def test_png_and_pfm_writers():
    w, h = 300, 257                                        # > 64 KB of scanlines: several stored blocks
    with tempfile.TemporaryDirectory() as tmp:
        png = os.path.join(tmp, "x.png")
        subprocess.check_call([tool(), "png", png, str(w), str(h)])
        data = open(png, "rb").read()
        assert data[:8] == b"\x89PNG\r\n\x1a\n"
        pos, chunks = 8, {}
        while pos < len(data):
            n, = struct.unpack(">I", data[pos:pos + 4])
            kind, body = data[pos + 4:pos + 8], data[pos + 8:pos + 8 + n]
            crc, = struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])
            assert crc == zlib.crc32(kind + body) & 0xffffffff
            chunks[kind] = chunks.get(kind, b"") + body
            pos += 12 + n
        assert struct.unpack(">IIBBBBB", chunks[b"IHDR"]) == (w, h, 8, 6, 0, 0, 0)
        raw = np.frombuffer(zlib.decompress(chunks[b"IDAT"]), np.uint8).reshape(h, 1 + 4 * w)
        assert (raw[:, 0] == 0).all()
        i = np.arange(w * h * 4, dtype=np.uint64)
        np.testing.assert_array_equal(raw[:, 1:].reshape(-1), ((i * 37 + i // 7) & 255).astype(np.uint8))
        pfm = os.path.join(tmp, "x.pfm")
        subprocess.check_call([tool(), "pfm", pfm, "5", "3"])
        data = open(pfm, "rb").read()
        head = b"PF\n5 3\n-1.0\n"
        assert data.startswith(head)
        px = np.frombuffer(data[len(head):], "<f4").reshape(3, 5, 3)[::-1]
        want = (np.arange(5 * 3 * 4, dtype=np.float32) * 0.25 - 3).reshape(3, 5, 4)[..., :3]
        np.testing.assert_array_equal(px, want)


def test_camera_fit():
    bmin, bmax, d = np.array([-1, -2, -3.0]), np.array([3, 1, 0.5]), np.array([0.3, -0.2, -1.0])
    fov, aspect = np.radians(45.0), 16 / 9
    r = run("fit", *bmin, *bmax, *d, fov, aspect)
    target = (bmin + bmax) / 2
    f = d / np.linalg.norm(d)
    s = np.cross(f, [0, 1, 0])
    s /= np.linalg.norm(s)
    u = np.cross(s, f)
    corners = np.array([[(bmax if c & m else bmin)[k] for k, m in enumerate((1, 2, 4))] for c in range(8)])
    v = corners @ np.stack([s, u, f]).T
    dims = v.max(0) - v.min(0)
    wide = dims[0] / dims[1] > aspect
    half = np.arctan(np.tan(fov / 2) * aspect) if wide else fov / 2
    dist = (dims[0] if wide else dims[1]) / (2 * np.tan(half)) + dims[2] / 2
    np.testing.assert_allclose(r["target"], target, rtol=1e-6)
    np.testing.assert_allclose(r["eye"], target - dist * f, rtol=1e-5)


def png_bytes(pixels, color, depth, filters, level=9, palette=None, trns=None):
    """A PNG of `pixels` (H x W x channels samples, unsigned) with the given filter type per row
    (the filters applied here as the encoder would), compressed by zlib at `level`."""
    h, w = pixels.shape[:2]
    ch = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[color]
    bpp_bits = ch * depth
    rows = []
    for y in range(h):
        if depth >= 8:
            row = pixels[y].reshape(-1).astype(">u2" if depth == 16 else np.uint8).tobytes()
        else:
            bits = "".join(format(int(v), f"0{depth}b") for v in pixels[y].reshape(-1))
            bits += "0" * (-len(bits) % 8)
            row = bytes(int(bits[i:i + 8], 2) for i in range(0, len(bits), 8))
        rows.append(np.frombuffer(row, np.uint8).astype(np.int32))
    bpp = max(1, bpp_bits // 8)
    out = bytearray()
    prev = np.zeros_like(rows[0])
    for y, cur in enumerate(rows):
        f = filters[y % len(filters)]
        a = np.concatenate([np.zeros(bpp, np.int32), cur[:-bpp]])
        c = np.concatenate([np.zeros(bpp, np.int32), prev[:-bpp]])
        b = prev
        if f == 0:
            enc = cur
        elif f == 1:
            enc = cur - a
        elif f == 2:
            enc = cur - b
        elif f == 3:
            enc = cur - (a + b) // 2
        else:
            p = a + b - c
            pa, pb, pc = np.abs(p - a), np.abs(p - b), np.abs(p - c)
            pred = np.where((pa <= pb) & (pa <= pc), a, np.where(pb <= pc, b, c))
            enc = cur - pred
        out += bytes([f]) + (enc % 256).astype(np.uint8).tobytes()
        prev = cur

    def chunk(t, body):
        return struct.pack(">I", len(body)) + t + body + struct.pack(">I", zlib.crc32(t + body) & 0xffffffff)

    png = b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, depth, color, 0, 0, 0))
    if palette is not None:
        png += chunk(b"PLTE", bytes(palette))
    if trns is not None:
        png += chunk(b"tRNS", bytes(trns))
    data = zlib.compress(bytes(out), level)
    return png + chunk(b"IDAT", data[:len(data) // 2]) + chunk(b"IDAT", data[len(data) // 2:]) + chunk(b"IEND", b"")


def test_png_decoder_matches_restatement():
    """Every colour type and bit depth the decoder takes, all five filters, stored / fixed /
    dynamic DEFLATE blocks (zlib levels 0, 1, 9) and a split IDAT, against the expected RGBA."""
    rng = np.random.default_rng(5)
    cases = []
    for color, depth in ((0, 1), (0, 2), (0, 4), (0, 8), (0, 16), (2, 8), (2, 16), (3, 1), (3, 4), (3, 8),
                         (4, 8), (4, 16), (6, 8), (6, 16)):
        h, w = 7, 13
        ch = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[color]
        hi = (1 << depth) - 1
        px = rng.integers(0, hi + 1, (h, w, ch))
        palette = trns = None
        if color == 3:
            n = hi + 1
            palette = rng.integers(0, 256, 3 * n).tolist()
            trns = rng.integers(0, 256, n // 2).tolist()
        cases.append((color, depth, px, palette, trns))
    with tempfile.TemporaryDirectory() as tmp:
        for k, (color, depth, px, palette, trns) in enumerate(cases):
            for level in (0, 1, 9):
                path = os.path.join(tmp, f"t{k}_{level}.png")
                open(path, "wb").write(png_bytes(px, color, depth, [0, 1, 2, 3, 4], level, palette, trns))
                r = run("pngread", path)
                assert r["ok"], (color, depth, r["error"])
                got = np.uint8(r["rgba"]).reshape(px.shape[0], px.shape[1], 4)
                if color == 3:
                    pal = np.uint8(palette).reshape(-1, 3)
                    alpha = np.full(len(pal), 255, np.uint8)
                    alpha[:len(trns)] = trns
                    want = np.concatenate([pal[px[..., 0]], alpha[px[..., 0]][..., None]], axis=2)
                else:
                    # samples to 8 bits: 16-bit keeps the high byte, low-depth grey is scaled
                    s8 = px >> 8 if depth == 16 else (px * 255 // ((1 << depth) - 1) if depth < 8 else px)
                    opaque = np.full(px.shape[:2] + (1,), 255)
                    if color in (0, 4):
                        alpha = s8[..., 1:2] if color == 4 else opaque
                        want = np.concatenate([s8[..., :1]] * 3 + [alpha], axis=2)
                    else:
                        alpha = s8[..., 3:4] if color == 6 else opaque
                        want = np.concatenate([s8[..., :3], alpha], axis=2)
                np.testing.assert_array_equal(got, np.uint8(want), err_msg=f"color {color} depth {depth} level {level}")
        bad = os.path.join(tmp, "bad.png")
        data = png_bytes(cases[5][2], 2, 8, [0])
        open(bad, "wb").write(data[:60])
        assert not run("pngread", bad)["ok"]
        open(bad, "wb").write(b"GIF89a")
        assert "not a PNG" in run("pngread", bad)["error"]
