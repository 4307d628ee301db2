"""The headless renderer (aurora_gb300/cli/agb_render.cpp, after Plasma's batch mode): an OBJ +
MTL scene with a Radiance HDR environment rendered by the CLI must match the same scene -- the
geometry and materials the loader produced, the environment the HDR reader decoded, the camera
the CLI reports -- rendered through the C ABI (the path the other parity tests check against the
oracle).  The light's cone (angular diameter 0.1, the interface's default) is computed with float
cos on the C++ side and in double here, so the comparison allows a last-bit difference there."""
import os
import re
import subprocess
import tempfile

import numpy as np
import pytest

from test_loaders import rgbe, run as loader

pytestmark = pytest.mark.gpu


def write_obj(path, meshes):
    """meshes: (name, material, positions, normals, texcoords, indices) -> OBJ + MTL next to it."""
    lines, base = ["mtllib scene.mtl"], [0, 0, 0]
    for name, mat, p, n, t, idx in meshes:
        lines.append(f"o {name}")
        lines += ["v %.9g %.9g %.9g" % tuple(v) for v in p]
        lines += ["vn %.9g %.9g %.9g" % tuple(v) for v in n]
        lines += ["vt %.9g %.9g" % tuple(v) for v in t]
        lines.append(f"usemtl {mat}")
        for tri in np.reshape(idx, (-1, 3)):
            lines.append("f " + " ".join("%d/%d/%d" % (base[0] + i + 1, base[2] + i + 1, base[1] + i + 1)
                                         for i in tri))
        base = [base[0] + len(p), base[1] + len(n), base[2] + len(t)]
    open(path, "w").write("\n".join(lines) + "\n")
    open(os.path.join(os.path.dirname(path), "scene.mtl"), "w").write(
        "newmtl blue\nKd 0.2 0.3 0.9\nKs 0.6 0.6 0.6\nPr 0.35\nNi 1.45\n"
        "newmtl floor\nKd 0.7 0.7 0.6\nPm 0.5\nPr 0.6\nd 0.8\n")


@pytest.mark.parametrize("ground,texture,mtlx", [(False, False, False), (True, False, False),
                                                 (False, True, False), (False, False, True)])
def test_cli_render_matches_c_abi(agb, oracle, ground, texture, mtlx):
    """With `ground`, the floor quad gives way to the CLI's ground plane (--ground_shadow 1
    --ground_reflection 1: Plasma's plane at the scene's lower bound, shadow opacity 1,
    reflection opacity 0.5).  With `texture`, the floor's MTL record names a PNG (map_Kd), which
    the C ABI side receives decoded from sRGB with the same formula.  With `mtlx`, --mtlx applies
    a MaterialX standard_surface to every instance (Plasma::applyMaterialXFile)."""
    from aurora_gb300 import _abi, api, build, scenes
    build.build()
    exe = build.CLI
    sp, sn, st, si = scenes.uv_sphere(24, 12, 1.0)
    sp = sp + np.float32([0, 1.0, 0])
    qp, qn, qt, qi = scenes.quad(4.0)
    env = scenes.hdr_env(32, 16, 5, sigma=1.0, suns=1, sun_radiance=200.0, sun_radius=1.5)[..., :3]
    with tempfile.TemporaryDirectory() as tmp:
        obj = os.path.join(tmp, "scene.obj")
        meshes = [("ball", "blue", sp, sn, st, si)]
        if not ground:
            meshes.append(("ground", "floor", qp, qn, qt, qi))
        write_obj(obj, meshes)
        if texture:
            from test_loaders import png_bytes
            tex_px = np.random.default_rng(9).integers(0, 256, (16, 24, 3))
            open(os.path.join(tmp, "floor.png"), "wb").write(png_bytes(tex_px, 2, 8, [0, 1, 4]))
            with open(os.path.join(tmp, "scene.mtl"), "a") as f:
                f.write("map_Kd floor.png\n")
        enc = np.array([[rgbe(px) for px in row] for row in env], np.uint8)
        hdr = os.path.join(tmp, "env.hdr")
        open(hdr, "wb").write(b"#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n\n-Y 16 +X 32\n" + enc.tobytes())
        out = os.path.join(tmp, "out.pfm")
        mtlx_file = os.path.join(tmp, "gold.mtlx")
        open(mtlx_file, "w").write(
            '<materialx version="1.38"><standard_surface name="S" type="surfaceshader">'
            '<input name="base_color" type="color3" value="0.944, 0.776, 0.373"/>'
            '<input name="metalness" type="float" value="1"/>'
            '<input name="specular_roughness" type="float" value="0.25"/>'
            '<input name="coat" type="float" value="0.5"/></standard_surface></materialx>')
        res = subprocess.run([exe, obj, "--output", out, "--dims", "64,48", "--output_spp", "8",
                              "--eye", "0.4,3,7", "--target", "0,0.8,0", "--fov", "45", "--env", hdr,
                              "--lightDir", "0.3,-1,-0.2", "--lightIntensity", "2", "--trace-depth", "4"]
                             + (["--ground_shadow", "1", "--ground_reflection", "1"] if ground else [])
                             + (["--mtlx", mtlx_file] if mtlx else []),
                             capture_output=True, text=True)
        assert res.returncode == 0, res.stderr
        mats = {k: np.array(re.search(rf"agb_render: {k}(( \S+){{16}})", res.stderr).group(1).split(),
                            np.float32).reshape(4, 4).T for k in ("view", "proj")}
        data = open(out, "rb").read()
        head = b"PF\n64 48\n-1.0\n"
        img = np.frombuffer(data[len(head):], "<f4").reshape(48, 64, 3)[::-1]
        scene = loader("obj", obj)
        env_f = np.reshape(loader("hdr", hdr)["rgb"], (16, 32, 3)).astype(np.float32)
        tex = loader("pngread", os.path.join(tmp, "floor.png")) if texture else None
    s = scenes.SceneDesc("cli")
    names = {m["path"]: k for k, m in enumerate(scene["materials"])}
    s.materials = scenes.materials(len(names))
    for m in scene["materials"]:
        for key, v in m["properties"].items():
            if not key.endswith("_image"):      # texture paths: bound below
                s.materials[key][names[m["path"]]] = v
    for inst in scene["instances"]:
        mesh = s.add_mesh(np.reshape(inst["positions"], (-1, 3)), np.reshape(inst["normals"], (-1, 3)),
                          np.reshape(inst["texcoords"], (-1, 2)), np.array(inst["indices"], np.uint32))
        s.instances.append(dict(mesh=mesh, material=names[inst["material"]],
                                xform=np.eye(4, dtype=np.float32)[:3].reshape(-1), layers=[]))
    if mtlx:
        gold = len(s.materials)
        s.materials = np.concatenate([s.materials, scenes.materials(1)])
        s.materials["base_color"][gold] = (0.944, 0.776, 0.373)
        s.materials["metalness"][gold] = 1.0
        s.materials["specular_roughness"][gold] = 0.25
        s.materials["coat"][gold] = 0.5
        for inst in s.instances:
            inst["material"] = gold
    if texture:
        # The C++ interface's decode of an sRGB 8-bit texture: v / 12.92 or ((v + 0.055) / 1.055)^2.4
        # in double precision, alpha / 255.
        rgba = np.float64(np.reshape(tex["rgba"], (tex["height"], tex["width"], 4))) / 255.0
        lin = np.where(rgba <= 0.04045, rgba / 12.92, ((rgba + 0.055) / 1.055) ** 2.4)
        lin[..., 3] = rgba[..., 3]
        # no sampler in an MTL file: the renderer's default sampler, nearest filtering
        tex_id = s.add_image(lin.astype(np.float32), _abi.FORMAT_RGBA32F, linear=False)
        s.textures = scenes.no_textures(len(names))
        floor = [m["path"] for m in scene["materials"] if m["properties"].get("base_color_image")][0]
        s.materials["has_base_color_image"][names[floor]] = 1
        s.textures["image"][names[floor], _abi.TEX_BASE_COLOR] = tex_id
    img_id = s.add_image(env_f, _abi.FORMAT_RGB32F)
    s.env_light = img_id
    s.env_background = img_id
    s.width, s.height, s.spp = 64, 48, 8
    d = np.float32([0.3, -1, -0.2])
    d = d / np.sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2])
    frame = scenes.frame_data(mats["view"].astype(np.float64), mats["proj"].astype(np.float64), trace_depth=4,
                              lights=[(tuple(d), (1.0, 1.0, 1.0), 2.0, 0.1)], scene_bounds=s.bounds())
    s.frame = frame
    if ground:
        s.ground_plane = _abi.ground_plane(position=scene["bounds"][0], shadow_opacity=1.0,
                                           reflection_opacity=0.5)
    with api.Renderer() as r:
        r.upload(s)
        r.render(0, 8, accumulation=_abi.ACCUM_RUNNING_MEAN)
        ref, _ = r.post_process(mode=_abi.ACCUM_RUNNING_MEAN)
    err = oracle.rel_mse(img, ref[..., :3])
    print(f"CLI vs C ABI: relMSE {err:.3g}, identical pixels {np.mean(np.all(img == ref[..., :3], axis=2)):.4f}")
    assert err < 1e-6
    assert img.max() > 0


def test_cli_gltf_camera_render_matches_c_abi(agb, oracle):
    """A .glb scene (a TRS-transformed sphere over a matrix-transformed floor, two
    pbrMetallicRoughness materials, a perspective camera node) rendered by the CLI from the file's
    camera (--camera 1) must match the loader's contents rendered through the C ABI."""
    from aurora_gb300 import _abi, api, build, scenes
    from test_gltf import Builder, sphere, write
    build.build()
    exe = build.CLI
    b = Builder()
    sp, sn, st, si = sphere(24, 12)
    qp, qn, qt, qi = [np.asarray(a) for a in scenes.quad(4.0)]
    prims = [
        {"attributes": {"POSITION": b.accessor(sp, "VEC3"), "NORMAL": b.accessor(sn, "VEC3"),
                        "TEXCOORD_0": b.accessor(st, "VEC2")},
         "indices": b.accessor(si.astype(np.uint32), "SCALAR", ctype=5125), "material": 0},
        {"attributes": {"POSITION": b.accessor(np.float32(qp), "VEC3"),
                        "NORMAL": b.accessor(np.float32(qn), "VEC3")},
         "indices": b.accessor(np.asarray(qi, np.uint16), "SCALAR", ctype=5123), "material": 1},
    ]
    doc = {
        "asset": {"version": "2.0"}, "scenes": [{"nodes": [0, 1, 2]}],
        "nodes": [
            {"mesh": 0, "translation": [0.2, 1.0, 0.1], "rotation": [0, 0.2588190, 0, 0.9659258],
             "scale": [1.0, 0.8, 1.0]},
            {"mesh": 1, "matrix": [1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, -0.05, 0, 1]},
            {"name": "view", "camera": 0, "translation": [0.5, 2.5, 6.5],
             "rotation": [-0.1736482, 0, 0, 0.9848078]},
        ],
        "meshes": [{"primitives": [prims[0]]}, {"primitives": [prims[1]]}],
        "materials": [
            {"pbrMetallicRoughness": {"baseColorFactor": [0.9, 0.3, 0.2, 1], "metallicFactor": 0.0,
                                      "roughnessFactor": 0.35}},
            {"pbrMetallicRoughness": {"baseColorFactor": [0.6, 0.6, 0.5, 1], "metallicFactor": 0.5,
                                      "roughnessFactor": 0.7}},
        ],
        "cameras": [{"type": "perspective",
                     "perspective": {"yfov": 0.8, "aspectRatio": 64 / 48, "znear": 0.1, "zfar": 200}}],
        "bufferViews": b.views, "accessors": b.accessors, "buffers": [{"byteLength": len(b.blob)}],
    }
    env = scenes.hdr_env(32, 16, 5, sigma=1.0, suns=1, sun_radiance=200.0, sun_radius=1.5)[..., :3]
    with tempfile.TemporaryDirectory() as tmp:
        glb = write(tmp, "glb", doc, bytes(b.blob))
        enc = np.array([[rgbe(px) for px in row] for row in env], np.uint8)
        hdr = os.path.join(tmp, "env.hdr")
        open(hdr, "wb").write(b"#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n\n-Y 16 +X 32\n" + enc.tobytes())
        out = os.path.join(tmp, "out.pfm")
        res = subprocess.run([exe, glb, "--output", out, "--dims", "64,48", "--output_spp", "8",
                              "--camera", "1", "--env", hdr, "--lightDir", "0.3,-1,-0.2",
                              "--lightIntensity", "2", "--trace-depth", "4"], capture_output=True, text=True)
        assert res.returncode == 0, res.stderr
        mats = {k: np.array(re.search(rf"agb_render: {k}(( \S+){{16}})", res.stderr).group(1).split(),
                            np.float32).reshape(4, 4).T for k in ("view", "proj")}
        data = open(out, "rb").read()
        head = b"PF\n64 48\n-1.0\n"
        img = np.frombuffer(data[len(head):], "<f4").reshape(48, 64, 3)[::-1]
        scene = loader("gltf", glb)
        env_f = np.reshape(loader("hdr", hdr)["rgb"], (16, 32, 3)).astype(np.float32)
    cam = np.float32(scene["cameras"][0]["view"]).reshape(4, 4).T
    np.testing.assert_array_equal(mats["view"], cam)
    s = scenes.SceneDesc("cli-gltf")
    names = {m["path"]: k for k, m in enumerate(scene["materials"])}
    s.materials = scenes.materials(len(names))
    for m in scene["materials"]:
        for key, v in m["properties"].items():
            if not key.endswith("_image"):      # texture paths: bound below
                s.materials[key][names[m["path"]]] = v
    for inst in scene["instances"]:
        tc = inst["texcoords"]
        mesh = s.add_mesh(np.reshape(inst["positions"], (-1, 3)), np.reshape(inst["normals"], (-1, 3)),
                          np.reshape(tc, (-1, 2)) if tc else None, np.array(inst["indices"], np.uint32))
        xf = np.float32(inst["transform"]).reshape(4, 4).T[:3].reshape(-1)
        s.instances.append(dict(mesh=mesh, material=names[inst["material"]], xform=xf, layers=[]))
    img_id = s.add_image(env_f, _abi.FORMAT_RGB32F)
    s.env_light = img_id
    s.env_background = img_id
    s.width, s.height, s.spp = 64, 48, 8
    d = np.float32([0.3, -1, -0.2])
    d = d / np.sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2])
    s.frame = scenes.frame_data(mats["view"].astype(np.float64), mats["proj"].astype(np.float64),
                                trace_depth=4, lights=[(tuple(d), (1.0, 1.0, 1.0), 2.0, 0.1)],
                                scene_bounds=s.bounds())
    with api.Renderer() as r:
        r.upload(s)
        r.render(0, 8, accumulation=_abi.ACCUM_RUNNING_MEAN)
        ref, _ = r.post_process(mode=_abi.ACCUM_RUNNING_MEAN)
    err = oracle.rel_mse(img, ref[..., :3])
    print(f"CLI (glTF, file camera) vs C ABI: relMSE {err:.3g}, "
          f"identical pixels {np.mean(np.all(img == ref[..., :3], axis=2)):.4f}")
    assert err < 1e-6
    assert img.max() > 0
