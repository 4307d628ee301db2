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


@pytest.mark.parametrize("ground", [False, True])
def test_cli_render_matches_c_abi(agb, oracle, ground):
    """With `ground`, the floor quad gives way to the CLI's ground plane (--ground_shadow 1
    --ground_reflection 1: Plasma's plane at the scene's lower bound, shadow opacity 1,
    reflection opacity 0.5)."""
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
        enc = np.array([[rgbe(px) for px in row] for row in env], np.uint8)
        hdr = os.path.join(tmp, "env.hdr")
        open(hdr, "wb").write(b"#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n\n-Y 16 +X 32\n" + enc.tobytes())
        out = os.path.join(tmp, "out.pfm")
        res = subprocess.run([exe, obj, "--output", out, "--dims", "64,48", "--output_spp", "8",
                              "--eye", "0.4,3,7", "--target", "0,0.8,0", "--fov", "45", "--env", hdr,
                              "--lightDir", "0.3,-1,-0.2", "--lightIntensity", "2", "--trace-depth", "4"]
                             + (["--ground_shadow", "1", "--ground_reflection", "1"] if ground else []),
                             capture_output=True, text=True)
        assert res.returncode == 0, res.stderr
        mats = {k: np.array(re.search(rf"agb_render: {k}(( \S+){{16}})", res.stderr).group(1).split(),
                            np.float32).reshape(4, 4).T for k in ("view", "proj")}
        data = open(out, "rb").read()
        head = b"PF\n64 48\n-1.0\n"
        img = np.frombuffer(data[len(head):], "<f4").reshape(48, 64, 3)[::-1]
        scene = loader("obj", obj)
        env_f = np.reshape(loader("hdr", hdr)["rgb"], (16, 32, 3)).astype(np.float32)
    s = scenes.SceneDesc("cli")
    names = {m["path"]: k for k, m in enumerate(scene["materials"])}
    s.materials = scenes.materials(len(names))
    for m in scene["materials"]:
        for key, v in m["properties"].items():
            s.materials[key][names[m["path"]]] = v
    for inst in scene["instances"]:
        mesh = s.add_mesh(np.reshape(inst["positions"], (-1, 3)), np.reshape(inst["normals"], (-1, 3)),
                          np.reshape(inst["texcoords"], (-1, 2)), np.array(inst["indices"], np.uint32))
        s.instances.append(dict(mesh=mesh, material=names[inst["material"]],
                                xform=np.eye(4, dtype=np.float32)[:3].reshape(-1), layers=[]))
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
