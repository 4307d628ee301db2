"""The Aurora-style C++ interface (include/aurora_gb300.hpp): a C++ client program builds a scene
through IScene (geometry callbacks, Standard Surface properties, instances with column-major
transforms, distant lights, environment properties and image) and renders it through IRenderer.
Its image must match the same scene rendered through the C ABI directly (the path every other
test checks against the oracle).  The camera's inverse view matrix is computed on both sides in
double precision by different routines and rounded to FP32, so the comparison allows a last-bit
difference there: relMSE below 1e-10."""
import os
import shutil
import struct
import subprocess
import tempfile

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def build_client():
    """Compiles tests/cpp/aurora_api_render.cpp against the built library; returns its path."""
    from aurora_gb300 import build
    lib = build.build()
    out_dir = os.path.join(ROOT, "aurora_gb300", "_build")
    exe = os.path.join(out_dir, "aurora_api_render")
    src = os.path.join(ROOT, "tests", "cpp", "aurora_api_render.cpp")
    if not os.path.exists(exe) or os.path.getmtime(exe) < max(os.path.getmtime(src), os.path.getmtime(lib)):
        gxx = shutil.which("g++") or "g++"
        subprocess.check_call([gxx, "-std=c++17", "-O2", "-I" + os.path.join(ROOT, "include"), src,
                               "-L" + out_dir, "-lagb_cuda", "-Wl,-rpath," + out_dir, "-o", exe + ".tmp"])
        os.replace(exe + ".tmp", exe)
    return exe


def test_cpp_client_builds_and_links():
    """CPU: the header compiles and the client links against libagb_cuda.so's exports."""
    assert os.access(build_client(), os.X_OK)


def materialx_document(mat, keys, name):
    """The material as a MaterialX standard_surface with one constant input per property (values
    printed with 9 significant digits, so each float reads back exactly)."""
    lines = ['<?xml version="1.0"?>', '<materialx version="1.38" colorspace="lin_rec709">',
             f'  <!-- {name}: constants only -->',
             f'  <standard_surface name="SR_{name}" type="surfaceshader">']
    for k in keys:
        v = mat[k]
        if k == "thin_walled":
            lines.append(f'    <input name="{k}" type="boolean" value="{"true" if int(v) else "false"}" />')
        elif np.ndim(v):
            lines.append(f'    <input name="{k}" type="color3" value="' +
                         ", ".join("%.9g" % np.float32(x) for x in v) + '" />')
        else:
            lines.append(f'    <input name="{k}" type="float" value="{"%.9g" % np.float32(v)}" />')
    lines += ['  </standard_surface>',
              f'  <surfacematerial name="M_{name}" type="material">',
              f'    <input name="surfaceshader" type="surfaceshader" nodename="SR_{name}" />',
              '  </surfacematerial>', '</materialx>']
    return "\n".join(lines)


def write_scene(path, s, view, proj, lights, depth, mtlx=False):
    from aurora_gb300 import _abi, scenes
    b = bytearray(b"AGBS")
    b += struct.pack("<5I", 1, s.width, s.height, s.spp, depth)
    b += np.asarray(view, np.float32).T.tobytes()   # column-major
    b += np.asarray(proj, np.float32).T.tobytes()
    b += struct.pack("<I", len(s.meshes))
    for m in s.meshes:
        b += struct.pack("<2I", len(m["positions"]), len(m["indices"]))
        b += np.asarray(m["positions"], np.float32).tobytes()
        for key in ("normals", "texcoords"):
            b += struct.pack("<B", 0 if m[key] is None else 1)
            if m[key] is not None:
                b += np.asarray(m[key], np.float32).tobytes()
        b += np.asarray(m["indices"], np.uint32).tobytes()
    b += struct.pack("<I", len(s.materials))
    for mi, mat in enumerate(s.materials):
        props = list(scenes._DEFAULTS.keys())
        if mtlx:
            doc = materialx_document(mat, props, f"m{mi}").encode()
            b += struct.pack("<II", 0xFFFFFFFF, len(doc)) + doc
            continue
        b += struct.pack("<I", len(props))
        for k in props:
            b += struct.pack("<B", len(k)) + k.encode()
            v = mat[k]
            if k == "thin_walled":
                b += struct.pack("<BB", 2, int(v))
            elif np.ndim(v):
                b += struct.pack("<B3f", 3, *[float(x) for x in v])
            else:
                b += struct.pack("<Bf", 1, float(v))
    b += struct.pack("<I", len(s.instances))
    for inst in s.instances:
        m4 = np.eye(4, dtype=np.float32)
        m4[:3, :] = np.asarray(inst["xform"], np.float32).reshape(3, 4)
        b += struct.pack("<2I", inst["mesh"], inst["material"]) + m4.T.tobytes()
    b += struct.pack("<I", len(lights))
    for d, c, i, a in lights:
        b += struct.pack("<8f", *d, *c, i, a)
    e = s.env
    b += np.concatenate([e["light_top"], e["light_bottom"], e["background_top"],
                         e["background_bottom"]]).astype(np.float32).tobytes()
    if s.env_light >= 0:
        im = s.images[s.env_light]
        b += struct.pack("<B2I", 1, im["width"], im["height"])
        b += np.asarray(im["pixels"], np.float32)[..., :3].tobytes()
    else:
        b += struct.pack("<B", 0)
    gp = getattr(s, "ground_plane", None)
    if gp is not None:
        b += struct.pack("<B", 1) + np.asarray(gp, _abi.GROUND_PLANE_DTYPE).reshape(1).tobytes()
    open(path, "wb").write(bytes(b))


@pytest.mark.gpu
@pytest.mark.parametrize("ground,mtlx", [(False, False), (True, False), (False, True)])
def test_cpp_interface_render_matches_c_abi(agb, oracle, ground, mtlx):
    """The same frame through the C++ interface and through the C ABI; with `ground`, the floor
    quad is replaced by a ground plane (IRenderer::createGroundPlanePointer,
    IScene::setGroundPlanePointer) with non-default values; with `mtlx`, every material reaches the
    interface as a MaterialX standard_surface document (setMaterialType(path, "MaterialX", doc))."""
    from aurora_gb300 import _abi, api, scenes
    exe = build_client()
    s = scenes.config_tiny(width=48, height=32, spp=8, lights=False)
    if ground:
        s.instances = s.instances[:4]   # the spheres (mesh 0); the floor quad is not referenced
        s.meshes = s.meshes[:1]
        s.ground_plane = _abi.ground_plane(position=(0.0, 0.05, 0.0), shadow_opacity=0.7,
                                           shadow_color=(0.1, 0.2, 0.3), reflection_opacity=0.4,
                                           reflection_color=(0.8, 0.6, 0.4),
                                           reflection_roughness=0.2)
    # Matrices as the client holds them (FP32); angular diameter 0 so cos(radius) = 1 exactly.
    view = np.asarray(scenes.look_at((0.4, 3.0, 7.0), (0.0, 0.8, 0.0)), np.float32)
    proj = np.asarray(scenes.perspective(45.0, s.width / s.height), np.float32)
    lights = [((0.3, -1.0, -0.2), (1.0, 0.95, 0.9), 2.0, 0.0)]
    depth = 4
    with tempfile.TemporaryDirectory() as tmp:
        scene_file, out_file = os.path.join(tmp, "scene.bin"), os.path.join(tmp, "out.bin")
        write_scene(scene_file, s, view, proj, lights, depth, mtlx=mtlx)
        subprocess.check_call([exe, scene_file, out_file])
        raw = open(out_file, "rb").read()
    w, h = struct.unpack("<2I", raw[:8])
    img = np.frombuffer(raw[8:], np.float32).reshape(h, w, 4)
    frame = scenes.frame_data(view.astype(np.float64), proj.astype(np.float64), trace_depth=depth,
                              lights=lights, scene_bounds=s.bounds())
    with api.Renderer() as r:
        r.upload(s)
        r.set_frame(frame)
        r.render(0, s.spp, accumulation=_abi.ACCUM_RUNNING_MEAN)
        ref, _ = r.post_process(mode=_abi.ACCUM_RUNNING_MEAN)
    err = oracle.rel_mse(img, ref)
    print(f"C++ interface vs C ABI: relMSE {err:.3g}, max abs {np.abs(img - ref).max():.3g}, "
          f"identical pixels {np.mean(np.all(img == ref, axis=2)):.4f}")
    assert err < 1e-10
    assert np.abs(img[..., :3]).max() > 0
