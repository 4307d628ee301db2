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


def materialx_document(mat, keys, name, textures=()):
    """The material as a MaterialX standard_surface with one constant input per property (values
    printed with 9 significant digits, so each float reads back exactly); `textures`: (input,
    PNG file) pairs wired through a node graph's tiledimage with the material's texture scale and
    offset."""
    lines = ['<?xml version="1.0"?>', '<materialx version="1.38" colorspace="lin_rec709">',
             f'  <!-- {name} -->',
             f'  <standard_surface name="SR_{name}" type="surfaceshader">']
    wired = {inp for inp, _ in textures}
    for inp, _ in textures:
        lines.append(f'    <input name="{inp}" type="color3" nodegraph="NG_{name}" output="out_{inp}" />')
    for k in keys:
        if k in wired:
            continue
        v = mat[k]
        if k == "thin_walled":
            lines.append(f'    <input name="{k}" type="boolean" value="{"true" if int(v) else "false"}" />')
        elif np.ndim(v):
            lines.append(f'    <input name="{k}" type="color3" value="' +
                         ", ".join("%.9g" % np.float32(x) for x in v) + '" />')
        else:
            lines.append(f'    <input name="{k}" type="float" value="{"%.9g" % np.float32(v)}" />')
    lines.append('  </standard_surface>')
    if textures:
        lines.append(f'  <nodegraph name="NG_{name}">')
        for inp, file in textures:
            sc = ", ".join("%.9g" % np.float32(x) for x in mat[inp + "_image_scale"])
            of = ", ".join("%.9g" % np.float32(x) for x in mat[inp + "_image_offset"])
            lines += [f'    <tiledimage name="img_{inp}" type="color3">',
                      f'      <input name="file" type="filename" value="{file}" colorspace="lin_rec709" />',
                      f'      <input name="uvtiling" type="vector2" value="{sc}" />',
                      f'      <input name="uvoffset" type="vector2" value="{of}" />',
                      '    </tiledimage>',
                      f'    <output name="out_{inp}" type="color3" nodename="img_{inp}" />']
        lines.append('  </nodegraph>')
    lines += [f'  <surfacematerial name="M_{name}" type="material">',
              f'    <input name="surfaceshader" type="surfaceshader" nodename="SR_{name}" />',
              '  </surfacematerial>', '</materialx>']
    return "\n".join(lines)


TEX_NAMES = {0: "base_color_image", 1: "specular_roughness_image", 2: "opacity_image",
             3: "normal_image", 4: "emission_color_image"}


def write_scene(path, s, view, proj, lights, depth, mtlx=False, docs=None):
    """The scene file tests/cpp/aurora_api_render.cpp reads: version 2 when the scene has material
    textures or layers (images, texture properties, per-instance layer lists; each distinct
    layer UV set becomes one more mesh with the base mesh's geometry).  docs (with mtlx): a
    MaterialX document per material index to send instead of the one made from its values."""
    from aurora_gb300 import _abi, scenes
    layered = any(inst.get("layers") for inst in s.instances)
    textured = s.textures is not None and bool((np.asarray(s.textures["image"]) >= 0).any())
    version = 2 if (layered or textured) else 1
    meshes = [dict(m) for m in s.meshes]
    layer_mesh, inst_layers = {}, []
    for inst in s.instances:
        ls = []
        for mat, uv in inst.get("layers") or []:
            key = (inst["mesh"], np.ascontiguousarray(uv, np.float32).tobytes())
            if key not in layer_mesh:
                base = s.meshes[inst["mesh"]]
                layer_mesh[key] = len(meshes)
                meshes.append(dict(positions=base["positions"], normals=None,
                                   texcoords=np.ascontiguousarray(uv, np.float32), indices=base["indices"]))
            ls.append((mat, layer_mesh[key]))
        inst_layers.append(ls)
    b = bytearray(b"AGBS")
    b += struct.pack("<5I", version, s.width, s.height, s.spp, depth)
    b += np.asarray(view, np.float32).T.tobytes()   # column-major
    b += np.asarray(proj, np.float32).T.tobytes()
    b += struct.pack("<I", len(meshes))
    for m in meshes:
        b += struct.pack("<2I", len(m["positions"]), len(m["indices"]))
        b += np.asarray(m["positions"], np.float32).tobytes()
        for key in ("normals", "texcoords"):
            b += struct.pack("<B", 0 if m[key] is None else 1)
            if m[key] is not None:
                b += np.asarray(m[key], np.float32).tobytes()
        b += np.asarray(m["indices"], np.uint32).tobytes()
    if version >= 2:
        b += struct.pack("<I", len(s.images))
        for im in s.images:
            px = np.asarray(im["pixels"])
            if im["format"] != _abi.FORMAT_RGBA8:
                px = np.zeros((im["height"], im["width"], 4), np.uint8)   # textures only; unused here
            # linearize off: the C ABI samples the bytes as they are
            b += struct.pack("<2IB", im["width"], im["height"], 0) + np.ascontiguousarray(px, np.uint8).tobytes()
    b += struct.pack("<I", len(s.materials))
    for mi, mat in enumerate(s.materials):
        props = list(scenes._DEFAULTS.keys())
        if mtlx:
            tex = []
            if textured:
                from test_loaders import png_bytes
                for slot, name in TEX_NAMES.items():
                    img = int(s.textures["image"][mi, slot])
                    if img >= 0:
                        png = os.path.join(os.path.dirname(path), f"tex{img}.png")
                        if not os.path.exists(png):
                            open(png, "wb").write(png_bytes(np.asarray(s.images[img]["pixels"]), 6, 8, [0]))
                        tex.append((name[:-len("_image")], png))
            doc = (docs[mi] if docs and mi in docs else materialx_document(mat, props, f"m{mi}", tex)).encode()
            b += struct.pack("<II", 0xFFFFFFFF, len(doc)) + doc
            continue
        tex = []
        if textured:
            for slot, name in TEX_NAMES.items():
                img = int(s.textures["image"][mi, slot])
                if img >= 0:
                    tex.append((name, img))
        # a bilinear image gets a sampler of the material's own (the default sampler is nearest)
        linear = {img: bool(s.images[img]["linear"]) for _, img in tex}
        count = len(props) + sum(6 if linear[img] else 5 for _, img in tex)
        b += struct.pack("<I", count)
        for k in props:
            b += struct.pack("<B", len(k)) + k.encode()
            v = mat[k]
            if k == "thin_walled":
                b += struct.pack("<BB", 2, int(v))
            elif np.ndim(v):
                b += struct.pack("<B3f", 3, *[float(x) for x in v])
            else:
                b += struct.pack("<Bf", 1, float(v))
        for name, img in tex:
            ipath = f"/image/{img}".encode()
            b += struct.pack("<B", len(name)) + name.encode() + struct.pack("<BB", 4, len(ipath)) + ipath
            for suffix in ("_offset", "_scale", "_pivot"):
                k = name + suffix
                b += struct.pack("<B", len(k)) + k.encode() + struct.pack("<B2f", 5, *map(float, mat[k]))
            k = name + "_rotation"
            b += struct.pack("<B", len(k)) + k.encode() + struct.pack("<Bf", 1, float(mat[k]))
            if linear[img]:
                k, sp = name + "_sampler", b"/sampler/linear"
                b += struct.pack("<B", len(k)) + k.encode() + struct.pack("<BB", 4, len(sp)) + sp
    b += struct.pack("<I", len(s.instances))
    for inst, ls in zip(s.instances, inst_layers):
        m4 = np.eye(4, dtype=np.float32)
        m4[:3, :] = np.asarray(inst["xform"], np.float32).reshape(3, 4)
        b += struct.pack("<2I", inst["mesh"], inst["material"]) + m4.T.tobytes()
        if version >= 2:
            b += struct.pack("<I", len(ls))
            for mat, mesh in ls:
                b += struct.pack("<2I", mat, mesh)
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


@pytest.mark.gpu
@pytest.mark.parametrize("mtlx,late", [(False, False), (True, False), (False, True), (True, True)])
def test_cpp_interface_textures_and_layers_match_c_abi(agb, oracle, mtlx, late):
    """Material textures (image paths, a transformed base-colour texture), samplers and material
    layers (layer_materials / layer_geometry, the layer's UVs from a geometry of its own) through
    the C++ interface, against the same scene through the C ABI; with `mtlx`, the materials are
    MaterialX documents whose textures are PNG files behind node-graph tiledimages.  With `late`,
    the client renders once before it sets the materials, so their images (two PNG files, sampled
    bilinearly, in the MaterialX case) are uploaded after the environment image took the
    context's first image handle."""
    from aurora_gb300 import _abi, api, scenes
    exe = build_client()
    s = scenes.config_layered(width=64, height=48, spp=4, trace_depth=4, blas=2, instances=6,
                              tri_range=(200, 1000), decal_size=64)
    color_img = int(s.textures["image"][6, _abi.TEX_BASE_COLOR])
    s.materials["has_base_color_image"][0] = 1
    s.textures["image"][0, _abi.TEX_BASE_COLOR] = color_img
    s.materials["base_color_image_scale"][0] = (2.0, 0.5)
    s.materials["base_color_image_offset"][0] = (0.1, 0.2)
    if not mtlx:  # a tiledimage has no pivot or rotation
        s.materials["base_color_image_pivot"][0] = (0.5, 0.5)
        s.materials["base_color_image_rotation"][0] = 0.3
    view = np.asarray(scenes.look_at((0.0, 15.0, 60.0), (0.0, 0.0, 0.0)), np.float32)
    proj = np.asarray(scenes.perspective(45.0, s.width / s.height), np.float32)
    depth = 4
    with tempfile.TemporaryDirectory() as tmp:
        scene_file, out_file = os.path.join(tmp, "scene.bin"), os.path.join(tmp, "out.bin")
        write_scene(scene_file, s, view, proj, [], depth, mtlx=mtlx)
        subprocess.check_call([exe, scene_file, out_file] + (["--late-materials"] if late else []))
        raw = open(out_file, "rb").read()
    w, h = struct.unpack("<2I", raw[:8])
    img = np.frombuffer(raw[8:], np.float32).reshape(h, w, 4)
    frame = scenes.frame_data(view.astype(np.float64), proj.astype(np.float64), trace_depth=depth,
                              lights=[], scene_bounds=s.bounds())
    with api.Renderer() as r:
        r.upload(s)
        r.set_frame(frame)
        r.render(0, s.spp, accumulation=_abi.ACCUM_RUNNING_MEAN)
        ref, _ = r.post_process(mode=_abi.ACCUM_RUNNING_MEAN)
    # Without the textures and layers the image differs: they reach the renderer.
    bare = scenes.config_layered(width=64, height=48, spp=4, trace_depth=4, blas=2, instances=6,
                                 tri_range=(200, 1000), decal_size=64)
    for inst in bare.instances:
        inst["layers"] = []
    with api.Renderer() as r:
        r.upload(bare)
        r.set_frame(frame)
        r.render(0, s.spp, accumulation=_abi.ACCUM_RUNNING_MEAN)
        plain, _ = r.post_process(mode=_abi.ACCUM_RUNNING_MEAN)
    err = oracle.rel_mse(img, ref)
    changed = np.mean(np.any(plain != ref, axis=2))
    print(f"C++ interface (textures, layers) vs C ABI: relMSE {err:.3g}, identical pixels "
          f"{np.mean(np.all(img == ref, axis=2)):.4f}; pixels the layers and textures change {changed:.3f}")
    assert err < 1e-10
    assert changed > 0.01   # the six small spheres cover a few percent of the frame
