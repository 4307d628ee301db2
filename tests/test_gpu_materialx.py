"""MaterialX node graphs on the GPU: programs the C++ layer compiles from documents, run per hit
by the shading (and transparent-shadow) kernels, against the oracle's interpreter of the same
operations at equal samples; and the C++ interface rendering a node-graph document."""
import os
import tempfile

import numpy as np
import pytest

import mtlx_graphs as mg
from test_loaders import run

pytestmark = pytest.mark.gpu


def compile_doc(doc, name):
    with tempfile.TemporaryDirectory() as tmp:
        path = os.path.join(tmp, name)
        open(path, "w").write(doc)
        out = run("mtlx", path)
    assert out["ok"] and out["warnings"] == "", out["warnings"]
    return mg.decode(out["properties"]["materialx_graph"])


def graph_scene(width=48, height=32, spp=4, transparent_shadows=False):
    """The tiny scene with the checker program on the floor and the pattern program (an RGBA8
    image, a normal map, emission, coat roughness, opacity) on two spheres."""
    from aurora_gb300 import _abi, scenes
    s = scenes.config_tiny(width=width, height=height, spp=spp)
    rng = np.random.default_rng(9)
    tex = s.add_image(rng.integers(0, 256, (16, 16, 4)).astype(np.uint8), _abi.FORMAT_RGBA8)
    ck_ops, ck_k, _ = compile_doc(mg.CHECKER, "c.mtlx")
    pt_ops, pt_k, images = compile_doc(mg.PATTERNS, "p.mtlx")
    assert len(images) == 1
    mg.attach(s, {4: (ck_ops, ck_k, []), 0: (pt_ops, pt_k, [tex]), 2: (pt_ops, pt_k, [tex])})
    if transparent_shadows:
        s.frame["is_force_opaque_shadows_enabled"] = 0
    return s


@pytest.mark.parametrize("transparent_shadows", [False, True])
def test_node_graph_materials_match_oracle(agb, oracle, transparent_shadows):
    from aurora_gb300 import _abi, api, scenes
    s = graph_scene(transparent_shadows=transparent_shadows)
    with api.Renderer() as r:
        r.upload(s)
        r.render(0, 4)
        g = r.read(_abi.ACCUM_RUNNING_MEAN)
    o = oracle.OracleScene(s).render(0, 4)
    err = oracle.rel_mse(g, o["mean"])
    print("node-graph scene: relMSE vs FP32 oracle", err)
    assert err < 1e-6
    o64 = oracle.OracleScene(s).render(0, 4, precision=64)
    err64 = oracle.rel_mse(g, o64["mean"])
    print("node-graph scene: relMSE vs FP64 oracle", err64)
    # At 4 samples the FP64 paths part from the FP32 ones wherever a hit or a node's discrete
    # output (floor, modulo, ifgreater, switch) lands on the other side of an edge; with
    # transparent shadows a shadow ray then also crosses a different set of half-transparent
    # surfaces.  The FP32 oracle, which makes the same FP32 decisions, is the parity check above.
    assert err64 < (5e-2 if transparent_shadows else 1e-3)
    # The programs change the picture: the same scene without them differs.
    plain = scenes.config_tiny(width=48, height=32, spp=4)
    plain.images, plain.materials = s.images, s.materials
    if transparent_shadows:
        plain.frame["is_force_opaque_shadows_enabled"] = 0
    with api.Renderer() as r:
        r.upload(plain)
        r.render(0, 4)
        p = r.read(_abi.ACCUM_RUNNING_MEAN)
    assert oracle.rel_mse(g, p) > 1e-3


def test_graphs_are_checked_and_cleared(agb):
    """agb_material_graphs_set refuses out-of-range operands; new materials drop the programs."""
    from aurora_gb300 import _abi, api
    s = graph_scene(width=16, height=12, spp=1)
    with api.Renderer() as r:
        r.upload(s)
        lib = _abi.library()
        g = s.graphs
        ops = np.ascontiguousarray(g["ops"]).copy()
        first = np.ascontiguousarray(g["first"], np.int32)
        count = np.ascontiguousarray(g["count"], np.int32)
        k = np.ascontiguousarray(g["consts"], np.float32)
        bad = ops.copy()
        bad["dst"][0] = _abi.GRAPH_REGS
        st = lib.agb_material_graphs_set(r.ctx, first.ctypes.data, count.ctypes.data, len(first),
                                         bad.ctypes.data, len(bad), k.ctypes.data, len(k))
        assert st == _abi.ERR_INVALID_ARG
        assert b"invalid operation" in lib.agb_last_error()
        st = lib.agb_material_graphs_set(r.ctx, first.ctypes.data, count.ctypes.data, len(first) - 1,
                                         ops.ctypes.data, len(ops), k.ctypes.data, len(k))
        assert st == _abi.ERR_INVALID_ARG
        r.render(0, 1)
        with_graphs = r.read(_abi.ACCUM_RUNNING_MEAN)
        mats = np.ascontiguousarray(s.materials)
        assert lib.agb_materials_set(r.ctx, mats.ctypes.data, None, len(mats)) == 0
        r.render(0, 1)
        without = r.read(_abi.ACCUM_RUNNING_MEAN)
    assert np.abs(with_graphs - without).max() > 0


def test_cpp_interface_node_graph_document_matches_c_abi(agb, oracle):
    """The floor material as the checker document through IScene::setMaterialType(path,
    "MaterialX", document): the C++ layer compiles its node graphs and sets the programs; the
    frame equals the C ABI render of the same program (the camera inverse is computed by a
    different routine, hence the tolerance)."""
    import struct
    import subprocess
    from aurora_gb300 import _abi, api, scenes
    from test_aurora_api import build_client, write_scene
    exe = build_client()
    s = scenes.config_tiny(width=48, height=32, spp=8, lights=False)
    s.materials[4] = scenes.materials(1)[0]
    s.materials["metalness"][4] = 0.3
    ck_ops, ck_k, _ = compile_doc(mg.CHECKER, "c.mtlx")
    mg.attach(s, {4: (ck_ops, ck_k, [])})
    view = np.asarray(scenes.look_at((0.4, 3.0, 7.0), (0.0, 0.8, 0.0)), np.float32)
    proj = np.asarray(scenes.perspective(45.0, s.width / s.height), np.float32)
    lights = [((0.3, -1.0, -0.2), (1.0, 0.95, 0.9), 2.0, 0.0)]
    depth = 4
    with tempfile.TemporaryDirectory() as tmp:
        scene_file, out_file = os.path.join(tmp, "scene.bin"), os.path.join(tmp, "out.bin")
        write_scene(scene_file, s, view, proj, lights, depth, mtlx=True, docs={4: mg.CHECKER})
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
    print(f"C++ interface (node-graph document) vs C ABI: relMSE {err:.3g}")
    assert err < 1e-10
    # and the checker is there: the floor's pixels take both colours
    assert np.abs(img[..., :3]).max() > 0


def test_noise_node_materials_match_oracle(agb, oracle):
    """The noise program (fractal3d, noise2d, cellnoise3d) on the spheres and the floor: the
    device's NOISE operations against the oracle's restatement of MaterialX's noise, whole renders."""
    from aurora_gb300 import _abi, api, scenes
    s = scenes.config_tiny(width=48, height=32, spp=4)
    ops, k, _ = compile_doc(mg.NOISE, "n.mtlx")
    assert (ops["op"] == _abi.GOP_NOISE).sum() == 5
    mg.attach(s, {0: (ops, k, []), 2: (ops, k, []), 4: (ops, k, [])})
    with api.Renderer() as r:
        r.upload(s)
        r.render(0, 4)
        g = r.read(_abi.ACCUM_RUNNING_MEAN)
    o = oracle.OracleScene(s).render(0, 4)
    err = oracle.rel_mse(g, o["mean"])
    print("noise scene: relMSE vs FP32 oracle", err)
    assert err < 1e-6
    o64 = oracle.OracleScene(s).render(0, 4, precision=64)
    err64 = oracle.rel_mse(g, o64["mean"])
    print("noise scene: relMSE vs FP64 oracle", err64)
    # Cell noise and the lattice cells of the Perlin noise are discrete: a hit whose FP64 position
    # lands in the neighbouring cell takes another value there.
    assert err64 < 1e-2
    plain = scenes.config_tiny(width=48, height=32, spp=4)
    with api.Renderer() as r:
        r.upload(plain)
        r.render(0, 4)
        p = r.read(_abi.ACCUM_RUNNING_MEAN)
    assert oracle.rel_mse(g, p) > 1e-3
