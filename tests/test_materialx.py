"""MaterialX documents with a standard_surface of constant inputs and image textures
(include/aurora_gb300_loaders.hpp, materialXToProperties) on the CPU: the properties they give,
what is refused with a warning, and the glTF AURORA_materials_materialX node extension that names
such a file."""
import json
import os
import tempfile

import numpy as np

from test_loaders import run

GOLD = """<?xml version="1.0"?>
<materialx version="1.38" colorspace="lin_rec709">
  <!-- a standard_surface reached through its surfacematerial -->
  <standard_surface name="SR_gold" type="surfaceshader">
    <input name="base" type="float" value="1" />
    <input name="base_color" type="color3" value="0.944, 0.776, 0.373" />
    <input name="metalness" type="float" value="1" />
    <input name="specular_roughness" type="float" value="0.25"/>
    <input name="thin_walled" type="boolean" value="true" />
    <input name="coat_color" type="color4" value="0.5,0.25,0.125,1" />
    <input name="specular_IOR" type="float" />
  </standard_surface>
  <standard_surface name="SR_unused" type="surfaceshader">
    <input name="base" type="float" value="0.1" />
  </standard_surface>
  <surfacematerial name="Gold" type="material">
    <input name="surfaceshader" type="surfaceshader" nodename="SR_gold" />
  </surfacematerial>
</materialx>
"""


def props(text, name="m.mtlx"):
    with tempfile.TemporaryDirectory() as tmp:
        path = os.path.join(tmp, name)
        open(path, "w").write(text)
        return run("mtlx", path)


def test_standard_surface_constants_become_properties():
    out = props(GOLD)
    assert out["ok"], out["warnings"]
    p = out["properties"]
    assert set(p) == {"base", "base_color", "metalness", "specular_roughness", "thin_walled", "coat_color"}
    assert p["base"] == 1.0 and p["metalness"] == 1.0 and p["thin_walled"] is True
    np.testing.assert_array_equal(np.float32(p["base_color"]), np.float32([0.944, 0.776, 0.373]))
    assert np.float32(p["specular_roughness"]) == np.float32(0.25)
    np.testing.assert_array_equal(np.float32(p["coat_color"]), np.float32([0.5, 0.25, 0.125]))


def test_bare_standard_surface_entities_and_single_quotes():
    doc = ("<materialx version='1.38'><standard_surface name='a&amp;b' type='surfaceshader'>"
           "<input name='emission' type='float' value='2.5'/>"
           "<input name='emission_color' type='vector3' value='1 0.5 0.25'/>"
           "</standard_surface></materialx>")
    out = props(doc)
    assert out["ok"], out["warnings"]
    assert out["properties"]["emission"] == 2.5
    assert out["properties"]["emission_color"] == [1.0, 0.5, 0.25]


def test_refusals_and_warnings():
    graph = GOLD.replace('<input name="metalness" type="float" value="1" />',
                         '<input name="metalness" type="float" nodename="noise1" />')
    out = props(graph)
    assert out["ok"] and "metalness" not in out["properties"]
    assert "node graph" in out["warnings"]
    other = ('<materialx version="1.38"><open_pbr_surface name="S" type="surfaceshader"/>'
             '<surfacematerial name="M" type="material"><input name="surfaceshader" '
             'type="surfaceshader" nodename="S"/></surfacematerial></materialx>')
    out = props(other)
    assert not out["ok"] and "open_pbr_surface" in out["warnings"]
    for bad, why in (("<materialx><standard_surface name='x'></materialx>", "mismatched end tag"),
                     ("<mtlx/>", "not <materialx>"),
                     ("<materialx/>", "no surface shader")):
        out = props(bad)
        assert not out["ok"] and why in out["warnings"], (bad, out["warnings"])
    out = props(GOLD.replace('type="color3" value="0.944, 0.776, 0.373"',
                             'type="color3" value="0.944, 0.776, 0.373" colorspace="srgb_texture"'))
    assert out["ok"] and "colour space srgb_texture" in out["warnings"]


def test_gltf_materialx_extension():
    from test_gltf import make_doc, write
    doc, blob, _ = make_doc()
    with tempfile.TemporaryDirectory() as tmp:
        open(os.path.join(tmp, "x.mtlx"), "w").write(GOLD)
        path = write(tmp, "glb", doc, blob)
        out = run("gltf", path)
        mtlx = os.path.join(tmp, "x.mtlx")
        assert out["ok"] and "MaterialX" not in out["warnings"]
        assert out["instances"][0]["material"] == "AURORA_mtlx:" + mtlx
        m = {x["path"]: x["properties"] for x in out["materials"]}["AURORA_mtlx:" + mtlx]
        assert m["metalness"] == 1.0 and m["thin_walled"] is True
        # without the file the node falls back to its glTF material, with a warning
        os.remove(mtlx)
        out = run("gltf", path)
        assert out["ok"] and "cannot read MaterialX file" in out["warnings"]
        assert out["instances"][0]["material"].endswith(":gltfMat:1")


def test_image_nodes_become_textures():
    """base_color through a node graph's tiledimage (sRGB file, tiling and offset), opacity
    straight from an image node; an image feeding metalness (no texture slot) is refused."""
    doc = """<?xml version="1.0"?>
<materialx version="1.38" colorspace="lin_rec709">
  <nodegraph name="NG">
    <tiledimage name="wood" type="color3">
      <input name="file" type="filename" value="textures/wood.png" colorspace="srgb_texture" />
      <input name="uvtiling" type="vector2" value="4, 2" />
      <input name="uvoffset" type="vector2" value="0.25, 0.5" />
    </tiledimage>
    <output name="out" type="color3" nodename="wood" />
  </nodegraph>
  <image name="mask" type="color3">
    <input name="file" type="filename" value="/abs/mask.png" />
  </image>
  <standard_surface name="S" type="surfaceshader">
    <input name="base_color" type="color3" nodegraph="NG" output="out" />
    <input name="opacity" type="color3" nodename="mask" />
    <input name="metalness" type="float" nodename="mask" />
    <input name="specular_roughness" type="float" value="0.5" />
  </standard_surface>
</materialx>
"""
    with tempfile.TemporaryDirectory() as tmp:
        path = os.path.join(tmp, "m.mtlx")
        open(path, "w").write(doc)
        out = run("mtlx", path)
    assert out["ok"], out["warnings"]
    wood = os.path.join(tmp, "textures/wood.png")
    p = out["properties"]
    assert p["base_color_image"] == f"MaterialXImage/{wood}:linearize:1"
    assert p["base_color_image_scale"] == [4.0, 2.0] and p["base_color_image_offset"] == [0.25, 0.5]
    assert p["opacity_image"] == "MaterialXImage//abs/mask.png:linearize:0"
    assert "metalness" not in p and "'metalness' is connected" in out["warnings"]
    assert p["specular_roughness"] == 0.5
    assert out["images"] == [
        {"property": "base_color_image", "image": p["base_color_image"], "file": wood, "linearize": True},
        {"property": "opacity_image", "image": p["opacity_image"], "file": "/abs/mask.png", "linearize": False}]


def test_obj_materials_from_materialx_files():
    """--loadMtlXForObj: an OBJ material with <name>.mtlx beside the OBJ file takes the document
    (OBJLoader.cpp:124-150); without the option, or without the file, the MTL record is used."""
    from test_loaders import write_scene
    with tempfile.TemporaryDirectory() as tmp:
        path = write_scene(tmp)
        open(os.path.join(tmp, "red.mtlx"), "w").write(GOLD)
        on = run("objmtlx", path)
        off = run("obj", path)
    red_on, glass_on = on["materials"]
    assert red_on["path"].endswith("-red:MaterialX-0") and red_on["properties"]["metalness"] == 1.0
    assert glass_on["path"].endswith("-glass:OBJFileMaterial-1")
    assert off["materials"][0]["path"].endswith("-red:OBJFileMaterial-0")
    assert on["instances"][0]["material"] == red_on["path"]


def test_node_graphs_compile_to_programs():
    """Inputs fed by node graphs become a per-hit program (the `materialx_graph` property): a
    custom node expanded from its nodedef's nodegraph, texture coordinates, object position,
    arithmetic; run by a numpy restatement of the operations, the program gives the graph's
    values."""
    import mtlx_graphs as mg
    from aurora_gb300 import _abi
    out = props(mg.CHECKER)
    assert out["ok"] and out["warnings"] == "", out["warnings"]
    p = out["properties"]
    assert np.float32(p["metalness"]) == np.float32(0.3)
    ops, consts, images = mg.decode(p["materialx_graph"])
    assert images == [] and len(ops) > 10
    rng = np.random.default_rng(3)
    P = 4096
    uv = rng.uniform(-2, 2, (P, 2)).astype(np.float32)
    pos = rng.uniform(-3, 3, (P, 3)).astype(np.float32)
    res = mg.evaluate(ops, consts, {_abi.GIN_TEXCOORD: uv, _abi.GIN_POSITION_OBJECT: pos})
    checker = np.mod(np.floor(uv[:, 0] * 8) + np.floor(uv[:, 1] * 6), 2).astype(np.float32)[:, None]
    fg, bg = np.float32([0.8, 0.2, 0.1]), np.float32([0.1, 0.3, 0.7])
    np.testing.assert_array_equal(res[_abi.GOUT_BASE_COLOR], bg + checker * (fg - bg))
    rough = np.clip(np.sin(pos[:, 0] * np.float32(3)), np.float32(0.15), np.float32(0.8))
    np.testing.assert_allclose(res[_abi.GOUT_SPECULAR_ROUGHNESS][:, 0], rough, atol=1e-6)


def test_node_graph_outputs_images_and_interfaces():
    """A node graph with its own interface input and five outputs: base_color (an image through
    scaled texture coordinates, tinted), emission_color (ifgreater on the luminance), normal (a
    normal map), coat_roughness (a switch over the world normal) and opacity (swizzle, power)."""
    import mtlx_graphs as mg
    from aurora_gb300 import _abi
    with tempfile.TemporaryDirectory() as tmp:
        path = os.path.join(tmp, "p.mtlx")
        open(path, "w").write(mg.PATTERNS)
        out = run("mtlx", path)
    assert out["ok"] and out["warnings"] == "", out["warnings"]
    ops, consts, images = mg.decode(out["properties"]["materialx_graph"])
    assert images == [f"MaterialXImage/{tmp}/pattern.png:linearize:0"]
    assert [im["property"] for im in out["images"]] == ["materialx_graph"]
    outs = set(ops["imm"][ops["op"] == _abi.GOP_OUTPUT])
    assert outs == {_abi.GOUT_BASE_COLOR, _abi.GOUT_EMISSION_COLOR, _abi.GOUT_NORMAL,
                    _abi.GOUT_COAT_ROUGHNESS, _abi.GOUT_OPACITY}
    rng = np.random.default_rng(4)
    P = 2048
    uv = rng.uniform(0, 1, (P, 2)).astype(np.float32)
    n = rng.normal(size=(P, 3)).astype(np.float32)
    n /= np.linalg.norm(n, axis=1, keepdims=True)
    t = np.cross(n, rng.normal(size=(P, 3))).astype(np.float32)
    t /= np.linalg.norm(t, axis=1, keepdims=True)
    img = rng.uniform(0, 1, (8, 8, 4)).astype(np.float32)
    res = mg.evaluate(ops, consts, {_abi.GIN_TEXCOORD: uv, _abi.GIN_NORMAL_WORLD: n, _abi.GIN_TANGENT_WORLD: t},
                      [img])
    x = np.floor(uv[:, 0] * 3 * 8).astype(int) % 8
    y = np.floor(uv[:, 1] * 3 * 8).astype(int) % 8
    tex = img[y, x, :3]
    np.testing.assert_allclose(res[_abi.GOUT_BASE_COLOR], tex * np.float32([0.9, 0.8, 0.6]), rtol=1e-6)
    lum = tex @ np.float32([0.2722287, 0.6740818, 0.0536895])
    glow = np.where((lum > 0.6)[:, None], np.float32([1.0, 0.5, 0.2]), 0)
    np.testing.assert_array_equal(res[_abi.GOUT_EMISSION_COLOR][np.abs(lum - 0.6) > 1e-5],
                                  glow[np.abs(lum - 0.6) > 1e-5])
    which = n[:, 1] + 1
    cr = np.where(which >= 2, 0.05, np.where(which >= 1, 0.3, 0.9)).astype(np.float32)
    np.testing.assert_array_equal(res[_abi.GOUT_COAT_ROUGHNESS][:, 0], cr)
    np.testing.assert_allclose(np.linalg.norm(res[_abi.GOUT_NORMAL], axis=1), 1, atol=1e-5)
    np.testing.assert_allclose(res[_abi.GOUT_OPACITY], tex[:, [1, 1, 2]] ** np.float32(0.25), rtol=1e-5)


def test_node_graph_refusals():
    """A node without an implementation leaves its input at the default, with a warning; the rest
    of the document still applies."""
    doc = """<materialx version="1.39">
  <worleynoise3d name="n" type="float" />
  <standard_surface name="S" type="surfaceshader">
    <input name="specular_roughness" type="float" nodename="n" />
    <input name="base_color" type="color3" nodename="missing" />
    <input name="metalness" type="float" value="0.5" />
  </standard_surface>
</materialx>"""
    out = props(doc)
    assert out["ok"]
    assert "materialx_graph" not in out["properties"] and out["properties"]["metalness"] == 0.5
    assert "node <worleynoise3d> is not supported" in out["warnings"]
    assert "node 'missing' not found" in out["warnings"]


def test_nested_custom_nodes_expand_per_instance():
    """A custom node whose implementation uses another custom node, instanced twice with
    different interface values: each expansion evaluates its own inner nodes (a node inside an
    implementation graph is a different value in each expansion chain)."""
    import mtlx_graphs as mg
    from aurora_gb300 import _abi
    doc = """<materialx version="1.39">
  <nodedef name="ND_scaleu" node="scaleu">
    <input name="k" type="float" value="1.0" />
    <output name="out" type="float" />
  </nodedef>
  <nodegraph name="NG_scaleu" nodedef="ND_scaleu">
    <texcoord name="uv" type="vector2" />
    <extract name="u" type="float">
      <input name="in" type="vector2" nodename="uv" />
      <input name="index" type="integer" value="0" />
    </extract>
    <multiply name="m" type="float">
      <input name="in1" type="float" nodename="u" />
      <input name="in2" type="float" interfacename="k" />
    </multiply>
    <output name="out" type="float" nodename="m" />
  </nodegraph>
  <nodedef name="ND_twice" node="twice">
    <input name="k" type="float" value="1.0" />
    <output name="out" type="float" />
  </nodedef>
  <nodegraph name="NG_twice" nodedef="ND_twice">
    <scaleu name="inner" type="float">
      <input name="k" type="float" interfacename="k" />
    </scaleu>
    <add name="sum" type="float">
      <input name="in1" type="float" nodename="inner" />
      <input name="in2" type="float" nodename="inner" />
    </add>
    <output name="out" type="float" nodename="sum" />
  </nodegraph>
  <twice name="a" type="float"><input name="k" type="float" value="2.0" /></twice>
  <twice name="b" type="float"><input name="k" type="float" value="5.0" /></twice>
  <combine3 name="c" type="color3">
    <input name="in1" type="float" nodename="a" />
    <input name="in2" type="float" nodename="b" />
    <input name="in3" type="float" value="0" />
  </combine3>
  <standard_surface name="S" type="surfaceshader">
    <input name="base_color" type="color3" nodename="c" />
  </standard_surface>
</materialx>"""
    out = props(doc)
    assert out["ok"] and out["warnings"] == "", out["warnings"]
    ops, consts, _ = mg.decode(out["properties"]["materialx_graph"])
    uv = np.float32([[0.25, 0.5], [0.5, 0.1], [-1.0, 0.0]])
    res = mg.evaluate(ops, consts, {_abi.GIN_TEXCOORD: uv})
    u = uv[:, 0]
    np.testing.assert_array_equal(res[_abi.GOUT_BASE_COLOR],
                                  np.stack([2 * (u * 2), 2 * (u * 5), 0 * u], axis=1))


def compound(kind, inputs, graph=""):
    body = "\n".join(f'    <input name="{n}" type="{t}" {v} />' for n, t, v in inputs)
    return f"""<materialx version="1.38">
  <adsk:{kind} name="S" type="surfaceshader">
{body}
  </adsk:{kind}>
  <surfacematerial name="M" type="material">
    <input name="surfaceshader" type="surfaceshader" nodename="S" />
  </surfacematerial>
{graph}
</materialx>"""


def test_adsk_compounds_map_to_standard_surface():
    """Autodesk's compound surface shaders (Prism materials): each mapped interface input drives
    its Standard Surface field (MaterialX/MaterialGenerator.cpp:90-114), the compound's fixed
    values are set, and inputs outside the map are not used."""
    def eq(value, want):
        return np.array_equal(np.float32(value), np.float32(want))
    out = props(compound("metal", [("metal_f0", "color3", 'value="0.9, 0.8, 0.7"'),
                                   ("surface_roughness", "float", 'value="0.3"'),
                                   ("surface_albedo", "color3", 'value="1, 0.5, 1"'),
                                   ("surface_anisotropy", "float", 'value="0.2"'),
                                   ("surface_rotation", "float", 'value="0.1"')]))
    assert out["ok"] and out["warnings"] == "", out["warnings"]
    p = out["properties"]
    assert eq(p["base_color"], [0.9, 0.8, 0.7]) and eq(p["metalness"], 1.0)
    assert eq(p["specular_roughness"], 0.3) and eq(p["coat_color"], [1.0, 0.5, 1.0])
    assert eq(p["specular_anisotropy"], 0.2) and eq(p["specular_rotation"], 0.1)

    p = props(compound("transparent", [("transparent_color", "color3", 'value="0.2, 0.4, 0.6"'),
                                       ("transparent_ior", "float", 'value="1.33"'),
                                       ("transparent_distance", "float", 'value="3"')]))["properties"]
    assert eq(p["transmission"], 1.0) and eq(p["transmission_color"], [0.2, 0.4, 0.6])
    assert eq(p["specular_IOR"], np.float32(1.33)) and "transparent_distance" not in p

    p = props(compound("glazing", [("glazing_transmission_color", "color3", 'value="0.5, 0.5, 0.5"'),
                                   ("glazing_f0", "color3", 'value="0.1, 0.1, 0.1"'),
                                   ("glazing_transmission_roughness", "float", 'value="0.05"'),
                                   ("glazing_backface_culling", "boolean", 'value="true"')]))["properties"]
    assert p["thin_walled"] is True and eq(p["transmission"], 1.0) and eq(p["transmission_color"], [0.5, 0.5, 0.5])
    assert eq(p["specular_color"], [0.1] * 3) and eq(p["specular_roughness"], 0.05)

    p = props(compound("layered", [("layered_diffuse", "color3", 'value="0.3, 0.2, 0.1"'),
                                   ("layered_fraction", "float", 'value="0.75"'),
                                   ("layered_bottom_f0", "color3", 'value="1, 1, 1"'),
                                   ("layered_roughness", "float", 'value="0.4"'),
                                   ("layered_f0", "float", 'value="0.04"')]))["properties"]
    assert eq(p["base_color"], [0.3, 0.2, 0.1]) and eq(p["coat"], 0.75)
    assert eq(p["specular_color"], [1.0, 1.0, 1.0]) and eq(p["specular_roughness"], 0.4)
    assert "layered_f0" not in p and "metalness" not in p

    # adsk:opaque: emission only with opaque_emission and a positive luminance; translucency
    # turns on subsurface.
    base = [("opaque_albedo", "color3", 'value="0.1, 0.2, 0.3"'),
            ("opaque_luminance_modifier", "color3", 'value="1, 0.9, 0.8"'),
            ("opaque_mfp_modifier", "color3", 'value="0.5, 0.25, 0.125"')]
    p = props(compound("opaque", base + [("opaque_emission", "boolean", 'value="true"'),
                                         ("opaque_luminance", "float", 'value="100"'),
                                         ("opaque_translucency", "boolean", 'value="true"')]))["properties"]
    assert eq(p["emission"], 1.0) and eq(p["subsurface"], 1.0)
    assert eq(p["emission_color"], [1.0, 0.9, 0.8])
    assert eq(p["subsurface_color"], [0.5, 0.25, 0.125]) and eq(p["base_color"], [0.1, 0.2, 0.3])
    p = props(compound("opaque", base + [("opaque_emission", "boolean", 'value="true"'),
                                         ("opaque_luminance", "float", 'value="0"'),
                                         ("opaque_translucency", "boolean", 'value="false"')]))["properties"]
    assert "emission" not in p and "subsurface" not in p

    out = props(compound("cloth", [("cloth_color", "color3", 'value="1, 1, 1"')]))
    assert not out["ok"] and "<adsk:cloth> is not supported" in out["warnings"]


def test_adsk_texture_nodes_compile_to_programs():
    """adsk:bitmap and adsk:normal_map in a compound's input graph: the file at texcoord x uv_scale
    + uv_offset, a bitmap's value x rgbamount (inverted on request), a normal map's xy scaled by
    normal_scale; a real-world scale other than 1 is reported as not applied."""
    import mtlx_graphs as mg
    from aurora_gb300 import _abi
    graph = """  <nodegraph name="G">
    <adsk:bitmap name="rough" type="float">
      <input name="file" type="filename" value="r.png" colorspace="lin_rec709" />
      <input name="uv_scale" type="vector2" value="2, 3" />
      <input name="uv_offset" type="vector2" value="0.25, 0.5" />
      <input name="rgbamount" type="float" value="0.5" />
      <input name="invert" type="boolean" value="true" />
    </adsk:bitmap>
    <adsk:bitmap name="albedo" type="color3">
      <input name="file" type="filename" value="a.png" colorspace="lin_rec709" />
      <input name="realworld_scale" type="vector2" value="24, 24" />
    </adsk:bitmap>
    <adsk:normal_map name="bump" type="vector3">
      <input name="file" type="filename" value="n.png" colorspace="lin_rec709" />
      <input name="normal_scale" type="float" value="0.5" />
    </adsk:normal_map>
    <output name="rough_out" type="float" nodename="rough" />
    <output name="albedo_out" type="color3" nodename="albedo" />
    <output name="bump_out" type="vector3" nodename="bump" />
  </nodegraph>"""
    doc = compound("opaque", [("surface_roughness", "float", 'nodegraph="G" output="rough_out"'),
                              ("opaque_albedo", "color3", 'nodegraph="G" output="albedo_out"'),
                              ("surface_normal", "vector3", 'nodegraph="G" output="bump_out"')], graph)
    out = props(doc)
    assert out["ok"]
    assert out["warnings"] == ("MaterialX <adsk:bitmap> 'albedo': realworld_scale / realworld_offset / "
                               "rotation_angle are not applied\n"), out["warnings"]
    ops, consts, images = mg.decode(out["properties"]["materialx_graph"])
    assert [i.split("/")[-1] for i in images] == ["r.png:linearize:0", "a.png:linearize:0", "n.png:linearize:0"]
    rng = np.random.default_rng(6)
    P = 1024
    uv = rng.uniform(0, 1, (P, 2)).astype(np.float32)
    n = np.tile(np.float32([0, 0, 1]), (P, 1))
    t = np.tile(np.float32([1, 0, 0]), (P, 1))
    imgs = [rng.uniform(0, 1, (8, 8, 4)).astype(np.float32) for _ in range(3)]
    res = mg.evaluate(ops, consts, {_abi.GIN_TEXCOORD: uv, _abi.GIN_NORMAL_WORLD: n,
                                    _abi.GIN_TANGENT_WORLD: t}, imgs)

    def texel(img, u):
        x = np.floor(u[:, 0] * 8).astype(int) % 8
        y = np.floor(u[:, 1] * 8).astype(int) % 8
        return img[y, x]
    uv2 = uv * np.float32([2, 3]) + np.float32([0.25, 0.5])
    np.testing.assert_allclose(res[_abi.GOUT_SPECULAR_ROUGHNESS][:, 0],
                               1 - texel(imgs[0], uv2)[:, 0] * np.float32(0.5), rtol=1e-6)
    np.testing.assert_array_equal(res[_abi.GOUT_BASE_COLOR], texel(imgs[1], uv)[:, :3])
    nm = texel(imgs[2], uv)[:, :3] * 2 - 1
    nm[:, :2] *= 0.5
    nm /= np.linalg.norm(nm, axis=1, keepdims=True)
    np.testing.assert_allclose(res[_abi.GOUT_NORMAL], nm, atol=1e-5)


def test_reference_prism_documents_load():
    """Every MaterialX document among the reference's own test assets whose surface shader is a
    standard_surface or an adsk compound loads (read from the reference tree where it is present:
    these are its files, not copies)."""
    import glob
    import pytest
    root = os.path.join(os.environ.get("AURORA_REFERENCE_ROOT", "/root/reference"), "Tests", "Assets", "Materials")
    files = sorted(glob.glob(os.path.join(root, "**", "*.mtlx"), recursive=True))
    if not files:
        pytest.skip("reference test assets not present")
    loaded, compounds = 0, 0
    for f in files:
        text = open(f, encoding="utf-8", errors="replace").read()
        out = run("mtlx", f)
        if "surfaceshader" not in text:
            assert not out["ok"]
            continue
        assert out["ok"], (f, out["warnings"])
        loaded += 1
        compounds += "<adsk:" in text and "standard_surface" not in text
    assert loaded >= 50 and compounds >= 30, (loaded, compounds)
    # The marble graph (a fractal3d whose octaves come from the graph's interface) compiles whole.
    import mtlx_graphs as mg
    from aurora_gb300 import _abi
    marble = os.path.join(root, "MarblegraphTest.mtlx")
    if os.path.exists(marble):
        out = run("mtlx", marble)
        assert out["ok"] and out["warnings"] == "", out["warnings"]
        ops, _, _ = mg.decode(out["properties"]["materialx_graph"])
        assert (ops["op"] == _abi.GOP_NOISE).sum() == 3


def test_noise_nodes_compile_to_programs():
    """noise2d, fractal3d and cellnoise3d compile to NOISE operations: the program gives the node
    formulas (noise x amplitude + pivot; amplitude x the octave sum; the cell's hash in [0, 1])
    over the numpy restatement of MaterialX's noise functions; the noise is 0 on the integer lattice
    and cell noise is constant inside a cell."""
    import mtlx_graphs as mg
    from aurora_gb300 import _abi
    out = props(mg.NOISE)
    assert out["ok"] and out["warnings"] == "", out["warnings"]
    ops, consts, _ = mg.decode(out["properties"]["materialx_graph"])
    assert (ops["op"] == _abi.GOP_NOISE).sum() == 5
    f = np.float32
    rng = np.random.default_rng(8)
    P = 4096
    uv = rng.uniform(-2, 2, (P, 2)).astype(f)
    pos = rng.uniform(-3, 3, (P, 3)).astype(f)
    res = mg.evaluate(ops, consts, {_abi.GIN_TEXCOORD: uv, _abi.GIN_POSITION_OBJECT: pos})
    grain = mg.perlin2(uv[:, 0] * f(8), uv[:, 1] * f(8)) * f(0.3) + f(0.45)
    np.testing.assert_array_equal(res[_abi.GOUT_SPECULAR_ROUGHNESS][:, 0], grain)
    p = pos * f(4)
    total, amp = np.zeros(P, f), f(1)
    for _ in range(3):
        total = total + amp * mg.perlin3(p[:, 0], p[:, 1], p[:, 2])
        amp = amp * f(0.45)
        p = p * f(2.1)
    t = (f(0.8) * total + f(0.5))[:, None]
    fg, bg = f([0.9, 0.85, 0.8]), f([0.15, 0.2, 0.3])
    np.testing.assert_array_equal(res[_abi.GOUT_BASE_COLOR], bg + t * (fg - bg))
    cells = mg.cell3(*(pos * f(4)).T)
    np.testing.assert_array_equal(res[_abi.GOUT_EMISSION_COLOR], f([0.6, 0.3, 0.1]) * cells[:, None])
    # Properties of the functions themselves.
    lattice = rng.integers(-50, 50, (512, 3)).astype(f)
    assert np.all(mg.perlin3(*lattice.T) == 0) and np.all(mg.perlin2(*lattice[:, :2].T) == 0)
    q = rng.uniform(-20, 20, (20000, 3)).astype(f)
    n3, n2 = mg.perlin3(*q.T), mg.perlin2(*q[:, :2].T)
    assert np.abs(n3).max() < 1.1 and np.abs(n2).max() < 1.1 and n3.std() > 0.1 and n2.std() > 0.1
    c = mg.cell3(*q.T)
    assert c.min() >= 0 and c.max() <= 1 and abs(c.mean() - 0.5) < 0.02
    inner = np.floor(q) + rng.uniform(0.01, 0.99, q.shape).astype(f)
    np.testing.assert_array_equal(mg.cell3(*inner.T), c)
    # colour-valued noise is refused with a warning
    bad = props(mg.NOISE.replace('<noise2d name="grain" type="float">', '<noise2d name="grain" type="color3">'))
    assert "type color3 is not supported" in bad["warnings"]


def test_compositing_nodes():
    """plus, minus and difference: mix x op(fg, bg) + (1 - mix) x bg."""
    import mtlx_graphs as mg
    from aurora_gb300 import _abi
    doc = """<materialx version="1.39">
  <texcoord name="uv" type="vector2" />
  <convert name="c" type="color3"><input name="in" type="vector2" nodename="uv" /></convert>
  <difference name="d" type="color3">
    <input name="fg" type="color3" nodename="c" />
    <input name="bg" type="color3" value="0.5, 0.25, 0.75" />
    <input name="mix" type="float" value="0.75" />
  </difference>
  <plus name="p" type="color3">
    <input name="fg" type="color3" nodename="d" />
    <input name="bg" type="color3" value="0.1, 0.2, 0.3" />
  </plus>
  <extract name="u" type="float"><input name="in" type="vector2" nodename="uv" /><input name="index" type="integer" value="0" /></extract>
  <minus name="m" type="float">
    <input name="fg" type="float" nodename="u" />
    <input name="bg" type="float" value="0.9" />
    <input name="mix" type="float" value="0.5" />
  </minus>
  <standard_surface name="S" type="surfaceshader">
    <input name="base_color" type="color3" nodename="p" />
    <input name="specular_roughness" type="float" nodename="m" />
  </standard_surface>
</materialx>"""
    out = props(doc)
    assert out["ok"] and out["warnings"] == "", out["warnings"]
    ops, consts, _ = mg.decode(out["properties"]["materialx_graph"])
    f = np.float32
    uv = np.random.default_rng(2).uniform(0, 1, (256, 2)).astype(f)
    res = mg.evaluate(ops, consts, {_abi.GIN_TEXCOORD: uv})
    c = np.concatenate([uv, np.zeros((256, 1), f)], 1)
    bg = f([0.5, 0.25, 0.75])
    d = f(0.75) * np.abs(bg - c) + (f(1) - f(0.75)) * bg
    p = f(1) * (f([0.1, 0.2, 0.3]) + d) + (f(1) - f(1)) * f([0.1, 0.2, 0.3])
    np.testing.assert_allclose(res[_abi.GOUT_BASE_COLOR], p, rtol=1e-6)
    m = f(0.5) * (f(0.9) - uv[:, 0]) + (f(1) - f(0.5)) * f(0.9)
    np.testing.assert_allclose(res[_abi.GOUT_SPECULAR_ROUGHNESS][:, 0], m, rtol=1e-6)


def test_oracle_noise_matches_numpy_restatement():
    """The oracle's MaterialX noise (C++, FP32) equals the numpy restatement bit for bit; its FP64
    form stays within 1e-5 of it: two independent writings of the same published functions (the
    device matches the FP32 oracle in the GPU render tests)."""
    import sys
    import mtlx_graphs as mg
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
    import pyoracle
    f = np.float32
    rng = np.random.default_rng(12)
    q = np.concatenate([rng.uniform(-40, 40, (20000, 3)), rng.integers(-9, 9, (500, 3)) + 0.5,
                        rng.integers(-9, 9, (500, 3))]).astype(f)
    want = [mg.perlin2(q[:, 0], q[:, 1]), mg.perlin3(q[:, 0], q[:, 1], q[:, 2]),
            mg.cell2(q[:, 0], q[:, 1]), mg.cell3(q[:, 0], q[:, 1], q[:, 2])]
    for kind in range(4):
        got = pyoracle.mx_noise(kind, q, precision=32).astype(f)
        np.testing.assert_array_equal(got, want[kind], err_msg=f"kind {kind}")
        got64 = pyoracle.mx_noise(kind, q, precision=64)
        assert np.abs(got64 - want[kind]).max() < 1e-5, kind


def test_smoothstep_crossproduct_rotate2d():
    """smoothstep (t^2 (3 - 2t) of the clamped ramp), crossproduct and rotate2d (degrees) compile
    to the operations that give MaterialX's formulas."""
    import mtlx_graphs as mg
    from aurora_gb300 import _abi
    doc = """<materialx version="1.39">
  <texcoord name="uv" type="vector2" />
  <rotate2d name="r" type="vector2">
    <input name="in" type="vector2" nodename="uv" />
    <input name="amount" type="float" value="30" />
  </rotate2d>
  <extract name="u" type="float"><input name="in" type="vector2" nodename="r" /><input name="index" type="integer" value="0" /></extract>
  <smoothstep name="s" type="float">
    <input name="in" type="float" nodename="u" />
    <input name="low" type="float" value="0.2" />
    <input name="high" type="float" value="0.7" />
  </smoothstep>
  <position name="p" type="vector3" />
  <crossproduct name="c" type="vector3">
    <input name="in1" type="vector3" nodename="p" />
    <input name="in2" type="vector3" value="0.3, -0.5, 0.8" />
  </crossproduct>
  <standard_surface name="S" type="surfaceshader">
    <input name="specular_roughness" type="float" nodename="s" />
    <input name="base_color" type="color3" nodename="c" />
  </standard_surface>
</materialx>"""
    out = props(doc)
    assert out["ok"] and out["warnings"] == "", out["warnings"]
    ops, consts, _ = mg.decode(out["properties"]["materialx_graph"])
    f = np.float32
    rng = np.random.default_rng(5)
    uv = rng.uniform(-1, 1, (512, 2)).astype(f)
    pos = rng.uniform(-2, 2, (512, 3)).astype(f)
    res = mg.evaluate(ops, consts, {_abi.GIN_TEXCOORD: uv, _abi.GIN_POSITION_OBJECT: pos})
    a = np.radians(30.0)
    u = np.cos(a) * uv[:, 0] + np.sin(a) * uv[:, 1]
    t = np.clip((u - 0.2) / 0.5, 0, 1)
    np.testing.assert_allclose(res[_abi.GOUT_SPECULAR_ROUGHNESS][:, 0], t * t * (3 - 2 * t), atol=2e-6)
    np.testing.assert_allclose(res[_abi.GOUT_BASE_COLOR], np.cross(pos, f([0.3, -0.5, 0.8])), atol=1e-6)
