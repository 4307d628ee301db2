"""Generates the committed golden fixtures from the reference checkout (run where the reference
tree exists; the fixtures travel, the reference does not).

  material_layout.json  offsets/types of the 400-byte Standard Surface block, parsed from the
                        reference test fixture Tests/Assets/TextFiles/DefaultMaterialUniformBuffer.slang
                        (pinned by Tests/AuroraInternals/Common/TestUniformBuffer.cpp:42-83).
  frame_layout.json     field order and types of RendererBase::FrameData, SceneBase::LightData and
                        EnvironmentBase::EnvironmentData, parsed from the reference headers.
  alias_ref.npz         alias tables and luminance integrals from the reference's own
                        AliasMap::build (AliasMap.cpp:71-166), compiled in place by
                        oracle/build_oracle.py, on seeded environment images.
  shaders_ref.npz       outputs of the reference's own shader functions compiled as host C++
                        (oracle/build_oracle.py build_reference_shaders): Standard Surface
                        evaluateMaterial / sampleMaterial / evaluateMaterialAndPDF on 4096 seeded
                        cases (inputs stored) with the per-case tolerances of tests/bsdf_cases.py,
                        sampleEnvironment on a seeded 64x32 environment, and random2D streams.
  aurora_interface.txt  the binary interface of the reference's public header
                        Libraries/Aurora/API/Aurora/Aurora.h (tests/cpp/aurora_abi_probe.cpp's
                        vtable slots, value-type layouts and enumerator values, compiled against
                        it) and the Names values of Libraries/Aurora/Source/AuroraNames.cpp.
"""
import ctypes
import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "oracle"))
from build_oracle import REFERENCE_ROOT as REF  # noqa: E402


def material_layout():
    path = os.path.join(REF, "Tests/Assets/TextFiles/DefaultMaterialUniformBuffer.slang")
    fields = []
    for line in open(path):
        m = re.match(r"\s*(float|float2|float3|int)\s+(\w+);\s*//\s*Offset:(\d+)\s+Property:(\w+)", line)
        if m:
            fields.append(dict(type=m.group(1), member=m.group(2), offset=int(m.group(3)),
                               property=m.group(4)))
    size = 0
    for line in open(path):
        if re.match(r"\s*int\s+_padding9;", line):
            size = 400
    return dict(source="Tests/Assets/TextFiles/DefaultMaterialUniformBuffer.slang", size=size,
                fields=fields)


def struct_fields(path, name):
    text = open(path).read()
    start = text.index("struct " + name)
    body = text[text.index("{", start) + 1:]
    depth, end = 1, 0
    for i, ch in enumerate(body):
        depth += ch == "{"
        depth -= ch == "}"
        if depth == 0:
            end = i
            break
    body = re.sub(r"//.*", "", body[:end])
    out = []
    for m in re.finditer(r"^\s*([\w:]+)\s+(\w+)(\[[^\]]+\])?\s*(=[^;]*)?;", body, re.M):
        if m.group(1) in ("static_assert", "return"):
            continue
        out.append(dict(type=m.group(1), name=m.group(2), array=m.group(3) or ""))
    return out


def frame_layout():
    src = os.path.join(REF, "Libraries/Aurora/Source")
    return dict(
        frame=struct_fields(os.path.join(src, "RendererBase.h"), "FrameData"),
        lights=struct_fields(os.path.join(src, "SceneBase.h"), "LightData"),
        distant_light=struct_fields(os.path.join(src, "SceneBase.h"), "DistantLight"),
        environment=struct_fields(os.path.join(src, "EnvironmentBase.h"), "EnvironmentData"),
    )


def alias_tables():
    import build_oracle
    path = build_oracle.build_reference_alias()
    lib = ctypes.CDLL(path)
    out = {}
    rng = np.random.default_rng(20261203)
    cases = [("lognormal_64x32", np.exp(rng.normal(0, 2, (32, 64, 3)))),
             ("constant_16x8", np.ones((8, 16, 3))),
             ("sun_32x16", np.where(rng.uniform(size=(16, 32, 1)) > 0.97, 500.0, 0.2) *
              np.ones((1, 1, 3))),
             ("ragged_7x5", rng.uniform(0, 3, (5, 7, 3)))]
    for name, img in cases:
        img = np.ascontiguousarray(img, np.float32)
        h, w = img.shape[:2]
        table = np.zeros((w * h, 4), np.uint32)
        integral = ctypes.c_float()
        lib.ref_alias_build(img.ctypes.data_as(ctypes.c_void_p), w, h,
                            table.ctypes.data_as(ctypes.c_void_p), ctypes.byref(integral))
        out[name + "_image"] = img
        out[name + "_alias"] = table[:, 0].copy()
        out[name + "_prob"] = table[:, 1].view(np.float32).copy()
        out[name + "_pdf"] = table[:, 2].view(np.float32).copy()
        out[name + "_integral"] = np.float32(integral.value)
    return out


def shader_references(n=4096, seed=2024):
    import pyoracle
    from aurora_gb300 import scenes
    from bsdf_cases import make_cases, tolerances
    assert pyoracle.ref_lib() is not None, "the reference tree is needed"
    m, idx, frames, V, L, rnd = make_cases(n, seed)
    out = dict(materials=m.view(np.uint8).copy(), idx=idx, frames=frames, V=V, L=L, rnd=rnd)
    for op in (0, 1, 2):
        r32, r64, tol = tolerances(pyoracle.ref_bsdf_batch, op, m, idx, frames, V, L, rnd)
        for tag, r in (("ref32", r32), ("ref64", r64)):
            for k, name in enumerate(("value", "dir", "pdf", "lobe")):
                out[f"op{op}_{tag}_{name}"] = r[k]
        out[f"op{op}_tol"] = tol
    img = scenes.hdr_env(64, 32, 3, sigma=1.0, suns=1, sun_radiance=200.0, sun_radius=1.5)
    rgba = np.ones((32, 64, 4), np.float32)
    rgba[..., :3] = img
    alias, integral = pyoracle.alias_build(img)
    env = np.ascontiguousarray(scenes.environment()).reshape(1).copy()
    env["has_light_tex"] = 1
    env["light_tex_luminance_integral"] = integral
    env_rnd = np.random.default_rng(seed + 1).uniform(size=(n, 2)).astype(np.float32)
    er, ed, ep = pyoracle.ref_env_sample(env, rgba, alias, env_rnd)
    out.update(env_image=img, env_alias=alias.view(np.uint8).copy(), env_integral=np.float64(integral),
               env_data=env.view(np.uint8).copy(), env_rnd=env_rnd, env_radiance=er, env_dir=ed,
               env_pdf=ep)
    streams = []
    for sample, width, px, py in ((0, 512, 0, 0), (7, 512, 511, 3), (63, 1920, 1000, 540),
                                  (4095, 3840, 3839, 2159), (1 << 24, 64, 5, 9)):
        streams.append(pyoracle.ref_random_stream(sample, width, px, py, 16))
    out["random_args"] = np.array([(0, 512, 0, 0), (7, 512, 511, 3), (63, 1920, 1000, 540),
                                   (4095, 3840, 3839, 2159), (1 << 24, 64, 5, 9)], np.uint32)
    out["random_streams"] = np.stack(streams)
    return out


if __name__ == "__main__":
    json.dump(material_layout(), open(os.path.join(HERE, "material_layout.json"), "w"), indent=1)
    json.dump(frame_layout(), open(os.path.join(HERE, "frame_layout.json"), "w"), indent=1)
    np.savez_compressed(os.path.join(HERE, "alias_ref.npz"), **alias_tables())
    np.savez_compressed(os.path.join(HERE, "shaders_ref.npz"), **shader_references())
    import aurora_interface
    aurora_interface.write_fixture(REF)
    print("golden fixtures written")
