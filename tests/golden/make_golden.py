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
"""
import ctypes
import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
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


if __name__ == "__main__":
    json.dump(material_layout(), open(os.path.join(HERE, "material_layout.json"), "w"), indent=1)
    json.dump(frame_layout(), open(os.path.join(HERE, "frame_layout.json"), "w"), indent=1)
    np.savez_compressed(os.path.join(HERE, "alias_ref.npz"), **alias_tables())
    print("golden fixtures written")
