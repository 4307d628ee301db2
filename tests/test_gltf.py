"""glTF 2.0 loading (include/aurora_gb300_loaders.hpp, after Applications/Plasma/glTFLoader.cpp) on
the CPU: synthetic files written here in the three container forms (embedded base64 buffer,
external .bin, binary .glb) must give the same scene contents, and those contents must match a
numpy restatement of the reference loader: node transforms (matrix or TRS, accumulated from the
parents in glm's product order), one geometry + instance per TRIANGLES primitive, FLOAT
attributes through strided buffer views, 8/16/32-bit or generated indices, generated normals,
pbrMetallicRoughness materials with the glTF defaults, camera nodes, scene bounds."""
import base64
import json
import os
import struct
import tempfile

import numpy as np

from test_loaders import run


def quat_matrix(q):
    x, y, z, w = [np.float32(v) for v in q]
    two, one = np.float32(2), np.float32(1)
    xx, yy, zz, xz, xy, yz = x * x, y * y, z * z, x * z, x * y, y * z
    wx, wy, wz = w * x, w * y, w * z
    cols = [[one - two * (yy + zz), two * (xy + wz), two * (xz - wy)],
            [two * (xy - wz), one - two * (xx + zz), two * (yz + wx)],
            [two * (xz + wy), two * (yz - wx), one - two * (xx + yy)]]
    return np.array(cols, np.float32)          # cols[c][row]


def node_matrix(node):
    """Column-major flat 16 (float32), as getNodeTransform builds it."""
    if "matrix" in node:
        return np.array(node["matrix"], np.float32)
    t = np.float32(node.get("translation", [0, 0, 0]))
    s = np.float32(node.get("scale", [1, 1, 1]))
    R = quat_matrix(node.get("rotation", [0, 0, 0, 1]))
    m = np.zeros(16, np.float32)
    for c in range(3):
        for r in range(3):
            m[c * 4 + r] = R[c][r] * s[c]
    m[12:15] = t
    m[15] = 1
    return m


def mul(A, B):
    """glm's column-major product, summed in its order."""
    r = np.zeros(16, np.float32)
    for c in range(4):
        for row in range(4):
            acc = A[0 * 4 + row] * B[c * 4 + 0]
            acc = np.float32(acc + A[1 * 4 + row] * B[c * 4 + 1])
            acc = np.float32(acc + A[2 * 4 + row] * B[c * 4 + 2])
            r[c * 4 + row] = np.float32(acc + A[3 * 4 + row] * B[c * 4 + 3])
    return r


def transform_points(m, p):
    out = np.empty_like(p)
    for r in range(3):
        acc = m[0 * 4 + r] * p[:, 0]
        acc = (acc + m[1 * 4 + r] * p[:, 1]).astype(np.float32)
        acc = (acc + m[2 * 4 + r] * p[:, 2]).astype(np.float32)
        out[:, r] = (acc + m[3 * 4 + r]).astype(np.float32)
    return out


class Builder:
    """Accumulates one binary buffer, buffer views and accessors."""

    def __init__(self):
        self.blob = bytearray()
        self.views, self.accessors = [], []

    def _view(self, data, stride=None):
        while len(self.blob) % 4:
            self.blob += b"\0"
        v = {"buffer": 0, "byteOffset": len(self.blob), "byteLength": len(data)}
        if stride:
            v["byteStride"] = stride
        self.blob += data
        self.views.append(v)
        return len(self.views) - 1

    def accessor(self, arr, type_, ctype=5126, view=None, offset=0, count=None):
        if view is None:
            view = self._view(np.ascontiguousarray(arr).tobytes())
        a = {"bufferView": view, "componentType": ctype, "count": int(count or len(arr)), "type": type_}
        if offset:
            a["byteOffset"] = offset
        self.accessors.append(a)
        return len(self.accessors) - 1

    def interleaved(self, pos, nrm):
        """POSITION and NORMAL accessors over one view with byteStride 24."""
        data = np.concatenate([pos, nrm], axis=1).astype(np.float32)
        v = self._view(data.tobytes(), stride=24)
        return (self.accessor(None, "VEC3", view=v, count=len(pos)),
                self.accessor(None, "VEC3", view=v, offset=12, count=len(pos)))


def sphere(n=6, m=4):
    from aurora_gb300 import scenes
    p, nr, t, i = scenes.uv_sphere(n, m, 1.0)
    return (np.asarray(p, np.float32), np.asarray(nr, np.float32), np.asarray(t, np.float32),
            np.asarray(i, np.uint32))


def make_doc():
    """A scene exercising each loader path; returns (doc, blob, expected primitives)."""
    b = Builder()
    sp, sn, st, si = sphere()
    quad_p = np.float32([[0, 0, 0], [1, 0, 0], [1, 0, 1], [0, 0, 1]])
    quad_i = np.uint8([0, 2, 1, 0, 3, 2])
    tri_p = np.float32([[0, 0, 0], [0, 1, 0], [0, 0, 1], [1, 1, 1], [2, 1, 1], [1, 2, 1]])
    pa, na = b.interleaved(sp, sn)
    prim_sphere = {"attributes": {"POSITION": pa, "NORMAL": na,
                                  "TEXCOORD_0": b.accessor(st, "VEC2")},
                   "indices": b.accessor(si.astype(np.uint16), "SCALAR", ctype=5123), "material": 1}
    prim_quad = {"attributes": {"POSITION": b.accessor(quad_p, "VEC3")},
                 "indices": b.accessor(quad_i, "SCALAR", ctype=5121), "material": 0}
    prim_tri = {"attributes": {"POSITION": b.accessor(tri_p, "VEC3")}}        # no indices
    prim_u32 = {"attributes": {"POSITION": b.accessor(quad_p, "VEC3")},
                "indices": b.accessor(quad_i.astype(np.uint32), "SCALAR", ctype=5125)}
    prim_lines = {"attributes": {"POSITION": b.accessor(quad_p, "VEC3")}, "mode": 1}
    prim_short = {"attributes": {"POSITION": b.accessor(np.int16([[1, 2, 3]] * 3), "VEC3", ctype=5122)}}
    doc = {
        "asset": {"version": "2.0"},
        "scene": 0,
        "scenes": [{"nodes": [0, 3]}, {"nodes": [5]}],
        "nodes": [
            {"name": "root", "translation": [1, 2, 3], "rotation": [0, 0.38268343, 0, 0.92387953],
             "scale": [2, 2, 2], "children": [1, 2]},
            {"name": "ball", "mesh": 0, "translation": [0, 1, 0],
             "extensions": {"AURORA_materials_materialX": {"materialXFile": "x.mtlx"}}},
            {"name": "cam", "camera": 0, "translation": [0, 1, 5]},
            {"name": "flat", "mesh": 1,
             "matrix": [1, 0, 0, 0, 0, 0.5, 0, 0, 0, 0, 1, 0, -3, 0, 0.25, 1], "children": [4]},
            {"name": "child", "mesh": 2, "rotation": [0.5, 0.5, 0.5, 0.5]},
            {"name": "second scene", "mesh": 3, "children": [6]},
            {"name": "ortho", "camera": 1, "rotation": [0, 0, 0.70710677, 0.70710677]},
        ],
        "meshes": [{"primitives": [prim_sphere]},
                   {"primitives": [prim_quad, prim_lines]},
                   {"primitives": [prim_tri, prim_short]},
                   {"primitives": [prim_u32]}],
        "materials": [
            {"name": "default"},
            {"pbrMetallicRoughness": {"baseColorFactor": [0.8, 0.2, 0.1, 1.0], "metallicFactor": 0.25,
                                      "roughnessFactor": 0.6}},
        ],
        "cameras": [
            {"type": "perspective", "perspective": {"yfov": 0.7, "aspectRatio": 1.5, "znear": 0.1,
                                                    "zfar": 100}},
            {"type": "orthographic", "orthographic": {"xmag": 2, "ymag": 1.5, "znear": 0.01, "zfar": 50}},
        ],
        "bufferViews": b.views,
        "accessors": b.accessors,
        "buffers": [{"byteLength": len(b.blob)}],
    }
    # (node chain, positions, normals or None, uvs or None, indices, material index or None)
    expected = [
        ([0, 1], sp, sn, st, si, 1),
        ([3], quad_p, None, None, quad_i.astype(np.uint32), 0),
        ([3, 4], tri_p, None, None, np.arange(6, dtype=np.uint32), None),
        ([5], quad_p, None, None, quad_i.astype(np.uint32), None),
    ]
    return doc, bytes(b.blob), expected


def write(tmp, form, doc, blob):
    doc = json.loads(json.dumps(doc))
    if form == "embedded":
        doc["buffers"][0]["uri"] = "data:application/octet-stream;base64," + base64.b64encode(blob).decode()
        path = os.path.join(tmp, "scene.gltf")
        open(path, "w").write(json.dumps(doc, indent=1))
    elif form == "external":
        doc["buffers"][0]["uri"] = "scene%20data.bin"
        open(os.path.join(tmp, "scene data.bin"), "wb").write(blob)
        path = os.path.join(tmp, "scene.gltf")
        open(path, "w").write(json.dumps(doc))
    else:
        js = json.dumps(doc).encode()
        js += b" " * (-len(js) % 4)
        bn = blob + b"\0" * (-len(blob) % 4)
        body = struct.pack("<II", len(js), 0x4E4F534A) + js + struct.pack("<II", len(bn), 0x004E4942) + bn
        path = os.path.join(tmp, "scene.glb")
        open(path, "wb").write(struct.pack("<III", 0x46546C67, 2, 12 + len(body)) + body)
    return path


def load(form):
    doc, blob, expected = make_doc()
    with tempfile.TemporaryDirectory() as tmp:
        path = write(tmp, form, doc, blob)
        return run("gltf", path), doc, expected, path


def test_gltf_container_forms_agree():
    outs = []
    for form in ("embedded", "external", "glb"):
        out, _, _, path = load(form)
        assert out["ok"], out["warnings"]
        # paths carry the file name; compare everything else
        for inst in out["instances"]:
            inst["instance"] = inst["instance"].split(":gltf")[1]
            inst["geometry"] = inst["geometry"].split(":gltf")[1]
            inst["material"] = inst["material"].split(":gltf")[-1]
        for m in out["materials"]:
            m["path"] = m["path"].split(":gltf")[1]
        out["warnings"] = out["warnings"].replace(os.path.dirname(path), "")
        outs.append(out)
    assert outs[0] == outs[1] == outs[2]


def test_gltf_translation_matches_restatement():
    out, doc, expected, path = load("glb")
    assert out["ok"]
    w = out["warnings"]
    assert "MaterialX" in w and "component type 5122" in w
    nodes = doc["nodes"]
    assert len(out["instances"]) == len(expected)
    bmin, bmax = np.full(3, np.inf, np.float32), np.full(3, -np.inf, np.float32)
    verts = tris = 0
    for k, (inst, (chain, p, n, t, idx, mat)) in enumerate(zip(out["instances"], expected)):
        assert inst["instance"] == f"{path}:gltfInst:{k}"
        assert inst["geometry"] == f"{path}:gltfGeom:{k}"
        m = np.eye(4, dtype=np.float32).reshape(-1)
        for ni in chain:
            m = mul(m, node_matrix(nodes[ni]))
        np.testing.assert_array_equal(np.float32(inst["transform"]), m, err_msg=str(chain))
        np.testing.assert_array_equal(np.float32(inst["positions"]).reshape(-1, 3), p)
        np.testing.assert_array_equal(np.uint32(inst["indices"]), idx)
        got_n = np.float32(inst["normals"]).reshape(-1, 3)
        if n is not None:
            np.testing.assert_array_equal(got_n, n)
        else:
            np.testing.assert_allclose(np.linalg.norm(got_n, axis=1), 1.0, atol=1e-6)
        if t is not None:
            np.testing.assert_array_equal(np.float32(inst["texcoords"]).reshape(-1, 2), t)  # no V flip
        else:
            assert inst["texcoords"] == []
        assert inst["material"] == ("" if mat is None else f"{path}:gltfMat:{mat}")
        wp = transform_points(m, p)
        bmin, bmax = np.minimum(bmin, wp.min(0)), np.maximum(bmax, wp.max(0))
        verts += len(p)
        tris += len(idx) // 3
    # The flat quad's generated normals: its face normal (p2 - p0) x (p1 - p0) = +Y for the
    # winding 0-2-1.
    quad_n = np.float32(out["instances"][1]["normals"]).reshape(-1, 3)
    np.testing.assert_allclose(quad_n, [[0, 1, 0]] * 4, atol=1e-7)
    np.testing.assert_array_equal(np.float32(out["bounds"][0]), bmin)
    np.testing.assert_array_equal(np.float32(out["bounds"][1]), bmax)
    assert out["vertices"] == verts and out["triangles"] == tris
    mats = {m["path"].split(":gltfMat:")[1]: m["properties"] for m in out["materials"]}
    assert mats["0"] == {"base_color": [1.0, 1.0, 1.0], "metalness": 1.0, "specular_roughness": 1.0}
    np.testing.assert_array_equal(np.float32(mats["1"]["base_color"]), np.float32([0.8, 0.2, 0.1]))
    assert np.float32(mats["1"]["metalness"]) == np.float32(0.25)
    assert np.float32(mats["1"]["specular_roughness"]) == np.float32(0.6)


def test_gltf_cameras_and_save_round_trip():
    out, doc, _, path = load("external")
    cams = out["cameras"]
    assert [c["name"] for c in cams] == ["cam", "ortho"]
    assert [c["type"] for c in cams] == ["perspective", "orthographic"]
    # the view is the inverse of the camera node's own transform (not its parents')
    for c, ni in zip(cams, (2, 6)):
        node = node_matrix(doc["nodes"][ni]).reshape(4, 4).T
        view = np.float32(c["view"]).reshape(4, 4).T
        np.testing.assert_allclose(view @ node, np.eye(4), atol=1e-6)
    np.testing.assert_array_equal(np.float32(cams[0]["values"]), np.float32([0.7, 1.5, 0, 0, 0.1, 100]))
    np.testing.assert_array_equal(np.float32(cams[1]["values"]), np.float32([0, 0, 2, 1.5, 0.01, 50]))
    with tempfile.TemporaryDirectory() as tmp:
        doc2, blob, _ = make_doc()
        src = write(tmp, "glb", doc2, blob)
        saved = os.path.join(tmp, "cameras.gltf")
        from test_loaders import tool
        import subprocess
        subprocess.check_call([tool(), "gltfsave", saved, src])
        again = run("gltf", saved)
        saved_doc = json.load(open(saved))
    assert again["ok"] and again["instances"] == []
    assert saved_doc["asset"]["version"] == "2.0" and len(saved_doc["nodes"]) == 2
    for a, b in zip(cams, again["cameras"]):
        assert a["name"] == b["name"] and a["type"] == b["type"] and a["values"] == b["values"]
        np.testing.assert_allclose(np.float32(a["view"]), np.float32(b["view"]), atol=1e-6)


def test_gltf_errors_are_reported():
    doc, blob, _ = make_doc()
    with tempfile.TemporaryDirectory() as tmp:
        path = write(tmp, "external", doc, blob)
        os.remove(os.path.join(tmp, "scene data.bin"))
        out = run("gltf", path)
        assert not out["ok"] and "cannot read buffer" in out["warnings"]
        bad = os.path.join(tmp, "bad.gltf")
        open(bad, "w").write('{"asset": {"version": "2.0"}, "nodes": [1, }')
        out = run("gltf", bad)
        assert not out["ok"] and "invalid JSON" in out["warnings"]
        # an accessor that runs past its buffer view skips the primitive with a warning
        doc2 = json.loads(json.dumps(doc))
        doc2["accessors"][0]["count"] = 10 ** 6
        out = run("gltf", write(tmp, "embedded", doc2, blob))
        assert out["ok"] and "outside its buffer" in out["warnings"]
        assert len(out["instances"]) == 3
