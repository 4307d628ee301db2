"""CPU tests: byte layouts against the reference's own definitions, the oracle against the
reference's alias-table build (live and through committed fixtures), the random-number generator
against an independent restatement, and the exported C-ABI symbols."""
import ctypes
import json
import os
import re

import numpy as np
import pytest

from conftest import ROOT

GOLDEN = os.path.join(ROOT, "tests", "golden")


def camel_to_snake(name):
    s = re.sub(r"(.)([A-Z][a-z]+)", r"\1_\2", name)
    s = re.sub(r"([a-z0-9])([A-Z])", r"\1_\2", s).lower()
    return s.replace("ao_vs", "aovs")


def test_material_block_matches_reference_layout():
    from aurora_gb300 import _abi
    ref = json.load(open(os.path.join(GOLDEN, "material_layout.json")))
    assert ref["size"] == 400 == _abi.MATERIAL_DTYPE.itemsize
    assert len(ref["fields"]) == 57
    sizes = {"float": 4, "int": 4, "float2": 8, "float3": 12}
    for f in ref["fields"]:
        name = f["property"]
        dt, off = _abi.MATERIAL_DTYPE.fields[name][:2]
        assert off == f["offset"], name
        assert dt.itemsize == sizes[f["type"]], name


def test_frame_and_environment_layouts_match_reference_order():
    from aurora_gb300 import _abi
    ref = json.load(open(os.path.join(GOLDEN, "frame_layout.json")))
    ours = [n for n in _abi.FRAME_DTYPE.names]
    theirs = [camel_to_snake(f["name"]) for f in ref["frame"] if f["name"] != "lights"]
    assert ours[: len(theirs)] == theirs
    assert ours[len(theirs):] == ["distant_lights", "distant_light_count", "_light_pad"]
    assert _abi.FRAME_DTYPE.fields["distant_lights"][1] == 368
    env = [f for f in ref["environment"] if f["type"] != "bool"]
    assert [camel_to_snake(f["name"]) for f in env] == list(_abi.ENV_DTYPE.names)
    light = [camel_to_snake(f["name"]) for f in ref["distant_light"]]
    assert light == list(_abi.DISTANT_LIGHT_DTYPE.names)


def test_oracle_layouts_match_abi(oracle):
    from aurora_gb300 import _abi
    L = oracle.lib()
    assert L.orc_layout(0) == _abi.MATERIAL_DTYPE.itemsize
    assert L.orc_layout(1) == _abi.FRAME_DTYPE.itemsize
    assert L.orc_layout(2) == _abi.ENV_DTYPE.itemsize
    assert L.orc_layout(3) == ctypes.sizeof(oracle.Mesh)
    assert L.orc_layout(4) == ctypes.sizeof(oracle.Instance)
    assert L.orc_layout(5) == ctypes.sizeof(oracle.Image)
    assert L.orc_layout(6) == ctypes.sizeof(oracle.Scene)
    assert L.orc_layout(7) == ctypes.sizeof(oracle.Layer)
    assert L.orc_layout(8) == _abi.GROUND_PLANE_DTYPE.itemsize


def test_oracle_alias_table_matches_reference_fixtures(oracle):
    g = np.load(os.path.join(GOLDEN, "alias_ref.npz"))
    names = sorted({k[: -len("_image")] for k in g.files if k.endswith("_image")})
    assert len(names) == 4
    for name in names:
        table, integral = oracle.alias_build(g[name + "_image"], precision=32)
        np.testing.assert_array_equal(table["alias"], g[name + "_alias"], err_msg=name)
        np.testing.assert_array_equal(table["prob"], g[name + "_prob"], err_msg=name)
        np.testing.assert_array_equal(table["pdf"], g[name + "_pdf"], err_msg=name)
        assert np.float32(integral) == g[name + "_integral"], name


def test_oracle_alias_table_matches_reference_source_live(oracle):
    import build_oracle
    path = build_oracle.build_reference_alias()
    if path is None:
        pytest.skip("reference tree not present on this host")
    ref = ctypes.CDLL(path)
    rng = np.random.default_rng(7)
    for (w, h) in [(128, 64), (33, 17), (1, 1), (2, 9)]:
        img = np.ascontiguousarray(np.exp(rng.normal(0, 1.5, (h, w, 3))), np.float32)
        table = np.zeros((w * h, 4), np.uint32)
        integ = ctypes.c_float()
        ref.ref_alias_build(img.ctypes.data_as(ctypes.c_void_p), w, h,
                            table.ctypes.data_as(ctypes.c_void_p), ctypes.byref(integ))
        ours, oi = oracle.alias_build(img)
        np.testing.assert_array_equal(ours["alias"], table[:, 0])
        np.testing.assert_array_equal(ours["prob"], table[:, 1].view(np.float32))
        np.testing.assert_array_equal(ours["pdf"], table[:, 2].view(np.float32))
        assert np.float32(oi) == np.float32(integ.value)


def implied_distribution(alias, prob):
    """Probability of each entry under Environment.slang's sampling: pick a bucket uniformly, keep
    it with probability min(prob, 1), else take its alias."""
    n = len(alias)
    keep = np.clip(prob.astype(np.float64), 0.0, 1.0)
    out = keep.copy()
    np.add.at(out, alias.astype(np.int64), 1.0 - keep)
    return out / n


def test_reference_alias_table_samples_luminance_times_solid_angle():
    g = np.load(os.path.join(GOLDEN, "alias_ref.npz"))
    img = g["lognormal_64x32_image"].astype(np.float64)
    h, w = img.shape[:2]
    lum = img @ np.array([0.2125, 0.7154, 0.0721])
    lat = np.pi / 2 - np.arange(h) * np.pi / h
    sa = (np.sin(lat) - np.sin(lat - np.pi / h)) * 2 * np.pi / w
    weight = (lum * sa[:, None]).reshape(-1)
    expect = weight / weight.sum()
    got = implied_distribution(g["lognormal_64x32_alias"], g["lognormal_64x32_prob"])
    # The reference sweeps in FP32, subtracting deficits from a running probability, so its
    # implied distribution drifts by up to ~4e-4 relative; the FP64 device build is held to 1e-6.
    np.testing.assert_allclose(got, expect, rtol=1e-3, atol=1e-9)


def pcg2d_python(sample, width, px, py, n):
    """Independent restatement of Random.slang:96-137 in Python integers."""
    M = 0xFFFFFFFF
    x, y = (py * width + px) & M, sample & M
    out = []
    for _ in range(n):
        x = (x + y * 1664525) & M
        y = (y + x * 1664525) & M
        x ^= x >> 16
        y ^= y >> 16
        x = (x + y * 1664525) & M
        y = (y + x * 1664525) & M
        x ^= x >> 16
        y ^= y >> 16
        out.append((np.float32(x) / np.float32(4294967296.0), np.float32(y) / np.float32(4294967296.0)))
    return np.array(out, np.float32)


def test_oracle_rng_matches_independent_restatement(oracle):
    for args in [(0, 512, 0, 0), (17, 1920, 1919, 1079), (4095, 3840, 123, 456)]:
        np.testing.assert_array_equal(oracle.random_stream(*args, 40), pcg2d_python(*args, 40))


def test_oracle_fp32_and_fp64_agree_and_bvh_matches_brute_force(oracle):
    from aurora_gb300 import scenes
    s = scenes.config_tiny()
    o = oracle.OracleScene(s)
    r32 = o.render(0, 4, precision=32)
    r64 = o.render(0, 4, precision=64)
    rb = o.render(0, 4, precision=32, brute=True)
    assert oracle.rel_mse(r32["mean"], r64["mean"]) < 1e-6
    np.testing.assert_array_equal(r32["mean"], rb["mean"])
    assert r32["rays"] > 0 and r32["shadow_rays"] > 0


def test_oracle_progressive_resume_equals_single_render(oracle):
    from aurora_gb300 import scenes
    o = oracle.OracleScene(scenes.config_tiny())
    a = o.render(0, 4, want_sum=True)
    b1 = o.render(0, 2, want_sum=True)
    b2 = o.render(2, 2, want_sum=True)
    np.testing.assert_allclose(b1["sum"] + b2["sum"], a["sum"], rtol=0, atol=1e-9)


def test_sheen_tables_identical():
    def numbers(path):
        txt = open(path).read()
        body = txt[txt.index("{", txt.index("256")) + 1: txt.index("};")]
        body = re.sub(r"//[^\n]*", "", body)
        return np.array([float(v.strip().rstrip("f")) for v in body.split(",") if v.strip()], np.float32)
    a = numbers(os.path.join(ROOT, "oracle", "sheen_lut.hpp"))
    b = numbers(os.path.join(ROOT, "aurora_gb300", "csrc", "agb_sheen_lut.cuh"))
    assert a.shape == (256,)
    np.testing.assert_array_equal(a, b)
    from build_oracle import REFERENCE_SOURCE
    ref = os.path.join(REFERENCE_SOURCE, "Shaders", "StandardSurfaceBSDF.slang")
    if os.path.exists(ref):
        src = open(ref).read()
        m = re.search(r"u_sheenAlbedo\[[^\]]*\] = \{(.*?)\};", src, re.S)
        vals = np.array([float(v) for v in m.group(1).replace("\n", " ").split(",") if v.strip()], np.float32)
        np.testing.assert_array_equal(a, vals)


def test_cabi_library_exports_every_declared_symbol():
    from aurora_gb300 import _abi, build
    build.build()
    header = open(os.path.join(ROOT, "include", "agb.h")).read()
    declared = set(re.findall(r"AGB_API\s+[\w\s\*]+?\b(agb_\w+)\s*\(", header))
    assert declared, "no declarations found"
    assert declared == set(_abi.SIGNATURES), declared ^ set(_abi.SIGNATURES)
    lib = ctypes.CDLL(_abi.LIB_PATH)
    for name in declared:
        assert hasattr(lib, name), name


def test_temporal_jitter_pins(oracle):
    """Halton (2, 3) jitter (PTRenderer.cpp:81-95,159-174) against an independent restatement in
    Python float32, and the library's host function (no GPU work) against it."""
    from aurora_gb300 import api, build
    build.build()

    def halton(index, base):
        result, scale = np.float32(0.0), np.float32(1.0) / np.float32(base)
        while index > 0:
            result = np.float32(result + scale * np.float32(index % base))
            index //= base
            scale = np.float32(scale / np.float32(base))
        return result

    for frame in range(40):
        for phases in (0, 8, 11):
            i = (frame % phases if phases else frame) + 1
            want = (float(np.float32(halton(i, 2) - np.float32(0.5))),
                    float(np.float32(halton(i, 3) - np.float32(0.5))))
            assert oracle.temporal_jitter(frame, phases) == want
            assert api.temporal_jitter(frame, phases) == want
    assert api.temporal_jitter(0) == (0.0, float(np.float32(1 / 3) - np.float32(0.5)))


def test_conv_entry_points_reject_bad_shapes_before_touching_the_gpu():
    """The convolution entry points check their arguments on the host: an odd width, a pooled or
    upsampled odd height, channel counts off the 16 grid, misaligned outputs."""
    import ctypes
    from aurora_gb300 import _abi
    lib = _abi.library()
    buf = ctypes.create_string_buffer(1 << 16)
    base = (ctypes.addressof(buf) + 255) // 256 * 256
    p = ctypes.c_void_p(base)
    conv = lib.agb_conv3x3_bf16
    pool = lib.agb_conv3x3_pool_bf16
    wgrad = lib.agb_conv3x3_wgrad_bf16
    cases = [
        (conv, (p, None, p, None, p, None, 1, 4, 5, 16, 0, 32, 0, 1, None), b"width must be even"),
        (conv, (p, None, p, None, p, None, 1, 5, 4, 16, 0, 32, 1, 1, None), b"even sizes"),
        (conv, (p, None, p, None, p, None, 1, 4, 4, 16, 0, 24, 0, 1, None), b"multiples of 16"),
        (conv, (p, None, p, None, ctypes.c_void_p(base + 16), None, 1, 4, 4, 16, 0, 32, 0, 1, None),
         b"32-byte aligned"),
        (pool, (p, None, p, None, p, p, 1, 3, 4, 16, 0, 32, 0, 1, None), b"even sizes"),
        (pool, (p, None, p, None, p, None, 1, 4, 4, 16, 0, 32, 0, 1, None), b"null pool output"),
        (wgrad, (p, None, p, p, 1, 4, 3, 16, 0, 32, 0, None), b"width must be even"),
    ]
    for fn, args, why in cases:
        assert fn(*args) == _abi.ERR_INVALID_ARG, why
        assert why in lib.agb_last_error(), (why, lib.agb_last_error())


def test_render_stats_layout_matches_ctypes(tmp_path):
    """agb_render_stats as the C compiler lays it out (include/agb.h) equals the ctypes mirror the
    Python host reads it through: size and the offsets of the fields appended last."""
    import shutil
    import subprocess
    from aurora_gb300 import _abi
    gcc = shutil.which("gcc")
    if not gcc:
        pytest.skip("no C compiler")
    include = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")
    src = tmp_path / "stats.c"
    src.write_text('#include <stddef.h>\n#include <stdio.h>\n#include "agb.h"\n'
                   'int main(void) { printf("%zu %zu %zu %zu\\n", sizeof(agb_render_stats), '
                   'offsetof(agb_render_stats, shading_points), '
                   'offsetof(agb_render_stats, closest_rays_per_bounce), '
                   'offsetof(agb_render_stats, shadow_rays_per_bounce)); return 0; }\n')
    exe = tmp_path / "stats"
    subprocess.check_call([gcc, "-I" + include, str(src), "-o", str(exe)])
    size, sp, cb, sb = map(int, subprocess.check_output([str(exe)]).split())
    S = _abi.RenderStats
    assert size == ctypes.sizeof(S)
    assert (sp, cb, sb) == (S.shading_points.offset, S.closest_rays_per_bounce.offset,
                            S.shadow_rays_per_bounce.offset)
