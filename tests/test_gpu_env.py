"""Environment importance sampling on the GPU: the alias table built from FP64 prefix sums has the
reference's per-texel pdf (AliasMap.cpp:113-114) and samples texels in proportion to
luminance x solid angle; sampling through it matches the oracle's restatement of
Environment.slang:137-186."""
import numpy as np
import pytest
import torch

from gpu_util import dev, empty, host

pytestmark = pytest.mark.gpu


def implied(alias, prob):
    n = len(alias)
    keep = np.clip(prob.astype(np.float64), 0.0, 1.0)
    out = keep.copy()
    np.add.at(out, alias.astype(np.int64), 1.0 - keep)
    return out / n


def exact_distribution(img):
    h, w = img.shape[:2]
    lum = (img[..., 0].astype(np.float32) * np.float32(0.2125) +
           img[..., 1].astype(np.float32) * np.float32(0.7154)) + \
        img[..., 2].astype(np.float32) * np.float32(0.0721)
    lat = np.pi / 2 - np.arange(h) * np.pi / h
    sa = (np.sin(lat) - np.sin(lat - np.pi / h)) * 2 * np.pi / w
    weight = (lum.astype(np.float64) * sa[:, None]).reshape(-1)
    return weight / weight.sum(), lum.reshape(-1), weight.sum()


def env_scene(img):
    from aurora_gb300 import _abi, scenes
    s = scenes.SceneDesc("env")
    k = s.add_image(img, _abi.FORMAT_RGB32F)
    s.env_light = s.env_background = k
    s.materials = scenes.materials(1)
    s.width = s.height = 4
    s.frame = scenes.frame_data(np.eye(4), scenes.perspective(45, 1))
    return s


def env_image(h, w, seed):
    from aurora_gb300 import scenes
    return scenes.hdr_env(w, h, seed) if h >= 32 else \
        np.random.default_rng(seed).uniform(0, 4, (h, w, 3)).astype(np.float32)


SHAPES = [((1024, 2048), 5), ((32, 64), 6), ((7, 13), 7), ((1, 1), 8)]


@pytest.mark.parametrize("shape,seed", SHAPES)
def test_reference_layout_table_is_bit_identical_to_reference(agb, oracle, shape, seed):
    """Default table: the reference's AliasMap::build reproduced bit for bit on the device."""
    from aurora_gb300 import api
    h, w = shape
    img = env_image(h, w, seed)
    with api.Renderer() as r:
        r.upload(env_scene(img))
        table, integral, i64 = r.environment_alias(fp64_integral=True)
    ref, ref_integral = oracle.alias_build(img)
    np.testing.assert_array_equal(table["alias"], ref["alias"])
    np.testing.assert_array_equal(table["prob"], ref["prob"])
    np.testing.assert_array_equal(table["pdf"], ref["pdf"])
    assert np.float32(integral) == np.float32(ref_integral)
    expect, lum, total = exact_distribution(img)
    assert abs(i64 - total) <= 1e-9 * total
    print(f"{w}x{h}: reference FP32 integral off by {ref_integral / total - 1:.2e}")


@pytest.mark.parametrize("shape,seed", SHAPES)
def test_fp64_layout_table_distribution_and_pdf(agb, oracle, shape, seed):
    """FP64 prefix-sum table: exact texel distribution, pdf = luminance / FP64 integral."""
    from aurora_gb300 import _abi, api
    h, w = shape
    img = env_image(h, w, seed)
    with api.Renderer() as r:
        r.set_environment_table(_abi.ENV_TABLE_FP64)
        r.upload(env_scene(img))
        table, integral, i64 = r.environment_alias(fp64_integral=True)
    expect, lum, total = exact_distribution(img)
    assert abs(i64 - total) <= 1e-9 * total
    assert np.float32(integral) == np.float32(i64)
    got = implied(table["alias"], table["prob"])
    np.testing.assert_allclose(got, expect, rtol=1e-5, atol=1e-12)
    assert (table["alias"] < w * h).all()
    np.testing.assert_allclose(table["pdf"], (lum / np.float32(i64)).astype(np.float32), rtol=1e-6)
    # Same per-texel formula as the reference, up to its FP32 integral drift.
    ref, ref_integral = oracle.alias_build(img)
    scaled = table["pdf"].astype(np.float64) * i64 / ref_integral
    np.testing.assert_allclose(scaled, ref["pdf"], rtol=2e-6, atol=0)


def test_environment_sampling_matches_oracle(agb, oracle):
    from aurora_gb300 import api, scenes
    img = scenes.hdr_env(256, 128, 3)
    s = env_scene(img)
    n = 100_000
    rnd = np.random.default_rng(1).uniform(size=(n, 2)).astype(np.float32)
    with api.Renderer() as r:
        r.upload(s)
        table, integral = r.environment_alias()
        d_rnd = dev(rnd)
        out_r, out_d, out_p = empty((n, 3), torch.float32), empty((n, 3), torch.float32), \
            empty((n,), torch.float32)
        r.env_sample(d_rnd.data_ptr(), n, out_r.data_ptr(), out_d.data_ptr(), out_p.data_ptr())
        gr, gd, gp = host(out_r), host(out_d), host(out_p)
    ref, ref_integral = oracle.alias_build(img)
    env = np.ascontiguousarray(s.env).reshape(1).copy()
    env["has_light_tex"] = 1
    env["light_tex_luminance_integral"] = ref_integral
    rgba = np.ones((128, 256, 4), np.float32)
    rgba[..., :3] = img
    orr, od, op = oracle.env_sample(env, rgba, ref, rnd)
    np.testing.assert_array_equal(gr, orr)
    np.testing.assert_array_equal(gp, op)
    np.testing.assert_array_equal(gd, od)


def test_all_black_environment(agb, oracle):
    from aurora_gb300 import _abi, api
    img = np.zeros((8, 16, 3), np.float32)
    with api.Renderer() as r:
        r.upload(env_scene(img))
        table, integral = r.environment_alias()
    ref, ref_integral = oracle.alias_build(img)  # the reference divides 0 by 0 here
    np.testing.assert_array_equal(table["alias"], ref["alias"])
    np.testing.assert_array_equal(table["prob"], ref["prob"])
    with api.Renderer() as r:
        r.set_environment_table(_abi.ENV_TABLE_FP64)
        r.upload(env_scene(img))
        table, integral = r.environment_alias()
    assert integral == 0.0
    assert (table["alias"] == np.arange(128)).all()
    assert (table["pdf"] == 0).all()
