"""The oracle pinned against the reference's own shader source.

oracle/build_oracle.py compiles the reference's unmodified Shaders/StandardSurfaceBSDF.slang,
BSDFCommon.slang, Sampling.slang, Random.slang, Environment.slang (with Globals, Colors and
Material) as host C++ through a mechanical rewrite and an HLSL vocabulary header
(oracle/ref_shim), in FP32 (the shaders' arithmetic) and FP64 (the same source in double).  Where
the reference tree is present these tests compare the oracle's restatement with it live on 100K
seeded cases per operation; everywhere they compare with tests/golden/shaders_ref.npz, made from
it by tests/golden/make_golden.py.  Tolerances: tests/bsdf_cases.py (1e-5 relative, or the
reference's own FP32 conditioning on the cases where that is larger; identical lobe choices)."""
import ctypes
import os

import numpy as np
import pytest

from bsdf_cases import check, make_cases, tolerances

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden", "shaders_ref.npz")


def golden():
    g = np.load(GOLDEN)
    from aurora_gb300 import _abi
    m = g["materials"].view(_abi.MATERIAL_DTYPE)
    return g, m


def need_reference(oracle):
    if oracle.ref_lib() is None:
        pytest.skip("the reference tree is not on this machine (the fixture tests cover it)")


@pytest.mark.parametrize("op", [0, 1, 2])
def test_oracle_bsdf_against_reference_source(oracle, op):
    need_reference(oracle)
    m, idx, frames, V, L, rnd = make_cases(100_000, 11 + op)
    r32, r64, tol = tolerances(oracle.ref_bsdf_batch, op, m, idx, frames, V, L, rnd)
    o32 = oracle.bsdf_batch(op, m, idx, frames, V, L, rnd, precision=32)
    print(check(op, o32, r32, tol, "FP32 oracle vs reference source FP32"))
    o64 = oracle.bsdf_batch(op, m, idx, frames, V, L, rnd, precision=64)
    print(check(op, o64, r64, tol, "FP64 oracle vs reference source FP64"))


@pytest.mark.parametrize("op", [0, 1, 2])
def test_oracle_bsdf_against_reference_fixture(oracle, op):
    g, m = golden()
    args = (m, g["idx"], g["frames"], g["V"], g["L"], g["rnd"])
    tol = g[f"op{op}_tol"]
    for prec in (32, 64):
        ref = tuple(g[f"op{op}_ref{prec}_{k}"] for k in ("value", "dir", "pdf", "lobe"))
        got = oracle.bsdf_batch(op, *args, precision=prec)
        print(check(op, got, ref, tol, f"FP{prec} oracle vs reference fixture"))


def test_fixture_matches_reference_source(oracle):
    """The committed fixture is what the reference source computes on this machine."""
    need_reference(oracle)
    g, m = golden()
    args = (m, g["idx"], g["frames"], g["V"], g["L"], g["rnd"])
    for op in (0, 1, 2):
        for prec in (32, 64):
            got = oracle.ref_bsdf_batch(op, *args, precision=prec)
            for k, name in enumerate(("value", "dir", "pdf", "lobe")):
                np.testing.assert_array_equal(got[k], g[f"op{op}_ref{prec}_{name}"])


def test_random_streams_match_reference(oracle):
    g, _ = golden()
    for args, want in zip(g["random_args"], g["random_streams"]):
        np.testing.assert_array_equal(oracle.random_stream(*[int(a) for a in args], 16), want)
        if oracle.ref_lib() is not None:
            np.testing.assert_array_equal(oracle.ref_random_stream(*[int(a) for a in args], 16), want)


def env_inputs(g):
    from aurora_gb300 import _abi
    img = g["env_image"]
    rgba = np.ones(img.shape[:2] + (4,), np.float32)
    rgba[..., :3] = img
    alias = g["env_alias"].view(_abi.ALIAS_DTYPE)
    env = g["env_data"].view(_abi.ENV_DTYPE).reshape(1)
    return img, rgba, alias, env


def test_environment_sampling_matches_reference(oracle):
    """sampleEnvironment (Environment.slang:137-186): texel radiance and pdf identical; the
    direction (latLongUVToDirection's sincos) within two FP32 ulps."""
    g, _ = golden()
    img, rgba, alias, env = env_inputs(g)
    ref_alias, _ = oracle.alias_build(img)
    np.testing.assert_array_equal(ref_alias.view(np.uint8), alias.view(np.uint8))
    r, d, p = oracle.env_sample(env, rgba, alias, g["env_rnd"])
    np.testing.assert_array_equal(r, g["env_radiance"])
    np.testing.assert_array_equal(p, g["env_pdf"])
    assert np.abs(d - g["env_dir"]).max() <= 2.4e-7


def test_environment_evaluation_matches_reference(oracle):
    """evaluateEnvironment (Environment.slang:98-133) as light (the texture) and as background
    (the gradient, as this environment has no background image): with nearest filtering (the
    renderer's default sampler) the same texels and the gradient within 1e-6 relative (its
    v coordinate comes from asin, last ulps); bilinear within 1e-4 relative (the interpolation
    weights come from atan2 / asin of the direction, whose last-ulp differences are scaled by the
    texel contrast)."""
    need_reference(oracle)
    g, _ = golden()
    img, rgba, alias, env = env_inputs(g)
    n = 50_000
    d = np.random.default_rng(2).normal(size=(n, 3))
    d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    bg = (np.arange(n) % 2).astype(np.int32)
    for linear in (0, 1):
        im = oracle.Image()
        im.rgba, im.width, im.height, im.linear = rgba.ctypes.data, rgba.shape[1], rgba.shape[0], linear
        out = np.zeros((n, 3), np.float32)
        oracle.lib().orc_env_evaluate(oracle._p(env), ctypes.byref(im), ctypes.byref(im),
                                      oracle._p(d), oracle._p(bg), n, oracle._p(out))
        ref = oracle.ref_env_evaluate(env, rgba, rgba, d, bg, linear=bool(linear))
        err = np.abs(out - ref).max(1) / np.maximum(np.abs(ref).max(1), 1e-6)
        print(f"linear {linear}: identical {np.mean((out == ref).all(1)):.4f}, max rel {err.max():.3g}")
        if linear:
            assert err.max() <= 1e-4
        else:
            np.testing.assert_array_equal(out[bg == 0], ref[bg == 0])
            assert err.max() <= 1e-6
