"""Standard Surface evaluate / sample / evaluate-with-pdf on the GPU (StandardSurfaceBSDF.slang:
598-1372) against the FP32 oracle (identical to 1e-5 on every case, identical lobes), against the
reference's own shader source compiled as host C++ (committed fixture) and against the FP64
oracle, with the per-case tolerance of tests/bsdf_cases.py; plus the random streams and
environment sampling against the reference source."""
import numpy as np
import pytest
import torch

from bsdf_cases import TOL, check, make_cases, tolerances
from gpu_util import dev, empty, host

pytestmark = pytest.mark.gpu


def run_gpu(op, m, idx, frames, V, L, rnd):
    from aurora_gb300 import api
    n = len(idx)
    out_v = empty((n, 3), torch.float32)
    out_d = empty((n, 3), torch.float32)
    out_p = empty((n,), torch.float32)
    out_l = empty((n,), torch.int32)
    dm = dev(m.view(np.uint8))
    args = [dev(idx), dev(frames), dev(V), dev(L), dev(rnd)]
    api.bsdf_batch(op, dm.data_ptr(), args[0].data_ptr(), args[1].data_ptr(), args[2].data_ptr(),
                   args[3].data_ptr(), args[4].data_ptr(), n, out_v.data_ptr(), out_d.data_ptr(),
                   out_p.data_ptr(), out_l.data_ptr())
    return host(out_v), host(out_d), host(out_p), host(out_l)


@pytest.mark.parametrize("op", [0, 1, 2])
def test_bsdf_matches_oracle(agb, oracle, op):
    """Device against the FP32 oracle on 200K seeded cases: every value, pdf and direction within
    1e-5 (normwise relative) and every lobe choice identical (the two share operation order and
    transcendental code)."""
    m, idx, frames, V, L, rnd = make_cases(200_000, 11 + op)
    got = run_gpu(op, m, idx, frames, V, L, rnd)
    ref = oracle.bsdf_batch(op, m, idx, frames, V, L, rnd, precision=32)
    tol = np.full((3, len(idx)), TOL, np.float32)
    print(check(op, got, ref, tol, "device vs FP32 oracle"))


@pytest.mark.parametrize("op", [0, 1, 2])
def test_bsdf_matches_reference_source(agb, op):
    """Device against the reference's own StandardSurfaceBSDF.slang compiled as host C++ (the
    committed fixture tests/golden/shaders_ref.npz: 4096 seeded cases, FP32 and FP64 builds), with
    the per-case tolerance of tests/bsdf_cases.py."""
    from test_reference_pin import golden
    g, m = golden()
    args = (m, g["idx"], g["frames"], g["V"], g["L"], g["rnd"])
    got = run_gpu(op, *args)
    for prec in (32, 64):
        ref = tuple(g[f"op{op}_ref{prec}_{k}"] for k in ("value", "dir", "pdf", "lobe"))
        print(check(op, got, ref, g[f"op{op}_tol"], f"device vs reference source FP{prec}"))


@pytest.mark.parametrize("op", [0, 1, 2])
def test_bsdf_close_to_fp64_oracle(agb, oracle, op):
    """Device against the FP64 oracle on 50K seeded cases, with the per-case conditioning
    tolerance of tests/bsdf_cases.py computed from the oracle's own FP32 and FP64 builds."""
    m, idx, frames, V, L, rnd = make_cases(50_000, 99 + op)
    got = run_gpu(op, m, idx, frames, V, L, rnd)
    _, r64, tol = tolerances(oracle.bsdf_batch, op, m, idx, frames, V, L, rnd)
    print(check(op, got, r64, tol, "device vs FP64 oracle"))


def test_random_stream_matches_reference_source(agb):
    """PCG2D streams (Random.slang:96-146) against the reference source's (fixture)."""
    from aurora_gb300 import api
    from test_reference_pin import golden
    g, _ = golden()
    for args, want in zip(g["random_args"], g["random_streams"]):
        out = empty((16, 2), torch.float32)
        api.random_stream(*[int(a) for a in args], 16, out.data_ptr())
        np.testing.assert_array_equal(host(out), want)


def test_environment_sampling_matches_reference_source(agb):
    """sampleEnvironment (Environment.slang:137-186) on the device against the reference source's
    (fixture): identical texel radiance and pdf, direction within two FP32 ulps."""
    from aurora_gb300 import _abi, api, scenes
    from test_reference_pin import golden
    g, _ = golden()
    img = g["env_image"]
    s = scenes.SceneDesc("env")
    k = s.add_image(img, _abi.FORMAT_RGB32F)
    s.env_light = s.env_background = k
    s.materials = scenes.materials(1)
    s.width = s.height = 4
    s.frame = scenes.frame_data(np.eye(4), scenes.perspective(45, 1))
    rnd = g["env_rnd"]
    n = len(rnd)
    with api.Renderer() as r:
        r.upload(s)
        table, integral = r.environment_alias()
        np.testing.assert_array_equal(table.view(np.uint8), g["env_alias"])
        d_rnd = dev(rnd)
        out_r, out_d, out_p = empty((n, 3), torch.float32), empty((n, 3), torch.float32), \
            empty((n,), torch.float32)
        r.env_sample(d_rnd.data_ptr(), n, out_r.data_ptr(), out_d.data_ptr(), out_p.data_ptr())
        gr, gd, gp = host(out_r), host(out_d), host(out_p)
    np.testing.assert_array_equal(gr, g["env_radiance"])
    np.testing.assert_array_equal(gp, g["env_pdf"])
    assert np.abs(gd - g["env_dir"]).max() <= 2.4e-7
