"""Standard Surface evaluate / sample / evaluate-with-pdf on the GPU against the FP32 oracle
(StandardSurfaceBSDF.slang:598-1372): values and pdfs within 1e-5 relative, identical lobes."""
import numpy as np
import pytest
import torch

from gpu_util import dev, empty, host, rel_err

pytestmark = pytest.mark.gpu

TOL = 1e-5


def make_cases(n, seed):
    from aurora_gb300 import scenes
    rng = np.random.default_rng(seed)
    nm = 64
    m = scenes.materials(nm)
    m["base"] = rng.uniform(0.2, 1.0, nm)
    m["base_color"] = rng.uniform(0.0, 1.0, (nm, 3))
    m["diffuse_roughness"] = np.where(rng.uniform(size=nm) < 0.3, rng.uniform(0, 1, nm), 0)
    m["metalness"] = rng.choice([0.0, 1.0, 0.5], nm)
    m["specular"] = rng.uniform(0.0, 1.0, nm)
    m["specular_color"] = rng.uniform(0.5, 1.0, (nm, 3))
    m["specular_roughness"] = rng.uniform(0.02, 1.0, nm)
    m["specular_IOR"] = rng.uniform(1.1, 2.5, nm)
    m["specular_anisotropy"] = np.where(rng.uniform(size=nm) < 0.3, rng.uniform(0, 1, nm), 0)
    m["specular_rotation"] = np.where(rng.uniform(size=nm) < 0.3, rng.uniform(0, 1, nm), 0)
    m["transmission"] = np.where(rng.uniform(size=nm) < 0.25, rng.uniform(0.2, 1, nm), 0)
    m["transmission_color"] = rng.uniform(0.5, 1.0, (nm, 3))
    m["thin_walled"] = (rng.uniform(size=nm) < 0.2).astype(np.int32)
    m["subsurface"] = np.where(rng.uniform(size=nm) < 0.25, rng.uniform(0.1, 1, nm), 0)
    m["subsurface_color"] = rng.uniform(0.2, 1.0, (nm, 3))
    m["sheen"] = np.where(rng.uniform(size=nm) < 0.3, rng.uniform(0.1, 1, nm), 0)
    m["sheen_roughness"] = rng.uniform(0.05, 1.0, nm)
    m["coat"] = np.where(rng.uniform(size=nm) < 0.5, rng.uniform(0.1, 1, nm), 0)
    m["coat_color"] = rng.uniform(0.5, 1.0, (nm, 3))
    m["coat_roughness"] = rng.uniform(0.02, 1.0, nm)
    m["coat_IOR"] = rng.uniform(1.2, 2.0, nm)
    m["coat_affect_color"] = np.where(rng.uniform(size=nm) < 0.3, rng.uniform(0, 1, nm), 0)
    m["coat_affect_roughness"] = np.where(rng.uniform(size=nm) < 0.3, rng.uniform(0, 1, nm), 0)
    idx = rng.integers(0, nm, n).astype(np.int32)
    N = rng.normal(size=(n, 3))
    N /= np.linalg.norm(N, axis=1, keepdims=True)
    up = np.where(np.abs(N[:, 1:2]) < 0.999, [[0, 1, 0]], [[1, 0, 0]])
    X = np.cross(N, up)
    X /= np.linalg.norm(X, axis=1, keepdims=True)
    Y = np.cross(N, X)
    frames = np.zeros((n, 12), np.float32)
    frames[:, 0:3], frames[:, 3:6], frames[:, 6:9] = N, X, Y
    V = rng.normal(size=(n, 3))
    V /= np.linalg.norm(V, axis=1, keepdims=True)
    # Mostly upper hemisphere, some lower (back faces, transmission).
    flip = (np.einsum("ij,ij->i", V, N) < 0) & (rng.uniform(size=n) < 0.8)
    V[flip] *= -1
    L = rng.normal(size=(n, 3))
    L /= np.linalg.norm(L, axis=1, keepdims=True)
    rnd = rng.uniform(size=(n, 2)).astype(np.float32)
    return m, idx, frames, V.astype(np.float32), L.astype(np.float32), rnd


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
    m, idx, frames, V, L, rnd = make_cases(200_000, 11 + op)
    gv, gd, gp, gl = run_gpu(op, m, idx, frames, V, L, rnd)
    ov, od, op_, ol = oracle.bsdf_batch(op, m, idx, frames, V, L, rnd, precision=32)
    fin = np.isfinite(ov).all(1) & np.isfinite(gv).all(1)
    assert fin.mean() > 0.999
    if op > 0:
        same_lobe = gl == ol
        assert same_lobe.mean() > 0.9999, f"lobe agreement {same_lobe.mean()}"
    else:
        same_lobe = np.ones(len(idx), bool)
    sel = fin & same_lobe
    scale = np.maximum(np.abs(ov[sel]).max(axis=1, keepdims=True), 1e-30)
    err = rel_err(gv[sel], ov[sel], 1e-6 * scale)
    frac = (err <= TOL).all(axis=1).mean()
    print(f"op {op}: {frac:.6f} within {TOL} relative; max {err.max():.3g}")
    assert frac >= 0.999, f"only {frac} of BSDF values within {TOL}"
    if op > 0:
        ep = rel_err(gp[sel], op_[sel], 1e-6)
        fp = (ep <= TOL).mean()
        print(f"pdf: {fp:.6f} within {TOL}; max {ep.max():.3g}")
        assert fp >= 0.999
    if op == 1:
        dd = np.abs(gd[sel] - od[sel]).max(axis=1)
        assert (dd <= TOL).mean() >= 0.999


def test_bsdf_fp32_close_to_fp64_oracle(agb, oracle):
    """The device FP32 results against the FP64 oracle: a looser, accuracy-only check."""
    m, idx, frames, V, L, rnd = make_cases(50_000, 99)
    gv = run_gpu(0, m, idx, frames, V, L, rnd)[0]
    ov = oracle.bsdf_batch(0, m, idx, frames, V, L, rnd, precision=64)[0]
    scale = np.maximum(np.abs(ov).max(axis=1, keepdims=True), 1e-30)
    err = rel_err(gv, ov, 1e-6 * scale)
    assert (err <= 1e-3).all(axis=1).mean() > 0.999
