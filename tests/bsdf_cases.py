"""Seeded Standard Surface BSDF cases shared by the oracle pins, the fixture generator and the GPU
tests, and the per-case tolerance those comparisons use.

Tolerance (against the reference's shader source compiled as host C++, oracle/ref_shim): a
result must agree with the reference's FP32 result within

    max(1e-5, 16 x cond, 4 x own)

normwise: the largest component difference over the reference's largest component (a BSDF value
is a colour; a direction, a unit vector, is compared absolutely; a pdf relatively), where `cond` is the largest relative change of the reference's FP64 result when every input (the
material's floats, the shading frame, V, L and the random pair) is perturbed by up to one FP32 ulp
(eight seeded draws), and `own` is the reference FP32 build's own error against its FP64 build.
On well-conditioned cases this is the 1e-5 bar: evaluateMaterial and evaluateMaterialAndPDF meet
it on every seeded case; sampleMaterial on about 99.7 % of them, the rest being samples whose FP32
evaluation is itself ill-conditioned (a sampled direction whose GGX density or Fresnel term
amplifies last-ulp differences of sqrt / sin / cos), where two correct FP32 implementations differ
by more and the bar follows the reference's own FP32 behaviour.  Lobe choices must agree on every
case.
"""
import numpy as np


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


TOL = 1e-5


def rel(a, b, scale):
    """Normwise relative error per case: max over components of |a - b|, over the case's scale
    (the largest component magnitude of the reference; 1-D inputs: the value's own magnitude)."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    if a.ndim == 1:
        return np.abs(a - b) / np.maximum(np.maximum(np.abs(a), np.abs(b)), 1e-30)
    return (np.abs(a - b) / np.maximum(scale, 1e-30)).max(axis=1)


def _perturb(a, rng):
    a = np.asarray(a, np.float64)
    return (a * (1.0 + 2.0 ** -23 * rng.uniform(-1, 1, a.shape))).astype(np.float32)


def _perturb_materials(m, rng):
    out = m.copy()
    for name in m.dtype.names:
        if m.dtype[name].base == np.float32 and not name.startswith("_"):
            out[name] = _perturb(m[name], rng)
    return out


def tolerances(ref_batch, op, m, idx, frames, V, L, rnd, draws=8, seed=5):
    """Per-case tolerances (value, direction, pdf) for operation `op`, from the reference's FP32 and
    FP64 builds (ref_batch(op, m, idx, frames, V, L, rnd, precision=...))."""
    r32 = ref_batch(op, m, idx, frames, V, L, rnd, precision=32)
    r64 = ref_batch(op, m, idx, frames, V, L, rnd, precision=64)
    scale = np.maximum(np.abs(r64[0]).max(axis=1, keepdims=True), 1e-30)
    rng = np.random.default_rng(seed)
    cond = np.zeros((3, len(idx)))
    for _ in range(draws):
        p = ref_batch(op, _perturb_materials(m, rng), idx, _perturb(frames, rng), _perturb(V, rng),
                      _perturb(L, rng), _perturb(rnd, rng), precision=64)
        cond[0] = np.maximum(cond[0], rel(p[0], r64[0], scale))
        cond[1] = np.maximum(cond[1], np.abs(p[1] - r64[1]).max(1))
        cond[2] = np.maximum(cond[2], rel(p[2], r64[2], None))
    own = np.stack([rel(r32[0], r64[0], scale), np.abs(r32[1] - r64[1]).max(1),
                    rel(r32[2], r64[2], None)])
    tol = np.maximum(TOL, np.maximum(16 * cond, 4 * own)).astype(np.float32)
    return r32, r64, tol


def check(op, got, ref, tol, label):
    """Asserts `got` (value, direction, pdf, lobe) against the reference results `ref` within the
    per-case tolerances; returns a summary line."""
    gv, gd, gp, gl = got
    rv, rd, rp, rl = ref
    scale = np.maximum(np.abs(rv).max(axis=1, keepdims=True), 1e-30)
    ev = rel(gv, rv, scale)
    plain = (ev <= TOL).mean()
    assert np.isfinite(gv).all(), f"{label}: non-finite values"
    assert (ev <= tol[0]).all(), f"{label}: {int((ev > tol[0]).sum())} values beyond tolerance, " \
        f"worst {ev.max():.3g}"
    line = f"{label} op {op}: values within 1e-5 {plain:.6f}, max {ev.max():.3g}"
    if op > 0:
        assert np.array_equal(gl, rl), f"{label}: {int((gl != rl).sum())} lobe choices differ"
        ep = rel(gp, rp, None)
        assert (ep <= tol[2]).all(), f"{label}: {int((ep > tol[2]).sum())} pdfs beyond tolerance"
        line += f"; pdfs within 1e-5 {(ep <= TOL).mean():.6f}, max {ep.max():.3g}"
    if op == 1:
        ed = np.abs(gd - rd).max(1)
        assert (ed <= tol[1]).all(), f"{label}: {int((ed > tol[1]).sum())} directions beyond tolerance"
        line += f"; directions within 1e-5 {(ed <= TOL).mean():.6f}"
    return line
