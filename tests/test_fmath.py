"""Accuracy of the single-precision transcendentals shared by the device code and the FP32 oracle
(aurora_gb300/csrc/agb_fmath.h) against double-precision libm."""
import numpy as np


def ulp_err(got, ref):
    got = got.astype(np.float64)
    ulp = np.spacing(np.abs(ref).astype(np.float32)).astype(np.float64)
    return np.abs(got - ref) / np.maximum(ulp, np.spacing(np.float32(1e-30)))


def test_sin_cos(oracle):
    x = np.concatenate([np.linspace(-10, 10, 200_001), [0.0, -0.0, 1e-30, np.pi / 4, np.pi]]).astype(np.float32)
    xd = x.astype(np.float64)
    s, c = oracle.fmath(0, x), oracle.fmath(1, x)
    # Absolute error relative to the unit circle: a few float ulps of 1.
    assert np.abs(s - np.sin(xd)).max() < 3e-7
    assert np.abs(c - np.cos(xd)).max() < 3e-7
    assert s[-5] == 0.0 and c[-5] == 1.0


def test_exp2_log2_pow(oracle):
    rng = np.random.default_rng(0)
    x = rng.uniform(-60, 60, 100_000).astype(np.float32)
    assert np.percentile(ulp_err(oracle.fmath(2, x), np.exp2(x.astype(np.float64))), 99.9) <= 4
    assert ulp_err(oracle.fmath(2, x), np.exp2(x.astype(np.float64))).max() <= 8
    y = np.exp(rng.uniform(-60, 60, 100_000)).astype(np.float32)
    l2 = oracle.fmath(3, y)
    assert np.abs(l2 - np.log2(y.astype(np.float64))).max() < 1e-5
    b = rng.uniform(0, 1, 100_000).astype(np.float32)
    e = rng.uniform(0.5, 40, 100_000).astype(np.float32)
    p = oracle.fmath(4, b, e)
    ref = np.power(b.astype(np.float64), e.astype(np.float64))
    ok = ref > 1e-30
    assert (np.abs(p[ok] - ref[ok]) / ref[ok]).max() < 2e-5
    assert oracle.fmath(4, np.float32([0.3, 0.0, 2.0]), np.float32([1.0, 2.0, 0.0])).tolist() == \
        [np.float32(0.3), 0.0, 1.0]
    assert np.isnan(oracle.fmath(4, np.float32([-0.5]), np.float32([2.0])))[0]


def test_atan2_asin(oracle):
    rng = np.random.default_rng(1)
    y = rng.normal(size=100_000).astype(np.float32)
    x = rng.normal(size=100_000).astype(np.float32)
    assert np.abs(oracle.fmath(5, y, x) - np.arctan2(y.astype(np.float64), x.astype(np.float64))).max() < 5e-7
    s = rng.uniform(-1, 1, 100_000).astype(np.float32)
    s[:3] = [1.0, -1.0, 0.0]
    assert np.abs(oracle.fmath(6, s) - np.arcsin(s.astype(np.float64))).max() < 1e-6
    edge = oracle.fmath(5, np.float32([0.0, -0.0, 1.0, 0.0]), np.float32([-1.0, -1.0, 0.0, 1.0]))
    np.testing.assert_allclose(edge, [np.pi, -np.pi, np.pi / 2, 0.0], rtol=1e-7)
