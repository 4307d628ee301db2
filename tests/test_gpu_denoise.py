"""Denoiser kernels on the tensor cores against the numpy oracle (oracle/denoise_ref.py), on BF16
operands: the 3x3 convolution (with the decoder's fused nearest-upsample + skip concatenation,
bias, ReLU) and its data-gradient form.  The kernels accumulate in FP32, so their FP32 outputs
must match the FP64 oracle within 1e-5 of sum |x w| per output."""
import numpy as np
import pytest

import denoise_ref as ref

pytestmark = pytest.mark.gpu


def to_dev(bits):
    import torch
    return torch.from_numpy(np.ascontiguousarray(bits).view(np.int16)).cuda()


def run_conv(agb, x0, x1, w, bias, B, H, W, up0, relu, flip=False):
    """Device conv: x0 / x1 BF16 bit arrays, w FP32 (9, Cin, Cout) of the layer."""
    import torch
    from aurora_gb300 import _abi
    cin, cout = w.shape[1], w.shape[2]
    kc0 = x0.shape[-1]
    kc1 = 0 if x1 is None else x1.shape[-1]
    kcout = cin if flip else cout
    wd = torch.from_numpy(np.ascontiguousarray(w, np.float32)).cuda()
    wp = torch.zeros(9 * cin * cout, dtype=torch.int16, device="cuda")
    _abi.check(agb.agb_pack_conv_weights(wd.data_ptr(), cin, cout, 1 if flip else 0, wp.data_ptr(), None))
    d0 = to_dev(x0)
    d1 = to_dev(x1) if x1 is not None else None
    bd = torch.from_numpy(np.asarray(bias, np.float32)).cuda() if bias is not None else None
    out32 = torch.zeros((B, H, W, kcout), dtype=torch.float32, device="cuda")
    out16 = torch.zeros((B, H, W, kcout), dtype=torch.int16, device="cuda")
    _abi.check(agb.agb_conv3x3_bf16(d0.data_ptr(), d1.data_ptr() if d1 is not None else None,
                                    wp.data_ptr(), bd.data_ptr() if bd is not None else None,
                                    out16.data_ptr(), out32.data_ptr(), B, H, W, kc0, kc1, kcout,
                                    1 if up0 else 0, 1 if relu else 0, None))
    return out32.cpu().numpy().astype(np.float64), out16.cpu().numpy().view(np.uint16)


CASES = [
    # B, H, W, C0, C1, Cout, up0, relu
    (2, 16, 24, 16, 0, 32, False, True),
    (1, 8, 8, 32, 16, 48, True, True),
    (1, 12, 20, 128, 0, 256, False, False),
    (3, 10, 14, 64, 64, 64, True, True),
    # edges: one row of two pixels, an odd height (a partial row tile), the smallest upsampled
    # input (1 x 1 at half resolution), a width over three 256-pixel tiles with two channel tiles
    (3, 1, 2, 16, 0, 32, False, True),
    (1, 5, 6, 32, 16, 48, False, False),
    (2, 2, 2, 16, 16, 16, True, True),
    (1, 3, 520, 64, 0, 128, False, True),
]


@pytest.mark.parametrize("case", CASES)
def test_conv3x3_matches_oracle(agb, case):
    B, H, W, C0, C1, Cout, up0, relu = case
    rng = np.random.default_rng(sum(case[:6]))
    h0, w0 = (H // 2, W // 2) if up0 else (H, W)
    x0 = ref.bf16_bits(rng.normal(0, 1, (B, h0, w0, C0)))
    x1 = ref.bf16_bits(rng.normal(0, 1, (B, H, W, C1))) if C1 else None
    w = ref.bf16(rng.normal(0, 0.2, (9, C0 + C1, Cout)))   # exact in BF16: packing is lossless
    bias = rng.normal(0, 0.1, Cout)
    g32, g16 = run_conv(agb, x0, x1, w, bias, B, H, W, up0, relu)
    xin = ref.from_bits(x0)
    if up0:
        xin = ref.upsample2(xin)
    if C1:
        xin = np.concatenate([xin, ref.from_bits(x1)], axis=3)
    want = ref.conv3x3(xin, w, bias)
    scale = ref.conv3x3(np.abs(xin), np.abs(w), np.abs(bias)) + 1e-30
    if relu:
        want = np.maximum(want, 0.0)
    err = np.abs(g32 - want) / scale
    print(f"conv {case}: max err / sum|xw| = {err.max():.3g}")
    assert err.max() < 1e-5
    # The BF16 output is the FP32 result rounded to nearest even.
    np.testing.assert_array_equal(g16, ref.bf16_bits(g32))


POOL_CASES = [
    # B, H, W, C0, C1, Cout, up0, relu: the encoder's pooled layers (32, 64, 128 channels), a
    # decoder-shaped input, and a width spanning two 256-pixel tiles
    (2, 16, 24, 16, 0, 32, False, True),
    (1, 8, 12, 64, 0, 64, False, True),
    (1, 6, 10, 128, 0, 128, False, True),
    (2, 12, 20, 32, 32, 64, True, True),
    (1, 4, 600, 16, 0, 32, False, False),
]


@pytest.mark.parametrize("case", POOL_CASES)
def test_conv3x3_fused_pool_matches_oracle(agb, case):
    """The 2x2 average pool in the convolution's epilogue equals a pool over the stored BF16
    outputs, bit for bit, and the convolution itself stays within the oracle's bound."""
    import torch
    from aurora_gb300 import _abi
    B, H, W, C0, C1, Cout, up0, relu = case
    rng = np.random.default_rng(sum(case[:6]) + 11)
    h0, w0 = (H // 2, W // 2) if up0 else (H, W)
    x0 = ref.bf16_bits(rng.normal(0, 1, (B, h0, w0, C0)))
    x1 = ref.bf16_bits(rng.normal(0, 1, (B, H, W, C1))) if C1 else None
    w = ref.bf16(rng.normal(0, 0.2, (9, C0 + C1, Cout)))
    bias = rng.normal(0, 0.1, Cout)
    wd = torch.from_numpy(np.ascontiguousarray(w, np.float32)).cuda()
    wp = torch.zeros(9 * (C0 + C1) * Cout, dtype=torch.int16, device="cuda")
    _abi.check(agb.agb_pack_conv_weights(wd.data_ptr(), C0 + C1, Cout, 0, wp.data_ptr(), None))
    d0 = to_dev(x0)
    d1 = to_dev(x1) if x1 is not None else None
    bd = torch.from_numpy(np.asarray(bias, np.float32)).cuda()
    out16 = torch.zeros((B, H, W, Cout), dtype=torch.int16, device="cuda")
    pool16 = torch.zeros((B, H // 2, W // 2, Cout), dtype=torch.int16, device="cuda")
    _abi.check(agb.agb_conv3x3_pool_bf16(d0.data_ptr(), d1.data_ptr() if d1 is not None else None,
                                         wp.data_ptr(), bd.data_ptr(), out16.data_ptr(),
                                         pool16.data_ptr(), B, H, W, C0, C1, Cout,
                                         1 if up0 else 0, 1 if relu else 0, None))
    o16 = out16.cpu().numpy().view(np.uint16)
    p16 = pool16.cpu().numpy().view(np.uint16)
    xin = ref.from_bits(x0)
    if up0:
        xin = ref.upsample2(xin)
    if C1:
        xin = np.concatenate([xin, ref.from_bits(x1)], axis=3)
    want = ref.conv3x3(xin, w, bias)
    if relu:
        want = np.maximum(want, 0.0)
    scale = ref.conv3x3(np.abs(xin), np.abs(w), np.abs(bias)) + 1e-30
    # BF16 outputs: within half a BF16 ulp (2^-8 relative) of the bound-respecting FP32 result.
    err = np.abs(ref.from_bits(o16) - want) / (scale + np.abs(want))
    assert err.max() < 2 ** -8 + 1e-5
    # The pool over the stored outputs in FP32, in the order ((x00 + x01) + x10) + x11.
    o = ref.from_bits(o16).astype(np.float32).reshape(B, H // 2, 2, W // 2, 2, Cout)
    s = ((o[:, :, 0, :, 0] + o[:, :, 0, :, 1]) + o[:, :, 1, :, 0]) + o[:, :, 1, :, 1]
    np.testing.assert_array_equal(p16, ref.bf16_bits(s * np.float32(0.25)))


@pytest.mark.parametrize("case", [(2, 16, 24, 32, 16), (1, 8, 12, 256, 128), (1, 6, 10, 48, 96)])
def test_conv3x3_data_gradient_matches_oracle(agb, case):
    B, H, W, Cin, Cout = case
    rng = np.random.default_rng(sum(case))
    w = ref.bf16(rng.normal(0, 0.2, (9, Cin, Cout)))
    dy = ref.bf16_bits(rng.normal(0, 1, (B, H, W, Cout)))
    g32, _ = run_conv(agb, dy, None, w, None, B, H, W, False, False, flip=True)
    want = ref.conv3x3_data_grad(ref.from_bits(dy), w)
    scale = ref.conv3x3_data_grad(np.abs(ref.from_bits(dy)), np.abs(w)) + 1e-30
    err = np.abs(g32 - want) / scale
    print(f"data grad {case}: max err / sum|dy w| = {err.max():.3g}")
    assert err.max() < 1e-5


def test_conv3x3_output_tiles_match_oracle(agb):
    """Cout above the 256 accumulator columns of one MMA tile runs as tiles of 128 channels."""
    rng = np.random.default_rng(7)
    B, H, W, C0, Cout = 1, 8, 12, 32, 384
    x0 = ref.bf16_bits(rng.normal(0, 1, (B, H, W, C0)))
    w = ref.bf16(rng.normal(0, 0.2, (9, C0, Cout)))
    bias = rng.normal(0, 0.1, Cout)
    g32, _ = run_conv(agb, x0, None, w, bias, B, H, W, False, False)
    xin = ref.from_bits(x0)
    want = ref.conv3x3(xin, w, bias)
    err = np.abs(g32 - want) / (ref.conv3x3(np.abs(xin), np.abs(w), np.abs(bias)) + 1e-30)
    assert err.max() < 1e-5
    # Data gradient of a layer with 384 input channels (the first decoder layer).
    dy = ref.bf16_bits(rng.normal(0, 1, (B, H, W, 128)))
    w2 = ref.bf16(rng.normal(0, 0.2, (9, 384, 128)))
    d32, _ = run_conv(agb, dy, None, w2, None, B, H, W, False, False, flip=True)
    want = ref.conv3x3_data_grad(ref.from_bits(dy), w2)
    err = np.abs(d32 - want) / (ref.conv3x3_data_grad(np.abs(ref.from_bits(dy)), np.abs(w2)) + 1e-30)
    print("384-channel tiles: max err", err.max())
    assert err.max() < 1e-5


WGRAD_CASES = [
    # B, H, W, C0, C1, Cout, up0
    (2, 16, 24, 16, 0, 32, False),
    (1, 8, 8, 32, 16, 48, True),
    (1, 10, 12, 256, 128, 128, True),
    (3, 9, 14, 64, 0, 256, False),
    # edges: two-pixel rows, a width over three 128-pixel units with an upsampled input
    (2, 3, 2, 16, 0, 16, False),
    (1, 4, 260, 32, 32, 64, True),
]


@pytest.mark.parametrize("case", WGRAD_CASES)
def test_conv3x3_weight_gradient_matches_oracle(agb, case):
    import torch
    from aurora_gb300 import _abi
    B, H, W, C0, C1, Cout, up0 = case
    rng = np.random.default_rng(sum(case[:6]) + 1)
    h0, w0 = (H // 2, W // 2) if up0 else (H, W)
    x0 = ref.bf16_bits(rng.normal(0, 1, (B, h0, w0, C0)))
    x1 = ref.bf16_bits(rng.normal(0, 1, (B, H, W, C1))) if C1 else None
    dy = ref.bf16_bits(rng.normal(0, 1, (B, H, W, Cout)))
    dw = torch.full((9, C0 + C1, Cout), 0.5, dtype=torch.float32, device="cuda")
    d0, d1, dd = to_dev(x0), (to_dev(x1) if C1 else None), to_dev(dy)
    _abi.check(agb.agb_conv3x3_wgrad_bf16(d0.data_ptr(), d1.data_ptr() if d1 is not None else None,
                                          dd.data_ptr(), dw.data_ptr(), B, H, W, C0, C1, Cout,
                                          1 if up0 else 0, None))
    g = dw.cpu().numpy().astype(np.float64) - 0.5
    xin = ref.from_bits(x0)
    if up0:
        xin = ref.upsample2(xin)
    if C1:
        xin = np.concatenate([xin, ref.from_bits(x1)], axis=3)
    want, _ = ref.conv3x3_weight_grad(xin, ref.from_bits(dy))
    scale, _ = ref.conv3x3_weight_grad(np.abs(xin), np.abs(ref.from_bits(dy)))
    err = np.abs(g - want) / (scale + 1e-30)
    print(f"wgrad {case}: max err / sum|x dy| = {err.max():.3g}")
    assert err.max() < 1e-5
