"""Oracle (test infrastructure, never imported by the product): the denoiser's mathematics in numpy
float64, the checker of the tensor-core kernels.

The reference has no learned denoiser (it ships NVIDIA NRD behind DirectX), so there is no
reference output to pin this against: it is the definition of the network the product implements
- 3x3 "same" convolutions in NHWC with weights w[tap][cin][cout] (tap = 3 (dy + 1) + (dx + 1)),
2x2 average pooling, nearest 2x upsampling, channel concatenation, ReLU, an L1 loss and Adam - and
its gradients.  Activations can be rounded to BF16 (round to nearest even) where the device stores
them, so that device and oracle see the same operands.
"""
import numpy as np


def bf16(x):
    """Rounds float values to BF16 (nearest even) and returns them as float64."""
    f = np.ascontiguousarray(x, np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint32) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def bf16_bits(x):
    f = np.ascontiguousarray(x, np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    return ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint16)


def from_bits(b):
    return (np.asarray(b, np.uint16).astype(np.uint32) << 16).view(np.float32).astype(np.float64)


TAPS = [(t // 3 - 1, t % 3 - 1) for t in range(9)]


def conv3x3(x, w, bias=None):
    """x (B, H, W, Cin), w (9, Cin, Cout) -> (B, H, W, Cout), zero padding."""
    B, H, W, _ = x.shape
    xp = np.pad(x, ((0, 0), (1, 1), (1, 1), (0, 0)))
    y = np.zeros((B, H, W, w.shape[2]))
    for t, (dy, dx) in enumerate(TAPS):
        y += xp[:, 1 + dy:1 + dy + H, 1 + dx:1 + dx + W, :] @ w[t]
    if bias is not None:
        y += bias
    return y


def conv3x3_data_grad(dy, w):
    """dX of conv3x3 for upstream gradient dy (B, H, W, Cout)."""
    B, H, W, _ = dy.shape
    dp = np.pad(dy, ((0, 0), (1, 1), (1, 1), (0, 0)))
    dx = np.zeros((B, H, W, w.shape[1]))
    for t, (oy, ox) in enumerate(TAPS):
        # y[p] += x[p + d] w[t]  =>  dx[q] += dy[q - d] w[t]^T
        dx += dp[:, 1 - oy:1 - oy + H, 1 - ox:1 - ox + W, :] @ w[t].T
    return dx


def conv3x3_weight_grad(x, dy):
    """(dW (9, Cin, Cout), db (Cout,)) of conv3x3."""
    B, H, W, Cin = x.shape
    xp = np.pad(x, ((0, 0), (1, 1), (1, 1), (0, 0)))
    dw = np.zeros((9, Cin, dy.shape[3]))
    flat = dy.reshape(-1, dy.shape[3])
    for t, (oy, ox) in enumerate(TAPS):
        dw[t] = xp[:, 1 + oy:1 + oy + H, 1 + ox:1 + ox + W, :].reshape(-1, Cin).T @ flat
    return dw, flat.sum(axis=0)


def upsample2(x):
    return x.repeat(2, axis=1).repeat(2, axis=2)


def upsample2_grad(d):
    B, H, W, C = d.shape
    return d.reshape(B, H // 2, 2, W // 2, 2, C).sum(axis=(2, 4))


def avgpool2(x):
    B, H, W, C = x.shape
    return x.reshape(B, H // 2, 2, W // 2, 2, C).mean(axis=(2, 4))


def avgpool2_grad(d):
    return upsample2(d) * 0.25
