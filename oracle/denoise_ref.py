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


# ----------------------------------------------------------------------------- the U-Net
# Activations: name -> (level, channels); layers: (in0, in1, out, up0, relu, level) in parameter
# order, as the product's agb_unet.cu defines them.
ACTS = {"x": (0, 16), "e0a": (0, 32), "s0": (0, 32), "p0": (1, 32), "e1a": (1, 64), "s1": (1, 64),
        "p1": (2, 64), "e2a": (2, 128), "s2": (2, 128), "p2": (3, 128), "ba": (3, 256),
        "bb": (3, 256), "d2a": (2, 128), "d2": (2, 128), "d1a": (1, 64), "d1": (1, 64),
        "d0a": (0, 32), "d0": (0, 32)}
LAYERS = [("x", None, "e0a", 0, 1, 0), ("e0a", None, "s0", 0, 1, 0),
          ("p0", None, "e1a", 0, 1, 1), ("e1a", None, "s1", 0, 1, 1),
          ("p1", None, "e2a", 0, 1, 2), ("e2a", None, "s2", 0, 1, 2),
          ("p2", None, "ba", 0, 1, 3), ("ba", None, "bb", 0, 1, 3),
          ("bb", "s2", "d2a", 1, 1, 2), ("d2a", None, "d2", 0, 1, 2),
          ("d2", "s1", "d1a", 1, 1, 1), ("d1a", None, "d1", 0, 1, 1),
          ("d1", "s0", "d0a", 1, 1, 0), ("d0a", None, "d0", 0, 1, 0),
          ("d0", None, None, 0, 0, 0)]
POOLS = {2: ("s0", "p0"), 4: ("s1", "p1"), 6: ("s2", "p2")}


def layer_shapes():
    out = []
    for in0, in1, o, _, _, _ in LAYERS:
        cin = ACTS[in0][1] + (ACTS[in1][1] if in1 else 0)
        out.append((cin, ACTS[o][1] if o else 16))
    return out


def split_params(flat):
    """Flat parameter vector -> [(w (9, cin, cout), b (cout,))]."""
    res, off = [], 0
    for cin, cout in layer_shapes():
        w = flat[off:off + 9 * cin * cout].reshape(9, cin, cout)
        off += 9 * cin * cout
        b = flat[off:off + cout]
        off += cout
        res.append((np.asarray(w, np.float64), np.asarray(b, np.float64)))
    return res


def _layer_input(acts, in0, in1, up0):
    x = acts[in0]
    if up0:
        x = upsample2(x)
    if in1:
        x = np.concatenate([x, acts[in1]], axis=3)
    return x


def unet_forward(flat, x, exact=False):
    """x: (B, H, W, 16) BF16 values as float64.  Returns the activations (BF16-rounded where the
    device stores them, unless exact) and the output (B, H, W, 16)."""
    rnd = (lambda v: v) if exact else bf16
    params = split_params(flat)
    acts = {"x": x}
    out = None
    for i, (in0, in1, o, up0, relu, _) in enumerate(LAYERS):
        if i in POOLS:
            s, p = POOLS[i]
            acts[p] = rnd(avgpool2(acts[s]))
        w, b = params[i]
        y = conv3x3(_layer_input(acts, in0, in1, up0), bf16(w), b)
        if relu:
            y = np.maximum(y, 0.0)
        if o:
            acts[o] = rnd(y)
        else:
            out = y
    return acts, out


def unet_loss_backward(flat, acts, out, target, exact=False):
    """L1 loss on log1p radiance (prediction = out[..., :3] + x[..., :3]) and the parameter
    gradients (flat, same layout), with the device's BF16 rounding of the per-layer gradients
    (unless exact)."""
    rnd = (lambda v: v) if exact else bf16
    params = split_params(flat)
    x = acts["x"]
    B, H, W, _ = x.shape
    n = B * H * W * 3
    pred = out[..., :3] + x[..., :3]
    t = np.log1p(np.maximum(target[..., :3], 0.0))
    d = pred - t
    loss = np.abs(d).sum() / n
    g_out = np.zeros_like(out)
    g_out[..., :3] = np.sign(d) / n
    grads = {k: np.zeros_like(v) for k, v in acts.items() if k != "x"}
    flat_grads = []
    for i in range(len(LAYERS) - 1, -1, -1):
        in0, in1, o, up0, relu, _ = LAYERS[i]
        w, b = params[i]
        gy = grads[o] if o else g_out
        dpre = rnd(gy * (acts[o] > 0) if relu else gy)
        xin = _layer_input(acts, in0, in1, up0)
        dw, db = conv3x3_weight_grad(xin, dpre)
        flat_grads.append((i, dw, db))
        if i > 0:
            dx = conv3x3_data_grad(dpre, bf16(w))
            c0 = ACTS[in0][1]
            g0 = dx[..., :c0]
            grads[in0] += upsample2_grad(g0) if up0 else g0
            if in1:
                grads[in1] += dx[..., c0:]
        if i in POOLS:
            s, p = POOLS[i]
            grads[s] += avgpool2_grad(grads[p])
    flat_grads.sort(key=lambda t: t[0])
    g = np.concatenate([np.concatenate([dw.reshape(-1), db]) for _, dw, db in flat_grads])
    return loss, g
