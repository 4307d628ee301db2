"""The learned denoiser end to end on the tensor cores: forward output, L1 loss and every layer's
parameter gradients against the numpy oracle (oracle/denoise_ref.py, which emulates the device's
BF16 storage points), then training on the renderer's own low / high sample-count pairs and what
the trained network gains over plain accumulation on a view it was not trained on."""
import ctypes

import numpy as np
import pytest

import denoise_ref as ref

pytestmark = pytest.mark.gpu


def denoiser(agb, seed=3):
    from aurora_gb300 import _abi
    h = ctypes.c_void_p()
    _abi.check(agb.agb_denoiser_create(0, None, seed, ctypes.byref(h)))
    return h


def param_count(agb):
    n = ctypes.c_uint64()
    agb.agb_denoiser_param_count(ctypes.byref(n))
    return n.value


def random_features(rng, B, H, W):
    f = np.zeros((B, H, W, 16), np.float32)
    f[..., 0:3] = rng.uniform(0, 2, (B, H, W, 3))
    f[..., 3:6] = rng.uniform(0, 1, (B, H, W, 3))
    f[..., 6:8] = rng.uniform(-1, 1, (B, H, W, 2))
    f[..., 8:10] = rng.uniform(0, 1, (B, H, W, 2))
    return ref.bf16_bits(f)


def test_unet_forward_loss_and_gradients_match_oracle(agb):
    import torch
    from aurora_gb300 import _abi
    rng = np.random.default_rng(5)
    B, H, W = 2, 32, 48
    xb = random_features(rng, B, H, W)
    x = ref.from_bits(xb)
    dn = denoiser(agb)
    try:
        n = param_count(agb)
        params = np.zeros(n, np.float32)
        _abi.check(agb.agb_denoiser_params(dn, params.ctypes.data, n))
        # Targets 0.2 away from the prediction in log space: the L1 gradient's sign is then the
        # same on both sides (near the target, rounding differences would flip it).
        acts, o = ref.unet_forward(params.astype(np.float64), x)
        pred = o[..., :3] + x[..., :3]
        step = np.where((pred > 0.3) & (rng.uniform(size=pred.shape) < 0.5), -0.2, 0.2)
        target = np.ones((B, H, W, 4), np.float32)
        target[..., :3] = np.expm1(pred + step)
        xd = torch.from_numpy(xb.view(np.int16)).cuda()
        td = torch.from_numpy(target).cuda()
        loss = ctypes.c_float()
        _abi.check(agb.agb_denoiser_train_step(dn, xd.data_ptr(), td.data_ptr(), B, H, W, 0.0, 0,
                                               ctypes.byref(loss)))
        grads = np.zeros(n, np.float32)
        _abi.check(agb.agb_denoiser_grads(dn, grads.ctypes.data, n))
        out = torch.zeros((B, H, W, 4), dtype=torch.float32, device="cuda")
        _abi.check(agb.agb_denoiser_forward(dn, xd.data_ptr(), B, H, W, out.data_ptr()))
        rad = out.cpu().numpy()
    finally:
        agb.agb_denoiser_destroy(dn)
    loss_ref, g_ref = ref.unet_loss_backward(params.astype(np.float64), acts, o, target)
    # The same network without any BF16 rounding of activations or gradients: how far BF16 storage
    # itself moves the gradients (the envelope the device must stay within).
    acts64, o64 = ref.unet_forward(params.astype(np.float64), x, exact=True)
    _, g_exact = ref.unet_loss_backward(params.astype(np.float64), acts64, o64, target, exact=True)
    print(f"loss device {loss.value:.6f} oracle {loss_ref:.6f}")
    assert abs(loss.value - loss_ref) < 1e-3 * loss_ref
    rad_ref = np.maximum(np.expm1(o[..., :3] + x[..., :3]), 0.0)
    # The network predicts log1p(radiance): compare there (absolute).  Activations are stored in
    # BF16 (8-bit mantissa): where FP32 and FP64 accumulation round an activation to neighbouring
    # BF16 values, the difference carries through the later layers.
    err = np.abs(np.log1p(rad[..., :3]) - np.log1p(rad_ref))
    print("log1p radiance: max abs err", err.max(), "median", np.median(err), "99.9%",
          np.quantile(err, 0.999))
    assert np.median(err) < 5e-4 and np.quantile(err, 0.999) < 1e-2 and err.max() < 5e-2
    # Per layer: relative L2 distance of the device's weight and bias gradients to the oracle's
    # (same BF16 storage points) and to the exact FP64 gradients, beside the distance between the
    # two oracles (the BF16 envelope).  Rounding the per-layer gradients and activations to BF16
    # compounds through the backward pass toward the bottleneck; the device must be no farther
    # from the exact gradients than the BF16-emulating oracle is, and close to that oracle.
    rel = lambda a, b: np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-12)
    off = 0
    for i, (cin, cout) in enumerate(ref.layer_shapes()):
        for name, size in (("w", 9 * cin * cout), ("b", cout)):
            g = grads[off:off + size].astype(np.float64)
            gr, ge = g_ref[off:off + size], g_exact[off:off + size]
            d_ref, d_exact, envelope = rel(g, gr), rel(g, ge), rel(gr, ge)
            print(f"layer {i:2d} {name}: |g| {np.linalg.norm(ge):.3e} vs BF16 oracle {d_ref:.2e} "
                  f"vs exact {d_exact:.2e} envelope {envelope:.2e}")
            assert d_exact < 1.5 * envelope + 2e-3, (i, name, d_exact, envelope)
            assert d_ref < 2.0 * envelope + 2e-3, (i, name, d_ref, envelope)
            off += size
    assert off == n


def render_pair(r, s, k, spp_lo, spp_hi):
    """Features of a spp_lo render and the spp_hi reference (Kahan mean) of view k."""
    import torch
    from aurora_gb300 import _abi, scenes
    m = np.asarray(s.frame["camera_inv_view"], np.float64).reshape(-1)
    a = 0.11 * k
    x, y, z = m[3], m[7], m[11]
    eye = (x * np.cos(a) + z * np.sin(a), y * (1.0 + 0.05 * np.sin(k)), -x * np.sin(a) + z * np.cos(a))
    f = scenes.frame_data(scenes.look_at(eye, (0.0, 0.0, 0.0)),
                          scenes.perspective(45.0, s.width / s.height), trace_depth=5,
                          scene_bounds=s.bounds(), aovs=True)
    r.set_frame(f)
    r.render(0, spp_lo, accumulation=_abi.ACCUM_RUNNING_MEAN | _abi.ACCUM_MOMENTS,
             seed_offset=1000 * k + 1)
    feat = torch.zeros((s.height, s.width, 16), dtype=torch.int16, device="cuda")
    _abi.check(_abi.library().agb_denoiser_features(r.ctx, feat.data_ptr()))
    noisy = r.read(_abi.ACCUM_RUNNING_MEAN).copy()
    r.render(0, spp_hi, accumulation=_abi.ACCUM_KAHAN, seed_offset=1000 * k + 500)
    target = r.read(_abi.ACCUM_KAHAN).copy()
    return feat, noisy, target


def test_trained_denoiser_beats_plain_accumulation(agb, oracle):
    """Train on 4-spp / 512-spp pairs of six views, evaluate on a seventh: the denoised image is
    closer to the reference than the 4-spp accumulation it was made from."""
    import torch
    from aurora_gb300 import _abi, api, scenes
    s = scenes.config_small(width=128, height=96, spp=4)
    lo, hi = 4, 512
    with api.Renderer() as r:
        r.upload(s)
        data = [render_pair(r, s, k, lo, hi) for k in range(7)]
    feats = torch.stack([d[0] for d in data[:6]])
    targets = torch.from_numpy(np.stack([d[2] for d in data[:6]])).cuda()
    dn = denoiser(agb, seed=11)
    try:
        losses = []
        for step in range(300):
            idx = [(step * 2 + j) % 6 for j in range(2)]
            fb = feats[idx].contiguous()     # held: the call reads these device buffers
            tb = targets[idx].contiguous()
            loss = ctypes.c_float()
            _abi.check(agb.agb_denoiser_train_step(dn, fb.data_ptr(), tb.data_ptr(), 2, s.height,
                                                   s.width, 2e-3, 1, ctypes.byref(loss)))
            losses.append(loss.value)
        feat, noisy, target = data[6]
        out = torch.zeros((s.height, s.width, 4), dtype=torch.float32, device="cuda")
        _abi.check(agb.agb_denoiser_forward(dn, feat.data_ptr(), 1, s.height, s.width, out.data_ptr()))
        den = out.cpu().numpy()
    finally:
        agb.agb_denoiser_destroy(dn)
    e_noisy = oracle.rel_mse(noisy[..., :3], target[..., :3])
    e_den = oracle.rel_mse(den[..., :3], target[..., :3])
    print(f"loss first 10 {np.mean(losses[:10]):.4f} last 10 {np.mean(losses[-10:]):.4f}")
    print(f"held-out view: relMSE plain {lo} spp {e_noisy:.4g}, denoised {e_den:.4g}")
    assert np.mean(losses[-10:]) < 0.7 * np.mean(losses[:10])
    assert e_den < 0.5 * e_noisy
