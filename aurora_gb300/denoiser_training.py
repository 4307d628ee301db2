"""Training the learned denoiser on the path tracer's own renders.

Pairs: seeded scenes of both plain-method types (the 8x8 sphere grid of the small configuration
and the instanced displaced icospheres of the large one, the latter at subdivision 6 -- 81,920
triangles, below a pixel at these crop sizes -- with a 512x256 environment), each seen from
several random orbit cameras as crop-sized frames (256x256 by default); per view the features of a
`spp_lo` render (noisy radiance, AOVs, luminance variance: agb_denoiser_features) and a `spp_hi`
reference rendered from independent random streams.  Training: the network's own tensor-core
forward and backward kernels (agb_denoiser_train_step: L1 loss on log1p radiance, Adam), a cosine
learning-rate schedule, random batches of views.  Device buffers come from torch (allocation
only); all compute is in libagb_cuda.
"""
import ctypes
import math
import time

import numpy as np

from . import _abi, api, scenes


def orbit_frame(s, rng, width, height, trace_depth):
    """A random camera around the scene's bounds: azimuth U[0, 2 pi), elevation U[10, 50] degrees,
    distance U[0.8, 1.6] x the bounds' radius over tan(fov / 2), looking at a point near the
    centre; denoising AOVs on."""
    lo, hi = s.bounds()
    c = 0.5 * (lo + hi)
    rad = 0.5 * float(np.linalg.norm(hi - lo))
    az = rng.uniform(0, 2 * math.pi)
    el = math.radians(rng.uniform(10, 50))
    dist = rng.uniform(0.8, 1.6) * rad / math.tan(math.radians(22.5))
    eye = c + dist * np.array([math.cos(el) * math.sin(az), math.sin(el), math.cos(el) * math.cos(az)])
    target = c + rng.normal(0, 0.15 * rad, 3)
    return scenes.frame_data(scenes.look_at(eye, target), scenes.perspective(45.0, width / height),
                             trace_depth=trace_depth, scene_bounds=(lo, hi), aovs=True)


def training_scene(kind, seed, size):
    if kind == "small":
        return scenes.config_small(seed=seed, width=size, height=size, spp=1)
    return scenes.config_large(seed=seed, width=size, height=size, spp=1, level=6, env_size=(512, 256))


def render_pair(r, s, frame, width, height, spp_lo, spp_hi, seed_offset):
    """(features int16 [H, W, 16] device, noisy RGBA [H, W, 4] device, reference RGBA device)."""
    import torch
    r.set_frame(frame)
    r.render(0, spp_lo, width=width, height=height,
             accumulation=_abi.ACCUM_RUNNING_MEAN | _abi.ACCUM_MOMENTS, seed_offset=seed_offset)
    feat = torch.zeros((height, width, 16), dtype=torch.int16, device="cuda")
    _abi.check(_abi.library().agb_denoiser_features(r.ctx, feat.data_ptr()))
    noisy = torch.from_numpy(r.read(_abi.ACCUM_RUNNING_MEAN, width, height).copy()).cuda()
    r.render(0, spp_hi, width=width, height=height, accumulation=_abi.ACCUM_KAHAN,
             seed_offset=seed_offset + (1 << 24))
    ref = torch.from_numpy(r.read(_abi.ACCUM_KAHAN, width, height).copy()).cuda()
    return feat, noisy, ref


def make_pairs(n_scenes, views_per_scene, size=256, spp_lo=4, spp_hi=256, seed=0):
    """Renders the training pairs; returns (features [N, H, W, 16], noisy [N, H, W, 4], reference
    [N, H, W, 4]) as device tensors, and the seconds it took."""
    import torch
    t0 = time.perf_counter()
    feats, noisy, refs = [], [], []
    rng = np.random.default_rng(seed)
    for i in range(n_scenes):
        kind = "small" if i % 2 == 0 else "large"
        s = training_scene(kind, seed * 1000 + i, size)
        with api.Renderer() as r:
            r.upload(s)
            depth = 5 if kind == "small" else 8
            for v in range(views_per_scene):
                f = orbit_frame(s, rng, size, size, depth)
                a, b, c = render_pair(r, s, f, size, size, spp_lo, spp_hi, seed_offset=(i * 97 + v) * 4096)
                feats.append(a)
                noisy.append(b)
                refs.append(c)
    torch.cuda.synchronize()
    return torch.stack(feats), torch.stack(noisy), torch.stack(refs), time.perf_counter() - t0


class Denoiser:
    """The U-Net (agb_denoiser_*) with training and inference helpers."""

    def __init__(self, seed=11, device=0):
        self.lib = _abi.library()
        self.handle = ctypes.c_void_p()
        _abi.check(self.lib.agb_denoiser_create(device, None, seed, ctypes.byref(self.handle)))

    def close(self):
        if self.handle:
            self.lib.agb_denoiser_destroy(self.handle)
            self.handle = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def train(self, feats, refs, steps, batch=4, lr=2e-3, lr_min=1e-4, seed=0):
        """Adam on random batches with a cosine schedule; returns the per-step losses."""
        import torch
        rng = np.random.default_rng(seed)
        n, h, w = feats.shape[0], feats.shape[1], feats.shape[2]
        losses = []
        loss = ctypes.c_float()
        for step in range(steps):
            idx = torch.from_numpy(rng.choice(n, size=min(batch, n), replace=False)).cuda()
            fb = feats.index_select(0, idx).contiguous()
            tb = refs.index_select(0, idx).contiguous()
            rate = lr_min + 0.5 * (lr - lr_min) * (1.0 + math.cos(math.pi * step / max(1, steps)))
            _abi.check(self.lib.agb_denoiser_train_step(self.handle, fb.data_ptr(), tb.data_ptr(), len(idx),
                                                        h, w, rate, 1, ctypes.byref(loss)))
            losses.append(loss.value)
        return losses

    def forward(self, feats):
        """Denoised RGBA [N, H, W, 4] (device) for features [N, H, W, 16]."""
        import torch
        n, h, w = feats.shape[0], feats.shape[1], feats.shape[2]
        out = torch.zeros((n, h, w, 4), dtype=torch.float32, device="cuda")
        _abi.check(self.lib.agb_denoiser_forward(self.handle, feats.contiguous().data_ptr(), n, h, w,
                                                 out.data_ptr()))
        return out

    def params(self):
        n = ctypes.c_uint64()
        self.lib.agb_denoiser_param_count(ctypes.byref(n))
        out = np.zeros(n.value, np.float32)
        _abi.check(self.lib.agb_denoiser_params(self.handle, out.ctypes.data, n.value))
        return out

    def set_params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        _abi.check(self.lib.agb_denoiser_set_params(self.handle, p.ctypes.data, p.size))


def rel_mse(x, ref, eps=1e-2):
    """mean over pixels and RGB of (x - r)^2 / (r^2 + eps), per image of a batch (torch)."""
    d = (x[..., :3] - ref[..., :3]).double()
    r = ref[..., :3].double()
    return (d * d / (r * r + eps)).mean(dim=tuple(range(1, x.dim())))
