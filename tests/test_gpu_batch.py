"""Batched rendering (agb_batch_render): requests of several scenes, resolutions, sample counts,
trace depths, seeds and cameras rendered by one wavefront per wave.  Each request's image (and
its denoising AOVs) must be bit-identical to the same request rendered alone with agb_render,
with one wave for the batch or many (a small path budget), and the batch must launch the
kernels of one wavefront per wave, not one per request."""
import numpy as np
import pytest

from aurora_gb300 import _abi

pytestmark = pytest.mark.gpu


def scene_set():
    from aurora_gb300 import scenes
    tiny = scenes.config_tiny(width=48, height=32, spp=4)            # depth 4, distant light
    small = scenes.config_small(width=64, height=48, spp=4)          # depth 5
    large = scenes.config_large(width=64, height=36, spp=2, level=5, instances=16,
                                env_size=(128, 64))                  # depth 8, glass, coat
    layered = scenes.config_layered(width=40, height=30, spp=2, blas=2, instances=6,
                                    tri_range=(200, 800), decal_size=64)   # textures, layers
    return [tiny, small, large, layered]


def requests(scs):
    """(scene index, width, height, spp, seed offset, jitter, AOVs)."""
    return [(0, 48, 32, 4, 0, None, False), (1, 64, 48, 3, 7, (0.25, -0.1), True),
            (2, 64, 36, 2, 0, None, False), (3, 40, 30, 2, 3, None, False),
            (0, 24, 16, 5, 11, (-0.3, 0.2), True), (2, 32, 18, 1, 5, None, True),
            (1, 16, 12, 6, 0, None, False)]


def frame_for(s, w, h, jitter, aovs):
    from aurora_gb300 import scenes
    f = np.asarray(s.frame).copy()
    f["view_size"] = f["view_size"]
    if jitter is not None:
        f["camera_jitter"] = jitter
        f["is_temporal_jitter_enabled"] = 1
    f["is_denoising_aovs_enabled"] = 1 if aovs else 0
    return f


def render_alone(r, f, w, h, spp, seed):
    from aurora_gb300 import api
    with api.View(r) as v:
        v.set_frame(f)
        v.render(0, spp, width=w, height=h, seed_offset=seed)
        out = (v.read(_abi.ACCUM_RUNNING_MEAN, w, h).copy(), v.read(_abi.ACCUM_KAHAN, w, h).copy())
        aov = v.aovs(w, h) if f["is_denoising_aovs_enabled"] else None
    return out, aov


@pytest.mark.parametrize("max_paths", [1 << 22, 3000])
def test_batch_matches_requests_rendered_alone(agb, max_paths):
    from aurora_gb300 import api
    scs = scene_set()
    rs = []
    try:
        for s in scs:
            r = api.Renderer()
            r.upload(s)
            rs.append(r)
        reqs = requests(scs)
        views, items, want = [], [], []
        for k, w, h, spp, seed, jit, aovs in reqs:
            f = frame_for(scs[k], w, h, jit, aovs)
            want.append(render_alone(rs[k], f, w, h, spp, seed))
            v = api.View(rs[k])
            v.set_frame(f)
            views.append(v)
            items.append(dict(view=v, width=w, height=h, spp=spp, seed_offset=seed))
        with api.Batch(max_paths=max_paths) as b:
            st = b.render(items, stats=True)
        per_wave = st["kernel_launches"]
        print(f"batch of {len(items)} requests over 4 scenes: {st['kernel_launches']} launches, "
              f"{st['paths']} paths, {st['gpu_ms']:.2f} ms")
        for (k, w, h, spp, seed, jit, aovs), v, (img, aov) in zip(reqs, views, want):
            np.testing.assert_array_equal(v.read(_abi.ACCUM_RUNNING_MEAN, w, h), img[0])
            np.testing.assert_array_equal(v.read(_abi.ACCUM_KAHAN, w, h), img[1])
            if aovs:
                got = v.aovs(w, h)
                for key in aov:
                    np.testing.assert_array_equal(got[key], aov[key])
        if max_paths >= 1 << 22:
            # One wavefront for all seven requests: camera, 8 bounces x 6 kernels, the depth
            # limit, finalize.
            assert per_wave == 1 + 8 * 6 + 1 + 1
        for v in views:
            v.close()
    finally:
        for r in rs:
            r.close()


def test_batch_progressive_continuation(agb):
    """A view accumulated over two batched calls (samples 0-2, then 3-5) equals one call."""
    from aurora_gb300 import api, scenes
    s = scenes.config_tiny(width=32, height=24, spp=6)
    with api.Renderer() as r:
        r.upload(s)
        with api.View(r) as a, api.View(r) as b, api.Batch() as bt:
            a.set_frame(s.frame)
            b.set_frame(s.frame)
            bt.render([dict(view=a, width=32, height=24, spp=6)])
            bt.render([dict(view=b, width=32, height=24, spp=3)])
            bt.render([dict(view=b, width=32, height=24, spp=3, start=3)])
            np.testing.assert_array_equal(a.read(_abi.ACCUM_KAHAN, 32, 24), b.read(_abi.ACCUM_KAHAN, 32, 24))
            np.testing.assert_array_equal(a.read(_abi.ACCUM_RUNNING_MEAN, 32, 24),
                                          b.read(_abi.ACCUM_RUNNING_MEAN, 32, 24))


def test_batch_rejects_bad_requests(agb):
    from aurora_gb300 import api, scenes
    s = scenes.config_tiny()
    with api.Renderer() as r:
        r.upload(s)
        with api.View(r) as v, api.Batch() as bt:
            with pytest.raises(_abi.AgbError):
                bt.render([dict(view=v, width=32, height=24, spp=1)])   # no frame set
            v.set_frame(s.frame)
            with pytest.raises(_abi.AgbError):
                bt.render([dict(view=v, width=32, height=24, spp=1), dict(view=v, width=32, height=24, spp=1)])
            with pytest.raises(_abi.AgbError):
                bt.render([dict(view=v, width=32, height=24, spp=1, start=4)])
