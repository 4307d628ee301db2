"""The serving loop (agb_server_*): requests of several resident scenes and resolutions overlap on
the device through pooled views; a request's image is the same rendered alone and in the middle
of a mix (renders are deterministic in scene, frame, sample count and seed offset: tolerance 0);
scenes and requests are admitted by HBM footprint; latencies are reported."""
import numpy as np
import pytest

from aurora_gb300 import _abi

pytestmark = pytest.mark.gpu


def scenes_and_frames():
    from aurora_gb300 import scenes
    out = []
    for k, s in enumerate([scenes.config_tiny(width=64, height=48, spp=4),
                           scenes.config_small(width=96, height=64, spp=4),
                           scenes.config_small(seed=3, width=96, height=64, spp=4)]):
        out.append(s)
    return out


def upload_all(sc):
    from aurora_gb300 import api
    rs = []
    for s in sc:
        r = api.Renderer()
        r.upload(s)
        rs.append(r)
    return rs


def test_request_same_alone_and_in_mix(agb):
    from aurora_gb300 import api
    sc = scenes_and_frames()
    rs = upload_all(sc)
    try:
        with api.Server(hbm_budget_bytes=8 << 30, max_slots=4) as srv:
            for k, r in enumerate(rs):
                assert srv.add_scene(k, r) == _abi.AGB_OK
            probe = dict(scene_id=1, frame=sc[1].frame, width=96, height=64, spp=8, seed_offset=7)
            st, alone, info = srv.wait(srv.submit(**probe))
            assert st == _abi.AGB_OK
            tickets = []
            rng = np.random.default_rng(0)
            for i in range(12):
                k = int(rng.integers(0, 3))
                w, h = [(64, 48), (96, 64), (128, 96)][int(rng.integers(0, 3))]
                tickets.append(srv.submit(k, sc[k].frame, w, h, int(rng.choice([1, 4, 16])),
                                          seed_offset=i))
                if i == 5:
                    mid = srv.submit(**probe)
            results = [srv.wait(t) for t in tickets]
            st2, mixed, info2 = srv.wait(mid)
        assert st2 == _abi.AGB_OK and all(r[0] == _abi.AGB_OK for r in results)
        np.testing.assert_array_equal(mixed, alone)
        # The same request through the direct render path.
        rs[1].set_frame(sc[1].frame)
        rs[1].render(0, 8, width=96, height=64, accumulation=_abi.ACCUM_RUNNING_MEAN, seed_offset=7)
        np.testing.assert_array_equal(rs[1].read(_abi.ACCUM_RUNNING_MEAN, 96, 64), alone)
        lat = [r[2]["latency_ms"] for r in results]
        print(f"mix of 12: latency p50 {np.percentile(lat, 50):.2f} ms p99 {np.percentile(lat, 99):.2f} ms")
        assert all(r[2]["latency_ms"] >= r[2]["render_ms"] >= 0 for r in results)
    finally:
        for r in rs:
            r.close()


def test_admission_by_hbm_budget(agb):
    from aurora_gb300 import api, scenes
    sc = scenes_and_frames()[:2] + [scenes.config_large(width=96, height=64, spp=4, level=7,
                                                        instances=4, env_size=(64, 32))]
    rs = upload_all(sc)
    try:
        sizes = [r.memory_bytes() for r in rs]
        budget = sizes[0] + sizes[1] + (24 << 20)
        assert sizes[2] > (24 << 20)
        with api.Server(hbm_budget_bytes=budget, max_slots=4) as srv:
            assert srv.add_scene(0, rs[0]) == _abi.AGB_OK
            assert srv.add_scene(1, rs[1]) == _abi.AGB_OK
            assert srv.add_scene(2, rs[2]) == _abi.ERR_OOM      # beyond the budget
            # A request whose render state cannot fit fails cleanly; small ones all complete,
            # queueing for memory.
            st, img, info = srv.wait(srv.submit(0, sc[0].frame, 4096, 4096, 16))
            assert st == _abi.ERR_OOM and img is None
            tickets = [srv.submit(i % 2, sc[i % 2].frame, 64, 48, 2, seed_offset=i) for i in range(10)]
            out = [srv.wait(t) for t in tickets]
            assert all(o[0] == _abi.AGB_OK for o in out)
            scene_bytes, render_bytes = srv.memory()
            assert scene_bytes == sizes[0] + sizes[1]
            assert scene_bytes + render_bytes <= budget
    finally:
        for r in rs:
            r.close()


def test_denoised_serving(agb):
    import ctypes
    from aurora_gb300 import api
    sc = scenes_and_frames()
    rs = upload_all(sc)
    dn = ctypes.c_void_p()
    _abi.check(agb.agb_denoiser_create(0, None, 5, ctypes.byref(dn)))
    try:
        with api.Server(hbm_budget_bytes=8 << 30, max_slots=2) as srv:
            srv.add_scene(1, rs[1])
            srv.set_denoiser(dn)
            st, den, _ = srv.wait(srv.submit(1, sc[1].frame, 96, 64, 4, seed_offset=3, denoise=True))
            st2, plain, _ = srv.wait(srv.submit(1, sc[1].frame, 96, 64, 4, seed_offset=3))
        assert st == _abi.AGB_OK and st2 == _abi.AGB_OK
        assert np.isfinite(den).all() and (den[..., 3] == 1).all()
        assert np.abs(den[..., :3] - plain[..., :3]).max() > 0
    finally:
        agb.agb_denoiser_destroy(dn)
        for r in rs:
            r.close()
