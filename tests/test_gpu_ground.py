"""Ground plane (GroundPlane.slang): matte shadows of the environment light and a matte GGX
reflection seen by camera rays, against the oracle's restatement at equal samples."""
import numpy as np
import pytest

from aurora_gb300 import _abi

pytestmark = pytest.mark.gpu

TILTED = tuple(np.array([0.15, 1.0, -0.1]) / np.linalg.norm([0.15, 1.0, -0.1]))

CASES = {
    # the reference's defaults for a new ground plane: reflection 0.5, roughness 0.1, black shadow
    "defaults": dict(),
    "shadow_only": dict(reflection_opacity=0.0, shadow_color=(0.3, 0.1, 0.05), shadow_opacity=0.8),
    # roughness 0 takes the GGX minimum alpha
    "mirror_only": dict(shadow_opacity=0.0, reflection_roughness=0.0, reflection_color=(0.9, 0.7, 0.5)),
    # opacity 1: every plane hit reflects (Pr = 0)
    "always_reflect": dict(reflection_opacity=1.0, reflection_roughness=0.4),
    # a tilted plane below the origin: the other branch of the tangent frame
    "tilted": dict(normal=TILTED, position=(0.0, -0.2, 0.0), reflection_opacity=0.3),
}


def ground_scene(width=48, height=32, spp=4, **values):
    """The tiny scene's four spheres over a ground plane at y = 0 (the floor quad removed), so
    the plane shows both the spheres' matte shadows and their reflection."""
    from aurora_gb300 import scenes
    s = scenes.config_tiny(width=width, height=height, spp=spp)
    s.instances = s.instances[:4]
    s.ground_plane = _abi.ground_plane(**values)
    return s


def render_gpu(s, spp, frame=None, aovs=False):
    from aurora_gb300 import api
    with api.Renderer() as r:
        r.upload(s)
        if frame is not None:
            r.set_frame(frame)
        st = r.render(0, spp, stats=True)
        out = dict(mean=r.read(_abi.ACCUM_RUNNING_MEAN), kahan=r.read(_abi.ACCUM_KAHAN), stats=st)
        if aovs:
            out["aov"] = r.aovs()
    return out


@pytest.mark.parametrize("case", sorted(CASES))
def test_ground_plane_matches_oracle(agb, oracle, case):
    s = ground_scene(**CASES[case])
    g = render_gpu(s, 4)
    o = oracle.OracleScene(s).render(0, 4, want_sum=True)
    err = oracle.rel_mse(g["mean"], o["mean"])
    same = np.mean(np.all(g["mean"] == o["mean"], axis=2))
    print(f"{case}: relMSE vs FP32 oracle {err:.3g}, identical pixels {same:.4f}")
    np.testing.assert_array_equal(g["mean"], o["mean"])
    # The plane changes the image against the same spheres without it (with the shadow alone,
    # only the shadowed pixels: a camera ray that misses the spheres ends on the background).
    bare = ground_scene(**CASES[case])
    bare.ground_plane = None
    b = render_gpu(bare, 4)
    changed = np.mean(np.any(b["mean"] != g["mean"], axis=2))
    print(f"{case}: pixels changed by the ground plane {changed:.3f}")
    assert changed > 0.05


def test_ground_plane_shadow_rays_are_counted(agb):
    s = ground_scene(reflection_opacity=0.0)
    with_plane = render_gpu(s, 2)["stats"]
    s.ground_plane = None
    without = render_gpu(s, 2)["stats"]
    print("shadow rays with / without the plane", with_plane["shadow_rays"], without["shadow_rays"])
    assert with_plane["shadow_rays"] > without["shadow_rays"]


def test_disabled_or_transparent_plane_changes_nothing(agb):
    """enabled = 0, or both opacities 0 (no random numbers drawn), give the image without a
    plane bit for bit."""
    base = ground_scene()
    base.ground_plane = None
    ref = render_gpu(base, 3)["mean"]
    for values in (dict(enabled=0), dict(reflection_opacity=0.0, shadow_opacity=0.0)):
        s = ground_scene(**values)
        np.testing.assert_array_equal(render_gpu(s, 3)["mean"], ref, err_msg=str(values))


def test_ground_plane_guide_aovs_match_oracle(agb, oracle):
    """Camera rays absorbed by the matte reflection write the plane's guide AOVs
    (writeGroundPlaneGuideAOVs): view depth, normal + max(roughness, 0.05), reflection colour,
    motion."""
    s = ground_scene(reflection_opacity=1.0, reflection_roughness=0.02,
                     reflection_color=(0.2, 0.4, 0.6))
    f = np.asarray(s.frame).copy()
    f["is_denoising_aovs_enabled"] = 1
    s.frame = f
    g = render_gpu(s, 2, aovs=True)
    o = oracle.OracleScene(s).render(0, 2, want_aov=True)
    for k in ("depth_view", "normal_roughness", "base_color_metalness", "motion"):
        np.testing.assert_array_equal(g["aov"][k], o["aov"][k], err_msg=k)
    np.testing.assert_array_equal(g["mean"], o["mean"])
    plane = np.all(g["aov"]["base_color_metalness"][..., :3] == np.float32([0.2, 0.4, 0.6]), axis=2)
    print("pixels showing the plane", plane.mean())
    assert plane.mean() > 0.2
    assert np.all(g["aov"]["normal_roughness"][plane] == np.float32([0.0, 1.0, 0.0, 0.05]))


def test_ground_plane_converges_to_fp64_oracle(agb, oracle):
    s = ground_scene(width=16, height=12, spp=1024)
    g = render_gpu(s, 1024)
    o = oracle.OracleScene(s).render(0, 1024, precision=64, want_sum=True)
    err = oracle.rel_mse(g["kahan"], o["sum"] / 1024)
    print("converged relMSE vs FP64 oracle", err)
    assert err < 1e-3


def test_ground_plane_rejects_zero_normal(agb):
    from aurora_gb300 import api
    with api.Renderer() as r:
        g = _abi.ground_plane(normal=(0.0, 0.0, 0.0))
        code = _abi.library().agb_ground_plane_set(r.ctx, _abi.ptr(g))
        assert code == _abi.ERR_INVALID_ARG
        assert _abi.library().agb_ground_plane_set(r.ctx, None) == 0


def test_ground_plane_with_transparent_shadows_and_small_waves(agb, oracle):
    """The plane's matte shadow ray is always opaque (shadeMatteShadow is called with true), also
    when the frame traces transparent shadows; and splitting the frame into waves of a few paths
    (each wave with its own counter blocks) changes no pixel."""
    from aurora_gb300 import api
    s = ground_scene(reflection_opacity=0.35, shadow_opacity=0.9)
    s.materials["opacity"][0] = (0.5, 0.3, 0.8)
    f = np.asarray(s.frame).copy()
    f["is_force_opaque_shadows_enabled"] = 0
    s.frame = f
    g = render_gpu(s, 4)
    o = oracle.OracleScene(s).render(0, 4)
    print("transparent shadows + ground plane: identical pixels",
          np.mean(np.all(g["mean"] == o["mean"], axis=2)))
    np.testing.assert_array_equal(g["mean"], o["mean"])
    with api.Renderer() as r:
        r.upload(s)
        r.render(0, 4, max_paths=s.width * s.height // 3)
        small = r.read(_abi.ACCUM_RUNNING_MEAN)
    np.testing.assert_array_equal(small, g["mean"])
