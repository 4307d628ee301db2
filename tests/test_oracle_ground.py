"""The oracle's ground plane (GroundPlane.slang) on the CPU: planes that cannot act leave the
image bit for bit as it is without one, and the plane that acts changes it."""
import numpy as np

from aurora_gb300 import _abi


def scene(**values):
    from aurora_gb300 import scenes
    s = scenes.config_tiny(width=24, height=16, spp=2)
    s.instances = s.instances[:4]
    s.ground_plane = None if values.get("none") else _abi.ground_plane(
        **{k: v for k, v in values.items() if k != "none"})
    return s


def render(oracle, s):
    return oracle.OracleScene(s).render(0, 2, threads=4)["mean"]


def test_inactive_ground_planes_change_nothing(oracle):
    ref = render(oracle, scene(none=True))
    for values in (dict(enabled=0),
                   dict(reflection_opacity=0.0, shadow_opacity=0.0),
                   # facing away from the camera above it: the plane is invisible from this side
                   dict(normal=(0.0, -1.0, 0.0))):
        img = render(oracle, scene(**values))
        np.testing.assert_array_equal(img, ref, err_msg=str(values))


def test_active_ground_plane_changes_the_image(oracle):
    ref = render(oracle, scene(none=True))
    img = render(oracle, scene())
    changed = np.mean(np.any(img != ref, axis=2))
    assert changed > 0.2, changed
    # the black matte shadow and a 0.5 reflection darken the plane pixels on average
    assert img[..., :3].sum() < ref[..., :3].sum()
