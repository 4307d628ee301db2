"""agb_environment_alias_build_noalloc: the environment alias-table build on the library's fixed
scratch array gives the same table and integrals as the allocating build behind
agb_environment_set, on two calls in a row (the second call reuses scratch the first one left
behind), for both table layouts.  Named to be collected last, so that it also runs after every
other GPU test has used the device."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# (height, width, seed): a 2:1 lat-long map, the largest accepted size, a ragged one, one texel.
SHAPES = [(256, 512, 11), (362, 724, 12), (7, 13, 13), (1, 1, 14)]


def _image(h, w, seed):
    from aurora_gb300 import scenes
    return scenes.hdr_env(w, h, seed) if h >= 32 else \
        np.random.default_rng(seed).uniform(0, 4, (h, w, 3)).astype(np.float32)


def _scene(img):
    from aurora_gb300 import _abi, scenes
    s = scenes.SceneDesc("env")
    k = s.add_image(img, _abi.FORMAT_RGB32F)
    s.env_light = s.env_background = k
    s.materials = scenes.materials(1)
    s.width = s.height = 4
    s.frame = scenes.frame_data(np.eye(4), scenes.perspective(45, 1))
    return s


def _allocating_build(img, layout):
    """The existing entry point: agb_environment_set, read back with agb_environment_alias."""
    from aurora_gb300 import api
    with api.Renderer() as r:
        r.set_environment_table(layout)
        r.upload(_scene(img))
        return r.environment_alias(fp64_integral=True)


def _noalloc_build(lib, rgba, table, layout):
    import torch
    from aurora_gb300 import _abi
    h, w = rgba.shape[:2]
    shading = ctypes.c_double()
    fp64 = ctypes.c_double()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    _abi.check(lib.agb_environment_alias_build_noalloc(
        ctypes.c_void_p(rgba.data_ptr()), w, h, layout, ctypes.c_void_p(table.data_ptr()),
        ctypes.byref(shading), ctypes.byref(fp64), stream))
    out = table.cpu().numpy().view(_abi.ALIAS_DTYPE).reshape(-1)
    return out, shading.value, fp64.value


@pytest.mark.parametrize("layout", [0, 1], ids=["reference_layout", "fp64_layout"])
@pytest.mark.parametrize("h,w,seed", SHAPES)
def test_noalloc_build_matches_allocating_build(agb, h, w, seed, layout):
    import torch
    from aurora_gb300 import _abi
    assert w * h <= _abi.ENV_NOALLOC_MAX_TEXELS
    img = _image(h, w, seed)
    want, want_shading, want_fp64 = _allocating_build(img, layout)
    rgba = np.concatenate([img, np.ones((h, w, 1), np.float32)], axis=2)
    rgba_dev = torch.from_numpy(np.ascontiguousarray(rgba)).cuda()
    for call in range(2):
        table = torch.full((h * w, 4), -1, dtype=torch.int32, device="cuda")
        got, shading, fp64 = _noalloc_build(agb, rgba_dev, table, layout)
        # Same kernels on the same inputs: the tables agree to the last bit (tolerance 0).
        np.testing.assert_array_equal(got["alias"], want["alias"], err_msg=f"call {call}")
        np.testing.assert_array_equal(got["prob"], want["prob"], err_msg=f"call {call}")
        np.testing.assert_array_equal(got["pdf"], want["pdf"], err_msg=f"call {call}")
        assert shading == want_shading, f"call {call}"
        assert fp64 == want_fp64, f"call {call}"


def test_noalloc_build_rejects_images_beyond_the_limit(agb):
    import torch
    from aurora_gb300 import _abi
    h, w = 513, 512
    assert w * h > _abi.ENV_NOALLOC_MAX_TEXELS
    rgba = torch.ones((h, w, 4), dtype=torch.float32, device="cuda")
    table = torch.zeros((h * w, 4), dtype=torch.int32, device="cuda")
    status = agb.agb_environment_alias_build_noalloc(
        ctypes.c_void_p(rgba.data_ptr()), w, h, 0, ctypes.c_void_p(table.data_ptr()), None, None,
        None)
    assert status == _abi.ERR_LIMIT
    assert b"exceeds the limit of 262144 texels" in agb.agb_last_error()
    assert int(table.abs().sum().item()) == 0
