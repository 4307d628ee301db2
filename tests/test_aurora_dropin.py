"""Aurora's own public interface (include/Aurora/Aurora.h, the reference's
Libraries/Aurora/API/Aurora/Aurora.h) served by libagb_cuda.so through Aurora::createRenderer.

CPU: the binary interface of this library's copy of the header (vtable slots of every virtual
function, sizes and member offsets of the value types, enumerator values) equals the reference
header's, live where the reference tree is present and against tests/golden/aurora_interface.txt
everywhere; the library defines every Aurora::Names string with the reference's value; the client
tests/cpp/aurora_dropin_render.cpp compiles and links against both headers.

GPU: the client renders through createRenderer and the image equals, bit for bit, the image the
path-keyed C++ layer's client renders (tests/cpp/aurora_api_render.cpp) from the same scene file,
and matches the C ABI within the camera-inverse rounding that test allows (relMSE below 1e-10)."""
import os
import struct
import subprocess
import sys
import tempfile

import numpy as np
import pytest

import aurora_interface as ai

sys.path.insert(0, os.path.join(ai.ROOT, "oracle"))


def reference_root():
    from build_oracle import REFERENCE_ROOT
    header = os.path.join(REFERENCE_ROOT, "Libraries", "Aurora", "API", "Aurora", "Aurora.h")
    return REFERENCE_ROOT if os.path.exists(header) else None


def need_reference():
    ref = reference_root()
    if ref is None:
        pytest.skip("the reference tree is not on this machine (the fixture tests cover it)")
    return ref


def lib_dir():
    from aurora_gb300 import build
    return os.path.dirname(build.build())


def build_client(includes=None, name="aurora_dropin_render"):
    """The client compiled against `includes` (default: this library's headers) and linked against
    libagb_cuda.so; returns its path."""
    out_dir = lib_dir()
    lib = os.path.join(out_dir, "libagb_cuda.so")
    exe = os.path.join(out_dir, name)
    deps = [ai.CLIENT, lib] + [os.path.join(d, f) for d in (includes or ai.MIRROR)
                               for d, _, fs in os.walk(d) for f in fs]
    if not os.path.exists(exe) or os.path.getmtime(exe) < max(map(os.path.getmtime, deps)):
        ai.compile_cpp(ai.CLIENT, includes or ai.MIRROR, exe + ".tmp",
                       ["-L" + out_dir, "-lagb_cuda", "-Wl,-rpath," + out_dir])
        os.replace(exe + ".tmp", exe)
    return exe


def test_interface_layout_matches_reference_fixture():
    layout, _ = ai.read_fixture()
    assert ai.probe_layout(ai.MIRROR) == layout


def test_interface_layout_matches_reference_header():
    ref = need_reference()
    mine, theirs = ai.probe_layout(ai.MIRROR), ai.probe_layout(ai.reference_includes(ref))
    assert mine == theirs
    assert len(mine.splitlines()) > 130


def test_fixture_matches_reference_source():
    ref = need_reference()
    layout, names = ai.read_fixture()
    assert ai.probe_layout(ai.reference_includes(ref)) == layout
    assert ai.reference_names(ref) == names


def test_library_defines_reference_names():
    _, names = ai.read_fixture()
    assert len(names) >= 46
    assert ai.library_names(names, lib_dir()) == names


def test_client_builds_against_this_header():
    assert os.access(build_client(), os.X_OK)


def test_client_builds_against_reference_header():
    """The unmodified reference header: a client compiled against it links against this library
    (Aurora::createRenderer and the Names strings resolve to libagb_cuda.so's definitions)."""
    ref = need_reference()
    assert os.access(build_client(ai.reference_includes(ref), "aurora_dropin_render_refheader"), os.X_OK)


def run_client(exe, scene_file, out_file, flags=()):
    subprocess.check_call([exe, scene_file, out_file] + list(flags))
    raw = open(out_file, "rb").read()
    w, h = struct.unpack("<2I", raw[:8])
    return np.frombuffer(raw[8:], np.float32).reshape(h, w, 4)


def c_abi_frame(s, view, proj, lights, depth):
    from aurora_gb300 import _abi, api, scenes
    frame = scenes.frame_data(view.astype(np.float64), proj.astype(np.float64), trace_depth=depth,
                              lights=lights, scene_bounds=s.bounds())
    with api.Renderer() as r:
        r.upload(s)
        r.set_frame(frame)
        r.render(0, s.spp, accumulation=_abi.ACCUM_RUNNING_MEAN)
        ref, _ = r.post_process(mode=_abi.ACCUM_RUNNING_MEAN)
    return ref


def compare(oracle, s, view, proj, lights, depth, flags, mtlx=False):
    from test_aurora_api import build_client as build_layer_client, write_scene
    exe, layer_exe = build_client(), build_layer_client()
    with tempfile.TemporaryDirectory() as tmp:
        scene_file = os.path.join(tmp, "scene.bin")
        write_scene(scene_file, s, view, proj, lights, depth, mtlx=mtlx)
        img = run_client(exe, scene_file, os.path.join(tmp, "a.bin"), flags)
        late = ["--late-materials"] if "--late-materials" in flags else []
        layer = run_client(layer_exe, scene_file, os.path.join(tmp, "b.bin"), late)
    ref = c_abi_frame(s, view, proj, lights, depth)
    err = oracle.rel_mse(img, ref)
    print(f"Aurora interface {' '.join(flags) or 'paths'}: identical to the C++ layer's client "
          f"{np.array_equal(img, layer)}; vs C ABI relMSE {err:.3g}, identical pixels "
          f"{np.mean(np.all(img == ref, axis=2)):.4f}")
    np.testing.assert_array_equal(img, layer)
    assert err < 1e-10
    assert np.abs(img[..., :3]).max() > 0
    return img, ref


@pytest.mark.gpu
@pytest.mark.parametrize("flags", [[], ["--pointers"]])
@pytest.mark.parametrize("ground,mtlx", [(False, False), (True, False), (False, True)])
def test_dropin_render_matches(agb, oracle, flags, ground, mtlx):
    """Spheres and a floor (or a ground plane with non-default values), a distant light, a constant
    environment; materials as property lists or MaterialX documents."""
    from aurora_gb300 import _abi, scenes
    s = scenes.config_tiny(width=48, height=32, spp=8, lights=False)
    if ground:
        s.instances = s.instances[:4]
        s.meshes = s.meshes[:1]
        s.ground_plane = _abi.ground_plane(position=(0.0, 0.05, 0.0), shadow_opacity=0.7,
                                           shadow_color=(0.1, 0.2, 0.3), reflection_opacity=0.4,
                                           reflection_color=(0.8, 0.6, 0.4),
                                           reflection_roughness=0.2)
    view = np.asarray(scenes.look_at((0.4, 3.0, 7.0), (0.0, 0.8, 0.0)), np.float32)
    proj = np.asarray(scenes.perspective(45.0, s.width / s.height), np.float32)
    lights = [((0.3, -1.0, -0.2), (1.0, 0.95, 0.9), 2.0, 0.0)]
    compare(oracle, s, view, proj, lights, 4, flags, mtlx=mtlx)


@pytest.mark.gpu
@pytest.mark.parametrize("flags,mtlx", [([], False), (["--pointers"], False), (["--late-materials"], False),
                                        (["--pointers", "--late-materials"], False),
                                        (["--loader"], True), (["--pointers", "--loader"], True)])
def test_dropin_textures_and_layers_match(agb, oracle, flags, mtlx):
    """Material textures with a transform, a bilinear sampler and material layers (layer material
    and layer geometry): path-keyed, or as image / sampler / material / geometry pointers with
    addInstancePointer's layer definitions; with --late-materials the material values arrive after
    a first render (a pointer material's values reach the scene at the next render); with `mtlx`
    the materials are MaterialX documents whose PNG textures the client's resource loader reads
    (setLoadResourceFunction)."""
    from aurora_gb300 import _abi, scenes
    s = scenes.config_layered(width=64, height=48, spp=4, trace_depth=4, blas=2, instances=6,
                              tri_range=(200, 1000), decal_size=64)
    color_img = int(s.textures["image"][6, _abi.TEX_BASE_COLOR])
    s.materials["has_base_color_image"][0] = 1
    s.textures["image"][0, _abi.TEX_BASE_COLOR] = color_img
    s.materials["base_color_image_scale"][0] = (2.0, 0.5)
    s.materials["base_color_image_offset"][0] = (0.1, 0.2)
    if not mtlx:  # a tiledimage has no pivot or rotation
        s.materials["base_color_image_pivot"][0] = (0.5, 0.5)
        s.materials["base_color_image_rotation"][0] = 0.3
    view = np.asarray(scenes.look_at((0.0, 15.0, 60.0), (0.0, 0.0, 0.0)), np.float32)
    proj = np.asarray(scenes.perspective(45.0, s.width / s.height), np.float32)
    compare(oracle, s, view, proj, [], 4, flags, mtlx=mtlx)


@pytest.mark.gpu
def test_dropin_environment_image(agb, oracle):
    """An environment light and background image (Float_RGB through setImageDescriptor)."""
    from aurora_gb300 import _abi, scenes
    s = scenes.config_tiny(width=48, height=32, spp=8, lights=False)
    env = np.random.default_rng(5).lognormal(0.0, 0.8, size=(32, 64, 3)).astype(np.float32)
    s.env_light = s.env_background = s.add_image(env, _abi.FORMAT_RGB32F)
    view = np.asarray(scenes.look_at((0.4, 3.0, 7.0), (0.0, 0.8, 0.0)), np.float32)
    proj = np.asarray(scenes.perspective(45.0, s.width / s.height), np.float32)
    compare(oracle, s, view, proj, [], 4, [])
