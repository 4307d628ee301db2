"""ctypes binding of libagb_cuda.so (include/agb.h).

The library is built in-tree (aurora_gb300/_build/libagb_cuda.so) by aurora_gb300.build.  There is
no fallback: importing the binding without the library raises, so a missing extension can never
turn into a silent CPU path.  The numpy dtypes below mirror the C structs byte for byte; the
layout test checks every offset against the reference's layouts.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libagb_cuda.so")

AGB_OK = 0
ERRORS = {-1: "invalid argument", -2: "CUDA error", -3: "out of memory", -4: "timeout",
          -5: "not ready", -6: "limit exceeded"}
ERR_LIMIT = -6
ERR_INVALID_ARG, ERR_CUDA, ERR_OOM, ERR_TIMEOUT, ERR_NOT_READY = -1, -2, -3, -4, -5

ACCUM_RUNNING_MEAN = 1
ACCUM_KAHAN = 2
ACCUM_MOMENTS = 4
FORMAT_RGBA8 = 0
FORMAT_RGBA32F = 1
FORMAT_RGB32F = 2
ENV_TABLE_REFERENCE = 0
ENV_TABLE_FP64 = 1
BVH_HOST, BVH_GPU = 0, 1
ENV_NOALLOC_MAX_TEXELS = 262144  # AGB_ENV_NOALLOC_MAX_TEXELS
WAVE_LARGEST = 0xFFFFFFFF  # AGB_WAVE_LARGEST: waves from half the free device memory
TEX_BASE_COLOR, TEX_SPECULAR_ROUGHNESS, TEX_OPACITY, TEX_NORMAL, TEX_EMISSION = range(5)


def _f(name, n=None):
    return (name, "<f4") if n is None else (name, "<f4", (n,))


def _i(name, n=None):
    return (name, "<i4") if n is None else (name, "<i4", (n,))


# Standard Surface block, 400 bytes (Shaders/DefaultMaterialUniformBuffer.slang).
MATERIAL_DTYPE = np.dtype([
    _f("base"), _f("base_color", 3), _f("diffuse_roughness"), _f("metalness"), _f("specular"),
    _i("_pad0"), _f("specular_color", 3), _f("specular_roughness"), _f("specular_IOR"),
    _f("specular_anisotropy"), _f("specular_rotation"), _f("transmission"),
    _f("transmission_color", 3), _f("subsurface"), _f("subsurface_color", 3), _i("_pad1"),
    _f("subsurface_radius", 3), _f("subsurface_scale"), _f("subsurface_anisotropy"), _f("sheen"),
    _i("_pad2"), _i("_pad3"), _f("sheen_color", 3), _f("sheen_roughness"), _f("coat"),
    _f("coat_color", 3), _f("coat_roughness"), _f("coat_anisotropy"), _f("coat_rotation"),
    _f("coat_IOR"), _f("coat_affect_color"), _f("coat_affect_roughness"), _f("emission"),
    _i("_pad4"), _f("emission_color", 3), _i("_pad5"), _f("opacity", 3), _i("thin_walled"),
    _i("has_base_color_image"), _f("base_color_image_offset", 2), _i("_pad6"),
    _f("base_color_image_scale", 2), _f("base_color_image_pivot", 2),
    _f("base_color_image_rotation"), _i("has_specular_roughness_image"),
    _f("specular_roughness_image_offset", 2), _f("specular_roughness_image_scale", 2),
    _f("specular_roughness_image_pivot", 2), _f("specular_roughness_image_rotation"),
    _i("has_emission_color_image"), _f("emission_color_image_offset", 2),
    _f("emission_color_image_scale", 2), _f("emission_color_image_pivot", 2),
    _f("emission_color_image_rotation"), _i("has_opacity_image"), _f("opacity_image_offset", 2),
    _f("opacity_image_scale", 2), _f("opacity_image_pivot", 2), _f("opacity_image_rotation"),
    _i("has_normal_image"), _f("normal_image_offset", 2), _f("normal_image_scale", 2),
    _f("normal_image_pivot", 2), _f("normal_image_rotation"), _i("_pad7"), _i("_pad8"), _i("_pad9"),
])
assert MATERIAL_DTYPE.itemsize == 400

MATERIAL_TEXTURES_DTYPE = np.dtype([_i("image", 5)])
# agb_graph_op: a material node-graph program operation (operation codes GOP_*, inputs GIN_*,
# outputs GOUT_*, as include/agb.h numbers them).
GRAPH_OP_DTYPE = np.dtype([("op", "u1"), ("dst", "u1"), ("a", "u1"), ("b", "u1"), ("c", "u1"), ("d", "u1"),
                           ("imm", "<u2")])
GRAPH_REGS = 32
(GOP_CONST, GOP_INPUT, GOP_ADD, GOP_SUB, GOP_MUL, GOP_DIV, GOP_MIN, GOP_MAX, GOP_POW, GOP_MOD, GOP_FLOOR,
 GOP_CEIL, GOP_ABS, GOP_SIN, GOP_COS, GOP_SQRT, GOP_SIGN, GOP_CLAMP, GOP_MIX, GOP_DOT, GOP_NORMALIZE,
 GOP_LENGTH, GOP_SWIZZLE, GOP_COMBINE, GOP_SELECT, GOP_IMAGE, GOP_NORMALMAP, GOP_OUTPUT, GOP_NOISE) = range(29)
(GIN_TEXCOORD, GIN_POSITION_WORLD, GIN_POSITION_OBJECT, GIN_NORMAL_WORLD, GIN_NORMAL_OBJECT,
 GIN_TANGENT_WORLD, GIN_BITANGENT_WORLD) = range(7)
(GOUT_BASE_COLOR, GOUT_SPECULAR_ROUGHNESS, GOUT_COAT_ROUGHNESS, GOUT_EMISSION_COLOR, GOUT_OPACITY,
 GOUT_NORMAL) = range(6)

DISTANT_LIGHT_DTYPE = np.dtype([_f("color_and_intensity", 4), _f("direction", 3), _f("cos_radius")])

# RendererBase::FrameData (RendererBase.h:136-241), 512 bytes.
FRAME_DTYPE = np.dtype([
    _f("camera_view_proj", 16), _f("camera_view_proj_prev", 16), _f("camera_inv_view", 16),
    _f("camera_inv_view_prev", 16), _f("view_size", 2), _f("camera_jitter", 2),
    _f("camera_jitter_prev", 2), _i("is_ortho_projection"), _f("focal_distance"),
    _f("lens_radius"), _f("time_delta_ms"), _i("is_temporal_jitter_enabled"), _f("scene_size"),
    _i("is_force_opaque_shadows_enabled"), _i("is_depth_ndc_enabled"),
    _i("is_diffuse_only_enabled"), _i("is_display_errors_enabled"), _i("is_denoising_enabled"),
    _i("is_denoising_aovs_enabled"), _i("trace_depth"), _f("max_luminance"),
    _i("is_russian_roulette_enabled"), _i("russian_roulette_start_depth"),
    _i("is_path_regularization_enabled"), _f("path_regularization_strength"),
    _f("indirect_bounce_clamp_scale"), _f("sky_view_z"), _f("_padding1", 2),
    ("distant_lights", DISTANT_LIGHT_DTYPE, (4,)), _i("distant_light_count"), _i("_light_pad", 3),
])
assert FRAME_DTYPE.itemsize == 512

# EnvironmentBase::EnvironmentData (EnvironmentBase.h:33-55), 268 bytes.
ENV_DTYPE = np.dtype([
    _f("light_top", 3), _f("_padding1"), _f("light_bottom", 3), _f("light_tex_luminance_integral"),
    _f("light_transform", 16), _f("light_transform_inv", 16), _f("background_top", 3),
    _f("_padding3"), _f("background_bottom", 3), _f("_padding4"), _f("background_transform", 16),
    _i("background_use_screen"), _i("has_light_tex"), _i("has_background_tex"),
])
assert ENV_DTYPE.itemsize == 268

ALIAS_DTYPE = np.dtype([("alias", "<u4"), _f("prob"), _f("pdf"), _f("_padding1")])

# agb_ground_plane (IGroundPlane values, Aurora.h:780-806), 64 bytes.
GROUND_PLANE_DTYPE = np.dtype([
    _i("enabled"), _f("position", 3), _f("normal", 3), _f("shadow_opacity"), _f("shadow_color", 3),
    _f("reflection_opacity"), _f("reflection_color", 3), _f("reflection_roughness"),
])
assert GROUND_PLANE_DTYPE.itemsize == 64


def ground_plane(**values):
    """An agb_ground_plane record with the reference's defaults for a new ground plane
    (PTGroundPlane.cpp:42-51), overridden by `values`."""
    g = np.zeros(1, GROUND_PLANE_DTYPE)
    g["enabled"] = 1
    g["normal"] = (0.0, 1.0, 0.0)
    g["shadow_opacity"] = 1.0
    g["reflection_opacity"] = 0.5
    g["reflection_color"] = (0.5, 0.5, 0.5)
    g["reflection_roughness"] = 0.1
    for k, v in values.items():
        g[k] = v
    return g


class Layer(ctypes.Structure):
    _fields_ = [("material", ctypes.c_int32), ("_pad", ctypes.c_int32),
                ("texcoords", ctypes.c_void_p)]


class Instance(ctypes.Structure):
    _fields_ = [("geometry", ctypes.c_int32), ("material", ctypes.c_int32),
                ("object_to_world", ctypes.c_float * 12), ("layer_count", ctypes.c_int32),
                ("_pad", ctypes.c_int32), ("layers", ctypes.c_void_p)]


class RenderOptions(ctypes.Structure):
    _fields_ = [("width", ctypes.c_uint32), ("height", ctypes.c_uint32),
                ("accumulation", ctypes.c_uint32), ("max_paths_in_flight", ctypes.c_uint32),
                ("env_filter_linear", ctypes.c_int32), ("seed_offset", ctypes.c_uint32),
                ("_pad", ctypes.c_int32 * 2)]


class RenderStats(ctypes.Structure):
    _fields_ = [("paths", ctypes.c_uint64), ("closest_rays", ctypes.c_uint64),
                ("shadow_rays", ctypes.c_uint64), ("node_visits", ctypes.c_uint64),
                ("tri_tests", ctypes.c_uint64), ("shadow_node_visits", ctypes.c_uint64),
                ("shadow_tri_tests", ctypes.c_uint64), ("kernel_launches", ctypes.c_uint64),
                ("gpu_ms", ctypes.c_double), ("kernel_ms", ctypes.c_double * 6),
                ("kernel_count", ctypes.c_uint64 * 6), ("shading_points", ctypes.c_uint64),
                ("closest_rays_per_bounce", ctypes.c_uint64 * 16), ("shadow_rays_per_bounce", ctypes.c_uint64 * 16)]

KERNEL_FAMILIES = ("camera", "trace_closest", "shade", "trace_shadow", "resolve", "finalize")


class AovBuffers(ctypes.Structure):
    _fields_ = [("depth_view", ctypes.c_void_p), ("normal_roughness", ctypes.c_void_p),
                ("base_color_metalness", ctypes.c_void_p), ("motion", ctypes.c_void_p)]


class TemporalSettings(ctypes.Structure):
    """agb_temporal_settings; defaults of PTRenderer.cpp:2043-2046."""
    _fields_ = [("is_reset", ctypes.c_uint32), ("blend_alpha_min", ctypes.c_float),
                ("blend_alpha_max", ctypes.c_float), ("speed_reference", ctypes.c_float)]


POST_SOURCE_TEMPORAL = 4
SERVE_DENOISE = 1


class ServeRequest(ctypes.Structure):
    _fields_ = [("scene", ctypes.c_int32), ("width", ctypes.c_uint32), ("height", ctypes.c_uint32),
                ("spp", ctypes.c_uint32), ("seed_offset", ctypes.c_uint32), ("flags", ctypes.c_int32),
                ("_pad", ctypes.c_uint32 * 2), ("frame", ctypes.c_uint8 * 512)]


class ServeResult(ctypes.Structure):
    _fields_ = [("id", ctypes.c_uint64), ("status", ctypes.c_int32), ("width", ctypes.c_uint32),
                ("height", ctypes.c_uint32), ("_pad", ctypes.c_int32), ("queue_ms", ctypes.c_double),
                ("render_ms", ctypes.c_double), ("latency_ms", ctypes.c_double)]

# Every symbol include/agb.h declares, with its ctypes signature.
_P = ctypes.c_void_p
_I32 = ctypes.c_int32
_U32 = ctypes.c_uint32
_I64 = ctypes.c_int64
_U64 = ctypes.c_uint64
SIGNATURES = {
    "agb_context_create": (_I32, [_I32, _P, ctypes.POINTER(_P)]),
    "agb_context_destroy": (_I32, [_P]),
    "agb_last_error": (ctypes.c_char_p, []),
    "agb_context_memory": (_I32, [_P, ctypes.POINTER(_U64)]),
    "agb_bytes_per_path": (_U64, []),
    "agb_view_create": (_I32, [_P, _P, ctypes.POINTER(_P)]),
    "agb_wait_poll": (_I32, [_P]),
    "agb_server_create": (_I32, [_I32, _U64, _I32, ctypes.POINTER(_P)]),
    "agb_server_destroy": (_I32, [_P]),
    "agb_server_add_scene": (_I32, [_P, _I32, _P]),
    "agb_server_set_denoiser": (_I32, [_P, _P]),
    "agb_server_submit": (_I32, [_P, ctypes.POINTER(ServeRequest), ctypes.POINTER(_U64)]),
    "agb_server_wait": (_I32, [_P, _U64, _I32, ctypes.POINTER(ServeResult), _P, _U64]),
    "agb_server_memory": (_I32, [_P, ctypes.POINTER(_U64), ctypes.POINTER(_U64)]),
    "agb_set_counting": (_I32, [_P, _I32]),
    "agb_set_profiling": (_I32, [_P, _I32]),
    "agb_geometry_create": (_I32, [_P, _P, _P, _P, _P, _U32, _U32, ctypes.POINTER(_I32)]),
    "agb_image_create": (_I32, [_P, _P, _U32, _U32, _I32, _I32, ctypes.POINTER(_I32)]),
    "agb_set_bvh_builder": (_I32, [_P, _I32]),
    "agb_geometry_bvh": (_I32, [_P, _I32, _P, _U64, _P, _U64, ctypes.POINTER(_I32), ctypes.POINTER(_I32),
                                ctypes.POINTER(_U32)]),
    "agb_tlas_read": (_I32, [_P, _P, _U64, _P, _U64, ctypes.POINTER(_I32), ctypes.POINTER(_I32),
                             ctypes.POINTER(_U32)]),
    "agb_materials_set": (_I32, [_P, _P, _P, _U32]),
    "agb_material_graphs_set": (_I32, [_P, _P, _P, _U32, _P, _U32, _P, _U32]),
    "agb_instances_set": (_I32, [_P, _P, _U32]),
    "agb_environment_set": (_I32, [_P, _P, _I32, _I32]),
    "agb_ground_plane_set": (_I32, [_P, _P]),
    "agb_environment_alias": (_I32, [_P, _P, _U64, ctypes.POINTER(ctypes.c_double),
                                      ctypes.POINTER(ctypes.c_double)]),
    "agb_set_environment_table": (_I32, [_P, _I32]),
    "agb_environment_alias_build_noalloc": (_I32, [_P, _U32, _U32, _I32, _P,
                                                   ctypes.POINTER(ctypes.c_double),
                                                   ctypes.POINTER(ctypes.c_double), _P]),
    "agb_frame_set": (_I32, [_P, _P]),
    "agb_render": (_I32, [_P, ctypes.POINTER(RenderOptions), _U32, _U32, ctypes.POINTER(RenderStats)]),
    "agb_wait": (_I32, [_P]),
    "agb_batch_create": (_I32, [_I32, _P, _U64, ctypes.POINTER(_P)]),
    "agb_batch_destroy": (_I32, [_P]),
    "agb_batch_render": (_I32, [_P, _P, _P, _P, _P, _U32, _P]),
    "agb_batch_poll": (_I32, [_P]),
    "agb_batch_set_scenes": (_I32, [_P, _P, _U32]),
    "agb_batch_set_profiling": (_I32, [_P, _I32]),
    "agb_accum_read_rect": (_I32, [_P, _I32, _U32, _U32, _U32, _U32, _P, _U64]),
    "agb_accum_read": (_I32, [_P, _I32, _P, _U64]),
    "agb_accum_device": (_I32, [_P, _I32, ctypes.POINTER(_P)]),
    "agb_last_sample_device": (_I32, [_P, ctypes.POINTER(_P)]),
    "agb_post_process": (_I32, [_P, _I32, _P, _I32, _I32, _P, _P]),
    "agb_accum_rel_mse": (_I32, [_P, _I32, _P, ctypes.c_double, ctypes.POINTER(ctypes.c_double)]),
    "agb_aov_read": (_I32, [_P, _P, _P, _P, _P]),
    "agb_aov_device": (_I32, [_P, ctypes.POINTER(AovBuffers)]),
    "agb_temporal_resolve": (_I32, [_P, ctypes.POINTER(TemporalSettings)]),
    "agb_temporal_read": (_I32, [_P, _P, _U64]),
    "agb_temporal_resolve_batch": (_I32, [_P, _P, _P, _P, _U32, _U32,
                                          ctypes.POINTER(TemporalSettings), _P, _P]),
    "agb_temporal_jitter": (None, [_U32, _U32, ctypes.POINTER(ctypes.c_float)]),
    "agb_tc_gemm_bf16": (_I32, [_P, _P, _P, _I32, _I32, _I32, _P]),
    "agb_conv3x3_bf16": (_I32, [_P, _P, _P, _P, _P, _P] + [_I32] * 8 + [_P]),
    "agb_conv3x3_pool_bf16": (_I32, [_P, _P, _P, _P, _P, _P] + [_I32] * 8 + [_P]),
    "agb_pack_conv_weights": (_I32, [_P, _I32, _I32, _I32, _P, _P]),
    "agb_conv3x3_wgrad_bf16": (_I32, [_P, _P, _P, _P] + [_I32] * 7 + [_P]),
    "agb_denoiser_create": (_I32, [_I32, _P, _U64, ctypes.POINTER(_P)]),
    "agb_denoiser_destroy": (_I32, [_P]),
    "agb_denoiser_param_count": (_I32, [ctypes.POINTER(_U64)]),
    "agb_denoiser_params": (_I32, [_P, _P, _U64]),
    "agb_denoiser_set_params": (_I32, [_P, _P, _U64]),
    "agb_denoiser_grads": (_I32, [_P, _P, _U64]),
    "agb_denoiser_forward": (_I32, [_P, _P, _I32, _I32, _I32, _P]),
    "agb_denoiser_train_step": (_I32, [_P, _P, _P, _I32, _I32, _I32, ctypes.c_float, _I32,
                                       ctypes.POINTER(ctypes.c_float)]),
    "agb_denoiser_features": (_I32, [_P, _P]),
    "agb_bsdf_batch": (_I32, [_I32, _P, _P, _P, _P, _P, _P, _I64, _P, _P, _P, _P, _P]),
    "agb_intersect_batch": (_I32, [_P, _P, _I64, _I32, _P, _P]),
    "agb_env_sample_batch": (_I32, [_P, _P, _I64, _P, _P, _P]),
    "agb_random_stream": (_I32, [_U32, _U32, _U32, _U32, _I32, _P, _P]),
    "agb_version": (ctypes.c_char_p, []),
}

_lib = None


class AgbError(RuntimeError):
    def __init__(self, code, message):
        super().__init__(f"{ERRORS.get(code, code)}: {message}")
        self.code = code


def library(path=None):
    """Loads libagb_cuda.so (raises if it has not been built)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(
            f"{p} is missing: build the CUDA extension first (python -c 'import __graft_entry__ "
            f"as g; g.build()')")
    lib = ctypes.CDLL(p)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def check(code):
    if code != AGB_OK:
        raise AgbError(code, library().agb_last_error().decode())
    return code


def ptr(a):
    """ctypes void pointer of a numpy array (None passes through)."""
    if a is None:
        return None
    return ctypes.c_void_p(a.ctypes.data)
