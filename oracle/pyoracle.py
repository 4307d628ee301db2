"""Oracle (test infrastructure): ctypes binding of oracle/_build/liboracle.so, the CPU restatement
of Aurora's path tracer.  Only the tests, the smoke check and bench.py's CPU-baseline leg import
this module; the product never does.

Scenes come from aurora_gb300.scenes.SceneDesc, converted to the oracle's own structs.  RGBA8
images are expanded to float as texel / 255 (FP32), RGB32F images get alpha 1, exactly as the
product's upload does.  The environment alias table is the reference's FP32 AliasMap::build
restated (pinned bit-for-bit against the reference source by the tests).
"""
import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import build_oracle  # noqa: E402

_lib = None


def mx_noise(kind, xyz, precision=32):
    """The oracle's MaterialX noise (kind 0 Perlin 2D, 1 Perlin 3D, 2 cell 2D, 3 cell 3D) at (n, 3)
    float32 points; float64 results (FP32 values exactly when precision is 32)."""
    xyz = np.ascontiguousarray(xyz, np.float32)
    out = np.zeros(len(xyz), np.float64)
    lib().orc_mx_noise(precision, kind, xyz.ctypes.data, len(xyz), out.ctypes.data)
    return out


def lib():
    global _lib
    if _lib is None:
        path = build_oracle.build_oracle()
        L = ctypes.CDLL(path)
        P = ctypes.c_void_p
        L.orc_layout.restype = ctypes.c_int
        L.orc_layout.argtypes = [ctypes.c_int]
        L.orc_random_stream.argtypes = [ctypes.c_uint32] * 4 + [ctypes.c_int, P]
        L.orc_mx_noise.argtypes = [ctypes.c_int, ctypes.c_int, P, ctypes.c_int64, P]
        L.orc_bsdf_batch.argtypes = [ctypes.c_int, ctypes.c_int, P, P, P, P, P, P, ctypes.c_int64,
                                     P, P, P, P]
        L.orc_alias_build.argtypes = [ctypes.c_int, P, ctypes.c_uint32, ctypes.c_uint32, P,
                                      ctypes.POINTER(ctypes.c_double)]
        L.orc_env_sample.argtypes = [ctypes.c_int, P, P, P, P, ctypes.c_int64, P, P, P]
        L.orc_env_evaluate.argtypes = [P, P, P, P, P, ctypes.c_int64, P]
        L.orc_intersect.argtypes = [ctypes.c_int, P, P, ctypes.c_int64, ctypes.c_int, ctypes.c_int,
                                    P, P]
        L.orc_render.restype = ctypes.c_double
        L.orc_render.argtypes = [ctypes.c_int, P, P, ctypes.c_uint32, ctypes.c_uint32,
                                 ctypes.c_uint32, ctypes.c_uint32, ctypes.c_int, ctypes.c_int, P, P,
                                 P, P, P]
        L.orc_post_process.argtypes = [P, ctypes.c_int64, P, ctypes.c_int, ctypes.c_int, P]
        L.orc_tracer_create.restype = P
        L.orc_tracer_create.argtypes = [ctypes.c_int, P, P, ctypes.c_uint32, ctypes.c_uint32,
                                        ctypes.c_int]
        L.orc_tracer_destroy.argtypes = [P]
        L.orc_fmath.argtypes = [ctypes.c_int, P, P, ctypes.c_int64, P]
        L.orc_tracer_set_aov.argtypes = [P, P, P, P, P]
        L.orc_tracer_set_seed_offset.argtypes = [P, ctypes.c_uint32]
        L.orc_tracer_set_ground_plane.argtypes = [P, P]
        L.orc_temporal_resolve.argtypes = [ctypes.c_int, P, P, P, P, ctypes.c_int, ctypes.c_int,
                                           ctypes.c_uint32, ctypes.c_float, ctypes.c_float,
                                           ctypes.c_float, P]
        L.orc_temporal_jitter.argtypes = [ctypes.c_uint32, ctypes.c_uint32, P]
        L.orc_tracer_render.restype = ctypes.c_double
        L.orc_tracer_render.argtypes = [P, P, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_int, P, P,
                                        P, P, P]
        _lib = L
    return _lib


_ref_lib = False


def ref_lib():
    """The reference's own shader functions compiled as host C++ (oracle/_ref/libshaders_ref.so,
    built from the reference tree by build_oracle.build_reference_shaders), or None where the
    reference tree is absent."""
    global _ref_lib
    if _ref_lib is False:
        path = build_oracle.build_reference_shaders()
        if path is None:
            _ref_lib = None
        else:
            L = ctypes.CDLL(path)
            P = ctypes.c_void_p
            for prec in (32, 64):
                getattr(L, f"ref{prec}_bsdf_batch").argtypes = [ctypes.c_int, ctypes.c_int, P, P, P, P,
                                                                P, P, ctypes.c_int64, P, P, P, P]
                getattr(L, f"ref{prec}_env_sample").argtypes = [P, P, ctypes.c_uint32, ctypes.c_uint32,
                                                                P, P, ctypes.c_int64, P, P, P]
                getattr(L, f"ref{prec}_env_evaluate").argtypes = [P, P, ctypes.c_uint32, ctypes.c_uint32,
                                                                  P, ctypes.c_uint32, ctypes.c_uint32,
                                                                  ctypes.c_int, P, P, ctypes.c_int64, P]
                getattr(L, f"ref{prec}_random_stream").argtypes = [ctypes.c_uint32] * 4 + [ctypes.c_int, P]
            _ref_lib = L
    return _ref_lib


def ref_bsdf_batch(op, mats, mat_index, frames, V, L, rnd, precision=32, denoising_aovs=False):
    """StandardSurfaceBSDF.slang's evaluateMaterial (op 0), sampleMaterial (1) and
    evaluateMaterialAndPDF (2) from the reference source itself, FP32 or FP64."""
    n = len(mat_index)
    val = np.zeros((n, 3), np.float32)
    d = np.zeros((n, 3), np.float32)
    pdf = np.zeros(n, np.float32)
    lobe = np.zeros(n, np.int32)
    c = np.ascontiguousarray
    getattr(ref_lib(), f"ref{precision}_bsdf_batch")(
        op, 1 if denoising_aovs else 0, _p(c(mats)), _p(c(mat_index, np.int32)),
        _p(c(frames, np.float32)), _p(c(V, np.float32)),
        _p(None if L is None else c(L, np.float32)), _p(None if rnd is None else c(rnd, np.float32)),
        n, _p(val), _p(d), _p(pdf), _p(lobe))
    return val, d, pdf, lobe


def ref_env_sample(env, light_rgba, alias, rnd, precision=32):
    """Environment.slang's sampleEnvironment from the reference source."""
    light_rgba = np.ascontiguousarray(light_rgba, np.float32)
    h, w = light_rgba.shape[:2]
    n = len(rnd)
    r = np.zeros((n, 3), np.float32)
    d = np.zeros((n, 3), np.float32)
    pdf = np.zeros(n, np.float32)
    getattr(ref_lib(), f"ref{precision}_env_sample")(
        _p(np.ascontiguousarray(env)), _p(light_rgba), w, h, _p(np.ascontiguousarray(alias)),
        _p(np.ascontiguousarray(rnd, np.float32)), n, _p(r), _p(d), _p(pdf))
    return r, d, pdf


def ref_env_evaluate(env, light_rgba, background_rgba, dirs, as_background, linear=False,
                     precision=32):
    """Environment.slang's evaluateEnvironment from the reference source."""
    light_rgba = np.ascontiguousarray(light_rgba, np.float32)
    background_rgba = np.ascontiguousarray(background_rgba, np.float32)
    n = len(dirs)
    out = np.zeros((n, 3), np.float32)
    getattr(ref_lib(), f"ref{precision}_env_evaluate")(
        _p(np.ascontiguousarray(env)), _p(light_rgba), light_rgba.shape[1], light_rgba.shape[0],
        _p(background_rgba), background_rgba.shape[1], background_rgba.shape[0], 1 if linear else 0,
        _p(np.ascontiguousarray(dirs, np.float32)), _p(np.ascontiguousarray(as_background, np.int32)),
        n, _p(out))
    return out


def ref_random_stream(sample_index, width, px, py, n):
    """Random.slang's pcg2DInit + random2D from the reference source (FP32)."""
    out = np.zeros((n, 2), np.float32)
    ref_lib().ref32_random_stream(sample_index, width, px, py, n, _p(out))
    return out


def _p(a):
    return None if a is None else ctypes.c_void_p(a.ctypes.data)


class Mesh(ctypes.Structure):
    _fields_ = [("positions", ctypes.c_void_p), ("normals", ctypes.c_void_p),
                ("texcoords", ctypes.c_void_p), ("indices", ctypes.c_void_p),
                ("vertexCount", ctypes.c_uint32), ("triangleCount", ctypes.c_uint32)]


class Layer(ctypes.Structure):
    _fields_ = [("material", ctypes.c_int32), ("texcoords", ctypes.c_void_p)]


class Instance(ctypes.Structure):
    _fields_ = [("mesh", ctypes.c_int32), ("material", ctypes.c_int32),
                ("objectToWorld", ctypes.c_float * 12), ("layerCount", ctypes.c_int32),
                ("layers", ctypes.c_void_p)]


class Image(ctypes.Structure):
    _fields_ = [("rgba", ctypes.c_void_p), ("width", ctypes.c_uint32), ("height", ctypes.c_uint32),
                ("linear", ctypes.c_int32)]


class Scene(ctypes.Structure):
    _fields_ = [("meshes", ctypes.c_void_p), ("meshCount", ctypes.c_int32),
                ("instances", ctypes.c_void_p), ("instanceCount", ctypes.c_int32),
                ("materials", ctypes.c_void_p), ("materialCount", ctypes.c_int32),
                ("materialTextures", ctypes.c_void_p), ("images", ctypes.c_void_p),
                ("imageCount", ctypes.c_int32), ("env", ctypes.c_void_p),
                ("envLight", ctypes.c_void_p), ("envBackground", ctypes.c_void_p),
                ("envAlias", ctypes.c_void_p), ("graphFirst", ctypes.c_void_p),
                ("graphCount", ctypes.c_void_p), ("graphOps", ctypes.c_void_p),
                ("graphConsts", ctypes.c_void_p)]


def image_to_rgba32f(im):
    px = im["pixels"]
    fmt = im["format"]
    if fmt == 0:  # RGBA8 UNORM
        return (px.astype(np.float32) / np.float32(255.0)).astype(np.float32)
    if fmt == 2:  # RGB32F
        out = np.ones(px.shape[:2] + (4,), np.float32)
        out[..., :3] = px
        return out
    return np.ascontiguousarray(px, np.float32)


def alias_build(rgb, precision=32):
    """AliasMap::build restated; returns (entries as structured array, integral)."""
    h, w = rgb.shape[:2]
    out = np.zeros(w * h, dtype=[("alias", "<u4"), ("prob", "<f4"), ("pdf", "<f4"), ("_p", "<f4")])
    integ = ctypes.c_double()
    rgb = np.ascontiguousarray(rgb[..., :3], np.float32)
    lib().orc_alias_build(precision, _p(rgb), w, h, _p(out), ctypes.byref(integ))
    return out, integ.value


class OracleScene:
    """Holds the oracle-side copy of a SceneDesc (and keeps its buffers alive)."""

    def __init__(self, s, alias=None, integral=None):
        """alias / integral: an environment table to sample with instead of the reference's
        (the device's table makes the two renders sample-identical)."""
        self.desc = s
        self._keep = []
        meshes = (Mesh * len(s.meshes))()
        for k, m in enumerate(s.meshes):
            meshes[k].positions = m["positions"].ctypes.data
            meshes[k].normals = None if m["normals"] is None else m["normals"].ctypes.data
            meshes[k].texcoords = None if m["texcoords"] is None else m["texcoords"].ctypes.data
            meshes[k].indices = m["indices"].ctypes.data
            meshes[k].vertexCount = len(m["positions"])
            meshes[k].triangleCount = len(m["indices"]) // 3
        insts = (Instance * len(s.instances))()
        for k, inst in enumerate(s.instances):
            insts[k].mesh = inst["mesh"]
            insts[k].material = inst["material"]
            insts[k].objectToWorld[:] = [float(x) for x in inst["xform"]]
            layers = inst.get("layers") or []
            insts[k].layerCount = len(layers)
            if layers:
                arr = (Layer * len(layers))()
                for j, (mat, uv) in enumerate(layers):
                    arr[j].material = mat
                    arr[j].texcoords = uv.ctypes.data
                self._keep.append(arr)
                insts[k].layers = ctypes.cast(arr, ctypes.c_void_p)
        rgba = [image_to_rgba32f(im) for im in s.images]
        imgs = (Image * max(1, len(rgba)))()
        for k, (im, px) in enumerate(zip(s.images, rgba)):
            imgs[k].rgba = px.ctypes.data
            imgs[k].width = im["width"]
            imgs[k].height = im["height"]
            imgs[k].linear = im["linear"]
        self.materials = np.ascontiguousarray(s.materials)
        self.textures = None if s.textures is None else np.ascontiguousarray(s.textures)
        self.env = np.ascontiguousarray(s.env).reshape(1).copy()
        self.alias = None
        if s.env_light >= 0:
            light = s.images[s.env_light]
            src = light["pixels"][..., :3] if light["format"] != 0 else rgba[s.env_light][..., :3]
            if alias is None:
                self.alias, integral = alias_build(np.ascontiguousarray(src, np.float32))
            else:
                self.alias = np.ascontiguousarray(alias).copy()
            self.env["light_tex_luminance_integral"] = integral
            self.env["has_light_tex"] = 1
        self.env["has_background_tex"] = 1 if s.env_background >= 0 else 0
        sc = Scene()
        sc.meshes = ctypes.cast(meshes, ctypes.c_void_p)
        sc.meshCount = len(s.meshes)
        sc.instances = ctypes.cast(insts, ctypes.c_void_p)
        sc.instanceCount = len(s.instances)
        sc.materials = self.materials.ctypes.data
        sc.materialCount = len(self.materials)
        sc.materialTextures = None if self.textures is None else self.textures.ctypes.data
        sc.images = ctypes.cast(imgs, ctypes.c_void_p)
        sc.imageCount = len(rgba)
        sc.env = self.env.ctypes.data
        sc.envLight = ctypes.addressof(imgs[s.env_light]) if s.env_light >= 0 else None
        sc.envBackground = ctypes.addressof(imgs[s.env_background]) if s.env_background >= 0 else None
        sc.envAlias = None if self.alias is None else self.alias.ctypes.data
        g = getattr(s, "graphs", None)
        if g is not None:
            gf = np.ascontiguousarray(g["first"], np.int32)
            gc = np.ascontiguousarray(g["count"], np.int32)
            gops = np.ascontiguousarray(g["ops"])
            gk = np.ascontiguousarray(g["consts"], np.float32).reshape(-1)
            sc.graphFirst, sc.graphCount = gf.ctypes.data, gc.ctypes.data
            sc.graphOps, sc.graphConsts = gops.ctypes.data, (gk.ctypes.data if gk.size else None)
            self._keep += [gf, gc, gops, gk]
        self._keep += [meshes, insts, imgs, rgba]
        self.scene = sc
        self.frame = np.ascontiguousarray(s.frame).reshape(1).copy()

    def tracer(self, precision=32, brute=False):
        """Builds (once) the oracle's BVHs for this scene and precision."""
        key = (precision, brute)
        if not hasattr(self, "_tracers"):
            self._tracers = {}
        if key not in self._tracers:
            t = lib().orc_tracer_create(precision, ctypes.byref(self.scene), _p(self.frame),
                                        self.desc.width, self.desc.height, 1 if brute else 0)
            gp = getattr(self.desc, "ground_plane", None)
            if gp is not None:
                self._ground = np.ascontiguousarray(gp).reshape(1).copy()
                lib().orc_tracer_set_ground_plane(t, _p(self._ground))
            self._tracers[key] = t
        return self._tracers[key]

    def close(self):
        for t in getattr(self, "_tracers", {}).values():
            lib().orc_tracer_destroy(t)
        self._tracers = {}

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def render(self, sample_start, sample_count, precision=32, threads=None, brute=False,
               want_mean=True, want_sum=False, want_last=False, rect=None, frame=None,
               want_aov=False, seed_offset=0):
        """Renders with the oracle.  want_aov: also return the denoising AOVs of the last sample
        (the frame must enable them); seed_offset: added to the sample index seeding the random
        streams."""
        s = self.desc
        t = self.tracer(precision, brute)
        lib().orc_tracer_set_seed_offset(t, seed_offset)
        aov = None
        if want_aov:
            aov = dict(depth_view=np.zeros((s.height, s.width), np.float32),
                       normal_roughness=np.zeros((s.height, s.width, 4), np.float32),
                       base_color_metalness=np.zeros((s.height, s.width, 4), np.float32),
                       motion=np.zeros((s.height, s.width, 4), np.float32))
            lib().orc_tracer_set_aov(t, _p(aov["depth_view"]), _p(aov["normal_roughness"]),
                                     _p(aov["base_color_metalness"]), _p(aov["motion"]))
        try:
            out = self._render(sample_start, sample_count, precision, threads, brute, want_mean,
                               want_sum, want_last, rect, frame)
        finally:
            if want_aov:
                lib().orc_tracer_set_aov(t, None, None, None, None)
        if want_aov:
            out["aov"] = aov
        return out

    def _render(self, sample_start, sample_count, precision, threads, brute, want_mean, want_sum,
                want_last, rect, frame):
        s = self.desc
        n = s.width * s.height * 4
        mean = np.zeros(n, np.float32) if want_mean else None
        acc = np.zeros(n, np.float64) if want_sum else None
        last = np.zeros(n, np.float32) if want_last else None
        stats = np.zeros(2, np.uint64)
        r = None if rect is None else np.asarray(rect, np.uint32)
        f = None if frame is None else np.ascontiguousarray(frame).reshape(1)
        if f is not None:
            self._frame_keep = f
        threads = threads or os.cpu_count() or 1
        secs = lib().orc_tracer_render(self.tracer(precision, brute), _p(f), sample_start,
                                       sample_count, threads, _p(mean), _p(acc), _p(last),
                                       _p(stats), _p(r))
        shape = (s.height, s.width, 4)
        out = dict(seconds=secs, rays=int(stats[0]), shadow_rays=int(stats[1]))
        if want_mean:
            out["mean"] = mean.reshape(shape)
        if want_sum:
            out["sum"] = acc.reshape(shape)
        if want_last:
            out["last"] = last.reshape(shape)
        return out

    def intersect(self, rays, any_hit=False, precision=32, brute=False):
        rays = np.ascontiguousarray(rays, np.float32)
        n = len(rays)
        tuv = np.zeros((n, 3), np.float32)
        ip = np.zeros((n, 2), np.int32)
        lib().orc_intersect(precision, ctypes.byref(self.scene), _p(rays), n, 1 if any_hit else 0,
                            1 if brute else 0, _p(tuv), _p(ip))
        return tuv, ip


def bsdf_batch(op, mats, mat_index, frames, V, L, rnd, precision=32):
    n = len(mat_index)
    val = np.zeros((n, 3), np.float32)
    d = np.zeros((n, 3), np.float32)
    pdf = np.zeros(n, np.float32)
    lobe = np.zeros(n, np.int32)
    c = np.ascontiguousarray
    lib().orc_bsdf_batch(op, precision, _p(c(mats)), _p(c(mat_index, np.int32)),
                         _p(c(frames, np.float32)), _p(c(V, np.float32)),
                         _p(None if L is None else c(L, np.float32)),
                         _p(None if rnd is None else c(rnd, np.float32)), n, _p(val), _p(d),
                         _p(pdf), _p(lobe))
    return val, d, pdf, lobe


def random_stream(sample_index, width, px, py, n):
    out = np.zeros((n, 2), np.float32)
    lib().orc_random_stream(sample_index, width, px, py, n, _p(out))
    return out


def env_sample(env, light_rgba, alias, rnd, linear=False, precision=32):
    img = Image()
    img.rgba = light_rgba.ctypes.data
    img.height, img.width = light_rgba.shape[:2]
    img.linear = 1 if linear else 0
    n = len(rnd)
    r = np.zeros((n, 3), np.float32)
    d = np.zeros((n, 3), np.float32)
    pdf = np.zeros(n, np.float32)
    lib().orc_env_sample(precision, _p(env), ctypes.byref(img), _p(alias),
                         _p(np.ascontiguousarray(rnd, np.float32)), n, _p(r), _p(d), _p(pdf))
    return r, d, pdf


def post_process(accum, brightness=(1.0, 1.0, 1.0), tone_map=False, gamma=True):
    a = np.ascontiguousarray(accum, np.float32)
    out = np.zeros_like(a)
    b = np.asarray(brightness, np.float32)
    lib().orc_post_process(_p(a), a.size // 4, _p(b), 1 if tone_map else 0, 1 if gamma else 0,
                           _p(out))
    return out


def fmath(which, x, y=None):
    """Evaluates one of agb_fmath.h's functions (0 sin, 1 cos, 2 exp2, 3 log2, 4 pow, 5 atan2,
    6 asin) on float32 inputs."""
    x = np.ascontiguousarray(x, np.float32)
    y = None if y is None else np.ascontiguousarray(y, np.float32)
    out = np.zeros_like(x)
    lib().orc_fmath(which, _p(x), _p(y), len(x), _p(out))
    return out


def temporal_resolve(accum, history, motion, depth_view, reset=False, alpha_min=1.0 / 16.0,
                     alpha_max=0.6, speed_reference=6.0, precision=32):
    """TemporalResolve.hlsl over whole (H, W, 4) images; depth_view (H, W)."""
    accum = np.ascontiguousarray(accum, np.float32)
    history = np.ascontiguousarray(history, np.float32)
    motion = np.ascontiguousarray(motion, np.float32)
    depth_view = np.ascontiguousarray(depth_view, np.float32)
    h, w = accum.shape[:2]
    out = np.zeros((h, w, 4), np.float32)
    lib().orc_temporal_resolve(precision, _p(accum), _p(history), _p(motion), _p(depth_view), w, h,
                               1 if reset else 0, alpha_min, alpha_max, speed_reference, _p(out))
    return out


def temporal_jitter(frame_index, phase_count=0):
    out = np.zeros(2, np.float32)
    lib().orc_temporal_jitter(frame_index, phase_count, _p(out))
    return float(out[0]), float(out[1])


def rel_mse(x, ref, eps=1e-2):
    """mean over pixels and RGB of (x - r)^2 / (r^2 + eps)."""
    x = np.asarray(x, np.float64)[..., :3]
    r = np.asarray(ref, np.float64)[..., :3]
    return float(np.mean((x - r) ** 2 / (r * r + eps)))
