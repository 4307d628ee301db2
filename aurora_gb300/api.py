"""Python host mirror of the renderer boundary, over the C ABI (include/agb.h).

`Renderer` uploads a SceneDesc (aurora_gb300.scenes) through the same calls Aurora's C++ backend
classes make -- geometry, images, materials, instances, environment, frame data -- then renders and
reads back, mirroring IRenderer::render(sampleStart, sampleCount) and IRenderBuffer::data()
(Aurora.h:714-751, 1196).  Errors from the library raise AgbError; there is no CPU path.
"""
import ctypes

import numpy as np

from . import _abi
from ._abi import check, library, ptr


class Renderer:
    def __init__(self, device=0, stream=None):
        self._lib = library()
        h = ctypes.c_void_p()
        check(self._lib.agb_context_create(device, stream, ctypes.byref(h)))
        self.ctx = h
        self.scene = None
        self._keep = []

    def close(self):
        if self.ctx:
            self._lib.agb_context_destroy(self.ctx)
            self.ctx = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ------------------------------------------------------------------------- scene upload
    def upload_geometry_only(self, s):
        """Creates the scene's meshes (BLAS builds) and nothing else; returns their handles."""
        self.scene = s
        out = []
        for m in s.meshes:
            g = ctypes.c_int32()
            check(self._lib.agb_geometry_create(self.ctx, ptr(m["positions"]), ptr(m["normals"]),
                                                ptr(m["texcoords"]), ptr(m["indices"]),
                                                len(m["positions"]), len(m["indices"]),
                                                ctypes.byref(g)))
            out.append(g.value)
        return out

    def upload(self, s):
        """Uploads a scenes.SceneDesc: the equivalent of IScene construction + the first update."""
        lib = self._lib
        geo = []
        for m in s.meshes:
            g = ctypes.c_int32()
            check(lib.agb_geometry_create(self.ctx, ptr(m["positions"]), ptr(m["normals"]),
                                          ptr(m["texcoords"]), ptr(m["indices"]),
                                          len(m["positions"]), len(m["indices"]), ctypes.byref(g)))
            geo.append(g.value)
        imgs = []
        for im in s.images:
            g = ctypes.c_int32()
            check(lib.agb_image_create(self.ctx, ptr(im["pixels"]), im["width"], im["height"],
                                       im["format"], im["linear"], ctypes.byref(g)))
            imgs.append(g.value)
        mats = np.ascontiguousarray(s.materials)
        tex = None if s.textures is None else np.ascontiguousarray(s.textures)
        check(lib.agb_materials_set(self.ctx, ptr(mats), ptr(tex), len(mats)))
        g = getattr(s, "graphs", None)
        if g is not None:
            first = np.ascontiguousarray(g["first"], np.int32)
            count = np.ascontiguousarray(g["count"], np.int32)
            ops = np.ascontiguousarray(g["ops"], _abi.GRAPH_OP_DTYPE).copy()
            img_op = ops["op"] == _abi.GOP_IMAGE
            ops["imm"][img_op] = np.asarray(imgs, np.uint16)[ops["imm"][img_op]] if img_op.any() else 0
            consts = np.ascontiguousarray(g["consts"], np.float32).reshape(-1, 4)
            check(lib.agb_material_graphs_set(self.ctx, ptr(first), ptr(count), len(first), ptr(ops), len(ops),
                                              ptr(consts), len(consts)))
        insts = (_abi.Instance * len(s.instances))()
        layer_arrays = []
        for k, inst in enumerate(s.instances):
            insts[k].geometry = geo[inst["mesh"]]
            insts[k].material = inst["material"]
            insts[k].object_to_world[:] = [float(x) for x in inst["xform"]]
            layers = inst.get("layers") or []
            insts[k].layer_count = len(layers)
            if layers:
                arr = (_abi.Layer * len(layers))()
                for j, (mat, uv) in enumerate(layers):
                    arr[j].material = mat
                    arr[j].texcoords = uv.ctypes.data
                layer_arrays.append(arr)
                insts[k].layers = ctypes.cast(arr, ctypes.c_void_p)
        check(lib.agb_instances_set(self.ctx, insts, len(s.instances)))
        env = np.ascontiguousarray(s.env).copy()
        check(lib.agb_environment_set(self.ctx, ptr(env.reshape(1)),
                                      imgs[s.env_light] if s.env_light >= 0 else -1,
                                      imgs[s.env_background] if s.env_background >= 0 else -1))
        gp = getattr(s, "ground_plane", None)
        gp = None if gp is None else np.ascontiguousarray(
            np.asarray(gp, dtype=_abi.GROUND_PLANE_DTYPE).reshape(1))
        check(lib.agb_ground_plane_set(self.ctx, ptr(gp)))
        self.set_frame(s.frame)
        self.scene = s

    def set_frame(self, frame):
        f = np.ascontiguousarray(np.asarray(frame, dtype=_abi.FRAME_DTYPE).reshape(1))
        check(self._lib.agb_frame_set(self.ctx, ptr(f)))

    # --------------------------------------------------------------------------- rendering
    def render(self, sample_start, sample_count, width=None, height=None,
               accumulation=_abi.ACCUM_RUNNING_MEAN | _abi.ACCUM_KAHAN, max_paths=0, stats=False,
               seed_offset=0):
        opt = _abi.RenderOptions()
        opt.seed_offset = seed_offset
        opt.width = width or self.scene.width
        opt.height = height or self.scene.height
        opt.accumulation = accumulation
        opt.max_paths_in_flight = max_paths
        st = _abi.RenderStats() if stats else None
        check(self._lib.agb_render(self.ctx, ctypes.byref(opt), sample_start, sample_count,
                                   ctypes.byref(st) if st is not None else None))
        if stats:
            out = {f: getattr(st, f) for f, _ in _abi.RenderStats._fields_}
            out["kernel_ms"] = dict(zip(_abi.KERNEL_FAMILIES, list(st.kernel_ms)))
            out["kernel_count"] = dict(zip(_abi.KERNEL_FAMILIES, list(st.kernel_count)))
            out["closest_rays_per_bounce"] = list(st.closest_rays_per_bounce)
            out["shadow_rays_per_bounce"] = list(st.shadow_rays_per_bounce)
            return out
        return None

    def wait(self):
        check(self._lib.agb_wait(self.ctx))

    def set_counting(self, enabled):
        check(self._lib.agb_set_counting(self.ctx, 1 if enabled else 0))

    def set_profiling(self, enabled):
        check(self._lib.agb_set_profiling(self.ctx, 1 if enabled else 0))

    def read_rect(self, rect, mode=_abi.ACCUM_KAHAN):
        """The accumulated image over rect = (x0, y0, x1, y1) (agb_accum_read_rect)."""
        x0, y0, x1, y1 = (int(v) for v in rect)
        out = np.empty((y1 - y0, x1 - x0, 4), np.float32)
        check(self._lib.agb_accum_read_rect(self.ctx, mode, x0, y0, x1 - x0, y1 - y0, ptr(out), out.size))
        return out

    def read(self, mode=_abi.ACCUM_RUNNING_MEAN, width=None, height=None, out=None):
        w = width or self.scene.width
        h = height or self.scene.height
        if out is None:
            out = np.empty((h, w, 4), np.float32)
        check(self._lib.agb_accum_read(self.ctx, mode, ptr(out), out.size))
        return out

    def accum_device_ptr(self, mode=_abi.ACCUM_RUNNING_MEAN):
        p = ctypes.c_void_p()
        check(self._lib.agb_accum_device(self.ctx, mode, ctypes.byref(p)))
        return p.value

    def post_process(self, mode=_abi.ACCUM_RUNNING_MEAN, brightness=(1.0, 1.0, 1.0),
                     tone_map=False, gamma=True):
        w, h = self.scene.width, self.scene.height
        o32 = np.empty((h, w, 4), np.float32)
        o8 = np.empty((h, w, 4), np.uint8)
        b = np.asarray(brightness, np.float32)
        check(self._lib.agb_post_process(self.ctx, mode, ptr(b), 1 if tone_map else 0,
                                         1 if gamma else 0, ptr(o32), ptr(o8)))
        return o32, o8

    def aovs(self, width=None, height=None):
        """Denoising AOVs of the last render (frame with is_denoising_aovs_enabled): dict of
        depth_view (H, W), normal_roughness, base_color_metalness, motion (H, W, 4)."""
        w = width or self.scene.width
        h = height or self.scene.height
        out = dict(depth_view=np.empty((h, w), np.float32),
                   normal_roughness=np.empty((h, w, 4), np.float32),
                   base_color_metalness=np.empty((h, w, 4), np.float32),
                   motion=np.empty((h, w, 4), np.float32))
        check(self._lib.agb_aov_read(self.ctx, ptr(out["depth_view"]), ptr(out["normal_roughness"]),
                                     ptr(out["base_color_metalness"]), ptr(out["motion"])))
        return out

    def temporal_resolve(self, reset=False, alpha_min=1.0 / 16.0, alpha_max=0.6, speed_reference=6.0):
        """Temporal resolve of the last render against the previous resolve."""
        st = _abi.TemporalSettings(1 if reset else 0, alpha_min, alpha_max, speed_reference)
        check(self._lib.agb_temporal_resolve(self.ctx, ctypes.byref(st)))

    def temporal_read(self, width=None, height=None):
        w = width or self.scene.width
        h = height or self.scene.height
        out = np.empty((h, w, 4), np.float32)
        check(self._lib.agb_temporal_read(self.ctx, ptr(out), out.size))
        return out

    def memory_bytes(self):
        b = ctypes.c_uint64()
        check(self._lib.agb_context_memory(self.ctx, ctypes.byref(b)))
        return b.value

    def set_environment_table(self, layout):
        """_abi.ENV_TABLE_REFERENCE (default) or _abi.ENV_TABLE_FP64; applies to the next upload."""
        check(self._lib.agb_set_environment_table(self.ctx, layout))

    def environment_alias(self, fp64_integral=False):
        """(table, integral the shading divides by[, FP64 integral])."""
        s = self.scene
        im = s.images[s.env_light]
        n = im["width"] * im["height"]
        out = np.zeros(n, dtype=_abi.ALIAS_DTYPE)
        integral = ctypes.c_double()
        i64 = ctypes.c_double()
        check(self._lib.agb_environment_alias(self.ctx, ptr(out), n, ctypes.byref(integral),
                                              ctypes.byref(i64)))
        if fp64_integral:
            return out, integral.value, i64.value
        return out, integral.value

    # ------------------------------------------------------------- unit entry points (device)
    def intersect(self, rays_dev_ptr, n, any_hit, out_tuv_ptr, out_ip_ptr):
        check(self._lib.agb_intersect_batch(self.ctx, ctypes.c_void_p(rays_dev_ptr), n,
                                            1 if any_hit else 0, ctypes.c_void_p(out_tuv_ptr),
                                            ctypes.c_void_p(out_ip_ptr)))

    def env_sample(self, rnd_ptr, n, out_r, out_d, out_pdf):
        check(self._lib.agb_env_sample_batch(self.ctx, ctypes.c_void_p(rnd_ptr), n,
                                             ctypes.c_void_p(out_r), ctypes.c_void_p(out_d),
                                             ctypes.c_void_p(out_pdf)))


def bsdf_batch(op, mats_ptr, idx_ptr, frames_ptr, v_ptr, l_ptr, rnd_ptr, n, out_value, out_dir,
               out_pdf, out_lobe, stream=None):
    """Device-array BSDF batch (agb_bsdf_batch); all arguments are device pointers (ints)."""
    vp = lambda x: None if x is None else ctypes.c_void_p(x)  # noqa: E731
    check(library().agb_bsdf_batch(op, vp(mats_ptr), vp(idx_ptr), vp(frames_ptr), vp(v_ptr),
                                   vp(l_ptr), vp(rnd_ptr), n, vp(out_value), vp(out_dir),
                                   vp(out_pdf), vp(out_lobe), stream))


class View(Renderer):
    """A view of an uploaded Renderer's scene (agb_view_create): its own stream, frame data and
    render buffers; destroy views before their Renderer."""

    def __init__(self, renderer, stream=None):
        self._lib = library()
        h = ctypes.c_void_p()
        check(self._lib.agb_view_create(renderer.ctx, stream, ctypes.byref(h)))
        self.ctx = h
        self.scene = renderer.scene
        self._keep = []


class Batch:
    """Batched rendering (agb_batch_*): several views or renderers, of one or several scenes and
    resolutions, rendered by one wavefront (one launch per stage for all of them)."""

    def __init__(self, max_paths=1 << 24, device=0, stream=None):
        self._lib = library()
        self.handle = ctypes.c_void_p()
        check(self._lib.agb_batch_create(device, stream, int(max_paths), ctypes.byref(self.handle)))

    def close(self):
        if self.handle:
            self._lib.agb_batch_destroy(self.handle)
            self.handle = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def render(self, items, stats=False):
        """items: dicts with keys view (a Renderer or View with its frame set), width, height, spp,
        and optionally start (0), seed_offset (0), accumulation (running mean | Kahan)."""
        n = len(items)
        views = (ctypes.c_void_p * n)(*[it["view"].ctx.value if isinstance(it["view"].ctx, ctypes.c_void_p)
                                        else it["view"].ctx for it in items])
        opts = (_abi.RenderOptions * n)()
        starts = (ctypes.c_uint32 * n)()
        counts = (ctypes.c_uint32 * n)()
        for k, it in enumerate(items):
            opts[k].width, opts[k].height = it["width"], it["height"]
            opts[k].accumulation = it.get("accumulation", _abi.ACCUM_RUNNING_MEAN | _abi.ACCUM_KAHAN)
            opts[k].seed_offset = it.get("seed_offset", 0)
            starts[k] = it.get("start", 0)
            counts[k] = it["spp"]
        st = _abi.RenderStats() if stats else None
        check(self._lib.agb_batch_render(self.handle, views, opts, starts, counts, n,
                                         ctypes.byref(st) if st is not None else None))
        if stats:
            out = {f: getattr(st, f) for f, _ in _abi.RenderStats._fields_}
            out["kernel_ms"] = dict(zip(_abi.KERNEL_FAMILIES, list(st.kernel_ms)))
            out["kernel_count"] = dict(zip(_abi.KERNEL_FAMILIES, list(st.kernel_count)))
            out["closest_rays_per_bounce"] = list(st.closest_rays_per_bounce)
            out["shadow_rays_per_bounce"] = list(st.shadow_rays_per_bounce)
            return out
        return None

    def poll(self):
        return self._lib.agb_batch_poll(self.handle) == _abi.AGB_OK


class Server:
    """The serving loop (agb_server_*): register uploaded Renderers as scenes, submit requests,
    wait for their images and latencies."""

    def __init__(self, hbm_budget_bytes, max_slots=4, device=0):
        self._lib = _abi.library()
        self.handle = ctypes.c_void_p()
        check(self._lib.agb_server_create(device, int(hbm_budget_bytes), max_slots,
                                          ctypes.byref(self.handle)))
        self._scenes = {}

    def close(self):
        if self.handle:
            self._lib.agb_server_destroy(self.handle)
            self.handle = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def add_scene(self, scene_id, renderer):
        """Registers an uploaded Renderer; returns the agb status (AGB_ERR_OOM beyond the budget)."""
        st = self._lib.agb_server_add_scene(self.handle, scene_id, renderer.ctx)
        if st == _abi.AGB_OK:
            self._scenes[scene_id] = renderer
        return st

    def set_denoiser(self, handle):
        check(self._lib.agb_server_set_denoiser(self.handle, handle))

    def submit(self, scene_id, frame, width, height, spp, seed_offset=0, denoise=False):
        r = _abi.ServeRequest()
        r.scene, r.width, r.height, r.spp = scene_id, width, height, spp
        r.seed_offset = seed_offset
        r.flags = _abi.SERVE_DENOISE if denoise else 0
        f = np.ascontiguousarray(np.asarray(frame, dtype=_abi.FRAME_DTYPE).reshape(1))
        ctypes.memmove(r.frame, f.ctypes.data, 512)
        rid = ctypes.c_uint64()
        check(self._lib.agb_server_submit(self.handle, ctypes.byref(r), ctypes.byref(rid)))
        return rid.value, (width, height)

    def wait(self, ticket, timeout_ms=-1):
        """(status, image (H, W, 4) or None, result dict)."""
        rid, (w, h) = ticket
        img = np.empty((h, w, 4), np.float32)
        res = _abi.ServeResult()
        st = self._lib.agb_server_wait(self.handle, rid, timeout_ms, ctypes.byref(res), ptr(img),
                                       img.size)
        info = dict(status=res.status, queue_ms=res.queue_ms, render_ms=res.render_ms,
                    latency_ms=res.latency_ms)
        return st, (img if st == _abi.AGB_OK else None), info

    def memory(self):
        a, b = ctypes.c_uint64(), ctypes.c_uint64()
        check(self._lib.agb_server_memory(self.handle, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value


def temporal_jitter(frame_index, phase_count=0):
    """Halton (2, 3) camera jitter in pixels for a frame (PTRenderer.cpp:159-174)."""
    out = (ctypes.c_float * 2)()
    _abi.library().agb_temporal_jitter(frame_index, phase_count, out)
    return float(out[0]), float(out[1])


def random_stream(sample_index, width, px, py, n, out_ptr):
    check(library().agb_random_stream(sample_index, width, px, py, n, ctypes.c_void_p(out_ptr), None))
