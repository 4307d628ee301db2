#!/usr/bin/env python3
"""Benchmark: path-samples/s of the GB300 path tracer on the large plain-method configuration
(1920x1080, 64 spp, up to 8 bounces, one 1,310,720-triangle icosphere BLAS instanced 64 times,
2048x1024 HDR environment), the configuration the headline metric is quoted on.

One step = one render of the frame at 64 samples per pixel from sample 0 (132,710,400 path
samples) through agb_render, scene resident in HBM.  L2 is flushed (a 256 MB write) between timed
steps, outside the timed region.  Device time comes from CUDA events on the renderer's stream.

  e2e          the same metric through the C ABI with host buffers: per step agb_frame_set from
               pinned host memory (512 bytes), agb_render, agb_accum_read of the RGBA32F image into
               pinned host memory; wall time per step.
  roofline     dominant kernel (closest-hit traversal): algorithmic bytes (node visits x 64 B +
               triangle tests x 48 B, counted by the kernels on the same samples) / its device time.
  cpu_baseline the FP32 oracle (the project's CPU restatement of the reference shaders, kind
               "port") on the host cores, on a bounded band of rows at 1 spp.

--impl reference times that CPU implementation alone (the reference itself has no CPU path).
--gpus N runs N independent replicas (one per rank); the path tracer needs no collective.
"""
import argparse
import json
import math
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "path-samples/s"
UNIT = "path-samples/s"


def parse_args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--config", default="large", choices=["large", "small", "stress"],
                   help="large: the headline configuration; small: the CPU-runnable one; stress: "
                        "3840x2160 layered-material progressive accumulation (a step = one "
                        "progressive call of --stress-chunk samples, default 64 steps = 4096 spp)")
    p.add_argument("--stress-chunk", type=int, default=64)
    p.add_argument("--stress-crop", type=int, default=32,
                   help="side of the square (centred on the instance nearest the middle of the frame) "
                        "the FP64 oracle renders at the full sample count for the stress "
                        "configuration's relMSE series (0: skip)")
    p.add_argument("--cpu-seconds", type=float, default=15.0)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--res", default=None, help="WxH override (profiling runs)")
    p.add_argument("--spp", type=int, default=None, help="samples per pixel override (profiling runs)")
    p.add_argument("--no-denoiser", action="store_true", help="skip the denoiser measurement")
    p.add_argument("--no-serve", action="store_true", help="skip the serving measurement")
    p.add_argument("--no-denoised-serving", action="store_true",
                   help="skip training the denoiser and the denoised-serving measurement")
    p.add_argument("--no-time-to-error", action="store_true", help="skip the time-to-relMSE measurement")
    p.add_argument("--serve-requests", type=int, default=160)
    p.add_argument("--ground-plane", action="store_true",
                   help="add a ground plane (the reference's defaults) under the scene (overhead runs)")
    p.add_argument("--max-paths", type=int, default=0xFFFFFFFF,
                   help="paths in flight per wave (0: the library's bounded default of 8 GiB of "
                        "wave buffers; default here 0xFFFFFFFF = AGB_WAVE_LARGEST, waves sized "
                        "from half the free device memory)")
    p.add_argument("--converged-crop", type=int, default=0,
                   help="side of a crop on which the time-to-relMSE reference (16,384 samples) is checked "
                        "against the FP64 oracle's render of the same streams (0: skip; 16 takes about "
                        "4 minutes of host time)")
    p.add_argument("--oracle-rows", type=int, default=8,
                   help="rows of the frame rendered by the FP64 oracle at the step's samples for "
                        "the reported relMSE (0: skip)")
    return p.parse_args()


def closest_dram_bytes_per_ray():
    """DRAM bytes (read + write) per closest-hit ray of k_trace_closest from the committed ncu
    summary, or None."""
    try:
        for line in open(os.path.join(ROOT, "profiles", "trace_closest_dram_large_config.txt")):
            if line.startswith("closest_bytes_per_ray"):
                return float(line.split()[1])
    except OSError:
        pass
    return None


def path_model(counted, value, peak):
    paths = max(1, counted["paths"])
    nodes_tris = (counted["node_visits"] + counted["shadow_node_visits"]) * 64 + \
        (counted["tri_tests"] + counted["shadow_tri_tests"]) * 48
    per_sample = (nodes_tris + counted.get("shading_points", 0) * 108) / paths + 64
    achieved = per_sample * value / 1e9
    return {"bytes_per_path_sample": per_sample, "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "shading_points_per_path": counted.get("shading_points", 0) / paths,
            "model": "sum over rays of node visits x 64 B + triangle tests x 48 B, + shaded hits x 108 B, "
                     "+ 32 B running mean + 32 B Kahan per sample"}


def simt_threads_per_instruction():
    """Active threads per executed instruction of k_trace_closest from the committed ncu summary
    (out of 32), or None."""
    try:
        for line in open(os.path.join(ROOT, "profiles", "trace_kernels_large_config.md")):
            if "threads per executed instruction" in line:
                return float(line.split("|")[2].split("/")[0])
    except (OSError, ValueError, IndexError):
        pass
    return None


def denoiser_flops_per_pixel(training=False):
    """2 x 9 x cin x cout per 3x3 convolution, per output pixel of its level, summed over the
    U-Net's 15 layers (x3 for a training step: forward, data gradient, weight gradient)."""
    layers = [(16, 32, 0), (32, 32, 0), (32, 64, 1), (64, 64, 1), (64, 128, 2), (128, 128, 2),
              (128, 256, 3), (256, 256, 3), (384, 128, 2), (128, 128, 2), (192, 64, 1),
              (64, 64, 1), (96, 32, 0), (32, 32, 0), (32, 16, 0)]
    f = sum(2.0 * 9 * ci * co / 4 ** lv for ci, co, lv in layers)
    return 3 * f if training else f


def bench_denoiser(torch, _abi, stream, peaks):
    """Tensor-core U-Net: 1920x1080 inference and training steps on 4 and 16 crops of 256^2, CUDA
    events on the denoiser's stream after warm-up."""
    import ctypes
    lib = _abi.library()
    h = ctypes.c_void_p()
    _abi.check(lib.agb_denoiser_create(0, ctypes.c_void_p(stream.cuda_stream), 1, ctypes.byref(h)))
    out = {}
    try:
        for tag, (B, H, W), train in (("inference_1080p", (1, 1080, 1920), False),
                                      ("training_4x256", (4, 256, 256), True),
                                      ("training_16x256", (16, 256, 256), True)):
            x = torch.zeros((B, H, W, 16), dtype=torch.int16, device="cuda")
            x[..., :10] = 0x3F00  # 0.5 in BF16
            rgba = torch.zeros((B, H, W, 4), dtype=torch.float32, device="cuda")
            loss = ctypes.c_float()
            if train:
                call = lambda: _abi.check(lib.agb_denoiser_train_step(
                    h, x.data_ptr(), rgba.data_ptr(), B, H, W, 1e-4, 1, ctypes.byref(loss)))
            else:
                call = lambda: _abi.check(lib.agb_denoiser_forward(h, x.data_ptr(), B, H, W,
                                                                   rgba.data_ptr()))
            for _ in range(3):
                call()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            n = 10
            torch.cuda.synchronize()
            e0.record(stream)
            for _ in range(n):
                call()
            e1.record(stream)
            e1.synchronize()
            ms = e0.elapsed_time(e1) / n
            tf = denoiser_flops_per_pixel(train) * B * H * W / (ms / 1000.0) / 1e12
            peak = peaks["bf16_tflops"] if peaks else 1900.0
            out[tag] = {"ms": ms, "achieved": tf, "peak": peak, "unit": "TFLOP/s",
                        "frac": tf / peak, "bound": "tensor",
                        "peak_source": "MEASURED_PEAKS.json bf16_tflops (burst, measured)" if peaks
                        else "fallback 1.9 PFLOP/s"}
    finally:
        lib.agb_denoiser_destroy(h)
    return out


def bench_time_to_rel_mse(torch, _abi, r, s, target=1e-3, ref_spp=16384, max_spp=16384, oracle_crop=0):
    """Wall time until the running image is within relMSE `target` (eps 1e-2) of a converged
    reference of the same frame.  The reference is this renderer's own ref_spp-sample mean over
    random streams independent of the timed run's (seed offsets 2^24 and 2^25 for its two halves;
    the renderer's agreement with the FP64 oracle is a test), so the measured relMSE also carries
    the reference's own noise, about relMSE(half A, half B) / 4, which is reported.  The timed loop
    renders progressively into the Kahan sum and evaluates relMSE on the GPU (agb_accum_rel_mse)
    after each call; the next call's sample count follows the error seen so far (relMSE ~ c / spp
    + c / ref_spp): 90 % of the predicted remainder, 8 to 256 samples, a multiple of 8."""
    import ctypes
    lib = _abi.library()
    r.set_frame(s.frame)
    half = ref_spp // 2
    err = ctypes.c_double(float("inf"))
    r.render(0, half, accumulation=_abi.ACCUM_KAHAN, seed_offset=1 << 24)
    ref_a = torch.from_numpy(r.read(_abi.ACCUM_KAHAN).copy()).cuda()
    r.render(0, half, accumulation=_abi.ACCUM_KAHAN, seed_offset=1 << 25)
    _abi.check(lib.agb_accum_rel_mse(r.ctx, _abi.ACCUM_KAHAN, ref_a.data_ptr(), 1e-2, ctypes.byref(err)))
    halves_rel_mse = err.value
    ref = (ref_a + torch.from_numpy(r.read(_abi.ACCUM_KAHAN).copy()).cuda()) * 0.5
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    spp, chunk, calls = 0, 8, 0
    while spp < max_spp:
        r.render(spp, chunk, accumulation=_abi.ACCUM_KAHAN)
        spp += chunk
        calls += 1
        _abi.check(lib.agb_accum_rel_mse(r.ctx, _abi.ACCUM_KAHAN, ref.data_ptr(), 1e-2, ctypes.byref(err)))
        if err.value <= target:
            break
        c = err.value / (1.0 / spp + 1.0 / ref_spp)
        room = target - c / ref_spp
        need = c / room if room > 0 else max_spp
        chunk = int(min(256, max(8, 8 * math.ceil(0.9 * (need - spp) / 8))))
        chunk = min(chunk, max_spp - spp)
    secs = time.perf_counter() - t0
    out = {"target_rel_mse": target, "eps": 1e-2, "seconds": secs, "spp": spp,
           "rel_mse": err.value, "reached": err.value <= target, "reference_spp": ref_spp,
           "reference_noise_rel_mse": halves_rel_mse / 4, "render_calls": calls,
           "path_samples": s.width * s.height * spp}
    if oracle_crop > 0:
        out["reference_vs_fp64_oracle"] = converged_crop_vs_oracle(s, ref.cpu().numpy(), half, oracle_crop)
    return out


def converged_crop_vs_oracle(s, ref, half, c):
    """The converged device image (two halves of `half` samples over the random streams offset by
    2^24 and 2^25) against the FP64 oracle's render of the same streams, on a c x c crop centred on
    the instance nearest the middle of the frame: the renderer's error once the per-sample noise
    has averaged out (relMSE eps 1e-2; equal-sample renders part where an FP64 decision differs)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    x0, y0 = stress_crop_origin(s, c)
    rect = (x0, y0, x0 + c, y0 + c)
    o = pyoracle.OracleScene(s)
    t0 = time.perf_counter()
    a = o.render(0, half, precision=64, want_sum=True, want_mean=False, rect=rect, seed_offset=1 << 24)["sum"]
    b = o.render(0, half, precision=64, want_sum=True, want_mean=False, rect=rect, seed_offset=1 << 25)["sum"]
    secs = time.perf_counter() - t0
    o.close()
    crop = (slice(y0, y0 + c), slice(x0, x0 + c))
    oracle_img = (a[crop] + b[crop]) / (2 * half)
    err = pyoracle.rel_mse(ref[crop], oracle_img)
    return {"rel_mse": err, "eps": 1e-2, "bar": 1e-3, "within_bar": err <= 1e-3, "spp": 2 * half,
            "crop": list(rect), "oracle_noise_rel_mse": pyoracle.rel_mse(a[crop] / half, b[crop] / half) / 4,
            "oracle": "FP64 CPU restatement of the reference shaders, the same sample streams",
            "oracle_seconds": secs}


def bench_serving(api, _abi, n_requests, rates=(200.0, 25.0)):
    """Serving loop on 8 resident scenes (seeds 0-7: the small configuration's type at even seeds,
    the large configuration's at odd ones, both at full size), Poisson arrivals, resolutions
    {640x360, 1280x720, 1920x1080} x spp {1, 4, 16}, a Halton camera jitter per request, 150 GB HBM
    budget, 32 requests in flight, merged into batched wavefronts."""
    from aurora_gb300 import scenes
    rs, frames = [], []
    for k in range(8):
        if k % 2 == 0:
            sc = scenes.config_small(seed=k, width=1920, height=1080, spp=1)
        else:
            sc = scenes.config_large(seed=k, width=1920, height=1080, spp=1)
        r = api.Renderer()
        r.upload(sc)
        rs.append(r)
        frames.append(sc.frame)
    res_choices = [(640, 360), (1280, 720), (1920, 1080)]
    out = {}
    try:
        for rate in rates:
            rng = np.random.default_rng(7)
            with api.Server(hbm_budget_bytes=150 << 30, max_slots=32) as srv:
                for k, r in enumerate(rs):
                    _abi.check(srv.add_scene(k, r))
                tickets, paths = [], 0
                t0 = time.perf_counter()
                t_next = 0.0
                for i in range(n_requests):
                    t_next += rng.exponential(1.0 / rate)
                    k = int(rng.integers(0, 8))
                    w, h = res_choices[int(rng.integers(0, 3))]
                    spp = int(rng.choice([1, 4, 16]))
                    f = frames[k].copy()
                    jx, jy = api.temporal_jitter(i)
                    f["camera_jitter"] = (jx, jy)
                    f["is_temporal_jitter_enabled"] = 1
                    delay = t0 + t_next - time.perf_counter()
                    if delay > 0:
                        time.sleep(delay)
                    tickets.append(srv.submit(k, f, w, h, spp, seed_offset=i))
                    paths += w * h * spp
                lat, queue = [], []
                for t in tickets:
                    st, img, info = srv.wait(t)
                    _abi.check(st)
                    lat.append(info["latency_ms"])
                    queue.append(info["queue_ms"])
                makespan = time.perf_counter() - t0
            out[f"offered_{int(rate)}_rps"] = {
                "requests": n_requests, "p50_latency_ms": float(np.percentile(lat, 50)),
                "p99_latency_ms": float(np.percentile(lat, 99)),
                "mean_queue_ms": float(np.mean(queue)), "frames_per_s": n_requests / makespan,
                "path_samples_per_s": paths / makespan}
    finally:
        for r in rs:
            r.close()
    return out


def bench_denoised_serving(api, _abi, train_scenes=48, views=8, steps=8000, eval_size=(1920, 1080),
                           ref_spp=1024, repeats=3):
    """The learned denoiser trained on the tracer's own pairs, then served: relMSE (eps 1e-2)
    against converged references of plain accumulation at 1-256 spp and of the denoised output at
    1 and 4 spp, each frame's serving latency (one request at a time, so the latency is the
    request's own, not queueing), and the latency ratio at equal relMSE.

    Training: `train_scenes` seeded scenes alternating the two plain-method types (256x256 views
    from random orbit cameras, `views` per scene), noisy input at 1 or 4 spp (half each), targets at
    256 spp from independent streams; `steps` Adam steps of 4 views (lr 1.5e-4 cosine to 7.5e-6).
    Evaluation: the 8 serving scenes (seeds 0-7, the small configuration's type at even seeds, the
    large one's at odd seeds, full size) seen from their own cameras at eval_size (the largest
    serving resolution), references at ref_spp from independent streams (their own noise is part
    of every relMSE; it is below the errors compared)."""
    import torch
    from aurora_gb300 import denoiser_training as dt, scenes
    t0 = time.perf_counter()
    parts = [dt.make_pairs(train_scenes // 2, views, size=256, spp_lo=lo, spp_hi=256, seed=lo)
             for lo in (1, 4)]
    feats = torch.cat([p[0] for p in parts])
    refs = torch.cat([p[2] for p in parts])
    pair_s = time.perf_counter() - t0
    dn = dt.Denoiser(seed=11)
    t0 = time.perf_counter()
    losses = dn.train(feats, refs, steps, batch=4, lr=1.5e-4, lr_min=7.5e-6)
    torch.cuda.synchronize()
    train_s = time.perf_counter() - t0
    del feats, refs, parts
    w, h = eval_size
    plain_spp = [1, 2, 4, 8, 16, 32, 64]
    den_spp = [1, 4]
    rows = []
    rs = []
    try:
        for k in range(8):
            sc = (scenes.config_small(seed=k, width=w, height=h, spp=1) if k % 2 == 0 else
                  scenes.config_large(seed=k, width=w, height=h, spp=1))
            r = api.Renderer()
            r.upload(sc)
            rs.append((r, sc))
        with api.Server(hbm_budget_bytes=150 << 30, max_slots=4) as srv:
            srv.set_denoiser(dn.handle)
            for k, (r, sc) in enumerate(rs):
                srv.add_scene(k, r)
            for k, (r, sc) in enumerate(rs):
                r.set_frame(sc.frame)
                r.render(0, ref_spp, width=w, height=h, accumulation=_abi.ACCUM_KAHAN, seed_offset=1 << 26)
                ref = r.read(_abi.ACCUM_KAHAN, w, h).copy()
                row = {"scene": k, "type": "small" if k % 2 == 0 else "large", "plain": {}, "denoised": {}}
                for mode, spps in (("plain", plain_spp), ("denoised", den_spp)):
                    for spp in spps:
                        lat, err = [], []
                        for rep in range(repeats):
                            st, img, info = srv.wait(srv.submit(k, sc.frame, w, h, spp, seed_offset=rep * 977,
                                                                denoise=mode == "denoised"))
                            _abi.check(st)
                            lat.append(info["latency_ms"])
                            err.append(rel_mse_np(img, ref))
                        row[mode][spp] = {"rel_mse": float(np.mean(err)), "p50_ms": float(np.percentile(lat, 50)),
                                          "p99_ms": float(np.percentile(lat, 99))}
                rows.append(row)
    finally:
        for r, _ in rs:
            r.close()
        dn.close()

    def mean_over(kind, mode, spp, key):
        return float(np.mean([r[mode][spp][key] for r in rows if kind in (None, r["type"])]))

    summary = {}
    for kind in (None, "small", "large"):
        tag = kind or "all"
        plain = [(spp, mean_over(kind, "plain", spp, "rel_mse"), mean_over(kind, "plain", spp, "p50_ms"))
                 for spp in plain_spp]
        entry = {"plain": {str(spp): {"rel_mse": e, "p50_ms": t} for spp, e, t in plain}}
        for spp in den_spp:
            e_d = mean_over(kind, "denoised", spp, "rel_mse")
            t_d = mean_over(kind, "denoised", spp, "p50_ms")
            # The plain sample count of equal relMSE, interpolated on log-log between the measured
            # counts; its latency likewise (None when plain accumulation never gets there here).
            eq = None
            for (s0, e0, t0_), (s1, e1, t1_) in zip(plain, plain[1:]):
                if e0 >= e_d >= e1 and e0 > 0 and e1 > 0:
                    a = math.log(e0 / e_d) / math.log(e0 / e1) if e0 != e1 else 0.0
                    eq = (s0 * (s1 / s0) ** a, t0_ * (t1_ / t0_) ** a)
                    break
            if eq is None and e_d <= plain[0][1] and e_d < plain[-1][1]:
                eq = None
            entry[f"denoised_{spp}spp"] = {
                "rel_mse": e_d, "p50_ms": t_d,
                "plain_spp_at_equal_rel_mse": eq[0] if eq else None,
                "plain_p50_ms_at_equal_rel_mse": eq[1] if eq else None,
                "p50_latency_ratio": (eq[1] / t_d) if eq else None,
                "beyond_measured_plain_range": eq is None and e_d < plain[-1][1]}
        summary[tag] = entry
    return {"resolution": [w, h], "reference_spp": ref_spp, "eps": 1e-2, "repeats": repeats,
            "training": {"scenes": train_scenes, "views_per_scene": views, "crop": 256,
                         "noisy_spp": [1, 4], "target_spp": 256, "steps": steps, "batch": 4,
                         "pairs_seconds": pair_s, "train_seconds": train_s,
                         "loss_first_100": float(np.mean(losses[:100])),
                         "loss_last_100": float(np.mean(losses[-100:]))},
            "summary": summary, "per_scene": rows}


def rel_mse_np(x, ref, eps=1e-2):
    x = np.asarray(x, np.float64)[..., :3]
    r = np.asarray(ref, np.float64)[..., :3]
    return float(np.mean((x - r) ** 2 / (r * r + eps)))


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def make_scene(name, res=None, spp=None):
    from aurora_gb300 import scenes
    kw = {}
    if res:
        w, h = (int(x) for x in res.lower().split("x"))
        kw.update(width=w, height=h)
    if spp:
        kw.update(spp=spp)
    if name == "small":
        return scenes.config_small(seed=0, **kw)
    if name == "stress":
        return scenes.config_stress(seed=0, **kw)
    return scenes.config_large(seed=0, **kw)


def workload(s, name):
    return {"workload": ("plain method, large: icosphere level 8 (1,310,720 tris) x64 instances, "
                         "1920x1080, 64 spp, 8 bounces, 2048x1024 HDR env")
            if name == "large" else
            "plain method, small: 8x8 UV spheres + quad, 512x512, 16 spp, 5 bounces",
            "width": s.width, "height": s.height, "spp": s.spp,
            "trace_depth": int(s.frame["trace_depth"]), "unique_triangles": s.unique_triangles,
            "instances": len(s.instances), "instanced_triangles": s.triangle_count,
            "seed": 0, "accumulation": "FP32 running mean + Kahan-compensated sum",
            "l2": "flushed between timed steps (256 MB write)", "parallelism": "replicas",
            **({"ground_plane": "enabled (defaults) at the scene's lower bound"}
               if getattr(s, "ground_plane", None) is not None else {})}


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-i", str(self.index), "-lms", "200"], stdout=self.file, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.file.flush()
        rows = []
        for line in open(self.file.name):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9 and parts[1].replace(".", "").isdigit():
                rows.append(parts)
        os.unlink(self.file.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = np.array([float(r[1]) for r in rows])
        mx = float(rows[0][2])
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for k, nm in enumerate(names):
                if r[5 + k].lower() in ("active", "1", "yes"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "samples": len(rows),
                "reasons": sorted(reasons)}


def measured_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        return None


def cpu_sample_plan(o, s, seconds, threads):
    """Sizes a bounded CPU sample of the frame: a band of rows around the middle, and more than
    one sample index once the whole frame takes less than `seconds`.  Returns (rect, spp)."""
    mid = s.height // 2
    probe_rows = max(4, s.height // 64)
    rect = (0, mid - probe_rows // 2, s.width, mid - probe_rows // 2 + probe_rows)
    r = o.render(0, 1, threads=threads, rect=rect, want_mean=False)
    rate = s.width * probe_rows / max(r["seconds"], 1e-6)
    want = rate * seconds
    rows = int(min(s.height, max(probe_rows, want / s.width)))
    spp = int(max(1, min(s.spp, round(want / (s.width * rows)))))
    y0 = max(0, mid - rows // 2)
    return (0, y0, s.width, y0 + rows), spp


def cpu_render_rate(s, seconds):
    """Oracle FP32 on all host cores over a bounded part of the frame; returns (paths/s, threads,
    description)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    o = pyoracle.OracleScene(s)
    threads = os.cpu_count() or 1
    o.tracer(32)  # build the BVHs outside the timed part
    rect, spp = cpu_sample_plan(o, s, seconds, threads)
    r = o.render(1, spp, threads=threads, rect=rect, want_mean=False)
    paths = (rect[2] - rect[0]) * (rect[3] - rect[1]) * spp
    o.close()
    return paths / r["seconds"], threads, (
        f"rows {rect[1]}-{rect[3]} of the {s.width}x{s.height} frame at {spp} spp (sample indices "
        f"1-{spp}), {paths} path samples, {r['seconds']:.1f} s, FP32 oracle, BVH build excluded")


def rel_mse_vs_fp64_oracle(s, img, rows, threads=None):
    """relMSE (eps 1e-2) of the renderer's image of the step (sum / n, the step's own samples
    0..spp-1) against the FP64 oracle's render of the same samples over a band of `rows` rows
    through the middle of the frame: the error of the benchmarked result itself."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    o = pyoracle.OracleScene(s)
    y0 = s.height // 2 - rows // 2
    rect = (0, y0, s.width, y0 + rows)
    t0 = time.perf_counter()
    ref = o.render(0, s.spp, precision=64, want_sum=True, want_mean=False, rect=rect,
                   threads=threads)
    secs = time.perf_counter() - t0
    o.close()
    band = slice(y0, y0 + rows)
    err = pyoracle.rel_mse(img[band], ref["sum"][band] / s.spp)
    return {"rel_mse": err, "eps": 1e-2, "bar": 1e-3, "within_bar": err <= 1e-3,
            "oracle": "FP64 CPU restatement of the reference shaders, same sample streams",
            "rows": [y0, y0 + rows], "spp": s.spp, "pixels": s.width * rows,
            "oracle_seconds": secs}


def stress_crop_origin(s, c):
    """Top-left corner of a c x c crop centred on the projection of the instance whose centre
    projects nearest to the middle of the frame (in front of the camera), so the crop sees
    geometry, not only the environment."""
    vp = np.asarray(s.frame["camera_view_proj"], np.float64).reshape(4, 4).T
    best, where = None, (s.width // 2, s.height // 2)
    for inst in s.instances:
        m = np.asarray(inst["xform"], np.float64).reshape(3, 4)
        q = vp @ np.append(m[:, 3], 1.0)
        if q[3] <= 0:
            continue
        x = (q[0] / q[3] * 0.5 + 0.5) * s.width
        y = (0.5 - q[1] / q[3] * 0.5) * s.height
        d = (x - s.width / 2) ** 2 + (y - s.height / 2) ** 2
        if c / 2 <= x <= s.width - c / 2 and c / 2 <= y <= s.height - c / 2 and (best is None or d < best):
            best, where = d, (int(x), int(y))
    return where[0] - c // 2, where[1] - c // 2


def run_stress(args):
    """Stress configuration (3840x2160; 16 BLAS of 10K-500K triangles, 1000 instances with a decal
    layer; Kahan-compensated progressive accumulation).  Warm-up: W calls of one chunk from sample
    0.  Timed: K progressive calls of `--stress-chunk` samples continuing the accumulation (the
    default K = 64 reaches 4096 spp); per call the frame data goes up from pinned host memory and the
    whole running image (Kahan sum / n) comes back into pinned host memory, both inside the e2e wall
    time; `value` is from CUDA events around the renders alone.  After every call the relMSE of a
    centred crop against the FP64 oracle's render of the same crop at the full sample count (the
    same sample streams) is recorded: the convergence series."""
    import torch
    from aurora_gb300 import _abi, api, build
    build.build()
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    chunk, steps = args.stress_chunk, args.steps
    total = chunk * steps
    t0 = time.perf_counter()
    s = make_scene("stress", args.res, total)
    gen_s = time.perf_counter() - t0
    stream = torch.cuda.Stream()
    r = api.Renderer(local, stream=stream.cuda_stream)
    t0 = time.perf_counter()
    r.upload(s)
    upload_s = time.perf_counter() - t0
    acc = _abi.ACCUM_KAHAN | _abi.ACCUM_RUNNING_MEAN
    for _ in range(args.warmup):
        r.render(0, chunk, accumulation=acc, max_paths=args.max_paths)
    r.set_profiling(True)
    frame_host = torch.from_numpy(np.frombuffer(np.ascontiguousarray(s.frame).tobytes(),
                                                np.uint8).copy()).pin_memory()
    frame_np = frame_host.numpy().view(_abi.FRAME_DTYPE)
    img_host = torch.empty((s.height, s.width, 4), dtype=torch.float32).pin_memory()
    img_np = img_host.numpy()
    c = args.stress_crop
    x0, y0 = stress_crop_origin(s, c)
    crops = []
    clocks = ClockSampler(local)
    torch.cuda.synchronize()
    clocks.start()
    render_ms, launches = 0.0, 0
    kernel_ms = {k: 0.0 for k in _abi.KERNEL_FAMILIES}
    wall0 = time.perf_counter()
    for k in range(steps):
        r.set_frame(frame_np)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        st = r.render(k * chunk, chunk, accumulation=acc, stats=True, max_paths=args.max_paths)
        e1.record(stream)
        r.read(_abi.ACCUM_KAHAN, out=img_np)
        e1.synchronize()
        render_ms += e0.elapsed_time(e1)
        launches += st["kernel_launches"]
        for f in _abi.KERNEL_FAMILIES:
            kernel_ms[f] += st["kernel_ms"][f]
        if c > 0:
            crops.append(img_np[y0:y0 + c, x0:x0 + c].copy())
    wall = time.perf_counter() - wall0
    clk = clocks.stop()
    paths = s.width * s.height * total
    out = {
        "metric": METRIC, "value": paths / (render_ms / 1000.0), "unit": UNIT, "n_gpus": 1,
        "steps": steps, "warmup": args.warmup, "ms_per_step": render_ms / steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded)",
        "config": {"workload": "plain method, stress with layered materials and accumulation: 16 BLAS "
                               "of 10K-500K triangles (4.09M unique), 1000 instances with an "
                               "alpha-masked decal layer (1024^2 RGBA8), 3840x2160, progressive to "
                               f"{total} spp, Kahan-compensated FP32",
                   "width": s.width, "height": s.height, "spp": total, "chunk_spp": chunk,
                   "trace_depth": int(s.frame["trace_depth"]), "unique_triangles": s.unique_triangles,
                   "instances": len(s.instances), "instanced_triangles": s.triangle_count,
                   "seed": 0, "l2": "inputs larger than L2 (scene and wave state)",
                   "scene_generation_s": gen_s, "upload_and_build_s": upload_s},
        "e2e": {"value": paths / wall, "unit": UNIT,
                "h2d_bytes_per_step": int(_abi.FRAME_DTYPE.itemsize),
                "d2h_bytes_per_step": int(s.width * s.height * 16), "ms_per_step": 1000.0 * wall / steps},
        "gpu_launches": int(launches),
        "kernel_ms_per_step": {f: v / steps for f, v in kernel_ms.items()},
        "clocks": clk,
    }
    r.close()
    if c > 0:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import pyoracle
        o = pyoracle.OracleScene(s)
        rect = (x0, y0, x0 + c, y0 + c)
        t0 = time.perf_counter()
        half = total // 2
        a = o.render(0, half, precision=64, want_sum=True, want_mean=False, rect=rect)["sum"]
        b = o.render(half, total - half, precision=64, want_sum=True, want_mean=False, rect=rect)["sum"]
        oracle_s = time.perf_counter() - t0
        o.close()
        ref = ((a + b) / total)[y0:y0 + c, x0:x0 + c]
        noise = pyoracle.rel_mse(a[y0:y0 + c, x0:x0 + c] / half,
                                 b[y0:y0 + c, x0:x0 + c] / (total - half)) / 4
        series = [[chunk * (k + 1), pyoracle.rel_mse(img, ref)] for k, img in enumerate(crops)]
        out["rel_mse_vs_fp64_oracle"] = {
            "series": series, "eps": 1e-2, "every_spp": chunk, "crop": list(rect),
            "reference": f"FP64 oracle, the same {total} sample streams",
            "reference_noise_rel_mse": noise, "final": series[-1][1],
            "first_spp_within_1e-3": next((n for n, e in series if e <= 1e-3), None),
            "oracle_seconds": oracle_s}
    print(json.dumps(out))


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    s = make_scene(args.config)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    o = pyoracle.OracleScene(s)
    threads = os.cpu_count() or 1
    o.tracer(32)
    # Each step: a bounded part of the frame sized to ~10 s on this host.
    rect, spp = cpu_sample_plan(o, s, 10.0, threads)
    for w in range(args.warmup):
        o.render(w * spp, spp, threads=threads, rect=rect, want_mean=False)
    secs = 0.0
    for k in range(args.steps):
        secs += o.render((args.warmup + k) * spp, spp, threads=threads, rect=rect,
                         want_mean=False)["seconds"]
    paths = (rect[2] - rect[0]) * (rect[3] - rect[1]) * spp * args.steps
    value = paths / secs
    sample = (f"rows {rect[1]}-{rect[3]} of the {s.width}x{s.height} frame, {spp} spp per step, "
              f"FP32 oracle port of the reference shaders on {threads} host threads")
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * secs / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded)", "config": workload(s, args.config),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference's own backend needs a Vulkan ray-tracing device (no CPU path); "
                "its lavapipe run is unavailable on this box, so its CPU restatement is timed"}))
    o.close()


def main():
    args = parse_args()
    if args.impl == "reference":
        run_reference(args)
        return
    if args.config == "stress":
        run_stress(args)
        return
    rank, world, local = dist_env()
    import torch
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    from aurora_gb300 import _abi, api, build
    build.build()
    s = make_scene(args.config, args.res, args.spp)
    if args.ground_plane:
        s.ground_plane = _abi.ground_plane(position=(0.0, float(s.bounds()[0][1]), 0.0))
    stream = torch.cuda.Stream()
    r = api.Renderer(local, stream=stream.cuda_stream)
    r.upload(s)
    paths_per_step = s.width * s.height * s.spp

    # Counting pass (untimed): node visits and triangle tests of exactly the timed work.
    r.set_counting(True)
    counted = r.render(0, s.spp, stats=True, max_paths=args.max_paths)
    r.set_counting(False)

    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    for _ in range(args.warmup):
        r.render(0, s.spp, max_paths=args.max_paths)
    r.set_profiling(True)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    clocks = ClockSampler(local)
    clocks.start()
    step_ms = []
    kernel_ms = {k: 0.0 for k in _abi.KERNEL_FAMILIES}
    kernel_count = {k: 0 for k in _abi.KERNEL_FAMILIES}
    launches = 0
    for _ in range(args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        st = r.render(0, s.spp, stats=True, max_paths=args.max_paths)
        e1.record(stream)
        e1.synchronize()
        step_ms.append(e0.elapsed_time(e1))
        launches += st["kernel_launches"]
        for k in _abi.KERNEL_FAMILIES:
            kernel_ms[k] += st["kernel_ms"][k]
            kernel_count[k] += st["kernel_count"][k]
    torch.cuda.synchronize()
    clk = clocks.stop()
    total_ms = float(sum(step_ms))
    if world > 1:
        t = torch.tensor([total_ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_ms = float(t.item())
    value = paths_per_step * args.steps * world / (total_ms / 1000.0)
    r.set_profiling(False)

    # End to end through the C ABI with host buffers.
    frame_host = torch.from_numpy(np.frombuffer(np.ascontiguousarray(s.frame).tobytes(),
                                                np.uint8).copy()).pin_memory()
    img_host = torch.empty((s.height, s.width, 4), dtype=torch.float32).pin_memory()
    img_np = img_host.numpy()
    frame_np = frame_host.numpy().view(_abi.FRAME_DTYPE)
    e2e_s = []
    for k in range(0 if args.no_e2e else args.warmup + args.steps):
        t0 = time.perf_counter()
        r.set_frame(frame_np)
        r.render(0, s.spp, max_paths=args.max_paths)
        r.read(_abi.ACCUM_KAHAN, out=img_np)
        if k >= args.warmup:
            e2e_s.append(time.perf_counter() - t0)
    e2e_time = float(np.sum(e2e_s)) if e2e_s else float("nan")
    if world > 1:
        t = torch.tensor([e2e_time], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        e2e_time = float(t.item())
    e2e_value = paths_per_step * args.steps * world / e2e_time

    # Roofline of the dominant kernel family.
    steps = args.steps
    closest_ms = kernel_ms["trace_closest"] / steps
    closest_bytes = counted["node_visits"] * 64 + counted["tri_tests"] * 48
    shadow_ms = kernel_ms["trace_shadow"] / steps
    shadow_bytes = counted["shadow_node_visits"] * 64 + counted["shadow_tri_tests"] * 48
    dominant = max(kernel_ms, key=lambda k: kernel_ms[k])
    peaks = measured_peaks()
    peak = peaks["hbm_gbs"] if peaks else 6800.0
    achieved = closest_bytes / (closest_ms / 1000.0) / 1e9
    dram_per_ray = closest_dram_bytes_per_ray()
    launches_closest = max(1.0, kernel_count["trace_closest"] / steps)
    roofline = {
        # The bytes model is HBM-shaped (node and triangle records per ray against the copy
        # bandwidth), but the kernel is bound by dependent L1 / L2 latency and SIMT efficiency:
        # DRAM carries about a ninth of the modelled bytes (the scene's working set mostly hits
        # L2).  Both figures are reported.
        "bound": "hbm", "bound_observed": "L1 / L2 latency and SIMT efficiency (not DRAM bandwidth)",
        "kernel": "k_trace_closest (closest-hit BVH2 traversal)",
        "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
        "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)" if peaks else "fallback 6.8 TB/s",
        "traffic": (int(dram_per_ray * counted["closest_rays"] / launches_closest)
                    if dram_per_ray is not None else None),
        "traffic_unit": "bytes per launch (DRAM read + write): the committed ncu capture's bytes per "
                        "closest-hit ray x this step's closest-hit rays per launch",
        "algorithmic_bytes_per_launch": int(closest_bytes / launches_closest),
        "algorithmic_bytes_per_step": int(closest_bytes),
        "launches_per_step": kernel_count["trace_closest"] / steps,
        "ms_per_step": closest_ms,
        "bytes_model": "node visits x 64 B (BVH2 node, both child boxes) + triangle tests x 48 B "
                       "(3 x float4 vertices), counted on the timed samples",
        "shadow_kernel": {"achieved_gbs": shadow_bytes / max(shadow_ms, 1e-9) / 1e6,
                          "ms_per_step": shadow_ms, "algorithmic_bytes_per_step": int(shadow_bytes)},
        "dram_frac": ((dram_per_ray * counted["closest_rays"] / (closest_ms / 1000.0)) / 1e9 / peak
                      if dram_per_ray is not None else None),
        "dram_frac_note": "DRAM bytes of the committed capture per closest-hit ray x this step's rays / "
                          "the kernel's time / the measured copy bandwidth",
        # The whole path's bytes per path sample: node and triangle records of every closest-hit
        # and shadow ray, a 108-byte shading fetch per shaded hit (counted as the points the
        # surface kernel hands on: a lower bound of the hits) and 32 + 32 bytes of FP32 + Kahan
        # accumulation per sample, times path-samples/s, against the copy bandwidth.
        "path_model": path_model(counted, value / world, peak),
        "simt_threads_per_instruction": simt_threads_per_instruction(),
        "dominant_family_by_time": dominant,
        "kernel_ms_per_step": {k: v / steps for k, v in kernel_ms.items()},
    }

    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
        "config": {**workload(s, args.config),
                   "wave": ("largest (AGB_WAVE_LARGEST: half the free device memory)"
                            if args.max_paths == 0xFFFFFFFF else
                            "library default (8 GiB of wave buffers)" if args.max_paths == 0 else
                            f"{args.max_paths} paths")},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(_abi.FRAME_DTYPE.itemsize),
                "d2h_bytes_per_step": int(s.width * s.height * 16),
                "ms_per_step": 1000.0 * e2e_time / args.steps},
        "gpu_launches": int(launches),
        "rays_per_step": {"closest": counted["closest_rays"], "shadow": counted["shadow_rays"],
                          "closest_per_bounce": [int(v) for v in counted["closest_rays_per_bounce"]],
                          "shadow_per_bounce": [int(v) for v in counted["shadow_rays_per_bounce"]]},
        "per_ray": {
            "closest_node_visits": counted["node_visits"] / max(1, counted["closest_rays"]),
            "closest_tri_tests": counted["tri_tests"] / max(1, counted["closest_rays"]),
            "shadow_node_visits": counted["shadow_node_visits"] / max(1, counted["shadow_rays"]),
            "shadow_tri_tests": counted["shadow_tri_tests"] / max(1, counted["shadow_rays"])},
        "roofline": roofline,
        "clocks": clk,
    }
    if world == 1 and args.oracle_rows > 0:
        out["rel_mse_vs_fp64_oracle"] = rel_mse_vs_fp64_oracle(
            s, r.read(_abi.ACCUM_KAHAN).copy(), args.oracle_rows)
    if world == 1 and not args.no_time_to_error:
        out["time_to_rel_mse"] = bench_time_to_rel_mse(torch, _abi, r, s, oracle_crop=args.converged_crop)
    if world == 1 and not args.no_denoiser:
        out["denoiser"] = bench_denoiser(torch, _abi, stream, measured_peaks())
    if world == 1 and not args.no_serve:
        out["serving"] = bench_serving(api, _abi, args.serve_requests)
    if world == 1 and not args.no_denoised_serving:
        out["denoised_serving"] = bench_denoised_serving(api, _abi)
    if world == 1 and not args.no_cpu_baseline:
        cpu, threads, sample = cpu_render_rate(s, args.cpu_seconds)
        out["cpu_baseline"] = {"value": cpu, "unit": UNIT, "cores": threads, "kind": "port",
                               "sample": sample}
    r.close()
    if rank == 0:
        print(json.dumps(out))
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
