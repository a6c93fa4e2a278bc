#!/usr/bin/env python3
"""Benchmark: ms/frame of the ReSTIR GI frame pipeline at 1920x1080.

Workload (one "step" = one frame): the procedural scene of 998,442 triangles
(ground plane, 4096 icospheres/boxes with GGX conductor/plastic materials, 16
emissive quads, seed 1), a camera translating 0.01 units and yawing 0.2 deg per
frame along a 32-frame path (longer runs play it forward and back), 1 spp path
depth 4, temporal reuse (M cap 20) + spatial reuse (5
neighbours in 30 px, shadow rays), FP32.  Inputs are synthetic.

value: device time per frame (CUDA events around K frames, all inputs resident).
e2e:   the same frames (same warm-up, a fresh context) through the C ABI with
       host buffers: each step uploads the frame's UBO from host memory and reads
       the RGBA8 image back into page-locked host memory, one frame in flight
       (xr_read_output_async, two frames in flight: frame k renders while the
       images of frames k-1 and k-2 are copied).
--impl reference: the CPU restatement of the reference pipeline (oracle) on the
       host cores, per step one bounded sample of the workload.

With --gpus N (torchrun) every rank renders an independent replica (the
pipeline has no cross-GPU exchange); value = max rank time / (K * N).
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

W, H = 1920, 1080          # overridden by --width/--height (profiling of smaller cases)
BOUNCES = 4
SCENE_KW = dict(seed=1, n_objects=4096, n_lights=16, extent=40.0, sphere_subdiv=2)
METRIC = "ms/frame 1080p & relMSE vs FP64 ref: plain ReSTIR GI vs ReSTIR GI+MLP cache"
# algorithmic bytes per pixel of the temporal reuse pass in the packed layout:
# reads G-buffer 16+4, candidate 16+16, reprojected pixel index 4, previous G-buffer 4+16,
# previous reservoir 32; writes reservoir 32
TEMPORAL_BYTES_PER_PX = 140
# spatial reuse, each pixel counted once: reservoir 32 + G-buffer 20 read, reservoir 32 + RGBA16F-sized output 8
# written (the recommended layout's figure; the RGBA8 image written here is 4 B)
SPATIAL_BYTES_PER_PX = 92
RESERVOIR_BYTES_PER_PX = TEMPORAL_BYTES_PER_PX + SPATIAL_BYTES_PER_PX   # 232
# DRAM bytes (read + write) of one k_temporal launch at 1920x1080 measured with ncu
# (dram__bytes_read.sum + dram__bytes_write.sum): 185.2 MB + 47.7 MB
TEMPORAL_DRAM_BYTES_1080P = 232.4e6
# DRAM bytes of one 1080p frame's four reservoir-pass kernels (ncu): k_temporal 232.4 MB, k_spatial_select
# 128.2 MB, k_spatial_resolve 215.9 MB (1080p captures), k_trace_shadow about 44 MB (its 960x540 capture
# scaled by the shadow rays traced)
PASSES_DRAM_BYTES_1080P = 621e6
# kernels per frame: raygen, (trace + shade) per bounce, temporal, spatial select,
# shadow trace, spatial resolve
FRAME_LAUNCHES = 1 + 2 * BOUNCES + 4


def workload(frames: int) -> str:
    return (f"procedural 1920x1080, 998442 triangles, {frames} frames of the 32-frame camera path (played forward "
            "and back), corrected ReSTIR GI (M cap 20, 5 neighbours, 30 px, shadow rays), depth 4")


def _peaks():
    try:
        return json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
    except Exception:
        return {}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self) -> dict | None:
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in Path(self.path).read_text().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = max(mx, float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws <= 1:
        return None, 0, 1, int(os.environ.get("LOCAL_RANK", "0"))
    import torch
    import torch.distributed as dist
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist.init_process_group("nccl")
    return dist, dist.get_rank(), ws, local


def _barrier(dist, local):
    if dist is not None:
        import torch
        dist.barrier()
        torch.cuda.synchronize(local)


def _max_over_ranks(dist, v: float, device: str = "cpu") -> float:
    """Largest value over the ranks (the slowest replica sets the job time)."""
    if dist is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_ms_per_frame(max_rank_ms: float, steps: int, world: int) -> float:
    """Replicas render `steps` frames each: job time per frame over all ranks' frames."""
    return max_rank_ms / (steps * world)


PATH_FRAMES = 32   # the camera path's length


def move_camera(cam, f: int) -> None:
    """Frame f's step along the 32-frame camera path (0.01 units along -z and 0.2
    degrees of yaw per frame).  Runs longer than the path play it forward, then
    back, so that every frame shows one of the path's own views and the camera
    keeps moving (temporal reuse stays continuous)."""
    s = 1.0 if (f // PATH_FRAMES) % 2 == 0 else -1.0
    cam.position[2] -= 0.01 * s
    cam.yaw_deg += 0.2 * s


def camera_ubos(xr, scene, n_frames):
    cam = xr._lib.XrCamera.from_buffer_copy(scene.camera)
    prev = None
    ubos = []
    for f in range(n_frames):
        move_camera(cam, f)
        u = xr.camera_ubo(cam, W, H, prev, f, BOUNCES, sky=False, reuse=True)
        prev = u
        ubos.append(u)
    return ubos


RELMSE_EPS = 1e-2


def relmse(img: "np.ndarray", ref: "np.ndarray") -> float:
    """mean over pixels and channels of (x - r)^2 / (r^2 + 1e-2)."""
    import numpy as np
    x = img[:, :3].astype(np.float64)
    return float(np.mean((x - ref) ** 2 / (ref ** 2 + RELMSE_EPS)))


RELMSE_EVAL_FRAMES = (16, 24, 32, 40, 48)


def _relmse_run(xr, scene, ubos, eval_frames, ref_spp, device, refs, cache: bool, n_neighbours: int,
                train_samples: int, visibility: int = 1, keep_images: dict | None = None) -> dict:
    """One variant along the camera path: relMSE at the evaluation frames (FP64
    references computed once and shared) and its median frame time; the HDR
    images of the evaluation frames go into keep_images when given."""
    import numpy as np
    L = xr._lib
    r = xr.Renderer(W, H, device=device)
    p = xr.params_default(W, H, write_hdr=1, write_pt=1)
    p.visibility = visibility
    if n_neighbours == 0:
        p.spatial_on = 0
    else:
        p.n_neighbours = n_neighbours
    r.set_params(p)
    r.upload_scene(scene)
    r.build_bvh()
    if cache:
        cp = xr.cache_params_default()
        cp.enabled = 1
        cp.train_samples = train_samples
        r.cache.set_params(cp)
    rel, rel_pt, ms, infer, train = [], [], [], [], []
    for f, u in enumerate(ubos[:max(eval_frames)]):
        r.render(u)
        ms.append(r.stats().ms_frame)
        if cache:
            cs = r.cache.stats()
            infer.append(cs.ms_infer)
            train.append(cs.ms_train)
        if f + 1 in eval_frames:
            hdr = r.read_output(L.XR_OUT_HDR)
            if f + 1 not in refs:
                t0 = time.perf_counter()
                refs[f + 1] = r.render_reference(u, 1_000_000, ref_spp)
                refs["seconds"] = refs.get("seconds", 0.0) + time.perf_counter() - t0
            rel.append(relmse(hdr, refs[f + 1]))
            if keep_images is not None:
                keep_images[f + 1] = hdr[:, :3].astype(np.float64)
            rel_pt.append(relmse(r.read_output(L.XR_OUT_PT), refs[f + 1]))
    entry = {"relmse": float(np.mean(rel)), "per_frame": [round(v, 4) for v in rel],
             "ms_per_frame": round(statistics.median(ms[8:]), 4), "n_neighbours": n_neighbours,
             "shadow_rays": bool(visibility and n_neighbours)}
    if cache:
        cs = r.cache.stats()
        entry.update({"ms_infer": round(statistics.median(infer[8:]), 4),
                      "ms_train": round(statistics.median(train[8:]), 4), "queries": cs.queries,
                      "train_samples": cs.train_samples, "adam_steps": cs.steps, "loss": round(cs.loss, 4)})
    else:
        entry["pt_1spp"] = float(np.mean(rel_pt))
    r.close()
    return entry


def measure_relmse(xr, scene, ubos, eval_frames, ref_spp: int, device: int, train_samples: int = 65536) -> dict:
    """relMSE against the FP64-accumulated reference (plain path tracer, `ref_spp`
    samples, at each evaluation frame's camera), averaged over the evaluation
    frames, for: plain ReSTIR GI (5 neighbours, shadow rays), ReSTIR GI + learned
    radiance cache with the same reuse settings, and ReSTIR GI + cache at equal
    frame time -- of the reuse settings tried (5 .. 1 neighbours with and without
    the spatial pass's shadow rays, no spatial pass) the one with the lowest relMSE
    whose median frame time does not exceed plain ReSTIR GI's (the cache's own
    settings stay as configured).  Also the error decomposition."""
    refs = {}
    plain = _relmse_run(xr, scene, ubos, eval_frames, ref_spp, device, refs, False, 5, train_samples)
    same = _relmse_run(xr, scene, ubos, eval_frames, ref_spp, device, refs, True, 5, train_samples)
    # equal time: of the cache variant's reuse settings (5 .. 1 neighbours with and without the
    # spatial shadow rays, no spatial pass) the one with the lowest relMSE whose median frame
    # time does not exceed plain ReSTIR GI's
    tried = [same]
    for vis in (1, 0):
        for nb in (5, 4, 3, 2, 1):
            if vis and nb == 5:
                continue
            tried.append(_relmse_run(xr, scene, ubos, eval_frames, ref_spp, device, refs, True, nb, train_samples,
                                     vis))
    tried.append(_relmse_run(xr, scene, ubos, eval_frames, ref_spp, device, refs, True, 0, train_samples, 0))
    fits = [t for t in tried if t["ms_per_frame"] <= plain["ms_per_frame"]]
    equal = min(fits, key=lambda t: t["relmse"]) if fits else min(tried, key=lambda t: t["ms_per_frame"])
    # for comparison: plain ReSTIR GI without the spatial shadow rays
    plain_nv = _relmse_run(xr, scene, ubos, eval_frames, ref_spp, device, refs, False, 5, train_samples, 0)
    # error decomposition: the cache replaces the path beyond the first secondary vertex
    # x_s; at depth 2 a path ends at x_s (its emission only), so plain ReSTIR GI at depth 2
    # against the depth-2 reference is the error of the part the cache cannot change --
    # its ratio to the depth-4 error bounds what a cache at x_s can achieve
    ubos2 = []
    for u in ubos:
        u2 = type(u).from_buffer_copy(u)
        u2.number_of_bounces = 2
        ubos2.append(u2)
    refs2, img2 = {}, {}
    depth2 = _relmse_run(xr, scene, ubos2, eval_frames, ref_spp, device, refs2, False, 5, train_samples,
                         keep_images=img2)
    import numpy as np
    # a perfect cache: the depth-2 estimate plus the exact (noise-free) suffix radiance ref4 - ref2,
    # against the same depth-4 reference as every variant
    ideal = float(np.mean([relmse(img2[f] + (refs[f] - refs2[f]), refs[f]) for f in eval_frames]))
    suffix_share = float(np.mean([np.mean(refs[f] - refs2[f]) / max(np.mean(refs[f]), 1e-30) for f in eval_frames]))
    return {"restir_gi": plain["relmse"], "restir_gi_mlp_cache": same["relmse"], "pt_1spp": plain["pt_1spp"],
            "ratio_cache_over_plain": round(same["relmse"] / plain["relmse"], 4),
            "restir_gi_mlp_cache_equal_time": equal["relmse"],
            "ratio_equal_time": round(equal["relmse"] / plain["relmse"], 4),
            "detail": {"restir_gi": plain, "restir_gi_mlp_cache": same, "restir_gi_mlp_cache_equal_time": equal,
                       "restir_gi_no_shadow_rays": plain_nv,
                       "cache_settings_tried": [{k: t[k] for k in ("n_neighbours", "shadow_rays", "relmse", "ms_per_frame")}
                                                for t in tried]},
            "decomposition": {
                "restir_gi_depth4": plain["relmse"],
                "restir_gi_depth2_vs_depth2_reference": depth2["relmse"],
                "perfect_cache": ideal,
                "perfect_cache_ratio": round(ideal / plain["relmse"], 4),
                "suffix_share_of_radiance": round(suffix_share, 4),
                "note": "the cache replaces the path beyond the first secondary vertex x_s; a perfect cache "
                        "leaves the depth-2 estimate (paths ending at x_s) plus the exact suffix radiance "
                        "(depth-4 minus depth-2 reference), whose relMSE against the depth-4 reference is "
                        "what any cache at x_s can reach at these settings",
                "ms_per_frame_depth2": depth2["ms_per_frame"]},
            "reference": f"FP64-accumulated plain path tracer, {ref_spp} spp, same path depth, "
                         f"at frames {list(eval_frames)} of the camera path",
            "eps": RELMSE_EPS, "reference_seconds": round(refs.get("seconds", 0.0), 2)}


def cpu_info() -> dict:
    """The host the CPU numbers were taken on: CPU model, cores, OpenMP threads."""
    model = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.strip().lower().startswith("model name:"):
                model = line.split(":", 1)[1].strip()
                break
    except Exception:
        pass
    if not model:
        try:
            for line in Path("/proc/cpuinfo").read_text().splitlines():
                if line.lower().startswith(("model name", "cpu part")):
                    model = line.split(":", 1)[1].strip()
                    break
        except Exception:
            pass
    import platform
    return {"cpu_model": model or "unknown", "arch": platform.machine(), "nproc": os.cpu_count(),
            "omp_num_threads": os.environ.get("OMP_NUM_THREADS", "unset (OpenMP uses every core)")}


def _oracle_frames(scene, ubos, warmup: int, max_frames: int, seconds_budget: float | None):
    """The oracle (OpenMP over pixels, all host threads) on full 1920x1080 frames of
    the camera path: `warmup` untimed frames, then timed frames until max_frames or
    the time budget.  Returns (timed frames, seconds)."""
    from oracle import binding as ob
    from oracle import workload as wl
    r = ob.OracleRenderer(ob.OracleScene.from_scene(scene), wl.params_default(W, H))
    for u in ubos[:warmup]:
        r.render(u)
    frames = 0
    t0 = time.perf_counter()
    for u in ubos[warmup:warmup + max_frames]:
        r.render(u)
        frames += 1
        if seconds_budget is not None and time.perf_counter() - t0 > seconds_budget:
            break
    return frames, time.perf_counter() - t0


def cpu_baseline(scene, ubos, seconds_budget: float = 20.0) -> dict:
    """The oracle on the host cores: consecutive full 1920x1080 frames of the same
    scene and camera path (from the first frame, so temporal reuse runs as in the
    benchmark) for about `seconds_budget` seconds."""
    frames, secs = _oracle_frames(scene, ubos, 0, len(ubos), seconds_budget)
    info = cpu_info()
    return {"value": secs * 1e3 / frames, "unit": "ms/frame", "cores": info["nproc"], "kind": "port",
            "sample": f"{frames} consecutive frames of the camera path at {W}x{H} (full frames, no scaling); "
                      "OpenMP over pixels", **info}


def run_reference(args):
    """The reference's CPU path (the oracle's restatement of its shaders; the
    reference itself needs Vulkan ray tracing, unavailable on this machine) on the same
    scene, camera path and settings at full resolution.  Scene and UBOs come from
    oracle/_build/libworkload.so: nothing of libxr.so is loaded."""
    dist, rank, ws, local = _dist()
    if rank != 0:
        return
    from oracle import workload as wl
    scene = wl.procedural(**SCENE_KW)
    cam = xr_camera_from(scene)
    ubos, prev = [], None
    for f in range(args.warmup + args.steps):
        move_camera(cam, f)
        prev = wl.camera_ubo(cam, W, H, prev, f, BOUNCES, sky=False, reuse=True)
        ubos.append(prev)
    frames, secs = _oracle_frames(scene, ubos, args.warmup, args.steps, None)
    v = secs * 1e3 / frames
    try:   # the CPU arm must not lean on the product library
        assert "libxr.so" not in Path("/proc/self/maps").read_text(), "the reference arm loaded libxr.so"
    except FileNotFoundError:
        pass
    info = cpu_info()
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "ms/frame", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": v, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": workload(args.steps), "resolution": [W, H]},
            "cpu_baseline": {"value": v, "unit": "ms/frame", "cores": info["nproc"], "kind": "port",
                             "sample": f"{args.steps} full {W}x{H} frames of the camera path after {args.warmup} "
                                       "warm-up frames; the reference itself needs Vulkan ray tracing, "
                                       "unavailable on this box", **info},
            "e2e": {"value": v, "unit": "ms/frame", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def xr_camera_from(scene):
    from xvk_ray_gb300 import _lib as L
    return L.XrCamera.from_buffer_copy(scene.camera)


def run_ours(args):
    dist, rank, ws, local = _dist()
    import ctypes as C

    import numpy as np

    import xvk_ray_gb300 as xr
    from xvk_ray_gb300 import _build
    _build.build_library()
    L = xr._lib
    lib = L.load()
    scene = xr.Scene.procedural(**SCENE_KW)
    n_frames = args.warmup + args.steps
    ubos = camera_ubos(xr, scene, 2 * n_frames + 8)
    r = xr.Renderer(W, H, device=local)
    r.set_params(xr.params_default(W, H))
    r.upload_scene(scene)
    r.build_bvh()
    r.set_graphs(True)   # each frame's launches replayed from a CUDA graph (one per frame parity)
    st = r.stats()
    bvh = {"nodes": st.bvh_nodes, "triangles": st.bvh_triangles, "depth": st.bvh_depth,
           "build_ms": round(st.ms_bvh_build, 2)}

    # ---- device-resident timing: K frames between two events ----
    fi = 0
    for _ in range(args.warmup):
        r.render(ubos[fi]); fi += 1
    r.sync()
    _barrier(dist, local)
    clocks = ClockSampler(local)
    clocks.start()
    L.check(lib.xr_event_record(r.ctx, 0), r.ctx)
    for _ in range(args.steps):
        r.render(ubos[fi]); fi += 1
    L.check(lib.xr_event_record(r.ctx, 1), r.ctx)
    ms = C.c_float()
    L.check(lib.xr_event_elapsed(r.ctx, 0, 1, C.byref(ms)), r.ctx)
    clk = clocks.stop()
    r.sync()
    total_ms = _max_over_ranks(dist, float(ms.value), f"cuda:{local}")
    ms_per_frame = whole_job_ms_per_frame(total_ms, args.steps, ws)

    # ---- per-pass breakdown (events inside the library, one frame at a time) ----
    t_init, t_temp, t_spat, rays, shadow = [], [], [], [], []
    for _ in range(min(args.steps, 16)):
        r.render(ubos[fi]); fi += 1
        s = r.stats()
        t_init.append(s.ms_initial); t_temp.append(s.ms_temporal); t_spat.append(s.ms_spatial)
        rays.append(s.rays_traced); shadow.append(s.shadow_rays)
    ms_init, ms_temp, ms_spat = (statistics.mean(t_init), statistics.mean(t_temp), statistics.mean(t_spat))
    rays_pf, shadow_pf = statistics.mean(rays), statistics.mean(shadow)

    st = r.stats()
    r.close()

    # ---- e2e through the C ABI with host buffers ----
    # The same frames as the device-timed region on a fresh context, after the same
    # warm-up: a frame's cost depends on the reservoirs' history, so both legs render
    # identical frames from identical states.  Two frames in flight, as a real-time
    # host runs: frame k renders while the RGBA8 images of frames k-1 and k-2 are
    # copied into page-locked host memory (three host images); the host waits for
    # frame k-2's image, so a stall of the host thread shorter than two frames does
    # not stall the GPU.
    r = xr.Renderer(W, H, device=local)
    r.set_params(xr.params_default(W, H))
    r.upload_scene(scene)
    r.build_bvh()
    r.set_graphs(True)
    for u in ubos[:args.warmup]:
        r.render(u)
    r.sync()
    pinned = [xr.PinnedBuffer(W * H * 4) for _ in range(3)]
    outs = [pb.array for pb in pinned]
    host_ubos = [L.XrUniformBufferObject.from_buffer_copy(u) for u in ubos[args.warmup:args.warmup + args.steps]]
    _barrier(dist, local)
    t0 = time.perf_counter()
    for k, u in enumerate(host_ubos):
        L.check(lib.xr_render_frame(r.ctx, C.byref(u)), r.ctx)
        if k >= 2:
            L.check(lib.xr_wait_output(r.ctx), r.ctx)   # frame k-2's image is in host memory
        L.check(lib.xr_read_output_async(r.ctx, outs[k % 3].ctypes.data, outs[k % 3].nbytes), r.ctx)
    for _ in range(min(args.steps, 2)):
        L.check(lib.xr_wait_output(r.ctx), r.ctx)
    e2e_ms = (time.perf_counter() - t0) * 1e3
    L.check(lib.xr_sync(r.ctx), r.ctx)   # device error flags of the e2e frames
    e2e_ms = whole_job_ms_per_frame(_max_over_ranks(dist, e2e_ms, f"cuda:{local}"), args.steps, ws)
    img_mean = float(outs[(args.steps - 1) % 3].reshape(-1, 4)[:, :3].mean())
    for pb in pinned:
        pb.free()
    st.error_flags |= r.stats().error_flags
    r.close()

    if rank != 0:
        return
    rel = None
    if args.relmse_spp > 0:
        rel = measure_relmse(xr, scene, ubos, RELMSE_EVAL_FRAMES, args.relmse_spp, local)
    peaks = _peaks()
    hbm = peaks.get("hbm_gbs")
    peak_note = "measured" if hbm else "fallback"
    hbm = hbm or 6800.0
    N = W * H
    temporal_gbs = TEMPORAL_BYTES_PER_PX * N / (ms_temp * 1e-3) / 1e9
    spatial_gbs = SPATIAL_BYTES_PER_PX * N / (ms_spat * 1e-3) / 1e9
    passes_gbs = RESERVOIR_BYTES_PER_PX * N / ((ms_temp + ms_spat) * 1e-3) / 1e9
    line = {
        "metric": METRIC, "value": round(ms_per_frame, 4), "unit": "ms/frame", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms_per_frame, 4), "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (procedural scene, seed 1)",
        "config": {"workload": workload(args.steps),
                   "resolution": [W, H], "triangles": scene.n_triangles, "bounces": BOUNCES,
                   "l2": "per-frame working set 0.66 GB > 129 MB L2 (no flush needed); BVH stays L2-resident",
                   "parallelism": f"replicas x{ws}", "launch": "frame graphs (xr_set_graphs)"},
        "passes_ms": {"initial_sample": round(ms_init, 4), "temporal": round(ms_temp, 4), "spatial": round(ms_spat, 4)},
        "rays_per_frame": rays_pf, "shadow_rays_per_frame": shadow_pf,
        "rays_per_s": (rays_pf + shadow_pf) / ((ms_init + ms_spat) * 1e-3),
        # the reservoir passes as one unit (232 B per pixel over temporal + spatial time, the
        # spatial pass with its shadow-ray traversal), and each pass on its own
        "roofline": {"kernel": "reservoir passes (k_temporal + k_spatial_select + k_trace_shadow + k_spatial_resolve)",
                     "bound": "hbm", "achieved": round(passes_gbs, 1), "peak": hbm, "unit": "GB/s",
                     "frac": round(passes_gbs / hbm, 4),
                     "traffic": PASSES_DRAM_BYTES_1080P if (W, H) == (1920, 1080) else None,
                     "traffic_unit": "bytes per frame (ncu, the four kernels)", "peak_source": peak_note,
                     "algorithmic_bytes_per_px": RESERVOIR_BYTES_PER_PX,
                     "passes": {"temporal": {"achieved": round(temporal_gbs, 1), "frac": round(temporal_gbs / hbm, 4),
                                             "algorithmic_bytes_per_px": TEMPORAL_BYTES_PER_PX, "ms": round(ms_temp, 4),
                                             "traffic": TEMPORAL_DRAM_BYTES_1080P if (W, H) == (1920, 1080) else None},
                                "spatial": {"achieved": round(spatial_gbs, 1), "frac": round(spatial_gbs / hbm, 4),
                                            "algorithmic_bytes_per_px": SPATIAL_BYTES_PER_PX, "ms": round(ms_spat, 4)}}},
        "bvh": bvh,
        "e2e": {"value": round(e2e_ms, 4), "unit": "ms/frame", "h2d_bytes_per_step": C.sizeof(L.XrUniformBufferObject),
                "d2h_bytes_per_step": W * H * 4},
        "gpu_launches": FRAME_LAUNCHES * args.steps,
        "clocks": clk,
        "relmse": rel,
        "image_mean_ldr": round(img_mean, 3),
        "device_error_flags": st.error_flags,
    }
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(scene, ubos, seconds_budget=args.cpu_seconds)
    print(json.dumps(line), flush=True)


# Configuration 0: the Cornell box at 256x256 (34 triangles of walls and boxes plus
# the light quad), 8 frames of a static camera, 1 spp, depth 4, the benchmark's reuse
# settings; relMSE against an FP64-accumulated reference of 65,536 spp.
CORNELL_FRAMES = 8
CORNELL_REF_SPP = 65536


def run_cornell(args):
    import numpy as np

    import xvk_ray_gb300 as xr
    from xvk_ray_gb300 import _build
    _build.build_library()
    L = xr._lib
    lib = L.load()
    w = h = 256
    scene = xr.Scene.cornell()
    cam = L.XrCamera.from_buffer_copy(scene.camera)
    ubos, prev = [], None
    n_frames = max(CORNELL_FRAMES, args.warmup + args.steps)
    for f in range(n_frames):
        prev = xr.camera_ubo(cam, w, h, prev, f, BOUNCES, sky=False, reuse=True)
        ubos.append(prev)
    res = {}
    for variant in ("restir_gi", "restir_gi_mlp_cache"):
        r = xr.Renderer(w, h)
        r.set_params(xr.params_default(w, h, write_hdr=1, write_pt=1))
        r.upload_scene(scene)
        r.build_bvh()
        if variant != "restir_gi":
            cp = xr.cache_params_default()
            cp.enabled = 1
            cp.train_samples = 8192
            r.cache.set_params(cp)
        if variant == "restir_gi":
            t0 = time.perf_counter()
            ref = r.render_reference(ubos[0], 1_000_000, CORNELL_REF_SPP)
            ref_s = time.perf_counter() - t0
        per_frame, pt = [], []
        for u in ubos[:CORNELL_FRAMES]:
            r.render(u)
            per_frame.append(relmse(r.read_output(L.XR_OUT_HDR), ref))
            pt.append(relmse(r.read_output(L.XR_OUT_PT), ref))
        # timing: the configuration's frames repeated along the same static camera
        r.sync()
        L.check(lib.xr_event_record(r.ctx, 0), r.ctx)
        for u in ubos[:args.steps]:
            r.render(u)
        L.check(lib.xr_event_record(r.ctx, 1), r.ctx)
        ms = ctypes.c_float()
        L.check(lib.xr_event_elapsed(r.ctx, 0, 1, ctypes.byref(ms)), r.ctx)
        res[variant] = {"relmse_per_frame": [round(v, 5) for v in per_frame], "relmse_frame8": per_frame[-1],
                        "pt_1spp": float(np.mean(pt)), "ms_per_frame": round(ms.value / args.steps, 5)}
        r.close()
    line = {"metric": METRIC, "value": res["restir_gi"]["ms_per_frame"], "unit": "ms/frame", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": res["restir_gi"]["ms_per_frame"],
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (procedural Cornell box)",
            "config": {"workload": "Cornell box 256x256, 34 + 2 triangles, 8 static frames, 1 spp, depth 4, "
                                   "corrected ReSTIR GI (M cap 20, 5 neighbours, 30 px, shadow rays)",
                       "reference": f"FP64-accumulated plain path tracer, {CORNELL_REF_SPP} spp "
                                    f"({ref_s:.1f} s on the GPU)"},
            "relmse": {"restir_gi": res["restir_gi"]["relmse_frame8"],
                       "restir_gi_mlp_cache": res["restir_gi_mlp_cache"]["relmse_frame8"],
                       "ratio_cache_over_plain": round(res["restir_gi_mlp_cache"]["relmse_frame8"] /
                                                       res["restir_gi"]["relmse_frame8"], 4),
                       "pt_1spp": res["restir_gi"]["pt_1spp"], "detail": res, "eps": RELMSE_EPS}}
    print(json.dumps(line), flush=True)


# The README's Scene1: Sibenik (asset/model/sb2, 75,277 triangles, 3 base-colour
# textures) at 1920x1080 from the reference's default camera, converted from the
# reference checkout by oracle/refpin/scenes.py.  Two settings: the reference's own
# (reference mode: 10 bounces, M caps 30/300, 6 neighbours in 5 px, no-op
# visibility) and the benchmark's corrected pipeline (depth 4, shadow rays).  Per
# pass: the initial sample alone is the 1-spp path tracer's work, + temporal, +
# spatial -- the README's three columns (its ReSTIR figures are the UI's frame time
# divided by 3, src/Editor/UI.cpp:169, on RT cores of an unstated GPU).


def run_sibenik(args):
    import numpy as np

    import xvk_ray_gb300 as xr
    from xvk_ray_gb300 import _build
    from oracle.refpin import scenes
    _build.build_library()
    L = xr._lib
    lib = L.load()
    scene = scenes.load("sibenik")
    out = {}
    for mode, pf, nb in (("reference_settings", xr.params_reference, 10), ("corrected", xr.params_default, BOUNCES)):
        cam = L.XrCamera.from_buffer_copy(scene.camera)
        ubos, prev = [], None
        for f in range(args.warmup + args.steps):
            cam.position[0] += 0.01
            cam.yaw_deg += 0.2
            prev = xr.camera_ubo(cam, W, H, prev, f, nb, sky=False, reuse=True)
            ubos.append(prev)
        r = xr.Renderer(W, H)
        r.set_params(pf(W, H))
        r.upload_scene(scene)
        r.build_bvh()
        r.set_graphs(True)
        for u in ubos[:args.warmup]:
            r.render(u)
        r.sync()
        clocks = ClockSampler(0)
        clocks.start()
        L.check(lib.xr_event_record(r.ctx, 0), r.ctx)
        for u in ubos[args.warmup:]:
            r.render(u)
        L.check(lib.xr_event_record(r.ctx, 1), r.ctx)
        ms = ctypes.c_float()
        L.check(lib.xr_event_elapsed(r.ctx, 0, 1, ctypes.byref(ms)), r.ctx)
        clk = clocks.stop()
        r.set_graphs(False)
        t_i, t_t, t_s = [], [], []
        for u in ubos[args.warmup:args.warmup + min(args.steps, 16)]:
            r.render(u)
            st = r.stats()
            t_i.append(st.ms_initial); t_t.append(st.ms_temporal); t_s.append(st.ms_spatial)
        img = r.read_output(L.XR_OUT_LDR8)
        out[mode] = {"ms_per_frame": round(ms.value / args.steps, 4), "bounces": nb,
                     "passes_ms": {"initial_sample_1spp_pt": round(statistics.mean(t_i), 4),
                                   "temporal": round(statistics.mean(t_t), 4),
                                   "spatial": round(statistics.mean(t_s), 4)},
                     "cumulative_ms": {"1spp_pt": round(statistics.mean(t_i), 4),
                                       "restir_temporal": round(statistics.mean(t_i) + statistics.mean(t_t), 4),
                                       "restir_spatial": round(statistics.mean(t_i) + statistics.mean(t_t) +
                                                               statistics.mean(t_s), 4)},
                     "rays_per_frame": st.rays_traced, "clocks": clk,
                     "image_mean_ldr": round(float(np.asarray(img).reshape(-1, 4)[:, :3].mean()), 3)}
        r.close()
    line = {"metric": METRIC, "value": out["reference_settings"]["ms_per_frame"], "unit": "ms/frame", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": out["reference_settings"]["ms_per_frame"],
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "the reference's bundled Sibenik scene (asset/model/sb2, CC-BY-4.0)",
            "config": {"workload": f"Sibenik 1920x1080, {scene.n_triangles} triangles, 3 textures, the "
                                   "reference's default camera moving 0.01 units and 0.2 degrees per frame",
                       "readme_published_ms": {"1spp_pt": 2.8, "restir_temporal": 2.9, "restir_spatial": 3.3,
                                               "note": "README.md:7, RT cores on an unstated GPU, ReSTIR columns "
                                                       "= UI frame time / 3 (src/Editor/UI.cpp:169): not comparable"}},
            "modes": out}
    print(json.dumps(line), flush=True)


# Batched workload: 64 views over 8 procedural scenes of ~10k .. 2M triangles
# (same generator as the 1080p scene), resolutions cycling 256^2, 512^2, 720p,
# 1080p, every view on its own camera path.
BATCH_SCENE_OBJECTS = (40, 128, 512, 1024, 2048, 4096, 6144, 8192)
BATCH_RES = ((256, 256), (512, 512), (1280, 720), (1920, 1080))
BATCH_VIEWS = 64


def batch_ubos(xr, scenes, views, n_frames):
    """Per frame, the UBO of every view: the scene's camera yawed by 7 degrees per
    view of that scene, then the benchmark motion (0.01 units, 0.2 degrees per frame)."""
    L = xr._lib
    cams, prevs = [], []
    for v, (s, w, h) in enumerate(views):
        cam = L.XrCamera.from_buffer_copy(scenes[s].camera)
        cam.yaw_deg += 7.0 * (v % 8)
        cams.append(cam)
        prevs.append(None)
    frames = []
    for f in range(n_frames):
        row = []
        for v, (s, w, h) in enumerate(views):
            cams[v].position[2] -= 0.01
            cams[v].yaw_deg += 0.2
            u = xr.camera_ubo(cams[v], w, h, prevs[v], f, BOUNCES, sky=False, reuse=True)
            prevs[v] = u
            row.append(u)
        frames.append(row)
    return frames


def run_batch(args):
    """One JSON line for the batched workload: every frame renders all 64 views in
    the same launches (replayed from a CUDA graph, launch sizes from the autotuner)."""
    import ctypes as C

    dist, rank, ws, local = _dist()
    import xvk_ray_gb300 as xr
    from xvk_ray_gb300 import _build
    _build.build_library()
    L = xr._lib
    lib = L.load()
    scenes = [xr.Scene.procedural(seed=10 + k, n_objects=o, n_lights=16, extent=40.0, sphere_subdiv=2)
              for k, o in enumerate(BATCH_SCENE_OBJECTS)]
    views = [(v // (BATCH_VIEWS // len(scenes)), *BATCH_RES[v % len(BATCH_RES)]) for v in range(BATCH_VIEWS)]
    n_frames = 3 + 2 * (args.warmup + args.steps)   # autotune, then graph and direct runs
    frames = batch_ubos(xr, scenes, views, n_frames)
    r = xr.Renderer(8, 8, device=local)
    t0 = time.perf_counter()
    r.upload_scenes(scenes)
    build_s = time.perf_counter() - t0
    r.set_views(views, xr.params_default(8, 8))
    tuning = r.autotune(frames[:3])
    fi = 3

    def timed(graphs: bool) -> float:
        nonlocal fi
        r.set_graphs(graphs)
        for _ in range(args.warmup):
            r.render_views(frames[fi]); fi += 1
        r.sync()
        _barrier(dist, local)
        L.check(lib.xr_event_record(r.ctx, 0), r.ctx)
        for _ in range(args.steps):
            r.render_views(frames[fi]); fi += 1
        L.check(lib.xr_event_record(r.ctx, 1), r.ctx)
        ms = C.c_float()
        L.check(lib.xr_event_elapsed(r.ctx, 0, 1, C.byref(ms)), r.ctx)
        r.sync()
        return _max_over_ranks(dist, float(ms.value), f"cuda:{local}") / args.steps

    clocks = ClockSampler(local)
    clocks.start()
    ms_graph = timed(True)
    clk = clocks.stop()
    st = r.stats()
    rays = st.rays_traced + st.shadow_rays
    ms_direct = timed(False)
    r.close()
    if rank != 0:
        return
    tris = [s.n_triangles for s in scenes]
    pixels = sum(w * h for _, w, h in views)
    line = {
        "metric": "rays/s, 64 views over 8 scenes (10k-2M triangles) at 256^2/512^2/720p/1080p, one frame of every view per step",
        "value": round(rays * ws / (ms_graph * 1e-3), 1), "unit": "rays/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms_graph, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (8 procedural scenes, seeds 10..17)",
        "config": {"workload": f"{BATCH_VIEWS} views, {len(scenes)} scenes, triangles {tris}, {pixels} pixels per frame, "
                               "corrected ReSTIR GI (M cap 20, 5 neighbours, 30 px, shadow rays), depth 4",
                   "views": [list(v) for v in views[:8]] + ["..."], "parallelism": f"replicas x{ws}",
                   "l2": "per-frame working set far larger than L2 (no flush needed)"},
        "per_view_ms": round(ms_graph / BATCH_VIEWS, 5),
        "rays_per_frame": int(rays),
        "ms_per_frame_direct_launches": round(ms_direct, 4),
        "graph_speedup": round(ms_direct / ms_graph, 4),
        "tuning": {"trace_ctas_per_sm": tuning.trace_ctas_per_sm, "shade_ctas_per_sm": tuning.shade_ctas_per_sm,
                   "refill_min": tuning.refill_min or "default (8)", "postpone_below": tuning.postpone_below or "default (8)",
                   "ray_bundle": ["8x4", "16x2", "4x8"][tuning.ray_bundle],
                   "temporal_block": tuning.temporal_block or "default (64)",
                   "spatial_block": tuning.spatial_block or "default (128)",
                   "ms_tuned": round(tuning.ms_per_frame, 4), "ms_all_defaults": round(tuning.ms_default, 4),
                   "configs_tried": tuning.configs_tried},
        "scene_build_s": round(build_s, 3),
        "gpu_launches": FRAME_LAUNCHES * args.steps,
        "clocks": clk,
    }
    print(json.dumps(line), flush=True)


# 4K workload: the 1080p scene's generator scaled to 32,768 objects and 64
# emissive quads (extent grown to keep the object density), four 3840x2160
# camera streams (yaw 0/90/180/270 degrees) rendered per launch.
SCENE_4K = dict(seed=1, n_objects=32768, n_lights=64, extent=40.0 * 8.0 ** 0.5, sphere_subdiv=2)
RES_4K = (3840, 2160)
STREAMS_4K = 4
MLP_FLOP_PER_QUERY = 2 * (4 * 64 * 64 + 16 * 64)          # 34,816 (forward)


def run_4k(args):
    """ms/frame of 4 x 3840x2160 streams of an 8M-triangle scene, plain ReSTIR GI
    and ReSTIR GI + learned cache, both replayed from frame graphs; relMSE of both
    against the FP64 reference of the last frame."""
    import ctypes as C

    import numpy as np
    dist, rank, ws, local = _dist()
    import xvk_ray_gb300 as xr
    from xvk_ray_gb300 import _build
    _build.build_library()
    L = xr._lib
    lib = L.load()
    scene = xr.Scene.procedural(**SCENE_4K)
    w, h = RES_4K
    views = [(0, w, h)] * STREAMS_4K
    n_frames = args.warmup + args.steps
    cams = []
    for k in range(STREAMS_4K):
        cam = L.XrCamera.from_buffer_copy(scene.camera)
        cam.yaw_deg += 90.0 * k
        cams.append(cam)
    frames, prev = [], [None] * STREAMS_4K
    for f in range(n_frames):
        row = []
        for k in range(STREAMS_4K):
            cams[k].position[2] -= 0.01
            cams[k].yaw_deg += 0.2
            u = xr.camera_ubo(cams[k], w, h, prev[k], f, BOUNCES, sky=False, reuse=True)
            prev[k] = u
            row.append(u)
        frames.append(row)
    peaks = _peaks()
    out, ref = {}, None
    for variant in ("restir_gi", "restir_gi_mlp_cache"):
        r = xr.Renderer(8, 8, device=local)
        r.upload_scenes([scene])
        r.set_views(views, xr.params_default(8, 8, write_hdr=1, write_pt=1))
        if variant == "restir_gi_mlp_cache":
            cp = xr.cache_params_default()
            cp.enabled = 1
            cp.train_samples = 65536
            r.cache.set_params(cp)
        r.set_graphs(True)
        for f in range(args.warmup):
            r.render_views(frames[f])
        r.sync()
        _barrier(dist, local)
        clocks = ClockSampler(local)
        clocks.start()
        L.check(lib.xr_event_record(r.ctx, 0), r.ctx)
        for f in range(args.warmup, n_frames):
            r.render_views(frames[f])
        L.check(lib.xr_event_record(r.ctx, 1), r.ctx)
        ms = C.c_float()
        L.check(lib.xr_event_elapsed(r.ctx, 0, 1, C.byref(ms)), r.ctx)
        clk = clocks.stop()
        st = r.stats()
        N = w * h * STREAMS_4K
        entry = {"ms_per_frame": round(_max_over_ranks(dist, float(ms.value), f"cuda:{local}") / args.steps, 4),
                 "passes_ms": {"initial_sample": round(st.ms_initial, 4), "temporal": round(st.ms_temporal, 4),
                               "spatial": round(st.ms_spatial, 4)},
                 "rays_per_frame": int(st.rays_traced + st.shadow_rays),
                 "temporal_hbm_gbs": round(TEMPORAL_BYTES_PER_PX * N / (st.ms_temporal * 1e-3) / 1e9, 1),
                 "clocks": clk}
        entry["rays_per_s"] = round(entry["rays_per_frame"] / (entry["ms_per_frame"] * 1e-3), 1)
        if variant == "restir_gi_mlp_cache":
            cs = r.cache.stats()
            flops = cs.queries * MLP_FLOP_PER_QUERY
            entry["cache"] = {"queries": cs.queries, "train_samples": cs.train_samples, "loss": round(cs.loss, 4),
                              "ms_infer": round(cs.ms_infer, 4), "ms_train": round(cs.ms_train, 4),
                              "inference_tflops": round(flops / (cs.ms_infer * 1e-3) / 1e12, 2),
                              "inference_tensor_frac_of_measured_bf16_peak":
                                  round(flops / (cs.ms_infer * 1e-3) / 1e12 / peaks["bf16_tflops"], 4)
                                  if peaks.get("bf16_tflops") else None}
        hdr = [r.read_view_output(v, L.XR_OUT_HDR) for v in range(STREAMS_4K)]
        if ref is None and args.relmse_spp > 0:
            ref = r.render_reference_views(frames[-1], 1_000_000, max(1, args.relmse_spp // 8))
            pt = [r.read_view_output(v, L.XR_OUT_PT) for v in range(STREAMS_4K)]
            out["pt_1spp"] = float(np.mean([relmse(p, q) for p, q in zip(pt, ref)]))
        if ref is not None:
            entry["relmse"] = float(np.mean([relmse(p, q) for p, q in zip(hdr, ref)]))
        out[variant] = entry
        r.close()
    if rank != 0:
        return
    plain, cached = out["restir_gi"], out["restir_gi_mlp_cache"]
    line = {
        "metric": "ms/frame, 4 camera streams x 3840x2160, 8M triangles, ReSTIR GI + learned cache (one launch set per frame, CUDA graph)",
        "value": cached["ms_per_frame"], "unit": "ms/frame", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": cached["ms_per_frame"], "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 (bf16 MLP)", "data": "synthetic (procedural scene, seed 1, 32768 objects, 64 emissive quads)",
        "config": {"workload": f"{STREAMS_4K} x {w}x{h}, {scene.n_triangles} triangles, {n_frames}-frame camera sweep, "
                               "corrected ReSTIR GI (M cap 20, 5 neighbours, 30 px, shadow rays) + learned cache, depth 4",
                   "parallelism": f"replicas x{ws}", "l2": "working set far larger than L2"},
        "restir_gi": plain, "restir_gi_mlp_cache": cached, "pt_1spp_relmse": out.get("pt_1spp"),
        "relmse_ratio_cache_over_plain": (round(cached["relmse"] / plain["relmse"], 4) if "relmse" in plain else None),
        "reference": (f"FP64-accumulated plain path tracer, {max(1, args.relmse_spp // 8)} spp, last frame"
                      if args.relmse_spp > 0 else None),
        "gpu_launches": FRAME_LAUNCHES * args.steps,
    }
    print(json.dumps(line), flush=True)


# Dynamic workload: the 1080p benchmark scene as one instance, DYN_INSTANCES
# instances of two small object scenes circling it (every transform changes every
# frame: the top-level BVH is rebuilt per frame) and one of them deforming (its
# BVH refitted per frame).
DYN_INSTANCES = 256
DYN_SMALL = dict(seed=77, n_objects=6, n_lights=0, extent=1.0, sphere_subdiv=2)


def run_dynamic(args):
    """ms/frame of the 1080p scene with moving instances and a deforming mesh:
    per frame one xr_update_vertices (upload + refit), one xr_set_instances
    (top-level rebuild) and one frame, timed on the host (wall clock) because
    both updates synchronise; device times of each part reported beside it."""
    import numpy as np

    dist, rank, ws, local = _dist()
    import xvk_ray_gb300 as xr
    from xvk_ray_gb300 import _build
    _build.build_library()
    big = xr.Scene.procedural(**SCENE_KW)
    small = xr.Scene.procedural(**DYN_SMALL)
    small2 = xr.Scene.procedural(**dict(DYN_SMALL, seed=78))

    def rot_y(a):
        c, s_ = np.cos(a), np.sin(a)
        return np.array([[c, 0, s_], [0, 1, 0], [-s_, 0, c]])

    def instances(f):
        out = [(0, np.hstack([np.eye(3), np.zeros((3, 1))]))]
        for k in range(DYN_INSTANCES):
            a = 2 * np.pi * k / DYN_INSTANCES + 0.01 * f * (1 + k % 3)
            rad = 6.0 + 30.0 * (k % 16) / 16.0
            m = np.zeros((3, 4))
            m[:, :3] = rot_y(a * 3.0) * (0.5 + 0.5 * (k % 4))
            m[:, 3] = [rad * np.cos(a), 1.0 + (k % 5), rad * np.sin(a)]
            out.append((1 + k % 2, m))
        return out

    def deformed(f):
        v = small2.vertices.copy()
        v[:, 1] += 0.1 * np.sin(2.0 * v[:, 0] + 0.3 * f)
        return v

    n_frames = args.warmup + args.steps
    ubos = camera_ubos(xr, big, n_frames + 2)
    # the animation is input data: every frame's instance records and vertices are ready in host memory
    inst_f = [xr.pack_instances(instances(f)) for f in range(n_frames)]
    vert_f = [np.ascontiguousarray(deformed(f), np.float32) for f in range(n_frames)]
    r = xr.Renderer(W, H, device=local)
    r.set_params(xr.params_default(W, H))
    r.upload_scenes([big, small, small2])
    fi = 0
    for _ in range(args.warmup):
        r.update_vertices(2, vert_f[fi])
        r.set_instances(inst_f[fi])
        r.render(ubos[fi]); fi += 1
    r.sync()
    _barrier(dist, local)
    clocks = ClockSampler(local)
    clocks.start()
    t_tlas, t_refit, t_frame = [], [], []
    t0 = time.perf_counter()
    for _ in range(args.steps):
        r.update_vertices(2, vert_f[fi])
        r.set_instances(inst_f[fi])
        r.render(ubos[fi]); fi += 1
        st = r.stats()   # synchronises: the frame's device times
        t_tlas.append(st.ms_tlas_build); t_refit.append(st.ms_refit); t_frame.append(st.ms_frame)
    wall = (time.perf_counter() - t0) * 1e3 / args.steps
    clk = clocks.stop()
    st = r.stats()
    r.close()
    wall = _max_over_ranks(dist, wall, f"cuda:{local}")
    if rank != 0:
        return
    line = {
        "metric": "ms/frame 1080p, 1M-triangle scene + 256 moving instances + a deforming mesh "
                  "(top-level rebuild and refit every frame)",
        "value": round(wall, 4), "unit": "ms/frame", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(wall, 4), "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (procedural scenes, seeds 1, 77, 78)",
        "config": {"workload": f"procedural 1920x1080, {big.n_triangles} + 256 x ~{small.n_triangles} triangles, "
                               "corrected ReSTIR GI, depth 4; per frame: update_vertices + set_instances + render",
                   "instances": DYN_INSTANCES + 1, "parallelism": f"replicas x{ws}"},
        "device_ms": {"frame": round(float(np.mean(t_frame)), 4), "tlas_build": round(float(np.mean(t_tlas)), 4),
                      "refit": round(float(np.mean(t_refit)), 4)},
        "tlas_nodes": st.tlas_nodes,
        "gpu_launches": FRAME_LAUNCHES * args.steps,
        "gpu_launches_note": "frame kernels only; each top-level build and refit adds its own launches",
        "clocks": clk,
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=240)
    ap.add_argument("--warmup", type=int, default=8)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=20.0)
    ap.add_argument("--relmse-spp", type=int, default=1024, help="spp of the FP64 reference (0: skip relMSE)")
    ap.add_argument("--width", type=int, default=1920, help="smaller extents are for profiling only")
    ap.add_argument("--height", type=int, default=1080)
    ap.add_argument("--objects", type=int, default=4096, help="scene objects (4096 -> 998,442 triangles)")
    ap.add_argument("--workload", default="frame", choices=["frame", "batch", "4k", "dynamic", "cornell", "sibenik"],
                    help="frame: 1080p / 1M triangles (the headline); cornell: configuration 0 (256x256, "
                         "8 frames, FP64 reference of 65,536 spp); batch: 64 views over 8 scenes; "
                         "4k: 4 x 3840x2160 streams, 8M triangles, learned cache; "
                         "dynamic: moving instances and a refitted mesh")
    args = ap.parse_args()
    global W, H
    W, H = args.width, args.height
    SCENE_KW["n_objects"] = args.objects
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "batch":
        run_batch(args)
    elif args.workload == "4k":
        run_4k(args)
    elif args.workload == "dynamic":
        run_dynamic(args)
    elif args.workload == "cornell":
        run_cornell(args)
    elif args.workload == "sibenik":
        run_sibenik(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
