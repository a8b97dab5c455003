#!/usr/bin/env python
"""Headline benchmark: the plain unidirectional path tracer at 1920x1080,
4 spp, max depth 8, Russian roulette from depth 3, next-event estimation
against 1024 emissive triangles, on a seeded procedural scene of 1.16M
triangles (512x512 value-noise height field + 2000 icospheres of 320
triangles + 512 emissive quads), SAH BVH with leaves of at most 4.

One step renders one frame through the attachment API (kgr_render).  `value`
is Mrays/s (camera + bounce + shadow rays) with the scene resident on the
device; `e2e` is the same metric through the C ABI with the frame read back
to pinned host memory every step.  The roofline entry is computed live from
CUDA events the library records after every launch on the render stream and
from the traversal visit counts of one counting frame.  `equal_relmse`
compares the radiance-cached tracer (BF16 and FP16 networks) with the plain
tracer on the radiance cache's own configuration, the ReSTIR DI box scene
at 1080p: ms/frame and relMSE against an FP64-accumulated 4096-spp render,
and the speed-up at equal or lower relMSE; `equal_relmse_terrain` repeats
it on the headline terrain frame.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Under torchrun each rank renders its own frame (replicas: the path does not
shard across GPUs); `value` is the sum over ranks divided by the slowest
rank's time.  `--impl reference` times the reference's per-pixel CPU path
(the oracle restatement) on all host cores on a bounded crop of the same
frame.
"""
import argparse
import ctypes
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "1080p ms/frame & Mrays/s at equal relMSE vs plain GPU PT; serve p50/p99 latency"
WORKLOAD = ("plain PT 1920x1080 4spp, max depth 8, RR from depth 3, NEE over 1024 emissive tris; "
            "procedural terrain 1.16M tris (512^2 height field + 2000 icospheres), SAH leaves<=4")

# Kernel behind each traversal stage, per layout.
KERNELS = {("trace_closest", "fast"): "fast_persistent_kernel<closest, fast>",
           ("shadow", "fast"): "shadow_resolve_kernel<fast> | fast_persistent_kernel<any, fast>",
           ("trace_closest", "wide"): "fast_persistent_kernel<closest, wide>",
           ("shadow", "wide"): "shadow_resolve_kernel<wide> | fast_persistent_kernel<any, wide>",
           ("trace_closest", "cw8"): "cw_persistent_kernel<closest>",
           ("shadow", "cw8"): "shadow_resolve_kernel<cw8> | cw_persistent_kernel<any>",
           ("trace_closest", "threaded"): "trace_closest_kernel<threaded>",
           ("shadow", "threaded"): "shadow_resolve_kernel<threaded>"}
# bytes a visit reads on each layout: (node, triangle)
LAYOUT_BYTES = {"fast": (64, 48), "wide": (128, 48), "cw8": (80, 48), "threaded": (48, 80)}
# DRAM bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum) of the
# traversal kernels at this workload: one ncu capture of the 9 closest-hit and
# 9 shadow launches of a timed 1080p frame (--cache-control none), averaged
# per launch; None where not captured.
TRAFFIC = {("trace_closest", "fast"): 173.3e6, ("shadow", "fast"): 279.0e6}


def parse(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=60)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--width", type=int, default=1920)
    ap.add_argument("--height", type=int, default=1080)
    ap.add_argument("--spp", type=int, default=4)
    ap.add_argument("--max-depth", type=int, default=8)
    ap.add_argument("--scene", default="terrain")
    ap.add_argument("--layout", default="auto", choices=["auto", "fast", "wide", "cw8", "threaded"],
                    help="auto: the autotuner picks layout, shadow kernel and block size before warm-up")
    ap.add_argument("--trace-shadow", choices=["grid", "persistent"], help="shadow kernel (with --layout)")
    ap.add_argument("--trace-block", type=int, choices=[64, 128, 256], help="traversal block size (with --layout)")
    ap.add_argument("--trace-occupancy", type=int, choices=[0, 1], help="register cap (with --layout)")
    ap.add_argument("--trace-stack", type=int, choices=[0, 8, 16], help="shared-memory stack entries (with --layout)")
    ap.add_argument("--trace-overlap", type=int, choices=[0, 1], default=1,
                    help="1: a bounce's shadow rays overlap the next bounce's closest hits (two streams)")
    ap.add_argument("--cpu-seconds", type=float, default=12.0, help="target CPU sample time per measurement")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-quality", action="store_true",
                    help="skip the cached-vs-plain comparison at equal relMSE")
    ap.add_argument("--ref-spp", type=int, default=4096, help="spp of the FP64-accumulated reference image")
    ap.add_argument("--quality-scene", default="box4k",
                    help="scene of the radiance-cache comparison (the ReSTIR DI box scene at 1080p)")
    ap.add_argument("--no-serve", action="store_true", help="skip the serving run")
    ap.add_argument("--no-restir", action="store_true", help="skip the ReSTIR DI (256^2) and GI (1080p) runs")
    ap.add_argument("--serve-seconds", type=float, default=1.0, help="arrival window of the 200 req/s phase")
    ap.add_argument("--no-mamba", action="store_true", help="skip the Mamba (editor GI mode) run")
    return ap.parse_args(argv)


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def aggregate_ranks(ms, rays, ws, device):
    """Whole-job totals of a timed region run on every rank: (the slowest
    rank's milliseconds, the rays of all ranks).  Identity on one rank."""
    if ws <= 1:
        return ms, rays
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(ms), float(rays)], dtype=torch.float64, device=device)
    tmax = t.clone()
    dist.all_reduce(tmax, op=dist.ReduceOp.MAX)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(tmax[0]), float(t[1])


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": float(max(smax)) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def make_scene(name):
    from artemis_gb300 import kgr
    g = kgr.Generated(name, 1)
    sc = kgr.Scene.from_generated(g, builder=kgr.BUILDER_SAH, max_leaf=4)
    return g, sc


def cpu_sample(osc, cam, args, target_s):
    """Oracle PT (reference per-pixel path, all host cores) on a crop of rows
    of the same frame, sized to about target_s seconds.  osc is an oracle
    Scene and cam a camera dict {center, ax_u, ax_v, ax_w}.  Returns
    (run(rows, frame) -> (seconds, rays, rows), rows, cores)."""
    from oracle import pyoracle
    cores = os.cpu_count() or 1
    mid = args.height // 2

    def run(rows, frame=0):
        r0 = max(0, mid - rows // 2)
        p = pyoracle.render_params(args.width, args.height, cam, max_depth=args.max_depth,
                                   spp=args.spp, russian_roulette=1, rr_start_depth=3, frame=frame,
                                   row_begin=r0, row_end=min(args.height, r0 + rows), threads=cores)
        bufs = [np.zeros((args.width * args.height, 4), np.float32) for _ in range(4)]
        t = time.perf_counter()
        _, st = pyoracle.render_pt(osc, p, bufs)
        dt = time.perf_counter() - t
        return dt, st.camera_rays + st.bounce_rays + st.shadow_rays, min(args.height, r0 + rows) - r0

    dt, rays, rows = run(4)
    want = int(max(4, min(args.height, 4 * target_s / max(dt, 1e-3))))
    return run, want, cores


def bench_reference(args):
    """The reference arm: the oracle's restatement of the reference's
    per-pixel path tracer on all host cores.  Everything it uses -- the
    procedural scene, the SAH BVH (leaves <= 4), the triangle lights and the
    camera frame -- comes from the oracle library alone (oracle/scene_ref.cpp,
    checked bit for bit against the product's by tests/test_oracle_scene.py);
    the product library is never loaded on this arm."""
    ws, rank, local = dist_env()
    if rank != 0:
        return
    from oracle import pyoracle
    g = pyoracle.GeneratedScene(args.scene, 1)
    osc = g.scene(max_leaf=4)
    cam = pyoracle.camera(g.eye, g.target, g.fov, args.width / args.height)
    # bound the whole run to about 150 s of CPU work however many steps are asked
    per_step = min(args.cpu_seconds, 150.0 / max(1, args.steps + args.warmup))
    run, rows, cores = cpu_sample(osc, cam, args, per_step)
    for _ in range(args.warmup):
        run(max(4, rows // 8))
    times, rays_total, rows_done = [], 0, 0
    for s in range(args.steps):
        dt, rays, r = run(rows, frame=s)
        times.append(dt)
        rays_total += rays
        rows_done += r
    mrays = rays_total / sum(times) / 1e6
    ms_frame = sum(times) / rows_done * args.height * 1e3
    sample = f"{rows} centre rows x {args.width} px x {args.spp} spp per step ({rows / args.height:.3f} of the frame)"
    line = {"metric": METRIC, "value": round(mrays, 4), "unit": "Mrays/s", "impl": "reference",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(ms_frame, 2), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded procedural scene, random-free camera)",
            "config": {"workload": WORKLOAD, "scene": args.scene, "triangles": int(len(g.indices)),
                       "lights": int(len(osc.lights)), "resolution": [args.width, args.height], "spp": args.spp,
                       "max_depth": args.max_depth, "crop": sample, "l2_flush": False,
                       "parallelism": f"{cores} host threads (OpenMP over pixels)"},
            "cpu_baseline": {"value": round(mrays, 4), "unit": "Mrays/s", "cores": cores, "kind": "port",
                             "sample": sample},
            "e2e": {"value": round(mrays, 4), "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def relmse_compare(args, scene_name, g, sc, W, H, stream, sptr):
    """ms/frame and relMSE of the plain and the radiance-cached tracer (BF16
    and FP16 networks) against an FP64-accumulated plain render of
    `--ref-spp` samples per pixel, on `scene_name` (g, sc: that scene, or
    None to generate it).

    relMSE = mean over pixels and RGB of (x - ref)^2 / (ref^2 + 0.01).  Each
    cached configuration is compared with the costliest plain configuration
    whose relMSE is still at or above its own, so the speed-up is at equal or
    lower error; the cache trains online (one Adam step per frame) for 300
    frames first and keeps training while it is timed.  `denoised` gives the
    relMSE of the same frames after the a-trous denoiser and the denoiser's
    own time (a post-process beside the comparison, not part of it)."""
    import torch

    from artemis_gb300 import kgr

    own = g is None
    if own:
        g = kgr.Generated(scene_name, 1)
        sc = kgr.Scene.from_generated(g)
    cam = kgr.camera(g.eye, g.target, g.fov, W / H)
    bufs = [torch.zeros((W * H, 4), dtype=torch.float32, device="cuda") for _ in range(4)]
    ptrs = [b.data_ptr() for b in bufs]

    def make(spp, cache=None):
        a = kgr.Attachment("path_tracer")
        a.attach(W, H)
        a.load()
        a.set_option("spp", spp)
        a.set_option("russian_roulette", True)
        a.set_option("rr_start_depth", 3)
        for k, v in args.trace_options.items():
            a.set_option(k, v)
        if cache:
            a.set_option("cache", True)
            a.set_option("cache_dtype", cache)
        return a

    def info(f):
        return kgr.launch_info(cam, W, H, ptrs, max_depth=args.max_depth, frame=f)

    t0 = time.perf_counter()
    per = 16
    ref = torch.zeros((W * H, 3), dtype=torch.float64, device="cuda")
    a = make(per)
    frames = max(1, args.ref_spp // per)
    for f in range(frames):
        a.render(info(1 << 20 | f), sc, sptr)
        ref += bufs[0][:, :3].double()
    ref /= frames
    a.close()
    torch.cuda.synchronize()
    ref_s = time.perf_counter() - t0

    def relmse():
        d = bufs[0][:, :3].double() - ref
        return (d * d / (ref * ref + 1e-2)).mean().item()

    dn = kgr.Denoiser(W, H)
    dout = torch.zeros((W * H, 4), dtype=torch.float32, device="cuda")

    def relmse_of(x):
        d = x[:, :3].double() - ref
        return (d * d / (ref * ref + 1e-2)).mean().item()

    def measure(a, first, n=8, warm=3, denoise=False):
        for f in range(warm):
            a.render(info(first + f), sc, sptr)
        ms, err, dms, derr = [], [], [], []
        for f in range(n):
            e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
            e0.record(stream)
            a.render(info(first + warm + f), sc, sptr)
            e1.record(stream)
            if denoise:
                dn.denoise(ptrs[0], ptrs[1], ptrs[2], ptrs[3], stream=sptr)
            e2.record(stream)
            e2.synchronize()
            ms.append(e0.elapsed_time(e1))
            err.append(relmse())
            if denoise:
                dms.append(e1.elapsed_time(e2))
                dn.copy_result(dhost)
                derr.append(relmse_of(torch.from_numpy(dhost).cuda()))
        r = (round(float(np.median(ms)), 3), round(float(np.mean(err)), 4))
        if denoise:
            r += (round(float(np.median(dms)), 3), round(float(np.mean(derr)), 4))
        return r

    dhost = np.zeros((W * H, 4), np.float32)
    plain, plain_dn = {}, {}
    for spp in (1, 2, 4, 8, 16, 32):
        a = make(spp)
        r = measure(a, 1000 * spp, denoise=spp <= 4)
        plain[spp] = r[:2]
        if spp <= 4:
            plain_dn[spp] = r[2:]
        a.close()
    cached, cached_dn = {"bf16": {}, "fp16": {}}, {}
    for dtype in ("bf16", "fp16"):
        for spp in (1, 2, 4):
            a = make(spp, cache=dtype)
            for f in range(300):
                a.render(info(50000 + f), sc, sptr)
            r = measure(a, 60000, denoise=dtype == "bf16")
            cached[dtype][spp] = r[:2]
            if dtype == "bf16":
                cached_dn[spp] = r[2:]
            a.close()
    dn.close()
    compare = []
    for dtype in ("bf16", "fp16"):
        for spp, (ms, err) in cached[dtype].items():
            worse = [k for k, (_, e) in plain.items() if e >= err]
            if worse:
                k = max(worse)
                compare.append({"dtype": dtype, "cached_spp": spp, "cached_ms": ms, "cached_relmse": err,
                                "plain_spp": k, "plain_ms": plain[k][0], "plain_relmse": plain[k][1],
                                "speedup": round(plain[k][0] / ms, 2)})
    best = max(compare, key=lambda c: c["speedup"]) if compare else None
    if own:
        sc.close()
    return {"scene": scene_name, "resolution": [W, H], "reference": f"plain PT, {frames * per} spp, FP64 mean",
            "reference_s": round(ref_s, 1), "relmse": "mean (x - ref)^2 / (ref^2 + 0.01)",
            "plain": {str(k): {"ms": v[0], "relmse": v[1]} for k, v in plain.items()},
            "cached_bf16": {str(k): {"ms": v[0], "relmse": v[1]} for k, v in cached["bf16"].items()},
            "cached_fp16": {str(k): {"ms": v[0], "relmse": v[1]} for k, v in cached["fp16"].items()},
            "at_equal_or_lower_relmse": compare, "best_speedup": best and best["speedup"],
            "denoised": {"denoiser": "a-trous, 5 passes, normal + albedo + position guides",
                         "plain": {str(k): {"denoise_ms": v[0], "relmse": v[1]} for k, v in plain_dn.items()},
                         "cached_bf16": {str(k): {"denoise_ms": v[0], "relmse": v[1]} for k, v in cached_dn.items()}}}


def restir_runs(args):
    """ReSTIR DI on the box scene (12 + 4096 + 128 triangles, 64 ceiling
    quads) at 256x256, 1 spp, 32 candidates, temporal reuse (M-cap 20), one
    spatial pass (5 neighbours, 30 px), depth 2: GPU ms/frame, and the
    oracle's per-pixel CPU frame on all host cores.

    ReSTIR GI on the 4.1M-triangle scene (65,536 emissive triangles,
    log-uniform radiance) at 1920x1080 over 16 frames of a camera orbit of
    0.5 degrees per frame with sub-pixel jitter: 32 DI candidates, one GI
    sample per pixel, temporal reuse (M-cap 30), 3 spatial iterations x 8
    neighbours, depth 8 with Russian roulette from 3.  ms/frame (median), and
    the relMSE of the last frame -- and of 1-spp and 4-spp plain frames -- against
    an FP64-accumulated plain render of `--ref-spp` samples at that camera."""
    import torch

    from oracle import pyoracle

    from artemis_gb300 import kgr

    out = {}
    stream = torch.cuda.current_stream()
    sptr = ctypes.c_void_p(stream.cuda_stream)

    def timed(fn):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fn()
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1)

    # --- ReSTIR DI, 256^2 (and the same scene at 1080p for the resampling roofline)
    g = kgr.Generated("box4k", 0x4B4F4252)
    sc = kgr.Scene.from_generated(g)
    opts = {"candidates": 32, "temporal": True, "temporal_mcap": 20, "spatial_passes": 1,
            "spatial_neighbors": 5, "spatial_radius": 30}
    k_nb, passes = opts["spatial_neighbors"], opts["spatial_passes"]
    l2_gbs = kgr.read_bandwidth(64 << 20, 50)
    hbm = measured_peaks()[0].get("hbm_gbs")

    def di_run(W, H, timed_frames):
        cam = kgr.camera(g.eye, g.target, g.fov, W / H)
        bufs = [torch.zeros((W * H, 4), dtype=torch.float32, device="cuda") for _ in range(4)]
        att = kgr.Attachment("restir_di")
        att.attach(W, H)
        att.load()
        for k, v in opts.items():
            att.set_option(k, v)
        info = lambda f: kgr.launch_info(cam, W, H, [b.data_ptr() for b in bufs], max_depth=2, frame=f)
        for f in range(5):
            att.render(info(f), sc, sptr)
        ms = [timed(lambda f=f: att.render(info(5 + f), sc, sptr)) for f in range(timed_frames)]
        # per-stage CUDA-event times of further frames: the resampling
        # kernels apart from the reuse passes' visibility rays
        att.set_option("profile", True)
        att.stage_times()
        nprof = 10
        for f in range(nprof):
            att.render(info(5 + timed_frames + f), sc, sptr)
        stages = att.stage_times()
        att.set_option("profile", False)
        frame = bufs[0][:, :3].double().clone()
        att.close()
        npix = W * H
        # algorithmic bytes per pixel per pass: temporal = two 32 B reservoir
        # reads + a 32 B write + 48 B of G-buffer; spatial = (1 + k)(32 + 48) B
        # + a 32 B write
        temporal_b = npix * (2 * 32 + 32 + 48)
        spatial_b = npix * ((1 + k_nb) * (32 + 48) + 32) * passes
        entry = {"resolution": [W, H], "gpu_ms_per_frame": round(float(np.median(ms)), 3)}
        for name, stage, nbytes in (("temporal", "restir_temporal", temporal_b),
                                    ("spatial", "restir_spatial", spatial_b)):
            t_ms = stages[stage][0] / nprof
            gbs = nbytes / (t_ms * 1e-3) / 1e9
            entry[name] = {"kernels_ms_per_frame": round(t_ms, 4), "bytes_per_frame": nbytes,
                           "achieved_gbs": round(gbs, 1), "l2_frac": round(gbs / l2_gbs, 4),
                           "hbm_frac": round(gbs / hbm, 4) if hbm else None,
                           "visibility_ms_per_frame": round(stages[stage + "_vis"][0] / nprof, 4)}
        return cam, frame, entry

    cam, di_frame, di256 = di_run(256, 256, 20)
    # relMSE of the ReSTIR DI frame against an FP64 mean of 4096 spp of the
    # plain tracer at the same depth (direct + one indirect bounce)
    W = H = 256
    bufs = [torch.zeros((W * H, 4), dtype=torch.float32, device="cuda") for _ in range(4)]
    ref = torch.zeros((W * H, 3), dtype=torch.float64, device="cuda")
    a = kgr.Attachment("path_tracer")
    a.attach(W, H)
    a.load()
    a.set_option("spp", 64)
    for f in range(64):
        a.render(kgr.launch_info(cam, W, H, [b.data_ptr() for b in bufs], max_depth=2, frame=1 << 20 | f), sc, sptr)
        ref += bufs[0][:, :3].double()
    ref /= 64
    a.set_option("spp", 1)
    a.render(kgr.launch_info(cam, W, H, [b.data_ptr() for b in bufs], max_depth=2, frame=4242), sc, sptr)
    plain1 = bufs[0][:, :3].double().clone()
    a.close()

    def relmse_di(x):
        d = x - ref
        return round((d * d / (ref * ref + 1e-2)).mean().item(), 4)

    osc = pyoracle.Scene(g.positions, g.normals, g.tris4(), g.materials_raw, sc.lights(), sc.bvh())
    state = pyoracle.RestirBuffers(W * H)
    t0 = time.perf_counter()
    p = pyoracle.render_params(W, H, kgr.camera_dict(cam), max_depth=2, spp=1, frame=0, candidates=32, temporal=1,
                               temporal_mcap=20, spatial_passes=1, spatial_neighbors=5, spatial_radius=30)
    pyoracle.render_restir(osc, p, state)
    cpu_s = time.perf_counter() - t0
    _, _, di1080 = di_run(1920, 1080, 10)
    # the direct light alone (max_depth 0), where ReSTIR's reuse acts: the
    # DI frame against plain 1 spp, also on 99.9% of pixels (the 0.1% worst
    # of each image trimmed: the reference's bias-corrected spatial weight
    # leaves a few outliers)
    ref0 = torch.zeros((W * H, 3), dtype=torch.float64, device="cuda")
    a = kgr.Attachment("path_tracer")
    a.attach(W, H)
    a.load()
    a.set_option("spp", 64)
    for f in range(64):
        a.render(kgr.launch_info(cam, W, H, [b.data_ptr() for b in bufs], max_depth=0, frame=1 << 21 | f), sc, sptr)
        ref0 += bufs[0][:, :3].double()
    ref0 /= 64
    a.set_option("spp", 1)
    a.render(kgr.launch_info(cam, W, H, [b.data_ptr() for b in bufs], max_depth=0, frame=4343), sc, sptr)
    plain0 = bufs[0][:, :3].double().clone()
    a.close()
    att0 = kgr.Attachment("restir_di")
    att0.attach(W, H)
    att0.load()
    for k, v in opts.items():
        att0.set_option(k, v)
    for f in range(30):
        att0.render(kgr.launch_info(cam, W, H, [b.data_ptr() for b in bufs], max_depth=0, frame=f), sc, sptr)
    di0 = bufs[0][:, :3].double().clone()
    att0.close()

    def relmse_pair(x, r):
        e = ((x - r) ** 2 / (r * r + 1e-2)).mean(dim=1)
        q = torch.quantile(e.float(), 0.999).item()
        return {"all": round(e.mean().item(), 4), "trimmed_999": round(e[e <= q].mean().item(), 4)}

    out["restir_di_256"] = {"gpu_ms_per_frame": di256["gpu_ms_per_frame"],
                            "cpu_oracle_ms_per_frame": round(cpu_s * 1e3, 1), "cpu_cores": os.cpu_count(),
                            "scene_triangles": sc.info().triangle_count,
                            "relmse": relmse_di(di_frame), "plain_1spp_relmse": relmse_di(plain1),
                            "relmse_reference": "plain PT at depth 2, 4096 spp, FP64 mean, same camera",
                            "direct_only": {"restir_di": relmse_pair(di0, ref0), "plain_1spp": relmse_pair(plain0, ref0),
                                            "reference": "plain PT at depth 0, 4096 spp, FP64 mean; DI frame 30"}}
    out["roofline_resampling"] = {
        "bound": "l2", "unit": "GB/s", "peak_l2_read_gbs": round(l2_gbs, 1), "peak_hbm_gbs": hbm,
        "work_unit": "per pixel per pass: temporal 2x32 + 32 + 48 B; spatial (1+k)(32+48) + 32 B, k = 5",
        "timing": "CUDA events after each launch on the render stream; resampling kernels only (temporal gather "
                  "and merge; spatial gather, resample and finish), the reuse passes' visibility rays apart",
        "c1_256": di256, "box_1080p": di1080}
    sc.close()

    # --- ReSTIR GI, 1080p, 16-frame orbit
    g = kgr.Generated("terrain_l", 1)
    sc = kgr.Scene.from_generated(g)
    W, H = 1920, 1080
    bufs = [torch.zeros((W * H, 4), dtype=torch.float32, device="cuda") for _ in range(4)]
    ptrs = [b.data_ptr() for b in bufs]
    eye0, tgt = np.array(g.eye, np.float64), np.array(g.target, np.float64)

    def orbit(f):
        a = np.radians(0.5 * f)
        d = eye0 - tgt
        e = tgt + np.array([d[0] * np.cos(a) + d[2] * np.sin(a), d[1], -d[0] * np.sin(a) + d[2] * np.cos(a)])
        return kgr.camera(e.astype(np.float32), g.target, g.fov, W / H)

    att = kgr.Attachment("restir_gi")
    att.attach(W, H)
    att.load()
    for k, v in {"candidates": 32, "gi_mcap": 30, "gi_spatial_iterations": 3, "gi_neighbors": 8,
                 "russian_roulette": True, "rr_start_depth": 3}.items():
        att.set_option(k, v)
    gi_ms = []
    for f in range(16):
        c = orbit(f)
        gi_ms.append(timed(lambda: att.render(kgr.launch_info(c, W, H, ptrs, max_depth=8, frame=f), sc, sptr)))
    last = [bufs[0][:, :3].double().clone()]
    # two more runs of the same orbit with other random streams: frame 15's
    # relMSE is dominated by a handful of pixels, so one run is a noisy figure
    for base in (1000, 2000):
        att.set_option("reset_history", True)
        for f in range(16):
            att.render(kgr.launch_info(orbit(f), W, H, ptrs, max_depth=8, frame=base + f), sc, sptr)
        last.append(bufs[0][:, :3].double().clone())
    att.close()
    cam = orbit(15)
    ref = torch.zeros((W * H, 3), dtype=torch.float64, device="cuda")

    def plain(spp, frames, first):
        a = kgr.Attachment("path_tracer")
        a.attach(W, H)
        a.load()
        a.set_option("spp", spp)
        a.set_option("russian_roulette", True)
        a.set_option("rr_start_depth", 3)
        return a

    per = 16
    a = plain(per, 0, 0)
    nref = max(1, args.ref_spp // per)
    for f in range(nref):
        a.render(kgr.launch_info(cam, W, H, ptrs, max_depth=8, frame=1 << 20 | f), sc, sptr)
        ref += bufs[0][:, :3].double()
    a.close()
    ref /= nref

    def relmse(x):
        d = x - ref
        return round((d * d / (ref * ref + 1e-2)).mean().item(), 4)

    def relmse_trimmed(x):
        e = ((x - ref) ** 2 / (ref * ref + 1e-2)).mean(dim=1)
        return round(e[e <= torch.quantile(e.float(), 0.999).item()].mean().item(), 4)

    res = {}
    for spp in (1, 4):
        a = plain(spp, 0, 0)
        a.render(kgr.launch_info(cam, W, H, ptrs, max_depth=8, frame=777), sc, sptr)
        ms_p = timed(lambda: a.render(kgr.launch_info(cam, W, H, ptrs, max_depth=8, frame=778), sc, sptr))
        frames = [bufs[0][:, :3].double().clone()]
        for f in (779, 780):
            a.render(kgr.launch_info(cam, W, H, ptrs, max_depth=8, frame=f), sc, sptr)
            frames.append(bufs[0][:, :3].double().clone())
        rel = [relmse(x) for x in frames]
        res[spp] = {"ms": round(ms_p, 3), "relmse_runs": rel, "relmse_mean": round(float(np.mean(rel)), 4),
                    "relmse_trimmed_999": relmse_trimmed(frames[0])}
        a.close()
    gi_rel = [relmse(x) for x in last]
    out["restir_gi_1080p"] = {"scene_triangles": sc.info().triangle_count, "lights": sc.info().light_count,
                              "frames": 16, "ms_per_frame_median": round(float(np.median(gi_ms)), 3),
                              "ms_first_frame": round(gi_ms[0], 3),
                              "relmse_last_frame": gi_rel[0], "relmse_last_frame_runs": gi_rel,
                              "relmse_last_frame_mean": round(float(np.mean(gi_rel)), 4),
                              "relmse_last_frame_trimmed_999": relmse_trimmed(last[0]),
                              "runs": "three runs of the orbit with independent random streams",
                              "plain_1spp": res[1], "plain_4spp": res[4],
                              "reference": f"plain PT, {nref * per} spp, FP64 mean, camera of frame 15"}
    sc.close()
    return out


def mamba_run(args, g, sc, W, H):
    """The "mamba" attachment (the editor's default GI mode, editor/mamba.cu:
    1094-1300) on the benchmark's scene and resolution with direct lighting,
    temporal and spatial reuse: 3 warm-up frames, then `MAMBA_FRAMES` frames
    timed one by one with CUDA events on the render stream (median), the
    first frame's time (it allocates most probes), the per-stage split of
    the timed frames, and one oracle frame of the same configuration on all
    host cores (oracle_mamba_frame; its third frame, state carried)."""
    import torch

    from artemis_gb300 import kgr

    stream = torch.cuda.current_stream()
    sptr = ctypes.c_void_p(stream.cuda_stream)
    bufs = [torch.zeros((W * H, 4), dtype=torch.float32, device="cuda") for _ in range(4)]
    ptrs = [b.data_ptr() for b in bufs]
    cam = kgr.camera(g.eye, g.target, g.fov, W / H)
    flags = {"direct_lighting": True, "temporal_reuse": True, "spatial_reuse": True}
    att = kgr.Attachment("mamba")
    att.attach(W, H)
    for k, v in {**flags, "profile": True}.items():
        att.set_option(k, v)
    att.load()

    def frame(f):
        info = kgr.launch_info(cam, W, H, ptrs, samples=f)
        info.time = 0.1 * f
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        att.render(info, sc, sptr)
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1)

    first = frame(0)
    for f in range(1, 3):
        frame(f)
    att.stage_times()
    ms = [frame(f) for f in range(3, 3 + MAMBA_FRAMES)]
    st = att.stage_times()
    counters = np.zeros(2, np.int32)
    att.debug_copy("mamba_counters", counters)
    launches = att.stats().kernel_launches
    att.close()
    out = {"scene": args.scene, "triangles": sc.info().triangle_count, "resolution": [W, H],
           "options": sorted(flags), "frames_timed": MAMBA_FRAMES,
           "ms_per_frame_median": round(float(np.median(ms)), 3), "ms_first_frame": round(first, 3),
           "stage_ms_per_frame": {k: round(v[0] / MAMBA_FRAMES, 3) for k, v in st.items()
                                  if v[1] and k in MAMBA_STAGES},
           "probes": int(counters[0]), "lookup_tables": int(counters[1]), "kernel_launches_per_frame": launches}
    if not args.no_cpu_baseline:
        try:
            from oracle import pyoracle
            osc = pyoracle.Scene(g.positions, g.normals, g.tris4(), g.materials_raw, sc.lights(), sc.bvh())
            om = pyoracle.Mamba(W, H, 1 << 16, 64)  # the probe count stays far below either capacity
            d = kgr.camera_dict(cam)
            for f in range(3):
                t0 = time.time()
                om.frame(osc, pyoracle.mamba_params(W, H, d, time=0.1 * f, samples=f,
                                                    **{k: int(v) for k, v in flags.items()}))
                dt = time.time() - t0
            om.close()
            out["cpu_oracle"] = {"ms_per_frame": round(dt * 1e3, 1), "cores": os.cpu_count(),
                                 "sample": "third frame, state carried from two before"}
        except Exception as exc:  # reported, not required
            out["cpu_oracle"] = {"ms_per_frame": None, "sample": f"failed: {exc}"}
    return out


MAMBA_FRAMES = 20
MAMBA_STAGES = ("generate", "trace_closest", "restir_primary", "restir_temporal", "restir_spatial",
                "restir_temporal_vis", "restir_spatial_vis", "mamba_secondary", "mamba_gather", "mamba_probes",
                "mamba_final")

SERVE_RES = [(320, 240), (640, 480), (1280, 720), (1920, 1080), (3840, 2160)]
SERVE_SCENES = ("terrain_s", "terrain_m", "terrain_l")  # 0.26M, 1.0M, 4.1M triangles


def serve_run(args):
    """The render server under a Poisson request stream: resolution uniform
    over SERVE_RES, spp uniform in [1, 16], scene uniform over three
    resident procedural scenes, half path-tracer and half ReSTIR DI requests
    (ReSTIR: spp frames accumulated), depth 8 with Russian roulette from 3,
    admission by a 120 GB budget.  Phase 1 offers 200 req/s for
    --serve-seconds; phase 2 offers half the request rate phase 1 completed,
    for 10 s.  `mpaths_per_s` counts pixels x spp of every completed request;
    `mrays_per_s` the camera, bounce and shadow rays of every tick, counted
    on the device (ReSTIR DI's reuse-pass visibility rays included).  Latency
    = submission to image in host memory;
    `latency_per_mpath` divides it by the request's paths (pixels x spp),
    which removes the 1700x spread of request sizes; `by_resolution` gives
    p50/p99 per resolution class; `slowdown` replays every request of the
    sustainable phase alone on the idle server and divides its latency in
    the stream by its latency alone.  The server schedules with processor
    sharing (KGR_SCHEDULE_FAIR) and tunes each scene's traversal launch shape
    before its first tick (the warm-up requests of every scene trigger it)."""
    from artemis_gb300 import kgr

    t_build = time.perf_counter()
    gens = [kgr.Generated(n, 1) for n in SERVE_SCENES]
    scenes = [kgr.Scene.from_generated(g) for g in gens]
    build_s = time.perf_counter() - t_build
    srv = kgr.Server(path_capacity=1 << 24, max_jobs=256, spp_per_tick=4, memory_budget=120 << 30,
                     policy=kgr.SCHEDULE_FAIR, autotune=True)
    sids = [srv.add_scene(sc) for sc in scenes]

    def submit(i, w, h, spp, kind, frame):
        g = gens[i]
        out = np.empty((w * h, 4), np.float32)
        return srv.submit(sids[i], w, h, spp, g.eye, g.target, g.fov, out, kind=kind, max_depth=8, frame=frame,
                          russian_roulette=True, rr_start_depth=3)

    # warm-up: every scene, resolution and kind once (each scene's launch-shape
    # tuning, ReSTIR attachments, graphs), so that none of it runs in a phase
    warm = [submit(i, w, h, 1, k, 0) for i in range(len(gens)) for (w, h) in SERVE_RES
            for k in (kgr.REQUEST_PATH_TRACER, kgr.REQUEST_RESTIR_DI)]
    for r in warm:
        srv.wait(r, 600000.0)

    def phase(rate, seconds, seed):
        rng = np.random.default_rng(seed)
        t, arrivals = 0.0, []
        while True:
            t += rng.exponential(1.0 / rate)
            if t > seconds:
                break
            w, h = SERVE_RES[rng.integers(len(SERVE_RES))]
            arrivals.append((t, int(rng.integers(3)), w, h, int(rng.integers(1, 17)),
                             kgr.REQUEST_PATH_TRACER if rng.random() < 0.5 else kgr.REQUEST_RESTIR_DI))
        s0 = srv.stats()
        t0 = time.perf_counter()
        ids = []
        for k, (ta, sc, w, h, spp, kind) in enumerate(arrivals):
            dt = ta - (time.perf_counter() - t0)
            if dt > 0:
                time.sleep(dt)
            ids.append(submit(sc, w, h, spp, kind, k))
        res = [srv.wait(r, 1200000.0) for r in ids]
        wall = time.perf_counter() - t0
        s1 = srv.stats()
        ok = [r for r in res if r.status == 0]
        lat = np.array([r.latency_ms for r in ok])
        mpaths = np.array([w * h * spp / 1e6 for (_, _, w, h, spp, _), r in zip(arrivals, res) if r.status == 0])
        norm = lat / mpaths
        q = lambda a, p: round(float(np.percentile(a, p)), 2) if len(a) else None
        res_of = [(w, h) for (_, _, w, h, _, _), r in zip(arrivals, res) if r.status == 0]
        by_res = {}
        for (w, h) in SERVE_RES:
            a = np.array([x for x, wh in zip(lat, res_of) if wh == (w, h)])
            if len(a):
                by_res[f"{w}x{h}"] = {"n": len(a), "p50": q(a, 50), "p99": q(a, 99)}
        phase.last = (arrivals, res)
        return {"offered_rps": rate, "window_s": seconds, "requests": len(arrivals), "completed": len(ok),
                "failed": len(res) - len(ok), "wall_s": round(wall, 2),
                "completed_rps": round(len(ok) / wall, 2),
                "mpaths_per_s": round(float(mpaths.sum()) / wall, 1),
                "mrays_per_s": round((s1.rays - s0.rays) / wall / 1e6, 1),
                "latency_ms": {"p50": q(lat, 50), "p90": q(lat, 90), "p99": q(lat, 99), "max": q(lat, 100)},
                "latency_per_mpath_ms": {"p50": q(norm, 50), "p99": q(norm, 99)},
                "by_resolution": by_res,
                "queue_ms_p50": q(np.array([r.queue_ms for r in ok]), 50),
                "ticks": int(s1.ticks - s0.ticks)}

    p1 = phase(200.0, args.serve_seconds, 1)
    p2 = phase(max(0.5, 0.5 * p1["completed_rps"]), 10.0, 2)
    # each request of the sustainable phase again, alone on the idle server:
    # its latency without other requests, and the slowdown (latency in the
    # stream / latency alone) that processor sharing keeps even across sizes
    arrivals, res = phase.last
    alone, slow, slow_res = [], [], []
    for k, ((_, sc, w, h, spp, kind), r) in enumerate(zip(arrivals, res)):
        if r.status != 0:
            continue
        a = srv.wait(submit(sc, w, h, spp, kind, k), 1200000.0)
        if a.status == 0:
            alone.append(a.latency_ms)
            slow.append(r.latency_ms / a.latency_ms)
            slow_res.append((w, h))
    slow = np.array(slow)
    qs = lambda a, p: round(float(np.percentile(a, p)), 2) if len(a) else None
    p2["slowdown"] = {"p50": qs(slow, 50), "p90": qs(slow, 90), "p99": qs(slow, 99), "max": qs(slow, 100),
                      "alone_latency_ms": {"p50": qs(np.array(alone), 50), "p99": qs(np.array(alone), 99)},
                      "by_resolution": {f"{w}x{h}": {"p50": qs(a, 50), "p99": qs(a, 99)} for (w, h) in SERVE_RES
                                        for a in [np.array([x for x, wh in zip(slow, slow_res) if wh == (w, h)])]
                                        if len(a)}}
    st = srv.stats()
    out = {"scenes": {n: sc.info().triangle_count for n, sc in zip(SERVE_SCENES, scenes)},
           "scene_build_s": round(build_s, 1),
           "server": {"path_capacity": 1 << 24, "max_jobs": 256, "spp_per_tick": 4, "memory_budget_gb": 120,
                      "graphs": True, "policy": "fair (processor sharing)", "autotune": True},
           "mean_jobs_per_tick": round(st.mean_jobs_per_tick, 2), "graph_replays": int(st.graph_replays),
           "peak_budget_gb": round(st.peak_budget_bytes / 2 ** 30, 2),
           "phase_200rps": p1, "phase_sustainable": p2}
    srv.close()
    for sc in scenes:
        sc.close()
    return out


def bench_ours(args):
    import torch

    from artemis_gb300 import kgr

    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.cuda.current_device()
    W, H = args.width, args.height
    g, sc = make_scene(args.scene)
    info_s = sc.info()
    cam = kgr.camera(g.eye, g.target, g.fov, W / H)
    bufs = [torch.zeros((W * H, 4), dtype=torch.float32, device="cuda") for _ in range(4)]
    att = kgr.Attachment("path_tracer")
    att.attach(W, H, dev)
    att.load()
    att.set_option("spp", args.spp)
    att.set_option("russian_roulette", True)
    att.set_option("rr_start_depth", 3)
    stream = torch.cuda.current_stream()
    sptr = ctypes.c_void_p(stream.cuda_stream)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def info_for(step, samples=0):
        return kgr.launch_info(cam, W, H, [b.data_ptr() for b in bufs], max_depth=args.max_depth,
                               samples=samples, accumulate=False, frame=step)

    tuned = None
    if args.layout == "auto":
        tuned = att.autotune(info_for(0), sc, frames=2, stream=sptr)
        layout = tuned["best"]["layout"]
    else:
        layout = args.layout
        for opt, v in (("trace_shadow", args.trace_shadow), ("trace_block", args.trace_block),
                       ("trace_occupancy", args.trace_occupancy), ("trace_stack", args.trace_stack)):
            if v is not None:
                att.set_option(opt, v)
    att.set_option("layout", layout)
    att.set_option("trace_overlap", bool(args.trace_overlap))
    t = att.trace_tune()
    # the comparison runs and the cached tracer use the same launch shape
    args.trace_options = {"layout": layout, "trace_shadow": t["shadow"], "trace_block": t["block"],
                          "trace_occupancy": t["occupancy"], "trace_stack": t["stack"],
                          "trace_overlap": bool(args.trace_overlap)}
    for s in range(args.warmup):
        att.render(info_for(s), sc, sptr)
    torch.cuda.synchronize()

    # traversal visit counts of one frame (untimed), on the timed layout and on
    # the reference's threaded layout: both layouts give bit-identical paths,
    # so the second count is the reference walk over the same rays
    visits = {}
    for lay in dict.fromkeys((layout, "threaded")):
        att.set_option("layout", lay)
        att.set_option("count_visits", True)
        att.render(info_for(0), sc, sptr)
        torch.cuda.synchronize()
        visits[lay] = att.visit_counts()
    att.set_option("count_visits", False)
    att.set_option("layout", layout)
    att.stats()

    # timed region
    att.set_option("profile", True)
    att.stage_times()
    clocks = ClockSampler(dev)
    clocks.start()
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    step_ms, rays = [], 0
    for s in range(args.steps):
        flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        att.render(info_for(args.warmup + s), sc, sptr)
        e1.record(stream)
        e1.synchronize()
        step_ms.append(e0.elapsed_time(e1))
        st = att.stats()
        rays += st.camera_rays + st.bounce_rays + st.shadow_rays
    torch.cuda.synchronize()
    if ws > 1:
        torch.distributed.barrier()
    clk = clocks.stop()
    stages = att.stage_times()
    att.set_option("profile", False)
    launches_per_frame = st.kernel_launches
    total_ms, rays = aggregate_ranks(float(sum(step_ms)), rays, ws, "cuda")
    value = rays / (total_ms * 1e-3) / 1e6

    # End to end through the C ABI with every frame read back to pinned host
    # memory, as a host streaming frames does it: frames alternate between two
    # output sets, frame s's readback runs on a copy stream while frame s+1
    # renders, and frame s+2 waits for it before writing into the same set.
    # Every step still pays its own device-to-host copy; the clock stops when
    # the last one has landed.
    sets = [bufs, [torch.zeros_like(b) for b in bufs]]
    hosts = [torch.empty((W * H, 4), dtype=torch.float32, pin_memory=True) for _ in range(2)]
    copy_stream = torch.cuda.Stream()
    rendered = [torch.cuda.Event() for _ in range(2)]
    read = [torch.cuda.Event() for _ in range(2)]
    torch.cuda.synchronize()
    if ws > 1:
        torch.distributed.barrier()
    t0 = time.perf_counter()
    e2e_rays = 0
    for s in range(args.steps):
        k = s & 1
        if s >= 2:
            stream.wait_event(read[k])
        att.render(kgr.launch_info(cam, W, H, [b.data_ptr() for b in sets[k]], max_depth=args.max_depth,
                                   samples=0, accumulate=False, frame=1000 + s), sc, sptr)
        rendered[k].record(stream)
        copy_stream.wait_event(rendered[k])
        with torch.cuda.stream(copy_stream):
            hosts[k].copy_(sets[k][0], non_blocking=True)
        read[k].record(copy_stream)
        st = att.stats()  # this frame's ray counts (waits for the frame, not for the copies)
        e2e_rays += st.camera_rays + st.bounce_rays + st.shadow_rays
    copy_stream.synchronize()
    stream.synchronize()
    e2e_s = time.perf_counter() - t0
    if ws > 1:
        torch.distributed.barrier()
    e2e_ms, e2e_rays = aggregate_ranks(e2e_s * 1e3, e2e_rays, ws, "cuda")
    e2e_value = e2e_rays / (e2e_ms * 1e-3) / 1e6

    peaks, peak_kind = measured_peaks()
    l2_gbs = kgr.read_bandwidth(64 << 20, 50, dev)
    # Dominant traversal stage and its algorithmic bytes per launch.  The
    # kernel's own layout fixes what one visit must read (fast BVH2: a 64 B
    # child-pair node per interior visit, a 48 B triangle record per test;
    # wide BVH4: 128 B nodes), times the visits the kernel itself makes
    # (visit counts of one counting frame), divided by the timed kernel's
    # per-launch CUDA-event time.  Its working set (nodes + triangle records,
    # about 80 MB at this workload) stays in the 129 MB L2, so the bound is
    # the L2 read bandwidth measured here by kgr_measure_read_bandwidth.
    # The bytes of the reference's threaded walk over the same rays (48 B per
    # interior record, 80 B per leaf record; 3.5x more visits) are kept as a
    # labelled extra, not as the fraction.
    def stage_bytes(v, node_b, tri_b):
        return {"trace_closest": v[0] * node_b + v[1] * tri_b, "shadow": v[2] * node_b + v[3] * tri_b}

    ref_bytes = stage_bytes(visits["threaded"], *LAYOUT_BYTES["threaded"])
    own_bytes = stage_bytes(visits[layout], *LAYOUT_BYTES[layout])
    # the dominant kernel is the closest-hit walk (48% of a frame's launch
    # time under ncu, against 29% for the shadow walk).  Its CUDA-event time
    # per launch comes from the timed frames.  With the bounce overlap on,
    # the shadow stage's events also span its co-run with the next closest-hit
    # launch, so stage times cannot pick the dominant kernel
    dom = "trace_closest"
    ms_dom, n_dom = stages[dom]
    launches_frame = n_dom / max(1, args.steps)
    launch_s = ms_dom / max(1, n_dom) * 1e-3
    own = own_bytes[dom] / max(1, launches_frame) / launch_s / 1e9
    ref_walk = ref_bytes[dom] / max(1, launches_frame) / launch_s / 1e9
    hbm = peaks.get("hbm_gbs")
    traffic = TRAFFIC.get((dom, layout))
    roofline = {"bound": "l2", "achieved": round(own, 1), "peak": round(l2_gbs, 1), "unit": "GB/s",
                "frac": round(own / l2_gbs, 4), "traffic": traffic,
                "kernel": KERNELS.get((dom, layout), dom),
                "peak_source": "L2 read bandwidth measured in this run by kgr_measure_read_bandwidth: a 64 MB "
                               "buffer read 50 times with 16-byte L2-cached loads, best of 5, CUDA events",
                "work_unit": f"{layout} layout: {LAYOUT_BYTES[layout][0]} B per node visit, "
                             f"{LAYOUT_BYTES[layout][1]} B per triangle test, visits counted by the kernel",
                "bytes_per_launch": int(own_bytes[dom] / max(1, launches_frame)),
                "launch_ms": round(launch_s * 1e3, 4),
                "hbm": {"peak": hbm, "peak_source": peak_kind, "frac": round(own / hbm, 4) if hbm else None,
                        "dram_traffic_frac_of_algorithmic": round(traffic / (own_bytes[dom] / max(1, launches_frame)), 4)
                        if traffic else None},
                "reference_walk": {"achieved": round(ref_walk, 1), "l2_frac": round(ref_walk / l2_gbs, 4),
                                   "note": "bytes the reference's threaded walk would read for the same rays "
                                           "(48 B per interior record, 80 B per leaf record); it makes about "
                                           "3.5x more visits than this kernel, so this is not a roofline"},
                "visits_per_frame": {"reference": list(visits["threaded"]), layout: list(visits[layout])}}

    quality = quality_terrain = None
    if rank == 0 and not args.no_quality:
        # the radiance-cache comparison on its own configuration (the
        # ReSTIR DI box scene at 1080p), then on the headline workload
        quality = relmse_compare(args, args.quality_scene, *((g, sc) if args.quality_scene == args.scene
                                                              else (None, None)), W, H, stream, sptr)
        if args.quality_scene != args.scene:
            quality_terrain = relmse_compare(args, args.scene, g, sc, W, H, stream, sptr)
    serve = None
    if rank == 0 and not args.no_serve:
        serve = serve_run(args)
    restir = None
    if rank == 0 and not args.no_restir:
        restir = restir_runs(args)
    mamba = None
    if rank == 0 and not args.no_mamba:
        mamba = mamba_run(args, g, sc, W, H)

    cpu_base = None
    if rank == 0 and not args.no_cpu_baseline:
        try:
            from oracle import pyoracle
            osc = pyoracle.Scene(g.positions, g.normals, g.tris4(), g.materials_raw, sc.lights(), sc.bvh())
            run, rows, cores = cpu_sample(osc, kgr.camera_dict(cam), args, args.cpu_seconds)
            dt, crays, r = run(rows)
            cpu_base = {"value": round(crays / dt / 1e6, 4), "unit": "Mrays/s", "cores": cores, "kind": "port",
                        "sample": f"{r} centre rows x {W} px x {args.spp} spp ({dt:.1f} s)"}
        except Exception as exc:  # the baseline is reported, not required
            cpu_base = {"value": None, "unit": "Mrays/s", "cores": os.cpu_count(), "kind": "port",
                        "sample": f"failed: {exc}"}

    if rank == 0:
        stage_ms = {k: round(v[0] / max(1, args.steps), 3) for k, v in stages.items() if v[1]}
        line = {"metric": METRIC, "value": round(value, 2), "unit": "Mrays/s", "n_gpus": ws,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(total_ms / args.steps, 3),
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic (seeded procedural scene, random-free camera)",
                "config": {"workload": WORKLOAD, "scene": args.scene, "triangles": info_s.triangle_count,
                           "lights": info_s.light_count, "resolution": [W, H], "spp": args.spp,
                           "max_depth": args.max_depth, "layout": layout, "trace_tune": att.trace_tune(),
                           "autotune": tuned,
                           "l2_flush": "256 MB buffer written between timed steps",
                           "parallelism": "replicas" if ws > 1 else "1 GPU"},
                "ms_per_frame": round(total_ms / args.steps, 3),
                "rays_per_frame": int(rays / args.steps / max(1, ws)),
                "stage_ms_per_frame": stage_ms,
                "roofline": roofline,
                "equal_relmse": quality,
                "equal_relmse_terrain": quality_terrain,
                "serve": serve,
                "restir": restir,
                "mamba": mamba,
                "cpu_baseline": cpu_base,
                "e2e": {"value": round(e2e_value, 2), "unit": "Mrays/s",
                        "h2d_bytes_per_step": ctypes.sizeof(kgr.LaunchInfo),
                        "d2h_bytes_per_step": W * H * 16,
                        "readback": "pinned host memory, double-buffered: frame s's copy overlaps frame s+1"},
                "gpu_launches": int(launches_per_frame * args.steps),
                "clocks": clk,
                "scene_build_ms": round(info_s.build_ms, 1)}
        print(json.dumps(line))
    att.close()
    sc.close()
    if ws > 1:
        torch.distributed.destroy_process_group()


def main():
    args = parse()
    if args.impl == "reference":
        bench_reference(args)
    else:
        bench_ours(args)


if __name__ == "__main__":
    main()
