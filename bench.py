"""Benchmark: ms per voxel-cone-tracing frame (voxelize + inject + mip +
trace) on the large plain frame: 262,144 triangles, 256^3 RGBA16F grid with
9 levels, 2048^2 shadow map, 1920x1080 G-buffer, 6 diffuse cones (60 deg) +
1 specular cone (10 deg); the cone sampler is the hybrid one (the level of
each trilinear-mip sample with the larger weight in exact fp32, the other
by the texture units), within 1e-3 of the fp64 cone-trace oracle.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--config large|cornell|batch|learned|dynamic]
                  [--filter software|hybrid|levels|hardware]

Our arm: inputs (triangles, shadow map, G-buffer) are resident in HBM; every
timed step is one vct_frame call through the C ABI, timed with CUDA events on
its stream, with a 256 MiB write between steps (outside the events) to flush
the 129 MB L2.  `e2e` repeats the measurement through the same C ABI with the
inputs in pinned host memory: each step copies the triangles, shadow map and
G-buffer to the device, runs the frame and copies the composite image back.

Outside the timed regions the default line also carries: the other cone
sampler's frame time (`samplers`); the oracle's single-threaded frame with
the whole frame traced (`cpu_baseline`); the frame's irradiance per sampler
against the fp64 and fp32 cone-trace oracle over every covered pixel, and
the radiance chain against the oracle's bit for bit (`accuracy`); and compact
runs of the batched family (`batch`) and of the learned path (`learned`).

Reference arm (--impl reference): the reference's path is OpenGL/GLSL, which
cannot run here (no graphics stack), so its CPU restatement (oracle/, the
same code that checks parity) is timed on all host threads; each step
voxelises, normalises, injects and filters the full grid and traces the
whole frame.

With --gpus N (launched by torchrun) every rank runs an independent replica
(the path does not shard a single frame); `value` is the job's effective
ms per frame: the slowest rank's total time over all frames of all ranks.
"""

from __future__ import annotations

import argparse
import json
import os
import platform
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "ms/frame voxelize+inject+mip+trace 256³@1080p"
WORKLOAD = "large plain frame: 262,144 tris, 256^3 RGBA16F x9 levels, 2048^2 shadow map, 1920x1080, 6+1 cones"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="large", choices=["large", "cornell", "batch", "learned", "dynamic"],
                    help="large plain frame (default), the small Cornell box, or the batched family: "
                         "--batch-scenes seeded scenes in one captured graph")
    ap.add_argument("--batch-scenes", type=int, default=32)
    ap.add_argument("--learned-scenes", type=int, default=None,
                    help="learned: held-out scenes timed (8; 2 in the default line's learned block)")
    ap.add_argument("--frames", type=int, default=120, help="dynamic: frames of the actor animation")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default launch shapes")
    ap.add_argument("--filter", default="hybrid", choices=["software", "hybrid", "levels", "hardware"],
                    help="cone sampler: fp32 trilinear (exact); the heavier-weighted level of each sample exact and "
                         "the other by the texture units (the default: within 1e-3 of the fp64 trace); texture "
                         "units per level + fp32 level blend; or texture units' trilinear-mip")
    ap.add_argument("--voxelizer", default="raster", choices=["raster", "tess"],
                    help="rasterising voxeliser (voxelize.geom/.frag, the benchmark frame's) or the "
                         "tessellation voxeliser (testTesselation.tesc/.tese)")
    ap.add_argument("--warp", default="none", choices=["none", "perspective"],
                    help="perspective: the voxelizeTesselationWarp froxel grid over the camera frustum")
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extra-configs", action="store_true",
                    help="large: skip the compact batched and learned blocks after the frame's line")
    ap.add_argument("--cpu-sample-rows", type=int, default=0,
                    help="rows of the frame the CPU oracle traces (0: every row; the batched family: 24)")
    ap.add_argument("--profile-frames", type=int, default=0,
                    help="only run this many frames (no timing, no JSON): the command profiled with ncu")
    return ap.parse_args()


# ------------------------------------------------------------------ dist
def dist_init(n):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if world > 1:
        import torch.distributed as dist

        backend = "nccl" if os.environ.get("VCT_BENCH_BACKEND", "nccl") == "nccl" else "gloo"
        dist.init_process_group(backend)
    return rank, world


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(x: float, world: int) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ---------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi clocks/throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "25"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        sms, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sms.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for name, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sms) if sms else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sms)}


# ------------------------------------------------------------- workloads
def make_scene(args):
    from vct_gb300 import scenes

    return scenes.make(args.config, seed=args.seed)


def algorithmic_bytes(sc, stats, launches_per_frame, sampler="software", fused_single=False):
    """Per-launch algorithmic HBM bytes of each frame kernel (the minimum a
    kernel must move: inputs read once, outputs written once).  The radiance
    chain is written in the layouts the sampler reads: the bordered fp32 copy
    (software, hybrid), the texture array's binary16 copy (hybrid, levels,
    hardware) and the linear binary16 chain.  A single-scene fused frame
    whose sampler reads both copies writes the linear chain only from level
    4 (the mip tail's source) on."""
    N = sc.dim
    nv = N ** 3
    T = sc.ntri
    W, H = sc.gbuffer_size
    P = W * H
    SW, SH = sc.shadow_size
    U = stats["unique_voxels"]
    C = stats.get("covered_pixels", P)
    lv = lambda a, b: sum((N >> l) ** 3 for l in range(a, min(b, sc.levels)))  # noqa: E731
    tex = sampler in ("hybrid", "levels", "hardware")
    pad = sampler in ("hybrid", "software")
    linear_from = 4 if (fused_single and tex and pad) else 0
    per_texel = (8 if tex else 0) + (16 if pad else 0)
    return {
        # triangles in (positions, normals, albedo); the 32-byte record of every occupied voxel read and
        # written once (fragments of one voxel meet in L2); the occupancy mask written once
        "accumulate": T * (36 + 36 + 12) + U * 32 * 2 + nv // 8,
        # shadow map read, lit bit set per texel (bit mask written once)
        "inject_mark": SW * SH * 4 + nv // 8,
        # occupancy and lit masks read; records of occupied voxels read and zeroed; colour and normal
        # level 0 written (RGBA16F); radiance levels 0-4 written in the sampler's copies (interiors of
        # the bordered one) and in the linear chain
        "resolve": nv // 8 * 2 + U * 32 * 2 + nv * 8 * 2 + lv(linear_from, 5) * 8 + lv(0, 5) * per_texel,
        # level 4 read, levels 5.. written (the linear chain and the sampler's copies)
        "mip_tail": (N >> 4) ** 3 * 8 + lv(5, 99) * (8 + per_texel),
        # G-buffer positions read for every pixel, normals and albedo only for covered ones (gp.w != 0),
        # composite float4 written for every pixel
        "trace": P * (16 + 16) + C * 32,
    }


def stage_rooflines(alg: dict, kernel_ms: dict, hbm_gbs: float, traffic: dict, fragments: int,
                    voxelizer: str) -> dict:
    """Every frame stage against the same HBM roofline (stage times from the
    context's timers; the voxelise stage includes the inject marking that
    overlaps it on the side stream), with the voxeliser's fragment (or point)
    rate and its rate of record reductions: four 64-bit adds and one occupancy
    OR per rasterised fragment; four adds per tessellated point, whose
    occupancy bit is set once per voxel."""
    stages = {}
    for k, b in (("accumulate", alg["accumulate"]), ("resolve+mips", alg["resolve"] + alg["mip_tail"]),
                 ("trace", alg["trace"])):
        gbs = b / (kernel_ms[k] * 1e-3) / 1e9
        stages[k] = {"ms": round(kernel_ms[k], 4), "algorithmic_bytes": int(b), "achieved_gbs": round(gbs, 1),
                     "frac": round(gbs / hbm_gbs, 4), "traffic": traffic.get(k)}
    t = kernel_ms["accumulate"] * 1e-3
    per = 4 if voxelizer == "tess" else 5
    stages["accumulate"]["fragments_per_s"] = round(fragments / t, 1)
    stages["accumulate"]["reductions_per_s"] = round(per * fragments / t, 1)
    return stages


SAMPLER_NAMES = ("software", "hybrid", "levels", "hardware")


def sampler_id(name: str) -> int:
    from vct_gb300 import _lib as L

    return {"software": L.VCT_FILTER_SOFTWARE, "hybrid": L.VCT_FILTER_HYBRID, "levels": L.VCT_FILTER_HARDWARE_LEVELS,
            "hardware": L.VCT_FILTER_HARDWARE}[name]


def frame_config(args, sc, world: int) -> dict:
    """The workload of a single-frame line, with the same keys in both arms."""
    headline = args.config == "large" and args.voxelizer == "raster" and args.warp == "none"
    return {"workload": WORKLOAD if headline else f"{args.config} scene, {args.voxelizer} voxeliser, {args.warp} warp",
            "scene": args.config, "voxelizer": args.voxelizer, "warp": args.warp, "seed": args.seed,
            "triangles": sc.ntri, "grid": sc.dim, "levels": sc.levels, "shadow_map": list(sc.shadow_size),
            "gbuffer": list(sc.gbuffer_size), "cones": "6x60deg + 1x10deg", "parallelism": f"replicas x{world}",
            "l2": "256 MiB buffer written between timed frames (outside the events)"}


def run_ours(args, rank, world):
    import torch

    from vct_gb300 import _lib as L
    from vct_gb300 import api

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = f"cuda:{local}"
    sc = make_scene(args)
    W, H = sc.gbuffer_size
    SW, SH = sc.shadow_size
    pos = torch.from_numpy(sc.positions).to(dev)
    nrm = torch.from_numpy(sc.normals).to(dev)
    alb = torch.from_numpy(sc.albedo).to(dev)
    tris = api.triangles(pos, nrm, alb)
    sm = torch.empty(SW * SH, dtype=torch.float32, device=dev)
    api.render_shadowmap(tris, sc, sm)
    keys = torch.empty(W * H, dtype=torch.int64, device=dev)
    gpos, gnrm, galb = (torch.empty(W * H * 4, dtype=torch.float32, device=dev) for _ in range(3))
    api.render_gbuffer(tris, sc, keys, gpos, gnrm, galb)
    del keys
    covered = int((gpos.view(-1, 4)[:, 3] != 0).sum())
    color = torch.empty(W * H * 4, dtype=torch.float32, device=dev)
    lights = api.light_array(sc.lights)
    shadow = api.shadow_desc(sc, sm)
    gb = api.gbuffer(gpos, gnrm, galb, W, H)
    out = api.trace_out(color=color)
    ctx = api.Context(api.config_for(sc, device=local))
    params = api.scene_params(sc)
    params.trace_filter = sampler_id(args.filter)
    params.voxelize_tesselation = int(args.voxelizer == "tess")
    params.warp_mode = L.VCT_WARP_PERSPECTIVE if args.warp == "perspective" else L.VCT_WARP_NONE
    ctx.set_params(params)
    stream = torch.cuda.current_stream()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    lib = L.load()

    def frame():
        ctx.frame(tris, lights, shadow, sc.eye, gb, out, stream)

    if args.profile_frames:
        for _ in range(args.profile_frames):
            frame()
        torch.cuda.synchronize()
        ctx.close()
        return None, sc, None

    for _ in range(max(3, args.warmup)):
        frame()
    torch.cuda.synchronize()
    # launch shapes from the library's autotuner (vct_autotune times each candidate over a few
    # frames; every shape gives bit-identical results), outside the timed region
    tune_s = 0.0
    if not args.no_autotune:
        t0 = time.perf_counter()
        ctx.autotune(tris, lights, shadow, sc.eye, gb, out, reps=5, stream=stream)
        tune_s = time.perf_counter() - t0
        for _ in range(max(3, args.warmup)):
            frame()
        torch.cuda.synchronize()
    tuning = api.tuning_dict(ctx.tuning())
    stats = ctx.stats()
    stats["covered_pixels"] = covered
    # samples per frame (counted once, outside the timed region)
    samples = torch.zeros(1, dtype=torch.int64, device=dev)
    ctx.frame(tris, lights, shadow, sc.eye, gb, api.trace_out(color=color, samples=samples), stream)
    torch.cuda.synchronize()
    n_samples = int(samples.item())

    def timed_frames(steps, clk_sampler=None):
        """`steps` frames, each between CUDA events on the launching stream,
        the L2 flushed before each (outside the events); per-stage timers."""
        ctx.enable_timers(True)
        starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
        ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
        stage = {k: 0.0 for k in ("voxelize_ms", "radiance_ms", "mipmap_ms", "render_ms", "total_ms")}
        for i in range(steps):
            flush.fill_(float(i))
            starts[i].record(stream)
            frame()
            ends[i].record(stream)
            for k, v in ctx.timers().items():  # waits for this frame's end event
                stage[k] += v
        torch.cuda.synchronize()
        ctx.enable_timers(False)
        return [s.elapsed_time(e) for s, e in zip(starts, ends)], {k: v / steps for k, v in stage.items()}

    # ---- timed region: K frames, per-frame events, L2 flushed between frames
    barrier(world)
    torch.cuda.synchronize()
    launches0 = lib.vct_launch_count()
    t_wall = time.perf_counter()
    with ClockSampler(local) as clk:
        frame_ms, stage = timed_frames(args.steps)
    barrier(world)
    wall_s = time.perf_counter() - t_wall
    launches = lib.vct_launch_count() - launches0
    total_ms = sum(frame_ms)
    total_ms_max = max_over_ranks(total_ms, world)
    ms_per_frame = total_ms_max / (args.steps * world)

    # ---- e2e through the C ABI with host buffers (pinned), copies timed
    h_pos, h_nrm, h_alb = (t.cpu().pin_memory() for t in (pos, nrm, alb))
    h_sm = sm.cpu().pin_memory()
    h_gpos, h_gnrm, h_galb = (t.cpu().pin_memory() for t in (gpos, gnrm, galb))
    h_color = torch.empty(W * H * 4, dtype=torch.float32).pin_memory()
    d_pos, d_nrm, d_alb, d_sm = (torch.empty_like(t, device=dev) for t in (h_pos, h_nrm, h_alb, h_sm))
    d_gpos, d_gnrm, d_galb = (torch.empty_like(t, device=dev) for t in (h_gpos, h_gnrm, h_galb))
    e_tris = api.triangles(d_pos, d_nrm, d_alb)
    e_shadow = api.shadow_desc(sc, d_sm)
    h2d = sum(t.numel() * t.element_size() for t in (h_pos, h_nrm, h_alb, h_sm, h_gpos, h_gnrm, h_galb))
    d2h = h_color.numel() * 4

    # Steps through the public API with frames in flight, as a renderer streams them: every step
    # uploads its triangles, shadow map and G-buffer from pinned host memory and reads its image
    # back, and those copies run on two copy streams beside the frames.  Step k+1's triangles and
    # shadow map go up once step k's volume pass has consumed them (during step k's trace), its
    # G-buffer into the other of two device buffers, and step k's image comes back while step
    # k+1's volume pass runs.  The K steps are timed as one region; each step moves 138 MB in and
    # 33 MB out and touches over 1 GB of HBM (more than L2), so no flush runs between them.
    up = torch.cuda.Stream(device=dev)
    down = torch.cuda.Stream(device=dev)
    d_gb = [(d_gpos, d_gnrm, d_galb)] + [tuple(torch.empty_like(t) for t in (d_gpos, d_gnrm, d_galb))]
    d_col = [color, torch.empty_like(color)]
    plans = [(api.gbuffer(*d_gb[par], W, H), api.trace_out(color=d_col[par])) for par in range(2)]
    ev_tri, ev_vol = torch.cuda.Event(), torch.cuda.Event()
    ev_gb = [torch.cuda.Event(), torch.cuda.Event()]
    ev_done = [torch.cuda.Event(), torch.cuda.Event()]
    ev_d2h = [torch.cuda.Event(), torch.cuda.Event()]

    def e2e_step(k):
        par = k & 1
        up.wait_event(ev_vol)  # the previous step's volume pass has read the triangles and shadow map
        with torch.cuda.stream(up):
            for d, h in ((d_pos, h_pos), (d_nrm, h_nrm), (d_alb, h_alb), (d_sm, h_sm)):
                d.copy_(h, non_blocking=True)
            ev_tri.record(up)
            up.wait_event(ev_done[par])  # the trace of two steps ago is done with this G-buffer
            for d, h in zip(d_gb[par], (h_gpos, h_gnrm, h_galb)):
                d.copy_(h, non_blocking=True)
            ev_gb[par].record(up)
        stream.wait_event(ev_tri)
        ctx.frame_volume(e_tris, lights, e_shadow, sc.eye, stream)
        ev_vol.record(stream)
        stream.wait_event(ev_gb[par])
        stream.wait_event(ev_d2h[par])  # the image of two steps ago has been read back
        g, o = plans[par]
        ctx.trace(g, sc.eye, o, stream)
        ev_done[par].record(stream)
        down.wait_event(ev_done[par])
        with torch.cuda.stream(down):
            h_color.copy_(d_col[par], non_blocking=True)
            ev_d2h[par].record(down)

    for k in range(max(3, args.warmup)):
        e2e_step(k)
    torch.cuda.synchronize()
    barrier(world)
    e_start, e_end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e_start.record(stream)
    for k in range(args.steps):
        e2e_step(k)
    stream.wait_stream(up)
    stream.wait_stream(down)
    e_end.record(stream)
    torch.cuda.synchronize()
    e2e_total = max_over_ranks(e_start.elapsed_time(e_end), world)
    e2e_ms = e2e_total / (args.steps * world)
    assert torch.isfinite(h_color).all(), "non-finite output"
    # the split, overlapped path gives the image of one vct_frame, bit for bit
    check = torch.empty_like(color)
    ctx.frame(tris, lights, shadow, sc.eye, gb, api.trace_out(color=check), stream)
    torch.cuda.synchronize()
    assert torch.equal(check.cpu().view(torch.int32), h_color.view(torch.int32)), "e2e image differs from vct_frame"
    del d_gb, d_col, plans, check

    # ---- outside the timed regions: the other samplers' frame times (same launch shapes), and
    # this frame's irradiance per sampler and radiance chain for the oracle's checks on rank 0
    others = [n for n in ("software", "hybrid") if n != args.filter]
    samplers = {args.filter: {"frame_ms": round(statistics.median(frame_ms), 4),
                              "trace_ms": round(stage["render_ms"], 4), "resolve_mips_ms": round(stage["mipmap_ms"], 4)}}
    irr_dev = torch.empty(W * H * 4, dtype=torch.float32, device=dev)
    art = {"irr": {}} if rank == 0 else None
    for name in [args.filter] + others:
        params.trace_filter = sampler_id(name)
        ctx.set_params(params)
        if name != args.filter:
            for _ in range(3):
                frame()
            fm, st = timed_frames(args.steps)
            samplers[name] = {"frame_ms": round(statistics.median(fm), 4), "trace_ms": round(st["render_ms"], 4),
                              "resolve_mips_ms": round(st["mipmap_ms"], 4)}
        if art is not None:
            ctx.frame(tris, lights, shadow, sc.eye, gb, api.trace_out(irradiance=irr_dev, color=color), stream)
            torch.cuda.synchronize()
            art["irr"][name] = irr_dev.cpu().numpy()
    params.trace_filter = sampler_id(args.filter)
    ctx.set_params(params)
    if art is not None:
        art["chain"] = np.concatenate([ctx.read_volume(L.VCT_VOLUME_RADIANCE, lv).cpu().numpy().view(np.uint16)
                                       for lv in range(sc.levels)])
        art["sm"] = sm.cpu().numpy()
        art["gbuf"] = tuple(t.cpu().numpy() for t in (gpos, gnrm, galb))
        art["stats"] = dict(stats)

    # ---- roofline of the dominant kernel
    alg = algorithmic_bytes(sc, stats, None, sampler=args.filter, fused_single=params.temporal_filter == 0)
    kernel_ms = {"accumulate": stage["voxelize_ms"], "inject_mark": stage["radiance_ms"],
                 "resolve+mips": stage["mipmap_ms"], "trace": stage["render_ms"]}
    dom = max(kernel_ms, key=kernel_ms.get)
    peaks = load_peaks()
    if dom == "resolve+mips":
        bytes_dom = alg["resolve"] + alg["mip_tail"]
    else:
        bytes_dom = alg[dom]
    achieved = bytes_dom / (kernel_ms[dom] * 1e-3) / 1e9
    headline = args.config == "large" and args.voxelizer == "raster" and args.warp == "none" and \
        args.filter == NCU_CAPTURE_SAMPLER
    traffic, traffic_note = ncu_traffic(headline)
    roofline = {"kernel": dom, "bound": "hbm", "achieved": round(achieved, 1), "peak": peaks["hbm_gbs"],
                "unit": "GB/s", "frac": round(achieved / peaks["hbm_gbs"], 4), "traffic": traffic.get(dom),
                **traffic_note, "peak_source": peaks["source"], "algorithmic_bytes": int(bytes_dom),
                "kernel_ms": round(kernel_ms[dom], 4)}
    if dom == "accumulate" and args.voxelizer == "tess":
        roofline["points_per_s"] = round(stats["total_voxel_fragments"] / (kernel_ms[dom] * 1e-3), 1)
        roofline["note"] = ("the tessellation voxeliser is bound by its point rate (every point interpolated, "
                            "mapped and summed into its voxel), not by HBM")
    if dom == "trace":
        roofline["samples_per_s"] = round(n_samples / (kernel_ms[dom] * 1e-3), 1)
        # the tracer's own ceiling: the sampler's peak rate with L1-resident texels (vct_sampler_rate)
        peak_rate = ctx.sampler_rate(params.trace_filter, 1 << 31, stream)
        roofline["sampler_peak_samples_per_s"] = round(peak_rate, 1)
        roofline["sampler_frac"] = round(n_samples / (kernel_ms[dom] * 1e-3) / peak_rate, 4)
        if traffic:
            roofline["issue"] = dict(NCU_TRACE_ISSUE, source="ncu capture of this workload")
        roofline["note"] = ("cone tracing is gather-bound, not HBM-bound: its HBM fraction counts only G-buffer "
                            "reads and the image write; its ceiling is the sampler's own peak rate "
                            "(sampler_peak_samples_per_s, vct_sampler_rate)")

    roofline["stages"] = stage_rooflines(alg, kernel_ms, peaks["hbm_gbs"], traffic,
                                         stats["total_voxel_fragments"], args.voxelizer)

    config = frame_config(args, sc, world)
    result = {
        "metric": METRIC, "value": round(ms_per_frame, 4), "unit": "ms/frame", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_per_frame * world, 4),
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f32 math, f16 volumes, u32 accumulators",
        "data": "synthetic seeded scene (no dataset); inputs resident in HBM",
        "config": config,
        "sampler": args.filter,
        "tuning": tuning, "autotuned": not args.no_autotune, "autotune_s": round(tune_s, 2),
        "stage_ms": {k: round(v, 4) for k, v in stage.items()},
        "frame_ms_min": round(min(frame_ms), 4), "frame_ms_median": round(statistics.median(frame_ms), 4),
        "wall_s": round(wall_s, 3),
        "samplers": samplers,
        "e2e": {"value": round(e2e_ms, 4), "unit": "ms/frame", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h),
                "path": "vct_frame_volume + vct_trace per step, frames in flight: the next step's uploads run "
                        "during this step's trace (G-buffer and image double-buffered), this step's image comes "
                        "back during the next volume pass; K steps timed as one region",
                "l2": "no flush: steps overlap, each moves 138 MB in and 33 MB out and touches over 1 GB of HBM"},
        "gpu_launches": int(launches),
        "roofline": roofline,
        "clocks": clk.summary(),
        "voxelize_stats": stats,
        "samples_per_frame": n_samples,
    }
    ctx.close()
    return result, sc, art


# ------------------------------------------------------------- batched
BATCH_METRIC = "ms per batch of 32 scenes voxelize+inject+mip+trace (one captured graph)"


def run_batch(args, rank, world, compact=False):
    """Batched family: --batch-scenes seeded scenes (triangles log-uniform in
    1k-200k, grids from {64,128,256}^3, G-buffers 320x180..1920x1080, 1-4
    lights) run as one vct_batch frame per step, replayed from a captured
    CUDA graph, with the launch shapes picked by the library's autotuner.
    Compared with the same scenes run as sequential vct_frame calls.  With
    `compact`, only the graph replays and the sequential frames are timed
    and a short summary is returned."""
    import torch

    from vct_gb300 import _lib as L
    from vct_gb300 import api, scenes

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = f"cuda:{local}"
    t0 = time.perf_counter()
    scs = [scenes.batch_scene(seed=args.seed + 1000 * rank, index=i) for i in range(args.batch_scenes)]
    gen_s = time.perf_counter() - t0
    filt = {"software": L.VCT_FILTER_SOFTWARE, "hybrid": L.VCT_FILTER_HYBRID, "levels": L.VCT_FILTER_HARDWARE_LEVELS,
            "hardware": L.VCT_FILTER_HARDWARE}[args.filter]
    inputs, descs, colors = [], [], []
    for sc in scs:
        W, H = sc.gbuffer_size
        SW, SH = sc.shadow_size
        pos, nrm, alb = (torch.from_numpy(a).to(dev) for a in (sc.positions, sc.normals, sc.albedo))
        tris = api.triangles(pos, nrm, alb)
        sm = torch.empty(SW * SH, dtype=torch.float32, device=dev)
        api.render_shadowmap(tris, sc, sm)
        keys = torch.empty(W * H, dtype=torch.int64, device=dev)
        gpos, gnrm, galb = (torch.empty(W * H * 4, dtype=torch.float32, device=dev) for _ in range(3))
        api.render_gbuffer(tris, sc, keys, gpos, gnrm, galb)
        del keys
        color = torch.empty(W * H * 4, dtype=torch.float32, device=dev)
        lights = api.light_array(sc.lights)
        inputs.append(dict(pos=pos, nrm=nrm, alb=alb, sm=sm, gpos=gpos, gnrm=gnrm, galb=galb, lights=lights))
        descs.append(api.scene_desc(tris, lights, api.shadow_desc(sc, sm), sc.eye,
                                    api.gbuffer(gpos, gnrm, galb, W, H), api.trace_out(color=color)))
        colors.append(color)
    b = api.Batch([api.config_for(sc, device=local) for sc in scs])
    for i, sc in enumerate(scs):
        b.set_params(api.scene_params(sc, trace_filter=filt), i)
    stream = torch.cuda.Stream()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    lib = L.load()
    torch.cuda.synchronize()
    b.frame(descs, stream)
    stream.synchronize()
    t0 = time.perf_counter()
    tuning = b.tuning() if args.no_autotune else b.autotune(descs, reps=3, stream=stream)
    tune_s = time.perf_counter() - t0

    def timed(step_fn, steps):
        st = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
        en = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
        for i in range(steps):
            with torch.cuda.stream(stream):
                flush.fill_(float(i))
            st[i].record(stream)
            step_fn()
            en[i].record(stream)
        stream.synchronize()
        return [a.elapsed_time(e) for a, e in zip(st, en)]

    # per-stage times of a direct (non-graph) batched frame
    b.enable_timers(True)
    stage = {k: 0.0 for k in ("voxelize_ms", "mipmap_ms", "render_ms", "total_ms")}
    for i in range(max(3, args.warmup) + args.steps):
        b.frame(descs, stream)
        t = b.timers()
        if i >= max(3, args.warmup):
            for k in stage:
                stage[k] += t[k] / args.steps
    b.enable_timers(False)
    direct_ms = timed(lambda: b.frame(descs, stream), args.steps)

    # the headline: graph replays
    b.capture(descs, stream)
    for _ in range(max(3, args.warmup)):
        b.replay(stream)
    stream.synchronize()
    barrier(world)
    launches0 = lib.vct_launch_count()
    with ClockSampler(local) as clk:
        graph_ms = timed(lambda: b.replay(stream), args.steps)
    launches = lib.vct_launch_count() - launches0
    total = max_over_ranks(sum(graph_ms), world)
    value = total / (args.steps * world)

    # sequential single-scene frames on the same contexts (default shapes, then the tuned ones)
    def sequential():
        for ctx, d in zip(b.scenes, descs):
            ctx.frame(d.triangles, (d.lights, d.n_lights), d.shadow, list(d.eye), d.gbuffer, d.out, stream)

    for _ in range(2):
        sequential()
    seq_default_ms = timed(sequential, args.steps)
    for ctx in b.scenes:
        ctx.set_tuning(tuning)
    seq_tuned_ms = timed(sequential, args.steps)
    if compact:
        b.close()
        return {"workload": f"{args.batch_scenes} seeded scenes of the batched family (seed {args.seed}): "
                            f"{sum(sc.ntri for sc in scs)} tris, grids {{64,128,256}}^3, "
                            f"{sum(sc.gbuffer_size[0] * sc.gbuffer_size[1] for sc in scs)} pixels",
                "graph_replay_ms": round(value, 4), "sequential_ms": round(statistics.median(seq_default_ms), 4),
                "sequential_tuned_ms": round(statistics.median(seq_tuned_ms), 4),
                "speedup_vs_sequential": round(statistics.median(seq_default_ms) / value, 3),
                "scenes_per_s": round(args.batch_scenes * 1e3 / value, 1), "launches_per_replay":
                    int(launches // max(1, args.steps)), "stage_ms": {k: round(v, 4) for k, v in stage.items()},
                "tuning": api.tuning_dict(tuning), "steps": args.steps,
                "l2": "256 MiB buffer written between timed steps (outside the events)"}, scs

    # e2e with batches in flight: every step copies all scenes' inputs from pinned host memory,
    # replays a captured batch graph and copies the images back.  Two batch objects (each with its
    # own contexts and graph) over two sets of device buffers alternate, so that one step's uploads
    # run on a copy stream while the previous step's graph replays, and its images come back while
    # the next one replays.  The K steps are timed as one region; each step moves 1.9 GB across the
    # host link, more than L2, so no flush runs between them.
    host = [{k: v.cpu().pin_memory() for k, v in d.items() if k != "lights"} for d in inputs]
    h_colors = [torch.empty(c.numel(), dtype=torch.float32).pin_memory() for c in colors]
    h2d = sum(t.numel() * t.element_size() for h in host for t in h.values())
    d2h = sum(c.numel() * 4 for c in colors)
    inputs2 = [dict({k: torch.empty_like(v) for k, v in d.items() if k != "lights"}, lights=d["lights"])
               for d in inputs]
    colors2 = [torch.empty_like(c) for c in colors]
    descs2 = []
    for sc, d, c in zip(scs, inputs2, colors2):
        W, H = sc.gbuffer_size
        descs2.append(api.scene_desc(api.triangles(d["pos"], d["nrm"], d["alb"]), d["lights"],
                                     api.shadow_desc(sc, d["sm"]), sc.eye,
                                     api.gbuffer(d["gpos"], d["gnrm"], d["galb"], W, H), api.trace_out(color=c)))
    b2 = api.Batch([api.config_for(sc, device=local) for sc in scs])
    for i, sc in enumerate(scs):
        b2.set_params(api.scene_params(sc, trace_filter=filt), i)
    b2.set_tuning(tuning)
    for d, h in zip(inputs2, host):
        for k, t in h.items():
            d[k].copy_(t)
    torch.cuda.synchronize()
    b2.frame(descs2, stream)
    b2.capture(descs2, stream)
    sets = [(b, inputs, colors), (b2, inputs2, colors2)]
    up, down = torch.cuda.Stream(device=dev), torch.cuda.Stream(device=dev)
    ev_up = [torch.cuda.Event(), torch.cuda.Event()]
    ev_done = [torch.cuda.Event(), torch.cuda.Event()]
    ev_d2h = [torch.cuda.Event(), torch.cuda.Event()]

    def e2e_step(k):
        par = k & 1
        bb, ins, cols = sets[par]
        with torch.cuda.stream(up):
            up.wait_event(ev_done[par])  # the replay of two steps ago has read these inputs
            for d, h in zip(ins, host):
                for name, t in h.items():
                    d[name].copy_(t, non_blocking=True)
            ev_up[par].record(up)
        stream.wait_event(ev_up[par])
        stream.wait_event(ev_d2h[par])  # the images of two steps ago have been read back
        bb.replay(stream)
        ev_done[par].record(stream)
        with torch.cuda.stream(down):
            down.wait_event(ev_done[par])
            for hc, c in zip(h_colors, cols):
                hc.copy_(c, non_blocking=True)
            ev_d2h[par].record(down)

    for k in range(max(3, args.warmup)):
        e2e_step(k)
    torch.cuda.synchronize()
    barrier(world)
    e_start, e_end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e_start.record(stream)
    for k in range(args.steps):
        e2e_step(k)
    stream.wait_stream(up)
    stream.wait_stream(down)
    e_end.record(stream)
    torch.cuda.synchronize()
    e2e_total = max_over_ranks(e_start.elapsed_time(e_end), world)
    e2e_ms = e2e_total / (args.steps * world)
    # both pipelines give the images of the direct batched frame, bit for bit
    ref_cols = [torch.empty_like(c) for c in colors]
    b.frame([api.scene_desc(d.triangles, (d.lights, d.n_lights), d.shadow, list(d.eye), d.gbuffer,
                            api.trace_out(color=r)) for d, r in zip(descs, ref_cols)], stream)
    stream.synchronize()
    for hc, r in zip(h_colors, ref_cols):
        assert torch.equal(hc.view(torch.int32), r.cpu().view(torch.int32)), "e2e batch image differs"
    b2.close()
    assert all(torch.isfinite(h).all() for h in h_colors), "non-finite output"

    # roofline of the dominant stage: algorithmic bytes summed over scenes
    stats = [ctx.stats(stream) for ctx in b.scenes]
    alg = [algorithmic_bytes(sc, st, None, sampler=args.filter) for sc, st in zip(scs, stats)]
    sums = {k: sum(a[k] for a in alg) for k in alg[0]}
    stage_bytes = {"voxelize_ms": sums["accumulate"],
                   "mipmap_ms": sums["inject_mark"] + sums["resolve"] + sums["mip_tail"],
                   "render_ms": sums["trace"]}
    dom = max(stage_bytes, key=lambda k: stage[k])
    peaks = load_peaks()
    achieved = stage_bytes[dom] / (stage[dom] * 1e-3) / 1e9
    names = {"voxelize_ms": "accumulate (voxelize setup+scan+raster)", "mipmap_ms": "inject_mark+resolve+mip_tail",
             "render_ms": "trace"}
    result = {
        "metric": BATCH_METRIC.replace("32", str(args.batch_scenes)), "value": round(value, 4), "unit": "ms/batch",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(value * world, 4),
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 math, f16 volumes, u32 accumulators", "data": "synthetic seeded scenes (no dataset)",
        "config": {"workload": f"batched family: {args.batch_scenes} scenes, triangles log-uniform 1k-200k, grids "
                               "{64,128,256}^3, G-buffers 320x180..1920x1080, 1-4 lights, 6+1 cones",
                   "seed": args.seed, "scenes": args.batch_scenes, "triangles": int(sum(sc.ntri for sc in scs)),
                   "voxels": int(sum(sc.dim ** 3 for sc in scs)),
                   "pixels": int(sum(sc.gbuffer_size[0] * sc.gbuffer_size[1] for sc in scs)),
                   "sampler": args.filter, "parallelism": f"replicas x{world}",
                   "l2": "256 MiB buffer written between timed steps (outside the events)",
                   "tuning": api.tuning_dict(tuning), "autotune_s": round(tune_s, 2)},
        "scenes_per_s": round(args.batch_scenes * 1e3 / value, 1),
        "direct_batch_ms": round(statistics.median(direct_ms), 4),
        "sequential_ms": {"default_shapes": round(statistics.median(seq_default_ms), 4),
                          "tuned_shapes": round(statistics.median(seq_tuned_ms), 4)},
        "speedup_vs_sequential": round(statistics.median(seq_default_ms) / value, 3),
        "stage_ms": {k: round(v, 4) for k, v in stage.items()},
        "e2e": {"value": round(e2e_ms, 4), "unit": "ms/batch", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h),
                "path": "graph replays of two batch objects over two buffer sets, batches in flight: a step's "
                        "uploads run during the previous replay, its images come back during the next; K steps "
                        "timed as one region",
                "l2": "no flush: steps overlap, each moves 1.9 GB across the host link"},
        "gpu_launches": int(launches),
        "roofline": {"kernel": names[dom], "bound": "hbm", "achieved": round(achieved, 1), "peak": peaks["hbm_gbs"],
                     "unit": "GB/s", "frac": round(achieved / peaks["hbm_gbs"], 4), "traffic": None,
                     "peak_source": peaks["source"], "algorithmic_bytes": int(stage_bytes[dom]),
                     "kernel_ms": round(stage[dom], 4)},
        "clocks": clk.summary(),
        "scene_list": [[sc.ntri, sc.dim, list(sc.gbuffer_size), len(sc.lights)] for sc in scs],
        "scene_gen_s": round(gen_s, 2),
    }
    b.close()
    return result, scs


# ------------------------------------------------------------- learned
LEARNED_METRIC = "ms per 1080p irradiance image: learned 2-cone+MLP vs plain 16-cone trace at matched RMSE"
# per-tile bounds (relative error of the network at 4 probe pixels of a 16x16 tile) and per-pixel bounds
# (the network's error estimate over the frame's RMS irradiance)
LEARNED_TILE_THRESHOLDS = (0.02, 0.03, 0.04, 0.06, 0.1)
LEARNED_PIXEL_THRESHOLDS = (0.015, 0.02, 0.03, 0.05, 0.1, 0.2, 0.5)


def pareto_front(points: list[dict]) -> list[dict]:
    """The operating points no other point beats on both time and error,
    fastest first."""
    front = []
    for p in sorted(points, key=lambda r: (r["ms"], r["rel_l2"])):
        if not front or p["rel_l2"] < front[-1]["rel_l2"]:
            front.append(p)
    return front


def run_learned(args, rank, world, compact=False):
    """Learned configuration on held-out scenes of the large frame's family
    (256^3, 1920x1080): the plain 16-cone irradiance trace against the
    learned trace (cheap quarter-resolution features + the trained network
    on every pixel) with no fallback, with the per-tile fallback (16-cone
    probes at 4 pixels per 16x16 tile, the tiles above a bound re-traced) and
    with the per-pixel fallback (the pixels whose error estimate, the
    network's fourth output, exceeds a bound re-traced), over a sweep of
    bounds.  The headline is the fastest operating point whose mean relative
    L2 error stays <= 2% ("matched RMSE"); the Pareto front of time against
    error is reported beside it."""
    import torch

    from vct_gb300 import _lib as L
    from vct_gb300 import api, learned, scenes

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    params = learned.load_params()
    if params is None:
        if compact:
            return {"unavailable": "no trained weights of this network in vct_gb300/weights"}
        raise SystemExit("no trained weights: run python -m vct_gb300.learned train first")
    W, H, dim = 1920, 1080, 256
    kw = dict(dim=dim, shadow=2048, gbuffer=(W, H))
    state = learned.FrameState(dim, (W, H), 2048, device=local)
    mlp = api.Mlp(device=local)
    mlp.set_params(params)
    stream = torch.cuda.current_stream()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=state.dev)
    lib = L.load()
    n_scenes = args.learned_scenes or (2 if compact else 8)
    seeds = [10_000_000 + 1000 * rank + i for i in range(n_scenes)]
    reps = max(1, args.steps)

    def timed(fn):
        for _ in range(max(3, args.warmup)):
            fn()
        ts = []
        for i in range(reps):
            flush.fill_(float(i))
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            b.record(stream)
            b.synchronize()
            ts.append(a.elapsed_time(b))
        return statistics.median(ts)

    modes = [("network", None)] + [("tile", t) for t in LEARNED_TILE_THRESHOLDS] + \
        [("pixel", t) for t in LEARNED_PIXEL_THRESHOLDS]

    def run(mode, t, want=False):
        if mode == "network":
            api.learned_trace(state.ctx, mlp, state.gb, state.sc.eye, state.out, float("inf"))
            return 0.0
        if mode == "tile":
            st = api.learned_trace(state.ctx, mlp, state.gb, state.sc.eye, state.out, t, want_stats=want)
            return st["fallback_tiles"] / st["tiles"] if want else None
        n = api.learned_trace_pixels(state.ctx, mlp, state.gb, state.sc.eye, state.out, t, want_count=want)
        return n / ncov if want else None

    plain_ms, feat_ms = [], []
    rec = {m: {"ms": [], "err": [], "fb": []} for m in modes}
    launches0 = lib.vct_launch_count()
    with ClockSampler(local) as clk:
        for seed in seeds:
            sc = scenes.large_family(seed, **kw)
            state.load(sc)
            plain_ms.append(timed(lambda: state.reference()))
            truth = state.ref.view(-1, 4)[:, :3].clone()
            mask = state.covered()
            ncov = max(1, int(mask.sum()))
            feat_ms.append(timed(lambda: state.features()))
            for m in modes:
                rec[m]["ms"].append(timed(lambda: run(*m)))
                rec[m]["fb"].append(run(*m, want=True))
                rec[m]["err"].append(learned.rel_l2(state.out.view(-1, 4)[:, :3], truth, mask))
    launches = lib.vct_launch_count() - launches0
    mean = lambda v: float(np.mean(v))  # noqa: E731
    sweep = [{"mode": m[0], "threshold": m[1], "ms": round(mean(rec[m]["ms"]), 4),
              "rel_l2": round(mean(rec[m]["err"]), 5), "rel_l2_max": round(float(np.max(rec[m]["err"])), 5),
              "fallback_fraction": round(mean(rec[m]["fb"]), 4),
              "fallback_of": {"network": "-", "tile": "tiles", "pixel": "covered pixels"}[m[0]]} for m in modes]
    plain = mean(plain_ms)
    for r in sweep:
        r["speedup_vs_plain16"] = round(plain / r["ms"], 3)
    ok = [r for r in sweep if r["rel_l2"] <= 0.02]
    matched = min(ok, key=lambda r: r["ms"]) if ok else None
    net_only = sweep[0]
    front = [{k: r[k] for k in ("mode", "threshold", "ms", "rel_l2", "speedup_vs_plain16")} for r in pareto_front(sweep)]
    summary = {"plain16_ms": round(plain, 4), "network_only_ms": net_only["ms"],
               "network_only_rel_l2": net_only["rel_l2"], "features_ms": round(mean(feat_ms), 4),
               "matched": ({k: matched[k] for k in ("mode", "threshold", "ms", "rel_l2", "fallback_fraction",
                                                     "speedup_vs_plain16")} if matched else None),
               "bar": "mean rel-L2 <= 0.02 against the 16-cone trace, fastest point meeting it",
               "target": "learned >= 3x faster than plain 16-cone at <= 2% (not met: see pareto)",
               "pareto": front}
    if compact:
        return dict({"workload": f"{len(seeds)} held-out scenes of the large frame's family, 256^3, {W}x{H}",
                     "steps": reps}, **summary)
    # e2e: G-buffer planes from pinned host memory, learned trace at the matched point, irradiance back
    h = [t.cpu().pin_memory() for t in (state.gpos, state.gnrm, state.galb)]
    h_out = torch.empty_like(state.out, device="cpu").pin_memory()
    head = matched or net_only

    def e2e():
        for d, src in zip((state.gpos, state.gnrm, state.galb), h):
            d.copy_(src, non_blocking=True)
        run(head["mode"], head["threshold"])
        h_out.copy_(state.out, non_blocking=True)

    e2e_ms = timed(e2e)
    net_ms = net_only["ms"] - mean(feat_ms)
    flops = 2.0 * (48 * 64 + 64 * 64 * 2 + 64 * 16) * W * H  # tensor-core work of the network (padded shapes)
    peaks = load_peaks()
    tflops = flops / (net_ms * 1e-3) / 1e12 if net_ms > 0 else None
    return dict({
        "metric": LEARNED_METRIC, "value": round(head["ms"], 4), "unit": "ms/frame", "n_gpus": world,
        "steps": reps, "warmup": max(3, args.warmup), "ms_per_step": round(head["ms"], 4),
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "bf16 network (fp32 accumulate), f32 cone math, f16 volumes",
        "data": "synthetic seeded held-out scenes of the large frame's family (no dataset)",
        "config": {"workload": "learned: 256^3, 1920x1080, quarter-res 2x90deg cones + MLP 42-64-64-64-4 vs 16 cones",
                   "scenes": len(seeds), "l2": "256 MiB buffer written between timed runs (outside the events)",
                   "weights": "vct_gb300/weights/learned_mlp.f32 (trained by python -m vct_gb300.learned train)"},
        "sweep": sweep,
        "e2e": {"value": round(e2e_ms, 4), "unit": "ms/frame", "h2d_bytes_per_step": int(sum(t.numel() * 4 for t in h)),
                "d2h_bytes_per_step": int(h_out.numel() * 4)},
        "gpu_launches": int(launches),
        "roofline": {"kernel": "mlp_infer_kernel (fused features gather + 4 tcgen05 layers)", "bound": "tensor",
                     "achieved": round(tflops, 1) if tflops else None, "peak": peaks["bf16_tflops"],
                     "unit": "TFLOP/s", "frac": round(tflops / peaks["bf16_tflops"], 4) if tflops else None,
                     "traffic": None, "peak_source": peaks["source"], "flops_per_frame": flops,
                     "kernel_ms": round(net_ms, 4), "note": "network time = learned (no fallback) - features"},
        "clocks": clk.summary(),
    }, **summary)


# ------------------------------------------------------------- dynamic
DYNAMIC_METRIC = ("ms per dynamic frame: 64 rigid actors + 199k-triangle environment re-voxelised into 256^3 with "
                  "the warp map and the temporal filter, traced from 8 viewpoints at 1280x720")


def run_dynamic(args, rank, world):
    """Dynamic warped frames: every frame moves 64 rigid actors (2k-8k
    triangles each) with vct_transform_actors, re-voxelises the 520k
    triangles into the 256^3 grid through the 32^3 warp map with the
    temporal radiance filter, and traces 8 viewpoints at 1280x720 with the
    plain 6+1 cones and with the learned form (network only).  Timed per
    frame with CUDA events: actor transform + vct_frame of viewpoint 0 +
    viewpoints 1-7 in one vct_trace_views launch (plain); the 8 learned
    traces (learned).
    The shadow map and the 8 G-buffers of each frame are set-up passes,
    rendered outside the timed regions."""
    import torch

    from vct_gb300 import _lib as L
    from vct_gb300 import api, learned, scenes

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = f"cuda:{local}"
    sc, actors = scenes.dynamic_scene(seed=args.seed + rank)
    views = [scenes.viewpoint(sc, k) for k in range(8)]
    W, H = sc.gbuffer_size
    SW, SH = sc.shadow_size
    pos0, nrm0, alb = (torch.from_numpy(a).to(dev) for a in (sc.positions, sc.normals, sc.albedo))
    local_tris = api.triangles(pos0, nrm0, alb)
    pos, nrm = pos0.clone(), nrm0.clone()
    tris = api.triangles(pos, nrm, alb)
    sm = torch.empty(SW * SH, dtype=torch.float32, device=dev)
    keys = torch.empty(W * H, dtype=torch.int64, device=dev)
    gbs = []
    for _ in views:
        g = [torch.empty(W * H * 4, dtype=torch.float32, device=dev) for _ in range(3)]
        gbs.append((g, api.gbuffer(g[0], g[1], g[2], W, H)))
    color = torch.empty(W * H * 4, dtype=torch.float32, device=dev)
    view_colors = [torch.empty(W * H * 4, dtype=torch.float32, device=dev) for _ in views[1:]]
    irr = torch.empty(W * H * 4, dtype=torch.float32, device=dev)
    ctx = api.Context(api.config_for(sc, device=local))
    params = api.scene_params(sc, temporal_filter=1, temporal_decay=0.8, warp_mode=L.VCT_WARP_TEXTURE)
    params.trace_filter = sampler_id(args.filter)
    ctx.set_params(params)
    mlp = api.Mlp(device=local)
    w = learned.load_params()
    if w is not None:
        mlp.set_params(w)
    lights = api.light_array(sc.lights)
    shadow = api.shadow_desc(sc, sm)
    stream = torch.cuda.current_stream()
    lib = L.load()
    ctx.enable_timers(True)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    plain, learned_ms, stages = [], [], {k: [] for k in ("voxelize_ms", "radiance_ms", "mipmap_ms", "render_ms")}
    frags = []
    n_frames = args.frames
    launches0 = lib.vct_launch_count()
    with ClockSampler(local) as clk:
        for f in range(max(3, args.warmup) + n_frames):
            t = f / 30.0
            models = actors.models(t)
            # set-up passes of this frame: shadow map and G-buffers of the moved geometry
            api.transform_actors(local_tris, models, pos, nrm, stream)
            api.render_shadowmap(tris, sc, sm, stream)
            for v, (g, _) in zip(views, gbs):
                api.render_gbuffer(tris, v, keys, g[0], g[1], g[2], stream)
            ev[0].record(stream)
            api.transform_actors(local_tris, models, pos, nrm, stream)
            ctx.frame(tris, lights, shadow, views[0].eye, gbs[0][1], api.trace_out(color=color), stream)
            ctx.trace_views([gb for _, gb in gbs[1:]], [v.eye for v in views[1:]],
                            [api.trace_out(color=c) for c in view_colors], stream)
            ev[1].record(stream)
            for v, (_, gb) in zip(views, gbs):
                api.learned_trace(ctx, mlp, gb, v.eye, irr, float("inf"), stream=stream)
            ev[2].record(stream)
            ev[2].synchronize()
            if f >= max(3, args.warmup):
                plain.append(ev[0].elapsed_time(ev[1]))
                learned_ms.append(ev[1].elapsed_time(ev[2]))
                for k, v in ctx.timers().items():
                    if k in stages:
                        stages[k].append(v)
                frags.append(ctx.stats(stream)["total_voxel_fragments"])
    launches = lib.vct_launch_count() - launches0
    med = lambda v: float(statistics.median(v))  # noqa: E731
    value = max_over_ranks(sum(plain), world) / (len(plain) * world)
    accuracy = None
    if rank == 0 and not args.no_cpu_baseline:
        # outside the timed region: view 0's irradiance on the last frame's chain and warp map
        # against the fp64 oracle tracing the same chain with exact warp-map lookups
        import oracle as O

        irr0 = torch.zeros(W * H * 4, dtype=torch.float32, device=dev)
        ctx.trace(gbs[0][1], views[0].eye, api.trace_out(irradiance=irr0), stream)
        torch.cuda.synchronize()
        chain = np.concatenate([ctx.read_volume(L.VCT_VOLUME_RADIANCE, lv).cpu().numpy().view(np.uint16)
                                for lv in range(sc.levels)])
        wmap = ctx.read_warpmap().cpu().numpy().view(np.uint16)
        gp, gn, ga = (t.cpu().numpy() for t in gbs[0][0])
        nthreads = os.cpu_count() or 1
        t0 = time.perf_counter()
        irr64, _, _, _ = O.trace(views[0], chain, gp, gn, ga, precision=64, nthreads=nthreads, want=("irr",),
                                 warp=O.warp(views[0], L.VCT_WARP_TEXTURE, wmap))
        a = irradiance_accuracy(irr0.cpu().numpy(), irr64, gp.reshape(-1, 4)[:, 3] != 0)
        accuracy = {"judge": "fp64 cone-trace oracle on the last frame's GPU chain and warp map (exact lookups), "
                             "view 0, every covered pixel", "sampler": args.filter,
                    "bar": "irradiance rel-L2 <= 1e-3 vs fp64",
                    "vs_fp64": {k: (round(v, 9) if isinstance(v, float) else v) for k, v in a.items()},
                    "meets_bar": bool(a["rel_l2"] <= 1e-3), "fp64_trace_s": round(time.perf_counter() - t0, 2),
                    "threads": nthreads}
    return {
        "metric": DYNAMIC_METRIC, "value": round(value, 4), "unit": "ms/frame", "n_gpus": world,
        "steps": n_frames, "warmup": max(3, args.warmup), "ms_per_step": round(value * world, 4),
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 math, f16 volumes, u32 accumulators; bf16 network", "data": "synthetic seeded dynamic scene",
        "config": {"workload": "dynamic warped frames: 64 rigid actors (2k-8k tris) + 199k static tris = "
                               f"{sc.ntri} tris, 256^3 + 32^3 warp map + temporal filter, 8 views 1280x720",
                   "frames": n_frames, "actors": len(actors.first), "triangles": sc.ntri, "sampler": args.filter,
                   "timed": "actor transform + vct_frame (view 0) + one vct_trace_views launch (views 1-7); shadow "
                            "map and G-buffers rendered outside the events"},
        "plain_ms_median": round(med(plain), 4), "learned_traces_ms_median": round(med(learned_ms), 4),
        "stage_ms_median_view0": {k: round(med(v), 4) for k, v in stages.items()},
        "fragments_per_frame_median": int(statistics.median(frags)),
        "gpu_launches": int(launches),
        "clocks": clk.summary(),
        "learned_weights": "trained" if w is not None else "untrained (timing only)",
        "accuracy": accuracy,
    }


# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) per launch of each frame
# stage, from one ncu capture of the large frame (`bench.py --profile-frames 3`, default
# launch shapes): accumulate = setup + raster, resolve+mips = resolve + tail; only for the
# default workload, and only while the frame kernels' sources hash to NCU_CAPTURE_DIGEST.
NCU_CAPTURE_DIGEST = "438e8eac75de4cad"
NCU_CAPTURE_SAMPLER = "hybrid"
NCU_TRAFFIC = {"accumulate": 18.891e6 + 262.704e6 + 161.262e6, "resolve+mips": 258.924e6 + 835.439e6 + 0.047e6,
               "inject_mark": 18.258e6 + 0.023e6, "trace": 89.188e6 + 12.723e6}
# Issue-side figures of the cone tracer (hybrid sampler) from its full capture of the same
# command: it is bound by issue and load latency at its occupancy, not HBM.  (Captured
# before the accumulator records moved to 2 x 2 slots; the tracer reads no records and its
# code is unchanged.)
NCU_TRACE_ISSUE = {"sm_throughput_frac": 0.633, "fma_pipe_frac": 0.437, "l1_hit_rate": 0.971,
                   "l1_lsu_data_pipe_frac": 0.661, "l1_tex_data_pipe_frac": 0.240}


def load_peaks() -> dict:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return {"hbm_gbs": d["hbm_gbs"], "bf16_tflops": d["bf16_tflops"], "source": "measured"}
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "source": "fallback"}


# ----------------------------------------------------------- CPU side
def cpu_frame(sc, nthreads: int, sample_rows: int = 0, shadowmap=None, gbuf=None, tesselation=False,
              warp_mode=0, want=("color",)) -> tuple[float, dict, np.ndarray, tuple]:
    """One CPU-oracle frame: voxelize/normalize/inject/mips of the full grid
    and the trace of the whole frame (sample_rows = 0) or of `sample_rows`
    evenly spaced rows, extrapolated to the full frame.  Returns the frame's
    ms, per-stage ms, the radiance chain and the trace's outputs (irradiance,
    specular, colour, samples)."""
    import oracle as O

    W, H = sc.gbuffer_size
    sm = O.render_shadowmap(sc, nthreads) if shadowmap is None else shadowmap
    gp, gn, ga = O.render_gbuffer(sc) if gbuf is None else gbuf
    w = O.warp(sc, warp_mode) if warp_mode else None
    t0 = time.perf_counter()
    if tesselation:
        count, sums, total = O.voxelize_tess(sc, nthreads=nthreads, warp=w)
    else:
        count, sums, total = O.voxelize(sc, sm, nthreads=nthreads, warp=w)
    t1 = time.perf_counter()
    chain = np.zeros(4 * O.chain_voxels(sc.dim, sc.levels), dtype=np.uint16)
    color, normal, _, _ = O.normalize(sc, count, sums, radiance=chain, nthreads=nthreads)
    t2 = time.perf_counter()
    O.inject(sc, sm, color, normal, chain, nthreads=nthreads, warp=w)
    t3 = time.perf_counter()
    O.build_mips(sc.dim, sc.levels, chain, nthreads)
    t4 = time.perf_counter()
    step = max(1, H // sample_rows) if sample_rows > 0 else 1
    traced = O.trace(sc, chain, gp, gn, ga, precision=32, rows=(0, H), row_step=step, nthreads=nthreads, want=want,
                     warp=w)
    t5 = time.perf_counter()
    rows_traced = len(range(0, H, step))
    t = {"voxelize_ms": (t1 - t0) * 1e3, "normalize_ms": (t2 - t1) * 1e3, "inject_ms": (t3 - t2) * 1e3,
         "mips_ms": (t4 - t3) * 1e3, "trace_ms": (t5 - t4) * 1e3 * H / rows_traced, "rows_traced": rows_traced}
    return (t4 - t0) * 1e3 + t["trace_ms"], t, chain, traced


def cpu_sample_text(detail: dict, H: int, nthreads: int) -> str:
    what = "the whole frame traced" if detail["rows_traced"] == H else (
        f"trace of {detail['rows_traced']} evenly spaced rows of {H}, scaled to the full frame")
    return f"one frame: full voxelize/normalize/inject/mips + {what}, {nthreads} thread(s)"


def accuracy_block(sc, art: dict, chain32: np.ndarray, irr32: np.ndarray, headline: str, nthreads: int,
                   warp_mode: int = 0) -> dict:
    """The frame's irradiance per sampler against the fp64 cone-trace oracle
    (the 1e-3 bar) and the fp32 oracle, over every covered pixel of the
    frame; and whether the GPU radiance chain equals the oracle's, bit for
    bit.  Inputs: the GPU's shadow map and G-buffer (bit-exact against the
    oracle's own) and the oracle's chain."""
    import oracle as O

    gp, gn, ga = art["gbuf"]
    w = O.warp(sc, warp_mode) if warp_mode else None
    t0 = time.perf_counter()
    irr64, _, _, _ = O.trace(sc, chain32, gp, gn, ga, precision=64, nthreads=nthreads, want=("irr",), warp=w)
    fp64_s = time.perf_counter() - t0
    cov = gp.reshape(-1, 4)[:, 3] != 0
    out = {"judge": "fp64 cone-trace oracle (exact trilinear) over every covered pixel of the frame",
           "bar": "irradiance rel-L2 <= 1e-3 vs fp64", "chain_bitexact": bool(np.array_equal(art["chain"], chain32)),
           "oracle_fp32_vs_fp64_rel_l2": irradiance_accuracy(irr32, irr64, cov)["rel_l2"],
           "fp64_trace_s": round(fp64_s, 2), "threads": nthreads, "samplers": {}}
    for name, g in art["irr"].items():
        a64 = irradiance_accuracy(g, irr64, cov)
        a32 = irradiance_accuracy(g, irr32, cov)
        out["samplers"][name] = {"vs_fp64": {k: (round(v, 9) if isinstance(v, float) else v) for k, v in a64.items()},
                                 "vs_fp32_oracle_rel_l2": a32["rel_l2"], "vs_fp32_oracle_max_rel": a32["max_rel"]}
    h = out["samplers"].get(headline)
    if h is not None:
        out["headline_sampler"] = headline
        out["headline_rel_l2_vs_fp64"] = h["vs_fp64"]["rel_l2"]
        out["meets_bar"] = bool(h["vs_fp64"]["rel_l2"] <= 1e-3)
    return out


# Arm Ltd. (implementer 0x41) part numbers of server cores, as /proc/cpuinfo prints them
ARM_PARTS = {"0xd0c": "Neoverse-N1", "0xd40": "Neoverse-V1", "0xd49": "Neoverse-N2", "0xd4f": "Neoverse-V2",
             "0xd8e": "Neoverse-N3", "0xd84": "Neoverse-V3"}


def cpu_model(cpuinfo: str | None = None) -> str:
    """The host CPU's model name: x86 /proc/cpuinfo's "model name", or an
    Arm core's part number mapped to its name (Grace is Neoverse-V2)."""
    if cpuinfo is None:
        try:
            cpuinfo = open("/proc/cpuinfo").read()
        except OSError:
            cpuinfo = ""
    part = impl = None
    for line in cpuinfo.splitlines():
        key, _, val = line.partition(":")
        key, val = key.strip().lower(), val.strip()
        if key == "model name" and val:
            return val
        if key == "cpu part" and part is None:
            part = val.lower()
        if key == "cpu implementer" and impl is None:
            impl = val.lower()
    if part is not None:
        name = ARM_PARTS.get(part) if impl in (None, "0x41") else None
        return f"{name} (Arm part {part})" if name else f"Arm part {part}, implementer {impl}"
    return platform.processor() or platform.machine()


def irradiance_accuracy(gpu: np.ndarray, ref: np.ndarray, covered: np.ndarray, floor_frac: float = 1e-3) -> dict:
    """Error of a GPU irradiance image against an oracle image (RGBA float
    arrays of the frame; alpha ignored) over the covered pixels: the relative
    L2 error over all covered pixels' RGB, and the per-pixel relative error
    |g - r| / |r| (Euclidean over RGB) of the pixels whose reference
    irradiance exceeds floor_frac times its root mean square (darker pixels'
    relative errors divide by almost nothing): maximum, 99.9th and 99th
    percentiles, and the fraction within 1e-3."""
    g = np.asarray(gpu, dtype=np.float64).reshape(-1, 4)[covered, :3]
    r = np.asarray(ref, dtype=np.float64).reshape(-1, 4)[covered, :3]
    d = np.linalg.norm(g - r, axis=1)
    n = np.linalg.norm(r, axis=1)
    tot = float(np.sqrt(np.sum(n * n)))
    out = {"rel_l2": float(np.sqrt(np.sum(d * d)) / tot) if tot > 0 else float(np.sqrt(np.sum(d * d))),
           "pixels": int(g.shape[0])}
    floor = floor_frac * float(np.sqrt(np.mean(n * n))) if n.size else 0.0
    sel = n > floor
    e = d[sel] / n[sel]
    out.update({"pixels_judged": int(sel.sum()), "judged_floor": floor,
                "max_rel": float(e.max()) if e.size else 0.0,
                "p999_rel": float(np.quantile(e, 0.999)) if e.size else 0.0,
                "p99_rel": float(np.quantile(e, 0.99)) if e.size else 0.0,
                "frac_within_1e-3": float(np.mean(e <= 1e-3)) if e.size else 1.0})
    return out


KERNEL_SOURCES = ("cone.cuh", "vct_device.cuh", "vct_internal.h", "warp.cuh", "voxelize.cu", "volume.cu", "trace.cu")


def kernel_sources_digest() -> str:
    """sha256 (first 16 hex digits) of the frame kernels' sources: the ncu
    traffic figures below hold only for the sources they were captured from."""
    import hashlib

    h = hashlib.sha256()
    for name in KERNEL_SOURCES:
        with open(os.path.join(ROOT, "vct_gb300", "csrc", name), "rb") as f:
            h.update(name.encode() + b"\0" + f.read())
    return h.hexdigest()[:16]


def ncu_traffic(headline: bool) -> tuple[dict, dict]:
    """The ncu DRAM traffic per frame stage (and the tracer's issue figures)
    when this workload's kernels are the ones they were captured from; else
    empty, with the reason."""
    if not headline:
        return {}, {"traffic_source": "no ncu capture of this workload"}
    digest = kernel_sources_digest()
    if digest != NCU_CAPTURE_DIGEST:
        return {}, {"traffic_stale": f"the frame kernels' sources (digest {digest}) changed since the ncu capture "
                                     f"(digest {NCU_CAPTURE_DIGEST}): traffic withheld"}
    return dict(NCU_TRAFFIC), {"traffic_source": "ncu dram read+write per launch, one capture of this workload",
                               "traffic_digest": digest}


def run_reference_batch(args, world):
    """Batched family on the CPU restatement: every scene of the batch per
    step (full voxelize/normalize/inject/mips, row-sampled trace scaled to the
    frame), all host threads."""
    from vct_gb300 import scenes

    nthreads = os.cpu_count() or 1
    rows = args.cpu_sample_rows or 24
    scs = [scenes.batch_scene(seed=args.seed, index=i) for i in range(args.batch_scenes)]
    times = []
    for i in range(args.warmup + args.steps):
        ms = sum(cpu_frame(sc, nthreads, rows)[0] for sc in scs)
        if i >= args.warmup:
            times.append(ms)
    value = sum(times) / len(times)
    sample = (f"each step: all {len(scs)} scenes, full voxelize/normalize/inject/mips + trace of "
              f"{rows} evenly spaced rows per scene scaled to the full frame")
    return {
        "impl": "reference", "metric": BATCH_METRIC.replace("32", str(args.batch_scenes)), "value": round(value, 2),
        "unit": "ms/batch", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(value, 2), "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 math, f16 volumes, u32 accumulators", "data": "synthetic seeded scenes (no dataset)",
        "config": {"workload": f"batched family: {args.batch_scenes} scenes", "seed": args.seed},
        "cpu_baseline": {"value": round(value, 2), "unit": "ms/batch", "cores": nthreads, "kind": "port",
                         "sample": sample, "cpu": cpu_model()},
        "e2e": {"value": round(value, 2), "unit": "ms/batch", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def run_reference(args, rank, world):
    """The reference's path on the host cores: its GLSL cannot run here (no
    graphics stack), so the oracle, which restates it, runs every stage of the
    same workload on all host threads, the whole frame traced every step."""
    if args.config == "batch":
        return run_reference_batch(args, world)
    sc = make_scene(args)
    nthreads = os.cpu_count() or 1
    import oracle as O

    sm = O.render_shadowmap(sc, nthreads)
    gbuf = O.render_gbuffer(sc)
    tess, warp_mode = args.voxelizer == "tess", 3 if args.warp == "perspective" else 0
    times = []
    for i in range(args.warmup + args.steps):
        ms, detail, _, _ = cpu_frame(sc, nthreads, args.cpu_sample_rows, sm, gbuf, tesselation=tess,
                                     warp_mode=warp_mode)
        if i >= args.warmup:
            times.append(ms)
    value = sum(times) / len(times)
    H = sc.gbuffer_size[1]
    return {
        "impl": "reference", "metric": METRIC, "value": round(value, 2), "unit": "ms/frame", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(value, 2), "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 math, f16 volumes, u32 accumulators",
        "data": "synthetic seeded scene (no dataset)",
        "config": dict(frame_config(args, sc, world), l2="not applicable: host cores"),
        "cpu_baseline": {"value": round(value, 2), "unit": "ms/frame", "cores": nthreads, "kind": "port",
                         "sample": "each step " + cpu_sample_text(detail, H, nthreads), "cpu": cpu_model(),
                         "why_port": "the reference's own path is OpenGL/GLSL, and this machine has no graphics stack"},
        "e2e": {"value": round(value, 2), "unit": "ms/frame", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "stage_ms_last": {k: round(v, 2) for k, v in detail.items()},
    }


def main():
    args = parse()
    rank, world = dist_init(args.gpus)
    if args.impl == "reference":
        if rank == 0:
            print(json.dumps(run_reference(args, rank, world)), flush=True)
        return
    if args.config == "dynamic":
        result = run_dynamic(args, rank, world)
        if rank == 0:
            print(json.dumps(result), flush=True)
        return
    if args.config == "learned":
        result = run_learned(args, rank, world)
        if rank == 0:
            print(json.dumps(result), flush=True)
        return
    if args.config == "batch":
        result, scs = run_batch(args, rank, world)
        if rank == 0 and not args.no_cpu_baseline:
            # one single-threaded oracle frame of the smallest scene of the batch, row-sampled trace,
            # scaled by the batch's voxel + pixel work relative to that scene
            small = min(scs, key=lambda s: s.dim ** 3 + s.gbuffer_size[0] * s.gbuffer_size[1])
            ms, detail, _, _ = cpu_frame(small, 1, args.cpu_sample_rows or 24)
            result["cpu_baseline"] = {"value": round(ms, 2), "unit": "ms/frame of the smallest scene", "cores": 1,
                                      "kind": "port", "sample": f"scene {small.name}: {small.ntri} tris, "
                                      f"{small.dim}^3, {small.gbuffer_size[0]}x{small.gbuffer_size[1]}, trace of "
                                      f"{detail['rows_traced']} rows scaled to the frame", "cpu": cpu_model()}
        if rank == 0:
            print(json.dumps(result), flush=True)
        return
    result, sc, art = run_ours(args, rank, world)
    if result is None:  # --profile-frames
        return
    if rank == 0 and not args.no_cpu_baseline:
        # the oracle on the GPU's own shadow map and G-buffer (both bit-exact against the oracle's): the
        # single-threaded baseline frame, whole frame traced (the tessellation voxeliser's hundreds of
        # millions of points take minutes on one core: all cores there)
        cores = 1 if args.voxelizer == "raster" else (os.cpu_count() or 1)
        warp_mode = 3 if args.warp == "perspective" else 0
        ms, detail, chain32, (irr32, _, _, _) = cpu_frame(
            sc, cores, args.cpu_sample_rows, art["sm"], art["gbuf"], tesselation=args.voxelizer == "tess",
            warp_mode=warp_mode, want=("irr", "color"))
        result["cpu_baseline"] = {"value": round(ms, 2), "unit": "ms/frame", "cores": cores, "kind": "port",
                                  "sample": cpu_sample_text(detail, sc.gbuffer_size[1], cores), "cpu": cpu_model(),
                                  "nproc": os.cpu_count(), "stage_ms": {k: round(v, 1) for k, v in detail.items()}}
        if detail["rows_traced"] == sc.gbuffer_size[1]:
            result["accuracy"] = accuracy_block(sc, art, chain32, irr32, args.filter, os.cpu_count() or 1,
                                                warp_mode)
    if rank == 0 and args.config == "large" and not args.no_extra_configs:
        # the benchmark's other configurations, compact and outside the timed region (rank 0 alone)
        import torch

        torch.cuda.empty_cache()
        result["batch"], _ = run_batch(args, 0, 1, compact=True)
        torch.cuda.empty_cache()
        result["learned"] = run_learned(args, 0, 1, compact=True)
    if rank == 0:
        print(json.dumps(result), flush=True)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
