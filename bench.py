#!/usr/bin/env python3
"""GB300 benchmark of the many-lights GI hot path (RSM -> VPLs -> ISM splat -> pull-push -> FG).

One step = one GI frame of the workload (default: 1920x1080, 1024 VPLs, 2^22 points, 4096^2 ISM
atlas of 128^2 ISMs, 6 pull-push levels, interleave 8, 16x16 same-class tiles with culling):
mlgi_gi_frame on inputs resident in HBM (`value`), and mlgi_gi_frame_host from pinned host
buffers with every input copied in and the radiance copied out per step (`e2e`).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--config c2_1920x1080_n1024]
    python bench.py --impl reference ...   # the CPU implementation of the path, all host cores

Prints one JSON line on rank 0. Multi-GPU (torchrun) runs independent replicas (weak scaling).
"""
from __future__ import annotations

import argparse
import datetime
import json
import os
import re
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path[:0] = [ROOT, os.path.join(ROOT, "many-lights-gi_gb300")]

METRIC = "1080p GI ms/frame"
UNIT = "ms/frame"
PASSES = ["vpl_process", "ism_clear", "ism_splat", "pullpush", "final_gather"]
# kernels of a frame and their slots in Context.last_timings(); the pull-push pass is four launches
def kernel_slots(cfg):
    """(kernel, index in mlgi_last_timings) of the kernels of a frame. The pull-push pass is one
    launch (`pyramid`, reported in the pass's last slot) when each ISM's pyramid runs in one block;
    the per-level launches over two halves of the ISM rows side by side are reported as the pass
    (`pullpush`, its last slot); one per-level sequence as level 1, the middle levels and push level
    1 (two or more levels), and push level 0."""
    import mlgi

    n = mlgi.pullpush_launches(cfg)
    halves = n in (8,) or (n == 4 and cfg.levels < 2)
    pp = [("pyramid", 10)] if n == 1 else [("pullpush", 10)] if halves else \
        [("pull1", 7), ("pullmid", 8), ("push1", 9), ("push0", 10)] if n == 4 else [("pull1", 7), ("push0", 10)]
    return [("vpl_process", 0), ("ism_clear", 1), ("ism_splat", 2)] + pp + [("final_gather", 4)]


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)  # about 1.5 s of timed frames at C2, for the clock samples
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="mlgi", choices=["mlgi", "reference"])
    ap.add_argument("--config", default="c2_1920x1080_n1024")
    ap.add_argument("--cpu-seconds", type=float, default=12.0, help="CPU-baseline sample budget")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--reference-seconds", type=float, default=60.0, help="reference arm: time budget of the frames")
    ap.add_argument("--slots", type=int, default=8, help="served form: frames in flight")
    ap.add_argument("--rate", type=float, default=2000.0, help="served form: Poisson arrival rate (req/s)")
    ap.add_argument("--duration", type=float, default=10.0, help="served form: seconds of arrivals")
    ap.add_argument("--seed", type=int, default=5, help="served form: request-stream seed")
    ap.add_argument("--views", type=int, default=32, help="batched form: views per batch")
    ap.add_argument("--batch-streams", type=int, default=4, help="batched form: streams of the concurrent form")
    ap.add_argument("--no-extras", action="store_true",
                    help="default workload: skip the bounded batched and served measurements")
    ap.add_argument("--extra-batch-steps", type=int, default=10, help="default workload: timed batches per form")
    ap.add_argument("--extra-serve-seconds", type=float, default=2.0,
                    help="default workload: seconds of arrivals per served/plain stream")
    return ap.parse_args()


def launches_per_frame(cfg):
    """Kernels of one timed mlgi_gi_frame: VPL processing and the atlas clear (one launch), splat,
    the pull-push pass's launches and final gathering. (Frames with per-pass timing launch the VPL
    pass and the clear separately.)"""
    import mlgi

    return 2 + mlgi.pullpush_launches(cfg) + 1


# ---- algorithmic bytes per pass and per kernel (one launch each per frame) ----------------------
def algorithmic_bytes(cfg, bucket_stride):
    """Bytes each pass and each kernel must move. Passes: VPL records; the atlas clear; the points
    (the splat's atomics stay in L2); pull-push as one ideal pass (keys in, final atlas out); and the
    gathering's G-buffer, radiance, one atlas texel per evaluated pair and the VPL records. Kernels
    of the pull-push pass add their pyramid levels: level 1 is 16 B per 4 atlas texels, level 2 per 16."""
    px = cfg.width * cfg.height
    nrm = 4 if cfg.reduced else 8
    atlas = cfg.atlas_w * cfg.atlas_h
    vrec = 24 if cfg.reduced else 48
    out = 2 if cfg.reduced else 4
    two = cfg.levels >= 2
    return {
        "vpl_process": cfg.n_vpl * (4 + 4 + 4 + 48 + 16),
        "ism_clear": atlas * 4,
        "ism_splat": cfg.n_points * 16 + cfg.n_vpl * 4,
        "pullpush": atlas * (4 + out),
        "final_gather": px * (4 + nrm + 12) + cfg.pairs * out + cfg.n_vpl * vrec,
        "pull1": atlas * 4 + atlas // 4 * 16,
        "pullmid": (atlas // 4 * 16 + atlas // 16 * 16) if two else 0,
        "push1": (atlas // 16 * 16 + atlas // 4 * 32) if two else 0,
        "push0": atlas // 4 * 16 + atlas * 4 + atlas * out,
        "pyramid": atlas * (4 + out),
    }


def measured_peak_gbs():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def ncu_traffic(kernel, key="traffic", workload="c2_1920x1080_n1024"):
    """Per-launch DRAM bytes (key "traffic") or issue-slot use in percent (key "issue") of `kernel`
    from the committed ncu summary of `workload` (a file under profiles/ named for it), if any."""
    pdir = os.path.join(ROOT, "profiles")
    for fn in sorted(os.listdir(pdir)) if os.path.isdir(pdir) else []:
        if workload not in fn:
            continue
        try:
            txt = open(os.path.join(ROOT, "profiles", fn)).read()
        except Exception:
            continue
        m = re.search(re.escape(key) + r"\[" + re.escape(kernel) + r"\]\s*=\s*([0-9.eE+]+)", txt)
        if m:
            return float(m.group(1))
    return None


class ClockSampler:
    """nvidia-smi clocks, throttle reasons and utilization sampled every 200 ms. mark(True) and
    mark(False) bracket the timed region; stop() then summarises the samples taken inside it (all
    samples when no sample fell inside, said in "window")."""

    FIELDS = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap,utilization.gpu")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = None
        self.t0 = self.t1 = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def mark(self, begin):
        if begin:
            self.t0 = time.time()
        else:
            self.t1 = time.time()

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 10:
                try:
                    parts[0] = datetime.datetime.strptime(parts[0], "%Y/%m/%d %H:%M:%S.%f").timestamp()
                except ValueError:
                    parts[0] = None  # kept, but it cannot be placed in the timed region
                rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return None
        window = "timed region"
        if self.t0 is not None:
            end = self.t1 if self.t1 is not None else float("inf")
            inside = [r for r in rows if r[0] is not None and self.t0 <= r[0] <= end]
            if inside:
                rows = inside
            else:
                window = "whole run (no sample inside the timed region)"
        else:
            window = "whole run"
        num = lambda v: v.replace(".", "").isdigit()
        sm = [float(r[2]) for r in rows if num(r[2])]
        mx = [float(r[3]) for r in rows if num(r[3])]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({n for r in rows for n, v in zip(names, r[6:10]) if v.lower().startswith("active")})
        busy = [float(r[10]) for r in rows if len(r) > 10 and num(r[10])]
        out = {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
               "reasons": reasons, "samples": len(rows), "window": window}
        # utilization.gpu averages over nvidia-smi's own period, which a timed region of a second or
        # two does not fill: it is reported for the long streams only
        if window != "timed region":
            out["gpu_busy_pct"] = statistics.median(busy) if busy else None
        return out


# ---- CPU implementation of the path (the oracle's FP32 restatement, all host threads) -----------
def cpu_frame_runner(cfg, scene):
    import numpy as np

    import mlgi
    from oracle import oracle as O

    perm = mlgi.shuffle_table(cfg.n_vpl)

    def frame(passes=None):
        """One frame; `passes`, when given, receives each pass's wall time in ms (the splat pass
        includes the atlas clear, as the oracle's splat returns a fresh atlas)."""
        t = [time.perf_counter()]
        pos, nrm, col, pn = O.vpl_process(scene.rsm_depth, scene.rsm_normal, scene.rsm_diffuse, cfg.n_vpl,
                                          scene.mat("inv_biased_light_vp"), cfg.light_intensity, 1, perm)
        t.append(time.perf_counter())
        keys = O.ism_splat(scene.points, scene.counts, scene.bucket_stride, pos, pn, cfg.n_vpl, cfg.ism_size,
                           cfg.grid_x, cfg.grid_y, cfg.z_far)
        t.append(time.perf_counter())
        fin = O.pullpush(keys, cfg.ism_size, cfg.levels, cfg.z_far)
        t.append(time.perf_counter())
        out = O.final_gather(scene.gbuf_depth, scene.gbuf_normal, scene.mat("inv_view_proj"), pos, nrm, col, fin,
                             cfg.ism_size, cfg.grid_x, cfg.grid_y, cfg.z_far, cfg.gi_intensity, cfg.clamp_value,
                             cfg.interleave, tile=cfg.tile if cfg.cull else 0, cutoff=cfg.influence_cutoff)
        t.append(time.perf_counter())
        if passes is not None:
            for name, a, b in zip(CPU_PASSES, t, t[1:]):
                passes.setdefault(name, []).append((b - a) * 1e3)
        return out

    return frame, O.max_threads()


CPU_PASSES = ("vpl_process", "ism_clear+ism_splat", "pullpush", "final_gather")


def time_cpu(cfg, scene, budget_s, min_frames=2):
    """Median ms per frame of the CPU chain, the median of each pass, the threads used and the
    number of frames timed."""
    frame, threads = cpu_frame_runner(cfg, scene)
    frame()  # warm
    times, passes = [], {}
    t_end = time.perf_counter() + budget_s
    while len(times) < min_frames or time.perf_counter() < t_end:
        t0 = time.perf_counter()
        frame(passes)
        times.append((time.perf_counter() - t0) * 1e3)
    return statistics.median(times), threads, len(times), {n: statistics.median(v) for n, v in passes.items()}


def config_dict(cfg):
    return {"workload": cfg.name, "resolution": f"{cfg.width}x{cfg.height}", "vpls": cfg.n_vpl,
            "points": cfg.n_points, "rsm": f"{cfg.rsm}x{cfg.rsm}",
            "ism": f"{cfg.ism_size}^2 x {cfg.grid_x}x{cfg.grid_y} = {cfg.atlas_w}x{cfg.atlas_h}",
            "pullpush_levels": cfg.levels, "interleave": cfg.interleave, "tile": cfg.tile, "cull": bool(cfg.cull),
            "influence_cutoff": cfg.influence_cutoff,
            "precision": "fp16/bf16 storage, fp32 math" if cfg.reduced else "fp32",
            "scene": "seeded procedural room (100-unit Cornell box, boxes, spheres, spot light)",
            "l2": "flushed between steps (256 MiB write, then a 256 MiB read so that no dirty line is written "
                  "back inside the timed region)"}


def reduce_max(values, world):
    """Each value's maximum over the ranks (replicas run in parallel, so the job takes as long as
    its slowest rank); the values themselves at world size 1."""
    if world <= 1:
        return [float(v) for v in values]
    import torch
    import torch.distributed as dist

    t = torch.tensor([float(v) for v in values], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t]


def run_reference(args, cfg, rank, world):
    if rank != 0:
        return
    import mlgi

    scene = mlgi.make_scene(cfg)
    frame, threads = cpu_frame_runner(cfg, scene)
    # args.warmup untimed frames, stopped early (after at least one) once they have taken a quarter
    # of the time bound, so that the whole run stays within a few minutes
    warmed = 0
    t_start = time.perf_counter()
    while warmed < args.warmup:
        frame()
        warmed += 1
        if time.perf_counter() - t_start > args.reference_seconds / 4:
            break
    # each step is one full frame on the host cores; the run is bounded to about a minute of frames
    times, passes = [], {}
    t_start = time.perf_counter()
    for _ in range(args.steps):
        t0 = time.perf_counter()
        frame(passes)
        times.append((time.perf_counter() - t0) * 1e3)
        if time.perf_counter() - t_start > args.reference_seconds and len(times) >= 3:
            break
    ms = statistics.median(times)
    line = {"impl": "reference", "metric": METRIC, "value": ms, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": config_dict(cfg),
            "cpu_baseline": {"value": ms, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"median of {len(times)} of {args.steps} full frames of {cfg.name} after "
                                       f"{warmed} warm-up frames (bounded to about {args.reference_seconds:.0f} s), "
                                       f"FP32 oracle restatement of the reference shaders, OpenMP on {threads} "
                                       f"threads",
                             "passes_ms": {n: statistics.median(v) for n, v in passes.items()}},
            "e2e": {"value": ms, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


class L2Flush:
    """Evicts the L2 between timed steps: writes a 256 MiB buffer (twice the 129 MB L2), then reads
    another 256 MiB one, so that the L2 holds clean lines only and the timed kernels pay for no
    write-back of the flush itself."""

    def __init__(self, dev):
        import torch

        self.w = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
        self.r = torch.zeros(64 << 20, dtype=torch.float32, device=dev)

    def __call__(self, i):
        self.w.fill_(i & 0xFF)
        self.r.max()


def post_passes(ctx, df, scene, cfg, stream, flush, steps, warmup):
    """The passes after the gathering on the reference's buffer formats: the gathered radiance packed
    to R11G11B10F, the bilateral blur on R11G11B10F buffers, and the composite to RGBA8. Mean CUDA-event
    time per launch over `steps` launches (L2 flushed before each), with each pass's algorithmic bytes:
    pack 12 + 4, blur 4 (GI) + 4 (depth) + 8 or 4 (normal) + 4 (out), composite 4 (GI) + 4 (albedo)
    + 4 (out) per pixel."""
    import numpy as np
    import torch

    import mlgi

    px = cfg.width * cfg.height
    words = torch.zeros(px, dtype=torch.int32, device=df.rgb.device)
    blurred = torch.zeros_like(words)
    out8 = torch.zeros_like(words)
    albedo = torch.from_numpy(np.ascontiguousarray(scene.gbuf_albedo.view(np.int32))).to(df.rgb.device)
    a, b = mlgi.depth_terms(scene)
    g = df.gbuffer_view()
    s = ctx.stream()
    passes = {
        "pack_r11g11b10f": (lambda: ctx.pack_r11g11b10f(df.rgb, words, px, s), px * 16),
        "gi_blur": (lambda: ctx.gi_blur(g, words, blurred, a, b, mlgi.R11G11B10F, s),
                    px * (4 + 4 + (4 if cfg.reduced else 8) + 4)),
        "composite": (lambda: ctx.composite(blurred, albedo, out8, cfg.width, cfg.height, 1.0, mlgi.R11G11B10F,
                                            mlgi.RGBA8, stream=s), px * 12),
    }
    peak, kind = measured_peak_gbs()
    out = {}
    torch.cuda.synchronize()
    with torch.cuda.stream(stream):
        for name, (fn, nbytes) in passes.items():
            for _ in range(warmup):
                fn()
            ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
            for e0, e1 in ev:
                flush(1)
                e0.record(stream)
                fn()
                e1.record(stream)
            torch.cuda.synchronize()
            ms = float(np.mean([e0.elapsed_time(e1) for e0, e1 in ev]))
            gbs = nbytes / (ms * 1e-3) / 1e9
            out[name] = {"ms": ms, "algorithmic_bytes": nbytes, "achieved_gbs": gbs, "frac": gbs / peak,
                         "peak_source": kind}
    ctx.check_device_status()
    return out


def run_gpu(args, cfg, rank, world, local_rank):
    import numpy as np
    import torch

    import mlgi
    from mlgi.device import DeviceFrame, host_frame_desc, pinned_inputs

    torch.cuda.set_device(local_rank)
    dev = f"cuda:{local_rank}"
    scene = mlgi.make_scene(cfg.replace(seed=cfg.seed + rank))
    ctx = mlgi.Context(local_rank)
    stream = torch.cuda.ExternalStream(ctx.stream(), device=dev)
    df = DeviceFrame(scene, dev)
    flush = L2Flush(dev)
    fd = df.frame_desc()
    out = df.radiance()
    # the timed frames run as a caller runs them, without per-pass events; the per-pass times come
    # from separate frames with them (below)
    ctx.set_timing(False)

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()

    # ---- device-resident frames (value) ----
    # nvidia-smi samples every 200 ms: it starts before the warm-up and stops after the timed loop
    sampler = ClockSampler(local_rank)
    sampler.start()
    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            ctx.gi_frame(fd, out, ctx.stream())
        ctx.check_device_status()
        barrier()
        starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
        ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
        sampler.mark(True)
        t0 = time.perf_counter()
        for i in range(args.steps):
            flush(i)
            starts[i].record(stream)
            ctx.gi_frame(fd, out, ctx.stream())
            ends[i].record(stream)
        barrier()
        wall = time.perf_counter() - t0
        sampler.mark(False)
        clocks = sampler.stop()
        ctx.check_device_status()
        # per-pass device times: the same frames with the per-pass events of mlgi_set_timing
        ctx.set_timing(True)
        n_pass = min(args.steps, 200)
        passes = np.zeros((n_pass, 11))
        for i in range(n_pass):
            flush(i)
            ctx.gi_frame(fd, out, ctx.stream())
            passes[i] = ctx.last_timings()
        ctx.set_timing(False)
        barrier()
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    total_ms = sum(step_ms)

    # the splat's atomicMin count for this frame (outside the timed region; a counting run of the
    # same cull and projection)
    ctx.vpl_process(df.rsm_view(), mlgi.vpl_params(scene.cfg, scene), df.vpl_buf())
    atomics = ctx.ism_splat_count(df.points_view(), df.vpl_buf(), scene.cfg.n_vpl, mlgi.ism_params(scene.cfg),
                                  df.atlas_view())

    # ---- end to end through the host-buffer C ABI call (e2e) ----
    pinned = pinned_inputs(scene)
    hfd = host_frame_desc(scene, pinned)
    rgb_host = pinned["rgb"].numpy()
    for _ in range(max(10, args.warmup)):  # includes the call that captures the frame's graph
        ctx.gi_frame_host(hfd, rgb_host)
    barrier()
    e2e_times = []
    for i in range(args.steps):
        flush(i)
        torch.cuda.synchronize()
        t = time.perf_counter()
        ctx.gi_frame_host(hfd, rgb_host)
        e2e_times.append((time.perf_counter() - t) * 1e3)
    e2e_total = sum(e2e_times)
    # one more host frame with per-pass events: the upload and download spans of the copy streams
    ctx.set_timing(True)
    ctx.gi_frame_host(hfd, rgb_host)
    t = ctx.last_timings()
    ctx.set_timing(False)
    e2e_passes = {"h2d_ms": float(t[5]), "d2h_tail_ms": float(t[6])}
    sizes = mlgi.FrameHostSizes()
    mlgi.lib().mlgi_frame_host_sizes_get(mlgi.C.byref(hfd), mlgi.C.byref(sizes))
    h2d = sizes.rsm_depth + sizes.rsm_normal + sizes.rsm_diffuse + sizes.points + sizes.counts + \
        sizes.gbuf_depth + sizes.gbuf_normal
    d2h = sizes.radiance

    post = post_passes(ctx, df, scene, cfg, stream, flush, min(args.steps, 200), args.warmup)

    total_ms, e2e_total = reduce_max([total_ms, e2e_total], world)
    if rank != 0:
        ctx.close()
        return

    frames = args.steps * world
    value = total_ms / frames
    mean_all = passes.mean(axis=0)
    mean_pass = mean_all[:5]
    kernel_ms = {n: float(mean_all[i]) for n, i in kernel_slots(cfg)}
    ab = algorithmic_bytes(cfg, scene.bucket_stride)
    # the dominant kernel (a pull-push pass of several launches is not one kernel)
    dom_name = max((k for k in kernel_ms if k != "pullpush"), key=kernel_ms.get)
    peak, peak_kind = measured_peak_gbs()
    achieved = ab[dom_name] / (kernel_ms[dom_name] * 1e-3) / 1e9
    traffic = ncu_traffic(dom_name, workload=cfg.name)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": statistics.mean(step_ms), "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32" if not cfg.reduced else "f32 (fp16/bf16 storage)",
        "data": "synthetic (seeded procedural room)", "config": config_dict(cfg),
        "gpixel_vpl_per_s": frames * cfg.width * cfg.height * cfg.n_vpl / (total_ms * 1e-3) / 1e9,
        "evaluated_pairs_per_s": frames * cfg.pairs / (total_ms * 1e-3),
        "splat_atomics_per_frame": atomics,
        "splat_atomics_per_s": atomics / (kernel_ms["ism_splat"] * 1e-3) if kernel_ms.get("ism_splat") else None,
        "passes_ms": {n: float(v) for n, v in zip(PASSES, mean_pass)},
        "kernels_ms": kernel_ms,
        "gpu_launches": launches_per_frame(cfg) * args.steps,
        "e2e": {"value": e2e_total / frames, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), **e2e_passes,
                "p50_ms": statistics.median(e2e_times), "min_ms": min(e2e_times),
                "h2d_gbs": h2d / (e2e_passes["h2d_ms"] * 1e-3) / 1e9 if e2e_passes["h2d_ms"] > 0 else None,
                "note": "uploads on a copy stream in the order the passes read them; each point range is "
                        "splatted, and the ISM rows it completes pulled and pushed, while the next arrives; "
                        "the gathering runs in bands of rows, each downloaded while the next is gathered "
                        "(d2h_tail_ms: download time left after the last band)"},
        "roofline": {"bound": "hbm", "kernel": dom_name, "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_source": peak_kind,
                     "algorithmic_bytes": ab[dom_name], "traffic": traffic,
                     "issue_busy_pct": ncu_traffic(dom_name, "issue", cfg.name),
                     "note": "FP32-issue-bound kernels (bit-exact IEEE division, no FMA contraction): "
                             "issue_busy_pct is the dominant kernel's issue-slot use from the committed "
                             "ncu summary"},
        "per_pass_frac": {n: ab[n] / (mean_pass[i] * 1e-3) / 1e9 / peak for i, n in enumerate(PASSES)
                          if mean_pass[i] > 0},
        "per_kernel_frac": {n: ab[n] / (t * 1e-3) / 1e9 / peak for n, t in kernel_ms.items() if t > 0},
        "clocks": clocks,
        "wall_s": wall,
        "post": post,
    }
    if not args.no_extras and world == 1:
        # the batched and served halves of the metric, bounded: a 32-view batch in both forms and a
        # few seconds of the served Poisson stream against the plain arm
        ctx.close()
        ctx = None
        b = measure_batch(local_rank, args.views, args.extra_batch_steps, 2, args.batch_streams)
        line["batched"] = {k: b[k] for k in ("views", "form", "ms_per_batch", "frames_per_s", "forms",
                                              "plain_ms_per_batch", "plain_frames_per_s", "speedup_vs_plain",
                                              "kernel_launches_per_batch", "steps", "warmup", "autotune_s")}
        line["batched"]["workload"] = "c4_batch32: 32 views of 8 rooms, autotuned"
        sv = measure_serve(local_rank, args.slots, args.rate, args.extra_serve_seconds, args.seed)
        line["served"] = {k: sv[k] for k in ("served", "plain", "served_at_75pct", "plain_at_75pct",
                                              "speedup_vs_plain", "single_frame_ms",
                                              "results_identical_served_vs_plain", "config")}
        line["served"]["workload"] = "c5_served_poisson (bounded duration)"
    if not args.no_cpu_baseline and world == 1:
        ms, threads, nframes, cpu_passes = time_cpu(cfg, scene, args.cpu_seconds)
        line["cpu_baseline"] = {"value": ms, "unit": UNIT, "cores": threads, "kind": "port",
                                "sample": f"{nframes} full {cfg.name} frames (median), FP32 oracle restatement "
                                          f"of the reference shaders, OpenMP on {threads} threads",
                                "passes_ms": cpu_passes}
    print(json.dumps(line), flush=True)
    if ctx is not None:
        ctx.close()


def c4_views(ctx, n_views=32, n_rooms=8, seed=4):
    """The batched 32-view workload: views of 8 seeded rooms with resolutions, VPL counts, point counts and precision
    drawn from the stated sets; interleave and ISM edge chosen by the autotuner."""
    import numpy as np

    import mlgi

    rng = np.random.default_rng(seed)
    views = []
    for v in range(n_views):
        w, h = [(854, 480), (1280, 720), (1920, 1080), (2560, 1440)][rng.integers(4)]
        n = int(rng.choice([256, 512, 1024, 2048, 4096]))
        pts = int(2 ** rng.integers(20, 24))
        reduced = bool(rng.integers(2))
        tune = ctx.autotune(w, h, n, pts, reduced=reduced, batched=True, min_vpls_per_pixel=16, min_ism_size=64,
                            seed=1000 + v % n_rooms)
        cfg = mlgi.Config(f"c4_view{v}_{w}x{h}_n{n}", w, h, 512, n, pts, tune.ism_size, tune.grid_x, tune.grid_y,
                          tune.levels, tune.interleave, 16, 8, tile=16, cull=1, reduced=reduced,
                          seed=1000 + v % n_rooms, light_yaw_deg=float(rng.uniform(-5, 5)),
                          light_pitch_deg=float(rng.uniform(-5, 5)), camera_orbit_deg=float(rng.uniform(-10, 10)))
        views.append(cfg)
    return views


def measure_batch(local_rank, n_views, steps, warmup, batch_streams):
    """Batched views (n_views views of 8 rooms), replayed from CUDA graphs in two forms -- one
    persistent launch per pass over all views (or over each of 2..4 view groups on their own
    streams), and each view's kernels spread over several streams -- against one mlgi_gi_frame per
    view on one stream. Returns the measurements as a dict."""
    import numpy as np
    import torch

    import mlgi
    from mlgi.device import Batch, DeviceFrame

    torch.cuda.set_device(local_rank)
    dev = f"cuda:{local_rank}"
    ctx = mlgi.Context(local_rank)
    t_tune = time.perf_counter()
    cfgs = c4_views(ctx, n_views=n_views)
    t_tune = time.perf_counter() - t_tune
    frames = [DeviceFrame.generated(c, dev) for c in cfgs]
    stream = torch.cuda.ExternalStream(ctx.stream(), device=dev)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]

    def timed(step):
        with torch.cuda.stream(stream):
            for _ in range(warmup):
                step()
            torch.cuda.synchronize()
            ev[0].record(stream)
            for _ in range(steps):
                step()
            ev[1].record(stream)
            torch.cuda.synchronize()
        return ev[0].elapsed_time(ev[1]) / steps

    sampler = ClockSampler(local_rank)
    sampler.start()
    forms, groups = {}, {}
    # the persistent form with 1..4 view groups (each group's passes on its own stream), the best
    # reported as "persistent"; the concurrent form on batch_streams streams
    for name, form, streams in [(f"persistent_g{g}", mlgi.BATCH_PERSISTENT, g) for g in (1, 2, 3, 4)] + \
                               [("concurrent", mlgi.BATCH_CONCURRENT, batch_streams)]:
        batch = Batch(ctx, frames, form, streams)
        ms = timed(lambda: batch.launch(ctx.stream()))
        r = {"ms_per_batch": ms, "frames_per_s": len(frames) / (ms * 1e-3), "kernel_launches": batch.kernel_launches()}
        if form == mlgi.BATCH_PERSISTENT:
            groups[streams] = dict(r, groups=streams)
        else:
            forms[name] = dict(r, streams=streams)
        batch.close()
    g_best = min(groups, key=lambda g: groups[g]["ms_per_batch"])
    forms = {"persistent": groups[g_best], **forms,
             "persistent_by_groups": {str(g): round(groups[g]["ms_per_batch"], 4) for g in groups}}
    # plain: the same views, one mlgi_gi_frame per view on one stream
    plain_ms = timed(lambda: [ctx.gi_frame(f.frame_desc(), f.radiance(), ctx.stream()) for f in frames])
    clocks = sampler.stop()
    # per-kernel device time of the plain form, summed over the views (one untimed extra pass)
    ctx.set_timing(True)
    plain_kernels = np.zeros(11)
    for f in frames:
        ctx.gi_frame(f.frame_desc(), f.radiance(), ctx.stream())
        plain_kernels += ctx.last_timings()
    ctx.set_timing(False)
    ctx.check_device_status()
    ctx.close()
    best = min(("persistent", "concurrent"), key=lambda k: forms[k]["ms_per_batch"])
    n = len(frames)
    return {"views": n, "form": best, "ms_per_batch": forms[best]["ms_per_batch"],
            "frames_per_s": n / (forms[best]["ms_per_batch"] * 1e-3), "forms": forms, "plain_ms_per_batch": plain_ms,
            "plain_frames_per_s": n / (plain_ms * 1e-3), "speedup_vs_plain": plain_ms / forms[best]["ms_per_batch"],
            "views_detail": [f"{c.width}x{c.height} N={c.n_vpl} pts=2^{int(np.log2(c.n_points))} "
                             f"I={c.interleave} ism={c.ism_size} {'fp16' if c.reduced else 'fp32'}" for c in cfgs],
            "plain_kernels_ms": {k: float(plain_kernels[i]) for k, i in
                                 [("vpl_process", 0), ("ism_clear", 1), ("ism_splat", 2), ("pull1", 7),
                                  ("pullmid", 8), ("push1", 9), ("push0 or pyramid", 10), ("final_gather", 4)]},
            "kernel_launches_per_batch": forms[best]["kernel_launches"], "steps": steps, "warmup": warmup,
            "autotune_s": t_tune, "clocks": clocks}


def run_batch(args, rank, world, local_rank):
    r = measure_batch(local_rank, args.views, args.steps, args.warmup, args.batch_streams)
    if rank == 0:
        print(json.dumps({
            "metric": f"batched GI ms per {args.views}-view batch", "value": r["ms_per_batch"], "unit": "ms/batch",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "higher_is_better": False,
            "dtype": "f32 / fp16-bf16 mixed", "data": "synthetic (seeded procedural rooms, generated on the GPU)",
            "config": {"workload": "c4_batch32", "views": r["views"], "rooms": 8, "form": r["form"],
                       "views_detail": r["views_detail"], "l2": "inputs larger than L2"},
            "frames_per_s": r["frames_per_s"], "forms": r["forms"], "plain_ms_per_batch": r["plain_ms_per_batch"],
            "plain_frames_per_s": r["plain_frames_per_s"], "speedup_vs_plain": r["speedup_vs_plain"],
            "plain_kernels_ms": r["plain_kernels_ms"],
            "gpu_launches": r["kernel_launches_per_batch"] * args.steps, "autotune_s": r["autotune_s"],
            "clocks": r["clocks"]}), flush=True)


def measure_serve(local_rank, slots, rate, duration, seed):
    """Served Poisson stream: open-loop arrivals (seeded) of frames drawn from the batched workload's
    size distribution (4 resolutions x 5 VPL counts x 4 point counts x 2 precisions), 8 rooms,
    light jitter +-5 degrees and a camera orbit step per request; served by the continuous-batching
    server, then the same request sequence through the plain arm (one frame at a time). Returns the
    measurements as a dict."""
    import numpy as np

    import mlgi
    from mlgi.serve import Server, shape_set

    shapes = shape_set()
    sv = Server(slots=slots, max_width=2560, max_height=1440, hbm_budget=150 << 30, device=local_rank)
    t = time.perf_counter()
    sv.prepare(shapes)
    t_prep = time.perf_counter() - t
    sampler = ClockSampler(local_rank)
    sampler.start()
    # warm-up: one short stream so that every room state of the run is not generated inside it
    sv.run_poisson(shapes, rate_hz=rate, duration_s=min(1.0, duration), seed=seed + 1)

    def stream(r, sd, plain):
        # nvidia-smi's utilization.gpu during the stream: the share of each sample period in which a
        # kernel ran (how busy the plain arm alone keeps the GPU)
        busy = ClockSampler(local_rank)
        busy.start()
        c, wall = sv.run_poisson(shapes, rate_hz=r, duration_s=duration, seed=sd, plain=plain)
        b = busy.stop()
        ok = c["status"] == mlgi.OK
        lat = c["latency_ms"][ok]
        return {"rate_hz": r, "requests": int(len(c)), "ok": int(ok.sum()), "wall_s": wall,
                "frames_per_s": float(ok.sum() / wall), "p50_ms": float(np.percentile(lat, 50)),
                "p99_ms": float(np.percentile(lat, 99)), "mean_queue_ms": float(c["queue_ms"][ok].mean()),
                "gpu_busy_pct": b.get("gpu_busy_pct") if b else None,
                "digests": {int(i): int(d) for i, d in zip(c["id"], c["digest"])}}

    runs = {"served": stream(rate, seed, False), "plain": stream(rate, seed, True)}
    # the same kind of stream at 75% of the served capacity just measured: latency below saturation
    rate75 = 0.75 * runs["served"]["frames_per_s"]
    runs["served_at_75pct"] = stream(rate75, seed + 3, False)
    runs["plain_at_75pct"] = stream(rate75, seed + 3, True)
    clocks = sampler.stop()
    st = sv.stats()
    # single-frame latency: the plain arm at a rate it sustains (10% of its throughput)
    light_rate = max(1.0, 0.1 * runs["plain"]["frames_per_s"])
    c1, _ = sv.run_poisson(shapes, rate_hz=light_rate, duration_s=duration, seed=seed + 2, plain=True)
    single = c1["latency_ms"][c1["status"] == mlgi.OK]
    sv.close()
    same = (runs["served"]["digests"] == runs["plain"]["digests"]
            and runs["served_at_75pct"]["digests"] == runs["plain_at_75pct"]["digests"])
    for r in runs.values():
        r.pop("digests")
    return {**runs, "speedup_vs_plain": runs["served"]["frames_per_s"] / runs["plain"]["frames_per_s"],
            "single_frame_ms": {"p50": float(np.percentile(single, 50)), "p99": float(np.percentile(single, 99)),
                                "rate_hz": light_rate},
            "results_identical_served_vs_plain": same, "prepare_s": t_prep, "server_stats": st,
            "config": {"rate_hz": rate, "duration_s": duration, "seed": seed, "rooms": 8, "shapes": len(shapes),
                       "slots": slots, "hbm_budget_gb": 150, "light_jitter_deg": 5, "orbit_step_deg": 0.5},
            "clocks": clocks}


def run_serve(args, rank, world, local_rank):
    r = measure_serve(local_rank, args.slots, args.rate, args.duration, args.seed)
    if rank == 0:
        cfg = r.pop("config")
        print(json.dumps({
            "metric": "served GI frames/s", "value": r["served"]["frames_per_s"], "unit": "frames/s",
            "n_gpus": world, "steps": r["served"]["requests"], "warmup": 1, "higher_is_better": True,
            "dtype": "f32 / fp16-bf16 mixed", "data": "synthetic (seeded procedural rooms, generated on the GPU)",
            "config": {"workload": "c5_served_poisson", **cfg}, **r}), flush=True)


def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    import mlgi

    cfg = mlgi.CONFIGS.get(args.config, mlgi.C2)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("gloo")
    try:
        if args.impl == "reference":
            run_reference(args, cfg, rank, world)
        elif args.config == "c4_batch32":
            run_batch(args, rank, world, local_rank)
        elif args.config == "c5_served":
            run_serve(args, rank, world, local_rank)
        else:
            run_gpu(args, cfg, rank, world, local_rank)
    finally:
        if world > 1:
            import torch.distributed as dist

            dist.destroy_process_group()


if __name__ == "__main__":
    main()
