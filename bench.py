"""Benchmark of the GB300 ray-tracing core.

Headline workload: the procedural terrain (1025x1025 diamond-square
heightfield, 2,097,152 triangles) at 1920x1080, one primary ray per pixel
plus one directional-sun shadow ray per hit, coloured Phong, RGB8 output.
A step is one frame through the fused render kernel.  Metric: Mrays/s
(primary + shadow rays per second, whole job).

  value  device-resident throughput: scene and hierarchy in HBM, output to
         a device buffer, CUDA events on the launching stream around each
         frame; the L2 is flushed (a 512 MB write) between frames.
  e2e    the same frame through the C ABI with a pinned HOST output buffer:
         camera/light/material structs in, RGB8 out (device-to-host copy
         inside the timed region), wall clock per call.

`--impl reference` times the reference's CPU path on the host cores: the
reference itself when it was compiled here (oracle/_ref), else the oracle's
C restatement, on a bounded band of rows per step with all host threads.

Multi-GPU (torchrun, N > 1): every rank renders its own replica of the
frame (no data-path collective; "replicas only"); value = all ranks' rays /
max-over-ranks time.
"""
from __future__ import annotations

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

METRIC = "Mrays/s (primary+shadow, 1 GB300)"
WORKLOAD = "terrain-2M-1080p"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=12.0, help="budget of the CPU baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-workloads", action="store_true", help="headline workload only")
    ap.add_argument("--size", type=int, default=1024, help="terrain cells per side (power of two)")
    ap.add_argument("--only", default=None, choices=sorted(WORKLOADS),
                    help="run one extra workload alone and print its JSON (for profiling)")
    return ap.parse_args()


def make_workload(size):
    from raptor_gb300 import scenes
    return scenes.terrain_scene(size_pow2=size)


# ------------------------------------------------------------------ clocks

class ClockSampler:
    """nvidia-smi samples (SM clock, max clock, power, throttle reasons)
    during the timed region."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, pw, reasons = [], [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx.append(float(p[2]))
                pw.append(float(p[3]))
            except ValueError:
                continue
            for nm, val in zip(names, p[5:9]):
                if val.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "power_w_max": float(max(pw)),
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------ CPU baseline

class CpuBaseline:
    """The reference's CPU path on this host's cores.  The reference itself
    (oracle/_ref) builds only on x86-64 (its simd.h includes immintrin.h), so
    on an Arm host this is the oracle's C restatement (kind "port"),
    which the tests pin to the reference's outputs.  The hierarchy is built
    once; each step renders a band of rows sized to `seconds` of work with
    all host threads."""

    def __init__(self, scene, frame, threads=None):
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as O
        if not os.path.exists(O.ORACLE_SO):
            O.build()
        self.threads = threads or os.cpu_count() or 1
        self.frame = frame
        t0 = time.perf_counter()
        self.scene = O.OracleScene(scene)
        self.build_s = time.perf_counter() - t0
        self.H = frame["camera"]["yres"]
        self.next_row = 0
        self.rows_per_s = None

    def step(self, seconds):
        if self.rows_per_s is None:   # probe 8 rows
            t = time.perf_counter()
            self.scene.render(self.frame, rows=(self.H // 2, self.H // 2 + 8), threads=self.threads)
            self.rows_per_s = 8 / max(time.perf_counter() - t, 1e-6)
        rows = int(max(8, min(self.H, seconds * self.rows_per_s)))
        r0 = self.next_row % self.H
        r1 = min(self.H, r0 + rows)
        self.next_row = r1 % self.H
        t = time.perf_counter()
        out = self.scene.render(self.frame, rows=(r0, r1), threads=self.threads)
        dt = time.perf_counter() - t
        self.last = {"rows": (r0, r1), "rays": int(out["rays"]), "seconds": dt}
        return out["rays"] / dt / 1e6

    def describe(self):
        r0, r1 = self.last["rows"]
        return {"cores": self.threads, "kind": "port",
                "sample": f"rows {r0}..{r1} of {self.H} ({self.last['rays']} rays) of the same frame per step; "
                          f"C restatement of bvh traversal + ray_trace_engine::ray_trace + coloured_mapper_shader "
                          f"(pinned to the reference's outputs); hierarchy build {self.build_s:.2f} s excluded"}


def cpu_baseline(scene, frame, seconds, threads=None):
    """One bounded sample of the CPU baseline (see CpuBaseline)."""
    cb = CpuBaseline(scene, frame, threads)
    v = cb.step(seconds)
    return dict(value=v, unit="Mrays/s", **cb.describe())


# --------------------------------------------------------------- distributed

def dist_init(n):
    if n <= 1 or "RANK" not in os.environ:
        return 0, 1
    import torch.distributed as dist
    dist.init_process_group("nccl")
    return dist.get_rank(), dist.get_world_size()


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, world, device="cuda"):
    """Max of a per-rank scalar over all ranks (NCCL on GPUs, gloo on CPU)."""
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_rate(rays_per_rank, max_seconds, world):
    """Whole-job Mrays/s: every rank traced rays_per_rank rays (its own
    replica); the job takes as long as the slowest rank."""
    return rays_per_rank * world / max_seconds / 1e6


# -------------------------------------------------------------------- main

def run_reference(args):
    """--impl reference: the reference's CPU path on all host cores, each
    step a bounded band of the same frame (rank 0 only)."""
    rank, world = dist_init(args.gpus)
    if rank != 0:
        return
    scene, frame = make_workload(args.size)
    cb = CpuBaseline(scene, frame)
    per_step = max(0.5, args.cpu_seconds / max(1, args.steps))
    for _ in range(args.warmup):
        cb.step(per_step / 2)
    rays = secs = 0.0
    for _ in range(args.steps):
        cb.step(per_step)
        rays += cb.last["rays"]
        secs += cb.last["seconds"]
    v = rays / secs / 1e6
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "Mrays/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": secs / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded diamond-square terrain, slope colours)",
            "config": {"workload": WORKLOAD, "triangles": int(scene["tris"].shape[0]), "resolution": [1920, 1080],
                       "rays": "primary + 1 directional shadow ray per hit"},
            "cpu_baseline": dict(value=v, unit="Mrays/s", **cb.describe()),
            "e2e": {"value": v, "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


NCU_SUMMARY = os.path.join(ROOT, "profiles", "k_render_terrain-2M-1080p_ncu.md")


def ncu_metric_sum(names):
    """Sum of byte counters of one k_render launch on this workload, from the
    committed ncu summary (a capture cannot run inside the timed bench), or
    None when any is missing."""
    scale = {"byte": 1.0, "Kbyte": 1e3, "Mbyte": 1e6, "Gbyte": 1e9}
    total, seen = 0.0, 0
    try:
        for line in open(NCU_SUMMARY):
            for name in names:
                if line.startswith(f"| `{name}` |"):
                    value, unit = line.split("|")[2].split()
                    total += float(value) * scale[unit]
                    seen += 1
    except (OSError, ValueError, KeyError):
        return None
    return total if seen == len(names) else None


def ncu_traffic():
    """DRAM bytes (read + write) of one k_render launch."""
    return ncu_metric_sum(("dram__bytes_read.sum", "dram__bytes_write.sum"))


def l2_copy_peak(stream):
    """L2-resident copy bandwidth measured here (GB/s, bytes read + bytes
    written): two 24 MB buffers, far inside the 129 MB L2, copied back and
    forth 64 times in one CUDA graph (a single copy lasts only microseconds,
    so separate launches would measure their own gaps), best of 10 replays
    -- the L2 counterpart of the HBM copy figure the roofline uses."""
    import torch
    n = 24 * 1024 * 1024 // 4
    a = torch.ones(n, dtype=torch.float32, device="cuda")
    b = torch.empty_like(a)
    reps = 64
    with torch.cuda.stream(stream):
        for _ in range(3):
            b.copy_(a)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=stream):
            for k in range(reps):
                (b if k % 2 == 0 else a).copy_(a if k % 2 == 0 else b)
        g.replay()
        best = float("inf")
        for _ in range(10):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            g.replay()
            e1.record(stream)
            e1.synchronize()
            best = min(best, e0.elapsed_time(e1) / reps)
    del g, a, b
    return 2 * n * 4 / (best / 1e3) / 1e9


# The extra workloads by name: (function, uses the L2 flush, steps from --steps).
WORKLOADS = {
    "icosphere-20k-512": ("workload_icosphere", True, lambda k: max(5, k)),
    "icosphere-20k-512-mirror": ("workload_icosphere_mirror", True, lambda k: max(5, k)),
    "glass-41k-512": ("workload_glass", True, lambda k: max(5, k)),
    "terrain-2M-1080p-tonemap": ("workload_terrain_tonemap", True, lambda k: max(3, k // 4)),
    "terrain-2M-ingest-ply": ("workload_ingest", False, lambda k: 3),
    "terrain-1M-1080p": ("workload_terrain_1m", True, lambda k: max(5, k // 2)),
    "terrain-2M-1080p-aa2x2": ("workload_terrain_aa", True, lambda k: max(3, k // 4)),
    "terrain-2M-1080p-soft16": ("workload_terrain_soft", True, lambda k: max(3, k // 4)),
    "glass-41k-512-soft16": ("workload_glass_soft", True, lambda k: max(3, k // 4)),
    "glass-41k-512-diffuse16": ("workload_glass_diffuse", True, lambda k: max(3, k // 4)),
    "instances-4M-720p-ao16": ("workload_instances_ao", True, lambda k: max(3, k // 4)),
    "batched-64-scenes": ("workload_batched", False, lambda k: max(3, k // 4)),
    "adjoint-50k-256": ("workload_adjoint", False, lambda k: max(5, k // 2)),
}


def run_one_workload(args):
    """--only NAME: one extra workload on its own (rank 0, one GPU)."""
    import torch
    from raptor_gb300 import core
    torch.cuda.set_device(0)
    ctx = core.Context(0)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx.set_stream(stream.cuda_stream)
    fn_name, flushed, steps = WORKLOADS[args.only]
    fn = globals()[fn_name]
    if flushed:
        flush = torch.empty(128 * 1024 * 1024, dtype=torch.float32, device="cuda")
        out = fn(ctx, stream, flush, steps(args.steps))
    else:
        out = fn(ctx, stream, steps(args.steps))
    print(json.dumps({"workload": args.only, **out}), flush=True)
    ctx.close()


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.only:
        return run_one_workload(args)
    import torch
    from raptor_gb300 import core
    rank, world = dist_init(args.gpus)
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(ROOT, "MEASURED_PEAKS.json")) else None
    hbm_peak = peaks["hbm_gbs"] if peaks else 6800.0
    peak_src = "measured" if peaks else "fallback"

    scene, frame = make_workload(args.size)
    cam = frame["camera"]
    W, H = cam["xres"], cam["yres"]
    ctx = core.Context(local)
    # a dedicated (non-default) stream, current for torch too: the L2 flush,
    # the CUDA events and the library's kernels are ordered on it
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx.set_stream(stream.cuda_stream)
    sc = core.Scene(ctx, scene)
    build_ms = sc.build()
    build_ms = min(build_ms, sc.build())   # second build: warm
    info = sc.info()

    rgb_dev = torch.empty((H, W, 3), dtype=torch.uint8, device="cuda")
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    # fetch counts for the roofline (instrumented kernel, outside the timed region)
    ctx.set_option(core.RT_OPT_COUNT_FETCHES, 1)
    cnt = sc.render(frame, rgb=rgb_dev)["stats"]
    ctx.set_option(core.RT_OPT_COUNT_FETCHES, 0)
    nodes_per_frame, tris_per_frame = cnt.nodes_fetched, cnt.tris_tested

    for _ in range(args.warmup):
        sc.render(frame, rgb=rgb_dev)
    torch.cuda.synchronize()
    barrier(world)
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    rays = 0
    kernel_ms = []
    barrier(world)
    torch.cuda.synchronize()
    for i in range(args.steps):
        flush.fill_(float(i))
        ev[i][0].record(stream)
        st = sc.render(frame, rgb=rgb_dev)["stats"]
        ev[i][1].record(stream)
        rays += st.primary_rays + st.secondary_rays
        kernel_ms.append(st.device_ms)
    torch.cuda.synchronize()
    barrier(world)
    step_ms = [a.elapsed_time(b) for a, b in ev]
    total_s = sum(step_ms) / 1e3
    total_s = max_over_ranks(total_s, world)
    value = aggregate_rate(rays, total_s, world)

    # e2e: the C ABI's rt_render with a pinned host output buffer (the call a
    # C or C++ caller makes: arguments built once), wall clock per call
    rgb_host = torch.empty((H, W, 3), dtype=torch.uint8).pin_memory()
    c_cam, c_lights = core.make_camera(frame["camera"]), core.make_lights(frame["lights"])
    c_mat, c_stats = core.make_material(frame["material"]), core.RtRenderStats()
    c_out = core.ptr(rgb_host)
    render_fn = core.lib().rt_render
    e2e_rays = 0
    torch.cuda.synchronize()
    barrier(world)
    t0 = time.perf_counter()
    for i in range(args.steps):
        rc = render_fn(sc.h, ctypes.byref(c_cam), c_lights, len(frame["lights"]), ctypes.byref(c_mat), c_out, None,
                       ctypes.byref(c_stats))
        if rc != 0:
            raise core.RtError(rc, core.lib().rt_last_error_string().decode())
        e2e_rays += c_stats.primary_rays + c_stats.secondary_rays
    e2e_s = max_over_ranks(time.perf_counter() - t0, world)
    clk = clocks.stop()
    e2e = aggregate_rate(e2e_rays, e2e_s, world)
    h2d = C_sizes()
    mean_kernel_ms = float(np.mean(kernel_ms))
    frame_rays = rays / args.steps
    # algorithmic bytes per frame: nodes fetched x 80 B + triangles tested x
    # 48 B + shading records (per hit: 32 B shade + 12 B indices + 36 B
    # attributes) + RGB8 output
    hits = st.primary_hits
    alg_bytes = nodes_per_frame * 80 + tris_per_frame * 48 + hits * (32 + 12 + 36) + W * H * 3
    achieved = alg_bytes / (mean_kernel_ms / 1e3) / 1e9
    # L2-referenced view: coherent rays re-read the upper tree levels from
    # L1/L2, so the same algorithmic bytes and the L2 traffic ncu counted
    # are set against the measured L2 copy bandwidth too
    l2_peak = l2_copy_peak(stream)
    l2_traffic = ncu_metric_sum(("lts__t_bytes.sum",)) if args.size == 1024 else None
    l2 = {"peak": l2_peak, "unit": "GB/s", "peak_source": "measured in this run (L2-resident copy)",
          "achieved": achieved, "frac": achieved / l2_peak, "traffic": l2_traffic,
          "traffic_gbs": l2_traffic / (mean_kernel_ms / 1e3) / 1e9 if l2_traffic else None,
          "traffic_frac": l2_traffic / (mean_kernel_ms / 1e3) / 1e9 / l2_peak if l2_traffic else None,
          "traffic_source": "lts__t_bytes.sum of the same launch in profiles/k_render_terrain-2M-1080p_ncu.md"}

    line = {"metric": METRIC, "value": value, "unit": "Mrays/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": float(np.mean(step_ms)), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded diamond-square terrain, slope colours)",
            "config": {"workload": WORKLOAD, "triangles": int(scene["tris"].shape[0]), "resolution": [W, H],
                       "rays": "primary + 1 directional shadow ray per hit", "rays_per_frame": frame_rays,
                       "l2": "flushed between frames (512 MB write)", "parallelism": f"replicas x{world}",
                       "bvh": info, "bvh_build_ms": build_ms},
            "e2e": {"value": e2e, "unit": "Mrays/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": W * H * 3},
            "gpu_launches": args.steps,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                         "frac": achieved / hbm_peak,
                         "traffic": ncu_traffic() if args.size == 1024 else None,
                         "traffic_source": "profiles/k_render_terrain-2M-1080p_ncu.md (one launch, ncu --set full)",
                         "kernel": "k_render<false>", "peak_source": peak_src,
                         "bytes_per_frame": alg_bytes, "nodes_per_ray": nodes_per_frame / frame_rays,
                         "tris_per_ray": tris_per_frame / frame_rays, "kernel_ms": mean_kernel_ms, "l2": l2},
            "clocks": clk}
    if not args.no_workloads:
        sc.close()
        wl = {}
        for name, (fn_name, flushed, steps) in WORKLOADS.items():
            if flushed:
                wl[name] = globals()[fn_name](ctx, stream, flush, steps(args.steps))
        del flush
        torch.cuda.empty_cache()
        for name, (fn_name, flushed, steps) in WORKLOADS.items():
            if not flushed:
                wl[name] = globals()[fn_name](ctx, stream, steps(args.steps))
        line["workloads"] = wl
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = {k: v for k, v in cpu_baseline(scene, frame, args.cpu_seconds).items()
                                if k != "build_seconds"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    sc.close()
    ctx.close()


def time_frames(fn, steps, stream, flush=None):
    """Sum of CUDA-event times of `steps` calls of fn() on `stream`, the L2
    flushed before each when `flush` is given.  Returns (seconds, last)."""
    import torch
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    last = None
    for i in range(steps):
        if flush is not None:
            flush.fill_(float(i))
        evs[i][0].record(stream)
        last = fn()
        evs[i][1].record(stream)
    torch.cuda.synchronize()
    return sum(a.elapsed_time(b) for a, b in evs) / 1e3, last


def workload_icosphere(ctx, stream, flush, steps):
    """Icosphere 20,480 + 2 ground triangles, 512x512, primary + point-light shadow."""
    import torch
    from raptor_gb300 import core, scenes
    scene, frame = scenes.icosphere_scene()
    sc = core.Scene(ctx, scene)
    rgb = torch.empty((512, 512, 3), dtype=torch.uint8, device="cuda")
    for _ in range(3):
        sc.render(frame, rgb=rgb)
    secs, st = time_frames(lambda: sc.render(frame, rgb=rgb)["stats"], steps, stream, flush)
    rays = (st.primary_rays + st.secondary_rays) * steps
    sc.close()
    return {"triangles": int(scene["tris"].shape[0]), "resolution": [512, 512], "Mrays_s": rays / secs / 1e6,
            "ms_per_frame": secs / steps * 1e3, "rays_per_frame": rays / steps}


def workload_terrain_aa(ctx, stream, flush, steps):
    """The headline terrain at 1920x1080 output with 2x2 anti-aliasing (the
    camera's x_a_res / y_a_res): 4 primary rays + shadow rays per output
    pixel, averaged into RGB8 in the same kernel."""
    import torch
    from raptor_gb300 import core, scenes
    scene, frame = scenes.terrain_scene()
    sc = core.Scene(ctx, scene)
    rgb = torch.empty((1080, 1920, 3), dtype=torch.uint8, device="cuda")
    for _ in range(3):
        sc.render_aa(frame, 2, 2, rgb=rgb)
    secs, st = time_frames(lambda: sc.render_aa(frame, 2, 2, rgb=rgb)["stats"], steps, stream, flush)
    rays = (st.primary_rays + st.secondary_rays) * steps
    sc.close()
    return {"triangles": int(scene["tris"].shape[0]), "resolution": [1920, 1080], "aa": [2, 2],
            "Mrays_s": rays / secs / 1e6, "ms_per_frame": secs / steps * 1e3, "rays_per_frame": rays / steps}


def workload_icosphere_mirror(ctx, stream, flush, steps):
    """The icosphere frame with a reflective material (rf 0.5: the camera
    ray and up to three mirror bounces per pixel, each with its shadow ray)."""
    import torch
    from raptor_gb300 import core, scenes
    scene, frame = scenes.icosphere_scene()
    frame = dict(frame, material=dict(frame["material"], rf=0.5))
    sc = core.Scene(ctx, scene)
    rgb = torch.empty((512, 512, 3), dtype=torch.uint8, device="cuda")
    for _ in range(3):
        sc.render(frame, rgb=rgb)
    secs, st = time_frames(lambda: sc.render(frame, rgb=rgb)["stats"], steps, stream, flush)
    rays = (st.primary_rays + st.secondary_rays) * steps
    sc.close()
    return {"triangles": int(scene["tris"].shape[0]), "resolution": [512, 512], "rf": 0.5,
            "Mrays_s": rays / secs / 1e6, "ms_per_frame": secs / steps * 1e3, "rays_per_frame": rays / steps}


def workload_glass(ctx, stream, flush, steps):
    """Per-triangle materials with refraction: a glass sphere (tran 0.6, ri
    1.5, rf 0.2) before an opaque sphere on a reflective ground (rf 0.3),
    20,480 triangles per sphere, 512x512, two lights; each pixel's ray tree
    of mirror and refracted rays, every hit with its shadow rays."""
    import torch
    from raptor_gb300 import core, scenes
    scene, frame = scenes.glass_scene(freq=32, res=512)
    sc = core.Scene(ctx, scene)
    rgb = torch.empty((512, 512, 3), dtype=torch.uint8, device="cuda")
    for _ in range(3):
        sc.render(frame, rgb=rgb)
    secs, st = time_frames(lambda: sc.render(frame, rgb=rgb)["stats"], steps, stream, flush)
    rays = (st.primary_rays + st.secondary_rays) * steps
    sc.close()
    return {"triangles": int(scene["tris"].shape[0]), "resolution": [512, 512],
            "Mrays_s": rays / secs / 1e6, "ms_per_frame": secs / steps * 1e3, "rays_per_frame": rays / steps}


def _glass_distributed(ctx, stream, flush, steps, diffuse):
    import torch
    from raptor_gb300 import core, scenes
    scene, frame = scenes.glass_scene(freq=32, res=512)
    frame = dict(frame, lights=[dict(frame["lights"][0], r=0.7), frame["lights"][1]])
    if diffuse:
        mats = [dict(frame["materials"][0], rfd=0.2), dict(frame["materials"][1], rfd=0.1, td=0.05)]
        frame = dict(frame, materials=mats, material=mats[0])
        kw = {"soft": 16, "diffuse": 16, "stream": core.RT_STREAM_PIXEL, "seed": 1}
    else:
        kw = {"soft": 16, "stream": core.RT_STREAM_REFERENCE, "offset": 0}
    sc = core.Scene(ctx, scene)
    rgb = torch.empty((512, 512, 3), dtype=torch.uint8, device="cuda")
    for _ in range(3):
        first = sc.render_distributed(frame, rgb=rgb, **kw)
    secs, st = time_frames(lambda: sc.render_distributed(frame, rgb=rgb, **kw)["stats"], steps, stream, flush)
    rays = st.primary_rays + st.secondary_rays
    sc.close()
    return {"triangles": int(scene["tris"].shape[0]), "resolution": [512, 512], "soft_samples": 16,
            "diffuse_samples": 16 if diffuse else 0, "stream": "pixel" if diffuse else "reference",
            "Mrays_s": rays * steps / secs / 1e6, "ms_per_frame": secs / steps * 1e3, "rays_per_frame": rays,
            "numbers_per_frame": first["stream_end"]}


def workload_glass_soft(ctx, stream, flush, steps):
    """The glass scene (refraction and mirror ray trees, 41k triangles,
    512x512) with soft shadows as the SOFT_SHADOW = 16 build renders them:
    16 rays to the spherical light (radius 0.7) at every hit of every tree
    ray, numbers from the reference's stream (counting pass, scan, shading
    pass; the slice already on the device)."""
    return _glass_distributed(ctx, stream, flush, steps, False)


def workload_glass_diffuse(ctx, stream, flush, steps):
    """The glass scene with diffuse reflections and refractions
    (DIFFUSE_REFLECTIONS = 16: 16 spread rays per reflection of a camera
    ray's hit, 4 at the next level, then 1; ground rfd 0.2, glass rfd 0.1
    and td 0.05) and 16 soft-shadow samples, per-pixel streams."""
    return _glass_distributed(ctx, stream, flush, steps, True)


def workload_ingest(ctx, stream, steps):
    """Scene ingest of the headline terrain (2,097,152 triangles) from a
    40 MB big-endian binary PLY held in host memory: rt_mesh_parse (host),
    then rt_scene_upload + rt_bvh_build (device); wall-clock, best of
    `steps`."""
    import time
    import numpy as np
    import torch
    from raptor_gb300 import core, scenes
    scene, _ = scenes.terrain_scene()
    v, t = scene["verts"], scene["tris"]
    hdr = ["ply", "format binary_big_endian 1.0", f"element vertex {len(v)}", "property float x",
           "property float y", "property float z", f"element face {len(t)}",
           "property list uchar int vertex_indices", "end_header"]
    faces = np.zeros(len(t), dtype=[("n", "u1"), ("i", ">i4", (3,))])
    faces["n"] = 3
    faces["i"] = t
    data = ("\n".join(hdr) + "\n").encode() + v.astype(">f4").tobytes() + faces.tobytes()
    best_parse = best_build = float("inf")
    for _ in range(steps):
        t0 = time.perf_counter()
        m = core.parse_mesh(data, core.RT_MESH_PLY)
        t1 = time.perf_counter()
        sc = core.Scene(ctx, m)
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        sc.close()
        best_parse = min(best_parse, t1 - t0)
        best_build = min(best_build, t2 - t1)
    assert m["tris"].shape[0] == t.shape[0]
    return {"triangles": int(t.shape[0]), "file_mb": len(data) / 1e6, "parse_ms": best_parse * 1e3,
            "upload_build_ms": best_build * 1e3, "parse_mb_s": len(data) / 1e6 / best_parse}


def workload_terrain_tonemap(ctx, stream, flush, steps):
    """The headline terrain frame (2,097,152 triangles, 1920x1080) through the
    framebuffer epilogue: float frame, exposure tone mapping (key 0.18) and
    sRGB gamma, then RGB8; the plain frame beside it; and the bilateral
    tone mapper with sRGB gamma (its grid, exact Gaussian blur by Fourier
    transforms in double, slice and compression)."""
    import torch
    from raptor_gb300 import core, scenes
    scene, frame = scenes.terrain_scene()
    sc = core.Scene(ctx, scene)
    rgb = torch.empty((1080, 1920, 3), dtype=torch.uint8, device="cuda")
    tone = {"mode": 5, "gamma": 2.2}
    out = {"triangles": int(scene["tris"].shape[0]), "resolution": [1920, 1080], "tone": tone}
    bil = {"mode": 8, "gamma": 2.2}
    for key, fn in (("plain", lambda: sc.render(frame, rgb=rgb)["stats"]),
                    ("tone_mapped", lambda: sc.render_tone_mapped(frame, tone, rgb=rgb)["stats"]),
                    ("bilateral", lambda: sc.render_tone_mapped(frame, bil, rgb=rgb)["stats"])):
        for _ in range(3):
            fn()
        secs, st = time_frames(fn, steps, stream, flush)
        out[key] = {"ms_per_frame": secs / steps * 1e3,
                    "Grays_s": (st.primary_rays + st.secondary_rays) * steps / secs / 1e9}
    sc.close()
    return out


def workload_terrain_1m(ctx, stream, flush, steps):
    """The 1,048,352-triangle terrain (725^2 vertices), 1920x1080: primary
    rays alone (no light) and primary + sun shadow rays."""
    import torch
    from raptor_gb300 import core, scenes
    scene, frame = scenes.terrain_scene(crop=725)
    sc = core.Scene(ctx, scene)
    rgb = torch.empty((1080, 1920, 3), dtype=torch.uint8, device="cuda")
    prim = dict(frame, lights=[])
    out = {"triangles": int(scene["tris"].shape[0]), "resolution": [1920, 1080]}
    for key, fr in (("primary_only", prim), ("primary_shadow", frame)):
        for _ in range(3):
            sc.render(fr, rgb=rgb)
        secs, st = time_frames(lambda: sc.render(fr, rgb=rgb)["stats"], steps, stream, flush)
        out[key] = {"Grays_s": (st.primary_rays + st.secondary_rays) * steps / secs / 1e9,
                    "ms_per_frame": secs / steps * 1e3, "primary_rays": st.primary_rays,
                    "secondary_rays": st.secondary_rays}
    sc.close()
    return out


def workload_terrain_soft(ctx, stream, flush, steps):
    """The headline terrain at 1920x1080 with soft shadows as the reference
    renders them with SOFT_SHADOW = 16: a spherical light (radius 40) beside
    the sun, 16 rays to the spherical light and one to the sun per hit, the
    random points from the reference's stream.  Frame time with the frame's
    slice of the stream already on the device (the same stream position
    every step); the wall time of the first frame (its slice generated on
    the host, then copied over); and the mean wall time of consecutive frames,
    each starting where the last one's numbers ended, as an animation draws
    them (each frame's slice generated on the host while the one before it
    renders)."""
    import torch
    from raptor_gb300 import core, scenes
    scene, frame = scenes.terrain_scene()
    frame = dict(frame, lights=[dict(scenes.point_light((300.0, 260.0, 500.0)), r=40.0), frame["lights"][0]])
    sc = core.Scene(ctx, scene)
    rgb = torch.empty((1080, 1920, 3), dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    first = sc.render_soft(frame, 16, 0, rgb=rgb)
    first_s = time.perf_counter() - t0
    for _ in range(2):
        sc.render_soft(frame, 16, 0, rgb=rgb)
    secs, st = time_frames(lambda: sc.render_soft(frame, 16, 0, rgb=rgb)["stats"], steps, stream, flush)
    # consecutive positions; the first of them was read ahead during the
    # frames above and is not counted
    pos = sc.render_soft(frame, 16, first["stream_end"], rgb=rgb)["stream_end"]
    torch.cuda.synchronize()
    n_consec = 5
    t0 = time.perf_counter()
    for _ in range(n_consec):
        pos = sc.render_soft(frame, 16, pos, rgb=rgb)["stream_end"]
    consec_s = (time.perf_counter() - t0) / n_consec
    sc.close()
    rays = st.primary_rays + st.secondary_rays
    return {"triangles": int(scene["tris"].shape[0]), "resolution": [1920, 1080], "samples": 16,
            "Mrays_s": rays * steps / secs / 1e6, "ms_per_frame": secs / steps * 1e3, "rays_per_frame": rays,
            "stream_numbers_per_frame": first["stream_end"],
            "ms_first_frame": first_s * 1e3, "ms_per_frame_consecutive_stream": consec_s * 1e3}


def workload_adjoint(ctx, stream, steps):
    """Differentiable render: 50,000-triangle displaced sphere at 256x256,
    primary + shadow; float forward vs hand-written adjoint, ms per frame."""
    import torch
    from raptor_gb300 import core, scenes
    scene, target_scene, frame = scenes.adjoint_scene()
    sc = core.Scene(ctx, scene)
    H, W = frame["camera"]["yres"], frame["camera"]["xres"]
    img = torch.empty((H, W, 3), dtype=torch.float32, device="cuda")
    dl = torch.randn((H, W, 3), dtype=torch.float32, device="cuda")
    gp = torch.empty((scene["verts"].shape[0], 3), dtype=torch.float32, device="cuda")
    gc = torch.empty_like(gp)
    for _ in range(3):
        sc.render_float(frame, img)
        sc.render_adjoint(frame, dl, gp, gc)
    fwd, _ = time_frames(lambda: sc.render_float(frame, img), steps, stream)
    adj, _ = time_frames(lambda: sc.render_adjoint(frame, dl, gp, gc), steps, stream)
    sc.close()
    return {"triangles": int(scene["tris"].shape[0]), "resolution": [W, H], "forward_ms": fwd / steps * 1e3,
            "adjoint_ms": adj / steps * 1e3, "adjoint_over_forward": adj / fwd}


def workload_instances_ao(ctx, stream, flush, steps):
    """2,000 instances x 2,000 triangles (4 M), 1280x720, 16 AO rays per hit
    within distance 5 (any-hit)."""
    import torch
    from raptor_gb300 import core, scenes
    scene, frame = scenes.instances_scene()
    sc = core.Scene(ctx, scene)
    rgb = torch.empty((720, 1280, 3), dtype=torch.uint8, device="cuda")
    for _ in range(2):
        sc.render(frame, rgb=rgb)
    secs, st = time_frames(lambda: sc.render(frame, rgb=rgb)["stats"], steps, stream, flush)
    rays = (st.primary_rays + st.secondary_rays) * steps
    out = {"triangles": int(scene["tris"].shape[0]), "resolution": [1280, 720], "Mrays_s": rays / secs / 1e6,
           "ms_per_frame": secs / steps * 1e3, "primary_rays": st.primary_rays, "ao_rays": st.secondary_rays,
           "bvh_build_ms": sc.build_ms}
    sc.close()
    return out


def workload_batched(ctx, stream, steps):
    """64 scenes (icosphere or heightfield, 1k-500k triangles log-uniform,
    resolutions 128^2 .. 1920x1080, primary+shadow or primary+4 AO): the
    plain form (one rt_render / rt_render_ao call per scene-frame) against
    the batched form (one graph-captured persistent launch, autotuned)."""
    import torch
    from raptor_gb300 import core, scenes
    items = scenes.batched_scenes()
    b = core.Batch(ctx)
    idx = [b.add_scene(sc) for sc, _ in items]
    build_ms = b.build()
    bufs = [torch.empty((fr["camera"]["yres"], fr["camera"]["xres"], 3), dtype=torch.uint8, device="cuda")
            for _, fr in items]
    b.set_jobs([core.make_job(i, fr, buf) for i, (_, fr), buf in zip(idx, items, bufs)])
    tune = b.autotune(reps=2)
    for _ in range(2):
        b.render(stats=False)
    secs_b, st = time_frames(lambda: b.render(stats=True), steps, stream)
    rays = st.primary_rays + st.secondary_rays
    # plain: one scene per call, each built on its own
    plain = [core.Scene(ctx, sc) for sc, _ in items]

    def plain_frame():
        for s, (_, fr), buf in zip(plain, items, bufs):
            s.render(fr, rgb=buf)
    for _ in range(2):
        plain_frame()
    secs_p, _ = time_frames(plain_frame, steps, stream)
    for s in plain:
        s.close()
    b.close()
    return {"scenes": len(items), "triangles": int(sum(sc["tris"].shape[0] for sc, _ in items)),
            "pixels": int(sum(fr["camera"]["xres"] * fr["camera"]["yres"] for _, fr in items)),
            "rays_per_frame": rays, "batched_Mrays_s": rays * steps / secs_b / 1e6,
            "plain_Mrays_s": rays * steps / secs_p / 1e6, "batched_ms": secs_b / steps * 1e3,
            "plain_ms": secs_p / steps * 1e3, "speedup": secs_p / secs_b, "autotune": tune,
            "batched_build_ms": build_ms}


def C_sizes():
    """Bytes of the per-frame inputs handed to the device: camera, one light
    and the material, passed by value as kernel parameters."""
    from raptor_gb300 import core
    import ctypes
    return ctypes.sizeof(core.RtCamera) + ctypes.sizeof(core.RtLight) + ctypes.sizeof(core.RtMaterial)


if __name__ == "__main__":
    main()
