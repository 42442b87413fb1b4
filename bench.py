#!/usr/bin/env python3
"""Benchmark of the light-probe bake on GB300.

Workload (one "step"): bake the 16x16x16 probe grid of the 64-box scene (778
triangles, open unit room, seeded sun + 128^2 cubemap sky) with 256 shared
Fibonacci directions per probe, L2 SH -- 1,048,576 primary rays plus the sun
shadow rays.  The chosen path (fused trace + projection, FP32) is timed with
inputs resident in HBM; the plain FP32 path (radiance tile + projection, the
drop-in) is timed beside it; `e2e` times the public C-ABI call with pinned host
probe positions in and host SH out.  L2 is flushed (256 MiB write) before every
timed step; each step is bracketed by CUDA events on the context's stream.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Prints one JSON line.  Under torchrun each rank bakes its own replica of the
workload (probes are independent: weak scaling, no data-path collective); the
max step time over ranks is reported.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
PKG = ROOT / "vulkan-light-bakery_gb300"
sys.path.insert(0, str(PKG))

SEED = 1
NBOXES = 64
GRID = (16, 16, 16)
NDIRS = 256
LMAX = 2
SKY_N = 128
WORKLOAD = "probe bake 16^3 probes x 256 Fibonacci dirs, 64-box scene (778 tris), sun + 128^2 cubemap sky, L2 SH"
METRIC_FULL = "probes/s, Grays/s, p99 bake latency: chosen vs plain FP32, <=1e-4 SH rel err"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-probes", type=int, default=1024, help="probes in the CPU baseline sample")
    ap.add_argument("--only", choices=["bake", "skybox", "projection", "bake_c2", "batch", "service", "refbake"],
                    default=None,
                    help="time one section alone (for profiling captures); prints its JSON object")
    return ap.parse_args()


def max_over_ranks(x: float, dist, device: str) -> float:
    """The largest of every rank's x (the job's time is its slowest replica's)."""
    import torch

    if dist is None:
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank: float, world: int, max_ms: float) -> float:
    """Replicas (weak scaling): every rank bakes the workload; the job's rate is
    all ranks' units over the slowest rank's time."""
    return world * units_per_rank / (max_ms / 1e3)


def workload_inputs():
    import vlb

    pos, idx, alb = vlb.synth_box_scene(SEED, NBOXES)
    sky = vlb.synth_cubemap(SEED, SKY_N)
    sun = vlb.synth_sun(SEED)
    bounds = np.concatenate([np.minimum(pos.min(0), 0), np.maximum(pos.max(0), 0)]).astype(np.float32)
    probes, _ = vlb.probe_grid_ref_order(bounds, GRID)
    return pos, idx, alb, sky, sun, probes


def cpu_model() -> str:
    """The host CPU's model line from /proc/cpuinfo (x86 "model name", Arm
    "CPU implementer/part"), else the machine type."""
    import platform

    try:
        info = open("/proc/cpuinfo").read().splitlines()
    except OSError:
        return platform.machine()
    for ln in info:
        if ln.lower().startswith("model name"):
            return ln.split(":", 1)[1].strip()
    impl = [ln.split(":", 1)[1].strip() for ln in info if ln.startswith("CPU implementer")]
    part = [ln.split(":", 1)[1].strip() for ln in info if ln.startswith("CPU part")]
    if impl and part:
        arm = {"0xd4f": "Neoverse-V2", "0xd40": "Neoverse-V1", "0xd0c": "Neoverse-N1", "0xd49": "Neoverse-N2"}
        name = arm.get(part[0].lower()) if impl[0].lower() == "0x41" else None
        return f"{platform.machine()} {name}" if name else f"{platform.machine()} implementer {impl[0]} part {part[0]}"
    return platform.machine()


def cpu_time_oracle(pos, idx, alb, sky, sun, probes, nthreads):
    """Times the FP64 CPU restatement (the oracle) on all host threads."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle as O

    d32, w = O.dirs_fibonacci(NDIRS)
    B = O.basis_matrix(d32.astype(np.float64), w, LMAX)
    sc = O.Scene(pos, idx, alb)
    t0 = time.perf_counter()
    out = sc.bake(probes, d32, B, sun, sky=sky, sky_n=SKY_N, nthreads=nthreads)
    dt = time.perf_counter() - t0
    return out, dt


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.dev = device_index
        self.proc = None
        self.lines: list[str] = []
        self.t = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.dev}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return
        self.t = threading.Thread(target=self._read, daemon=True)
        self.t.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        if self.t:
            self.t.join(timeout=2)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def load_profile_figure(name: str, kernel: str):
    """A per-launch figure `name[kernel]: value` from the committed ncu summaries, if any."""
    for f in sorted((ROOT / "profiles").glob("*.md")):
        for ln in f.read_text().splitlines():
            if ln.startswith(f"{name}[{kernel}]:"):
                try:
                    return float(ln.split(":", 1)[1].split()[0])
                except ValueError:
                    pass
    return None


def load_traffic(kernel: str):
    """DRAM bytes per launch of `kernel` from the committed ncu summary, if any."""
    return load_profile_figure("traffic_bytes_per_launch", kernel)


def issue_roofline(torch, kernel: str, avg_ms: float, clk: dict):
    """The trace kernel's real bound: warp instructions issued per second (the
    per-launch count from the committed ncu summary over the live launch time)
    against the SM issue peak (SMs x 4 schedulers x the maximum SM clock)."""
    inst = load_profile_figure("warp_instructions_per_launch", kernel)
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    mhz = clk.get("sm_max_mhz") or 2070.0
    peak = sms * 4 * mhz * 1e6
    achieved = inst / (avg_ms * 1e-3) if inst and avg_ms > 0 else None
    return {"unit": "warp instructions/s", "achieved": achieved, "peak": peak,
            "frac": achieved / peak if achieved else None, "warp_instructions_per_launch": inst,
            "peak_source": f"{sms} SMs x 4 issue slots x {mhz:.0f} MHz"}


def run_reference(args, rank: int):
    if rank != 0:
        return None
    pos, idx, alb, sky, sun, probes = workload_inputs()
    nthreads = os.cpu_count() or 1
    sample = probes[: args.cpu_probes]
    for _ in range(args.warmup):
        cpu_time_oracle(pos, idx, alb, sky, sun, sample[:64], nthreads)
    times = []
    for _ in range(args.steps):
        _, dt = cpu_time_oracle(pos, idx, alb, sky, sun, sample, nthreads)
        times.append(dt)
    pps = len(sample) * len(times) / sum(times)
    line = {
        "impl": "reference", "metric": "probes/s", "metric_full": METRIC_FULL, "value": pps, "unit": "probes/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * sum(times) / len(times), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
        "config": {"workload": WORKLOAD, "probes_per_step": len(sample), "l2": "n/a (CPU)"},
        "cpu_baseline": {"value": pps, "unit": "probes/s", "cores": nthreads, "kind": "port",
                         "sample": f"first {len(sample)} of {len(probes)} probes, {NDIRS} dirs each, per step",
                         "cpu": cpu_model()},
        "e2e": {"value": pps, "unit": "probes/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference bake needs Vulkan ray tracing (unavailable on this box); its math runs here as "
                "the FP64 multithreaded CPU restatement",
    }
    return line


def main():
    args = parse()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        line = run_reference(args, rank)
        if line is not None:
            print(json.dumps(line), flush=True)
        return 0
    assert args.warmup >= 3, "at least 3 warm-up steps"
    import torch

    import vlb

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    # a dedicated stream: the library runs on it and the torch events record on it
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx = vlb.Context(local)
    ctx.set_stream(stream.cuda_stream)
    if args.only:
        peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
        fn = {"bake": bake_measure, "skybox": skybox_measure, "projection": projection_measure,
              "bake_c2": bake_c2_measure, "batch": batch_measure, "service": service_measure,
              "refbake": refbake_measure}[args.only]
        print(json.dumps(fn(ctx, torch, stream, args.steps, peaks.get("hbm_gbs", 6800.0))), flush=True)
        return 0
    pos, idx, alb, sky, sun, probes = workload_inputs()
    scene = ctx.scene(pos, idx, alb)
    dirs = ctx.fibonacci(NDIRS)
    skyh = ctx.sky(sky, SKY_N)
    P = probes.shape[0]
    K = vlb.k_of(LMAX)
    d_probes = torch.from_numpy(probes).cuda()
    d_out = torch.empty((P, K, 3), dtype=torch.float32, device="cuda")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    params = {
        "fused": vlb.bake_params(dirs, LMAX, vlb.PREC_FUSED, sun, sky=skyh),
        "fp32": vlb.bake_params(dirs, LMAX, vlb.PREC_FP32, sun, sky=skyh),
    }
    chosen = "fused"

    def barrier():
        if dist is not None:
            dist.barrier()

    def timed(pname: str, steps: int, profile: bool = False):
        p = params[pname]
        ctx.set_profiling(profile)
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        barrier()
        torch.cuda.synchronize()
        l0 = ctx.launch_count
        for a, b in evs:
            flush.zero_()
            a.record(stream)
            ctx.bake(scene, d_probes, p, out=d_out)
            b.record(stream)
        torch.cuda.synchronize()
        barrier()
        ctx.set_profiling(False)
        ms = [a.elapsed_time(b) for a, b in evs]
        return ms, ctx.launch_count - l0

    for name in params:
        timed(name, args.warmup)
    clocks = ClockSampler(local)
    clocks.start()
    ms_chosen, launches = timed(chosen, args.steps)
    ms_plain, _ = timed("fp32", args.steps)
    clk = clocks.stop()
    res_chosen = d_out.cpu().numpy().copy()
    # per-kernel device time of the chosen path (library events on the same stream)
    ctx.profile_reset()
    timed(chosen, min(args.steps, 20), profile=True)
    prof = ctx.profile()
    # per-ray work counts for the algorithmic bytes (one debug bake, untimed)
    stats = ctx_trace_stats(ctx, scene, probes, params["fp32"])
    shadow_rays = stats["shadow_rays"]

    def agg(ms):
        return max_over_ranks(sum(ms), dist, "cuda")

    tot_chosen = agg(ms_chosen)
    tot_plain = agg(ms_plain)
    value = whole_job_rate(P * args.steps, world, tot_chosen)
    plain = whole_job_rate(P * args.steps, world, tot_plain)

    # e2e: public call with pinned host buffers (H2D probes, D2H SH) inside the timed region
    h_probes = torch.from_numpy(probes).pin_memory()
    h_out = torch.empty((P, K, 3), dtype=torch.float32).pin_memory()
    for _ in range(3):
        ctx.bake(scene, h_probes, params[chosen], out=h_out)
    e2e_ms = []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ctx.bake(scene, h_probes, params[chosen], out=h_out)
        e2e_ms.append(1e3 * (time.perf_counter() - t0))
    e2e_value = whole_job_rate(P * args.steps, world, agg(e2e_ms))

    if rank != 0:
        return 0
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    # roofline of the dominant kernel: algorithmic bytes = node + triangle fetches per launch
    kname = max(prof, key=lambda k: prof[k][1])  # the chosen path's dominant kernel
    klaunch, kms = prof.get(kname, (0, 0.0))
    k_avg_ms = kms / max(klaunch, 1)
    # DRAM-level algorithmic bytes of one trace launch: the radiance tile it
    # writes plus everything it must read once (probes and their order, the
    # direction table, the scene's nodes, triangles and albedo, one sky texel
    # per direction).  The node and triangle fetches its lanes request (L1
    # level, re-read many times) are reported beside it.
    ntri = int(idx.shape[0])
    bytes_per_launch = (P * NDIRS * 3 * 4 + P * 16 + NDIRS * (16 + 4 + 12)
                        + max(ntri - 1, 0) * 64 + ntri * (48 + 16))
    achieved = bytes_per_launch / (k_avg_ms * 1e-3) / 1e9 if k_avg_ms > 0 else None
    traffic = load_traffic(kname)
    step_ms = sorted(ms_chosen)
    p50 = step_ms[len(step_ms) // 2]
    p99 = step_ms[min(len(step_ms) - 1, int(round(0.99 * (len(step_ms) - 1))))]
    # CPU baseline: the FP64 restatement on a bounded probe sample, all host threads
    sample = probes[: args.cpu_probes]
    ref_sh, cpu_dt = cpu_time_oracle(pos, idx, alb, sky, sun, sample, os.cpu_count() or 1)
    got = res_chosen[: len(sample)].astype(np.float64)
    err = np.linalg.norm((got - ref_sh).reshape(len(sample), -1), axis=1) / np.maximum(
        np.linalg.norm(ref_sh.reshape(len(sample), -1), axis=1), 1e-30)
    line = {
        "metric": "probes/s", "metric_full": METRIC_FULL, "value": value, "unit": "probes/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": tot_chosen / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded SplitMix64 scene, sky and sun)",
        "config": {"workload": WORKLOAD, "probes": P, "dirs_per_probe": NDIRS, "triangles": int(idx.shape[0]),
                   "lmax": LMAX, "path": "VLB_PREC_FUSED (FP32; library picks the schedule: "
                                         + "+".join(sorted(prof)) + ")",
                   "l2": "flushed (256 MiB write) before every timed step", "parallelism": f"replicas x{world}"},
        "grays_per_s": value * NDIRS / 1e9, "grays_incl_shadow_per_s": value * (NDIRS + shadow_rays / P) / 1e9,
        "latency_ms": {"p50": p50, "p99": p99},
        "plain_fp32": {"value": plain, "unit": "probes/s", "p99_ms": sorted(ms_plain)[-1]},
        "sh_rel_err_vs_fp64": {"max": float(err.max()), "mean": float(err.mean()),
                               "p99": float(np.quantile(err, 0.99)),
                               "frac_within_1e-4": float((err < 1e-4).mean()), "probes": len(sample),
                               "note": "probes above 1e-4 own a ray within 1e-6 of a triangle edge or of tmin "
                                       "(FP32 decision); with those decisions replayed in FP64 every probe is "
                                       "within 1e-4 (tests/test_gpu_bake.py)"},
        "e2e": {"value": e2e_value, "unit": "probes/s", "h2d_bytes_per_step": int(P * 12),
                "d2h_bytes_per_step": int(P * K * 12)},
        "gpu_launches": int(launches),
        "roofline": {"kernel": kname, "bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                     "frac": (achieved / hbm_peak) if achieved else None, "traffic": traffic,
                     "algorithmic_bytes_per_launch": bytes_per_launch, "avg_launch_ms": k_avg_ms,
                     "l1_requested_bytes_per_launch": stats["bytes"],
                     "l1_requested_gbs": stats["bytes"] / (k_avg_ms * 1e-3) / 1e9 if k_avg_ms > 0 else None,
                     "note": "the trace kernel is bound by instruction issue and L1 latency (scene L1/L2 "
                             "resident); its DRAM traffic is the radiance tile, so the HBM fraction is low "
                             "by nature",
                     "node_tests_per_ray": stats["node_tests_per_ray"],
                     "node_fetches_per_ray": stats["node_fetches_per_ray"],
                     "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)" if peaks else "fallback 6.8 TB/s",
                     "issue": issue_roofline(torch, kname, k_avg_ms, clk)},
        "kernels_ms": {k: {"launches": v[0], "avg_ms": v[1] / max(v[0], 1)} for k, v in prof.items()},
        "cpu_baseline": {"value": len(sample) / cpu_dt, "unit": "probes/s", "cores": os.cpu_count() or 1,
                         "kind": "port", "sample": f"first {len(sample)} of {P} probes, {NDIRS} dirs each",
                         "cpu": cpu_model()},
        "clocks": clk,
        "skybox_c0": skybox_measure(ctx, torch, stream, args.steps, hbm_peak),
        "projection_c2": projection_measure(ctx, torch, stream, args.steps, hbm_peak),
        "bake_c2": bake_c2_measure(ctx, torch, stream, args.steps, hbm_peak),
        "batch_c3": batch_measure(ctx, torch, stream, args.steps, hbm_peak),
        "service_c4": service_measure(ctx, torch, stream, args.steps, hbm_peak),
        "reference_bake": refbake_measure(ctx, torch, stream, args.steps, hbm_peak),
    }
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


def bake_measure(ctx, torch, stream, steps, hbm_peak):
    """The headline workload's chosen path alone (config 1, VLB_PREC_FUSED):
    `steps` bakes with inputs resident in HBM, per-kernel library times."""
    import vlb

    pos, idx, alb, sky, sun, probes = workload_inputs()
    scene = ctx.scene(pos, idx, alb)
    p = vlb.bake_params(ctx.fibonacci(NDIRS), LMAX, vlb.PREC_FUSED, sun, sky=ctx.sky(sky, SKY_N))
    d_probes = torch.from_numpy(probes).cuda()
    out = torch.empty((probes.shape[0], vlb.k_of(LMAX), 3), dtype=torch.float32, device="cuda")
    for _ in range(3):
        ctx.bake(scene, d_probes, p, out=out)
    torch.cuda.synchronize()
    ctx.profile_reset()
    ctx.set_profiling(True)
    for _ in range(steps):
        ctx.bake(scene, d_probes, p, out=out)
    torch.cuda.synchronize()
    ctx.set_profiling(False)
    return {"workload": WORKLOAD, "kernels_ms": {k: v[1] / max(v[0], 1) for k, v in ctx.profile().items()}}


def skybox_measure(ctx, torch, stream, steps, hbm_peak):
    """Config 0 skybox projection: the literal single 6x128^2 cubemap (latency)
    and a batch of 1024 of them resident in HBM (1.21 GB > L2, streaming)."""
    import vlb

    n, count = 128, 1024
    one = torch.from_numpy(vlb.synth_cubemap(SEED, n)).cuda()
    maps = one.unsqueeze(0).expand(count, -1, -1, -1, -1).contiguous()
    maps.mul_(torch.linspace(0.5, 1.5, count, device="cuda").view(count, 1, 1, 1, 1))
    out = torch.empty((count, vlb.k_of(LMAX), 3), dtype=torch.float32, device="cuda")
    out1 = torch.empty((1, vlb.k_of(LMAX), 3), dtype=torch.float32, device="cuda")

    def run(x, cnt, o, k):
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(k)]
        for a, b in evs:
            a.record(stream)
            ctx.skybox_sh(x, vlb.SKY_CUBEMAP, n, n, LMAX, count=cnt, out=o)
            b.record(stream)
        torch.cuda.synchronize()
        return [a.elapsed_time(b) for a, b in evs]

    run(maps, count, out, 3)
    run(one, 1, out1, 3)
    ctx.profile_reset()
    ctx.set_profiling(True)
    ms_b = run(maps, count, out, steps)
    ctx.set_profiling(False)
    prof = ctx.profile()
    ms_1 = run(one, 1, out1, steps)
    kname = [k for k in prof if k.startswith("skybox_sh")][0]
    kl, kms = prof[kname]
    bytes_per_launch = count * 6 * n * n * 12
    k_avg = kms / max(kl, 1)
    achieved = bytes_per_launch / (k_avg * 1e-3) / 1e9
    return {
        "workload": f"skybox SH, {count} cubemaps 6x{n}x{n} RGB FP32 resident in HBM per call, L{LMAX}",
        "cubemaps_per_s": count * len(ms_b) / (sum(ms_b) / 1e3),
        "single_cubemap_us": 1e3 * sorted(ms_1)[len(ms_1) // 2],
        "roofline": {"kernel": kname, "bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                     "frac": achieved / hbm_peak, "algorithmic_bytes_per_launch": bytes_per_launch,
                     "avg_launch_ms": k_avg, "traffic": load_traffic(kname)},
    }


def projection_measure(ctx, torch, stream, steps, hbm_peak, nprobes=262144, S=1024):
    """Config 2 projection: a [262,144 x 3, 1024] radiance tile resident in
    HBM, BF16 through the tcgen05 kernel (hi/lo BF16 basis, FP32
    accumulation) and FP32 through the CUDA-core kernel."""
    import vlb

    ds = ctx.fibonacci(S)
    g = torch.Generator(device="cuda").manual_seed(SEED)
    t16 = (torch.rand((nprobes * 3, S), generator=g, device="cuda") * 5).to(torch.bfloat16)
    out = torch.empty((nprobes, vlb.k_of(LMAX), 3), dtype=torch.float32, device="cuda")

    def run(tile, dtype, k):
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(k)]
        for a, b in evs:
            a.record(stream)
            ctx.project(tile, nprobes, ds, LMAX, dtype=dtype, out=out)
            b.record(stream)
        torch.cuda.synchronize()
        return [a.elapsed_time(b) for a, b in evs]

    bits = t16.view(torch.int16)
    run(bits, vlb.DTYPE_BF16, 3)
    ms16 = run(bits, vlb.DTYPE_BF16, steps)
    t32 = t16.float()
    run(t32, vlb.DTYPE_F32, 3)
    ms32 = run(t32, vlb.DTYPE_F32, steps)
    del t32
    b16 = nprobes * 3 * S * 2 + out.numel() * 4
    b32 = nprobes * 3 * S * 4 + out.numel() * 4
    m16 = sorted(ms16)[len(ms16) // 2]
    m32 = sorted(ms32)[len(ms32) // 2]
    flops = 2 * nprobes * 3 * S * 32  # the MMA work (N = 32: high and low basis halves)
    return {
        "workload": f"SH projection of a [{nprobes}x3, {S}] radiance tile resident in HBM, L{LMAX}",
        "bf16_tcgen05": {"probes_per_s": nprobes / (m16 / 1e3), "ms": m16,
                         "roofline": {"kernel": "project_tc", "bound": "hbm", "achieved": b16 / (m16 * 1e-3) / 1e9,
                                      "peak": hbm_peak, "unit": "GB/s",
                                      "frac": b16 / (m16 * 1e-3) / 1e9 / hbm_peak,
                                      "algorithmic_bytes_per_launch": b16, "mma_tflops": flops / (m16 * 1e-3) / 1e12,
                                      "traffic": load_traffic("project_tc")}},
        "fp32_cuda_cores": {"probes_per_s": nprobes / (m32 / 1e3), "ms": m32,
                            "achieved_gbs": b32 / (m32 * 1e-3) / 1e9},
    }


def bake_c2_measure(ctx, torch, stream, steps, hbm_peak, sample=64):
    """Config 2 as a whole bake: the config-1 scene scaled to 4096 boxes (49,162
    triangles), 64^3 = 262,144 probes x 1024 Fibonacci directions (268 M primary
    rays), L2 SH; BF16 radiance tile + tcgen05 hi/lo projection vs the plain
    FP32 path, inputs resident in HBM, L2 flushed before every bake.  Error vs
    the FP64 oracle on a probe sample."""
    import vlb

    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle as O

    pos, idx, alb = vlb.synth_box_scene(SEED, 4096)
    sky = vlb.synth_cubemap(SEED, SKY_N)
    sun = vlb.synth_sun(SEED)
    bounds = np.concatenate([np.minimum(pos.min(0), 0), np.maximum(pos.max(0), 0)]).astype(np.float32)
    probes, _ = vlb.probe_grid_ref_order(bounds, (64, 64, 64))
    scene = ctx.scene(pos, idx, alb)
    ds = ctx.fibonacci(1024)
    skyh = ctx.sky(sky, SKY_N)
    P, K = probes.shape[0], vlb.k_of(LMAX)
    d_probes = torch.from_numpy(probes).cuda()
    out = torch.empty((P, K, 3), dtype=torch.float32, device="cuda")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    steps = max(3, min(steps, 5))
    res = {"workload": f"config 2 bake: {int(idx.shape[0])} triangles, {P} probes x 1024 dirs, L{LMAX} SH",
           "primary_rays": P * 1024}
    outs = {}
    for name, prec in (("mixed_bf16_tcgen05", vlb.PREC_MIXED), ("fp32", vlb.PREC_FP32)):
        p = vlb.bake_params(ds, LMAX, prec, sun, sky=skyh)
        ctx.bake(scene, d_probes, p, out=out)
        torch.cuda.synchronize()
        ctx.profile_reset()
        ctx.set_profiling(True)
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        for a, b in evs:
            flush.zero_()
            a.record(stream)
            ctx.bake(scene, d_probes, p, out=out)
            b.record(stream)
        torch.cuda.synchronize()
        ctx.set_profiling(False)
        ms = sorted(a.elapsed_time(b) for a, b in evs)[len(evs) // 2]
        outs[name] = out.cpu().numpy().copy()
        res[name] = {"ms": ms, "probes_per_s": P / (ms / 1e3), "grays_per_s": P * 1024 / (ms / 1e3) / 1e9,
                     "kernels_ms": {k: v[1] / max(v[0], 1) for k, v in ctx.profile().items()}}
    # error vs the FP64 oracle on an evenly spread probe sample
    sel = np.linspace(0, P - 1, sample).astype(int)
    d32, w = O.dirs_fibonacci(1024)
    B = O.basis_matrix(d32.astype(np.float64), w, LMAX)
    orc = O.Scene(pos, idx, alb)
    t0 = time.perf_counter()
    ref = orc.bake(probes[sel], d32, B, sun, sky=sky, sky_n=SKY_N)
    cpu_s = time.perf_counter() - t0
    res["cpu_oracle"] = {"probes_per_s": sample / cpu_s, "threads": os.cpu_count() or 1, "cpu": cpu_model(),
                         "sample": f"{sample} evenly spread probes x 1024 dirs ({cpu_s:.2f} s)",
                         "full_bake_s": cpu_s * P / sample, "label": "extrapolated from the sample"}
    for name in outs:
        g = outs[name][sel].astype(np.float64)
        e = np.linalg.norm((g - ref).reshape(sample, -1), axis=1) / np.maximum(
            np.linalg.norm(ref.reshape(sample, -1), axis=1), 1e-30)
        res[name]["rel_err_vs_fp64"] = {"max": float(e.max()), "median": float(np.median(e)), "probes": sample}
    e = np.linalg.norm((outs["mixed_bf16_tcgen05"] - outs["fp32"]).reshape(P, -1), axis=1) / np.maximum(
        np.linalg.norm(outs["fp32"].reshape(P, -1), axis=1), 1e-30)
    res["mixed_vs_fp32_all_probes"] = {"max": float(e.max()), "mean": float(e.mean())}
    return res


def batch_volumes(seed=SEED, nvol=256):
    """Uneven batch: per volume a seeded box scene (boxes log-uniform in
    [16, 16384]), probes log-uniform in [64, 32768] at uniform positions in the
    scene bounds, rays per probe drawn from {64, 256, 1024}."""
    import vlb

    rng = np.random.default_rng(seed + 1000)
    boxes = np.exp(rng.uniform(np.log(16), np.log(16384), nvol)).astype(int)
    nprobes = np.exp(rng.uniform(np.log(64), np.log(32768), nvol)).astype(int)
    rays = rng.choice([64, 256, 1024], nvol)
    vols = []
    for i in range(nvol):
        pos, idx, alb = vlb.synth_box_scene(seed * 7919 + i, int(boxes[i]))
        lo = np.minimum(pos.min(0), 0)
        hi = np.maximum(pos.max(0), 0)
        probes = (lo + rng.random((int(nprobes[i]), 3)) * (hi - lo)).astype(np.float32)
        vols.append((pos, idx, alb, probes, int(rays[i]), vlb.synth_sun(seed * 104729 + i)))
    return vols


def refbake_measure(ctx, torch, stream, steps, hbm_peak, reps=3):
    """The reference baker's own workload on the config-1 scene: a 7^3 probe grid
    over the origin-inclusive bounds in the reference's order, one ray per pixel
    of the 3141 x 1000 equirect env map (3,141,000 rays per probe, 1.08e9 in
    all), L3 (16 coefficients), FP32 and BF16 + tcgen05; device-resident
    probes and output, L2 flushed before each bake."""
    import vlb

    pos, idx, alb, sky, sun, _ = workload_inputs()
    scene = ctx.scene(pos, idx, alb)
    probes, _ = vlb.probe_grid_ref_order(scene.bounds(include_origin=True), (7, 7, 7))
    P, W, H = probes.shape[0], 3141, 1000
    ds = ctx.equirect(W, H)
    skyh = ctx.sky(sky, SKY_N)
    d_probes = torch.from_numpy(probes).cuda()
    out = torch.empty((P, 16, 3), dtype=torch.float32, device="cuda")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    res = {"workload": f"{P} probes (7^3 reference grid) x {W}x{H} equirect rays, config-1 scene, L3",
           "primary_rays": P * W * H}
    for name, prec in (("fp32", vlb.PREC_FUSED), ("mixed_bf16_tcgen05", vlb.PREC_MIXED)):
        p = vlb.bake_params(ds, 3, prec, sun, sky=skyh)
        ctx.bake(scene, d_probes, p, out=out)
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(reps)]
        torch.cuda.synchronize()
        for a, b in evs:
            flush.zero_()
            a.record(stream)
            ctx.bake(scene, d_probes, p, out=out)
            b.record(stream)
        torch.cuda.synchronize()
        ms = sorted(a.elapsed_time(b) for a, b in evs)[len(evs) // 2]
        res[name] = {"ms": ms, "grays_per_s": P * W * H / (ms / 1e3) / 1e9}
    return res


def batch_measure(ctx, torch, stream, steps, hbm_peak):
    """Config 3: 256 uneven bake jobs in one batch (one persistent trace launch
    over all jobs, one tcgen05 projection per direction set, replayed as a CUDA
    graph).  BF16 radiance, FP32 accumulation, L2 SH.  Inputs and outputs
    resident in HBM for `value`; `e2e` passes pinned host probes and outputs."""
    import vlb

    vols = batch_volumes()
    sky = ctx.sky(vlb.synth_cubemap(SEED, SKY_N), SKY_N)
    dsets = {S: ctx.fibonacci(S) for S in (64, 256, 1024)}
    K = vlb.k_of(LMAX)
    scenes, plist, jobs, hjobs = [], [], [], []
    for pos, idx, alb, probes, S, sun in vols:
        sc = ctx.scene(pos, idx, alb)
        p = vlb.bake_params(dsets[S], LMAX, vlb.PREC_MIXED, sun, sky=sky)
        scenes.append(sc)
        plist.append(p)
        n = probes.shape[0]
        jobs.append((sc, torch.from_numpy(probes).cuda(), torch.empty((n, K, 3), device="cuda"), p))
        hjobs.append((sc, torch.from_numpy(probes).pin_memory(), torch.empty((n, K, 3)).pin_memory(), p))
    P = sum(v[3].shape[0] for v in vols)
    rays = sum(v[3].shape[0] * v[4] for v in vols)
    tris = [int(v[1].shape[0]) for v in vols]
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    steps = max(3, min(steps, 10))
    t0 = time.perf_counter()
    sched, tune_ms = ctx.batch_autotune(jobs, plist[0], reps=1)
    tune_s = time.perf_counter() - t0

    def run(js, k, profile=False):
        ctx.set_profiling(profile)
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(k)]
        l0 = ctx.launch_count
        for a, b in evs:
            flush.zero_()
            a.record(stream)
            ctx.bake_batch(js, plist[0])
            b.record(stream)
        torch.cuda.synchronize()
        ctx.set_profiling(False)
        return [a.elapsed_time(b) for a, b in evs], ctx.launch_count - l0

    run(jobs, 3)  # direct, capture, replay
    ms, launches = run(jobs, steps)
    # per-kernel times (direct launches, library events)
    ctx.profile_reset()
    direct = vlb.BatchSchedule(sched.dirs_per_item, sched.cost_order, 0)
    ctx.set_profiling(True)
    for _ in range(2):
        flush.zero_()
        ctx.bake_batch(jobs, plist[0], direct)
    torch.cuda.synchronize()
    ctx.set_profiling(False)
    prof = ctx.profile()
    # the same jobs as 256 separate vlb_bake calls (device buffers, no sync between)
    def singles():
        for sc, pr, o, p in jobs:
            ctx.bake(sc, pr, p, out=o)
    singles()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    flush.zero_()
    a.record(stream)
    singles()
    b.record(stream)
    torch.cuda.synchronize()
    single_ms = a.elapsed_time(b)
    # e2e: pinned host probes in, host SH out, through the public call
    run(hjobs, 3)
    e2e = []
    for _ in range(steps):
        flush.zero_()
        torch.cuda.synchronize()
        t = time.perf_counter()
        ctx.bake_batch(hjobs, plist[0])
        e2e.append(1e3 * (time.perf_counter() - t))
    tot = sum(ms)
    tr = prof.get("trace_batch", (0, 0.0))
    return {
        "workload": f"{len(vols)} bake jobs: boxes log-uniform 16-16384 ({min(tris)}-{max(tris)} tris), probes "
                    f"log-uniform 64-32768 (total {P}), rays per probe in {{64,256,1024}} (total {rays} primary), "
                    f"L{LMAX} SH, BF16 radiance + tcgen05 projection, CUDA graph replay",
        "probes_per_s": P * len(ms) / (tot / 1e3), "grays_per_s": rays * len(ms) / (tot / 1e3) / 1e9,
        "ms_per_batch": tot / len(ms), "p99_ms": sorted(ms)[-1], "gpu_launches_per_batch": launches / len(ms),
        "schedule": {"dirs_per_item": sched.dirs_per_item, "cost_order": sched.cost_order,
                     "autotune_s": tune_s, "autotune_best_ms": tune_ms},
        "kernels_ms": {k: {"launches": v[0], "avg_ms": v[1] / max(v[0], 1)} for k, v in prof.items()},
        "trace_batch_grays_per_s": rays / (tr[1] / max(tr[0], 1) * 1e-3) / 1e9 if tr[0] else None,
        "separate_bakes": {"ms": single_ms, "probes_per_s": P / (single_ms / 1e3),
                           "note": "the same 256 jobs as separate vlb_bake calls"},
        "e2e": {"probes_per_s": P * len(e2e) / (sum(e2e) / 1e3), "h2d_bytes_per_step": int(P * 12),
                "d2h_bytes_per_step": int(P * K * 12)},
        "l2": "flushed (256 MiB write) before every timed batch",
    }


SERVICE_BOXES = (64, 512, 4096, 16384, 32768, 65536, 131072, 170000)


def service_requests(nreq, rate, seed, scenes_bounds):
    """Seeded request stream: Poisson arrivals at `rate` per second; bakes of
    log-uniform 16-16384 probes at uniform positions in a uniformly chosen
    resident scene with 256 or 1024 rays; 20% relights of an earlier bake
    with a new seeded sun direction and intensity."""
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, nreq))
    reqs = []
    for i in range(nreq):
        if i >= 4 and rng.random() < 0.2:
            reqs.append(dict(t=t[i], relight=int(rng.integers(0, i)), sun_seed=int(rng.integers(1 << 30)),
                             intensity=float(rng.uniform(1, 10))))
            continue
        sc = int(rng.integers(0, len(scenes_bounds)))
        lo, hi = scenes_bounds[sc]
        n = int(np.exp(rng.uniform(np.log(16), np.log(16384))))
        reqs.append(dict(t=t[i], relight=None, scene=sc, S=int(rng.choice([256, 1024])),
                         probes=(lo + rng.random((n, 3)) * (hi - lo)).astype(np.float32),
                         sun_seed=int(rng.integers(1 << 30)), intensity=5.0))
    return reqs


def service_run(ctx, svc, scenes, dsets, sky, reqs, lmax, prec):
    """Open-loop run: a submitter thread issues the requests at their arrival
    times; the caller collects them.  Returns latencies (ms) and wall time."""
    import vlb

    tickets = [None] * len(reqs)
    params = [None] * len(reqs)
    base = [None] * len(reqs)  # bake index each request resolves to
    t0 = time.perf_counter()

    def submit_all():
        for i, r in enumerate(reqs):
            dt = r["t"] - (time.perf_counter() - t0)
            if dt > 0:
                time.sleep(dt)
            if r["relight"] is None:
                base[i] = i
                p = vlb.bake_params(dsets[r["S"]], lmax, prec, vlb.synth_sun(r["sun_seed"]),
                                    sun_intensity=r["intensity"], sky=sky)
                params[i] = p
                tickets[i] = svc.submit(scenes[r["scene"]], r["probes"], p, keep_hits=True)
            else:
                j = r["relight"]
                while base[j] is None or tickets[base[j]] is None:
                    time.sleep(0.0001)
                b = base[j]
                base[i] = b
                p = vlb.bake_params(dsets[reqs[b]["S"]], lmax, prec, vlb.synth_sun(r["sun_seed"]),
                                    sun_intensity=r["intensity"], sky=sky)
                params[i] = p
                tickets[i] = svc.submit(None, None, p, relight_of=tickets[b])

    th = threading.Thread(target=submit_all)
    th.start()
    lat = []
    for i in range(len(reqs)):
        while tickets[i] is None:
            time.sleep(0.0001)
        _, ms = svc.wait(tickets[i], timeout_ms=600000)
        lat.append(ms)
    th.join()
    wall = time.perf_counter() - t0
    return lat, wall, base


def service_measure(ctx, torch, stream, steps, hbm_peak, nreq=160):
    """Config 4: the bake service over 8 resident box scenes (64 ... 170,000
    boxes, 778 ... 2,040,010 triangles), Poisson arrivals swept over rates
    relative to the measured capacity, 20% relights, 64 GiB budget."""
    import vlb

    t0 = time.perf_counter()
    scenes, bounds, tris = [], [], []
    for i, nb in enumerate(SERVICE_BOXES):
        pos, idx, alb = vlb.synth_box_scene(SEED * 31 + i, nb)
        scenes.append(ctx.scene(pos, idx, alb))
        bounds.append((np.minimum(pos.min(0), 0), np.maximum(pos.max(0), 0)))
        tris.append(int(idx.shape[0]))
    build_s = time.perf_counter() - t0
    dsets = {S: ctx.fibonacci(S) for S in (256, 1024)}
    sky = ctx.sky(vlb.synth_cubemap(SEED, SKY_N), SKY_N)
    out = {"workload": f"bake service: {len(scenes)} resident box scenes ({min(tris)}-{max(tris)} tris), requests "
                       "of log-uniform 16-16384 probes x {256,1024} rays, 20% relights (kept hits, new sun), "
                       "Poisson arrivals, 64 GiB budget, L2 SH",
           "scene_build_s": build_s}

    def run(prec, rate, n, seed):
        svc = vlb.Service(ctx, budget_bytes=64 << 30, lmax=LMAX, precision=prec)
        reqs = service_requests(n, rate, seed, bounds)
        lat, wall, base = service_run(ctx, svc, scenes, dsets, sky, reqs, LMAX, prec)
        st = svc.stats()
        svc.close()
        lat = np.array(lat)
        return {"rate_offered": rate, "requests": n, "p50_ms": float(np.percentile(lat, 50)),
                "p99_ms": float(np.percentile(lat, 99)), "probes_per_s": st["probes"] / wall,
                "grays_per_s": st["rays"] / wall / 1e9, "batches": st["batches"], "relights": st["relights"],
                "relights_rebaked": st["relights_rebaked"], "evictions": st["evictions"],
                "bytes_peak": st["bytes_peak"], "wall_s": wall}

    # capacity: every request at t = 0 (closed burst)
    cap = run(vlb.PREC_MIXED, 1e9, nreq // 2, SEED + 7)
    capacity = cap["requests"] / cap["wall_s"]
    out["capacity_req_per_s"] = capacity
    out["burst"] = cap
    # open-loop runs of about 5 s each (20 to nreq requests)
    def nfor(rate):
        return int(min(nreq, max(20, rate * 5.0)))

    out["mixed_bf16"] = [run(vlb.PREC_MIXED, f * capacity, nfor(f * capacity), SEED + 11 + k)
                         for k, f in enumerate((0.3, 0.6, 0.9))]
    out["fp32"] = [run(vlb.PREC_FP32, 0.6 * capacity, nfor(0.6 * capacity), SEED + 12)]
    return out


def ctx_trace_stats(ctx, scene, probes, params):
    """Per-launch traversal work of the instrumented bake: node (64 B) and
    triangle (48 B) fetches as the kernel requests them (once per packet
    visit in packet mode, once per lane visit in lane mode), node tests once
    per ray."""
    import vlb

    st = vlb.trace_stats(ctx, scene, probes, params)
    rays = st["rays"] + st["shadow_rays"]
    return {"bytes": st["node_fetches"] * 64 + st["tri_fetches"] * 48,
            "node_fetches_per_ray": st["node_fetches"] / rays,
            "node_tests_per_ray": st["node_tests"] / rays, "shadow_rays": st["shadow_rays"]}


if __name__ == "__main__":
    sys.exit(main())
