#!/usr/bin/env python3
"""Benchmark of the light-probe bake on GB300.

Workload (one "step"): bake the 64x64x64 probe grid (262,144 probes, the
reference's breadth-first grid order over the scene bounds) of the 4096-box
scene (49,162 triangles, open unit room, seeded sun + 128^2 cubemap sky) with
1024 shared Fibonacci directions per probe, L2 SH -- 268,435,456 primary rays
plus the sun shadow rays.  The chosen path is the library's default
(VLB_PREC_FP32: the lane walk traces into an FP32 radiance tile, a CUDA-core
kernel projects it), timed with inputs resident in HBM; the one-kernel path
(VLB_PREC_FUSED: trace, shading and projection in one kernel, no tile), the
mixed path (BF16 hi/lo tile + tcgen05 projection) and the one-BF16 form are
timed beside it; `e2e` times the public C-ABI call with
pinned host probe positions in and host SH out.  L2 is flushed (256 MiB
write) before every timed step; each step is bracketed by CUDA events on the
context's stream.  Accuracy is measured against the FP64 oracle on a spread
probe sample, directly and with the device's per-ray decisions replayed.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Prints one JSON line.  Under torchrun each rank bakes its own replica of the
workload (probes are independent: weak scaling, no data-path collective); the
max step time over ranks is reported.  `--impl reference` times the FP64 CPU
restatement (the reference's own bake needs Vulkan ray tracing) on a probe
sample of the same workload per step, building its inputs with the oracle's
own generators (no product library).
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
NBOXES = 4096
GRID = (64, 64, 64)
NDIRS = 1024
LMAX = 2
SKY_N = 128
WORKLOAD = ("probe bake 64^3 probes x 1024 Fibonacci dirs, 4096-box scene (49,162 tris), sun + 128^2 cubemap "
            "sky, L2 SH")
METRIC_FULL = "probes/s, Grays/s, p99 bake latency of the default path, <=1e-4 SH rel err"
# The trace kernels' per-launch figures from ncu captures (the named profile
# gives the command): DRAM bytes read + written and warp instructions issued
# per launch of the headline workload, ncu's L1 and issue utilisation.
TRACE_NCU = {
    "trace_tile": {"capture": "profiles/trace_tile_c2.md", "scaled_from": "32^3 probes x 8",
                   "dram_bytes": 3415800000, "warp_instructions": 126470600000,
                   "l1tex_throughput_pct": 79.8, "issue_active_pct": 75.4},
    "trace_fused_lane": {"capture": "profiles/trace_tile_c2.md", "scaled_from": "32^3 probes x 8",
                         "dram_bytes": 86500000, "warp_instructions": 125671000000,
                         "l1tex_throughput_pct": 71.4, "issue_active_pct": 70.3},
}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-probes", type=int, default=8192, help="probes in the CPU baseline sample")
    ap.add_argument("--ref-probes", type=int, default=1024, help="probes per step of the reference arm")
    ap.add_argument("--only", choices=["bake", "c1", "skybox", "projection", "batch", "service", "refbake"],
                    default=None,
                    help="time one section alone (for profiling captures); prints its JSON object")
    ap.add_argument("--no-sections", action="store_true", help="headline only (skip the C0/C1/C3/C4 sections)")
    ap.add_argument("--bake-precision", choices=["fp32", "fused"], default="fp32",
                    help="--only bake: the path to time")
    ap.add_argument("--bake-grid", type=int, default=GRID[0],
                    help="--only bake: probes per grid axis (a smaller grid for ncu captures)")
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


def grid_probes(gen, nboxes=NBOXES, grid=GRID, seed=SEED):
    """Scene, sky, sun and the reference-order probe grid of a workload, from
    the library's (`gen` = vlb) or the oracle's (`gen` = oracle) generators."""
    pos, idx, alb = gen.synth_box_scene(seed, nboxes)
    sky = gen.synth_cubemap(seed, SKY_N)
    sun = gen.synth_sun(seed)
    pos = np.asarray(pos, np.float32).reshape(-1, 3)
    bounds = np.concatenate([np.minimum(pos.min(0), 0), np.maximum(pos.max(0), 0)]).astype(np.float32)
    probes, _ = gen.probe_grid_ref_order(bounds, grid)
    return pos, np.asarray(idx).reshape(-1, 3), np.asarray(alb).reshape(-1, 3), sky, sun, probes


def workload_inputs():
    import vlb

    return grid_probes(vlb)


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


def _oracle():
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle as O

    return O


def spread(n_total: int, n: int) -> np.ndarray:
    """n probe indices spread evenly over the grid."""
    return np.unique(np.linspace(0, n_total - 1, min(n, n_total)).astype(np.int64))


def cpu_time_oracle(pos, idx, alb, sky, sun, probes, nthreads, ndirs=NDIRS, lmax=LMAX):
    """Times the FP64 CPU restatement (the oracle) on all host threads."""
    O = _oracle()
    d32, w = O.dirs_fibonacci(ndirs)
    B = O.basis_matrix(d32.astype(np.float64), w, lmax)
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


def config_dict(P, ntri):
    """The workload's config (identical in both arms)."""
    return {"workload": WORKLOAD, "probes": int(P), "dirs_per_probe": NDIRS, "triangles": int(ntri), "lmax": LMAX}


def run_reference(args, rank: int):
    """The reference arm: the reference bakes with Vulkan ray tracing, which
    this box cannot run, so its math runs as the FP64 CPU restatement on all
    host threads; each step bakes a spread sample of the workload's probes.
    Inputs come from the oracle's own generators (no product library)."""
    if rank != 0:
        return None
    O = _oracle()
    pos, idx, alb, sky, sun, probes = grid_probes(O)
    nthreads = os.cpu_count() or 1
    sample = probes[spread(probes.shape[0], args.ref_probes)]
    for _ in range(args.warmup):
        cpu_time_oracle(pos, idx, alb, sky, sun, sample[:64], nthreads)
    times = []
    for _ in range(args.steps):
        _, dt = cpu_time_oracle(pos, idx, alb, sky, sun, sample, nthreads)
        times.append(dt)
    pps = len(sample) * len(times) / sum(times)
    return {
        "impl": "reference", "metric": "probes/s", "metric_full": METRIC_FULL, "value": pps, "unit": "probes/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * sum(times) / len(times), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded SplitMix64 scene, sky and sun)",
        "config": config_dict(probes.shape[0], idx.shape[0]),
        "cpu_baseline": {"value": pps, "unit": "probes/s", "cores": nthreads, "kind": "port",
                         "sample": f"{len(sample)} probes spread over the {probes.shape[0]}-probe grid, "
                                   f"{NDIRS} dirs each, per step", "cpu": cpu_model()},
        "e2e": {"value": pps, "unit": "probes/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference bake needs Vulkan ray tracing (unavailable on this box); its math runs here as "
                "the FP64 multithreaded CPU restatement, inputs from the oracle's generators",
    }


def rel_err(got, ref):
    g = np.asarray(got, np.float64).reshape(got.shape[0], -1)
    r = np.asarray(ref, np.float64).reshape(ref.shape[0], -1)
    return np.linalg.norm(g - r, axis=1) / np.maximum(np.linalg.norm(r, axis=1), 1e-30)


def accuracy_vs_fp64(ctx, scene, probes, params, pos, idx, alb, sky, sun, nsample=256, ndirs=NDIRS, lmax=LMAX,
                     timed_rows=None):
    """SH error per probe against the FP64 oracle on a spread sample: with the
    device's per-ray hit and shadow decisions replayed (FP32 cannot decide
    rays within ~1e-6 of a triangle edge; the replay isolates the arithmetic
    of shading and projection), and directly.  timed_rows: the SH of a timed
    bake of all `probes`; its sampled rows are the ones checked (a ray's
    decisions do not depend on the other probes of a bake, so the sample
    bake's decisions are the timed bake's), and their difference from the
    sample bake's own SH is reported (the FP32 tile of a small bake is
    projected in sample splits added in FP64, a large one unsplit)."""
    O = _oracle()
    sel = spread(probes.shape[0], nsample)
    sh, hit, vis, _ = ctx.bake(scene, probes[sel], params, debug=True)
    extra = {}
    if timed_rows is not None:
        got = timed_rows[sel]
        extra = {"checked": "the timed bake's rows", "timed_equals_sample_bake": bool(np.array_equal(got, sh)),
                 "timed_vs_sample_bake_max_rel": float(rel_err(got, sh).max())}
        sh = got
    d32, w = O.dirs_fibonacci(ndirs)
    B = O.basis_matrix(d32.astype(np.float64), w, lmax)
    orc = O.Scene(pos, idx, alb)
    ref = orc.bake(probes[sel], d32, B, sun, sky=sky, sky_n=SKY_N)
    rep = orc.bake(probes[sel], d32, B, sun, sky=sky, sky_n=SKY_N, force_hit=hit, force_vis=vis)
    e, er = rel_err(sh, ref), rel_err(sh, rep)
    return {"max": float(er.max()), "mean": float(er.mean()), "direct_max": float(e.max()),
            "direct_frac_within_1e-4": float((e < 1e-4).mean()), "probes": int(len(sel)),
            "note": "max/mean: decisions replayed; direct: the oracle's own FP64 decisions", **extra}


def trace_roofline(kname, k_avg_ms, stats, clk, sms, hbm_peak, peaks_measured, P, ntri, K, C, tile):
    """Roofline of the trace kernel.  It is bound by L1 throughput and
    instruction issue together (the scene's nodes and triangles stay in
    L1/L2), not by HBM: `bound` is the issue view, the one measured live, with
    the L1 view beside (the committed ncu capture shows the L1 data stage at
    80 % and issue at 75 %).  L1: the node and triangle bytes the lanes
    request (counted by an instrumented bake of the same rays) over the live
    launch time, against the nominal 128 B/clock/SM.  Issue: the capture's
    warp instructions per launch over the live launch time, against 4 issue
    slots/clock/SM.  The HBM view (algorithmic DRAM bytes) is kept beside."""
    mhz = clk.get("sm_max_mhz") or 2070.0
    secs = k_avg_ms * 1e-3 if k_avg_ms > 0 else None
    l1_bytes = stats["bytes"]
    l1_peak = sms * 128 * mhz * 1e6 / 1e9
    issue_peak = sms * 4 * mhz * 1e6
    ncu = TRACE_NCU.get(kname, {"capture": None, "dram_bytes": None, "warp_instructions": None,
                                "l1tex_throughput_pct": None, "issue_active_pct": None})
    wi = ncu["warp_instructions"]
    if tile:
        # one tile launch: probes and their order in, the FP32 radiance tile
        # out, the scene's nodes, triangles and albedo, the direction tables
        dram_alg = (P * (12 + 4) + P * NDIRS * 12 + max(ntri - 1, 0) * 64 + ntri * (48 + 16)
                    + NDIRS * (16 + 16 + 4))
    else:
        # one fused launch: probes and their order in, SH out, the chunk
        # partials written and read once, the scene, the direction and basis tables
        dram_alg = (P * (12 + 4 + K * 12 + 4) + (P * C * K * 3 * 4 * 2 if C > 1 else 0) + max(ntri - 1, 0) * 64
                    + ntri * (48 + 16) + NDIRS * (16 + 16 + 4 + 64))
    l1 = {"achieved": l1_bytes / secs / 1e9 if secs else None, "peak": l1_peak, "unit": "GB/s",
          "peak_source": f"nominal L1: {sms} SMs x 128 B/clock x {mhz:.0f} MHz (no measured L1 peak)",
          "requested_bytes_per_launch": l1_bytes}
    l1["frac"] = l1["achieved"] / l1_peak if l1["achieved"] else None
    issue = {"achieved": wi / secs if wi and secs else None, "peak": issue_peak, "unit": "warp instructions/s",
             "warp_instructions_per_launch": wi, "peak_source": f"{sms} SMs x 4 issue slots x {mhz:.0f} MHz"}
    issue["frac"] = issue["achieved"] / issue_peak if issue["achieved"] else None
    hbm = {"achieved": dram_alg / secs / 1e9 if secs else None, "peak": hbm_peak, "unit": "GB/s",
           "algorithmic_bytes_per_launch": dram_alg,
           "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)" if peaks_measured else "fallback 6.8 TB/s"}
    hbm["frac"] = hbm["achieved"] / hbm_peak if hbm["achieved"] else None
    # The issue view is the one measured live (the capture's instructions over
    # this run's launch time); the L1 data stage (ncu's wavefront throughput,
    # which the requested bytes understate) is the co-limit and stays beside.
    main = issue if wi else l1
    bound = "issue" if main is issue else "l1"
    return {"kernel": kname, "bound": bound, "achieved": main["achieved"], "peak": main["peak"], "unit": main["unit"],
            "frac": main["frac"], "traffic": ncu["dram_bytes"], "avg_launch_ms": k_avg_ms,
            "peak_source": main["peak_source"], "l1": l1, "issue": issue, "hbm": hbm, "ncu": ncu,
            "node_tests_per_ray": stats["node_tests_per_ray"], "node_fetches_per_ray": stats["node_fetches_per_ray"]}


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
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    if args.only:
        BAKE_ONLY.update(precision=args.bake_precision, grid=args.bake_grid)
        fn = {"bake": bake_measure, "c1": c1_measure, "skybox": skybox_measure, "projection": projection_measure,
              "batch": batch_measure, "service": service_measure, "refbake": refbake_measure}[args.only]
        print(json.dumps(fn(ctx, torch, stream, args.steps, hbm_peak)), flush=True)
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
        "mixed": vlb.bake_params(dirs, LMAX, vlb.PREC_MIXED, sun, sky=skyh),
        "bf16": vlb.bake_params(dirs, LMAX, vlb.PREC_BF16, sun, sky=skyh),
    }
    chosen = "fp32"  # the library's default precision

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
        timed(name, args.warmup if name in ("fused", "fp32") else 1)
    clocks = ClockSampler(local)
    clocks.start()
    ms_chosen, launches = timed(chosen, args.steps)
    rows = {chosen: d_out.cpu().numpy()}  # each path's last timed output, for its accuracy
    ms_fused, _ = timed("fused", args.steps)
    rows["fused"] = d_out.cpu().numpy()
    clk = clocks.stop()
    side = {}
    for n in ("mixed", "bf16"):
        side[n] = timed(n, max(3, args.steps // 3))[0]
        rows[n] = d_out.cpu().numpy()
    # per-kernel device time of the chosen path (library events on the same stream)
    ctx.profile_reset()
    timed(chosen, min(args.steps, 5), profile=True)
    prof = ctx.profile()
    ctx.profile_reset()
    timed("fused", min(args.steps, 5), profile=True)
    prof_fused = ctx.profile()
    # per-ray work counts for the L1 bytes (one instrumented bake, untimed)
    stats = ctx_trace_stats(ctx, scene, d_probes, params["fp32"])

    def agg(ms):
        return max_over_ranks(sum(ms), dist, "cuda")

    tot_chosen = agg(ms_chosen)
    tot_fused = agg(ms_fused)
    value = whole_job_rate(P * args.steps, world, tot_chosen)
    fused_value = whole_job_rate(P * args.steps, world, tot_fused)

    # e2e: public call with pinned host buffers (H2D probes, D2H SH) inside the timed region
    h_probes = torch.from_numpy(probes).pin_memory()
    h_out = torch.empty((P, K, 3), dtype=torch.float32).pin_memory()
    for _ in range(2):
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
    # accuracy of every timed path's own output rows against FP64 on a probe sample
    acc = {n: accuracy_vs_fp64(ctx, scene, probes, params[n], pos, idx, alb, sky, sun, timed_rows=rows[n])
           for n in params}
    ntri = int(idx.shape[0])
    per = -(-NDIRS // 4)         # the fused walk's chunk: at most 4 per probe,
    D = min(-(-per // 64) * 64, 4096)  # a multiple of 64 rays, at most 4096
    C = -(-NDIRS // D)
    sms = torch.cuda.get_device_properties(local).multi_processor_count

    def roof_of(pr, tile):
        kname = max(pr, key=lambda k: pr[k][1])
        klaunch, kms = pr.get(kname, (0, 0.0))
        return trace_roofline(kname, kms / max(klaunch, 1), stats, clk, sms, hbm_peak, bool(peaks), P, ntri, K, C,
                              tile)

    roof = roof_of(prof, True)
    roof_fused = roof_of(prof_fused, False)
    step_ms = sorted(ms_chosen)
    p50 = step_ms[len(step_ms) // 2]
    p99 = step_ms[min(len(step_ms) - 1, int(round(0.99 * (len(step_ms) - 1))))]
    # CPU baseline: the FP64 restatement on a bounded spread sample, all host threads
    csel = spread(P, args.cpu_probes)
    _, cpu_dt = cpu_time_oracle(pos, idx, alb, sky, sun, probes[csel], os.cpu_count() or 1)
    cpu_pps = len(csel) / cpu_dt
    line = {
        "metric": "probes/s", "metric_full": METRIC_FULL, "value": value, "unit": "probes/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": tot_chosen / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded SplitMix64 scene, sky and sun)",
        "config": config_dict(P, ntri),
        "timing": {"path": "VLB_PREC_FP32, the library default (" + "+".join(sorted(prof)) + ")",
                   "l2": "flushed (256 MiB write) before every timed step", "parallelism": f"replicas x{world}"},
        "grays_per_s": value * NDIRS / 1e9,
        "grays_incl_shadow_per_s": value * (NDIRS + stats["shadow_rays"] / P) / 1e9,
        "latency_ms": {"p50": p50, "p99": p99},
        "fused_one_kernel": {"value": fused_value, "unit": "probes/s", "ms": tot_fused / args.steps,
                             "p99_ms": sorted(ms_fused)[-1], "rel_err_vs_fp64": acc["fused"],
                             "roofline": roof_fused,
                             "kernels_ms": {k: {"launches": v[0], "avg_ms": v[1] / max(v[0], 1)}
                                            for k, v in prof_fused.items()}},
        "precisions": {
            "fp32": {"ms": tot_chosen / args.steps, "rel_err_vs_fp64": acc["fp32"]},
            "fused": {"ms": tot_fused / args.steps, "rel_err_vs_fp64": acc["fused"]},
            "mixed_bf16_hilo_tcgen05": {"ms": sum(side["mixed"]) / len(side["mixed"]),
                                        "rel_err_vs_fp64": acc["mixed"]},
            "bf16_tcgen05": {"ms": sum(side["bf16"]) / len(side["bf16"]), "rel_err_vs_fp64": acc["bf16"],
                             "note": "one BF16 per radiance sample: the stated-error form"}},
        "sh_rel_err_vs_fp64": acc["fp32"],
        "e2e": {"value": e2e_value, "unit": "probes/s", "h2d_bytes_per_step": int(P * 12),
                "d2h_bytes_per_step": int(P * K * 12)},
        "gpu_launches": int(launches),
        "roofline": roof,
        "kernels_ms": {k: {"launches": v[0], "avg_ms": v[1] / max(v[0], 1)} for k, v in prof.items()},
        "cpu_baseline": {"value": cpu_pps, "unit": "probes/s", "cores": os.cpu_count() or 1, "kind": "port",
                         "sample": f"{len(csel)} probes spread over the {P}-probe grid, {NDIRS} dirs each "
                                   f"({cpu_dt:.1f} s); the whole bake extrapolates to {P / cpu_pps:.0f} s",
                         "cpu": cpu_model()},
        "clocks": clk,
    }
    if not args.no_sections:
        line["c1"] = c1_measure(ctx, torch, stream, args.steps, hbm_peak)
        line["skybox_c0"] = skybox_measure(ctx, torch, stream, args.steps, hbm_peak)
        line["projection_c2"] = projection_measure(ctx, torch, stream, args.steps, hbm_peak)
        line["batch_c3"] = batch_measure(ctx, torch, stream, args.steps, hbm_peak)
        line["service_c4"] = service_measure(ctx, torch, stream, args.steps, hbm_peak)
        line["reference_bake"] = refbake_measure(ctx, torch, stream, args.steps, hbm_peak)
        # probes/s of the mixed-precision, batched and served forms over the
        # plain FP32 path on the same work (the stated target is 5x)
        b3, s4 = line["batch_c3"], line["service_c4"]
        line["vs_plain_fp32"] = {
            "c2_mixed_bake": line["precisions"]["fp32"]["ms"] / line["precisions"]["mixed_bf16_hilo_tcgen05"]["ms"],
            "c3_mixed_batch_vs_separate_fp32_bakes": b3["separate_bakes"]["ms"]
            / b3["mixed_bf16_hilo_tcgen05"]["ms_per_batch"],
            "c4_served_mixed_vs_sequential_fp32_bakes": s4["served_mixed_vs_plain_fp32"],
            "target": 5.0}
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


BAKE_ONLY = {"precision": "fp32", "grid": GRID[0]}


def bake_measure(ctx, torch, stream, steps, hbm_peak):
    """The headline workload's bake alone (the 4096-box scene, n^3 probes x
    1024 directions; --bake-precision, --bake-grid): `steps` bakes with inputs
    resident in HBM, per-kernel library times (for profiling captures)."""
    import vlb

    n = BAKE_ONLY["grid"]
    pos, idx, alb, sky, sun, probes = grid_probes(vlb, NBOXES, (n, n, n))
    scene = ctx.scene(pos, idx, alb)
    prec = vlb.PREC_FUSED if BAKE_ONLY["precision"] == "fused" else vlb.PREC_FP32
    p = vlb.bake_params(ctx.fibonacci(NDIRS), LMAX, prec, sun, sky=ctx.sky(sky, SKY_N))
    d_probes = torch.from_numpy(probes).cuda()
    out = torch.empty((probes.shape[0], vlb.k_of(LMAX), 3), dtype=torch.float32, device="cuda")
    ctx.bake(scene, d_probes, p, out=out)
    torch.cuda.synchronize()
    ctx.profile_reset()
    ctx.set_profiling(True)
    for _ in range(steps):
        ctx.bake(scene, d_probes, p, out=out)
    torch.cuda.synchronize()
    ctx.set_profiling(False)
    return {"workload": f"probe bake {n}^3 probes x {NDIRS} Fibonacci dirs, {NBOXES}-box scene, "
                        f"{BAKE_ONLY['precision']}",
            "kernels_ms": {k: v[1] / max(v[0], 1) for k, v in ctx.profile().items()}}


def c1_measure(ctx, torch, stream, steps, hbm_peak):
    """Config 1: the 64-box scene (778 triangles), 16^3 = 4096 grid probes x 256
    Fibonacci directions, L2 SH; fused, plain FP32 and mixed paths, inputs
    resident in HBM, L2 flushed before every bake; accuracy vs FP64 on a sample."""
    import vlb

    pos, idx, alb, sky, sun, probes = grid_probes(vlb, 64, (16, 16, 16))
    scene = ctx.scene(pos, idx, alb)
    ds = ctx.fibonacci(256)
    skyh = ctx.sky(sky, SKY_N)
    P = probes.shape[0]
    dp = torch.from_numpy(probes).cuda()
    out = torch.empty((P, vlb.k_of(LMAX), 3), dtype=torch.float32, device="cuda")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    res = {"workload": f"16^3 probes x 256 Fibonacci dirs, 64-box scene ({int(idx.shape[0])} tris), L{LMAX} SH",
           "probes": P}
    for name, prec in (("fused", vlb.PREC_FUSED), ("fp32", vlb.PREC_FP32), ("mixed", vlb.PREC_MIXED)):
        p = vlb.bake_params(ds, LMAX, prec, sun, sky=skyh)
        for _ in range(3):
            ctx.bake(scene, dp, p, out=out)
        ctx.profile_reset()
        ctx.set_profiling(True)
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        for a, b in evs:
            flush.zero_()
            a.record(stream)
            ctx.bake(scene, dp, p, out=out)
            b.record(stream)
        torch.cuda.synchronize()
        ctx.set_profiling(False)
        ms = sorted(a.elapsed_time(b) for a, b in evs)
        res[name] = {"ms": ms[len(ms) // 2], "probes_per_s": P / (ms[len(ms) // 2] / 1e3),
                     "kernels_ms": {k: v[1] / max(v[0], 1) for k, v in ctx.profile().items()},
                     "rel_err_vs_fp64": accuracy_vs_fp64(ctx, scene, probes, p, pos, idx, alb, sky, sun, 512, 256)}
    return res


# DRAM bytes per launch of the skybox kernel on this section's 1024-map batch,
# from the ncu capture summarised in profiles/skybox_c0.md.
SKYBOX_NCU = {"skybox_cube_group": 1247949000}


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
    kname = [k for k in prof if k.startswith("skybox")][0]
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
                     "avg_launch_ms": k_avg, "traffic": SKYBOX_NCU.get(kname)},
    }


# DRAM bytes per launch of the projection kernels from ncu captures of this
# section's tiles (profiles/project_tc_c2.md; None where not captured).
PROJECT_NCU = {"project_tc": 1640284160, "project_tc_split": None}


def projection_measure(ctx, torch, stream, steps, hbm_peak, nprobes=262144, S=1024):
    """Config 2 projection: a [262,144 x 3, 1024] radiance tile resident in
    HBM -- BF16 hi/lo pairs (the mixed-precision tile, 4 bytes a sample) and
    one BF16 a sample through the tcgen05 kernel (hi/lo BF16 basis, FP32
    accumulation), FP32 through the CUDA-core kernel."""
    import vlb

    ds = ctx.fibonacci(S)
    g = torch.Generator(device="cuda").manual_seed(SEED)
    t32 = torch.rand((nprobes * 3, S), generator=g, device="cuda") * 5
    out = torch.empty((nprobes, vlb.k_of(LMAX), 3), dtype=torch.float32, device="cuda")

    def run(tile, dtype, k):
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(k)]
        for a, b in evs:
            a.record(stream)
            ctx.project(tile, nprobes, ds, LMAX, dtype=dtype, out=out)
            b.record(stream)
        torch.cuda.synchronize()
        return sorted(a.elapsed_time(b) for a, b in evs)[k // 2]

    res = {"workload": f"SH projection of a [{nprobes}x3, {S}] radiance tile resident in HBM (1.6-3.2 GB, "
                       f"larger than L2), L{LMAX}"}
    outb = out.numel() * 4
    kern = {vlb.DTYPE_F32: "project_f32", vlb.DTYPE_BF16: "project_tc", vlb.DTYPE_BF16_SPLIT: "project_tc_split"}
    for name, dtype, esz in (("fp32_cuda_cores", vlb.DTYPE_F32, 4), ("mixed_hilo_tcgen05", vlb.DTYPE_BF16_SPLIT, 4),
                             ("bf16_tcgen05", vlb.DTYPE_BF16, 2)):
        if dtype == vlb.DTYPE_F32:
            tile = t32
        elif dtype == vlb.DTYPE_BF16:
            tile = t32.to(torch.bfloat16).view(torch.int16)
        else:
            hi = t32.to(torch.bfloat16)
            tile = torch.cat([hi, (t32 - hi.float()).to(torch.bfloat16)], dim=1).contiguous().view(torch.int16)
            del hi
        run(tile, dtype, 3)
        ms = run(tile, dtype, steps)
        nb = nprobes * 3 * S * esz + outb
        res[name] = {"probes_per_s": nprobes / (ms / 1e3), "ms": ms,
                     "roofline": {"kernel": kern[dtype], "bound": "hbm", "achieved": nb / (ms * 1e-3) / 1e9,
                                  "peak": hbm_peak, "unit": "GB/s", "frac": nb / (ms * 1e-3) / 1e9 / hbm_peak,
                                  "algorithmic_bytes_per_launch": nb,
                                  "traffic": PROJECT_NCU.get(kern[dtype])}}
        if dtype != vlb.DTYPE_F32:
            kk = 2 * S if dtype == vlb.DTYPE_BF16_SPLIT else S
            res[name]["roofline"]["mma_tflops"] = 2 * nprobes * 3 * kk * 32 / (ms * 1e-3) / 1e12
        if tile is not t32:
            del tile
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
    """The reference baker's own workload on the 64-box scene: a 7^3 probe grid
    over the origin-inclusive bounds in the reference's order, one ray per pixel
    of the 3141 x 1000 equirect env map (3,141,000 rays per probe, 1.08e9 in
    all), L3 (16 coefficients), fused, plain FP32 and mixed; device-resident
    probes and output, L2 flushed before each bake."""
    import vlb

    pos, idx, alb, sky, sun, _ = grid_probes(vlb, 64, (16, 16, 16))  # the 64-box (778-triangle) scene
    scene = ctx.scene(pos, idx, alb)
    probes, _ = vlb.probe_grid_ref_order(scene.bounds(include_origin=True), (7, 7, 7))
    P, W, H = probes.shape[0], 3141, 1000
    ds = ctx.equirect(W, H)
    skyh = ctx.sky(sky, SKY_N)
    d_probes = torch.from_numpy(probes).cuda()
    out = torch.empty((P, 16, 3), dtype=torch.float32, device="cuda")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    res = {"workload": f"{P} probes (7^3 reference grid) x {W}x{H} equirect rays, 64-box scene, L3",
           "primary_rays": P * W * H}
    for name, prec in (("fused", vlb.PREC_FUSED), ("fp32", vlb.PREC_FP32), ("mixed_bf16_hilo_tcgen05", vlb.PREC_MIXED)):
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
    """Config 3: 256 uneven bake jobs in one batch, replayed as a CUDA graph,
    L2 SH.  Chosen: the default FP32 tile path (one persistent lane-walk
    launch over every job's rays, one projection per direction set); beside
    it the one-kernel path (VLB_PREC_FUSED, no tile) and the mixed path (BF16
    hi/lo tile, one tcgen05 projection per direction set).
    Inputs and outputs resident in HBM; `e2e` passes pinned host probes and
    outputs.  Accuracy: a sample of jobs against the FP64 oracle with the
    device's decisions replayed."""
    import vlb

    vols = batch_volumes()
    sky_np = vlb.synth_cubemap(SEED, SKY_N)
    sky = ctx.sky(sky_np, SKY_N)
    dsets = {S: ctx.fibonacci(S) for S in (64, 256, 1024)}
    K = vlb.k_of(LMAX)
    scenes = [ctx.scene(pos, idx, alb) for pos, idx, alb, _, _, _ in vols]
    dprobes = [torch.from_numpy(v[3]).cuda() for v in vols]
    douts = [torch.empty((v[3].shape[0], K, 3), device="cuda") for v in vols]
    P = sum(v[3].shape[0] for v in vols)
    rays = sum(v[3].shape[0] * v[4] for v in vols)
    tris = [int(v[1].shape[0]) for v in vols]
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    steps = max(3, min(steps, 10))
    res = {"workload": f"{len(vols)} bake jobs: boxes log-uniform 16-16384 ({min(tris)}-{max(tris)} tris), probes "
                       f"log-uniform 64-32768 (total {P}), rays per probe in {{64,256,1024}} (total {rays} primary), "
                       f"L{LMAX} SH, CUDA graph replay",
           "l2": "flushed (256 MiB write) before every timed batch"}

    def jobs_for(prec):
        plist = [vlb.bake_params(dsets[S], LMAX, prec, sun, sky=sky) for _, _, _, _, S, sun in vols]
        return [(sc, pr, o, p) for sc, pr, o, p in zip(scenes, dprobes, douts, plist)], plist

    def run(js, p0, k, sched=None, profile=False):
        ctx.set_profiling(profile)
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(k)]
        l0 = ctx.launch_count
        for a, b in evs:
            flush.zero_()
            a.record(stream)
            ctx.bake_batch(js, p0, sched)
            b.record(stream)
        torch.cuda.synchronize()
        ctx.set_profiling(False)
        return [a.elapsed_time(b) for a, b in evs], ctx.launch_count - l0

    O = _oracle()
    for name, prec in (("fused", vlb.PREC_FUSED), ("mixed_bf16_hilo_tcgen05", vlb.PREC_MIXED),
                       ("plain_fp32", vlb.PREC_FP32)):
        jobs, plist = jobs_for(prec)
        r = {}
        if prec != vlb.PREC_MIXED:
            t0 = time.perf_counter()
            sched, tune_ms = ctx.batch_autotune(jobs, plist[0], reps=1)
            r["schedule"] = {f: getattr(sched, f) for f, _ in vlb.BatchSchedule._fields_}
            r["schedule"].update({"autotune_s": time.perf_counter() - t0, "autotune_best_ms": tune_ms})
            trials, cls = ctx.batch_tune_log()
            default_ms = trials[0][1]
            r["autotune"] = {
                "size_class": cls, "default_ms": default_ms, "best_ms": tune_ms,
                "gain_vs_default": default_ms / tune_ms - 1.0,
                # a measured margin: a winner more than 1 % faster than the default
                "winner": "tuned" if default_ms > 1.01 * tune_ms else "default (no trial beats it by more than 1 %)",
                "trials": [dict(sched, ms=ms) for sched, ms in trials]}
        run(jobs, plist[0], 3)  # direct, capture, replay
        ms, launches = run(jobs, plist[0], steps)
        ctx.profile_reset()
        direct = vlb.BatchSchedule(*(getattr(sched, f) for f, _ in vlb.BatchSchedule._fields_)) \
            if prec != vlb.PREC_MIXED else vlb.BatchSchedule(0, 1, 0)
        direct.graph = 0  # direct launches, so the library's per-kernel events see each kernel
        ctx.set_profiling(True)
        for _ in range(2):
            flush.zero_()
            ctx.bake_batch(jobs, plist[0], direct)
        torch.cuda.synchronize()
        ctx.set_profiling(False)
        prof = ctx.profile()
        tot = sum(ms)
        r.update({"probes_per_s": P * len(ms) / (tot / 1e3), "grays_per_s": rays * len(ms) / (tot / 1e3) / 1e9,
                  "ms_per_batch": tot / len(ms), "p99_ms": sorted(ms)[-1],
                  "gpu_launches_per_batch": launches / len(ms),
                  "kernels_ms": {k: {"launches": v[0], "avg_ms": v[1] / max(v[0], 1)} for k, v in prof.items()}})
        # accuracy: a spread sample of jobs (up to 64 probes each) vs FP64, decisions replayed
        errs = []
        for k in np.linspace(0, len(vols) - 1, 6).astype(int):
            pos, idx, alb, probes, S, sun = vols[k]
            sel = spread(probes.shape[0], 64)
            got = douts[k].cpu().numpy()[sel]
            sh, hit, vis, _ = ctx.bake(scenes[k], probes[sel], plist[k], debug=True)
            d32, w = O.dirs_fibonacci(S)
            B = O.basis_matrix(d32.astype(np.float64), w, LMAX)
            rep = O.Scene(pos, idx, alb).bake(probes[sel], d32, B, sun, sky=sky_np, sky_n=SKY_N, force_hit=hit,
                                              force_vis=vis)
            errs.append(rel_err(got, rep))
            if prec == vlb.PREC_FUSED:
                assert np.array_equal(sh, got)  # a batch job bakes like the job alone
        e = np.concatenate(errs)
        r["rel_err_vs_fp64"] = {"max": float(e.max()), "mean": float(e.mean()), "probes": int(e.size),
                                "note": "6 jobs spread over the batch, decisions replayed"}
        res[name] = r
    res["fused_vs_plain_fp32"] = res["fused"]["probes_per_s"] / res["plain_fp32"]["probes_per_s"]
    # the chosen jobs as 256 separate vlb_bake calls (device buffers, no sync between)
    jobs, plist = jobs_for(vlb.PREC_FP32)

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
    res["separate_bakes"] = {"ms": single_ms, "probes_per_s": P / (single_ms / 1e3),
                             "note": "the same 256 jobs as separate vlb_bake calls (FP32 tile path)"}
    # e2e: pinned host probes in, host SH out, through the public call
    hjobs = [(sc, torch.from_numpy(v[3]).pin_memory(), torch.empty((v[3].shape[0], K, 3)).pin_memory(), p)
             for sc, v, p in zip(scenes, vols, plist)]
    run(hjobs, plist[0], 3)
    e2e = []
    for _ in range(steps):
        flush.zero_()
        torch.cuda.synchronize()
        t = time.perf_counter()
        ctx.bake_batch(hjobs, plist[0])
        e2e.append(1e3 * (time.perf_counter() - t))
    res["e2e"] = {"probes_per_s": P * len(e2e) / (sum(e2e) / 1e3), "h2d_bytes_per_step": int(P * 12),
                  "d2h_bytes_per_step": int(P * K * 12)}
    return res


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
    relative to the measured capacity of the default (FP32 tile) service, 20%
    relights, 64 GiB budget; the one-kernel and mixed services at 0.6 x
    capacity."""
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

    def run(prec, rate, n, seed, slice_probes=0):
        svc = vlb.Service(ctx, budget_bytes=64 << 30, lmax=LMAX, precision=prec, slice_probes=slice_probes)
        reqs = service_requests(n, rate, seed, bounds)
        lat, wall, base = service_run(ctx, svc, scenes, dsets, sky, reqs, LMAX, prec)
        st = svc.stats()
        svc.close()
        lat = np.array(lat)
        return {"rate_offered": rate, "requests": n, "p50_ms": float(np.percentile(lat, 50)),
                "p90_ms": float(np.percentile(lat, 90)), "p99_ms": float(np.percentile(lat, 99)),
                "max_ms": float(lat.max()), "probes_per_s": st["probes"] / wall,
                "grays_per_s": st["rays"] / wall / 1e9, "batches": st["batches"], "relights": st["relights"],
                "relights_rebaked": st["relights_rebaked"], "evictions": st["evictions"],
                "bytes_peak": st["bytes_peak"], "wall_s": wall}

    # capacity of the default (FP32) service: every request at t = 0 (closed burst)
    cap = run(vlb.PREC_FP32, 1e9, nreq // 2, SEED + 7)
    capacity = cap["requests"] / cap["wall_s"]
    out["capacity_req_per_s"] = capacity
    out["burst"] = cap

    # The same burst two more ways: served by the mixed-precision (BF16 hi/lo
    # + tcgen05) service, and through the plain FP32 path, one vlb_bake per
    # request in arrival order with host buffers (the plain path keeps no
    # hits, so a relight re-bakes its original probes in full).
    out["burst_mixed_bf16_hilo"] = run(vlb.PREC_MIXED, 1e9, nreq // 2, SEED + 7)
    breqs = service_requests(nreq // 2, 1e9, SEED + 7, bounds)

    def plain_sequential():
        n = 0
        t = time.perf_counter()
        for r in breqs:
            b = r
            while b["relight"] is not None:
                b = breqs[b["relight"]]
            p = vlb.bake_params(dsets[b["S"]], LMAX, vlb.PREC_FP32, vlb.synth_sun(r["sun_seed"]),
                                sun_intensity=r["intensity"], sky=sky)
            ctx.bake(scenes[b["scene"]], b["probes"], p)
            n += b["probes"].shape[0]
        return n, time.perf_counter() - t

    plain_sequential()
    n, wall = plain_sequential()
    out["burst_plain_fp32_sequential"] = {"requests": len(breqs), "probes": n, "wall_s": wall,
                                          "probes_per_s": n / wall}
    out["served_mixed_vs_plain_fp32"] = out["burst_mixed_bf16_hilo"]["probes_per_s"] / (n / wall)

    # open-loop runs of about 5 s each (20 to nreq requests)
    def nfor(rate):
        return int(min(nreq, max(20, rate * 5.0)))

    out["slice_probes"] = 2048
    out["fp32"] = [run(vlb.PREC_FP32, f * capacity, nfor(f * capacity), SEED + 11 + k)
                   for k, f in enumerate((0.3, 0.6, 0.9))]
    # the same 0.3 x stream without slicing (whole requests per batch)
    out["fp32_unsliced"] = [run(vlb.PREC_FP32, 0.3 * capacity, nfor(0.3 * capacity), SEED + 11, 0xFFFFFFFF)]
    out["fused"] = [run(vlb.PREC_FUSED, 0.6 * capacity, nfor(0.6 * capacity), SEED + 12)]
    out["mixed_bf16_hilo"] = [run(vlb.PREC_MIXED, 0.6 * capacity, nfor(0.6 * capacity), SEED + 12)]
    # the floor under p99: the largest request the stream can hold (16,384
    # probes x 1,024 rays in the densest scene) alone in an idle service
    big = service_requests(1, 1.0, SEED + 5, bounds)[0]
    lo, hi = bounds[-1]
    probes = (lo + np.random.default_rng(SEED + 5).random((16384, 3)) * (hi - lo)).astype(np.float32)
    svc = vlb.Service(ctx, budget_bytes=64 << 30, lmax=LMAX, precision=vlb.PREC_FP32)
    alone = []
    for r in range(4):
        p = vlb.bake_params(dsets[1024], LMAX, vlb.PREC_FP32, vlb.synth_sun(big["sun_seed"] + r), sky=sky)
        alone.append(svc.wait(svc.submit(scenes[-1], probes, p))[1])
    svc.close()
    out["largest_request_alone_ms"] = float(np.median(alone[1:]))
    return out


def ctx_trace_stats(ctx, scene, probes, params):
    """Per-launch traversal work of the instrumented bake: node (64 B) and
    triangle (48 B) fetches as the kernel requests them (once per packet
    visit in packet mode, once per lane visit in lane mode), node tests once
    per ray."""
    import vlb

    st = vlb.trace_stats(ctx, scene, probes, params)
    rays = st["rays"] + st["shadow_rays"]
    return {"bytes": st["node_fetches"] * st["node_bytes"] + st["tri_fetches"] * 48,
            "node_fetches_per_ray": st["node_fetches"] / rays,
            "node_tests_per_ray": st["node_tests"] / rays, "shadow_rays": st["shadow_rays"]}


if __name__ == "__main__":
    sys.exit(main())
