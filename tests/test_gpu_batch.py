"""Batched bakes (vlb_bake_batch): many (scene, probes) jobs in one persistent
trace launch.  Every job's output must be bit-identical to vlb_bake of that
job alone with the same parameters, whatever the batch composition, the
schedule (directions per work item, job order), graph replay or output
residency; one job is also checked against the FP64 oracle.
"""
import numpy as np
import pytest

import oracle as O
import parity
import vlb

pytestmark = pytest.mark.gpu


def _uniform_probes(rng, bounds, n):
    lo, hi = bounds[:3], bounds[3:]
    return (lo + rng.random((n, 3)) * (hi - lo)).astype(np.float32)


@pytest.fixture(scope="module")
def batch_world(ctx):
    """Uneven jobs: scenes of 1..2000 boxes, 0..3000 probes, two direction sets."""
    rng = np.random.default_rng(7)
    sky = ctx.sky(vlb.synth_cubemap(5, 32), 32)
    dsets = {64: ctx.fibonacci(64), 256: ctx.fibonacci(256)}
    spec = [(1, 37, 64), (2000, 3000, 256), (64, 1, 256), (300, 33, 64), (16, 0, 64), (5, 500, 256),
            (700, 1029, 64), (64, 31, 256)]
    jobs = []
    for i, (nb, n, S) in enumerate(spec):
        pos, idx, alb = vlb.synth_box_scene(100 + i, nb)
        scene = ctx.scene(pos, idx, alb)
        probes = _uniform_probes(rng, scene.bounds(), n)
        sun = vlb.synth_sun(200 + i)
        jobs.append(dict(scene=scene, probes=probes, S=S, sun=sun, pos=pos, idx=idx, alb=alb))
    return dict(jobs=jobs, sky=sky, dsets=dsets)


def _job_params(w, j, lmax, precision, intensity=5.0):
    return vlb.bake_params(w["dsets"][j["S"]], lmax=lmax, precision=precision, sun=j["sun"], sun_intensity=intensity,
                           sky=w["sky"])


def _singles(ctx, w, plist):
    return [ctx.bake(j["scene"], j["probes"], p) if len(j["probes"]) else np.empty((0, p.lmax ** 2 + 2 * p.lmax + 1, 3),
                                                                                    np.float32)
            for j, p in zip(w["jobs"], plist)]


@pytest.mark.parametrize("precision,lmax", [(vlb.PREC_MIXED, 2), (vlb.PREC_FP32, 2), (vlb.PREC_MIXED, 3),
                                            (vlb.PREC_FUSED, 2), (vlb.PREC_FUSED, 3), (vlb.PREC_BF16, 2)])
def test_batch_matches_single_bakes(ctx, batch_world, precision, lmax):
    w = batch_world
    plist = [_job_params(w, j, lmax, precision) for j in w["jobs"]]
    ref = _singles(ctx, w, plist)
    batch_p = plist[0]
    jobs = [(j["scene"], j["probes"], None, p) for j, p in zip(w["jobs"], plist)]
    outs = ctx.bake_batch(jobs, batch_p)
    for i, (a, b) in enumerate(zip(outs, ref)):
        assert a.shape == b.shape
        assert np.array_equal(a, b), (i, np.abs(a - b).max())


def test_batch_schedule_and_graph_invariance(ctx, batch_world):
    import torch

    w = batch_world
    plist = [_job_params(w, j, 2, vlb.PREC_MIXED) for j in w["jobs"]]
    ref = _singles(ctx, w, plist)
    jobs = [(j["scene"], j["probes"], None, p) for j, p in zip(w["jobs"], plist)]
    for dpw in (1, 8, 64):
        for order in (0, 1):
            outs = ctx.bake_batch(jobs, plist[0], vlb.BatchSchedule(dpw, order, 0))
            assert all(np.array_equal(a, b) for a, b in zip(outs, ref)), (dpw, order)
    # same shape three times: direct, capture + replay, replay
    for _ in range(3):
        outs = ctx.bake_batch(jobs, plist[0], vlb.BatchSchedule(16, 1, 1))
        assert all(np.array_equal(a, b) for a, b in zip(outs, ref))
    # device outputs and device probes (scattered by the kernel), mixed with host ones
    djobs, douts = [], []
    for k, (j, p) in enumerate(zip(w["jobs"], plist)):
        n = len(j["probes"])
        if k % 2 == 0:
            o = torch.empty((n, 9, 3), dtype=torch.float32, device="cuda")
            pr = torch.from_numpy(j["probes"]).cuda() if n else j["probes"]
        else:
            o, pr = None, j["probes"]
        djobs.append((j["scene"], pr, o, p))
    for _ in range(3):
        outs = ctx.bake_batch(djobs, plist[0], vlb.BatchSchedule(16, 1, 1))
        torch.cuda.synchronize()
        for a, b in zip(outs, ref):
            a = a.cpu().numpy() if hasattr(a, "cpu") else a
            assert np.array_equal(a, b)


def test_batch_autotune(ctx, batch_world):
    w = batch_world
    plist = [_job_params(w, j, 2, vlb.PREC_MIXED) for j in w["jobs"]]
    ref = _singles(ctx, w, plist)
    jobs = [(j["scene"], j["probes"], None, p) for j, p in zip(w["jobs"], plist)]
    sched, ms = ctx.batch_autotune(jobs, plist[0], reps=1)
    assert sched.dirs_per_item in (0, 1, 2, 4, 8, 16) and sched.cost_order in (0, 1) and ms > 0
    trials, cls = ctx.batch_tune_log()
    assert len(trials) == 12 and trials[0][0]["dirs_per_item"] == 0 and trials[0][0]["cost_order"] == 1
    assert ms == min(t for _, t in trials)
    ntris = max(j["scene"].ntris for j in w["jobs"])
    assert cls == (0 if ntris < 4096 else 1 if ntris < 65536 else 2 if ntris < (1 << 20) else 3)
    for _ in range(3):  # the tuned schedule of the class, graph on
        outs = ctx.bake_batch(jobs, plist[0])
        assert all(np.array_equal(a, b) for a, b in zip(outs, ref))
    # fused: one knob at a time from the default, which is the first trial
    fl = [_job_params(w, j, 2, vlb.PREC_FUSED) for j in w["jobs"]]
    fjobs = [(j["scene"], j["probes"], None, p) for j, p in zip(w["jobs"], fl)]
    fsched, fms = ctx.batch_autotune(fjobs, fl[0], reps=1)
    trials, _ = ctx.batch_tune_log()
    first = trials[0][0]
    assert (first["ctas_per_sm"], first["node_steps"], first["refill_idle"], first["cost_order"]) == (8, 6, 32, 1)
    assert 10 <= len(trials) <= 12 and fms == min(t for _, t in trials)
    fref = _singles(ctx, w, fl)
    outs = ctx.bake_batch(fjobs, fl[0])
    assert all(np.array_equal(a, b) for a, b in zip(outs, fref))


def test_fused_batch_schedule_and_graph_invariance(ctx, batch_world):
    """The fused walk's launch knobs (register budget, node steps per turn,
    refill threshold, job order) and graph replay change no bit of any job."""
    import torch

    w = batch_world
    plist = [_job_params(w, j, 3, vlb.PREC_FUSED) for j in w["jobs"]]
    ref = _singles(ctx, w, plist)
    jobs = [(j["scene"], j["probes"], None, p) for j, p in zip(w["jobs"], plist)]
    for occ, steps, refill, order in ((7, 1, 1, 0), (8, 6, 16, 1), (9, 16, 32, 1), (9, 4, 8, 0), (7, 12, 24, 1)):
        outs = ctx.bake_batch(jobs, plist[0], vlb.BatchSchedule(0, order, 0, occ, steps, refill))
        assert all(np.array_equal(a, b) for a, b in zip(outs, ref)), (occ, steps, refill, order)
    djobs = []
    for k, (j, p) in enumerate(zip(w["jobs"], plist)):
        n = len(j["probes"])
        o = torch.empty((n, 16, 3), dtype=torch.float32, device="cuda") if k % 2 == 0 else None
        djobs.append((j["scene"], j["probes"], o, p))
    for _ in range(3):  # direct, capture + replay, replay
        outs = ctx.bake_batch(djobs, plist[0], vlb.BatchSchedule(0, 1, 1, 8, 6, 16))
        torch.cuda.synchronize()
        for a, b in zip(outs, ref):
            a = a.cpu().numpy() if hasattr(a, "cpu") else a
            assert np.array_equal(a, b)
    with pytest.raises(vlb.VlbError):
        ctx.bake_batch(jobs, plist[0], vlb.BatchSchedule(0, 1, 0, 5, 6, 16))
    # the autotuner sweeps the fused knobs and keeps a schedule that bakes the same bits
    sched, ms = ctx.batch_autotune(jobs, plist[0], reps=1)
    assert sched.ctas_per_sm in (7, 8, 9) and sched.node_steps in (2, 4, 6, 8, 12, 16) and ms > 0
    assert sched.refill_idle in (4, 8, 16, 24, 32) and sched.graph == 1
    outs = ctx.bake_batch(jobs, plist[0])
    assert all(np.array_equal(a, b) for a, b in zip(outs, ref))
    # a single fused bake with the tuned knobs bakes the same bits too
    j = w["jobs"][1]
    assert np.array_equal(ctx.bake(j["scene"], j["probes"], plist[1]), ref[1])


def test_batch_job_vs_oracle(ctx, batch_world):
    """One batched job (300 boxes, 33 probes) against the FP64 oracle, FP32 path."""
    w = batch_world
    plist = [_job_params(w, j, 2, vlb.PREC_FP32) for j in w["jobs"]]
    jobs = [(j["scene"], j["probes"], None, p) for j, p in zip(w["jobs"], plist)]
    outs = ctx.bake_batch(jobs, plist[0])
    j = w["jobs"][3]
    d32, wt = O.dirs_fibonacci(j["S"])
    B = O.basis_matrix(d32.astype(np.float64), wt, 2)
    orc = O.Scene(j["pos"], j["idx"], j["alb"])
    sky = vlb.synth_cubemap(5, 32)
    sh, hit, vis, rad = ctx.bake(j["scene"], j["probes"], plist[3], debug=True)
    assert np.array_equal(outs[3], sh)
    rep = orc.bake(j["probes"], d32, B, j["sun"], sky=sky, sky_n=32, force_hit=hit, force_vis=vis)
    assert parity.per_probe_rel(outs[3], rep).max() < parity.SH_TOL


def test_batch_invalid(ctx, batch_world):
    w = batch_world
    j = w["jobs"][0]
    p2 = _job_params(w, j, 2, vlb.PREC_MIXED)
    p3 = _job_params(w, j, 3, vlb.PREC_MIXED)
    with pytest.raises(vlb.VlbError) as e:
        ctx.bake_batch([(j["scene"], j["probes"], None, p3)], p2)
    assert e.value.status == vlb.ERR_INVALID
    pf = _job_params(w, j, 2, vlb.PREC_FP32)
    with pytest.raises(vlb.VlbError):
        ctx.bake_batch([(j["scene"], j["probes"], None, pf)], p2)
    assert ctx.bake_batch([], p2) == []
    # a FUSED batch of one job is the fused single bake
    pu = _job_params(w, j, 2, vlb.PREC_FUSED)
    a = ctx.bake_batch([(j["scene"], j["probes"], None)], pu)[0]
    b = ctx.bake(j["scene"], j["probes"], pu)
    assert np.array_equal(a, b)
