"""Full-size configurations: size-independent properties at the benchmark sizes.

Config 2 (49,162 triangles, 262,144 probes x 1024 directions): every
precision bakes deterministically; the fused FP32 path (the timed one) and the
mixed BF16 hi/lo path agree with the FP64 oracle within 1e-4 on a probe
sample (decisions replayed as in tests/parity.py) and within 2e-5 of the
plain FP32 path on every probe; the one-BF16 form stays within its stated
bound.  Config 3 (the bench's 256 uneven jobs): the fused batch is
deterministic, schedule-independent, and every sampled job equals its own
single bake bit for bit.
"""
import sys
from pathlib import Path

import numpy as np
import pytest

import oracle as O
import parity
import vlb

pytestmark = pytest.mark.gpu
sys.path.insert(0, str(Path(__file__).resolve().parents[1]))


@pytest.fixture(scope="module")
def c2(ctx):
    pos, idx, alb = vlb.synth_box_scene(1, 4096)
    sky = vlb.synth_cubemap(1, 128)
    sun = vlb.synth_sun(1)
    bounds = np.concatenate([np.minimum(pos.min(0), 0), np.maximum(pos.max(0), 0)]).astype(np.float32)
    probes, _ = vlb.probe_grid_ref_order(bounds, (64, 64, 64))
    return pos, idx, alb, sky, sun, probes


def test_config2_full_bake(ctx, c2):
    torch = pytest.importorskip("torch")
    pos, idx, alb, sky, sun, probes = c2
    assert idx.shape[0] == 49162 and probes.shape[0] == 262144
    scene = ctx.scene(pos, idx, alb)
    ds = ctx.fibonacci(1024)
    skyh = ctx.sky(sky, 128)
    dp = torch.from_numpy(probes).cuda()
    res = {}
    for name, prec in (("fp32", vlb.PREC_FP32), ("fused", vlb.PREC_FUSED), ("mixed", vlb.PREC_MIXED),
                       ("bf16", vlb.PREC_BF16)):
        p = vlb.bake_params(ds, 2, prec, sun, sky=skyh)
        a = torch.empty((probes.shape[0], 9, 3), device="cuda")
        b = torch.empty_like(a)
        ctx.bake(scene, dp, p, out=a)
        ctx.bake(scene, dp, p, out=b)
        torch.cuda.synchronize()
        assert torch.equal(a, b), name  # deterministic
        res[name] = a.cpu().numpy()
        del a, b
    for name in ("fused", "mixed"):
        e = parity.per_probe_rel(res[name], res["fp32"])
        print(f"{name} vs fp32 on all probes: max {e.max():.3e} mean {e.mean():.3e}")
        assert e.max() < 2e-5, (name, e.max())
    e = parity.per_probe_rel(res["bf16"], res["fp32"])
    assert e.max() < 5e-3 and e.mean() < 1e-3, (e.max(), e.mean())
    # the timed (fused) path and the mixed path vs the FP64 oracle on a spread
    # sample, decisions replayed
    sel = np.linspace(0, probes.shape[0] - 1, 24).astype(int)
    d32, w = O.dirs_fibonacci(1024)
    B = O.basis_matrix(d32.astype(np.float64), w, 2)
    orc = O.Scene(pos, idx, alb)
    o_sh, o_hit, o_vis, o_edge, _ = orc.bake(probes[sel], d32, B, sun, sky=sky, sky_n=128, per_ray=True)
    for name, prec in (("fused", vlb.PREC_FUSED), ("mixed", vlb.PREC_MIXED)):
        p = vlb.bake_params(ds, 2, prec, sun, sky=skyh)
        sh, hit, vis, rad = ctx.bake(scene, probes[sel], p, debug=True)
        assert np.array_equal(sh, res[name][sel]), name  # the sample bakes like the full grid
        cls = parity.classify(orc, probes[sel], d32, sun, hit, vis, o_hit, o_vis, o_edge)
        assert not cls["unexplained"], cls["unexplained"][:5]
        rep = orc.bake(probes[sel], d32, B, sun, sky=sky, sky_n=128, force_hit=hit, force_vis=vis)
        err = parity.per_probe_rel(sh, rep)
        print(f"{name} vs FP64 oracle (decisions replayed): max {err.max():.3e}")
        assert err.max() < parity.SH_TOL, (name, err.max())


def test_config3_full_batch(ctx):
    import bench

    vols = bench.batch_volumes()
    assert len(vols) == 256
    sky = ctx.sky(vlb.synth_cubemap(1, 128), 128)
    dsets = {S: ctx.fibonacci(S) for S in (64, 256, 1024)}
    jobs, plist = [], []
    for pos, idx, alb, probes, S, sun in vols:
        p = vlb.bake_params(dsets[S], 2, vlb.PREC_FUSED, sun, sky=sky)
        jobs.append((ctx.scene(pos, idx, alb), probes, None, p))
        plist.append(p)
    a = ctx.bake_batch(jobs, plist[0])
    b = ctx.bake_batch(jobs, plist[0], vlb.BatchSchedule(4, 0, 0))
    assert all(np.array_equal(x, y) for x, y in zip(a, b))  # schedule-independent, deterministic
    rng = np.random.default_rng(0)
    for k in rng.choice(len(jobs), 12, replace=False):
        sc, probes, _, p = jobs[k]
        assert np.array_equal(a[k], ctx.bake(sc, probes, p)), k
