"""The reference baker's own shading (VLB_SHADE_REF_PHONG) and its carry-over
accumulator (VLB_BAKE_REF_ACCUMULATE) vs the FP64 oracle.

The workload is the reference bake's own shape: a 7x7x7 probe grid over the
scene bounds extended to the origin (src/baker/light_baker.cpp:80-101), the
equirect direction set of its env maps (shaders/env_map.rgen:18-28), lmax 3
(16 coefficients), the point light at (1, 10, 1) with bias 0.005 and Phong
0.5/0.5/16 (shaders/env_map.rchit:51-102), every sample sRGB-encoded and
stored as 8-bit UNORM.  Decisions are classified as in the Lambert bake
(shadow rays toward the point light); samples agree exactly except where
FP32 rounding moves a value across a UNORM rounding boundary (one step of
1/255); SH within 1e-4 of the oracle replayed with the device's decisions.
"""
import numpy as np
import pytest

import oracle as O
import parity
import vlb

pytestmark = pytest.mark.gpu

LIGHT = (1.0, 10.0, 1.0)
W, H = 128, 64  # equirect directions (8192)
LMAX = 3


def ref_inputs(seed=1, nboxes=64, counts=(7, 7, 7)):
    pos, idx, alb = vlb.synth_box_scene(seed, nboxes)
    sky = vlb.synth_cubemap(seed, 64)
    bounds = np.concatenate([np.minimum(pos.min(0), 0), np.maximum(pos.max(0), 0)]).astype(np.float32)
    probes, _ = vlb.probe_grid_ref_order(bounds, counts)
    return pos, idx, alb, sky, probes


def unorm_steps(a, b):
    """Per-sample difference in UNORM steps (both sides hold k/255 values)."""
    return np.abs(np.rint(np.asarray(a, np.float64) * 255) - np.rint(np.asarray(b, np.float64) * 255))


@pytest.fixture(scope="module")
def oracle_run():
    pos, idx, alb, sky, probes = ref_inputs()
    d32, bdirs, w = O.dirs_equirect(W, H)
    B = O.basis_matrix(bdirs, w, LMAX)
    orc = O.Scene(pos, idx, alb)
    sun = np.array([0.0, 1.0, 0.0], np.float32)  # unused by this shading
    o_sh, o_hit, o_vis, o_edge, o_rad = orc.bake(probes, d32, B, sun, sky=sky, sky_n=64, per_ray=True, shading=1,
                                                 light=LIGHT)
    return dict(pos=pos, idx=idx, alb=alb, sky=sky, probes=probes, d32=d32, B=B, orc=orc, sun=sun, o_sh=o_sh,
                o_hit=o_hit, o_vis=o_vis, o_edge=o_edge, o_rad=o_rad)


@pytest.mark.parametrize("prec", [vlb.PREC_FP32, vlb.PREC_FUSED, vlb.PREC_MIXED])
@pytest.mark.parametrize("with_sky", [False, True])
def test_reference_shading_parity(ctx, oracle_run, prec, with_sky):
    r = oracle_run
    if not with_sky:
        # the reference's bake binds no sky: misses are black
        o_sh, o_hit, o_vis, o_edge, o_rad = r["orc"].bake(r["probes"], r["d32"], r["B"], r["sun"], per_ray=True,
                                                          shading=1, light=LIGHT)
    else:
        o_sh, o_hit, o_vis, o_edge, o_rad = r["o_sh"], r["o_hit"], r["o_vis"], r["o_edge"], r["o_rad"]
    scene = ctx.scene(r["pos"], r["idx"], r["alb"])
    skyh = ctx.sky(r["sky"], 64) if with_sky else None
    p = vlb.bake_params(ctx.equirect(W, H), LMAX, prec, r["sun"], sky=skyh, shading=vlb.SHADE_REF_PHONG,
                        light_pos=LIGHT)
    sh, hit, vis, rad = ctx.bake(scene, r["probes"], p, debug=True)
    assert sh.shape == (343, 16, 3)
    cls = parity.classify(r["orc"], r["probes"], r["d32"], r["sun"], hit, vis, o_hit, o_vis, o_edge, light=LIGHT)
    print("reference shading decisions:", {k: v for k, v in cls.items() if k != "unexplained"})
    assert not cls["unexplained"], cls["unexplained"][:10]
    assert cls["hit_mismatch"] + cls["shadow_mismatch"] <= 1e-3 * cls["rays"]
    # replay the device's decisions: every sample is the oracle's UNORM value,
    # or one step away where FP32 rounding crossed a rounding boundary
    rep, _, _, _, rep_rad = r["orc"].bake(r["probes"], r["d32"], r["B"], r["sun"], sky=r["sky"] if with_sky else None,
                                          sky_n=64 if with_sky else 0, force_hit=hit, force_vis=vis, per_ray=True,
                                          shading=1, light=LIGHT)
    steps = unorm_steps(rad, rep_rad)
    flips = int((steps > 0).sum())
    print(f"UNORM samples one step off: {flips} of {steps.size}")
    assert steps.max() <= 1 and flips <= 2e-3 * steps.size
    assert np.all(np.abs(rad * 255 - np.rint(rad * 255)) < 1e-4)  # stored values are k/255
    err_rep = parity.per_probe_rel(sh, rep)
    print(f"replayed vs oracle: max {err_rep.max():.3e}")
    assert err_rep.max() < parity.SH_TOL
    err = parity.per_probe_rel(sh, o_sh)
    mism = ((hit != o_hit) | (vis != o_vis)).any(axis=1)
    bad = err >= parity.SH_TOL
    print(f"direct vs oracle: max {err.max():.3e}; probes over 1e-4: {int(bad.sum())}; with edge rays: "
          f"{int(mism.sum())}")
    assert not np.any(bad & ~mism)


def test_reference_shading_paths_agree(ctx, oracle_run):
    """The packet request (walked per lane under this shading), the lane walk
    and the fused lane walk give the same samples; the packet fused kernel
    refuses this shading."""
    r = oracle_run
    scene = ctx.scene(r["pos"], r["idx"], r["alb"])
    ds = ctx.equirect(W, H)
    outs = []
    for prec, flags in ((vlb.PREC_FP32, vlb.BAKE_TRAVERSAL_PACKET), (vlb.PREC_FP32, vlb.BAKE_TRAVERSAL_LANE),
                        (vlb.PREC_FUSED, 0)):
        p = vlb.bake_params(ds, LMAX, prec, r["sun"], shading=vlb.SHADE_REF_PHONG, light_pos=LIGHT, flags=flags)
        outs.append(ctx.bake(scene, r["probes"][:64], p, debug=True))
    for sh, hit, vis, rad in outs[1:]:
        assert np.array_equal(hit, outs[0][1]) and np.array_equal(vis, outs[0][2])
        assert np.array_equal(rad, outs[0][3])
        assert parity.per_probe_rel(sh, outs[0][0]).max() < 1e-5
    p = vlb.bake_params(ds, LMAX, vlb.PREC_FUSED, r["sun"], shading=vlb.SHADE_REF_PHONG, light_pos=LIGHT,
                        flags=vlb.BAKE_FORCE_FUSED_KERNEL)
    with pytest.raises(vlb.VlbError):
        ctx.bake(scene, r["probes"][:64], p)


def test_light_inside_the_scene(ctx):
    """A point light among the boxes: shadow rays end at the light, so a box
    behind it does not occlude."""
    pos, idx, alb, sky, probes = ref_inputs(seed=4, nboxes=32, counts=(3, 3, 3))
    light = (0.5, 0.55, 0.5)
    d32, bdirs, w = O.dirs_equirect(64, 32)
    B = O.basis_matrix(bdirs, w, 2)
    orc = O.Scene(pos, idx, alb)
    sun = np.array([0.0, 1.0, 0.0], np.float32)
    o_sh, o_hit, o_vis, o_edge, _ = orc.bake(probes, d32, B, sun, per_ray=True, shading=1, light=light)
    scene = ctx.scene(pos, idx, alb)
    p = vlb.bake_params(ctx.equirect(64, 32), 2, vlb.PREC_FUSED, sun, shading=vlb.SHADE_REF_PHONG, light_pos=light)
    sh, hit, vis, rad = ctx.bake(scene, probes, p, debug=True)
    cls = parity.classify(orc, probes, d32, sun, hit, vis, o_hit, o_vis, o_edge, light=light)
    assert not cls["unexplained"], cls["unexplained"][:10]
    rep = orc.bake(probes, d32, B, sun, force_hit=hit, force_vis=vis, shading=1, light=light)
    assert parity.per_probe_rel(sh, rep).max() < parity.SH_TOL


@pytest.mark.parametrize("prec", [vlb.PREC_FP32, vlb.PREC_FUSED])
def test_carry_over_accumulator(ctx, oracle_run, prec):
    """VLB_BAKE_REF_ACCUMULATE: probe i holds the sum of probes 0..i, added in
    FP64 and rounded once (1 ulp of FP32 against numpy's FP64 running sum)."""
    r = oracle_run
    scene = ctx.scene(r["pos"], r["idx"], r["alb"])
    ds = ctx.equirect(W, H)
    base = vlb.bake_params(ds, LMAX, prec, r["sun"], shading=vlb.SHADE_REF_PHONG, light_pos=LIGHT)
    acc = vlb.bake_params(ds, LMAX, prec, r["sun"], shading=vlb.SHADE_REF_PHONG, light_pos=LIGHT,
                          flags=vlb.BAKE_REF_ACCUMULATE)
    sh = ctx.bake(scene, r["probes"], base)
    out = ctx.bake(scene, r["probes"], acc)
    want = np.cumsum(sh.astype(np.float64), axis=0)
    scale = np.abs(np.cumsum(np.abs(sh.astype(np.float64)), axis=0))
    assert np.all(np.abs(out - want) <= np.abs(want) * 2.0 ** -23 + scale * 1e-13)
    assert np.array_equal(out[0], sh[0])
    # the running sum of a ragged batch (not a multiple of the 256-probe chunk)
    n = 300
    out_n = ctx.bake(scene, r["probes"][:n], acc)
    assert np.array_equal(out_n, out[:n])
