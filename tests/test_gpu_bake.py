"""Probe bake (trace + shade + projection) vs the FP64 oracle.

Protocol (tests/parity.py): per-ray hit triangles and shadow decisions must
match the oracle except on rays FP32 cannot decide (within 1e-6 of an edge);
their count is reported.  SH must be within 1e-4 relative (L2 per probe) of
the oracle replayed with the device's decisions, and the direct comparison
may exceed it only on probes that own an edge ray.
"""
import numpy as np
import pytest

import oracle as O
import parity
import vlb

pytestmark = pytest.mark.gpu


def c1_inputs(seed=1, nboxes=64, counts=(16, 16, 16), S=256, n_sky=128):
    pos, idx, alb = vlb.synth_box_scene(seed, nboxes)
    sky = vlb.synth_cubemap(seed, n_sky)
    sun = vlb.synth_sun(seed)
    bounds = np.concatenate([np.minimum(pos.min(0), 0), np.maximum(pos.max(0), 0)]).astype(np.float32)
    probes, _ = vlb.probe_grid_ref_order(bounds, counts)
    return pos, idx, alb, sky, sun, probes, S


def run_parity(ctx, pos, idx, alb, sky, sun, probes, S, lmax=2, precision=vlb.PREC_FP32, n_sky=128):
    scene = ctx.scene(pos, idx, alb)
    ds = ctx.fibonacci(S)
    skyh = ctx.sky(sky, n_sky) if sky is not None else None
    p = vlb.bake_params(ds, lmax=lmax, precision=precision, sun=sun, sky=skyh)
    sh, hit, vis, rad = ctx.bake(scene, probes, p, debug=True)
    d32, w = O.dirs_fibonacci(S)
    B = O.basis_matrix(d32.astype(np.float64), w, lmax)
    orc = O.Scene(pos, idx, alb)
    o_sh, o_hit, o_vis, o_edge, o_rad = orc.bake(probes, d32, B, sun, sky=sky, sky_n=n_sky if sky is not None else 0,
                                                 per_ray=True)
    cls = parity.classify(orc, probes, d32, sun, hit, vis, o_hit, o_vis, o_edge)
    rep = orc.bake(probes, d32, B, sun, sky=sky, sky_n=n_sky if sky is not None else 0, force_hit=hit, force_vis=vis)
    mism = ((hit != o_hit) | (vis != o_vis)).any(axis=1)
    return sh, hit, vis, rad, o_sh, mism, cls, rep


def test_config1_full_grid_parity(ctx):
    pos, idx, alb, sky, sun, probes, S = c1_inputs()
    sh, hit, vis, rad, o_sh, mism, cls, rep = run_parity(ctx, pos, idx, alb, sky, sun, probes, S)
    print("C1 parity:", {k: v for k, v in cls.items() if k != "unexplained"})
    assert not cls["unexplained"], cls["unexplained"][:10]
    assert cls["hit_mismatch"] + cls["shadow_mismatch"] <= 1e-3 * cls["rays"]
    err_rep = parity.per_probe_rel(sh, rep)
    assert err_rep.max() < parity.SH_TOL, err_rep.max()
    err = parity.per_probe_rel(sh, o_sh)
    bad = err >= parity.SH_TOL
    print(f"direct vs oracle: max {err.max():.3e}; probes over 1e-4: {int(bad.sum())}; probes with edge rays: "
          f"{int(mism.sum())}")
    assert not np.any(bad & ~mism)


@pytest.mark.parametrize("lmax", [2, 3])
def test_paths_agree(ctx, lmax):
    pos, idx, alb, sky, sun, probes, S = c1_inputs(seed=3, counts=(8, 8, 8))
    scene = ctx.scene(pos, idx, alb)
    ds = ctx.fibonacci(S)
    skyh = ctx.sky(sky, 128)
    plain = ctx.bake(scene, probes, vlb.bake_params(ds, lmax, vlb.PREC_FP32, sun, sky=skyh))
    fused = ctx.bake(scene, probes, vlb.bake_params(ds, lmax, vlb.PREC_FUSED, sun, sky=skyh))
    pk = vlb.bake_params(ds, lmax, vlb.PREC_FUSED, sun, sky=skyh)
    pk.flags = vlb.BAKE_FORCE_FUSED_KERNEL
    kernel = ctx.bake(scene, probes, pk)
    assert parity.per_probe_rel(kernel, plain).max() < 1e-5
    # the one-kernel schedule is deterministic and independent of the batch
    kernel2 = ctx.bake(scene, probes[::-1].copy(), pk)[::-1]
    assert np.array_equal(kernel, kernel2)
    assert parity.per_probe_rel(fused, plain).max() < 1e-5
    # the fused lane walk is deterministic, independent of the probe order and
    # of the per-ray debug outputs
    fused2 = ctx.bake(scene, probes[::-1].copy(), vlb.bake_params(ds, lmax, vlb.PREC_FUSED, sun, sky=skyh))[::-1]
    assert np.array_equal(fused, fused2)
    fused_dbg, hit, vis, rad = ctx.bake(scene, probes, vlb.bake_params(ds, lmax, vlb.PREC_FUSED, sun, sky=skyh),
                                        debug=True)
    assert np.array_equal(fused, fused_dbg)
    _, hit_p, vis_p, rad_p = ctx.bake(scene, probes, vlb.bake_params(ds, lmax, vlb.PREC_FP32, sun, sky=skyh),
                                      debug=True)
    assert np.array_equal(hit, hit_p) and np.array_equal(vis, vis_p) and np.array_equal(rad, rad_p)
    # mixed precision: BF16 hi/lo radiance pairs on the tensor cores, within
    # the FP32 tolerance (hi + lo keeps ~16 mantissa bits of every sample)
    mixed = ctx.bake(scene, probes, vlb.bake_params(ds, lmax, vlb.PREC_MIXED, sun, sky=skyh))
    e = parity.per_probe_rel(mixed, plain)
    print(f"mixed (BF16 hi/lo tile) vs fp32: max {e.max():.3e} mean {e.mean():.3e}")
    assert e.max() < 2e-5, e.max()
    # the half-size form: one BF16 per sample, its stated error.  BF16 keeps 8
    # mantissa bits per radiance sample (relative rounding up to 2^-9); samples
    # on one flat lit face share one radiance value, so their rounding errors
    # are equal and do not average out: ~1e-3 per probe.
    bf16 = ctx.bake(scene, probes, vlb.bake_params(ds, lmax, vlb.PREC_BF16, sun, sky=skyh))
    e = parity.per_probe_rel(bf16, plain)
    print(f"bf16 (one BF16 a sample) vs fp32: max {e.max():.3e} mean {e.mean():.3e}")
    assert e.max() < 5e-3 and e.mean() < 2e-3


def test_fused_large_direction_set(ctx):
    """A direction set whose basis does not stay in L2 (1024 x 300 equirect,
    19.7 MB of basis rows): the fused walk takes its work items chunk by chunk
    across the probes; the sums keep their per-probe order, so the result is
    the probe-major walk's and matches the tile path."""
    pos, idx, alb, sky, sun, probes, S = c1_inputs(seed=8, counts=(3, 2, 2))
    scene = ctx.scene(pos, idx, alb)
    ds = ctx.equirect(1024, 300)
    skyh = ctx.sky(sky, 128)
    fused = ctx.bake(scene, probes, vlb.bake_params(ds, 3, vlb.PREC_FUSED, sun, sky=skyh))
    plain = ctx.bake(scene, probes, vlb.bake_params(ds, 3, vlb.PREC_FP32, sun, sky=skyh))
    assert parity.per_probe_rel(fused, plain).max() < 1e-5
    again = ctx.bake(scene, probes[::-1].copy(), vlb.bake_params(ds, 3, vlb.PREC_FUSED, sun, sky=skyh))[::-1]
    assert np.array_equal(fused, again)
    one = ctx.bake(scene, probes[3:4], vlb.bake_params(ds, 3, vlb.PREC_FUSED, sun, sky=skyh))
    assert np.array_equal(fused[3:4], one)


def test_lmax3_reference_layout_and_radiance(ctx):
    pos, idx, alb, sky, sun, probes, S = c1_inputs(seed=5, counts=(4, 4, 4), S=64)
    sh, hit, vis, rad, o_sh, o_hit, cls, rep = run_parity(ctx, pos, idx, alb, sky, sun, probes, S, lmax=3)
    assert sh.shape == (64, 16, 3) and sh.dtype == np.float32  # 192 bytes per probe
    assert parity.per_probe_rel(sh, rep).max() < parity.SH_TOL


@pytest.mark.parametrize("nboxes,counts", [(64, (8, 8, 8)), (3000, (3, 3, 3))])
def test_traversal_modes_agree(ctx, nboxes, counts):
    """Packet and lane traversal give the same per-ray decisions and radiance,
    bit for bit (dense probes in a small scene; sparse probes in a large one)."""
    pos, idx, alb, sky, sun, probes, S = c1_inputs(seed=11, nboxes=nboxes, counts=counts)
    scene = ctx.scene(pos, idx, alb)
    ds = ctx.fibonacci(S)
    skyh = ctx.sky(sky, 128)
    res = []
    for flag in (vlb.BAKE_TRAVERSAL_PACKET, vlb.BAKE_TRAVERSAL_LANE):
        p = vlb.bake_params(ds, 2, vlb.PREC_FP32, sun, sky=skyh)
        p.flags = flag
        res.append(ctx.bake(scene, probes, p, debug=True))
    (sa, ha, va, ra), (sb, hb, vb, rb) = res
    diff = np.argwhere((ha != hb) | (va != vb))
    if len(diff):
        d32, w = O.dirs_fibonacci(S)
        B = O.basis_matrix(d32.astype(np.float64), w, 2)
        orc = O.Scene(pos, idx, alb)
        sel = np.unique(diff[:, 0])[:8]
        o_sh, o_hit, o_vis, o_edge, o_rad = orc.bake(probes[sel], d32, B, sun, sky=sky, sky_n=128, per_ray=True)
        for p_, s_ in diff[:12]:
            if p_ in sel:
                k = int(np.where(sel == p_)[0][0])
                print(f"probe {p_} {probes[p_]} dir {s_} {d32[s_]}: packet {ha[p_, s_]}/{va[p_, s_]} lane "
                      f"{hb[p_, s_]}/{vb[p_, s_]} oracle {o_hit[k, s_]}/{o_vis[k, s_]} edge {o_edge[k, s_]:.3e}")
    assert len(diff) == 0, f"{len(diff)} of {ha.size} rays differ"
    assert np.array_equal(ra, rb) and np.array_equal(sa, sb)
    if nboxes > 1000:  # the sparse case against the oracle too
        d32, w = O.dirs_fibonacci(S)
        B = O.basis_matrix(d32.astype(np.float64), w, 2)
        orc = O.Scene(pos, idx, alb)
        o_sh, o_hit, o_vis, o_edge, o_rad = orc.bake(probes, d32, B, sun, sky=sky, sky_n=128, per_ray=True)
        cls = parity.classify(orc, probes, d32, sun, hb, vb, o_hit, o_vis, o_edge)
        assert not cls["unexplained"], cls["unexplained"][:10]


def _big_triangles(seed, n):
    """n large random triangles across the unit cube (every grid cell holds
    most of them: the grids overflow and the rays walk the tree)."""
    rng = np.random.default_rng(seed)
    pos = rng.random((3 * n, 3)).astype(np.float32)
    idx = np.arange(3 * n, dtype=np.uint32).reshape(n, 3)
    alb = rng.uniform(0.2, 0.8, (n, 3)).astype(np.float32)
    return pos, idx, alb


@pytest.mark.parametrize("case", ["c1", "random_probes", "far_probes", "overflow", "one_triangle"])
def test_grid_mode_agrees(ctx, case):
    """Grid mode (per-direction triangle grids) gives the tree walk's per-ray
    decisions, radiance and coefficients bit for bit: dense grid probes,
    random probes in a 3.6k-triangle scene (16 x 16 cells), probes far
    outside the scene (their rays walk the tree), grids that overflow their
    capacity (all rays walk the tree) and a one-triangle scene."""
    rng = np.random.default_rng(7)
    S = 256
    sun = vlb.synth_sun(3)
    if case == "c1":
        pos, idx, alb, sky, sun, probes, S = c1_inputs(seed=11)
    elif case in ("random_probes", "far_probes"):
        pos, idx, alb = vlb.synth_box_scene(5, 300)
        probes = rng.random((2048, 3)).astype(np.float32)
        if case == "far_probes":
            probes[::3] = probes[::3] * 600.0 - 300.0
    elif case == "overflow":
        pos, idx, alb = _big_triangles(2, 4000)
        probes = rng.random((512, 3)).astype(np.float32)
    else:
        pos = np.float32([[0.1, 0.1, 0.5], [0.9, 0.2, 0.5], [0.4, 0.9, 0.5]])
        idx, alb = np.uint32([[0, 1, 2]]), np.float32([[0.5, 0.6, 0.7]])
        probes = rng.random((300, 3)).astype(np.float32)
    scene = ctx.scene(pos, idx, alb)
    ds = ctx.fibonacci(S)
    res = []
    for flag in (vlb.BAKE_TRAVERSAL_GRID, vlb.BAKE_TRAVERSAL_LANE):
        p = vlb.bake_params(ds, 2, vlb.PREC_FP32, sun)
        p.flags = flag
        ctx.profile_reset(); ctx.set_profiling(True)
        res.append(ctx.bake(scene, probes, p, debug=True))
        ctx.set_profiling(False)
        if flag == vlb.BAKE_TRAVERSAL_GRID:
            assert "grid_build" in ctx.profile()
    (sa, ha, va, ra), (sb, hb, vb, rb) = res
    diff = np.argwhere((ha != hb) | (va != vb))
    assert len(diff) == 0, f"{len(diff)} of {ha.size} rays differ, first {diff[:5].tolist()}"
    assert np.array_equal(ra, rb) and np.array_equal(sa, sb)
    assert (hb >= 0).any()


@pytest.mark.parametrize("nboxes,counts", [(64, (16, 16, 16)), (4000, (6, 6, 6))])
def test_traversal_trees_agree(ctx, nboxes, counts):
    """The clustered traversal tree and the Karras LBVH, each walked as the
    binary tree or as the 8-wide quantised tree collapsed from it, give the
    same per-ray decisions and radiance, bit for bit; the clustered tree visits
    fewer nodes than the LBVH, and the wide trees fewer than the binary ones."""
    pos, idx, alb, sky, sun, probes, S = c1_inputs(seed=13, nboxes=nboxes, counts=counts)
    skyh = ctx.sky(sky, 128)
    ds = ctx.fibonacci(S)
    res, work = [], []
    trees = (vlb.SCENE_TRAVERSAL_WIDE, vlb.SCENE_TRAVERSAL_LBVH | vlb.SCENE_TRAVERSAL_WIDE, 0,
             vlb.SCENE_TRAVERSAL_LBVH)
    for flags in trees:
        scene = ctx.scene(pos, idx, alb, flags=flags)
        p = vlb.bake_params(ds, 2, vlb.PREC_FP32, sun, sky=skyh)
        p.flags = vlb.BAKE_TRAVERSAL_LANE  # a tree walk in all four
        res.append(ctx.bake(scene, probes, p, debug=True))
        st = vlb.trace_stats(ctx, scene, probes, p)
        work.append(st["node_tests"] / (st["rays"] + st["shadow_rays"]))
    print("node visits per ray (clustered wide, LBVH wide, clustered binary, LBVH binary):",
          [f"{w:.1f}" for w in work])
    sa, ha, va, ra = res[0]
    for sb, hb, vb, rb in res[1:]:
        assert np.array_equal(ha, hb) and np.array_equal(va, vb)
        assert np.array_equal(ra, rb) and np.array_equal(sa, sb)
    assert work[2] < work[3] and work[0] < work[2] and work[1] < work[3]


def _wide_edge_scenes():
    """Scenes that stress the quantised boxes: far from the origin, flat (zero
    extent on an axis), coincident and overlapping triangles, two triangles."""
    rng = np.random.default_rng(17)
    out = {}
    pos, idx, alb = vlb.synth_box_scene(19, 300)
    out["offset_1000"] = (pos + np.float32([1000.0, -1000.0, 250.0]), idx, alb)
    p = rng.random((3 * 400, 3)).astype(np.float32)
    p[:, 1] = 0.5  # every triangle in the plane y = 0.5
    out["flat"] = (p, np.arange(3 * 400, dtype=np.uint32).reshape(-1, 3), rng.uniform(0.2, 0.8, (400, 3)))
    t = rng.random((3, 3)).astype(np.float32)
    out["coincident"] = (np.tile(t, (64, 1)), np.arange(3 * 64, dtype=np.uint32).reshape(-1, 3),
                         rng.uniform(0.2, 0.8, (64, 3)))
    p = (rng.random((3 * 500, 3)) * 2 - 0.5).astype(np.float32)
    out["big_overlap"] = (p, np.arange(3 * 500, dtype=np.uint32).reshape(-1, 3), rng.uniform(0.2, 0.8, (500, 3)))
    out["two"] = (np.float32([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 0.5], [1, 0, 0.5], [0, 1, 0.5]]),
                  np.arange(6, dtype=np.uint32).reshape(2, 3), np.float32([[0.5] * 3, [0.7] * 3]))
    return out


@pytest.mark.parametrize("case", ["offset_1000", "flat", "coincident", "big_overlap", "two"])
def test_wide_tree_edge_scenes(ctx, case):
    """The wide walk equals the binary walk bit for bit on scenes that stress
    the quantisation, for grid and random probes, in the tile and fused walks."""
    pos, idx, alb = _wide_edge_scenes()[case]
    alb = np.asarray(alb, np.float32)
    lo, hi = pos.min(0), pos.max(0)
    rng = np.random.default_rng(3)
    probes = np.concatenate([vlb.probe_grid_ref_order(np.concatenate([lo, hi]).astype(np.float32), (5, 5, 5))[0],
                             (lo + rng.random((100, 3)) * (hi - lo)).astype(np.float32)])
    ds = ctx.fibonacci(256)
    sun = vlb.synth_sun(5)
    wide = ctx.scene(pos, idx, alb, flags=vlb.SCENE_TRAVERSAL_WIDE)
    binary = ctx.scene(pos, idx, alb)
    for prec in (vlb.PREC_FP32, vlb.PREC_FUSED):
        p = vlb.bake_params(ds, 2, prec, sun)
        a = ctx.bake(wide, probes, p, debug=True)
        b = ctx.bake(binary, probes, p, debug=True)
        for x, y in zip(a, b):
            assert np.array_equal(x, y), (case, prec)


def test_empty_scene_sees_sky(ctx):
    sky = vlb.synth_cubemap(4, 32)
    pos = np.zeros((3, 3), np.float32)
    idx = np.zeros((0, 3), np.uint32)
    probes = np.float32([[0, 0, 0], [0.3, 0.2, 0.1]])
    scene = ctx.scene(pos, idx)
    ds = ctx.fibonacci(256)
    sh = ctx.bake(scene, probes, vlb.bake_params(ds, 2, sun=(0, 1, 0), sky=ctx.sky(sky, 32)))
    d32, w = O.dirs_fibonacci(256)
    ref = O.Scene(pos, idx, np.zeros((0, 3))).bake(probes, d32, O.basis_matrix(d32.astype(np.float64), w, 2),
                                                  [0, 1, 0], sky=sky, sky_n=32)
    assert parity.per_probe_rel(sh, ref).max() < 1e-5
    assert np.allclose(sh[0], sh[1])


def test_single_triangle_and_black_sky(ctx):
    pos = np.float32([[-1, 0, -1], [1, 0, -1], [0, 0, 1]])
    idx = np.uint32([[0, 1, 2]])
    alb = np.float32([[0.5, 0.25, 1.0]])
    probes = np.float32([[0, 0.5, 0], [0.1, -0.2, 0.0], [5, 5, 5]])
    sh, hit, vis, rad, o_sh, o_hit, cls, rep = run_parity(ctx, pos, idx, alb, None, [0.2, 1, 0.1], probes, 256)
    assert not cls["unexplained"]
    assert parity.per_probe_rel(sh, rep).max() < parity.SH_TOL


def test_device_resident_probes_and_output(ctx):
    torch = pytest.importorskip("torch")
    pos, idx, alb, sky, sun, probes, S = c1_inputs(seed=9, counts=(4, 4, 4))
    scene = ctx.scene(pos, idx, alb)
    ds = ctx.fibonacci(S)
    p = vlb.bake_params(ds, 2, vlb.PREC_FP32, sun, sky=ctx.sky(sky, 128))
    host = ctx.bake(scene, probes, p)
    out = torch.empty((probes.shape[0], 9, 3), dtype=torch.float32, device="cuda")
    ctx.bake(scene, torch.from_numpy(probes).cuda(), p, out=out)
    ctx.synchronize()
    assert np.array_equal(out.cpu().numpy(), host)


def test_bake_async_on_caller_stream(ctx):
    """vlb_bake_async on a caller-owned stream: returns before the bake is
    done, records the caller's event after it, gives vlb_bake's result; host
    arrays are refused."""
    torch = pytest.importorskip("torch")
    pos, idx, alb, sky, sun, probes, S = c1_inputs(seed=10, counts=(8, 8, 8))
    scene = ctx.scene(pos, idx, alb)
    p = vlb.bake_params(ctx.fibonacci(S), 3, vlb.PREC_FP32, sun, sky=ctx.sky(sky, 128))
    want = ctx.bake(scene, probes, p)
    stream = torch.cuda.Stream()
    done = torch.cuda.Event()
    done.record(stream)  # creates the event
    d_probes = torch.from_numpy(probes).cuda()
    out = torch.zeros((probes.shape[0], 16, 3), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    ctx.set_stream(stream.cuda_stream)
    try:
        ctx.bake_async(scene, d_probes, p, out, done)
        done.synchronize()
        assert np.array_equal(out.cpu().numpy(), want)
        with pytest.raises(vlb.VlbError) as e:
            ctx.bake_async(scene, probes, p, out, done)
        assert e.value.status == vlb.ERR_INVALID
        ctx.synchronize()
    finally:
        ctx.set_stream(None)


def test_context_close_closes_its_objects_first():
    """Closing a context with its scene, direction set and sky still referenced
    destroys them first (their destroy calls use the context), so dropping
    them afterwards is safe."""
    import gc

    c = vlb.Context(0)
    pos, idx, alb = vlb.synth_box_scene(2, 4)
    scene, ds, sky = c.scene(pos, idx, alb), c.fibonacci(64), c.sky(vlb.synth_cubemap(2, 8), 8)
    out = c.bake(scene, np.float32([[0.5, 0.5, 0.5]]), vlb.bake_params(ds, 2, sky=sky))
    assert np.isfinite(out).all()
    c.close()
    assert scene.h is None and ds.h is None and sky.h is None
    del scene, ds, sky
    gc.collect()


def test_invalid_params(ctx):
    pos, idx, alb = vlb.synth_box_scene(1, 2)
    scene = ctx.scene(pos, idx, alb)
    ds = ctx.fibonacci(64)
    p = vlb.bake_params(ds, 4)
    with pytest.raises(vlb.VlbError) as e:
        ctx.bake(scene, np.zeros((1, 3), np.float32), p)
    assert e.value.status == vlb.ERR_INVALID
    p = vlb.bake_params(ds, 2, sun=(0, 0, 0))
    with pytest.raises(vlb.VlbError):
        ctx.bake(scene, np.zeros((1, 3), np.float32), p)
