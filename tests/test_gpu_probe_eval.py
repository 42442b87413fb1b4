"""Evaluating a baked grid (vlb_probe_eval, vlb_sh_eval_dirs) vs the FP64 oracle.

Probe evaluation restates main.rchit:124-168 / sh.rmiss:23-39 with the
intended math (real grid origin, breadth-first probe order, K coefficients,
0 when no probe is visible).  Visibility decisions must match the oracle's
except where the oracle's shadow margin is within 1e-5 of an edge; RGB within
1e-4 relative (FP32 vs FP64) where all eight decisions match.
"""
import numpy as np
import pytest

import oracle as O
import vlb

pytestmark = pytest.mark.gpu


def _grid_case(seed, nboxes, counts, lmax, npts):
    pos, idx, alb = vlb.synth_box_scene(seed, nboxes)
    bounds = np.concatenate([np.minimum(pos.min(0), 0), np.maximum(pos.max(0), 0)]).astype(np.float32)
    probes, step = vlb.probe_grid_ref_order(bounds, counts)
    rng = np.random.default_rng(seed)
    K = (lmax + 1) ** 2
    coeffs = rng.standard_normal((probes.shape[0], K, 3)).astype(np.float32)
    pts = (bounds[:3] + rng.random((npts, 3)) * (bounds[3:] - bounds[:3])).astype(np.float32)
    nrm = rng.standard_normal((npts, 3)).astype(np.float32)
    return pos, idx, alb, bounds, step, coeffs, pts, nrm


@pytest.mark.parametrize("lmax", [2, 3])
def test_probe_eval_no_occluders(ctx, lmax):
    pos, idx, alb, bounds, step, coeffs, pts, nrm = _grid_case(4, 8, (6, 4, 5), lmax, 5000)
    out, vis = ctx.probe_eval(None, coeffs, lmax, bounds[:3], step, (6, 4, 5), pts, nrm)
    ref, rvis, _ = O.probe_eval(None, coeffs, lmax, bounds[:3], step, (6, 4, 5), pts, nrm)
    assert np.all(vis == 255) and np.all(rvis == 255)
    scale = np.abs(ref).max()
    assert np.abs(out - ref).max() < 1e-5 * scale


def test_probe_eval_with_visibility(ctx):
    counts = (7, 7, 7)  # the reference's grid (light_baker.cpp:38)
    pos, idx, alb, bounds, step, coeffs, pts, nrm = _grid_case(9, 64, counts, 2, 4000)
    scene = ctx.scene(pos, idx, alb)
    orc = O.Scene(pos, idx, alb)
    out, vis = ctx.probe_eval(scene, coeffs, 2, bounds[:3], step, counts, pts, nrm)
    ref, rvis, margin = O.probe_eval(orc, coeffs, 2, bounds[:3], step, counts, pts, nrm, margins=True)
    diff = np.unpackbits((vis ^ rvis)[:, None], axis=1, bitorder="little")[:, :8].astype(bool)
    near = np.abs(margin) < 1e-5
    print(f"visibility: {int(diff.sum())} of {diff.size} decisions differ, all within 1e-5 of an edge: "
          f"{bool(np.all(near[diff]))}; occluded fraction {1 - np.unpackbits(rvis).mean():.3f}")
    assert np.all(near[diff])
    same = ~diff.any(axis=1)
    scale = np.maximum(np.abs(ref[same]).max(axis=1), 1e-3)
    err = np.abs(out[same] - ref[same]).max(axis=1) / scale
    assert err.max() < 1e-4, err.max()
    assert 0 < np.unpackbits(rvis).mean() < 1  # the case has both visible and occluded probes
    # no visible probe: 0, not 0/0 (a point inside a closed box, off its diagonals)
    box_pos = np.float32([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]])
    q = [[0, 1, 2], [0, 2, 3], [4, 6, 5], [4, 7, 6], [0, 5, 1], [0, 4, 5], [3, 2, 6], [3, 6, 7], [0, 3, 7],
         [0, 7, 4], [1, 5, 6], [1, 6, 2]]
    inner = ctx.scene(box_pos * 0.2 + 0.4, np.uint32(q))
    o2, v2 = ctx.probe_eval(inner, np.ones((8, 9, 3), np.float32), 2, [0, 0, 0], [1, 1, 1], (2, 2, 2),
                            np.float32([[0.47, 0.53, 0.51]]), np.float32([[0, 1, 0]]))
    assert v2[0] == 0 and np.all(o2 == 0)


def test_probe_eval_reads_the_bake(ctx):
    """Bake an L3 grid with the library, then evaluate the baked coefficients at
    random points: device and oracle agree (the bake-to-viewer round trip)."""
    pos, idx, alb = vlb.synth_box_scene(3, 16)
    bounds = np.concatenate([np.minimum(pos.min(0), 0), np.maximum(pos.max(0), 0)]).astype(np.float32)
    counts = (4, 4, 4)
    probes, step = vlb.probe_grid_ref_order(bounds, counts)
    scene = ctx.scene(pos, idx, alb)
    sh = ctx.bake(scene, probes, vlb.bake_params(ctx.fibonacci(256), 3, vlb.PREC_FP32, vlb.synth_sun(3)))
    rng = np.random.default_rng(2)
    pts = (bounds[:3] + rng.random((500, 3)) * (bounds[3:] - bounds[:3])).astype(np.float32)
    nrm = rng.standard_normal((500, 3)).astype(np.float32)
    out, vis = ctx.probe_eval(scene, sh, 3, bounds[:3], step, counts, pts, nrm)
    ref, rvis, margin = O.probe_eval(O.Scene(pos, idx, alb), sh, 3, bounds[:3], step, counts, pts, nrm, margins=True)
    same = vis == rvis
    assert same.mean() > 0.98
    scale = np.maximum(np.abs(ref[same]).max(axis=1), 1e-3)
    assert (np.abs(out[same] - ref[same]).max(axis=1) / scale).max() < 1e-4


@pytest.mark.parametrize("lmax", [2, 3])
def test_sh_eval_dirs(ctx, lmax):
    K = (lmax + 1) ** 2
    rng = np.random.default_rng(lmax)
    c = rng.standard_normal((K, 3)).astype(np.float32)
    d = rng.standard_normal((3000, 3)).astype(np.float32)
    out = ctx.sh_eval_dirs(c, lmax, d)
    dn = d.astype(np.float64) / np.linalg.norm(d.astype(np.float64), axis=1, keepdims=True)
    ref = O.sh_basis(lmax, dn) @ c.astype(np.float64)
    assert np.abs(out - ref).max() < 1e-5 * np.abs(ref).max()


def test_probe_eval_invalid(ctx):
    with pytest.raises(vlb.VlbError):
        ctx.probe_eval(None, np.zeros((8, 9, 3), np.float32), 2, [0, 0, 0], [0, 1, 1], (2, 2, 2),
                       np.zeros((1, 3), np.float32), np.ones((1, 3), np.float32))
    with pytest.raises(vlb.VlbError):
        ctx.probe_eval(None, np.zeros((8, 9, 3), np.float32), 4, [0, 0, 0], [1, 1, 1], (2, 2, 2),
                       np.zeros((1, 3), np.float32), np.ones((1, 3), np.float32))
