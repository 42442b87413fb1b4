"""Small edge-case bakes run under both builds of libvlb.so (the normal one and
the bounds-check variant), one process per build: `python bounds_cases.py
OUT.npz` with VLB_LIB naming the library.  Writes every case's outputs (or
its status code) to OUT.npz plus the library's build flags; the test
compares the two files.

Cases: one probe; one triangle; an empty scene (every ray misses); a probe
inside a closed box (every ray hits); ragged probe and direction counts (not
multiples of 32 or 8); every precision and traversal mode; the wide tree;
the reference shading and running sums; a batch with a relight-free mix of
scenes; the skybox and tile projections.
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]
for p in (str(ROOT / "vulkan-light-bakery_gb300"),):
    if p not in sys.path:
        sys.path.insert(0, p)

import vlb  # noqa: E402


def one_box():
    """The 12 triangles of the unit cube."""
    v = np.array([[x, y, z] for x in (0, 1) for y in (0, 1) for z in (0, 1)], np.float32)
    quads = [(0, 1, 3, 2), (4, 6, 7, 5), (0, 4, 5, 1), (2, 3, 7, 6), (0, 2, 6, 4), (1, 5, 7, 3)]
    idx = []
    for a, b, c, d in quads:
        idx += [(a, b, c), (a, c, d)]
    return v, np.array(idx, np.uint32), np.full((12, 3), 0.6, np.float32)


def run(out_path: str) -> None:
    ctx = vlb.Context(0)
    res: dict[str, np.ndarray] = {"build_flags": np.array([lib_flags()])}

    def rec(name, fn):
        try:
            r = fn()
        except vlb.VlbError as e:
            res[name + "/status"] = np.array([e.status])
            return
        if isinstance(r, tuple):
            for i, x in enumerate(r):
                res[f"{name}/{i}"] = np.asarray(x)
        else:
            res[name] = np.asarray(r)

    sun = (0.3, 0.8, 0.2)
    pos, idx, alb = vlb.synth_box_scene(7, 64)
    scenes = {
        "boxes": ctx.scene(pos, idx, alb),
        "boxes_wide": ctx.scene(pos, idx, alb, flags=vlb.SCENE_TRAVERSAL_WIDE),
        "one_tri": ctx.scene(np.float32([[0, 0, 1], [1, 0, 1], [0, 1, 1]]), np.uint32([[0, 1, 2]]),
                             np.float32([[0.5, 0.4, 0.3]])),
        "empty": ctx.scene(np.zeros((0, 3), np.float32), np.zeros((0, 3), np.uint32), np.zeros((0, 3), np.float32)),
        "closed": ctx.scene(*one_box()),
    }
    sky = ctx.sky(vlb.synth_cubemap(7, 16), 16)
    rng = np.random.default_rng(7)
    probe_sets = {
        "one": np.float32([[0.25, 0.5, 0.4]]),
        "ragged": (rng.random((37, 3)) * 1.2 - 0.1).astype(np.float32),
        "inside": np.float32([[0.5, 0.5, 0.5], [0.2, 0.7, 0.4]]),
    }
    dsets = {"fib100": ctx.fibonacci(100), "fib256": ctx.fibonacci(256), "eq16x8": ctx.equirect(16, 8)}
    precs = {"fp32": vlb.PREC_FP32, "fused": vlb.PREC_FUSED, "mixed": vlb.PREC_MIXED, "bf16": vlb.PREC_BF16}
    modes = {"auto": 0, "packet": vlb.BAKE_TRAVERSAL_PACKET, "lane": vlb.BAKE_TRAVERSAL_LANE,
             "grid": vlb.BAKE_TRAVERSAL_GRID}
    cases = [("boxes", "one"), ("boxes", "ragged"), ("boxes_wide", "ragged"), ("one_tri", "ragged"),
             ("empty", "ragged"), ("closed", "inside")]
    for sn, pn in cases:
        for dn in ("fib100", "eq16x8"):
            for prn, prec in precs.items():
                for mn, mode in modes.items():
                    if prn != "fp32" and mn not in ("auto", "lane"):
                        continue
                    for lmax in (2, 3):
                        p = vlb.bake_params(dsets[dn], lmax, prec, sun, sky=sky, flags=mode)
                        rec(f"bake/{sn}/{pn}/{dn}/{prn}/{mn}/{lmax}",
                            lambda: ctx.bake(scenes[sn], probe_sets[pn], p, debug=prn != "fused"))
    # the reference shading and its running sums
    for prn in ("fp32", "fused"):
        p = vlb.bake_params(dsets["eq16x8"], 3, precs[prn], sun, shading=vlb.SHADE_REF_PHONG,
                            flags=vlb.BAKE_REF_ACCUMULATE)
        rec(f"ref/{prn}", lambda: ctx.bake(scenes["boxes"], probe_sets["ragged"], p))
    # a batch over mixed scenes and direction sets
    for prn in ("fused", "mixed", "fp32"):
        p = vlb.bake_params(dsets["fib256"], 2, precs[prn], sun, sky=sky)
        jobs = [(scenes["boxes"], probe_sets["ragged"], None), (scenes["one_tri"], probe_sets["one"], None),
                (scenes["closed"], probe_sets["inside"], None), (scenes["empty"], probe_sets["ragged"][:5], None)]
        rec(f"batch/{prn}", lambda: tuple(ctx.bake_batch(jobs, p)))
    # skybox and tile projections
    cm = vlb.synth_cubemap(8, 24)
    rec("skybox", lambda: ctx.skybox_sh(cm, vlb.SKY_CUBEMAP, 24, 24, 3))
    rad = rng.random((5, 3, 100)).astype(np.float32)
    rec("project_f32", lambda: ctx.project(rad, 5, dsets["fib100"], 3))
    np.savez(out_path, **res)
    ctx.close()


def lib_flags() -> int:
    return int(vlb.lib.vlb_build_flags())


if __name__ == "__main__":
    run(sys.argv[1])
